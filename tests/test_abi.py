"""The C-ABI library loads and exports every function that include/*.h
declares; host-only entry points behave as the reference's (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load

HEADERS = ["IOStructures.h", "kernels.h", "full-train.h", "budgeted-train.h", "LIBIRWLS-predict.h",
           "ParallelAlgorithms.h", "irwls_gpu.h"]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(os.path.join(H.ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = load()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_the_reference_abi():
    assert C.sizeof(_abi.SvmSample) == 16
    assert C.sizeof(_abi.SvmDataset) == 48
    assert _abi.Properties.separator.offset == 56 and C.sizeof(_abi.Properties) == 72
    assert C.sizeof(_abi.Model) == 72 and _abi.Model.bias.offset == 56
    assert C.sizeof(_abi.PredictProperties) == 32


def _argv(words):
    arr = (C.c_char_p * (len(words) + 1))(*[w.encode() for w in words], None)
    pp = C.pointer(arr)
    return arr, C.cast(pp, C.POINTER(C.POINTER(C.c_char_p)))


def test_parse_full_train_options():
    lib = load()
    lib.parseTrainFULLParameters.restype = _abi.Properties
    lib.parseTrainFULLParameters.argtypes = [C.POINTER(C.c_int), C.c_void_p]
    words = ["full-train", "-g", "0.05", "-c", "10", "-w", "300", "-k", "0", "train.txt", "model.bin"]
    arr = (C.c_char_p * len(words))(*[w.encode() for w in words])
    pa = C.pointer(arr)
    argc = C.c_int(len(words))
    pp = C.pointer(C.cast(arr, C.POINTER(C.c_char_p)))
    p = lib.parseTrainFULLParameters(C.byref(argc), pp)
    assert (p.Kgamma, p.C, p.MaxSize, p.kernelType, p.Eta, p.size) == (0.05, 10.0, 300, 0, 0.001, 10)
    assert argc.value == 3
    assert pp.contents[1] == b"train.txt" and pp.contents[2] == b"model.bin"


def test_scalar_kernel_api_matches_oracle():
    g = H.golden("budget_sgma")
    p = H.params(g)
    tr, _ = H.datasets(g)
    lib, port = load(), H.port()
    prop = _abi.make_properties(gamma=p["gamma"], kernel=1)
    for i, j in [(0, 1), (5, 9), (tr.l, 3), (tr.l + 1, tr.l), (7, 7)]:
        assert lib.kernelFunction(tr.struct, i, j, prop) == port.kernelFunction(tr.struct, i, j, prop)
    prop.kernelType = 0
    assert lib.kernelFunction(tr.struct, 2, 3, prop) == port.kernelFunction(tr.struct, 2, 3, prop)


def test_training_without_gpu_fails_loudly():
    """No silent CPU path: with no device the entry points return NULL and
    report why."""
    lib = load()
    if lib.irwls_gpu_available():
        pytest.skip("a GPU is present")
    g = H.golden("full_smallws")
    tr, _ = H.datasets(g)
    prop = _abi.make_properties(gamma=0.5, working_set=7)
    assert not lib.trainFULL(tr.struct, prop)
    assert lib.irwls_last_error() != 0
    assert b"CUDA" in lib.irwls_last_error_message() or b"device" in lib.irwls_last_error_message()


@pytest.mark.parametrize("seed", [0, 1, 2, 7, 12345, 2**31 - 1, 2**32 - 1])
def test_batch_generator_reproduces_libc_rand(seed):
    """Batch workers draw from the library's restatement of glibc's rand():
    it must give exactly the libc sequence after srand(seed)."""
    lib = load()
    n = 2000
    out = (C.c_int * n)()
    lib.irwls_rand_sequence(seed, n, out)
    libc = C.CDLL(None)
    libc.srand(C.c_uint(seed))
    ref = [libc.rand() for _ in range(n)]
    assert list(out) == ref
