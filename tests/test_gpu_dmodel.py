"""Models on the GPU (irwls_dmodel_*, libirwls_gb300/csrc/dev_model.cu):

- packing the reference's own weights on the device (full and budgeted
  golden cases, centroids that are class-mean rows included) and storing the
  model writes the reference's model file byte for byte;
- a model file read on the device predicts exactly what the host model
  predicts (the reference's soft and hard outputs), and stores back to the
  same bytes;
- a support-vector-free model and bad inputs fail cleanly.
"""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
VP = C.c_void_p
CASES = ["full_dense", "full_sparse", "full_linear", "budget_sgma", "budget_sgma_dense", "budget_linear",
         "budget_random"]


def _lib():
    lib = load()
    lib.irwls_dmodel_full.restype = VP
    lib.irwls_dmodel_full.argtypes = [VP, _abi.Properties, PD]
    lib.irwls_dmodel_budgeted.restype = VP
    lib.irwls_dmodel_budgeted.argtypes = [VP, _abi.Properties, PI, PD]
    lib.irwls_dmodel_read.restype = VP
    lib.irwls_dmodel_read.argtypes = [C.c_char_p]
    lib.irwls_dmodel_store.restype = C.c_int
    lib.irwls_dmodel_store.argtypes = [VP, C.c_char_p]
    lib.irwls_dmodel_predict.restype = PD
    lib.irwls_dmodel_predict.argtypes = [VP, _abi.SvmDataset, _abi.PredictProperties, C.c_int]
    lib.irwls_dmodel_info.argtypes = [VP, PI, PI, PD]
    lib.irwls_dmodel_free.argtypes = [VP]
    return lib


def _pack(lib, case):
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    if p["kind"] == "full":
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], working_set=p["w"])
        res = lib.irwls_resident_upload(tr.struct, prop, 0)
        b = np.ascontiguousarray(g["beta"])
        dm = lib.irwls_dmodel_full(res, prop, b.ctypes.data_as(PD))
    else:
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=p["size"])
        res = lib.irwls_resident_upload(tr.struct, prop, 1)
        c = np.ascontiguousarray(g["centroids"].astype(np.int32))
        w = np.ascontiguousarray(g["weights"])
        dm = lib.irwls_dmodel_budgeted(res, prop, c.ctypes.data_as(PI), w.ctypes.data_as(PD))
    assert res and dm, lib.irwls_last_error_message()
    return g, te, res, dm


def _tmp():
    with tempfile.NamedTemporaryFile(delete=False, suffix=".model") as f:
        return f.name


@pytest.mark.parametrize("case", CASES)
def test_device_packing_stores_the_reference_bytes(case):
    lib = _lib()
    g, te, res, dm = _pack(lib, case)
    path = _tmp()
    try:
        assert lib.irwls_dmodel_store(dm, path.encode()) == 0, lib.irwls_last_error_message()
        assert open(path, "rb").read() == g["model_bytes"].tobytes()
        # the packed model predicts the reference's outputs
        soft = H.arr(lib.irwls_dmodel_predict(dm, te.struct, _abi.make_predict_properties(labels=0), 1), te.l)
        hard = H.arr(lib.irwls_dmodel_predict(dm, te.struct, _abi.make_predict_properties(labels=0), 0), te.l)
        assert H.rel_err(soft, g["soft"]) < 1e-12
        assert np.array_equal(hard, g["hard"])
    finally:
        os.unlink(path)
        lib.irwls_dmodel_free(dm)
        lib.irwls_resident_free(res)


@pytest.mark.parametrize("case", ["full_sparse", "budget_sgma_dense", "full_linear"])
def test_read_predicts_like_the_host_model_and_stores_back(case):
    lib = _lib()
    g = H.golden(case)
    _, te = H.datasets(g)
    src, dst = _tmp(), _tmp()
    try:
        open(src, "wb").write(g["model_bytes"].tobytes())
        dm = lib.irwls_dmodel_read(src.encode())
        assert dm, lib.irwls_last_error_message()
        n, ne, b = C.c_int(), C.c_int(), C.c_double()
        lib.irwls_dmodel_info(dm, C.byref(n), C.byref(ne), C.byref(b))
        assert 36 + 16 * n.value + 16 * ne.value == len(g["model_bytes"].tobytes())
        # host model read from the same file
        libc = C.CDLL(None)
        libc.fopen.restype = VP
        libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        libc.fclose.argtypes = [VP]
        hm = _abi.Model()
        fp = libc.fopen(src.encode(), b"rb")
        lib.readModel(C.byref(hm), VP(fp))
        libc.fclose(VP(fp))
        for soft in (1, 0):
            dev = H.arr(lib.irwls_dmodel_predict(dm, te.struct, _abi.make_predict_properties(labels=0), soft), te.l)
            host = H.predict(lib, te, hm, soft)
            assert np.array_equal(dev.view(np.int64), host.view(np.int64))
        assert lib.irwls_dmodel_store(dm, dst.encode()) == 0
        assert open(dst, "rb").read() == g["model_bytes"].tobytes()
        lib.irwls_dmodel_free(dm)
    finally:
        os.unlink(src)
        os.unlink(dst)


def test_no_support_vectors_and_bad_inputs():
    lib = _lib()
    g = H.golden("full_dense")
    p = H.params(g)
    tr, te = H.datasets(g)
    prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"])
    res = lib.irwls_resident_upload(tr.struct, prop, 0)
    beta = np.zeros(tr.l + 1)
    beta[-1] = 0.25
    dm = lib.irwls_dmodel_full(res, prop, beta.ctypes.data_as(PD))
    assert dm, lib.irwls_last_error_message()
    soft = H.arr(lib.irwls_dmodel_predict(dm, te.struct, _abi.make_predict_properties(labels=0), 1), te.l)
    assert np.all(soft == 0.25)
    lib.irwls_dmodel_free(dm)
    bad = np.array([0, tr.l + 5], dtype=np.int32)
    w = np.ones(2)
    pb = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=2)
    assert not lib.irwls_dmodel_budgeted(res, pb, bad.ctypes.data_as(PI), w.ctypes.data_as(PD))
    assert not lib.irwls_dmodel_read(b"/nonexistent/model")
    lib.irwls_resident_free(res)
