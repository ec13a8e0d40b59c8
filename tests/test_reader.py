"""Host-side boundary (no GPU): the library's libsvm readers, the Python
dataset builder and the binary model file against the reference's own
outputs (tests/golden)."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load

LIBC = C.CDLL(None)
LIBC.fopen.restype = C.c_void_p
LIBC.fopen.argtypes = [C.c_char_p, C.c_char_p]
LIBC.fclose.argtypes = [C.c_void_p]


def _rows_equal(ds, n, g, key):
    rows, y, q = _abi.dataset_rows(ds, n)
    lens = g[key + "_lens"]
    assert [len(r[0]) for r in rows] == list(lens)
    idx = np.concatenate([r[0] for r in rows]) if lens.sum() else np.zeros(0, np.int32)
    val = np.concatenate([r[1] for r in rows]) if lens.sum() else np.zeros(0)
    assert np.array_equal(idx, g[key + "_idx"])
    assert np.array_equal(val, g[key + "_val"])
    assert np.array_equal(y, g[key + "_y"])
    assert np.array_equal(q, g[key + "_q"])


@pytest.mark.parametrize("key,labeled", [("dense", True), ("onehot", True), ("unlabeled", False)])
def test_reader_matches_reference(key, labeled):
    g = np.load(os.path.join(H.GOLDEN, "reader.npz"))
    lib = load()
    with tempfile.NamedTemporaryFile(suffix=".libsvm", delete=False) as f:
        f.write(g[key + "_text"].tobytes())
        path = f.name
    try:
        ds = lib.readTrainFile(path.encode()) if labeled else lib.readUnlabeledFile(path.encode())
        assert ds.l == int(g[key + "_l"])
        assert ds.sparse == int(g[key + "_sparse"])
        assert ds.maxdim == int(g[key + "_maxdim"])
        _rows_equal(ds, ds.l + (2 if labeled else 0), g, key)
        lib.freeDataset(ds)
    finally:
        os.unlink(path)


@pytest.mark.parametrize("key", ["dense", "onehot"])
def test_python_builder_matches_reference_reader(key):
    """The dataset builder used by the tests and the benchmark lays rows out as
    the reference's readTrainFile does."""
    g = np.load(os.path.join(H.GOLDEN, "reader.npz"))
    text = g[key + "_text"].tobytes().decode().splitlines()
    indptr, idx, val, y = [0], [], [], []
    for line in text:
        toks = line.split()
        y.append(float(toks[0]))
        for t in toks[1:]:
            a, b = t.split(":")
            idx.append(int(a))
            val.append(float(b))
        indptr.append(len(idx))
    hd = _abi.build_dataset(indptr, idx, val, y)
    assert hd.sparse == int(g[key + "_sparse"])
    assert hd.maxdim == int(g[key + "_maxdim"])
    _rows_equal(hd.struct, hd.n_rows, g, key)


@pytest.mark.parametrize("case", ["full_dense", "budget_sgma"])
def test_model_file_bytes_match_reference(case):
    """calculate*Model + storeModel write the reference's bytes for the
    reference's own weights; readModel reads them back."""
    g = H.golden(case)
    p = H.params(g)
    tr, _ = H.datasets(g)
    lib = load()
    if p["kind"] == "full":
        b = np.ascontiguousarray(g["beta"])
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], working_set=p["w"])
        mdl = lib.calculateFULLModel(prop, tr.struct, b.ctypes.data_as(C.POINTER(C.c_double)))
    else:
        c = np.ascontiguousarray(g["centroids"].astype(np.int32))
        w = np.ascontiguousarray(g["weights"])
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=p["size"])
        mdl = lib.calculateBudgetedModel(prop, tr.struct, c.ctypes.data_as(C.POINTER(C.c_int)),
                                         w.ctypes.data_as(C.POINTER(C.c_double)))
    with tempfile.NamedTemporaryFile(delete=False) as f:
        path = f.name
    try:
        fp = LIBC.fopen(path.encode(), b"wb")
        lib.storeModel(C.byref(mdl), C.c_void_p(fp))
        LIBC.fclose(C.c_void_p(fp))
        data = open(path, "rb").read()
        assert data == g["model_bytes"].tobytes()
        m2 = _abi.Model()
        fp = LIBC.fopen(path.encode(), b"rb")
        lib.readModel(C.byref(m2), C.c_void_p(fp))
        LIBC.fclose(C.c_void_p(fp))
        assert m2.nSVs == mdl.nSVs and m2.nElem == mdl.nElem and m2.bias == mdl.bias
        assert np.array_equal(np.ctypeslib.as_array(m2.weights, shape=(m2.nSVs,)),
                              np.ctypeslib.as_array(mdl.weights, shape=(mdl.nSVs,)))
        assert 36 + 16 * mdl.nSVs + 16 * mdl.nElem == len(data)
    finally:
        os.unlink(path)


def test_write_output_format():
    lib = load()
    lib.writeOutput.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_int]
    v = np.array([1.0, -1.0, 0.123456789])
    with tempfile.NamedTemporaryFile(delete=False) as f:
        path = f.name
    try:
        lib.writeOutput(path.encode(), v.ctypes.data_as(C.POINTER(C.c_double)), 3)
        assert open(path).read() == "1.000000\n-1.000000\n0.123457\n"
    finally:
        os.unlink(path)
