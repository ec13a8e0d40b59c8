"""The host half of the device libsvm reader (irwls_dataset_assemble in
libirwls_gb300/csrc/io.c): from parsed rows -- labels, entries with -1
terminators, row norms, the sparse flag and the largest indices -- it builds
the dataset readTrainFile builds, class-mean rows included (sums in row
order, the negative mean's norm divided by the positive count). Checked
without a GPU: the rows are parsed here (Python's float() rounds as strtod
does) and the result must equal readTrainFile's field for field, bit for
bit."""
import ctypes as C
import os
import random
import tempfile

import numpy as np

from libirwls_gb300 import _abi, load

REC = np.dtype([("index", "<i4"), ("pad", "<i4"), ("value", "<f8")])


def _parse(text):
    """Rows of well-formed libsvm text as the device reader hands them over."""
    rows, y, q, lens = [], [], [], []
    maxidx = 0
    for line in text.decode().split("\n"):
        if not line.strip():
            continue
        toks = line.split()
        y.append(float(toks[0]))
        qq = 0.0
        for t in toks[1:]:
            i, v = t.split(":")
            rows.append((int(i), 0, float(v)))
            qq = qq + float(v) * float(v)
            maxidx = max(maxidx, int(i))
        rows.append((-1, 0, 0.0))
        lens.append(len(toks) - 1)
        q.append(qq)
    rec = np.array(rows, dtype=REC)
    start = np.concatenate([[0], np.cumsum(np.array(lens) + 1)[:-1]]).astype(np.int64)
    # the reference's sparse flag: entry dm of a row against entry dm of the whole array
    sparse = 0
    for s0, n in zip(start, lens):
        for dm in range(n):
            if rec[dm]["index"] != rec[s0 + dm]["index"]:
                sparse = 1
    max_index = max([rec[s0 + n - 1]["index"] for s0, n in zip(start, lens) if n] + [0])
    elements = int(sum(lens)) + len(lens)
    return rec, start, np.array(y), np.array(q), elements, maxidx, max_index, sparse


def _text(seed, n, d):
    rng = random.Random(seed)
    lines = []
    for _ in range(n):
        idx = sorted(rng.sample(range(1, d + 1), rng.randint(1, d)))
        lines.append(rng.choice(["1", "-1"]) + "".join(" %d:%r" % (i, rng.uniform(-5, 5)) for i in idx))
    return ("\n".join(lines) + "\n").encode()


def _fields(ds):
    rows, y, q = _abi.dataset_rows(ds, ds.l + 2)
    return ds.l, ds.sparse, ds.maxdim, rows, y, q


def test_assembly_equals_host_reader():
    lib = load()
    fn = lib.irwls_dataset_assemble
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_abi.SvmDataset), C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_void_p,
                   C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    for seed, n, d in [(1, 400, 30), (2, 50, 3), (3, 1, 8)]:
        text = _text(seed, n, d)
        rec, start, y, q, elements, maxidx, max_index, sparse = _parse(text)
        ds = _abi.SvmDataset()
        assert fn(C.byref(ds), len(y), elements, maxidx, max_index, sparse, rec.ctypes.data, len(rec),
                  start.ctypes.data_as(C.POINTER(C.c_longlong)), y.ctypes.data_as(C.POINTER(C.c_double)),
                  q.ctypes.data_as(C.POINTER(C.c_double))) == 0
        with tempfile.NamedTemporaryFile(delete=False, suffix=".libsvm") as f:
            f.write(text)
            path = f.name
        try:
            host = lib.readTrainFile(path.encode())
        finally:
            os.unlink(path)
        a, b = _fields(ds), _fields(host)
        assert a[:3] == b[:3]
        for (ia, va), (ib, vb) in zip(a[3], b[3]):
            assert np.array_equal(ia, ib) and np.array_equal(va.view(np.int64), vb.view(np.int64))
        assert np.array_equal(a[4].view(np.int64), b[4].view(np.int64))
        assert np.array_equal(a[5].view(np.int64), b[5].view(np.int64))
        lib.freeDataset(ds)
        lib.freeDataset(host)
