"""ctypes mirror of the LIBIRWLS C ABI (include/*.h of this repository).

The structs are field-for-field the reference's (include/IOStructures.h:44-122
in RobeDM/LIBIRWLS), so one loader drives any shared object that exports the
reference API: this package's libirwls_gb300.so, and the CPU checkers used
by the tests.

Datasets built here (``build_dataset``) reproduce, from CSR arrays, the exact
in-memory layout that the reference's libsvm reader produces
(src/IOStructures.c:88-275): rows in file order with index -1 terminators,
two class-mean rows appended at l and l+1, ``quadratic_value`` summed in file
order, the ``sparse`` flag rule, and the reader's quirk of dividing the
negative-mean norm by the positive count (src/IOStructures.c:259).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np


class SvmSample(C.Structure):
    _fields_ = [("index", C.c_int), ("value", C.c_double)]


class SvmDataset(C.Structure):
    _fields_ = [
        ("l", C.c_int),
        ("sparse", C.c_int),
        ("maxdim", C.c_int),
        ("y", C.POINTER(C.c_double)),
        ("x", C.POINTER(C.POINTER(SvmSample))),
        ("quadratic_value", C.POINTER(C.c_double)),
        ("features", C.POINTER(SvmSample)),
    ]


class Properties(C.Structure):
    _fields_ = [
        ("Kgamma", C.c_double),
        ("kernelType", C.c_int),
        ("C", C.c_double),
        ("Threads", C.c_int),
        ("MaxSize", C.c_int),
        ("size", C.c_int),
        ("algorithm", C.c_int),
        ("Eta", C.c_double),
        ("file", C.c_int),
        ("separator", C.c_char_p),
        ("verbose", C.c_int),
    ]


class PredictProperties(C.Structure):
    _fields_ = [
        ("Labels", C.c_int),
        ("Threads", C.c_int),
        ("Soft", C.c_int),
        ("file", C.c_int),
        ("separator", C.c_char_p),
        ("verbose", C.c_int),
    ]


class Model(C.Structure):
    _fields_ = [
        ("Kgamma", C.c_double),
        ("kernelType", C.c_int),
        ("sparse", C.c_int),
        ("nSVs", C.c_int),
        ("nElem", C.c_int),
        ("weights", C.POINTER(C.c_double)),
        ("x", C.POINTER(C.POINTER(SvmSample))),
        ("quadratic_value", C.POINTER(C.c_double)),
        ("maxdim", C.c_int),
        ("bias", C.c_double),
        ("features", C.POINTER(SvmSample)),
    ]


SAMPLE_DTYPE = np.dtype([("index", np.int32), ("value", np.float64)], align=True)
assert SAMPLE_DTYPE.itemsize == C.sizeof(SvmSample) == 16


def make_properties(gamma=1.0, C_=1.0, kernel=1, threads=1, working_set=500, size=10,
                    algorithm=1, eta=0.001, verbose=0) -> Properties:
    p = Properties()
    p.Kgamma = gamma
    p.kernelType = kernel
    p.C = C_
    p.Threads = threads
    p.MaxSize = working_set
    p.size = size
    p.algorithm = algorithm
    p.Eta = eta
    p.file = 1
    p.separator = b","
    p.verbose = verbose
    return p


def make_predict_properties(labels=0, soft=1, threads=1, verbose=0) -> PredictProperties:
    p = PredictProperties()
    p.Labels = labels
    p.Threads = threads
    p.Soft = soft
    p.file = 1
    p.separator = b","
    p.verbose = verbose
    return p


def bind_api(lib: C.CDLL) -> C.CDLL:
    """Declares argument/return types of every reference entry point the
    shared object exports (missing ones are skipped)."""
    D = C.c_double
    PD = C.POINTER(C.c_double)
    PI = C.POINTER(C.c_int)
    sig = {
        "trainFULL": (PD, [SvmDataset, Properties]),
        "subIRWLS": (PD, [SvmDataset, Properties, PD, PD, PD]),
        "rpermute": (PI, [C.c_int]),
        "SGMA": (PI, [SvmDataset, Properties]),
        "randomCentroids": (PI, [SvmDataset, Properties]),
        "IRWLSpar": (PD, [SvmDataset, PI, Properties]),
        "test": (PD, [SvmDataset, Model, PredictProperties]),
        "softTest": (PD, [SvmDataset, Model, PredictProperties]),
        "kernelFunction": (D, [SvmDataset, C.c_int, C.c_int, Properties]),
        "kernelTest": (D, [SvmDataset, C.c_int, Model, C.c_int]),
        "initMemory": (None, [C.c_int, C.c_int]),
        "freeMemory": (None, [C.c_int]),
        "updateMemory": (None, [C.c_int, C.c_int]),
        "calculateFULLModel": (Model, [Properties, SvmDataset, PD]),
        "calculateBudgetedModel": (Model, [Properties, SvmDataset, PI, PD]),
        "readTrainFile": (SvmDataset, [C.c_char_p]),
        "readUnlabeledFile": (SvmDataset, [C.c_char_p]),
        "readTrainFileCSV": (SvmDataset, [C.c_char_p, C.c_char_p]),
        "readUnlabeledFileCSV": (SvmDataset, [C.c_char_p, C.c_char_p]),
        "freeDataset": (None, [SvmDataset]),
        "freeModel": (None, [Model]),
        "ParallelLinearSystem": (None, [PD, C.c_int, C.c_int, C.c_int, C.c_int, PD, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_int, PD, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int]),
        "ParallelChol": (None, [PD, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
        "ParallelVectorMatrixT": (None, [PD, C.c_int, PD, PD, C.c_int]),
        "ParallelVectorMatrix": (None, [PD, C.c_int, PD, PD, C.c_int]),
        "port_solve": (None, [PD, C.c_int, PD, PD]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    return lib


def load_library(path: str) -> C.CDLL:
    """dlopen with RTLD_LOCAL so that several implementations of the same API
    can live in one process."""
    return bind_api(C.CDLL(os.path.abspath(path), mode=os.RTLD_NOW | os.RTLD_LOCAL))


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class HostDataset:
    """An svm_dataset whose arrays are owned by numpy (never freed by C)."""

    def __init__(self, features: np.ndarray, row_start: np.ndarray, y: np.ndarray,
                 q: np.ndarray, l: int, sparse: int, maxdim: int):
        self.features = features
        self.row_start = row_start
        self.y = y
        self.q = q
        self.l = l
        self.sparse = sparse
        self.maxdim = maxdim
        base = features.ctypes.data
        self._rowptrs = (C.POINTER(SvmSample) * len(row_start))()
        for i, s in enumerate(row_start.tolist()):
            self._rowptrs[i] = C.cast(base + 16 * s, C.POINTER(SvmSample))
        self.struct = SvmDataset()
        self.struct.l = l
        self.struct.sparse = sparse
        self.struct.maxdim = maxdim
        self.struct.y = _ptr(y, C.c_double)
        self.struct.x = C.cast(self._rowptrs, C.POINTER(C.POINTER(SvmSample)))
        self.struct.quadratic_value = _ptr(q, C.c_double)
        self.struct.features = C.cast(base, C.POINTER(SvmSample))

    @property
    def n_rows(self) -> int:
        return len(self.row_start)


def _row_sums_in_order(vals2d: np.ndarray) -> np.ndarray:
    """Left-to-right sums of each row (padding entries are +0.0)."""
    acc = np.zeros(vals2d.shape[0])
    for k in range(vals2d.shape[1]):
        acc = acc + vals2d[:, k]
    return acc


def build_dataset(indptr, indices, values, y, with_means: bool = True) -> HostDataset:
    """Reference-reader layout of a labeled libsvm file given as CSR arrays
    (indices are the file's 1-based feature indices, strictly increasing per
    row). ``with_means`` appends the class-mean rows as readTrainFile does;
    without it the layout is that of readUnlabeledFile."""
    indptr = np.asarray(indptr, dtype=np.int64)
    indices = np.asarray(indices, dtype=np.int32)
    values = np.asarray(values, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    l = len(indptr) - 1
    lens = np.diff(indptr)
    maxlen = int(lens.max()) if l else 0
    maxidx = int(indices.max()) if len(indices) else 0

    # per-row padded value matrix, for in-order norms
    pad = np.zeros((l, max(maxlen, 1)))
    col = np.arange(len(values)) - np.repeat(indptr[:-1], lens)
    row = np.repeat(np.arange(l), lens)
    pad[row, col] = values
    q_rows = _row_sums_in_order(pad * pad)

    n_real = int(indptr[-1]) + l
    if with_means:
        elements = n_real + 2 * (maxidx + 2)
    else:
        elements = n_real
    feats = np.zeros(elements, dtype=SAMPLE_DTYPE)
    pos = np.arange(len(values)) + row          # each earlier row adds one terminator
    feats["index"][pos] = indices
    feats["value"][pos] = values
    row_start = (indptr[:-1] + np.arange(l)).astype(np.int64)
    feats["index"][row_start + lens] = -1

    # sparse flag: entry dm of any row compared with features[dm] of the array
    sparse = 0
    if l and maxlen:
        ref_idx = feats["index"][:maxlen]
        if np.any(indices != ref_idx[col]):
            sparse = 1

    if not with_means:
        return HostDataset(feats, row_start, y.copy(), q_rows, l, sparse, maxidx)

    pos_rows = y == 1.0
    n_pos = float(np.count_nonzero(pos_rows))
    n_neg = float(l - np.count_nonzero(pos_rows))
    mean_p = np.zeros(maxidx + 1)
    mean_n = np.zeros(maxidx + 1)
    ent_pos = np.repeat(pos_rows, lens)
    np.add.at(mean_p, indices[ent_pos], values[ent_pos])     # sequential, in file order
    np.add.at(mean_n, indices[~ent_pos], values[~ent_pos])
    j = n_real
    starts = [row_start, np.array([j])]
    kp = np.nonzero(mean_p != 0.0)[0]
    vp = mean_p[kp] / n_pos
    feats["index"][j:j + len(kp)] = kp
    feats["value"][j:j + len(kp)] = vp
    qp = 0.0
    for v in vp:
        qp = qp + v * v
    j += len(kp)
    feats["index"][j] = -1
    j += 1
    starts.append(np.array([j]))
    kn = np.nonzero(mean_n != 0.0)[0]
    vn = mean_n[kn] / n_neg
    feats["index"][j:j + len(kn)] = kn
    feats["value"][j:j + len(kn)] = vn
    qn = 0.0
    for v in mean_n[kn] / n_pos:       # the reference reader divides by the positive count here
        qn = qn + v * v
    j += len(kn)
    feats["index"][j] = -1
    rs = np.concatenate(starts).astype(np.int64)
    yy = np.concatenate([y, [1.0, -1.0]])
    qq = np.concatenate([q_rows, [qp, qn]])
    return HostDataset(feats, rs, yy, qq, l, sparse, maxidx)


def dataset_rows(ds: SvmDataset, n_rows: int):
    """Reads rows back from any svm_dataset (e.g. one made by a C reader) as a
    list of (indices, values) arrays plus y and quadratic_value."""
    rows = []
    for i in range(n_rows):
        p = ds.x[i]
        idx, val = [], []
        k = 0
        while p[k].index != -1:
            idx.append(p[k].index)
            val.append(p[k].value)
            k += 1
        rows.append((np.array(idx, dtype=np.int32), np.array(val)))
    y = np.ctypeslib.as_array(ds.y, shape=(n_rows,)).copy()
    q = np.ctypeslib.as_array(ds.quadratic_value, shape=(n_rows,)).copy()
    return rows, y, q
