"""Python 3 module with the surface of the reference's `LIBIRWLS` extension
(python-package/pythonmodule.c, method table pythonmodule.h:143-150), running
on the GPU library:

    full_train(data, labels, gamma=1., C=1., threads=1, workingSet=500,
               eta=0.001, kernel=1, verbose=1)              -> classifier
    budgeted_train(data, labels, gamma=1., C=1., threads=1, size=10,
                   algorithm=0, kernel=1, verbose=1)          -> classifier
    predict(classifier, data, labels=None, threads=1, Soft=0, verbose=1)
                                                              -> numpy array
    save(classifier, file)
    load(file)                                                -> classifier

`data` is an (n, d) array, `labels` an (n,) array of +1/-1. As in the
reference, the arrays become datasets the way its module builds them (every
non-zero value is feature j+1; budgeted training appends the module's
class-mean rows, pythonmodule.c:213-355), budgeted training defaults to
random centroids (`algorithm=0`) and full training to a working set of 500.
A classifier is a `Classifier` object that owns the C `model`; `predict` and
`save` also accept a PyCapsule named "CLASSIFIER" holding a `model*`, which is
what the reference's extension returns.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _abi, check, load as _load_lib

_libc = ct.CDLL(None)
_libc.fopen.restype = ct.c_void_p
_libc.fopen.argtypes = [ct.c_char_p, ct.c_char_p]
_libc.fclose.argtypes = [ct.c_void_p]
_libc.free.argtypes = [ct.c_void_p]

_capsule_get = ct.pythonapi.PyCapsule_GetPointer
_capsule_get.restype = ct.c_void_p
_capsule_get.argtypes = [ct.py_object, ct.c_char_p]


class Classifier:
    """A trained model (C `model` struct) owned by Python."""

    def __init__(self, mdl: _abi.Model):
        self.model = mdl

    def __del__(self):
        try:
            _load_lib().freeModel(self.model)
        except Exception:
            pass

    @property
    def nSVs(self) -> int:
        return self.model.nSVs

    @property
    def bias(self) -> float:
        return self.model.bias

    def weights(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.model.weights, shape=(self.model.nSVs,)).copy()


def _model_of(classifier) -> _abi.Model:
    if isinstance(classifier, Classifier):
        return classifier.model
    ptr = _capsule_get(classifier, b"CLASSIFIER")
    return ct.cast(ptr, ct.POINTER(_abi.Model)).contents


def _arrays(data, labels):
    X = np.ascontiguousarray(np.asarray(data, dtype=np.float64))
    if X.ndim != 2:
        raise ValueError("data must be a 2-D array")
    y = np.ascontiguousarray(np.asarray(labels, dtype=np.float64)) if labels is not None else np.zeros(X.shape[0])
    if y.shape[0] != X.shape[0]:
        raise ValueError("labels must have one entry per row of data")
    return X, y


def _props(gamma, C_, threads, working_set, eta, size, algorithm, kernel, verbose):
    return _abi.make_properties(gamma=gamma, C_=C_, kernel=kernel, threads=threads, working_set=working_set,
                                size=size, algorithm=algorithm, eta=eta, verbose=verbose)


def full_train(data, labels, gamma=1.0, C=1.0, threads=1, workingSet=500, eta=0.001, kernel=1, verbose=1):
    """Full SVM by IRWLS (pythonmodule.c:451-508)."""
    lib = _load_lib()
    X, y = _arrays(data, labels)
    PD = C_double_p()
    ds = lib.irwls_dataset_from_dense(X.ctypes.data_as(PD), y.ctypes.data_as(PD), X.shape[0], X.shape[1])
    p = _props(gamma, C, threads, workingSet, eta, 10, 0, kernel, verbose)
    try:
        lib.initMemory(threads, workingSet + 1)
        beta = check(lib.trainFULL(ds, p), "full_train")
        mdl = lib.calculateFULLModel(p, ds, beta)
        _libc.free(ct.cast(beta, ct.c_void_p))
    finally:
        lib.freeDataset(ds)
    return Classifier(mdl)


def budgeted_train(data, labels, gamma=1.0, C=1.0, threads=1, size=10, algorithm=0, kernel=1, verbose=1):
    """Budgeted SVM: random (algorithm=0) or SGMA (1) centroids, then IRWLS
    (pythonmodule.c:370-438)."""
    lib = _load_lib()
    X, y = _arrays(data, labels)
    PD = C_double_p()
    ds = lib.irwls_dataset_from_dense_with_means(X.ctypes.data_as(PD), y.ctypes.data_as(PD), X.shape[0],
                                                 X.shape[1])
    p = _props(gamma, C, threads, 0, 0.001, size, algorithm, kernel, verbose)
    try:
        lib.initMemory(threads, size)
        cent = lib.randomCentroids(ds, p) if algorithm == 0 else check(lib.SGMA(ds, p), "budgeted_train (SGMA)")
        w = check(lib.IRWLSpar(ds, cent, p), "budgeted_train (IRWLS)")
        mdl = lib.calculateBudgetedModel(p, ds, cent, w)
        _libc.free(ct.cast(cent, ct.c_void_p))
        _libc.free(ct.cast(w, ct.c_void_p))
    finally:
        lib.freeDataset(ds)
    return Classifier(mdl)


def set_precision(mode):
    """Budgeted training's arithmetic for this process: "fp64" (the
    reference's, the default) or "mixed" (tensor-core SGMA scores and an
    IRWLS Gram from exact integer digit products on the tensor cores; same
    loops and random draws). Not part of the
    reference module."""
    modes = {"fp64": 0, "mixed": 1}
    if mode not in modes:
        raise ValueError("precision must be one of %s" % sorted(modes))
    _load_lib().irwls_set_precision(modes[mode])


def get_precision():
    return {0: "fp64", 1: "mixed"}[_load_lib().irwls_get_precision()]


def predict(classifier, data, labels=None, threads=1, Soft=0, verbose=1):
    """Decision values (Soft=1) or +-1 labels; prints the accuracy when labels
    are given (pythonmodule.c:72-128)."""
    lib = _load_lib()
    X, y = _arrays(data, labels)
    PD = C_double_p()
    ds = lib.irwls_dataset_from_dense(X.ctypes.data_as(PD), y.ctypes.data_as(PD), X.shape[0], X.shape[1])
    pp = _abi.make_predict_properties(labels=1 if labels is not None else 0, soft=Soft, threads=threads,
                                      verbose=verbose)
    try:
        f = lib.softTest if Soft else lib.test
        out = check(f(ds, _model_of(classifier), pp), "predict")
        res = np.ctypeslib.as_array(out, shape=(X.shape[0],)).copy()
        _libc.free(ct.cast(out, ct.c_void_p))
    finally:
        lib.freeDataset(ds)
    return res


def save(classifier, file):
    """Writes the model in the reference's binary format."""
    lib = _load_lib()
    fp = _libc.fopen(str(file).encode(), b"wb")
    if not fp:
        raise OSError("cannot open %s" % file)
    try:
        lib.storeModel(ct.byref(_model_of(classifier)), ct.c_void_p(fp))
    finally:
        _libc.fclose(ct.c_void_p(fp))


def load(file):
    """Reads a model written by save(), storeModel or the reference's CLIs."""
    lib = _load_lib()
    fp = _libc.fopen(str(file).encode(), b"rb")
    if not fp:
        raise OSError("Input file with the trained model not found: %s" % file)
    mdl = _abi.Model()
    try:
        lib.readModel(ct.byref(mdl), ct.c_void_p(fp))
    finally:
        _libc.fclose(ct.c_void_p(fp))
    return Classifier(mdl)


def C_double_p():
    return ct.POINTER(ct.c_double)
