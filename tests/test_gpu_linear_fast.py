"""Linear-kernel prediction fast path (irwls_set_linear_fast_path): a
kernelType-0 model predicts through W = sum_j w_j sv_j. Off by default; when
on, the decision values equal the reference's (golden full_linear and
budget_linear cases) up to summation order -- within 1e-10 of max |f| -- and
the labels agree wherever |f| is above that; on a larger sparse model the
same holds against the kernel-sum path."""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load, synth

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
TOL = 1e-10


def _model(lib, case):
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    if p["kind"] == "full":
        b = np.ascontiguousarray(g["beta"])
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"])
        mdl = lib.calculateFULLModel(prop, tr.struct, b.ctypes.data_as(PD))
    else:
        c = np.ascontiguousarray(g["centroids"].astype(np.int32))
        w = np.ascontiguousarray(g["weights"])
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=p["size"])
        mdl = lib.calculateBudgetedModel(prop, tr.struct, c.ctypes.data_as(PI), w.ctypes.data_as(PD))
    return g, te, mdl, (tr, b if p["kind"] == "full" else (c, w))


def _both(lib, te, mdl):
    lib.irwls_set_linear_fast_path(0)
    soft0, hard0 = H.predict(lib, te, mdl, 1), H.predict(lib, te, mdl, 0)
    lib.irwls_set_linear_fast_path(1)
    try:
        soft1, hard1 = H.predict(lib, te, mdl, 1), H.predict(lib, te, mdl, 0)
    finally:
        lib.irwls_set_linear_fast_path(0)
    return soft0, hard0, soft1, hard1


def _agree(soft, hard, ref_soft, ref_hard):
    scale = np.abs(ref_soft).max()
    assert np.abs(soft - ref_soft).max() <= TOL * scale
    clear = np.abs(ref_soft) > TOL * scale
    assert np.array_equal(hard[clear], ref_hard[clear])


def test_fast_path_is_off_by_default():
    assert load().irwls_get_linear_fast_path() == 0


@pytest.mark.parametrize("case", ["full_linear", "budget_linear"])
def test_fast_path_matches_reference_predictions(case):
    lib = load()
    g, te, mdl, _ = _model(lib, case)
    soft0, hard0, soft1, hard1 = _both(lib, te, mdl)
    assert H.rel_err(soft0, g["soft"]) < 1e-12  # the kernel-sum path, as pinned elsewhere
    _agree(soft1, hard1, g["soft"], g["hard"])


def test_fast_path_on_a_large_sparse_model():
    lib = load()
    d = synth.sparse_linear_pool(6000, seed=5)
    tr = _abi.build_dataset(d.indptr[:4001], d.indices[:d.indptr[4000]], d.values[:d.indptr[4000]], d.y[:4000])
    n0 = d.indptr[4000]
    te = _abi.build_dataset(d.indptr[4000:] - n0, d.indices[n0:], d.values[n0:], d.y[4000:])
    rng = np.random.default_rng(2)
    beta = np.where(rng.random(4001) < 0.6, rng.standard_normal(4001), 0.0)
    beta[-1] = 0.3
    prop = _abi.make_properties(gamma=1.0, C_=1.0, kernel=0)
    mdl = lib.calculateFULLModel(prop, tr.struct, np.ascontiguousarray(beta).ctypes.data_as(PD))
    soft0, hard0, soft1, hard1 = _both(lib, te, mdl)
    _agree(soft1, hard1, soft0, hard0)
