"""CPU oracle (oracle/irwls_port.c) against the golden outputs of the
reference itself (tests/golden, made by tests/golden/make_golden.py from the
reference compiled from its own sources)."""
import platform

import numpy as np
import pytest

import harness as H

X86 = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("case", [c for c in H.FULL_CASES if c != "full_cfg1"])
def test_full_oracle_matches_reference(case):
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    beta, _, _ = H.run_full(H.port(), tr, p)
    ref = g["beta"]
    assert np.array_equal(beta[:-1] != 0, ref[:-1] != 0)
    assert H.rel_err(beta, ref) < H.REL_TOL
    if X86:  # same BLAS, same arithmetic order: bit-identical
        assert np.array_equal(beta, ref)


@pytest.mark.parametrize("case", [c for c in H.BUDGET_CASES if c != "budget_cfg2_reduced"])
def test_budget_oracle_matches_reference(case):
    g = H.golden(case)
    p = H.params(g)
    tr, _ = H.datasets(g)
    cent, w, _, _, _ = H.run_budget(H.port(), tr, p)
    assert np.array_equal(cent, g["centroids"])
    assert H.rel_err(w, g["weights"]) < H.REL_TOL
    if X86:
        assert np.array_equal(w, g["weights"])


@pytest.mark.parametrize("case", ["full_dense", "full_linear", "budget_sgma"])
def test_predict_oracle_matches_reference(case):
    import ctypes as C
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    port = H.port()
    if p["kind"] == "full":
        _, ptr, prop = H.run_full(port, tr, p)
        from libirwls_gb300 import _abi
        mdl = _build_full_model(prop, tr, ptr)
    else:
        cent, w, cptr, wptr, prop = H.run_budget(port, tr, p)
        mdl = _build_budget_model(prop, tr, cptr, wptr)
    soft = H.predict(port, te, mdl, 1)
    hard = H.predict(port, te, mdl, 0)
    assert H.rel_err(soft, g["soft"]) < H.REL_TOL
    assert np.array_equal(hard, g["hard"])


def _build_full_model(prop, tr, beta_ptr):
    from libirwls_gb300 import load
    return load().calculateFULLModel(prop, tr.struct, beta_ptr)


def _build_budget_model(prop, tr, cptr, wptr):
    from libirwls_gb300 import load
    return load().calculateBudgetedModel(prop, tr.struct, cptr, wptr)


def test_solver_oracle_matches_reference():
    import ctypes as C
    z = np.load(H.GOLDEN + "/solver.npz")
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    PD = C.POINTER(C.c_double)
    for k in keys:
        A = z[k + "_A"]
        b = z[k + "_b"]
        n = len(b)
        M = np.asfortranarray(A).ravel(order="F").copy()
        x = np.zeros(n)
        H.port().port_solve(M.ctypes.data_as(PD), n, b.ctypes.data_as(PD), x.ctypes.data_as(PD))
        assert H.rel_err(x, z[k + "_x"]) < 1e-12, k
        if X86:
            assert np.array_equal(x, z[k + "_x"]), k
