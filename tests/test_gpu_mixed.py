"""Precision form (irwls_set_precision(IRWLS_PRECISION_MIXED)) of budgeted and
full IRWLS.

SGMA: the candidate scores come from tensor-core products of three bf16
pieces per value (FP32 accuracy) on the Nystrom features Q = K_nm L^-T, with
the factor and its solves in FP64. Its scores differ from the FP64 form by
about 1e-7 relative, so it may pick a different centroid where two
candidates score within that margin; on the seeded reference cases below
every step's argmax agrees with the reference.

IRWLSpar: the Gram K1 = KC + A'^T A' is formed on the tensor cores from
exact integer digits of A' (48-bit fixed point per column, about 2^-45 of
the column scales per row) instead of FP64; the factor, solves, residual and
convergence test stay FP64. Its weights therefore differ from
the reference's by the solve's sensitivity to that rounding; the bar is the
objective the weights reach and the labels they predict."""
import numpy as np
import pytest

import harness as H
from libirwls_gb300 import load

pytestmark = pytest.mark.gpu

# Relative primal-objective difference allowed against the reference (the
# precision form's contract is 1e-4). Measured: 1e-12 and below on the RBF
# cases, 1.0e-7 on the rank-deficient linear-kernel case, 9e-7 on the
# 200000-row benchmark workload against the FP64 form.
PRIMAL_TOL = {"budget_linear": 1e-5}


@pytest.mark.parametrize("case", ["budget_sgma", "budget_sgma_dense", "budget_random", "budget_linear",
                                  "budget_cfg2_reduced"])
def test_mixed_budgeted_matches_reference(case):
    lib = load()
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    lib.irwls_set_precision(1)
    try:
        cent, w, cptr, wptr, prop = H.run_budget(lib, tr, p)
    finally:
        lib.irwls_set_precision(0)
    assert lib.irwls_tc_status() == 0
    assert np.array_equal(cent, g["centroids"])
    ref = H.budget_primal(tr, g["centroids"], g["weights"], p["gamma"], p["C"], p["kernel"])
    got = H.budget_primal(tr, cent, w, p["gamma"], p["C"], p["kernel"])
    print("%s: weights rel err %.3g, primal rel err %.3g" % (case, H.rel_err(w, g["weights"]),
                                                             abs(got - ref) / abs(ref)))
    assert abs(got - ref) <= PRIMAL_TOL.get(case, 1e-6) * abs(ref)
    mdl = lib.calculateBudgetedModel(prop, tr.struct, cptr, wptr)
    try:
        labels = H.predict(lib, te, mdl, 0)
    finally:
        lib.freeModel(mdl)
    agree = float((labels == g["hard"]).mean())
    assert agree >= 0.999


# Relative dual-objective difference allowed for full IRWLS (the precision
# form's contract is 1e-4).
DUAL_TOL = 1e-5


@pytest.mark.parametrize("case", H.FULL_CASES)
def test_mixed_full_matches_reference(case):
    lib = load()
    g = H.golden(case)
    p = H.params(g)
    tr, te = H.datasets(g)
    lib.irwls_set_precision(1)
    try:
        beta, ptr, prop = H.run_full(lib, tr, p)
    finally:
        lib.irwls_set_precision(0)
    assert lib.irwls_tc_status() == 0
    ref = H.dual_objective(tr, g["beta"], p["gamma"], p["kernel"])
    got = H.dual_objective(tr, beta, p["gamma"], p["kernel"])
    same_sv = np.array_equal(np.nonzero(beta[:-1])[0], np.nonzero(g["beta"][:-1])[0])
    print("%s: beta rel err %.3g, dual rel err %.3g, same SV set %s" % (case, H.rel_err(beta, g["beta"]),
                                                                      abs(got - ref) / abs(ref), same_sv))
    assert abs(got - ref) <= DUAL_TOL * abs(ref)
    mdl = lib.calculateFULLModel(prop, tr.struct, ptr)
    try:
        labels = H.predict(lib, te, mdl, 0)
    finally:
        lib.freeModel(mdl)
    assert float((labels == g["hard"]).mean()) >= 0.999
