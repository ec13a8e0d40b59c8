"""Parity of the plain FP64 GPU form with the reference at the benchmark
workloads' full sizes (fixtures written by tests/golden/make_golden_large.py
from the reference itself, run with -t 1):

- full IRWLS, 100000 rows x 784 features (8-bit values / 255, 19 % nonzero),
  RBF gamma 0.02, C 10, working set 500: the reference's support-vector set,
  weights and bias within 1e-9 of the largest weight, the dual objective
  within 1e-9, identical labels and decision values within 1e-9 on the
  10000-row held-out set; the precision form within its contract (dual 1e-4,
  labels 99.9 %);
- budgeted IRWLS, 200000 rows x 54 features, RBF gamma 0.1, C 100, budget
  1000: the reference's 1000 centroids, weights within the measured
  thread-partition bar, identical labels on the 20000-row held-out set.

The inputs are rebuilt from the generators' seeds; their SHA-256 digests
must equal the fixtures' (so both machines train on the same numbers)."""
import json
import os

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load, synth

pytestmark = pytest.mark.gpu


def _fixture(name):
    path = os.path.join(H.GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    z = np.load(path, allow_pickle=False)
    return {k: z[k] for k in z.files}


def _full_sets(cfg):
    tr, te = synth.precision_full_workload(cfg["n"], cfg["n_test"], seed=cfg["seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    return tr, hd, ht


def _dual(tr, beta, gamma):
    """D(beta) = sum_i y_i beta_i - 1/2 beta^T K beta (RBF) in FP64 on the
    host, from the CSR rows of the support vectors."""
    sv = np.nonzero(beta[:tr.n])[0]
    Xs = np.zeros((len(sv), tr.d + 1))
    for k, i in enumerate(sv):
        a, b = tr.indptr[i], tr.indptr[i + 1]
        Xs[k, tr.indices[a:b]] = tr.values[a:b]
    sq = (Xs * Xs).sum(1)
    K = np.exp(-gamma * np.maximum(sq[:, None] + sq[None, :] - 2 * Xs @ Xs.T, 0.0))
    bs = beta[sv]
    return float((tr.y[sv] * bs).sum() - 0.5 * bs @ K @ bs)


@pytest.fixture(scope="module")
def cfg3():
    g = _fixture("full_cfg3")
    cfg = json.loads(str(g["params"]))
    tr, hd, ht = _full_sets(cfg)
    assert synth.dataset_digest(hd) == str(g["train_digest"]), "training set differs from the fixture's"
    assert synth.dataset_digest(ht) == str(g["test_digest"]), "held-out set differs from the fixture's"
    beta = np.zeros(hd.l + 1)
    beta[g["sv"]] = g["beta_sv"]
    beta[hd.l] = g["bias"]
    return g, cfg, tr, hd, ht, beta


def _train(lib, hd, cfg, precision):
    p = {"gamma": cfg["gamma"], "C": cfg["C"], "w": cfg["w"], "kernel": cfg["kernel"]}
    lib.irwls_set_precision(precision)
    try:
        return H.run_full(lib, hd, p)
    finally:
        lib.irwls_set_precision(0)


def test_full_cfg3_plain_matches_reference(cfg3):
    g, cfg, tr, hd, ht, ref = cfg3
    lib = load()
    beta, ptr, prop = _train(lib, hd, cfg, 0)
    assert np.array_equal(np.nonzero(beta[:-1])[0], g["sv"]), "support-vector sets differ"
    err = H.rel_err(beta, ref)
    d_ref = _dual(tr, ref, cfg["gamma"])
    d_got = _dual(tr, beta, cfg["gamma"])
    print("cfg3 plain: %d SVs, beta rel err %.3g, dual rel err %.3g" % (len(g["sv"]), err,
                                                                      abs(d_got - d_ref) / abs(d_ref)))
    assert err <= H.REL_TOL
    assert abs(d_got - d_ref) <= 1e-9 * abs(d_ref)
    mdl = lib.calculateFULLModel(prop, hd.struct, ptr)
    try:
        soft = H.predict(lib, ht, mdl, 1)
        hard = H.predict(lib, ht, mdl, 0)
    finally:
        lib.freeModel(mdl)
    assert np.array_equal(hard, g["hard"].astype(np.float64))
    assert H.rel_err(soft, g["soft"]) <= H.REL_TOL


def test_full_cfg3_precision_meets_its_contract(cfg3):
    g, cfg, tr, hd, ht, ref = cfg3
    lib = load()
    beta, ptr, prop = _train(lib, hd, cfg, 1)
    assert lib.irwls_tc_status() == 0
    d_ref = _dual(tr, ref, cfg["gamma"])
    d_got = _dual(tr, beta, cfg["gamma"])
    sv = np.nonzero(beta[:-1])[0]
    print("cfg3 precision: %d SVs (reference %d, %d shared), pieces %d, dual rel err %.3g"
          % (len(sv), len(g["sv"]), len(np.intersect1d(sv, g["sv"])), lib.irwls_last_tc_pieces(),
             abs(d_got - d_ref) / abs(d_ref)))
    assert abs(d_got - d_ref) <= 1e-4 * abs(d_ref)
    mdl = lib.calculateFULLModel(prop, hd.struct, ptr)
    try:
        hard = H.predict(lib, ht, mdl, 0)
    finally:
        lib.freeModel(mdl)
    assert float((hard == g["hard"]).mean()) >= 0.999


def test_budget_cfg2_full_plain_matches_reference():
    g = _fixture("budget_cfg2_full")
    cfg = json.loads(str(g["params"]))
    tr = synth.budgeted_workload(cfg["n"], seed=cfg["seed"], label_seed=cfg["label_seed"])
    te = synth.budgeted_test_set(cfg["n_test"], seed=cfg["test_seed"], label_seed=cfg["label_seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    assert synth.dataset_digest(hd) == str(g["train_digest"]), "training set differs from the fixture's"
    assert synth.dataset_digest(ht) == str(g["test_digest"]), "held-out set differs from the fixture's"
    lib = load()
    p = {"gamma": cfg["gamma"], "C": cfg["C"], "size": cfg["size"], "algorithm": cfg["algorithm"],
         "kernel": cfg["kernel"]}
    cent, w, cptr, wptr, prop = H.run_budget(lib, hd, p)
    assert np.array_equal(cent, g["centroids"]), "%d of %d centroids differ" % (
        int((cent != g["centroids"]).sum()), len(cent))
    err = H.rel_err(w, g["weights"])
    print("cfg2 plain: weights rel err %.3g" % err)
    # the 20000-row reduction of this workload moves by 1.5e-9 between the
    # reference's own 1- and multi-thread runs; the bar is that order
    assert err <= BUDGET_CFG2_TOL
    mdl = lib.calculateBudgetedModel(prop, hd.struct, cptr, wptr)
    try:
        soft = H.predict(lib, ht, mdl, 1)
        hard = H.predict(lib, ht, mdl, 0)
    finally:
        lib.freeModel(mdl)
    assert np.array_equal(hard, g["hard"].astype(np.float64))
    assert H.rel_err(soft, g["soft"]) <= BUDGET_CFG2_TOL


BUDGET_CFG2_TOL = 1e-8


def test_budget_cfg2_full_precision_meets_its_contract():
    """The precision form on the same 200000-row workload, against the
    reference's run: its 1000 centroids (the tensor-core scores rank the
    candidates as the FP64 ones do here), the budgeted primal objective
    1/2 w^T (K_mm + 1e-5 I) w + C sum_i max(0, 1 - y_i f_i) within 1e-4
    relative (the model has no dual; the IRWLSpar system's condition number
    is about 1e13, so equally good weight vectors differ by far more than the
    objective does) and at least 99.9 % of its held-out labels."""
    g = _fixture("budget_cfg2_full")
    cfg = json.loads(str(g["params"]))
    tr = synth.budgeted_workload(cfg["n"], seed=cfg["seed"], label_seed=cfg["label_seed"])
    te = synth.budgeted_test_set(cfg["n_test"], seed=cfg["test_seed"], label_seed=cfg["label_seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    lib = load()
    p = {"gamma": cfg["gamma"], "C": cfg["C"], "size": cfg["size"], "algorithm": cfg["algorithm"],
         "kernel": cfg["kernel"]}
    lib.irwls_set_precision(1)
    try:
        cent, w, cptr, wptr, prop = H.run_budget(lib, hd, p)
    finally:
        lib.irwls_set_precision(0)
    assert lib.irwls_tc_status() == 0
    assert np.array_equal(cent, g["centroids"]), "%d of %d centroids differ" % (
        int((cent != g["centroids"]).sum()), len(cent))
    mdl = lib.calculateBudgetedModel(prop, hd.struct, cptr, wptr)
    try:
        soft = H.predict(lib, ht, mdl, 1)
        hard = H.predict(lib, ht, mdl, 0)
    finally:
        lib.freeModel(mdl)
    agree = float((hard == g["hard"].astype(np.float64)).mean())
    p_ref = H.budget_primal(hd, g["centroids"], g["weights"], cfg["gamma"], cfg["C"], cfg["kernel"])
    p_got = H.budget_primal(hd, cent, w, cfg["gamma"], cfg["C"], cfg["kernel"])
    print("cfg2 precision: primal rel err %.3g, weights rel err %.3g, decision values rel err %.3g, labels %.5f"
          % (abs(p_got - p_ref) / abs(p_ref), H.rel_err(w, g["weights"]), H.rel_err(soft, g["soft"]), agree))
    assert abs(p_got - p_ref) <= 1e-4 * abs(p_ref)
    assert agree >= 0.999
