"""The full-size fixtures (tests/golden/make_golden_large.py) on the CPU: the
seeded generators rebuild exactly the datasets the reference trained on
(SHA-256 of every number the training reads), and the fixtures are the
reference's own outputs, not the restatement's."""
import json
import os

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, synth


def _fixture(name):
    path = os.path.join(H.GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    z = np.load(path, allow_pickle=False)
    return {k: z[k] for k in z.files}


def test_full_cfg3_fixture_inputs_rebuild():
    g = _fixture("full_cfg3")
    assert str(g["generator"]) == "ref"
    cfg = json.loads(str(g["params"]))
    tr, te = synth.precision_full_workload(cfg["n"], cfg["n_test"], seed=cfg["seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    assert synth.dataset_digest(hd) == str(g["train_digest"])
    assert synth.dataset_digest(ht) == str(g["test_digest"])
    assert np.all(g["beta_sv"] != 0) and np.all(np.diff(g["sv"]) > 0)
    assert set(np.unique(g["hard"])) <= {-1, 1}


def test_budget_cfg2_fixture_inputs_rebuild():
    g = _fixture("budget_cfg2_full")
    assert str(g["generator"]) == "ref"
    cfg = json.loads(str(g["params"]))
    tr = synth.budgeted_workload(cfg["n"], seed=cfg["seed"], label_seed=cfg["label_seed"])
    te = synth.budgeted_test_set(cfg["n_test"], seed=cfg["test_seed"], label_seed=cfg["label_seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    assert synth.dataset_digest(hd) == str(g["train_digest"])
    assert synth.dataset_digest(ht) == str(g["test_digest"])
    assert len(np.unique(g["centroids"])) == cfg["size"]
    assert set(g["centroids"][:2].tolist()) == {cfg["n"], cfg["n"] + 1}  # the class-mean rows come first
