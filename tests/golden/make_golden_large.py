"""Generates the golden fixtures of the two benchmark workloads at their full
sizes by running the REFERENCE LIBIRWLS itself (oracle/_ref/libirwls_ref.so,
compiled from the reference's own sources by ``make -C oracle ref``),
single-threaded (-t 1 semantics, OpenBLAS serial):

- ``budget_cfg2_full``: budgeted IRWLS (SGMA + IRWLSpar), 200000 rows, d = 54
  (10 N(0,1) + one-hot 4 + one-hot 40), RBF gamma = 0.1, C = 100, budget
  m = 1000, srand(1) as the budgeted-train CLI leaves it; prediction of a
  20000-row held-out set labelled by the same network;
- ``full_cfg3``: full IRWLS, 100000 rows x 784 features (8-bit values / 255,
  19 % nonzero, ten seeded prototypes, 0-4 against 5-9), RBF gamma = 0.02,
  C = 10, working set 500, srand(0) as the full-train CLI seeds it; prediction
  of a 10000-row held-out set.

The inputs are far too large to commit, so each fixture stores the
generator's seeds and a SHA-256 digest of the dataset as the library sees it
(``synth.dataset_digest``), plus the reference's outputs: centroids and
weights, or the support-vector indices, their weights and the bias; the
decision values and labels of the held-out set; the training time.

Run from the repository root where the reference sources exist (a -t 1
training of the budgeted workload takes about two hours of one core):

    make -C oracle ref REF=<reference checkout> && \
        python tests/golden/make_golden_large.py budget_cfg2_full full_cfg3

``--lib port`` runs the CPU restatement (oracle/_build/libirwls_port.so)
instead, with its SGMA candidate loop on all cores (its candidate draws keep
the one-thread order, so its centroids are the -t 1 reference's) and
everything else single-threaded; that output goes to a path given by
``--out`` and serves to cross-check the restatement at full size.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

os.environ["OPENBLAS_NUM_THREADS"] = "1"

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from libirwls_gb300 import _abi, synth  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")

CASES = {
    "budget_cfg2_full": dict(kind="budget", n=200_000, n_test=20_000, seed=20240602, test_seed=20240604,
                             label_seed=20240603, gamma=0.1, C=100.0, size=1000, algorithm=1, kernel=1),
    "full_cfg3": dict(kind="full", n=100_000, n_test=10_000, seed=20240606, gamma=0.02, C=10.0, w=500, kernel=1),
}


def datasets(cfg):
    """The case's training and held-out sets, rebuilt from its seeds."""
    if cfg["kind"] == "budget":
        tr = synth.budgeted_workload(cfg["n"], seed=cfg["seed"], label_seed=cfg["label_seed"])
        te = synth.budgeted_test_set(cfg["n_test"], seed=cfg["test_seed"], label_seed=cfg["label_seed"])
    else:
        tr, te = synth.precision_full_workload(cfg["n"], cfg["n_test"], seed=cfg["seed"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    return hd, ht


def arr(ptr, n, dtype=np.float64):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype).copy()


def packer(lib):
    """The library whose calculate*Model packs the model: the reference's own,
    or, for the restatement (which has none), this repository's host C
    packing, which writes the same model bytes."""
    try:
        lib.calculateFULLModel
        return lib
    except AttributeError:
        return _abi.load_library(os.path.join(ROOT, "libirwls_gb300", "libirwls_gb300.so"))


def run_case(lib, libc, cfg, sgma_threads=1):
    hd, ht = datasets(cfg)
    out = dict(train_digest=np.array(synth.dataset_digest(hd)), test_digest=np.array(synth.dataset_digest(ht)))
    t0 = time.perf_counter()
    if cfg["kind"] == "full":
        p = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], kernel=cfg["kernel"], working_set=cfg["w"])
        lib.initMemory(1, cfg["w"] + 1)
        libc.srand(0)
        b = lib.trainFULL(hd.struct, p)
        out["train_seconds"] = np.array(time.perf_counter() - t0)
        beta = arr(b, hd.l + 1)
        sv = np.nonzero(beta[:hd.l])[0].astype(np.int32)
        out["sv"] = sv
        out["beta_sv"] = beta[sv]
        out["bias"] = np.array(beta[hd.l])
        mdl = packer(lib).calculateFULLModel(p, hd.struct, b)
    else:
        p = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], kernel=cfg["kernel"], size=cfg["size"],
                                 algorithm=cfg["algorithm"], threads=sgma_threads)
        lib.initMemory(1, cfg["size"])
        libc.srand(1)
        c = lib.SGMA(hd.struct, p) if cfg["algorithm"] == 1 else lib.randomCentroids(hd.struct, p)
        out["sgma_seconds"] = np.array(time.perf_counter() - t0)
        p.Threads = 1
        w = lib.IRWLSpar(hd.struct, c, p)
        out["train_seconds"] = np.array(time.perf_counter() - t0)
        out["centroids"] = arr(c, cfg["size"], np.int32)
        out["weights"] = arr(w, cfg["size"])
        mdl = packer(lib).calculateBudgetedModel(p, hd.struct, c, w)
    pp = _abi.make_predict_properties(labels=0, soft=1)
    out["soft"] = arr(lib.softTest(ht.struct, mdl, pp), ht.l)
    pp.Soft = 0
    out["hard"] = arr(lib.test(ht.struct, mdl, pp), ht.l).astype(np.int8)
    out["params"] = np.array(json.dumps(cfg))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cases", nargs="+", choices=sorted(CASES))
    ap.add_argument("--lib", choices=["ref", "port"], default="ref")
    ap.add_argument("--out", default=None, help="output folder (default: tests/golden; required with --lib port)")
    a = ap.parse_args()
    if a.lib == "ref":
        # the reference's library functions run OpenMP loops at the default
        # team size unless its CLI called omp_set_num_threads; one thread
        # gives the -t 1 run (libgomp reads this when the library loads)
        os.environ["OMP_NUM_THREADS"] = "1"
    if a.lib == "port" and not a.out:
        ap.error("--lib port writes cross-check files only: give --out")
    path = os.path.join(ROOT, "oracle", "_ref", "libirwls_ref.so") if a.lib == "ref" else \
        os.path.join(ROOT, "oracle", "_build", "libirwls_port.so")
    lib = _abi.load_library(path)
    libc = C.CDLL(None)
    threads = (os.cpu_count() or 1) if a.lib == "port" else 1
    for name in a.cases:
        out = run_case(lib, libc, CASES[name], sgma_threads=threads)
        out["generator"] = np.array(a.lib)
        np.savez_compressed(os.path.join(a.out or OUT, name + ".npz"), **out)
        print("wrote %s (%.1f s training)" % (name, float(out["train_seconds"])), flush=True)


if __name__ == "__main__":
    main()
