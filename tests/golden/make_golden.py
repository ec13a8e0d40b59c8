"""Generates the golden fixtures of the parity tests by running the REFERENCE
LIBIRWLS itself (oracle/_ref/libirwls_ref.so, compiled from the reference's
own sources by ``make -C oracle ref``).

Run from the repository root, in a machine where the reference sources exist:

    make -C oracle ref && python tests/golden/make_golden.py

Each case stores its inputs (CSR arrays and labels), its parameters, and the
reference's outputs, so the fixtures do not depend on the generators' random
streams. The reference is run single-threaded (-t 1 semantics), with
srand(0) before full training (as its full-train CLI does) and srand(1)
before budgeted training (glibc's default seed, which its budgeted-train CLI
keeps). OpenBLAS runs single-threaded.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

# the reference links a single-threaded BLAS; keep OpenBLAS serial so the
# factorizations follow one fixed order
os.environ["OPENBLAS_NUM_THREADS"] = "1"
# the reference's library functions run their OpenMP loops at the default team
# size unless a CLI calls omp_set_num_threads; one thread is the -t 1 run
os.environ["OMP_NUM_THREADS"] = "1"

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from libirwls_gb300 import _abi, synth  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def gen(spec):
    kind, kw = spec
    if kind == "dense":
        X, y = synth.two_gaussians(kw["n"], kw["d"], kw["seed"])
        return synth.from_dense(X, y, keep_zeros=True)
    if kind == "onehot":
        return synth.mixed_onehot(kw["n"], kw["seed"])
    raise ValueError(kind)


CASES = {
    # full IRWLS
    "full_dense": dict(kind="full", train=("dense", dict(n=600, d=8, seed=11)),
                       test=("dense", dict(n=200, d=8, seed=12)), gamma=0.05, C=10.0, w=100, kernel=1),
    "full_sparse": dict(kind="full", train=("onehot", dict(n=1500, seed=13)),
                        test=("onehot", dict(n=300, seed=14)), gamma=0.1, C=10.0, w=150, kernel=1),
    "full_linear": dict(kind="full", train=("dense", dict(n=400, d=6, seed=15)),
                        test=("dense", dict(n=100, d=6, seed=16)), gamma=1.0, C=1.0, w=80, kernel=0),
    "full_smallws": dict(kind="full", train=("dense", dict(n=300, d=5, seed=17)),
                         test=("dense", dict(n=50, d=5, seed=18)), gamma=0.5, C=1.0, w=7, kernel=1),
    # the dense full-IRWLS workload at its full size
    "full_cfg1": dict(kind="full", train=("dense", dict(n=4000, d=20, seed=20240601)),
                      test=("dense", dict(n=1000, d=20, seed=20240611)), gamma=0.05, C=10.0, w=500, kernel=1),
    # budgeted IRWLS
    "budget_sgma": dict(kind="budget", train=("onehot", dict(n=3000, seed=21)),
                        test=("onehot", dict(n=500, seed=22)), gamma=0.1, C=100.0, size=40, algorithm=1, kernel=1),
    "budget_sgma_dense": dict(kind="budget", train=("dense", dict(n=1200, d=8, seed=23)),
                              test=("dense", dict(n=200, d=8, seed=24)), gamma=0.2, C=10.0, size=30, algorithm=1, kernel=1),
    "budget_random": dict(kind="budget", train=("onehot", dict(n=2000, seed=25)),
                          test=("onehot", dict(n=300, seed=26)), gamma=0.1, C=10.0, size=50, algorithm=0, kernel=1),
    "budget_linear": dict(kind="budget", train=("dense", dict(n=800, d=6, seed=27)),
                          test=("dense", dict(n=100, d=6, seed=28)), gamma=1.0, C=1.0, size=12, algorithm=1, kernel=0),
    # the budgeted workload at a tenth of its rows and budget
    "budget_cfg2_reduced": dict(kind="budget", train=("onehot", dict(n=20000, seed=20240602)),
                                test=("onehot", dict(n=2000, seed=20240612)), gamma=0.1, C=100.0, size=100,
                                algorithm=1, kernel=1),
}


def arr(ptr, n, dtype=np.float64):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype).copy()


def run_case(ref, libc, name, cfg):
    tr = gen(cfg["train"])
    te = gen(cfg["test"])
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    out = dict(train_indptr=tr.indptr, train_indices=tr.indices, train_values=tr.values, train_y=tr.y,
               test_indptr=te.indptr, test_indices=te.indices, test_values=te.values, test_y=te.y)
    if cfg["kind"] == "full":
        p = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], kernel=cfg["kernel"], working_set=cfg["w"])
        ref.initMemory(1, cfg["w"] + 1)
        libc.srand(0)
        b = ref.trainFULL(hd.struct, p)
        beta = arr(b, hd.l + 1)
        mdl = ref.calculateFULLModel(p, hd.struct, b)
        out["beta"] = beta
    else:
        p = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], kernel=cfg["kernel"], size=cfg["size"],
                                 algorithm=cfg["algorithm"])
        ref.initMemory(1, cfg["size"])
        libc.srand(1)
        c = ref.SGMA(hd.struct, p) if cfg["algorithm"] == 1 else ref.randomCentroids(hd.struct, p)
        w = ref.IRWLSpar(hd.struct, c, p)
        out["centroids"] = arr(c, cfg["size"], np.int32)
        out["weights"] = arr(w, cfg["size"])
        mdl = ref.calculateBudgetedModel(p, hd.struct, c, w)
    pp = _abi.make_predict_properties(labels=0, soft=1)
    out["soft"] = arr(ref.softTest(ht.struct, mdl, pp), ht.l)
    pp.Soft = 0
    out["hard"] = arr(ref.test(ht.struct, mdl, pp), ht.l)
    # model file bytes as written by the reference's storeModel
    fd, path = tempfile.mkstemp()
    os.close(fd)
    fp = libc.fopen(path.encode(), b"wb")
    ref.storeModel(C.byref(mdl), C.c_void_p(fp))
    libc.fclose(C.c_void_p(fp))
    out["model_bytes"] = np.frombuffer(open(path, "rb").read(), dtype=np.uint8)
    os.unlink(path)
    out["params"] = np.array(json.dumps({k: v for k, v in cfg.items()}))
    return out


def reader_case(ref, name, data, labeled):
    fd, path = tempfile.mkstemp(suffix=".libsvm")
    os.close(fd)
    synth.write_libsvm(path, data, labeled=labeled)
    d = ref.readTrainFile(path.encode()) if labeled else ref.readUnlabeledFile(path.encode())
    n = d.l + 2 if labeled else d.l
    rows, y, q = _abi.dataset_rows(d, n)
    text = open(path, "rb").read()
    os.unlink(path)
    lens = np.array([len(r[0]) for r in rows])
    return dict(text=np.frombuffer(text, dtype=np.uint8), l=d.l, sparse=d.sparse, maxdim=d.maxdim,
                lens=lens, idx=np.concatenate([r[0] for r in rows]) if lens.sum() else np.zeros(0, np.int32),
                val=np.concatenate([r[1] for r in rows]) if lens.sum() else np.zeros(0), y=y, q=q)


def solver_cases(ref):
    """ParallelLinearSystem with one thread on SPD and on bordered systems."""
    rng = np.random.default_rng(31)
    ref.initMemory(1, 256)
    out = {}
    for n, bordered in [(5, False), (37, False), (64, False), (200, False), (9, True), (51, True), (251, True)]:
        if bordered:
            m = n - 1
            X = rng.standard_normal((m, 4))
            K = np.exp(-0.3 * ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
            yv = np.where(rng.random(m) < 0.5, 1.0, -1.0)
            H = np.zeros((n, n))
            H[:m, :m] = K * np.outer(yv, yv) + np.diag(1.0 / (rng.random(m) * 5 + 0.01))
            H[:m, m] = yv
            H[m, :m] = yv
        else:
            A = rng.standard_normal((n, n))
            H = A @ A.T + n * np.eye(n)
        b = rng.standard_normal(n)
        M = np.asfortranarray(H.copy())
        Mf = M.ravel(order="F").copy()
        x = np.zeros(n)
        PD = C.POINTER(C.c_double)
        ref.ParallelLinearSystem(Mf.ctypes.data_as(PD), n, n, 0, 0, b.ctypes.data_as(PD), n, 1, 0, 0, n, 1,
                                 x.ctypes.data_as(PD), n, 1, 0, 0, 1)
        key = "solve_%d_%s" % (n, "bordered" if bordered else "spd")
        out[key + "_A"] = H
        out[key + "_b"] = b
        out[key + "_x"] = x
        out[key + "_L"] = Mf.reshape((n, n), order="F")
    return out


def main():
    ref_path = os.path.join(ROOT, "oracle", "_ref", "libirwls_ref.so")
    ref = _abi.load_library(ref_path)
    ref.storeModel.argtypes = [C.POINTER(_abi.Model), C.c_void_p]
    ref.storeModel.restype = None
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    only = set(sys.argv[1:])
    for name, cfg in CASES.items():
        if only and name not in only:
            continue
        out = run_case(ref, libc, name, cfg)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
        print("wrote", name, flush=True)
    if not only or "reader" in only:
        rd = {}
        for key, data, labeled in [
            ("dense", gen(("dense", dict(n=40, d=5, seed=41))), True),
            ("onehot", gen(("onehot", dict(n=60, seed=42))), True),
            ("unlabeled", gen(("onehot", dict(n=30, seed=43))), False),
        ]:
            for k, v in reader_case(ref, key, data, labeled).items():
                rd[key + "_" + k] = v
        np.savez_compressed(os.path.join(OUT, "reader.npz"), **rd)
        print("wrote reader", flush=True)
    if not only or "solver" in only:
        np.savez_compressed(os.path.join(OUT, "solver.npz"), **solver_cases(ref))
        print("wrote solver", flush=True)


if __name__ == "__main__":
    main()
