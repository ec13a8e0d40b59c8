#!/usr/bin/env python
"""Benchmark of the budgeted-IRWLS training path (SGMA centroid selection +
IRWLS weighted least squares) on one GB300.

Workload: n = 200,000 rows, d = 54 (10 N(0,1) features + one-hot groups of 4
and 40; labels from a seeded random 2-layer tanh network with 5% flipped;
seeded synthetic data, since the reference's public demo set is not available
offline), RBF gamma = 0.1, C = 100, budget m = 1000, 64 candidates per SGMA
step (the count the reference hard-codes).

One step = one complete training (SGMA + IRWLSpar) of that workload. Both
forms are timed in the same run, on the same resident dataset:
  plain FP64 : the reference's arithmetic, the form the parity tests pin;
  precision  : SGMA scores on the tensor cores from three bf16 pieces of Q
               and W (exactly their FP32 values), IRWLSpar's Gram from
               exact integer digit products on the tensor cores,
               factors/solves/residuals in FP64.
  value : train seconds per step of the precision form when it meets the
          accuracy bars against the plain run of the same job (the budgeted
          model has no bias and no dual, so its objective bar is the relative
          difference of the primal 1/2 w^T K_mm w + C sum hinge <= 1e-4; held-
          out accuracy change <= 0.1%), else of the plain form; dataset
          resident on the GPU, CUDA events on the library's stream, L2
          flushed between steps. The plain form, the denominator of the
          speed-up, takes 16 s per training: it is timed on min(K, 3) steps
          after one warm-up.
  e2e   : the same form through the reference-facing C ABI (SGMA() +
          IRWLSpar() on the host svm_dataset), host-to-device copies of the
          dataset and device-to-host copies of the results included.
  roofline: the dominant kernel of that form. Precision form: the tensor-core
          Gram, its algorithmic work n_act (m + 1) m flops per IRWLSpar
          iteration (the FP64 SYRK it replaces) against the measured
          sustained bf16 peak; the rate of its bf16 digit-pair products is a
          separate field. Plain form: the FP64 SGMA GEMM against a live FP64
          probe.
  kernels : the other measured kernel rooflines of both forms.
  cpu_baseline: one complete training of the workload (SGMA to m = 1000,
          IRWLSpar to convergence) by the CPU restatement of the reference
          (oracle/irwls_port.c: reference arithmetic, OpenMP loops and
          BLAS/LAPACK calls) on all host cores, measured, not extrapolated;
          its centroids are compared with the plain GPU form's.
  full784 : the full-IRWLS workload of the precision form (below), both forms
          with their accuracy bars, timed in the same run.

`--form plain|mixed` times one form only (no accuracy comparison).
`--workload full` measures the dense full-IRWLS workload instead (n = 4000
train rows, d = 20, two Gaussian classes with 10% flipped labels, RBF gamma =
0.05, C = 10, working set 500), `--workload full784` the full-IRWLS workload
of the precision form (n = 100000, d = 784 8-bit values at 19% density from
10 prototypes, RBF gamma = 0.02, C = 10); both time the two forms with the
same bars (dual objective instead of primal); their CPU baseline is the
restatement's whole training on all host cores, measured on the whole
workload.

`--workload batch` measures the batching form: 72 SVMs (a C x gamma grid of
RBF SVMs plus linear ones) on subsets of 2000-50000 rows trained concurrently
(worker count from the library's autotuner) against the same SVMs trained one
at a time; every SVM's weights must be bitwise identical in both.

`--workload learned` measures the learned-proposal form: a network trained on
traces of random-candidate SGMA on 20 small sets proposes SGMA candidates on
a 1M-row set (budget 2000 by default, --budget to change), against random
candidates; it reports train seconds, the Nystrom residual of both, the
primal objective and the held-out accuracy.

`--impl reference` times complete CPU trainings of the same workload (the
reference sources are not present on the GPU host, so the restatement, pinned
bit for bit to the reference, stands in for it) and prints its line with
"impl": "reference". One training of the budgeted workload takes minutes on
the host cores, so the arm times as many complete trainings as fit in about
four minutes (at least one) instead of K, and says how many in "steps"; no
sample is ever scaled up.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "train s at ≤1e-4 rel dual-obj err: mixed/batched/learned vs plain FP64 GPU IRWLS"
N_ROWS, BUDGET, GAMMA, COST, SEED = 200_000, 1000, 0.1, 100.0, 20240602
# wall-clock budget of the reference arm's complete CPU trainings (at least one runs)
REF_ARM_BUDGET_S = 240.0
# the plain FP64 form (16 s per training of the budgeted workload) is timed on
# at most this many steps after one warm-up
PLAIN_STEPS = 3

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rows", type=int, default=N_ROWS)
    ap.add_argument("--budget", type=int, default=BUDGET)
    ap.add_argument("--parse-rows", type=int, default=None,
                    help="rows of the parse workload's file (default 1000000; smaller only for profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end measurement")
    ap.add_argument("--no-full784", dest="with_full784", action="store_false",
                    help="leave the full-IRWLS 100000 x 784 workload out of the default line")
    ap.add_argument("--workload", default="budgeted", choices=["budgeted", "full", "full784", "batch", "learned", "linear_predict", "parse", "model_io"])
    ap.add_argument("--form", default="both", choices=["both", "plain", "mixed"],
                    help="forms to time: both (headline = precision form if it meets the accuracy bars), "
                         "or only one of them")
    return ap.parse_args()


# One score launch at order s on the budgeted workload: Q's three bf16 pieces
# of the s columns rounded up to a 32-column block (6 B per entry), the 64
# residuals of every row (4 B each) and the rows' FP32 CSR (value and index,
# 8 B per stored entry, plus the row pointer and norm, 8 B per row).
def score_launch_bytes(rows, s, hd):
    nnz = len(hd.features) - hd.l
    return rows * (-(-s // 32) * 32) * 6 + rows * 64 * 4 + nnz * 8 + rows * 8


# The score kernel's 501st launch on the 200000-row workload (order 502), one
# ncu pass: dram bytes read + written, and its duration (ms).
SCORE_TRAFFIC_502 = 635705088 + 42572544
SCORE_MS_502 = 0.120


def workload(rows):
    from libirwls_gb300 import _abi, synth

    data = synth.budgeted_workload(rows, seed=SEED)
    hd = _abi.build_dataset(data.indptr, data.indices, data.values, data.y)
    return hd


def props(budget, algorithm=1, threads=1):
    from libirwls_gb300 import _abi

    return _abi.make_properties(gamma=GAMMA, C_=COST, size=budget, algorithm=algorithm, threads=threads)


def config(args, extra=None):
    c = {
        "workload": "budgeted IRWLS (SGMA + weighted LS): n=%d, d=54 (10 N(0,1) + one-hot 4 + one-hot 40), "
                    "RBF gamma=0.1, C=100, budget m=%d, 64 candidates per SGMA step" % (args.rows, args.budget),
        "n": args.rows, "d": 54, "gamma": GAMMA, "C": COST, "budget": args.budget, "candidates_per_step": 64,
        "form": "plain FP64", "parallelism": "replicas" if args.gpus > 1 else "single GPU",
        "l2": "flushed between timed steps (512 MiB overwrite); K_nm alone is %.1f GB"
              % (args.rows * args.budget * 8 / 1e9),
    }
    if extra:
        c.update(extra)
    return c


# ----------------------------------------------------------------------------
# CPU baseline: complete trainings by the restatement of the reference
# ----------------------------------------------------------------------------

def load_port():
    """The CPU restatement of the reference (test and benchmark
    infrastructure: the CPU baseline only)."""
    from libirwls_gb300 import _abi

    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    port_path = os.path.join(ROOT, "oracle", "_build", "libirwls_port.so")
    if not os.path.exists(port_path):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return _abi.load_library(port_path)


def cpu_baseline(hd, budget, gpu_centroids=None):
    """One complete training of the budgeted workload (SGMA to the full
    budget, then IRWLSpar to convergence) by the restatement on all host
    cores, timed end to end. Its SGMA candidate draws keep the reference's
    one-thread order, so its centroids are those of the reference run with
    -t 1; they are compared with the plain GPU form's when given."""
    import numpy as np

    port = load_port()
    cores = os.cpu_count() or 1
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    p = props(budget, threads=cores)
    port.initMemory(cores, budget)
    libc.srand(1)
    t0 = time.perf_counter()
    c = port.SGMA(hd.struct, p)
    t1 = time.perf_counter()
    w = port.IRWLSpar(hd.struct, c, p)
    t2 = time.perf_counter()
    cent = np.ctypeslib.as_array(c, shape=(budget,)).copy()
    libc.free(C.cast(c, C.c_void_p))
    libc.free(C.cast(w, C.c_void_p))
    out = {"value": round(t2 - t0, 3), "unit": "s", "cores": cores, "kind": "port",
           "sample": "one complete training of the whole workload (SGMA to m=%d, IRWLSpar to convergence) by the "
                     "CPU restatement of the reference (reference arithmetic, OpenMP loops and BLAS/LAPACK calls), "
                     "%d OpenMP threads, measured: SGMA %.1f s + IRWLSpar %.1f s" % (budget, cores, t1 - t0, t2 - t1)}
    if gpu_centroids is not None:
        out["centroids_identical_to_gpu_plain"] = int((cent == gpu_centroids).sum())
    return out


def timed_cpu_runs(one, steps):
    """Complete CPU trainings (`one()` returns a cpu_baseline dict) until
    `steps` have run or REF_ARM_BUDGET_S has passed, at least one."""
    t0, runs = time.perf_counter(), []
    while len(runs) < max(steps, 1):
        runs.append(one())
        if time.perf_counter() - t0 > REF_ARM_BUDGET_S:
            break
    base = dict(runs[-1])
    base["value"] = round(statistics.mean(r["value"] for r in runs), 3)
    base["sample"] += "; mean of %d complete training(s)" % len(runs)
    return base, len(runs)


def reference_line(args, base, timed, cfg):
    v = base["value"]
    return {"metric": METRIC, "value": v, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
            "steps": timed, "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": round(v * 1000, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)", "config": cfg, "cpu_baseline": base,
            "note": "each step is one complete CPU training of the whole workload (minutes each), so the arm "
                    "times %d of them within its %.0f s budget instead of the %d requested; a CPU run needs no "
                    "warm-up" % (timed, REF_ARM_BUDGET_S, args.steps),
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    hd = workload(args.rows)
    base, timed = timed_cpu_runs(lambda: cpu_baseline(hd, args.budget), args.steps)
    print(json.dumps(reference_line(args, base, timed, config(args))), flush=True)


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------

class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


PROFILE_SLOTS = {"sgma_scores": 0, "sgma_candidate_solves": 5, "sgma_select_and_factor": 6, "irwls_gram": 1,
                 "irwls_gram_slicing": 7, "irwls_cholesky": 3}
PRIMAL_BAR, ACC_BAR = 1e-4, 1e-3


def profile_read(lib, slot, steps):
    ms, n = C.c_double(), C.c_longlong()
    lib.irwls_profile_read(slot, C.byref(ms), C.byref(n))
    return ms.value / 1000.0 / max(steps, 1), n.value // max(steps, 1)


def measured_peaks():
    """Measured HBM / bf16 peaks of this GPU pool, if present."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured (MEASURED_PEAKS.json)"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback (one earlier GB300 measurement)"


def timed_trainings(lib, libc, res, p, steps, warmup, cent, w, precision, clocks=None):
    """`warmup` untimed then `steps` timed trainings of one form on the
    resident dataset (L2 flushed before each; CUDA events on the library's
    stream). Returns mean seconds, per-stage profile, launches and the clock
    record."""
    lib.irwls_set_precision(precision)

    def step():
        libc.srand(1)
        if lib.irwls_resident_budgeted(res, p, cent.ctypes.data_as(PI), w.ctypes.data_as(PD)) != 0:
            raise SystemExit("training failed: " + lib.irwls_last_error_message().decode())

    for _ in range(warmup):
        step()
    lib.irwls_profile_enable(1)
    lib.irwls_profile_reset()
    launches0 = lib.irwls_kernel_launches()
    lib.irwls_gram_tc_flops(1)
    if clocks:
        clocks.start()
    times = []
    for _ in range(steps):
        lib.irwls_l2_flush(512 << 20)
        lib.irwls_timer_start()
        step()
        times.append(lib.irwls_timer_stop() / 1000.0)
    clk = clocks.stop() if clocks else None
    launches = lib.irwls_kernel_launches() - launches0
    prof = {name: profile_read(lib, slot, steps) for name, slot in PROFILE_SLOTS.items()}
    lib.irwls_profile_enable(0)
    iters, nact = C.c_int(), C.c_int()
    lib.irwls_last_run_info(C.byref(iters), C.byref(nact))
    return {"s": statistics.mean(times), "prof": prof, "launches": launches / max(steps, 1), "clocks": clk,
            "iters": iters.value, "nact": nact.value, "gram_flops": lib.irwls_last_gram_flops(),
            "gram_tc_flops": lib.irwls_gram_tc_flops(1) / max(steps, 1), "steps": steps, "warmup": warmup}


def end_to_end(lib, libc, hd, p, args, precision, ref_cent, steps):
    """SGMA() + IRWLSpar() through the reference-facing C ABI on the host
    svm_dataset: host-to-device copies of the dataset and device-to-host
    copies of the results inside the timed region."""
    import numpy as np

    lib.irwls_set_precision(precision)
    h0, d0 = C.c_longlong(), C.c_longlong()
    lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
    e_times = []
    for _ in range(steps):
        lib.irwls_l2_flush(512 << 20)
        t0 = time.perf_counter()
        libc.srand(1)
        lib.initMemory(1, args.budget)
        cp = lib.SGMA(hd.struct, p)
        wp = lib.IRWLSpar(hd.struct, cp, p)
        if not cp or not wp:
            raise SystemExit("e2e training failed: " + lib.irwls_last_error_message().decode())
        e_times.append(time.perf_counter() - t0)
        got = np.ctypeslib.as_array(cp, shape=(args.budget,)).copy()
    h1, d1 = C.c_longlong(), C.c_longlong()
    lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
    assert np.array_equal(got, ref_cent), "end-to-end run selected different centroids"
    return {"value": round(statistics.mean(e_times), 3), "unit": "s",
            "h2d_bytes_per_step": int((h1.value - h0.value) // steps),
            "d2h_bytes_per_step": int((d1.value - d0.value) // steps), "steps": steps}


def primal_objective(hd, cent, w, gamma, cost, f):
    """Budgeted primal 1/2 w^T (K_mm + 1e-5 I) w + C sum_i max(0, 1 - y_i f_i)
    in FP64 on the host (f = K_nm w from the library's prediction path)."""
    import numpy as np

    from libirwls_gb300 import _abi

    rows, y, q = _abi.dataset_rows(hd.struct, hd.n_rows)
    d = max(int(r[0].max()) for r in rows if len(r[0])) + 1
    Xc = np.zeros((len(cent), d))
    for k, c in enumerate(cent):
        Xc[k, rows[c][0]] = rows[c][1]
    qc = q[cent]
    Kmm = np.exp(-gamma * (qc[:, None] + qc[None, :] - 2.0 * Xc @ Xc.T)) + 1e-5 * np.eye(len(cent))
    return float(0.5 * w @ Kmm @ w + cost * np.maximum(0.0, 1.0 - y[:hd.l] * f).sum())


def quality(lib, hd, p, cent, w):
    """Primal objective on the training rows and accuracy on the held-out
    rows (labelled by the training set's network) of one trained model."""
    import numpy as np

    from libirwls_gb300 import _abi, synth

    te = synth.budgeted_test_set(20000)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    c = np.ascontiguousarray(cent, dtype=np.int32)
    ww = np.ascontiguousarray(w)
    mdl = lib.calculateBudgetedModel(p, hd.struct, c.ctypes.data_as(PI), ww.ctypes.data_as(PD))
    soft = np.ctypeslib.as_array(lib.softTest(hd.struct, mdl, _abi.make_predict_properties(soft=1)),
                                 shape=(hd.l,)).copy()
    pred = np.ctypeslib.as_array(lib.test(ht.struct, mdl, _abi.make_predict_properties(soft=0)),
                                 shape=(ht.l,)).copy()
    lib.freeModel(mdl)
    return primal_objective(hd, c, ww, GAMMA, COST, soft), float((pred == te.y).mean())


def breakdown(run):
    return {k: round(v[0], 4) for k, v in run["prof"].items()}


def replicas():
    """(world, rank, local rank) of this process. Under torchrun every rank is
    an independent replica of the workload on its own GPU (the path has no
    exchange step, so no collective touches the data); gloo carries only the
    barriers and the max of the step times."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # the C library uses the current device
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    """The slowest rank's value (every rank gets it)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    world, rank, local = replicas()
    import numpy as np

    from libirwls_gb300 import load

    lib = load()
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    libc = C.CDLL(None)
    hd = workload(args.rows)
    p = props(args.budget)
    res = lib.irwls_resident_upload(hd.struct, p, 1)
    if not res:
        raise SystemExit(lib.irwls_last_error_message().decode())
    forms = {"both": (0, 1), "plain": (0,), "mixed": (1,)}[args.form]
    head = forms[-1]
    # the headline form runs K steps after W warm-ups; the plain form, when it
    # is only the denominator of the speed-up, runs fewer (16 s each)
    plan = {prec: (args.steps, args.warmup) if prec == head else (min(args.steps, PLAIN_STEPS), min(args.warmup, 1))
            for prec in forms}
    runs, cents, weights = {}, {}, {}
    for prec in forms:
        cent = np.zeros(args.budget, np.int32)
        w = np.zeros(args.budget)
        barrier(world)
        runs[prec] = timed_trainings(lib, libc, res, p, plan[prec][0], plan[prec][1], cent, w, prec,
                                     Clocks(local) if prec == head else None)
        cents[prec], weights[prec] = cent, w
    lib.irwls_resident_free(res)
    barrier(world)
    step_s = max_over_ranks(runs[head]["s"], world)
    e2e = {prec: None if args.no_e2e else
           end_to_end(lib, libc, hd, p, args, prec, cents[prec], plan[prec][0] if prec == head else min(args.steps, 2))
           for prec in forms}
    lib.irwls_set_precision(0)
    if rank != 0:
        return

    peaks, peak_src = measured_peaks()
    fp64_peak = lib.irwls_fp64_peak_tflops(5)
    sgma_flops = sum(2.0 * args.rows * s * 64 for s in range(2, args.budget))
    kernels = {}
    if 0 in runs:
        g_s = runs[0]["prof"]["sgma_scores"][0]
        ach = sgma_flops / g_s / 1e12 if g_s > 0 else 0.0
        kernels["sgma_gemm_kernel (plain FP64)"] = {
            "bound": "fp64", "achieved": round(ach, 4), "peak": round(fp64_peak, 4), "unit": "TFLOP/s",
            "frac": round(ach / fp64_peak, 4) if fp64_peak else None,
            "share_of_step": round(g_s / runs[0]["s"], 4)}
        gr_s = runs[0]["prof"]["irwls_gram"][0]
        ach = runs[0]["gram_flops"] / gr_s / 1e12 if gr_s > 0 else 0.0
        kernels["gram_kernel (plain FP64)"] = {
            "bound": "fp64", "achieved": round(ach, 4), "peak": round(fp64_peak, 4), "unit": "TFLOP/s",
            "frac": round(ach / fp64_peak, 4) if fp64_peak else None,
            "share_of_step": round(gr_s / runs[0]["s"], 4)}
    if 1 in runs:
        gr_s = runs[1]["prof"]["irwls_gram"][0]
        alg = runs[1]["gram_flops"] / gr_s / 1e12 if gr_s > 0 else 0.0
        tc = runs[1]["gram_tc_flops"] / gr_s / 1e12 if gr_s > 0 else 0.0
        sus = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops")
        kernels["gram_tc_kernel (precision form, exact integer digit products on tcgen05)"] = {
            "bound": "tensor", "achieved": round(alg, 3), "peak": sus,
            "unit": "TFLOP/s algorithmic (n_act (m+1) m flops per IRWLSpar iteration, the FP64 SYRK replaced)",
            "frac": round(alg / sus, 4) if sus else None,
            "peak_source": peak_src + " bf16 sustained (the kernel runs inside a seconds-long training)",
            "digit_product_tflops": round(tc, 2),
            "digit_product_pipe_frac": round(tc / sus, 4) if sus else None,
            "digit_products_per_algorithmic_product": round(runs[1]["gram_tc_flops"] / runs[1]["gram_flops"], 2)
            if runs[1]["gram_flops"] else None,
            "share_of_step": round(gr_s / runs[1]["s"], 4),
            "slicing_share_of_step": round(runs[1]["prof"]["irwls_gram_slicing"][0] / runs[1]["s"], 4)}
        sc_s = runs[1]["prof"]["sgma_scores"][0]
        nl = max(1, args.budget - 2)  # score launches (orders 2 ... m - 1)
        sc_bytes = sum(score_launch_bytes(args.rows, s, hd) for s in range(2, args.budget))
        ach = sc_bytes / sc_s / 1e9 if sc_s > 0 else 0.0
        kernels["sgma_tc_score_ws_kernel (precision form, tcgen05 on three bf16 pieces)"] = {
            "bound": "hbm", "achieved": round(ach, 1), "peak": peaks.get("hbm_gbs"),
            "unit": "GB/s algorithmic (per launch at order s: Q's three bf16 pieces of the s columns rounded up "
                    "to 32, read once; the 64 residuals of every row written; the rows' FP32 CSR read)",
            "frac": round(ach / peaks["hbm_gbs"], 4) if peaks.get("hbm_gbs") else None,
            "peak_source": peak_src + " HBM copy", "launches": nl,
            "avg_launch_us": round(sc_s / nl * 1e6, 2),
            "algorithmic_tflops": round(sgma_flops / sc_s / 1e12, 2) if sc_s > 0 else None,
            "share_of_step": round(sc_s / runs[1]["s"], 4)}
    # roofline: the dominant kernel of the headline form
    if head == 1:
        k = kernels["sgma_tc_score_ws_kernel (precision form, tcgen05 on three bf16 pieces)"]
        # DRAM traffic of one launch from a full-size, one-pass ncu capture (the
        # 501st score launch of this workload, order 502, the mean order of
        # the run): profiles/sgma_tc_score_ws_kernel_200k_traffic.md
        lb = score_launch_bytes(args.rows, 502, hd)
        traffic = SCORE_TRAFFIC_502
        roofline = dict(k, kernel="sgma_tc_score_ws_kernel", traffic=traffic,
                        traffic_launch={"launch": "501st of 998 (order 502)", "duration_ms": SCORE_MS_502,
                                        "algorithmic_bytes": lb,
                                        "traffic_over_algorithmic": round(traffic / lb, 3) if traffic else None,
                                        "source": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,"
                                                  "gpu__time_duration.sum (one pass)"})
        g = kernels["gram_tc_kernel (precision form, exact integer digit products on tcgen05)"]
        # the Gram's last launch (62357 active rows), from the same kind of
        # capture: profiles/gram_tc_kernel_200k_m1000_traffic.md
        g["traffic_launch"] = {"launch": "last of 42 (active rows 62357)", "duration_ms": 1.517,
                               "traffic": 894986752 + 3068672, "algorithmic_bytes": 62357 * 1001 * 8}
    else:
        k = kernels["sgma_gemm_kernel (plain FP64)"]
        roofline = dict(k, kernel="sgma_gemm_kernel", traffic=None,
                        peak_source="measured live: FP64 FMA-chain probe of the library "
                                    "(irwls_fp64_peak_tflops); MEASURED_PEAKS.json has no FP64 figure")

    accuracy, value, form = None, step_s, ("plain FP64" if head == 0 else "precision (mixed)")
    if forms == (0, 1):
        obj = {prec: quality(lib, hd, p, cents[prec], weights[prec]) for prec in forms}
        rel = abs(obj[1][0] - obj[0][0]) / abs(obj[0][0])
        dacc = obj[1][1] - obj[0][1]
        ok = rel <= PRIMAL_BAR and abs(dacc) <= ACC_BAR
        accuracy = {"objective": "primal 1/2 w^T (K_mm + 1e-5 I) w + C sum_i max(0, 1 - y_i f_i): the budgeted "
                                 "model has no bias and no dual, so its objective bar is on the primal",
                    "primal_rel_err_vs_plain": rel, "primal_plain": obj[0][0], "primal_mixed": obj[1][0],
                    "test_acc_plain": obj[0][1], "test_acc_mixed": obj[1][1], "test_acc_change": dacc,
                    "centroids_identical": int((cents[1] == cents[0]).sum()),
                    "bars": {"primal_rel_err": PRIMAL_BAR, "test_acc_change": ACC_BAR}, "meets_bars": ok}
        if not ok:
            # the precision form missed the bar: report the plain form as the value
            head, value, form = 0, runs[0]["s"], "plain FP64 (precision form missed the accuracy bar)"
    plain = None
    if 0 in runs:
        plain = {"value": round(runs[0]["s"], 3), "unit": "s", "steps": runs[0]["steps"],
                 "warmup": runs[0]["warmup"], "e2e": e2e[0], "launches": int(runs[0]["launches"]),
                 "breakdown_s": breakdown(runs[0]), "par_iterations": runs[0]["iters"],
                 "active_rows_final": runs[0]["nact"]}
    full784 = None
    if args.with_full784 and forms == (0, 1):
        fa = argparse.Namespace(**vars(args))
        fa.workload, fa.no_cpu = "full784", True
        full784 = full_measure(fa, lib, libc)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "s", "n_gpus": world if world > 1 else args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value * 1000, 1),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == 0 else "bf16 pieces x6 (SGMA scores) + exact bf16 digit products (IRWLSpar Gram) + f64 (factors, solves)",
            "data": "synthetic (seeded generator)",
            "config": config(args, {"form": form, "par_iterations": runs[head]["iters"],
                                    "active_rows_final": runs[head]["nact"]}),
            "e2e": e2e[head], "gpu_launches": int(runs[head]["launches"] * args.steps), "roofline": roofline,
            "cpu_baseline": None if args.no_cpu else cpu_baseline(hd, args.budget, cents.get(0)),
            "clocks": runs[forms[-1]]["clocks"], "breakdown_s": breakdown(runs[head]),
            "speedup_vs_plain_fp64": round(runs[0]["s"] / value, 2) if 0 in runs else None,
            "accuracy": accuracy, "plain_fp64": plain, "kernels": kernels, "full784": full784}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# full-IRWLS workloads
# ----------------------------------------------------------------------------
FULL = {
    "full": dict(n=4000, n_test=1000, d=20, seed=20240601, gamma=0.05, C=10.0, w=500,
                 desc="full IRWLS: n=4000, d=20 dense (two Gaussian classes, means +-0.5, 10% labels flipped), "
                      "RBF gamma=0.05, C=10, working set 500"),
    "full784": dict(n=100_000, n_test=10_000, d=784, seed=20240606, gamma=0.02, C=10.0, w=500,
                    desc="full IRWLS: n=100000 train / 10000 test, d=784 sparse-valued dense (8-bit values / 255, "
                         "19% nonzero, 10 seeded prototypes, 0-4 vs 5-9), RBF gamma=0.02, C=10, working set 500"),
}


def full_workload(cfg):
    from libirwls_gb300 import _abi, synth

    if cfg["d"] == 784:
        tr, te = synth.precision_full_workload(cfg["n"], cfg["n_test"], seed=cfg["seed"])
    else:
        X, y = synth.two_gaussians(cfg["n"] + cfg["n_test"], cfg["d"], cfg["seed"])
        tr = synth.from_dense(X[:cfg["n"]], y[:cfg["n"]], keep_zeros=True)
        te = synth.from_dense(X[cfg["n"]:], y[cfg["n"]:], keep_zeros=True)
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    return hd, ht, te.y


def full_props(cfg, threads=1):
    from libirwls_gb300 import _abi

    return _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], working_set=cfg["w"], threads=threads, verbose=0)


def full_config(cfg, form):
    return {"workload": cfg["desc"], "n": cfg["n"], "d": cfg["d"], "gamma": cfg["gamma"], "C": cfg["C"],
            "working_set": cfg["w"], "form": form, "parallelism": "single GPU",
            "l2": "flushed between timed steps (512 MiB overwrite)"}


def full_cpu(hd, cfg, gpu_beta=None):
    """One complete training of the workload by the restatement on all host
    cores, measured (no sample is scaled). With `gpu_beta` (the plain GPU
    form's weights) it also reports whether the support-vector sets agree."""
    import numpy as np

    port = load_port()
    cores = os.cpu_count() or 1
    libc = C.CDLL(None)
    port.initMemory(cores, cfg["w"] + 1)
    libc.srand(0)
    t0 = time.perf_counter()
    b = port.trainFULL(hd.struct, full_props(cfg, threads=cores))
    dt = time.perf_counter() - t0
    beta = np.ctypeslib.as_array(b, shape=(hd.l + 1,)).copy()
    libc.free.argtypes = [C.c_void_p]
    libc.free(C.cast(b, C.c_void_p))
    out = {"value": round(dt, 3), "unit": "s", "cores": cores, "kind": "port",
           "sample": "one complete training of the whole workload by the CPU restatement of the reference "
                     "(reference arithmetic, OpenMP loops and BLAS/LAPACK calls), %d OpenMP threads, measured" % cores}
    if gpu_beta is not None:
        out["support_vector_sets_identical_to_gpu_plain"] = bool(np.array_equal(beta[:-1] != 0, gpu_beta[:-1] != 0))
    return out


def dual_objective(hd, beta, gamma):
    """D(beta) = sum_i y_i beta_i - 1/2 beta^T K beta over the support vectors
    (RBF, norm form), in FP64 on the host."""
    import numpy as np

    from libirwls_gb300 import _abi

    rows, y, q = _abi.dataset_rows(hd.struct, hd.l)
    sv = np.nonzero(beta[:hd.l])[0]
    d = max([int(rows[i][0].max()) for i in sv if len(rows[i][0])] + [0]) + 1
    Xs = np.zeros((len(sv), d))
    for k, i in enumerate(sv):
        Xs[k, rows[i][0]] = rows[i][1]
    qs = q[sv]
    K = np.exp(-gamma * np.maximum(qs[:, None] + qs[None, :] - 2 * Xs @ Xs.T, 0.0))
    b = beta[sv]
    return float((y[sv] * b).sum() - 0.5 * b @ K @ b)


def run_full(args):
    from libirwls_gb300 import load

    cfg = FULL[args.workload]
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        hd, _, _ = full_workload(cfg)
        base, timed = timed_cpu_runs(lambda: full_cpu(hd, cfg), args.steps)
        print(json.dumps(reference_line(args, base, timed, full_config(cfg, "plain FP64"))), flush=True)
        return
    lib = load()
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    print(json.dumps(full_measure(args, lib, C.CDLL(None))), flush=True)


def full_measure(args, lib, libc):
    """Both forms of a full-IRWLS workload on its resident dataset, their
    end-to-end runs through trainFULL, the accuracy bars (dual objective,
    held-out accuracy) and, unless args.no_cpu, a complete CPU training.
    Returns the JSON line as a dict."""
    import numpy as np

    from libirwls_gb300 import _abi

    cfg = FULL[args.workload]
    hd, ht, yt = full_workload(cfg)
    p = full_props(cfg)
    res = lib.irwls_resident_upload(hd.struct, p, 0)
    forms = {"both": (0, 1), "plain": (0,), "mixed": (1,)}[args.form]
    runs, betas = {}, {}
    for prec in forms:
        lib.irwls_set_precision(prec)
        beta = np.zeros(hd.l + 1)

        def step():
            libc.srand(0)
            if lib.irwls_resident_full(res, p, beta.ctypes.data_as(PD)) != 0:
                raise SystemExit("training failed: " + lib.irwls_last_error_message().decode())

        for _ in range(args.warmup):
            step()
        lib.irwls_profile_enable(1)
        lib.irwls_profile_reset()
        launches0 = lib.irwls_kernel_launches()
        clocks = Clocks(0) if prec == forms[-1] else None
        if clocks:
            clocks.start()
        times = []
        for _ in range(args.steps):
            lib.irwls_l2_flush(512 << 20)
            lib.irwls_timer_start()
            step()
            times.append(lib.irwls_timer_stop() / 1000.0)
        clk = clocks.stop() if clocks else None
        prof = {name: profile_read(lib, slot, args.steps) for name, slot in (("kernel_rowsums", 2),
                                                                             ("cholesky_solves", 3))}
        lib.irwls_profile_enable(0)
        runs[prec] = {"s": statistics.mean(times), "launches": lib.irwls_kernel_launches() - launches0,
                      "clocks": clk, "prof": prof}
        betas[prec] = beta.copy()
    lib.irwls_resident_free(res)
    e2e = {}
    for prec in forms:
        if args.no_e2e:
            e2e[prec] = None
            continue
        lib.irwls_set_precision(prec)
        h0, d0 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
        e_times = []
        for _ in range(args.steps):
            lib.irwls_l2_flush(512 << 20)
            t0 = time.perf_counter()
            libc.srand(0)
            lib.initMemory(1, cfg["w"] + 1)
            bp = lib.trainFULL(hd.struct, p)
            if not bp:
                raise SystemExit("e2e training failed: " + lib.irwls_last_error_message().decode())
            e_times.append(time.perf_counter() - t0)
            libc.free.argtypes = [C.c_void_p]
            libc.free(C.cast(bp, C.c_void_p))
        h1, d1 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
        e2e[prec] = {"value": round(statistics.mean(e_times), 3), "unit": "s",
                     "h2d_bytes_per_step": int((h1.value - h0.value) // args.steps),
                     "d2h_bytes_per_step": int((d1.value - d0.value) // args.steps)}
    lib.irwls_set_precision(0)

    def test_acc(beta):
        bb = np.ascontiguousarray(beta)
        mdl = lib.calculateFULLModel(p, hd.struct, bb.ctypes.data_as(PD))
        pred = np.ctypeslib.as_array(lib.test(ht.struct, mdl, _abi.make_predict_properties(soft=0)),
                                     shape=(ht.l,)).copy()
        lib.freeModel(mdl)
        return float((pred == yt).mean())

    head = forms[-1]
    accuracy = None
    if forms == (0, 1):
        d0, d1 = dual_objective(hd, betas[0], cfg["gamma"]), dual_objective(hd, betas[1], cfg["gamma"])
        a0, a1 = test_acc(betas[0]), test_acc(betas[1])
        rel = abs(d1 - d0) / abs(d0)
        ok = rel <= PRIMAL_BAR and abs(a1 - a0) <= ACC_BAR
        accuracy = {"dual_rel_err_vs_plain": rel, "dual_plain": d0, "dual_mixed": d1, "test_acc_plain": a0,
                    "test_acc_mixed": a1, "test_acc_change": a1 - a0,
                    "support_vectors": {"plain": int((betas[0][:-1] != 0).sum()),
                                        "mixed": int((betas[1][:-1] != 0).sum())},
                    "bars": {"dual_rel_err": PRIMAL_BAR, "test_acc_change": ACC_BAR}, "meets_bars": ok}
        if not ok:
            head = 0
    r = runs[head]
    value = r["s"]
    peak = lib.irwls_fp64_peak_tflops(3)
    roofline = {"bound": "latency" if head == 0 else "mixed",
                "kernel": "kernel row sums (FP64 ordered) and Cholesky solves",
                "achieved": None, "peak": round(peak, 4), "unit": "TFLOP/s", "frac": None, "traffic": None,
                "share_of_step": {k: round(v[0] / value, 4) for k, v in r["prof"].items()},
                "launches_per_step": {k: int(v[1]) for k, v in r["prof"].items()}}
    base = None if args.no_cpu else full_cpu(hd, cfg, betas.get(0))
    plain = None
    if 0 in runs and head != 0:
        plain = {"value": round(runs[0]["s"], 3), "unit": "s", "e2e": e2e[0],
                 "breakdown_s": {k: round(v[0], 4) for k, v in runs[0]["prof"].items()}}
    return {"metric": METRIC, "value": round(value, 3), "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value * 1000, 1),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == 0 else "bf16x6 (error updates off the exact set) + f64",
            "data": "synthetic (seeded generator)",
            "config": full_config(cfg, "plain FP64" if head == 0 else "precision (mixed)"),
            "e2e": e2e[head], "gpu_launches": int(r["launches"]), "roofline": roofline,
            "cpu_baseline": base, "clocks": runs[forms[-1]]["clocks"],
            "speedup_vs_plain_fp64": round(runs[0]["s"] / value, 2) if 0 in runs else None,
            "accuracy": accuracy, "plain_fp64": plain}


# ----------------------------------------------------------------------------
# batching form: many SVMs trained concurrently
# ----------------------------------------------------------------------------
BATCH_DESC = ("batching form: 64 RBF SVMs (C in logspace(-1,3,8) x gamma in logspace(-3,0,8)) + 8 linear SVMs, "
              "full IRWLS, working set 500, each on its own subset (n log-uniform in [2000, 50000]) of a CSR pool "
              "(d=300, 3% density, binary/[0,1] values, labels from a seeded sparse linear rule, 8% flipped)")


def batch_cpu(hds, prs, k=3):
    """The restatement trains the k smallest SVMs of the batch on all host
    cores; scaled to the batch by total rows."""
    from libirwls_gb300 import _abi

    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    port_path = os.path.join(ROOT, "oracle", "_build", "libirwls_port.so")
    if not os.path.exists(port_path):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    port = _abi.load_library(port_path)
    cores = os.cpu_count() or 1
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    order = sorted(range(len(hds)), key=lambda i: hds[i].l)[:k]
    t0 = time.perf_counter()
    for i in order:
        p = prs[i]
        p.Threads = cores
        port.initMemory(cores, p.MaxSize + 1)
        libc.srand(i)
        libc.free(C.cast(port.trainFULL(hds[i].struct, p), C.c_void_p))
        p.Threads = 1
    dt = time.perf_counter() - t0
    rows_s = sum(hds[i].l for i in order)
    scale = sum(h.l for h in hds) / rows_s
    return {"value": round(dt * scale, 3), "unit": "s", "cores": cores, "kind": "port",
            "sample": "CPU restatement of the reference, %d OpenMP threads, on the %d smallest SVMs (%d rows, "
                      "%.1f s), scaled by total rows x %.1f" % (cores, k, rows_s, dt, scale)}


def run_batch(args):
    import numpy as np

    from libirwls_gb300 import _abi, load, synth

    pool, jobs = synth.batch_workload()
    hds, prs = [], []
    for rows, kern, cost, gamma in jobs:
        sub = synth.subset(pool, rows)
        hds.append(_abi.build_dataset(sub.indptr, sub.indices, sub.values, sub.y))
        prs.append(_abi.make_properties(gamma=gamma, C_=cost, kernel=kern, working_set=500))
    n = len(jobs)
    cfg = {"workload": BATCH_DESC, "svms": n, "rows_total": int(sum(h.l for h in hds)),
           "rows_min": int(min(h.l for h in hds)), "rows_max": int(max(h.l for h in hds)),
           "form": "batching (concurrent trainings on separate streams)", "parallelism": "single GPU",
           "l2": "the datasets (tens of MB each) are uploaded per training; L2 flushed between steps"}
    if args.impl == "reference":
        base = batch_cpu(hds, prs)
        print(json.dumps({"metric": METRIC, "value": base["value"], "unit": "s", "impl": "reference",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": base["value"] * 1000,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded generator)", "config": cfg, "cpu_baseline": base,
                          "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    lib = load()
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    dss = (_abi.SvmDataset * n)(*[h.struct for h in hds])
    pp = (_abi.Properties * n)(*prs)
    seeds = (C.c_uint * n)(*range(n))
    workers = lib.irwls_batch_autotune(dss, pp, n, 8)
    if workers <= 0:
        raise SystemExit("autotune failed: " + lib.irwls_last_error_message().decode())

    def batch(w):
        out = (PD * n)()
        lib.irwls_l2_flush(512 << 20)
        lib.irwls_dev_sync()
        h0, d0 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
        t0 = time.perf_counter()
        if lib.irwls_full_train_batch(dss, pp, seeds, n, w, out) != 0:
            raise SystemExit("batch failed: " + lib.irwls_last_error_message().decode())
        dt = time.perf_counter() - t0
        h1, d1 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
        res = [np.ctypeslib.as_array(out[i], shape=(hds[i].l + 1,)).copy() for i in range(n)]
        return dt, res, h1.value - h0.value, d1.value - d0.value

    seq_s, seq_res, _, _ = batch(1)
    for _ in range(args.warmup):
        batch(workers)
    launches0 = lib.irwls_kernel_launches()
    clocks = Clocks(0)
    clocks.start()
    times, h2d, d2h = [], 0, 0
    for _ in range(args.steps):
        dt, res, hb, db = batch(workers)
        times.append(dt)
        h2d, d2h = hb, db
    clk = clocks.stop()
    launches = lib.irwls_kernel_launches() - launches0
    identical = all(np.array_equal(a, b) for a, b in zip(res, seq_res))
    value = statistics.mean(times)
    nsv = [int((r[:-1] != 0).sum()) for r in res]
    mixed = None
    if args.form == "mixed":
        # the same batch in the precision form (tensor-core error updates,
        # cluster working-set solves), against the sequential FP64 run
        lib.irwls_set_precision(1)
        try:
            for _ in range(args.warmup):
                batch(workers)
            mt = []
            for _ in range(args.steps):
                dt, mres, _, _ = batch(workers)
                mt.append(dt)
        finally:
            lib.irwls_set_precision(0)
        same_sv = sum(int(np.array_equal(a[:-1] != 0, b[:-1] != 0)) for a, b in zip(mres, seq_res))
        werr = max(float(np.abs(a - b).max()) / prs[i].C for i, (a, b) in enumerate(zip(mres, seq_res)))
        mv = statistics.mean(mt)
        mixed = {"value": round(mv, 3), "unit": "s", "steps": args.steps,
                 "speedup_vs_plain_fp64": round(seq_s / mv, 2),
                 "svms_with_the_fp64_support_vectors": same_sv, "svms": n,
                 "max_weight_diff_over_C": werr,
                 "form": "batching + precision form (error updates off the exact set on the tensor cores, "
                         "working-set solves by the FP32 cluster Cholesky with FP64 refinement)"}
    line = {"metric": METRIC, "value": round(value, 3), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": dict(cfg, workers=workers, autotuned=True),
            "e2e": {"value": round(value, 3), "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "note": "the batch API takes host svm_datasets: every timed step uploads them"},
            "gpu_launches": int(launches // max(args.steps, 1)),
            "roofline": {"bound": "latency", "kernel": "concurrent trainings", "achieved": None, "peak": None,
                         "unit": None, "frac": None, "traffic": None},
            "cpu_baseline": None if args.no_cpu else batch_cpu(hds, prs), "clocks": clk,
            "sequential_plain_fp64_s": round(seq_s, 3), "speedup_vs_plain_fp64": round(seq_s / value, 2),
            "svms_per_s": round(n / value, 2), "identical_to_sequential": bool(identical),
            "support_vectors": {"min": min(nsv), "max": max(nsv), "total": sum(nsv)},
            "precision_form": mixed}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# linear-kernel prediction through the primal weights
# ----------------------------------------------------------------------------
LINP = dict(n_sv_rows=50_000, n_test=200_000, cpu_rows=20_000, seed=20240611)
LINP_DESC = ("linear-kernel prediction: softTest of 200000 sparse test rows (d=300, 3%% nonzero, values binary or "
             "U[0,1]) against a linear model of %d support vectors (seeded weights): the primal fast path "
             "(irwls_set_linear_fast_path) against the per-support-vector kernel sum")


def run_linear_predict(args):
    import numpy as np

    from libirwls_gb300 import _abi, load, synth

    n_sv, n_te = LINP["n_sv_rows"], LINP["n_test"]
    pool = synth.sparse_linear_pool(n_sv + n_te, seed=LINP["seed"])
    cut = int(pool.indptr[n_sv])
    tr = _abi.build_dataset(pool.indptr[:n_sv + 1], pool.indices[:cut], pool.values[:cut], pool.y[:n_sv])
    te = _abi.build_dataset(pool.indptr[n_sv:] - cut, pool.indices[cut:], pool.values[cut:], pool.y[n_sv:])
    rng = np.random.default_rng(LINP["seed"])
    beta = np.ascontiguousarray(np.where(rng.random(n_sv + 1) < 0.6, rng.standard_normal(n_sv + 1), 0.0))
    nsv = int((beta[:-1] != 0).sum())
    prop = _abi.make_properties(gamma=1.0, C_=1.0, kernel=0)
    pp = _abi.make_predict_properties(labels=0, soft=1)
    metric = "linear-kernel prediction s (soft decision values of %d test rows)" % n_te
    cfg = {"workload": LINP_DESC % nsv, "test_rows": n_te, "support_vectors": nsv, "d": 300,
           "nnz_test": int(pool.indptr[-1] - cut), "form": "primal fast path", "parallelism": "single GPU",
           "l2": "flushed before each call; the test set is uploaded by every call"}
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]

    def cpu_line():
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        port_path = os.path.join(ROOT, "oracle", "_build", "libirwls_port.so")
        if not os.path.exists(port_path):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
        port = _abi.load_library(port_path)
        cores = os.cpu_count() or 1
        k = LINP["cpu_rows"]
        sub = _abi.build_dataset(pool.indptr[n_sv:n_sv + k + 1] - cut, pool.indices[cut:int(pool.indptr[n_sv + k])],
                                 pool.values[cut:int(pool.indptr[n_sv + k])], pool.y[n_sv:n_sv + k])
        # the model is packed by this library's host packing (byte-identical to
        # the reference's calculateFULLModel, no device work, not timed)
        from libirwls_gb300 import load as load_ours

        pc = _abi.make_properties(gamma=1.0, C_=1.0, kernel=0, threads=cores)
        mdl_c = load_ours().calculateFULLModel(pc, tr.struct, beta.ctypes.data_as(PD))
        ppc = _abi.make_predict_properties(labels=0, soft=1, threads=cores)
        t0 = time.perf_counter()
        libc.free(C.cast(port.softTest(sub.struct, mdl_c, ppc), C.c_void_p))
        dt = time.perf_counter() - t0
        return {"value": round(dt * n_te / k, 3), "unit": "s", "cores": cores, "kind": "port",
                "sample": "the restatement's softTest (per-support-vector kernel sum, OpenMP over test rows) on "
                          "the first %d test rows, scaled to %d" % (k, n_te)}

    if args.impl == "reference":
        base = cpu_line()
        print(json.dumps({"metric": metric, "value": base["value"], "unit": "s", "impl": "reference",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": base["value"] * 1000,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded generator)", "config": cfg, "cpu_baseline": base,
                          "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    lib = load()
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    mdl = lib.calculateFULLModel(prop, tr.struct, beta.ctypes.data_as(PD))

    def predict(fast):
        lib.irwls_set_linear_fast_path(fast)
        lib.irwls_l2_flush(512 << 20)
        lib.irwls_dev_sync()
        h0, d0 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
        t0 = time.perf_counter()
        ptr = lib.softTest(te.struct, mdl, pp)
        dt = time.perf_counter() - t0
        if not ptr:
            raise SystemExit("prediction failed: " + lib.irwls_last_error_message().decode())
        f = np.ctypeslib.as_array(ptr, shape=(n_te,)).copy()
        libc.free(C.cast(ptr, C.c_void_p))
        h1, d1 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
        return dt, f, h1.value - h0.value, d1.value - d0.value

    predict(0)
    kern_s, f_kern, _, _ = predict(0)
    for _ in range(args.warmup):
        predict(1)
    lib.irwls_profile_enable(1)
    lib.irwls_profile_reset()
    launches0 = lib.irwls_kernel_launches()
    clocks = Clocks(0)
    clocks.start()
    times = []
    for _ in range(args.steps):
        dt, f_fast, h2d, d2h = predict(1)
        times.append(dt)
    clk = clocks.stop()
    launches = lib.irwls_kernel_launches() - launches0
    k_s = profile_read(lib, 4, args.steps)[0]
    lib.irwls_profile_enable(0)
    lib.irwls_set_linear_fast_path(0)
    value = statistics.mean(times)
    scale = float(np.abs(f_kern).max())
    diff = float(np.abs(f_fast - f_kern).max() / scale)
    clear = np.abs(f_kern) > 1e-10 * scale
    labels_equal = bool(np.array_equal(np.sign(f_fast[clear]), np.sign(f_kern[clear])))
    peaks, peak_src = measured_peaks()
    nnz = cfg["nnz_test"]
    # test CSR entries, row pointers and decision values, plus the model's dense
    # rows read once to form W (nsv x 300 doubles)
    alg = nnz * 12 + (n_te + 1) * 4 + n_te * 8 + nsv * 300 * 8
    ach = alg / k_s / 1e9 if k_s > 0 else 0.0
    line = {"metric": metric, "value": round(value, 4), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 2), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": cfg,
            "e2e": {"value": round(value, 4), "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "note": "softTest takes a host svm_dataset: every call uploads the test set and the model"},
            "gpu_launches": int(launches // max(args.steps, 1)),
            "roofline": {"bound": "hbm", "kernel": "linear_w_kernel + linear_dot_kernel",
                         "achieved": round(ach, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": round(ach / peaks["hbm_gbs"], 4) if peaks.get("hbm_gbs") else None,
                         "traffic": None, "peak_source": peak_src, "kernel_s": round(k_s, 6),
                         "algorithmic_bytes": alg},
            "cpu_baseline": None if args.no_cpu else cpu_line(), "clocks": clk,
            "kernel_sum_path_s": round(kern_s, 4), "speedup_vs_kernel_sum": round(kern_s / value, 2),
            "parity": {"max_abs_diff_over_max_abs_f": diff, "labels_equal_where_clear": labels_equal}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# the libsvm reader on the device
# ----------------------------------------------------------------------------
PARSE = dict(n=1_000_000, seed=20240612)
PARSE_DESC = ("libsvm reader: readTrainFile of a %d-row file of the learned-form workload's shape (32 dense features "
              "written with 17 significant digits, labels +-1; %.0f MB of text): the device reader "
              "(readTrainFileGPU: file read, both strtok passes and every strtod/strtol on the GPU, class-mean rows "
              "on the host) against the host reader")


def run_parse(args):
    import numpy as np

    from libirwls_gb300 import _abi, load, synth

    lib = load()
    if args.impl != "reference" and not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    n = args.parse_rows or PARSE["n"]
    path = os.path.join(tempfile.gettempdir(), "irwls_parse_%d.libsvm" % n)
    X, y = synth.gauss_mixture(n, seed=PARSE["seed"])
    synth.write_libsvm(path, synth.from_dense(X, y, keep_zeros=True))
    with open(path, "rb") as f:
        text = f.read()
    mb = len(text) / 1e6
    metric = "libsvm read s (%d rows, %.0f MB)" % (n, mb)
    cfg = {"workload": PARSE_DESC % (n, mb), "rows": n, "features": 32, "bytes": len(text),
           "form": "device reader", "parallelism": "single GPU", "l2": "the text (%.0f MB) exceeds L2" % mb}

    def host_read():
        t0 = time.perf_counter()
        ds = lib.readTrainFile(path.encode())
        return time.perf_counter() - t0, ds

    if args.impl == "reference":
        dt, ds = host_read()
        lib.freeDataset(ds)
        base = {"value": round(dt, 3), "unit": "s", "cores": 1, "kind": "port",
                "sample": "the reference's reader restated (host C, single thread, strtok/strtod as the reference) "
                          "on the whole file"}
        print(json.dumps({"metric": metric, "value": base["value"], "unit": "s", "impl": "reference",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": base["value"] * 1000,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded generator)", "config": cfg, "cpu_baseline": base,
                          "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        os.unlink(path)
        return
    lib.readTrainFileGPU.restype = _abi.SvmDataset
    lib.readTrainFileGPU.argtypes = [C.c_char_p]
    lib.irwls_parse_libsvm.restype = C.c_int
    lib.irwls_parse_libsvm.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(_abi.SvmDataset)]

    def dev_read():
        lib.irwls_dev_sync()
        h0, d0 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
        t0 = time.perf_counter()
        ds = lib.readTrainFileGPU(path.encode())
        dt = time.perf_counter() - t0
        h1, d1 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
        return dt, ds, h1.value - h0.value, d1.value - d0.value

    def same(a, b):
        if (a.l, a.sparse, a.maxdim) != (b.l, b.sparse, b.maxdim):
            return False
        ra, ya, qa = _abi.dataset_rows(a, a.l + 2)
        rb, yb, qb = _abi.dataset_rows(b, b.l + 2)
        return (all(np.array_equal(i1, i2) and np.array_equal(v1.view(np.int64), v2.view(np.int64))
                    for (i1, v1), (i2, v2) in zip(ra, rb))
                and np.array_equal(ya.view(np.int64), yb.view(np.int64))
                and np.array_equal(qa.view(np.int64), qb.view(np.int64)))

    for _ in range(args.warmup):
        _, ds, _, _ = dev_read()
        lib.freeDataset(ds)
    lib.irwls_profile_enable(1)
    lib.irwls_profile_reset()
    launches0 = lib.irwls_kernel_launches()
    clocks = Clocks(0)
    clocks.start()
    times = []
    for _ in range(args.steps):
        lib.irwls_l2_flush(512 << 20)
        dt, ds, h2d, d2h = dev_read()
        times.append(dt)
        last = ds
    clk = clocks.stop()
    launches = lib.irwls_kernel_launches() - launches0
    k_s = profile_read(lib, 8, args.steps)[0]
    lib.irwls_profile_enable(0)
    mem_t0 = time.perf_counter()
    ds_mem = _abi.SvmDataset()
    rc = lib.irwls_parse_libsvm(text, len(text), C.byref(ds_mem))
    mem_s = time.perf_counter() - mem_t0
    value = statistics.mean(times)
    host_s, host_ds = host_read() if not args.no_cpu else (None, None)
    identical = bool(same(last, host_ds)) if host_ds is not None else None
    peaks, peak_src = measured_peaks()
    ach = len(text) / k_s / 1e9 if k_s > 0 else 0.0
    line = {"metric": metric, "value": round(value, 3), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (exact decimal conversion)",
            "data": "synthetic (seeded generator)", "config": cfg,
            "e2e": {"value": round(value, 3), "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "note": "from the file name to the host svm_dataset, file read included"},
            "gpu_launches": int(launches // max(args.steps, 1)),
            "roofline": {"bound": "issue (byte-serial tokenising, one thread per line)", "kernel": "pass1/pass2/sparse",
                         "achieved": round(ach, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s of text",
                         "frac": round(ach / peaks["hbm_gbs"], 4) if peaks.get("hbm_gbs") else None,
                         "traffic": None, "peak_source": peak_src, "kernel_s": round(k_s, 4)},
            "cpu_baseline": None if host_s is None else {
                "value": round(host_s, 3), "unit": "s", "cores": 1, "kind": "port",
                "sample": "the reference's reader restated (host C readTrainFile, single thread) on the whole file"},
            "clocks": clk, "in_memory_parse_s": round(mem_s, 3) if rc == 0 else None,
            "identical_to_host_reader": identical}
    print(json.dumps(line), flush=True)
    lib.freeDataset(last)
    if rc == 0:
        lib.freeDataset(ds_mem)
    if host_ds is not None:
        lib.freeDataset(host_ds)
    os.unlink(path)


# ----------------------------------------------------------------------------
# models on the device: packing, the model file
# ----------------------------------------------------------------------------
MODEL_IO_DESC = ("model I/O: a full-IRWLS model of %d support vectors packed from the 200000-row budgeted workload "
                 "(d=54 sparse; seeded weights, half of them zero), stored to a model file and read back: "
                 "on the device (irwls_dmodel_full / _store / _read) against the host "
                 "(calculateFULLModel / storeModel / readModel)")


def run_model_io(args):
    import numpy as np

    from libirwls_gb300 import _abi, load

    lib = load()
    hd = workload(N_ROWS)
    rng = np.random.default_rng(20240613)
    beta = np.ascontiguousarray(np.where(rng.random(hd.l + 1) < 0.5, rng.standard_normal(hd.l + 1), 0.0))
    nsv = int((beta[:-1] != 0).sum())
    prop = _abi.make_properties(gamma=GAMMA, C_=COST, kernel=1)
    metric = "model pack + store + read s (%d support vectors)" % nsv
    cfg = {"workload": MODEL_IO_DESC % nsv, "support_vectors": nsv, "rows": hd.l, "form": "device model",
           "parallelism": "single GPU",
           "l2": "not flushed: the model (about %.0f MB) fits in L2, and the file writes dominate" %
                 (16 * (nsv + 13 * nsv) / 1e6)}
    d = tempfile.mkdtemp()
    path_h, path_d = os.path.join(d, "host.model"), os.path.join(d, "dev.model")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]

    def host_path():
        t0 = time.perf_counter()
        mdl = lib.calculateFULLModel(prop, hd.struct, beta.ctypes.data_as(PD))
        fp = libc.fopen(path_h.encode(), b"wb")
        lib.storeModel(C.byref(mdl), C.c_void_p(fp))
        libc.fclose(C.c_void_p(fp))
        m2 = _abi.Model()
        fp = libc.fopen(path_h.encode(), b"rb")
        lib.readModel(C.byref(m2), C.c_void_p(fp))
        libc.fclose(C.c_void_p(fp))
        dt = time.perf_counter() - t0
        lib.freeModel(mdl)
        lib.freeModel(m2)
        return dt

    if args.impl == "reference":
        dt = host_path()
        base = {"value": round(dt, 3), "unit": "s", "cores": 1, "kind": "port",
                "sample": "the reference's model packing and model file I/O restated (host C, single thread)"}
        print(json.dumps({"metric": metric, "value": base["value"], "unit": "s", "impl": "reference",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": base["value"] * 1000,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded generator)", "config": cfg, "cpu_baseline": base,
                          "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    lib.irwls_dmodel_full.restype = C.c_void_p
    lib.irwls_dmodel_full.argtypes = [C.c_void_p, _abi.Properties, PD]
    lib.irwls_dmodel_read.restype = C.c_void_p
    lib.irwls_dmodel_read.argtypes = [C.c_char_p]
    lib.irwls_dmodel_store.argtypes = [C.c_void_p, C.c_char_p]
    lib.irwls_dmodel_free.argtypes = [C.c_void_p]
    res = lib.irwls_resident_upload(hd.struct, prop, 0)

    def dev_path():
        lib.irwls_dev_sync()
        h0, d0 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h0), C.byref(d0))
        t0 = time.perf_counter()
        dm = lib.irwls_dmodel_full(res, prop, beta.ctypes.data_as(PD))
        if not dm or lib.irwls_dmodel_store(dm, path_d.encode()) != 0:
            raise SystemExit("device model failed: " + lib.irwls_last_error_message().decode())
        dm2 = lib.irwls_dmodel_read(path_d.encode())
        lib.irwls_dev_sync()
        dt = time.perf_counter() - t0
        h1, d1 = C.c_longlong(), C.c_longlong()
        lib.irwls_transfer_bytes(C.byref(h1), C.byref(d1))
        lib.irwls_dmodel_free(dm)
        lib.irwls_dmodel_free(dm2)
        return dt, h1.value - h0.value, d1.value - d0.value

    for _ in range(args.warmup):
        dev_path()
    launches0 = lib.irwls_kernel_launches()
    clocks = Clocks(0)
    clocks.start()
    times = []
    for _ in range(args.steps):
        dt, h2d, d2h = dev_path()
        times.append(dt)
    clk = clocks.stop()
    launches = lib.irwls_kernel_launches() - launches0
    host_s = host_path()
    identical = open(path_h, "rb").read() == open(path_d, "rb").read()
    value = statistics.mean(times)
    line = {"metric": metric, "value": round(value, 4), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1000, 2), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": cfg,
            "e2e": {"value": round(value, 4), "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "note": "from the resident dataset and host weights to a file "
                                                            "and back to a device model, file writes included"},
            "gpu_launches": int(launches // max(args.steps, 1)),
            "roofline": {"bound": "file I/O and host-device copies", "kernel": None, "achieved": None, "peak": None,
                         "unit": None, "frac": None, "traffic": None},
            "cpu_baseline": {"value": round(host_s, 4), "unit": "s", "cores": 1, "kind": "port",
                             "sample": "the reference's model packing and model file I/O restated (host C)"},
            "clocks": clk, "model_file_bytes": os.path.getsize(path_d), "identical_model_files": bool(identical)}
    print(json.dumps(line), flush=True)
    lib.irwls_resident_free(res)
    os.unlink(path_h)
    os.unlink(path_d)
    os.rmdir(d)


# ----------------------------------------------------------------------------
# learned-proposal form of SGMA
# ----------------------------------------------------------------------------
LEARN = dict(n=1_000_000, n_test=20_000, gamma=0.5, C=10.0, trace_sets=10, trace_rows=20_000, pool=4096)
LEARN_DESC = ("learned-proposal form, budgeted IRWLS (precision form): n=%d, d=32 dense (mixture of 50 seeded "
              "Gaussians with random covariances, labels by component parity, 3%% flipped), RBF gamma=0.5, C=10, "
              "budget m=%d; network 8-128-128-1 (ReLU) scores a %d-candidate pool per step and keeps the best 32 "
              "of each label (with 8 random ones of each label) for the exact SGMA score; trained on traces of "
              "SGMA on %d sets of %d rows (budget %d) with mixtures of their own, random candidates then on-policy")


def _row(hd, i):
    """(indices, values) of row i of a host svm_dataset."""
    import numpy as np

    idx, val = [], []
    p = hd.struct.x[i]
    k = 0
    while p[k].index != -1:
        idx.append(p[k].index)
        val.append(p[k].value)
        k += 1
    return np.asarray(idx), np.asarray(val)


def run_learned(args):
    import numpy as np

    from libirwls_gb300 import _abi, learned, load, synth

    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned-proposal form (its "
                          "random-candidate SGMA at 1M rows and budget 2000 runs for hours on the host)"}))
        return
    budget = args.budget if args.budget != BUDGET else 2000
    cfg = LEARN
    lib = load()
    if not lib.irwls_gpu_available():
        raise SystemExit("no CUDA device: " + lib.irwls_last_error_message().decode())
    libc = C.CDLL(None)
    # traces and the network
    t0 = time.perf_counter()
    runs = []
    # traces at the workload's budget: a candidate's state depends on how many
    # centroids cover its component, not on the dataset size
    tprops = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], size=budget, algorithm=1)
    for k in range(cfg["trace_sets"]):
        X, y = synth.gauss_mixture(cfg["trace_rows"], 1000 + k, family_seed=5000 + k)
        d = synth.from_dense(X, y, keep_zeros=True)
        runs.append((_abi.build_dataset(d.indptr, d.indices, d.values, d.y), tprops))
    lib.initMemory(1, budget)
    libc.srand(1)
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    net, n_trace = learned.fit(runs, seed=11, rounds=2, epochs=10, batch=1024, lr=1e-3, pool=cfg["pool"])
    net_s = time.perf_counter() - t0
    # the workload
    X, y = synth.gauss_mixture(cfg["n"] + cfg["n_test"], 77)
    tr = synth.from_dense(X[:cfg["n"]], y[:cfg["n"]], keep_zeros=True)
    te = synth.from_dense(X[cfg["n"]:], y[cfg["n"]:], keep_zeros=True)
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    p = _abi.make_properties(gamma=cfg["gamma"], C_=cfg["C"], size=budget, algorithm=1)
    res = lib.irwls_resident_upload(hd.struct, p, 1)
    if not res:
        raise SystemExit(lib.irwls_last_error_message().decode())
    lib.irwls_set_precision(1)
    out = {}
    clocks = Clocks(0)
    for form in ("random", "learned"):
        if form == "learned":
            net.install(pool=cfg["pool"])
        cent = np.zeros(budget, np.int32)
        w = np.zeros(budget)

        def step():
            libc.srand(1)
            if lib.irwls_resident_budgeted(res, p, cent.ctypes.data_as(PI), w.ctypes.data_as(PD)) != 0:
                raise SystemExit("training failed: " + lib.irwls_last_error_message().decode())

        for _ in range(args.warmup):
            step()
        if form == "learned":
            clocks.start()
            launches0 = lib.irwls_kernel_launches()
        times = []
        for _ in range(args.steps):
            lib.irwls_l2_flush(512 << 20)
            lib.irwls_timer_start()
            step()
            times.append(lib.irwls_timer_stop() / 1000.0)
        resid = lib.irwls_last_nystrom_residual()
        out[form] = {"s": statistics.mean(times), "residual": resid, "cent": cent.copy(), "w": w.copy()}
        net.uninstall()
    clk = clocks.stop()
    launches = lib.irwls_kernel_launches() - launches0
    lib.irwls_set_precision(0)
    lib.irwls_resident_free(res)
    # quality: primal objective (f from the library's prediction path) and held-out accuracy
    ytr = np.asarray(tr.y)
    for form, r in out.items():
        c = np.ascontiguousarray(r["cent"], dtype=np.int32)
        ww = np.ascontiguousarray(r["w"])
        mdl = lib.calculateBudgetedModel(p, hd.struct, c.ctypes.data_as(PI), ww.ctypes.data_as(PD))
        f = np.ctypeslib.as_array(lib.softTest(hd.struct, mdl, _abi.make_predict_properties(soft=1)),
                                  shape=(hd.l,)).copy()
        pred = np.ctypeslib.as_array(lib.test(ht.struct, mdl, _abi.make_predict_properties(soft=0)),
                                     shape=(ht.l,)).copy()
        lib.freeModel(mdl)
        Xc = np.zeros((budget, 33))
        for k, i in enumerate(c):
            ix, v = _row(hd, int(i))
            Xc[k, ix] = v
        sq = (Xc * Xc).sum(1)
        Kmm = np.exp(-cfg["gamma"] * np.maximum(sq[:, None] + sq[None, :] - 2 * Xc @ Xc.T, 0.0))
        r["primal"] = float(0.5 * ww @ (Kmm + 1e-5 * np.eye(budget)) @ ww +
                            cfg["C"] * np.maximum(0.0, 1.0 - ytr * f).sum())
        r["test_acc"] = float((pred == np.asarray(te.y)).mean())
    L, R = out["learned"], out["random"]
    line = {"metric": METRIC, "value": round(L["s"], 3), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(L["s"] * 1000, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 pieces x6 (SGMA scores) + f32 (network) + exact bf16 digit products (IRWLSpar Gram) + f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": LEARN_DESC % (cfg["n"], budget, cfg["pool"], cfg["trace_sets"], cfg["trace_rows"],
                                                 budget),
                       "n": cfg["n"], "d": 32, "budget": budget, "pool": cfg["pool"], "form": "learned proposals",
                       "parallelism": "single GPU", "l2": "flushed between timed steps"},
            "e2e": None, "gpu_launches": int(launches // max(args.steps, 1)),
            "roofline": {"bound": "see the budgeted workload's kernels", "kernel": None, "achieved": None,
                         "peak": None, "unit": None, "frac": None, "traffic": None},
            "cpu_baseline": None, "clocks": clk,
            "nystrom_residual": {"random_candidates": R["residual"], "learned_proposals": L["residual"],
                                 "reduction": 1.0 - L["residual"] / R["residual"]},
            "random_candidates_s": round(R["s"], 3),
            "primal": {"random": R["primal"], "learned": L["primal"],
                       "rel_change": (L["primal"] - R["primal"]) / abs(R["primal"])},
            "test_acc": {"random": R["test_acc"], "learned": L["test_acc"]},
            "network": {"trace_rows": int(n_trace), "sets_build_s": round(build_s, 2),
                        "traces_and_training_s": round(net_s, 2),
                        "rounds": "random-candidate traces, then on-policy traces of the first network"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload in FULL:
        run_full(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "linear_predict":
        run_linear_predict(args)
    elif args.workload == "parse":
        run_parse(args)
    elif args.workload == "model_io":
        run_model_io(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
