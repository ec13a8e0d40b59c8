"""Builds libirwls_gb300.so in-tree: CUDA sources with nvcc for sm_103a, host C
sources with gcc, linked into one shared library with the CUDA runtime
linked statically. Run ``python -m libirwls_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libirwls_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
                     *inc, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        # -ffp-contract=off: host arithmetic (dataset norms, class means) rounds
        # like the reference's x86 build on every host
        jobs.append(["gcc", "-O3", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-Wall", "-Wno-parentheses",
                     *inc, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [j[-1] for j in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lm", "-Xlinker", "-Bsymbolic"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
