"""The allocation-free solve, irwls_chol_solve_noalloc, checked through the C
ABI against the library's regular solve (ParallelLinearSystem) on the same
systems.

It exists for callers that cannot let a library allocate device memory while
they run (a process whose pool allocator owns the device's memory, or code
that must not risk the device-wide synchronization of cudaMalloc/cudaFree).
Here the caller's buffers come from PyTorch, the stream is PyTorch's, and the
entry point only uses its own static scratch. It is called twice in a row on
two systems each time, because every call shares (and leaves behind) the same
scratch. This file runs last so that a stop at its first failure has already
run every other test; it also passes on its own in a fresh process (the first
call does the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import load

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
TOL = 1e-12  # the same kernels run on both paths; the results are expected bit-identical


def _entry(lib):
    f = lib.irwls_chol_solve_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def _regular_solve(lib, A, b):
    n = len(b)
    M = np.asfortranarray(A).ravel(order="F").copy()
    x = np.zeros(n)
    lib.ParallelLinearSystem(M.ctypes.data_as(PD), n, n, 0, 0, b.ctypes.data_as(PD), n, 1, 0, 0, n, 1,
                             x.ctypes.data_as(PD), n, 1, 0, 0, 1)
    return np.tril(M.reshape((n, n), order="F")), x


def test_noalloc_solve_matches_regular_solve():
    torch = pytest.importorskip("torch")
    lib = load()
    assert lib.irwls_gpu_available(), lib.irwls_last_error_message()
    solve = _entry(lib)
    z = np.load(H.GOLDEN + "/solver.npz")
    stream = torch.cuda.current_stream()
    for call in range(2):
        for key, want_info in (("solve_200_spd", 0), ("solve_251_bordered", 251)):
            A, b = z[key + "_A"], z[key + "_b"]
            n, ld = len(b), len(b) + 1
            L_ref, x_ref = _regular_solve(lib, A, b)
            # caller-owned device buffers: column-major with leading dimension ld
            cm = np.zeros((n, ld))
            cm[:, :n] = A.T
            dM = torch.tensor(cm, dtype=torch.float64, device="cuda")
            db = torch.tensor(b, dtype=torch.float64, device="cuda")
            dx = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
            dinfo = torch.full((1,), -1, dtype=torch.int32, device="cuda")
            rc = solve(dM.data_ptr(), n, ld, db.data_ptr(), dx.data_ptr(), dinfo.data_ptr(),
                       C.c_void_p(stream.cuda_stream))
            torch.cuda.synchronize()
            assert rc == 0, lib.irwls_last_error_message()
            x = dx.cpu().numpy()
            L = np.tril(dM.cpu().numpy()[:, :n].T)
            assert H.rel_err(x, x_ref) <= TOL, (call, key)
            assert H.rel_err(L, L_ref) <= TOL, (call, key)
            assert int(dinfo.item()) == want_info, (call, key)


def test_noalloc_rejects_orders_above_its_limit():
    lib = load()
    solve = _entry(lib)
    rc = solve(None, 4097, 4098, None, None, None, None)
    assert rc == -11
    assert b"4096" in lib.irwls_last_error_message()
