"""The allocation-free solve, irwls_chol_solve_noalloc, checked through the C
ABI against the library's regular solve (ParallelLinearSystem) on the same
systems.

It exists for callers that cannot let a library allocate device memory while
they run (a process whose pool allocator owns the device's memory, or code
that must not risk the device-wide synchronization of cudaMalloc/cudaFree).
Here the caller's buffers come from PyTorch, the stream is PyTorch's, and the
entry point only uses its own static scratch. It is called twice in a row on
two systems each time, because every call shares (and leaves behind) the same
scratch. The orders run up to the documented limit (4096, every diagonal
block of the scratch and a multi-CTA backward sweep), including one that is
not a multiple of 32, and the two modes without a right-hand side argument
(row n already filled) and without a solution (factor only). This file runs
last so that a stop at its first failure has already run every other test; it
also passes on its own in a fresh process (the first call does the per-device
set-up).
"""
import ctypes as C
import os
import subprocess
import sys

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


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    return A @ A.T + np.eye(n), rng.standard_normal(n)


def _device_system(torch, A, b, ld, with_rhs_row):
    n = len(b)
    cm = np.zeros((n, ld))
    cm[:, :n] = A.T
    if with_rhs_row:
        cm[:, n] = b
    return torch.tensor(cm, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("n", [4096, 4095, 1000])
def test_noalloc_large_orders_and_modes(n):
    torch = pytest.importorskip("torch")
    lib = load()
    assert lib.irwls_gpu_available(), lib.irwls_last_error_message()
    solve = _entry(lib)
    stream = torch.cuda.current_stream()
    A, b = _spd(n, n)
    L_ref, x_ref = _regular_solve(lib, A, b)
    ld = n + 1
    for call in range(2):
        # right-hand side already in row n (d_b = NULL)
        dM = _device_system(torch, A, b, ld, True)
        dx = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        dinfo = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        rc = solve(dM.data_ptr(), n, ld, None, dx.data_ptr(), dinfo.data_ptr(), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        assert rc == 0, lib.irwls_last_error_message()
        assert H.rel_err(dx.cpu().numpy(), x_ref) <= TOL, (call, n)
        assert H.rel_err(np.tril(dM.cpu().numpy()[:, :n].T), L_ref) <= TOL, (call, n)
        assert int(dinfo.item()) == 0
        # factor only (d_x = NULL)
        dM = _device_system(torch, A, b, ld, False)
        dinfo.fill_(-1)
        rc = solve(dM.data_ptr(), n, ld, None, None, dinfo.data_ptr(), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        assert rc == 0, lib.irwls_last_error_message()
        assert H.rel_err(np.tril(dM.cpu().numpy()[:, :n].T), L_ref) <= TOL, (call, n)
        assert int(dinfo.item()) == 0


def test_noalloc_first_call_keeps_the_cooperative_sweep():
    """In a fresh process whose first solve is the allocation-free one, the
    later solves still take the multi-CTA backward sweep."""
    code = ("import sys, ctypes as C; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import numpy as np, torch\n"
            "from libirwls_gb300 import load\n"
            "import test_zz_no_alloc as T\n"
            "lib = load(); solve = T._entry(lib)\n"
            "A, b = T._spd(600, 1); n = 600\n"
            "dM = T._device_system(torch, A, b, n + 1, True)\n"
            "dx = torch.zeros(n, dtype=torch.float64, device='cuda')\n"
            "assert solve(dM.data_ptr(), n, n + 1, None, dx.data_ptr(), None, None) == 0\n"
            "torch.cuda.synchronize()\n"
            "print(lib.irwls_chol_sweep_ctas(600), lib.irwls_chol_sweep_ctas(4096))\n"
            % (H.ROOT, os.path.dirname(os.path.abspath(__file__))))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ctas = [int(v) for v in r.stdout.split()[-2:]]
    assert ctas == [3, 16], ctas


def test_noalloc_leaves_a_pending_error_alone():
    """A CUDA error the caller left pending in its own runtime is neither
    consumed nor taken for one of the call's launches: the library links the
    CUDA runtime statically, so the caller's error state is not its own, and
    the call solves normally."""
    torch = pytest.importorskip("torch")
    lib = load()
    solve = _entry(lib)
    torch.zeros(1, device="cuda")
    cudart = None
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            cudart = C.CDLL(name)
            break
        except OSError:
            continue
    if cudart is None:
        pytest.skip("the caller's CUDA runtime is not loadable by name")
    A, b = _spd(64, 3)
    _, x_ref = _regular_solve(lib, A, b)
    dM = _device_system(torch, A, b, 65, True)
    dx = torch.zeros(64, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # a non-sticky error in the caller's runtime (an invalid device ordinal),
    # left pending across the call; no torch call runs until it is read back
    assert cudart.cudaSetDevice(C.c_int(100000)) != 0
    rc = solve(dM.data_ptr(), 64, 65, None, dx.data_ptr(), None, None)
    assert rc == 0, lib.irwls_last_error_message()
    assert cudart.cudaGetLastError() != 0
    assert cudart.cudaGetLastError() == 0
    torch.cuda.synchronize()
    assert H.rel_err(dx.cpu().numpy(), x_ref) <= TOL


def test_noalloc_rejects_orders_above_its_limit():
    lib = load()
    solve = _entry(lib)
    rc = solve(None, 4097, 4098, None, None, None, None)
    assert rc == -11
    assert b"4096" in lib.irwls_last_error_message()
