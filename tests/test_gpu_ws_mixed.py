"""The precision form's working-set solve of full IRWLS (irwls_ws_solve_mixed:
FP32 Cholesky inside one 16-CTA thread-block cluster, FP64 iterative
refinement), through the C ABI.

The reference solves the bordered system [H y; y^T 0] with dpotrf + dpotrs
(src/ParallelAlgorithms.c:361-388); its last pivot fails by construction and
the solve goes on with the stored Schur complement, which equals, in exact
arithmetic, x_n = (r_n - y^T H^-1 r) / s^2 and x = H^-1 r - H^-1 y x_n with
s = y^T H^-1 y. Checked here:

- the reference's own solution of a 251 x 251 bordered system (solver.npz,
  written by the reference build) within 1e-10;
- seeded working-set-like systems (RBF kernel block times the labels plus
  diag(1/a)) at orders 1 ... 512, including orders around the 32-row block
  edges, against that formula evaluated in FP64 with numpy;
- the orders and systems it hands back to the FP64 solve (return value 1):
  order 513, an H with a negative pivot;
- whole precision-form trainings (the 4000-row full-IRWLS golden case): the
  reference's support-vector set and its dual objective within 1e-9, with
  every working-set solve done by the cluster path.
"""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import load

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
TOL = 1e-11


def _lib():
    lib = load()
    assert lib.irwls_gpu_available(), lib.irwls_last_error_message()
    lib.irwls_ws_solve_mixed.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.irwls_ws_solve_mixed.restype = C.c_int
    lib.irwls_ws_mixed_counts.argtypes = [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.c_int]
    lib.irwls_ws_mixed_counts.restype = None
    return lib


def _counts(lib, reset=0):
    s, f = C.c_longlong(0), C.c_longlong(0)
    lib.irwls_ws_mixed_counts(C.byref(s), C.byref(f), reset)
    return s.value, f.value


def _solve(lib, M, rhs):
    """M: the (n1+1) x (n1+1) bordered matrix (lower triangle and row n1 are
    read); returns (status, x)."""
    torch = pytest.importorskip("torch")
    n = M.shape[0]
    ld = n + 3  # a leading dimension above the minimum
    A = np.zeros((n, ld))
    A[:, :n] = M.T  # column c of M is row c of A (column-major storage)
    dA = torch.tensor(A.ravel(), dtype=torch.float64, device="cuda")
    db = torch.tensor(rhs, dtype=torch.float64, device="cuda")
    dx = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = lib.irwls_ws_solve_mixed(dA.data_ptr(), n - 1, ld, db.data_ptr(), dx.data_ptr())
    torch.cuda.synchronize()
    assert float(dA.cpu().numpy().reshape(n, ld)[:, :n].T[0, 0]) == M[0, 0]  # H is left unmodified
    return st, dx.cpu().numpy()


def _schur(M, rhs):
    n1 = M.shape[0] - 1
    Hm = np.tril(M[:n1, :n1]) + np.tril(M[:n1, :n1], -1).T
    y = M[n1, :n1]
    u = np.linalg.solve(Hm, y)
    v = np.linalg.solve(Hm, rhs[:n1])
    s = y @ u
    xn = (rhs[n1] - y @ v) / (s * s)
    return np.concatenate([v - u * xn, [xn]])


def _system(n1, seed, d=8, gamma=0.5):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n1, d))
    y = np.where(rng.random(n1) < 0.5, -1.0, 1.0)
    sq = (X * X).sum(1)
    K = np.exp(-gamma * np.maximum(sq[:, None] + sq[None, :] - 2 * X @ X.T, 0.0))
    inv_a = rng.uniform(1e-3, 0.1, n1)
    M = np.zeros((n1 + 1, n1 + 1))
    M[:n1, :n1] = K * np.outer(y, y) + np.diag(inv_a)
    M[n1, :n1] = y
    M[:n1, n1] = y
    rhs = np.concatenate([rng.uniform(-1, 2, n1), [rng.uniform(-1, 1)]])
    return M, rhs


def test_reference_bordered_solution():
    lib = _lib()
    if lib.irwls_ws_mixed_max() == 0:
        pytest.skip("no 16-CTA cluster on this device")
    z = np.load(H.GOLDEN + "/solver.npz")
    M, b, want = z["solve_251_bordered_A"], z["solve_251_bordered_b"], z["solve_251_bordered_x"]
    st, x = _solve(lib, M, b)
    assert st == 0
    err = H.rel_err(x, want)
    print("251 bordered: rel err vs the reference %.3g" % err)
    assert err <= 1e-10


@pytest.mark.parametrize("n1", [1, 2, 31, 32, 33, 64, 100, 255, 449, 500, 511, 512])
def test_working_set_systems_match_fp64(n1):
    lib = _lib()
    if lib.irwls_ws_mixed_max() == 0:
        pytest.skip("no 16-CTA cluster on this device")
    M, rhs = _system(n1, 1000 + n1)
    st, x = _solve(lib, M, rhs)
    assert st == 0
    want = _schur(M, rhs)
    err = H.rel_err(x, want)
    print("n1=%d: rel err %.3g" % (n1, err))
    assert err <= TOL


def test_systems_handed_back_to_fp64():
    lib = _lib()
    if lib.irwls_ws_mixed_max() == 0:
        pytest.skip("no 16-CTA cluster on this device")
    assert lib.irwls_ws_mixed_max() == 512
    M, rhs = _system(513, 7)
    st, _ = _solve(lib, M, rhs)
    assert st == 1  # above the cluster's order
    M, rhs = _system(200, 8)
    M[37, 37] = -5.0  # H is not positive definite: the FP32 pivot of row 37 fails
    st, _ = _solve(lib, M, rhs)
    assert st == 1
    # the next system solves normally
    M, rhs = _system(200, 9)
    st, x = _solve(lib, M, rhs)
    assert st == 0 and H.rel_err(x, _schur(M, rhs)) <= TOL


def test_precision_full_training_uses_cluster_solves():
    lib = _lib()
    if lib.irwls_ws_mixed_max() == 0:
        pytest.skip("no 16-CTA cluster on this device")
    g = H.golden("full_cfg1")
    p = H.params(g)
    hd, _ = H.datasets(g)
    _counts(lib, reset=1)
    lib.irwls_set_precision(1)
    try:
        beta, _, _ = H.run_full(lib, hd, p)
    finally:
        lib.irwls_set_precision(0)
    solves, fallbacks = _counts(lib, reset=1)
    print("cluster solves %d, FP64 fallbacks %d, beta rel err %.3g" % (solves, fallbacks,
                                                                      H.rel_err(beta, g["beta"])))
    assert solves > 100 and fallbacks == 0
    assert np.array_equal(beta[:-1] != 0, g["beta"][:-1] != 0)
    d_ref = H.dual_objective(hd, g["beta"], p["gamma"], p["kernel"])
    d_got = H.dual_objective(hd, beta, p["gamma"], p["kernel"])
    assert abs(d_got - d_ref) <= 1e-9 * abs(d_ref)
