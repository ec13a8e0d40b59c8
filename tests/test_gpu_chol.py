"""The two Cholesky factorizations of the library give the same bits: the
data-flow one (one cooperative launch; a tile takes each panel's update as
soon as that panel is published) and the multi-launch panel sequence. Checked
through ParallelLinearSystem (reference src/ParallelAlgorithms.c:361-388) on
SPD and bordered systems of orders around the 32-column panel boundaries and
up to 2049, the right-hand side riding along as row n or not; and against
the reference's own solves in the solver fixture."""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import load

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)


def _solve(lib, A, b, path):
    lib.irwls_debug_chol_path(path)
    try:
        n = len(b)
        M = np.asfortranarray(A).ravel(order="F").copy()
        x = np.zeros(n)
        lib.ParallelLinearSystem(M.ctypes.data_as(PD), n, n, 0, 0, b.ctypes.data_as(PD), n, 1, 0, 0, n, 1,
                                 x.ctypes.data_as(PD), n, 1, 0, 0, 1)
        assert lib.irwls_last_error() in (0, 1), lib.irwls_last_error_message()
        return M.reshape((n, n), order="F"), x
    finally:
        lib.irwls_debug_chol_path(0)


def _factor(lib, A, path):
    lib.irwls_debug_chol_path(path)
    try:
        n = A.shape[0]
        M = np.asfortranarray(A).ravel(order="F").copy()
        lib.ParallelChol(M.ctypes.data_as(PD), n, n, 0, 0, n, 1, 0)
        return M.reshape((n, n), order="F")
    finally:
        lib.irwls_debug_chol_path(0)


def _system(n, bordered, seed):
    rng = np.random.default_rng(seed)
    if bordered:
        m = n - 1
        X = rng.standard_normal((m, 4))
        K = np.exp(-0.3 * ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
        yv = np.where(rng.random(m) < 0.5, 1.0, -1.0)
        H_ = np.zeros((n, n))
        H_[:m, :m] = K * np.outer(yv, yv) + np.diag(1.0 / (rng.random(m) * 5 + 0.01))
        H_[:m, m] = yv
        H_[m, :m] = yv
    else:
        A = rng.standard_normal((n, n)) / np.sqrt(n)
        H_ = A @ A.T + np.eye(n)
    return H_, rng.standard_normal(n)


@pytest.mark.parametrize("n,bordered", [(1, False), (5, False), (31, False), (32, False), (33, True), (64, False),
                                        (65, True), (200, False), (251, True), (500, False), (501, True),
                                        (1000, False), (1024, False), (2049, False)])
def test_dataflow_and_multilaunch_factorizations_agree_bitwise(n, bordered):
    lib = load()
    A, b = _system(n, bordered, n)
    L1, x1 = _solve(lib, A, b, 1)
    L2, x2 = _solve(lib, A, b, 2)
    assert np.array_equal(np.tril(L1), np.tril(L2))
    assert np.array_equal(x1, x2)
    F1 = _factor(lib, A, 1)
    F2 = _factor(lib, A, 2)
    assert np.array_equal(F1, F2)
    assert np.array_equal(np.tril(F1), np.tril(L1))


def test_dataflow_matches_reference_solves():
    lib = load()
    z = np.load(H.GOLDEN + "/solver.npz")
    for key in ("solve_5_spd", "solve_37_spd", "solve_64_spd", "solve_200_spd", "solve_9_bordered",
                "solve_51_bordered", "solve_251_bordered"):
        L, x = _solve(lib, z[key + "_A"], z[key + "_b"], 2)
        assert H.rel_err(x, z[key + "_x"]) <= 1e-10, key
        assert H.rel_err(np.tril(L), np.tril(z[key + "_L"])) <= 1e-10, key
