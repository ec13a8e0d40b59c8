"""The split-BF16 tcgen05 GEMM of the precision form (libirwls_gb300/csrc/
dev_tc.cu) against an FP64 product on the host.

Bar: every entry within 4e-5 * sum_k |a_ik b_jk| + 1e-6 of the exact product
(the hi/lo split keeps 16 significant bits per operand, so each product term
carries a relative error of about 2^-16; accumulation is FP32)."""
import ctypes as C

import numpy as np
import pytest

from libirwls_gb300 import load

pytestmark = pytest.mark.gpu


class Dev:
    def __init__(self, lib):
        self.lib = lib
        lib.irwls_dev_malloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        lib.irwls_dev_h2d.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        lib.irwls_dev_d2h.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        lib.irwls_dev_free.argtypes = [C.c_void_p]
        lib.irwls_split_bf16_f64.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                             C.c_int]
        lib.irwls_tc_gemm.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_longlong, C.c_int,
                                      C.c_int]
        self.bufs = []

    def alloc(self, nbytes):
        p = C.c_void_p()
        assert self.lib.irwls_dev_malloc(C.byref(p), nbytes) == 0
        self.bufs.append(p)
        return p

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = self.alloc(a.nbytes)
        self.lib.irwls_dev_h2d(p, a.ctypes.data, a.nbytes)
        return p

    def get(self, p, shape, dtype):
        out = np.empty(shape, dtype)
        self.lib.irwls_dev_d2h(out.ctypes.data, p, out.nbytes)
        assert self.lib.irwls_dev_sync() == 0
        return out

    def free(self):
        for p in self.bufs:
            self.lib.irwls_dev_free(p)


def _split(dev, X, ld):
    rows, cols = X.shape
    dX = dev.put(X)
    hi = dev.alloc(rows * ld * 2)
    lo = dev.alloc(rows * ld * 2)
    assert dev.lib.irwls_split_bf16_f64(dX, rows, cols, cols, hi, lo, ld) == 0
    return hi, lo


@pytest.mark.parametrize("M,N,K,bn,splits", [(128, 64, 64, 64, 1), (300, 64, 512, 64, 1), (257, 200, 640, 128, 1),
                                             (200, 200, 1024, 128, 4)])
def test_split_bf16_gemm(M, N, K, bn, splits):
    lib = load()
    assert lib.irwls_gpu_available()
    dev = Dev(lib)
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((N, K))
    ld = K
    ahi, alo = _split(dev, A, ld)
    bhi, blo = _split(dev, B, ld)
    Cd = dev.alloc(splits * M * N * 4)
    rc = lib.irwls_tc_gemm(ahi, alo, ld, M, bhi, blo, ld, N, K, Cd, N, splits, M * N, 0, bn)
    assert rc == 0, lib.irwls_last_error_message()
    got = dev.get(Cd, (splits, M, N), np.float32).astype(np.float64).sum(axis=0)
    assert lib.irwls_tc_status() == 0
    ref = A @ B.T
    bound = 4e-5 * (np.abs(A) @ np.abs(B).T) + 1e-6
    err = np.abs(got - ref)
    dev.free()
    assert np.all(err <= bound), float((err / bound).max())
