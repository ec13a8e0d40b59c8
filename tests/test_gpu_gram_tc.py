"""The tensor-core Gram of the precision form's IRWLSpar
(libirwls_gb300/csrc/dev_gram_tc.cu): K1 = KC + A'^T A' with
A' = [sd * KSC[act, :], day], from exact base-128 integer digits.

- Exactness: with integer entries below 2^20 every value is exact in the
  48-bit fixed point of its column and every sum below 2^53, so the result must
  equal the int64 product bit for bit -- across drains (one split-K chunk of
  2500 rows: five drains of 512 rows) and across chunks.
- Accuracy on RBF-like data with weights spread over six decades, against an
  FP64 product: |G - G_ref|_ij <= 2^-40 sigma_i sigma_j sqrt(nact), sigma the
  column scales (the dropped digit levels weigh about 2^-46 sigma_i sigma_j per row
  and carry random signs).
- Bit for bit on real-valued data: every step of the kernel is exact or
  correctly rounded, so K1 must equal the host model of its arithmetic
  (tests/gram_digits.py) -- RBF-like columns with weights over six decades;
  and columns that hit the edge cases: ties of the fixed-point rounding, a
  power-of-two and a just-above maximum, a zero column, subnormal entries,
  tiny columns, a constant column whose integer sum passes 2^63, and column
  maxima that are products rounding onto or next to a power of two (the
  column scales' exact fallback).
- No active rows: K1 = KC.
"""
import ctypes as C

import numpy as np
import pytest

import gram_digits as gd
from libirwls_gb300 import load

pytestmark = pytest.mark.gpu

VP = C.c_void_p


def _lib():
    lib = load()
    lib.irwls_dev_malloc.argtypes = [C.POINTER(VP), C.c_size_t]
    lib.irwls_dev_h2d.argtypes = [VP, VP, C.c_size_t]
    lib.irwls_dev_d2h.argtypes = [VP, VP, C.c_size_t]
    lib.irwls_dev_memset.argtypes = [VP, C.c_int, C.c_size_t]
    lib.irwls_dev_free.argtypes = [VP]
    lib.irwls_par_gram_tc_bytes.restype = C.c_size_t
    lib.irwls_par_gram_tc_bytes.argtypes = [C.c_int, C.c_int]
    lib.irwls_par_gram_part_bytes.restype = C.c_size_t
    lib.irwls_par_gram_part_bytes.argtypes = [C.c_int, C.c_int]
    lib.irwls_par_gram_tc.argtypes = [VP, C.c_int, VP, C.c_int, VP, VP, VP, VP, C.c_int, VP, C.c_int, VP]
    return lib


def _gram(KSC, act, sd, day, KC, P):
    lib = _lib()
    l, m = KSC.shape
    nact = len(act)
    ld = m + 1
    bufs = []

    def alloc(n):
        p = VP()
        assert lib.irwls_dev_malloc(C.byref(p), max(int(n), 16)) == 0
        bufs.append(p)
        return p

    def put(a):
        a = np.ascontiguousarray(a)
        p = alloc(a.nbytes)
        if a.nbytes:
            lib.irwls_dev_h2d(p, a.ctypes.data, a.nbytes)
        return p

    try:
        dK, dact, dsd, dday, dKC = put(KSC), put(act.astype(np.int32)), put(sd), put(day), put(KC)
        dK1 = alloc(ld * ld * 8)
        lib.irwls_dev_memset(dK1, 0, ld * ld * 8)
        dpart = alloc(lib.irwls_par_gram_part_bytes(m, P))
        dws = alloc(lib.irwls_par_gram_tc_bytes(l, m))
        assert lib.irwls_par_gram_tc(dK, m, dact, nact, dsd, dday, dKC, dK1, ld, dpart, P, dws) == 0
        K1 = np.empty((ld, ld))
        lib.irwls_dev_d2h(K1.ctypes.data, dK1, K1.nbytes)
        assert lib.irwls_dev_sync() == 0, lib.irwls_last_error_message()
    finally:
        for p in bufs:
            lib.irwls_dev_free(p)
    # column-major: element (r, c) at K1[c, r]; rows 0..m, columns c <= r, c < m
    G = np.full((m + 1, m), np.nan)
    for c in range(m):
        G[c:, c] = K1[c, c:]
    return G


def _lower(M):
    r, c = np.indices(M.shape)
    return c <= r


@pytest.mark.parametrize("P", [1, 6])
@pytest.mark.parametrize("l,m,nact", [(3000, 200, 2500), (700, 129, 333)])
def test_gram_tc_exact_on_integers(l, m, nact, P):
    rng = np.random.default_rng(l + m + P)
    KSC = rng.integers(-(1 << 20), 1 << 20, size=(l, m)).astype(np.float64)
    act = np.sort(rng.choice(l, nact, replace=False))
    sd = np.ones(nact)
    day = rng.integers(-(1 << 20), 1 << 20, size=nact).astype(np.float64)
    KC = rng.integers(-1000, 1000, size=(m, m)).astype(np.float64)
    G = _gram(KSC, act, sd, day, KC, P)
    A = np.concatenate([KSC[act].astype(np.int64), day.astype(np.int64)[:, None]], axis=1)
    ref = (A.T @ A)[:, :m].astype(np.float64)
    ref[:m] += KC
    low = _lower(G)
    assert np.array_equal(G[low], ref[low])


def test_gram_tc_accuracy_rbf_like():
    rng = np.random.default_rng(7)
    l, m, nact = 6000, 300, 5200
    X = rng.standard_normal((l, 12))
    Cn = X[rng.choice(l, m, replace=False)]
    d2 = ((X[:, None, :] - Cn[None, :, :]) ** 2).sum(-1)
    KSC = np.exp(-0.1 * d2)
    act = np.sort(rng.choice(l, nact, replace=False))
    sd = 10.0 ** rng.uniform(-3, 3, nact)
    day = rng.standard_normal(nact) * sd
    KC = np.exp(-0.1 * ((Cn[:, None, :] - Cn[None, :, :]) ** 2).sum(-1))
    G = _gram(KSC, act, sd, day, KC, 4)
    A = np.concatenate([sd[:, None] * KSC[act], day[:, None]], axis=1)
    ref = (A.T @ A)[:, :m]
    ref[:m] += KC
    sig = 2.0 ** np.ceil(np.log2(np.abs(A).max(0)))
    bound = 2.0 ** -40 * np.outer(sig, sig[:m]) * np.sqrt(nact)
    low = _lower(G)
    err = np.abs(G - ref)
    assert np.all(err[low] <= bound[low]), float(np.max(err[low] / bound[low]))


def test_gram_tc_no_active_rows():
    rng = np.random.default_rng(3)
    l, m = 100, 70
    KSC = rng.random((l, m))
    KC = rng.random((m, m))
    G = _gram(KSC, np.zeros(0, np.int32), np.zeros(0), np.zeros(0), KC, 4)
    low = _lower(G[:m])
    assert np.array_equal(G[:m][low], KC[low])
    assert np.all(G[m] == 0.0)


def _rbf_case(rng):
    l, m, nact = 6000, 300, 5200
    X = rng.standard_normal((l, 12))
    Cn = X[rng.choice(l, m, replace=False)]
    KSC = np.exp(-0.1 * ((X[:, None, :] - Cn[None, :, :]) ** 2).sum(-1))
    act = np.sort(rng.choice(l, nact, replace=False))
    sd = 10.0 ** rng.uniform(-3, 3, nact)
    day = rng.standard_normal(nact) * sd
    KC = np.exp(-0.1 * ((Cn[:, None, :] - Cn[None, :, :]) ** 2).sum(-1))
    return KSC, act, sd, day, KC


def _edge_case(rng):
    l, m, nact = 3000, 129, 2500
    act = np.sort(rng.choice(l, nact, replace=False))
    KSC = rng.uniform(-1, 1, (l, m))
    KSC[:, 0] = 1.0                                          # constant: T(0, 0) = 2500 * 2^52 > 2^63
    KSC[:, 1] = (2 * rng.integers(-2 ** 20, 2 ** 20, l) + 1) * 2.0 ** -49  # ties at sigma = 1/2
    KSC[act[0], 1] = 0.5                                     # power-of-two maximum
    KSC[:, 2] = 0.0                                          # zero column
    KSC[:, 3] *= 2.0 ** -200                                 # tiny column
    KSC[::7, 3] = 1e-310                                     # subnormal entries
    KSC[:, 4] = np.clip(KSC[:, 4], -0.5, 0.5)
    KSC[act[5], 4] = np.nextafter(0.5, 1.0)                  # maximum just above a power of two
    sd = np.ones(nact)
    day = rng.standard_normal(nact)
    KC = rng.standard_normal((m, m))
    return KSC, act, sd, day, KC


def _scale_boundary_case(rng):
    """Columns whose largest entry sd_i * KSC_ic is an FP64 product that
    rounds onto, just below or just above a power of two, so that the column
    scale comes from the kernel's exact fallback next to those boundaries."""
    l, m, nact = 2000, 65, 1800
    act = np.sort(rng.choice(l, nact, replace=False))
    sd = rng.uniform(1.0, 2.0, nact)
    KSC = rng.uniform(-1.0, 1.0, (l, m)) * 0.2
    for c in range(1, m - 1):
        p = int(rng.integers(nact))
        target = 2.0 ** int(rng.integers(-4, 4))
        k = target / sd[p]
        k += int(rng.integers(-3, 4)) * np.spacing(k)
        KSC[:, c] *= target
        KSC[act[p], c] = k if c % 2 else -k
    day = rng.standard_normal(nact)
    KC = rng.standard_normal((m, m))
    return KSC, act, sd, day, KC


@pytest.mark.parametrize("P", [1, 4])
@pytest.mark.parametrize("make", [_rbf_case, _edge_case, _scale_boundary_case])
def test_gram_tc_bit_exact_against_host_model(make, P):
    KSC, act, sd, day, KC = make(np.random.default_rng(11))
    G = _gram(KSC, act, sd, day, KC, P)
    # the split-K chunks: the same on any part with at least P x tiles SMs
    ref = gd.gram(KSC, act, sd, day, KC, P, 1 << 30)
    low = _lower(G)
    assert np.array_equal(np.isnan(ref), ~low)
    assert np.array_equal(G[low].view(np.int64), ref[low].view(np.int64)), int(
        np.sum(G[low].view(np.int64) != ref[low].view(np.int64)))
