"""The host model of the tensor-core Gram's arithmetic (tests/gram_digits.py),
checked on the CPU before it is used to pin the kernel bit for bit:

- the balanced base-128 digits rebuild N exactly and stay within +-64, so
  every digit product is exact in bf16 and a 512-row level sum stays below
  2^24;
- the fixed-point conversion rounds ties away from zero and drops subnormals;
- on integer columns below 2^20 the model is the exact integer product;
- on RBF-like columns with weights over six decades it is within the stated
  bound of the FP64 product, and the split-K chunking does not change it by
  more than the final roundings.
"""
import numpy as np

import gram_digits as gd

BIG = 1 << 30  # SM count: any part with at least P x tiles SMs chunks alike


def test_digits_rebuild_and_range():
    rng = np.random.default_rng(1)
    N = rng.integers(-(1 << 48), (1 << 48) + 1, size=20000)
    N[:6] = [1 << 48, -(1 << 48), (1 << 48) - 1, -(1 << 48) + 1, 0, (1 << 47) + (1 << 41)]
    d = gd.digits(N)
    back = sum(d[s] * (np.int64(128) ** s) for s in range(gd.GS))
    assert np.array_equal(back, N)
    for s in range(gd.GS - 1):
        assert d[s].min() >= -64 and d[s].max() <= 63
    assert np.abs(d[gd.GS - 1]).max() <= 64
    # a level over 512 rows: at most 7 pairs of products <= 64^2
    assert 7 * 512 * 64 * 64 < 1 << 24


def test_fixed48_rounding():
    e = 0
    q = 2.0 ** -49  # half a unit of the 48-bit fixed point at sigma = 1
    v = np.array([3 * q, -3 * q, 5 * q, -5 * q, q, 1.0, -1.0, 0.0, 1e-310, 2.0 ** -48])
    assert list(gd.fixed48(v, e)) == [2, -2, 3, -3, 1, 1 << 48, -(1 << 48), 0, 0, 1]
    assert list(gd.fixed48(v, None)) == [0] * len(v)


def test_column_exponents():
    A = np.array([[0.5, 0.0, -0.75, 1e-310, 3.0], [-0.25, 0.0, 0.1, 0.0, -4.0]])
    assert gd.column_exponents(A) == [-1, None, 0, None, 2]


def test_model_is_exact_on_integers():
    rng = np.random.default_rng(2)
    l, m, nact = 900, 70, 700
    KSC = rng.integers(-(1 << 20), 1 << 20, size=(l, m)).astype(np.float64)
    act = np.sort(rng.choice(l, nact, replace=False))
    day = rng.integers(-(1 << 20), 1 << 20, size=nact).astype(np.float64)
    KC = rng.integers(-1000, 1000, size=(m, m)).astype(np.float64)
    G = gd.gram(KSC, act, np.ones(nact), day, KC, 3, BIG)
    A = np.concatenate([KSC[act].astype(np.int64), day.astype(np.int64)[:, None]], axis=1)
    ref = (A.T @ A)[:, :m].astype(np.float64)
    ref[:m] += KC
    low = ~np.isnan(G)
    assert np.array_equal(G[low], ref[low])


def test_model_accuracy_and_chunking():
    rng = np.random.default_rng(3)
    l, m, nact = 1500, 90, 1300
    X = rng.standard_normal((l, 6))
    Cn = X[rng.choice(l, m, replace=False)]
    KSC = np.exp(-0.2 * ((X[:, None, :] - Cn[None, :, :]) ** 2).sum(-1))
    act = np.sort(rng.choice(l, nact, replace=False))
    sd = 10.0 ** rng.uniform(-3, 3, nact)
    day = rng.standard_normal(nact) * sd
    KC = np.zeros((m, m))
    G1 = gd.gram(KSC, act, sd, day, KC, 1, BIG)
    G4 = gd.gram(KSC, act, sd, day, KC, 4, BIG)
    assert gd.chunking(nact, m, 4, BIG)[0] == 4
    A = gd.column_values(KSC, act, sd, day)
    ref = (A.T @ A)[:, :m]
    sig = 2.0 ** np.ceil(np.log2(np.abs(A).max(0)))
    bound = 2.0 ** -40 * np.outer(sig, sig[:m]) * np.sqrt(nact)
    low = ~np.isnan(G1)
    assert np.all(np.abs(G1 - ref)[low] <= bound[low])
    # the chunks differ from one sum only by the roundings of the partials
    assert np.all(np.abs(G4 - G1)[low] <= 4 * 2.0 ** -52 * np.abs(ref)[low] + bound[low] * 2.0 ** -10)


def _fast_ceil_log2_product(a, b):
    """The column-scale rule of gram_colmax_kernel (prod_ceil_log2 in
    libirwls_gb300/csrc/dev_gram_tc.cu), restated: ceil(log2 |RN(a b)|) from
    the operands' exponents and an FP32 product of their leading 23 mantissa
    bits, or None where the kernel takes the FP64 product instead."""
    import struct
    ua = struct.unpack("<Q", struct.pack("<d", abs(a)))[0]
    ub = struct.unpack("<Q", struct.pack("<d", abs(b)))[0]
    Ea, Eb = ua >> 52, ub >> 52
    if not (Ea > 0 and Eb > 0 and 1030 <= Ea + Eb <= 3060):
        return None
    m52 = (1 << 52) - 1
    ma, mb = ua & m52, ub & m52
    e = Ea + Eb - 2046
    if ma == 0 and mb == 0:
        return e
    fa = np.frombuffer(struct.pack("<I", 0x3F800000 | (ma >> 29)), np.float32)[0]
    fb = np.frombuffer(struct.pack("<I", 0x3F800000 | (mb >> 29)), np.float32)[0]
    pr = np.float32(fa * fb)
    if pr <= np.float32(2.0) - np.float32(2.0 ** -18):
        return e + 1
    if np.float32(2.0) + np.float32(2.0 ** -17) <= pr <= np.float32(4.0) - np.float32(2.0 ** -17):
        return e + 2
    return None


def test_column_scale_rule_matches_exact_products():
    """Where the rule decides, it gives ceil(log2) of the FP64 product:
    random pairs over wide exponent ranges, and pairs built next to the
    mantissa products 2 and 4 (where rounding can land on a power of two and
    the kernel falls back to the FP64 product)."""
    rng = np.random.default_rng(17)
    pairs = [(rng.uniform(1, 2) * 2.0 ** rng.integers(-40, 40), rng.uniform(1, 2) * 2.0 ** rng.integers(-40, 40))
             for _ in range(20000)]
    for _ in range(4000):
        a = rng.uniform(1, 2)
        for t in (2.0, 4.0):
            for k in (-3, -1, 0, 1, 3):
                b = t / a
                pairs.append((a * 2.0 ** int(rng.integers(-8, 8)), b + k * np.spacing(b)))
    decided = 0
    for a, b in pairs:
        got = _fast_ceil_log2_product(a, b)
        if got is None:
            continue
        decided += 1
        v = abs(a * b)
        m, ex = np.frexp(v)  # v = m 2^ex, m in [0.5, 1)
        want = int(ex) - (1 if m == 0.5 else 0)
        assert got == want, (a, b, got, want)
    # the random pairs are decided by the rule; the built ones sit within
    # 2^-50 of the boundaries and go to the FP64 product
    assert decided >= 19900
