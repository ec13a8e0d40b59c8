"""The three bf16 pieces of the precision form's SGMA operands
(libirwls_gb300/csrc/blocked_bf16.cuh, bf16_pieces3), restated on the host:
hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid), each subtraction
exact in FP32, so that hi + mid + lo == x for every FP32 x the form stores
(|x| above 2^-100 here: Q and W entries are bounded by one), and the six
piece products the score kernel keeps leave out only terms below about
2^-24 of the product."""
import numpy as np


def bf16(x):
    """Round FP32 values to bf16 (nearest, ties to even), as FP32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def pieces(x):
    x = np.asarray(x, np.float32)
    hi = bf16(x)
    r1 = (x - hi).astype(np.float32)
    mid = bf16(r1)
    lo = bf16((r1 - mid).astype(np.float32))
    return hi, mid, lo


def test_pieces_rebuild_fp32_exactly():
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(200000) * 10.0 ** rng.uniform(-30, 1, 200000)).astype(np.float32)
    x[:4] = [1.0, -1.0, np.float32(1.0) - np.float32(2.0 ** -24), np.float32(2.0 ** -100)]
    # below about 2^-102 the lo piece would be an FP32 subnormal
    x = x[np.abs(x) >= np.float32(2.0 ** -100)]
    hi, mid, lo = pieces(x)
    # each piece is a bf16 value and the subtractions were exact
    for p in (hi, mid, lo):
        assert np.array_equal(bf16(p), p)
    assert np.array_equal(((hi + mid).astype(np.float32) + lo).astype(np.float32), x)


def test_dropped_products_are_below_2_pow_minus_24():
    rng = np.random.default_rng(6)
    q = rng.uniform(-1, 1, 50000).astype(np.float32)
    w = rng.uniform(-1, 1, 50000).astype(np.float32)
    qh, qm, ql = pieces(q)
    wh, wm, wl = pieces(w)
    kept = (qh.astype(np.float64) * wh + qh.astype(np.float64) * wm + qm.astype(np.float64) * wh
            + qh.astype(np.float64) * wl + qm.astype(np.float64) * wm + ql.astype(np.float64) * wh)
    exact = q.astype(np.float64) * w.astype(np.float64)
    assert np.all(np.abs(kept - exact) <= 2.0 ** -23 * np.abs(exact) + 1e-300)
