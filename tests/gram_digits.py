"""Host model of the arithmetic of the tensor-core Gram
(libirwls_gb300/csrc/dev_gram_tc.cu, irwls_par_gram_tc), for tests.

Every step of that kernel is exact or correctly rounded, so its output is a
function of the inputs alone and this model reproduces it bit for bit:

1. v_pc = fl(sd_p * KSC[act_p, c]) for c < m, day_p for c = m; column scale
   sigma_c = 2^e_c, the smallest power of two >= max_p |v_pc| (e = None: the
   column is zero or subnormal);
2. N_pc = round(v_pc * 2^(48 - e_c)), ties away from zero, subnormal v -> 0;
   N in 7 balanced base-128 digits d_0 .. d_6 (d_s in [-64, 63], d_6 the rest);
3. per split-K chunk z (16-row stages [z spc, (z + 1) spc)), the integer
   T_z(i, j) = sum_p sum_{s + t >= 6} 128^(s + t - 6) d_s(p, i) d_t(p, j);
4. part_z = ldexp(fma(double(hi), 2^32, lo), e_i + e_j - 54), T = hi 2^32 + lo;
5. K1 = ((0 + part_0) + part_1 + ...) + KC (row m: no KC).

The digit-level products are formed in FP64 matrix products: every entry is
an integer sum below 2^53, so they are exact whatever the BLAS order.
"""
import math

import numpy as np

GS, GBITS, GFRAC, GM, GN, GBK = 7, 7, 48, 128, 64, 16
GSCALE = 2 * GFRAC - GBITS * (GS - 1)


def column_values(KSC, act, sd, day):
    """A' = [sd * KSC[act, :], day] as the kernel forms it (one IEEE product)."""
    act = np.asarray(act, dtype=np.int64)
    return np.concatenate([np.asarray(sd)[:, None] * KSC[act], np.asarray(day)[:, None]], axis=1)


def column_exponents(A):
    """e_c with sigma_c = 2^e_c >= max |A'_.c|, or None for a zero column."""
    out = []
    for c in range(A.shape[1]):
        mx = float(np.abs(A[:, c]).max()) if A.shape[0] else 0.0
        if mx < 2.2250738585072014e-308:  # zero or subnormal maximum
            out.append(None)
            continue
        mant, ex = math.frexp(mx)  # mx = mant 2^ex, mant in [0.5, 1)
        out.append(ex - 1 if mant == 0.5 else ex)
    return out


def fixed48(v, e):
    """round(v 2^(48 - e)) for a column v with |v| <= 2^e, from the bits of
    each entry: ties away from zero, subnormal entries -> 0."""
    v = np.asarray(v, dtype=np.float64)
    if e is None:
        return np.zeros(v.shape, dtype=np.int64)
    mant, ex = np.frexp(np.abs(v))
    M = (mant * 2.0 ** 53).astype(np.int64)  # |v| = M 2^(ex - 53), M < 2^53
    sh = 53 - ex.astype(np.int64) + e - GFRAC
    normal = np.abs(v) >= 2.2250738585072014e-308
    assert np.all(sh[normal] >= 4)
    shc = np.clip(sh, 1, 63)
    N = np.where(normal & (sh < 64), (M + (np.int64(1) << (shc - 1))) >> shc, 0)
    return np.where(v < 0, -N, N)


def digits(N):
    """Balanced base-128 digits d_0 .. d_6 of N (int64 arrays)."""
    out = []
    N = N.copy()
    base = 1 << GBITS
    for s in range(GS - 1):
        d = N & (base - 1)
        d = np.where(d >= base // 2, d - base, d)
        out.append(d)
        N = (N - d) >> GBITS
    out.append(N)
    return out


def chunking(nact, m, P, sms):
    """(pz, spc): the split-K chunks irwls_par_gram_tc uses."""
    ct, nt = -(-(m + 1) // GM), -(-m // GN)
    npb = -(-max(nact, 1) // GBK)
    tiles = sum(1 for i in range(ct) for j in range(nt) if GN * j <= GM * i + GM - 1)
    pz = max(1, min(P, sms // max(tiles, 1)))
    pz = min(pz, npb)
    spc = -(-npb // pz)
    return -(-npb // spc), spc


def gram(KSC, act, sd, day, KC, P, sms):
    """The (m + 1) x m lower part of K1 as irwls_par_gram_tc returns it
    (entries above the diagonal NaN)."""
    m = KSC.shape[1]
    nact = len(act)
    A = column_values(KSC, act, sd, day)
    es = column_exponents(A)
    N = np.zeros(A.shape, dtype=np.int64)
    for c in range(m + 1):
        N[:, c] = fixed48(A[:, c], es[c])
    D = [d.astype(np.float64) for d in digits(N)]
    pz, spc = chunking(nact, m, P, sms)
    total = np.zeros((m + 1, m))
    for z in range(pz):
        r0, r1 = z * spc * GBK, min(nact, (z + 1) * spc * GBK)
        T = None
        for u in range(2 * (GS - 1), GS - 2, -1):  # Horner from the top level
            L = np.zeros((m + 1, m))
            for s in range(u - (GS - 1), GS):
                L += D[s][r0:r1].T @ D[u - s][r0:r1, :m]
            Li = L.astype(np.int64).astype(object)
            T = Li if T is None else T * (1 << GBITS) + Li
        part = np.zeros((m + 1, m))
        for i in range(m + 1):
            for j in range(min(i + 1, m)):
                if es[i] is None or es[j] is None:
                    continue
                t = int(T[i, j])
                hi, lo = t >> 32, t & 0xFFFFFFFF
                td = float(int(float(hi)) * (1 << 32) + lo)
                part[i, j] = math.ldexp(td, es[i] + es[j] - GSCALE)
        total = total + part
    out = total.copy()
    out[:m] += KC
    r, c = np.indices(out.shape)
    out[c > r] = np.nan
    return out
