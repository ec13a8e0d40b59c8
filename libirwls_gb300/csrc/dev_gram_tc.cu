// dev_gram_tc.cu -- the precision form's IRWLSpar Gram on the tensor cores,
// through exact integer slices.
//
//   G = A'^T A',   A' = [sd * KSC[act, :], day]   (nact x (m + 1)),
//
// the K1/K2 system of IRWLSpar (reference src/budgeted-train.c:379-430).
// FP64 on this part runs at about 1/64 of the FP32 rate, so the product is
// formed on the bf16 tensor cores with every partial sum exact:
//
// 1. Each column c of A' gets a power of two sigma_c >= max_p |A'_pc| (a
//    column-max pass), and each entry becomes the integer
//    N_pc = round(A'_pc / sigma_c * 2^48), |N| <= 2^48, by integer operations
//    on its bits. N is written in 7 balanced base-128 digits d_0 .. d_6
//    (d_0 lowest), |d_s| <= 64: small integers, exact in bf16.
// 2. sum_p N_pi N_pj = sum_u 128^u L_u(i, j), L_u = sum_{s+t=u} sum_p
//    d_s(p,i) d_t(p,j). The levels u = 6 ... 12 are kept (28 digit pairs);
//    the dropped levels weigh at most about 2^-46 of the top one, so each
//    entry of G carries an error of about 2^-46 max|A'_.i| max|A'_.j| per
//    row, the accuracy of the double-float Gram this replaces.
// 3. A CTA owns a 128 x 64 tile of G and one split-K chunk of the rows. Per
//    16-row stage the 28 digit-pair products go to 7 level accumulators of
//    128 x 64 FP32 in tensor memory (448 of its 512 columns). Every product
//    is an integer of magnitude <= 64^2 = 4096 and a level sums at most 7
//    pairs, so over 512 rows every partial sum is an integer below
//    7 * 512 * 4096 < 2^24: exact in FP32, whatever the order of
//    accumulation. Every 512 rows the epilogue drains the levels into a
//    96-bit integer per entry (T += sum_u 128^(u-6) L_u), so the whole sum
//    stays exact.
// 4. G_ij = sigma_i sigma_j 2^-54 T_ij, written as the FP64 partials that
//    gram_reduce_kernel adds to KC.
//
// Operands reach shared memory by bulk copies: the slices are stored in the
// shared-memory image of a stage (per 128-column tile and 16-row block, the 8
// digit pieces of 128 x 16 in canonical K-major core-matrix order). Warp 0
// copies, lane 0 of warp 1 issues the MMAs, warps 4-11 drain. Every wait is
// bounded; a timeout sets device flag word 1.
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "dev_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int GS = 7;                  // digits per entry
constexpr int GBITS = 7;               // digit base 2^7
constexpr int GFRAC = 48;              // N = round(v * 2^48), |v| <= 1
constexpr int GPAIRS = GS * (GS + 1) / 2;            // digit pairs of the kept levels
constexpr int GSCALE = 2 * GFRAC - GBITS * (GS - 1);  // G = sigma_i sigma_j 2^-GSCALE T
constexpr int GM = 128, GN = 64;       // tile of G: rows (A' columns) x columns
constexpr int GBK = 16;                // rows of A' per stage
constexpr int GPIECE = GM * GBK;       // elements of one digit piece (4 KB)
constexpr int GDRAIN = 32;             // stages between drains (512 rows)
constexpr int GNS = 5;                 // ring stages
constexpr int G_THREADS = 384;
constexpr uint32_t A_STAGE = GS * GPIECE * 2;      // 28 KB: 7 pieces of 128 rows
constexpr uint32_t B_PIECE = GN * GBK * 2;         // 2 KB: 64 rows of one piece
constexpr uint32_t G_STAGE = A_STAGE + GS * B_PIECE;  // 42 KB
static_assert(GS * 64 <= 512, "level accumulators exceed tensor memory");
static_assert((long long)GS * GDRAIN * GBK * (1 << (2 * (GBITS - 1))) < (1LL << 24), "level sums must stay exact");

// Element offset of (row r of the 128-row tile, k of the 16-row block) in a
// digit piece: 8 x 8 core matrices, 128 bytes apart along k, 256 along r.
__device__ __forceinline__ int piece_off(int r, int k) { return (r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); }

// ceil(log2 |v|) from the bits of a normal double v: its exponent, plus one
// unless v is a power of two.
__device__ __forceinline__ int ceil_log2_bits(unsigned long long b) {
    return (int)((b >> 52) & 0x7ff) - 1023 + ((b & ((1ULL << 52) - 1)) != 0 ? 1 : 0);
}

constexpr int NO_EXP = -2000;  // zero or subnormal: no scale

// ceil(log2 |v|) of v = RN(a * b), the FP64 product, or NO_EXP when v is zero
// or subnormal. Away from the products whose rounding can land on a power
// of two (mantissa products within 2^-18 of 2 or 4) and from the exponent
// range's ends, it follows from the operands' exponents and an FP32 product
// of their leading mantissa bits (relative error below 2^-21), with no FP64
// operation; the rest take the FP64 product.
__device__ __forceinline__ int prod_ceil_log2(double a, double b) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffULL;
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b) & 0x7fffffffffffffffULL;
    const int Ea = (int)(ua >> 52), Eb = (int)(ub >> 52);
    if (Ea > 0 && Eb > 0 && Ea + Eb >= 1030 && Ea + Eb <= 3060) {
        const unsigned long long ma = ua & ((1ULL << 52) - 1), mb = ub & ((1ULL << 52) - 1);
        const int e = Ea + Eb - 2046;  // exponent of the product of the leading ones
        if (ma == 0 && mb == 0) return e;  // two powers of two: the exact product
        const float pr = __uint_as_float(0x3f800000u | (uint32_t)(ma >> 29)) *
                         __uint_as_float(0x3f800000u | (uint32_t)(mb >> 29));
        if (pr <= 2.0f - 0x1p-18f) return e + 1;                       // in (1, 2): not a power of two
        if (pr >= 2.0f + 0x1p-17f && pr <= 4.0f - 0x1p-17f) return e + 2;  // in (2, 4)
    }
    const unsigned long long v = (unsigned long long)__double_as_longlong(__dmul_rn(a, b)) & 0x7fffffffffffffffULL;
    return (v >> 52) == 0 ? NO_EXP : ceil_log2_bits(v);
}

// Column scales of A': per column the largest ceil(log2 |v|) over the active
// rows, stored as the bits of 2^that (so that col_exp reads it back; a
// column with no normal entry stays 0). A CTA takes GCM rows and a block of
// 1024 columns (all of a row's columns when m < 1024: one contiguous stream
// per row), thread t the columns t, t + 256, ... of the block; two rows'
// loads in flight. The maximum does not depend on the order the entries are
// visited in.
constexpr int GCM = 64;
__global__ void __launch_bounds__(256) gram_colmax_kernel(const double *__restrict__ KSC, int m,
                                                          const int *__restrict__ act, int nact,
                                                          const double *__restrict__ sd,
                                                          const double *__restrict__ day,
                                                          unsigned long long *__restrict__ cmax) {
    constexpr int CPT = 4;  // columns per thread: 1024 per block
    const int p0 = blockIdx.x * GCM, p1 = min(nact, p0 + GCM);
    const int cb = 1024 * blockIdx.y;
    int mx[CPT];
#pragma unroll
    for (int u = 0; u < CPT; ++u) mx[u] = NO_EXP;
    auto visit = [&](int p, const double *x) {
#pragma unroll
        for (int u = 0; u < CPT; ++u) {
            const int c = cb + threadIdx.x + 256 * u;
            int k = NO_EXP;
            if (c < m) {
                k = prod_ceil_log2(sd[p], x[u]);
            } else if (c == m) {
                const unsigned long long b = (unsigned long long)__double_as_longlong(day[p]) & 0x7fffffffffffffffULL;
                k = (b >> 52) == 0 ? NO_EXP : ceil_log2_bits(b);
            }
            mx[u] = k > mx[u] ? k : mx[u];
        }
    };
    for (int p = p0; p < p1; p += 2) {
        double x0[CPT], x1[CPT];
        const double *r0 = KSC + (size_t)act[p] * m, *r1 = KSC + (size_t)act[p + 1 < p1 ? p + 1 : p] * m;
#pragma unroll
        for (int u = 0; u < CPT; ++u) {
            const int c = cb + threadIdx.x + 256 * u;
            x0[u] = c < m ? r0[c] : 0.0;
            x1[u] = c < m ? r1[c] : 0.0;
        }
        visit(p, x0);
        if (p + 1 < p1) visit(p + 1, x1);
    }
#pragma unroll
    for (int u = 0; u < CPT; ++u) {
        const int c = cb + threadIdx.x + 256 * u;
        if (c <= m && mx[u] > NO_EXP) atomicMax(cmax + c, (unsigned long long)(mx[u] + 1023) << 52);
    }
}

// sigma_c = 2^e_c, the smallest power of two >= the column maximum (e = -1100:
// the column is zero).
__device__ __forceinline__ int col_exp(unsigned long long mxbits) {
    const int E = (int)((mxbits >> 52) & 0x7ff);
    if (E == 0) return -1100;
    const bool pow2 = (mxbits & ((1ULL << 52) - 1)) == 0;
    return E - 1023 + (pow2 ? 0 : 1);
}

// round(v * 2^(48 - e)) for |v| <= 2^e, ties away from zero, from the bits of
// v (no FP64 pipe).
__device__ __forceinline__ long long fixed48(double v, int e) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0) return 0;  // zero (subnormals, below 2^-1022, are dropped)
    const unsigned long long M = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
    // v = M 2^(E - 1075); N = M 2^(E - 1075 + 47 - e) = M >> sh
    const int sh = 1075 + e - GFRAC - E;  // >= 4 since |v| <= 2^e
    long long N = 0;
    if (sh < 64) N = (long long)((M + (1ULL << (sh - 1))) >> sh);
    return (b >> 63) ? -N : N;
}

// The slices of A'. Thread = (column c, group of 8 rows): the 7 digits of the
// group's entries, one 16-byte store per digit piece. Rows >= nact and
// columns > m are written as zeros.
__global__ void __launch_bounds__(256) gram_slice_kernel(const double *__restrict__ KSC, int m,
                                                         const int *__restrict__ act, int nact,
                                                         const double *__restrict__ sd,
                                                         const double *__restrict__ day,
                                                         const unsigned long long *__restrict__ cmax, int ncols,
                                                         int npb, __nv_bfloat16 *__restrict__ S) {
    __shared__ uint16_t bf[129];  // bf16 bits of -64 ... 64
    if (threadIdx.x < 129) {
        const __nv_bfloat16 h = __float2bfloat16_rn((float)((int)threadIdx.x - 64));
        bf[threadIdx.x] = *(const uint16_t *)&h;
    }
    __syncthreads();
    const long long items = (long long)ncols * npb * 2;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < items;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t % ncols);
        const long long g = t / ncols;  // 8-row group
        const int pb = (int)(g >> 1), half = (int)(g & 1);
        const int e = c <= m ? col_exp(cmax[c]) : -1100;
        uint32_t w[GS][4];  // digit s of the 8 rows, packed bf16 pairs
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int p = pb * GBK + half * 8 + k;
            long long N = 0;
            if (p < nact && c <= m && e > -1100) {
                const double v = c < m ? __dmul_rn(sd[p], KSC[(size_t)act[p] * m + c]) : day[p];
                N = fixed48(v, e);
            }
#pragma unroll
            for (int s = 0; s < GS; ++s) {
                int d;
                if (s < GS - 1) {
                    d = (int)(N & 127);
                    if (d >= 64) d -= 128;
                    N = (N - d) >> 7;
                } else {
                    d = (int)N;  // |d| <= 64
                }
                const uint32_t hb = bf[d + 64];
                if (k & 1) w[s][k >> 1] |= hb << 16;
                else w[s][k >> 1] = hb;
            }
        }
        const int ct = c >> 7, r = c & 127;
        const size_t base = ((size_t)ct * npb + pb) * GS * GPIECE + piece_off(r, half * 8);
#pragma unroll
        for (int s = 0; s < GS; ++s)
            *(uint4 *)(S + base + (size_t)s * GPIECE) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}

// tcgen05.ld of 4 consecutive columns of this warp's 32 lanes.
__device__ __forceinline__ void tc_ld4(uint32_t addr, float *v) {
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
    v[0] = __uint_as_float(r0);
    v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2);
    v[3] = __uint_as_float(r3);
}

// Records the first wait that ran out in device flag word 1 as
// role * 10^8 + cta * 1000 + stage (role 1: producer empty, 2: producer
// drain, 3: MMA acc-empty, 4: MMA full, 5: MMA done, 6: drain acc-full).
__device__ __forceinline__ void gram_timeout(int *flags, int role, int cta, int k) {
    atomicCAS(flags + 1, 0, role * 100000000 + min(cta, 99999) * 1000 + min(max(k, 0), 999));
}

// 96-bit accumulator hi * 2^32 + lo (hi signed).
struct Acc96 {
    long long hi;
    uint32_t lo;
};

__device__ __forceinline__ void acc_add(Acc96 &a, long long xh, uint32_t xl) {
    const uint32_t lo = a.lo + xl;
    a.hi += xh + (lo < xl ? 1 : 0);
    a.lo = lo;
}

// Tile (I, J) of G for split-K chunk z: rows 128 I ... of G (columns of A'),
// columns 64 J ...; stages [z * spc, min(npb, (z + 1) * spc)) of 16 rows.
__global__ void __launch_bounds__(G_THREADS, 1) gram_tc_kernel(const __nv_bfloat16 *__restrict__ S, int npb, int spc,
                                                               int m, const unsigned long long *__restrict__ cmax,
                                                               double *__restrict__ part, int *flags) {
    const int J = blockIdx.x, I = blockIdx.y, z = blockIdx.z;
    if (GN * J > GM * I + GM - 1 || GN * J >= m) return;  // above the diagonal or past the last column
    extern __shared__ __align__(1024) unsigned char g_smem[];
    __shared__ __align__(8) uint64_t full[GNS], empty[GNS], accf, acce, done;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    unsigned char *smem = g_smem + ((1024 - (smem_u32(g_smem) & 1023)) & 1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k0 = z * spc, nst = max(0, min(npb, k0 + spc) - k0);
    const int cta = (int)(blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
    const int nblk = (nst + GDRAIN - 1) / GDRAIN;
    if (threadIdx.x == 0) {
        for (int b = 0; b < GNS; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        mbar_init(&accf, 1);
        mbar_init(&acce, 8);
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // producer: the A tile's 8 pieces in one copy, the B half-pieces in 8
        if (lane == 0) {
            const uint32_t base = smem_u32(smem);
            const __nv_bfloat16 *Ab = S + ((size_t)I * npb + k0) * GS * GPIECE;
            const __nv_bfloat16 *Bb = S + ((size_t)(J >> 1) * npb + k0) * GS * GPIECE + (J & 1) * (GN / 8) * 128;
            int issued = 0;
            for (int k = 0; k < nst; ++k) {
                const int slot = k % GNS;
                if (k >= GNS && !mbar_wait(smem_u32(&empty[slot]), (uint32_t)(k / GNS - 1) & 1u)) {
                    gram_timeout(flags, 1, cta, k);
                    abort_flag = 1;
                }
                if (abort_flag) break;
                const uint32_t sb = base + slot * G_STAGE, fb = smem_u32(&full[slot]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(G_STAGE));
                bulk_g2s(sb, Ab + (size_t)k * GS * GPIECE, A_STAGE, fb);
#pragma unroll
                for (int s = 0; s < GS; ++s)
                    bulk_g2s(sb + A_STAGE + s * B_PIECE, Bb + ((size_t)k * GS + s) * GPIECE, B_PIECE, fb);
                issued = k + 1;
            }
            for (int k = issued > GNS ? issued - GNS : 0; k < issued; ++k)
                if (!mbar_wait(smem_u32(&full[k % GNS]), (uint32_t)(k / GNS) & 1u)) {
                    gram_timeout(flags, 2, cta, k);
                    abort_flag = 1;
                }
        }
        __syncwarp();
    } else if (warp == 1) {
        // MMA issue: level u - 6 += sum_{s+t=u} A_s B_t, u = 6 ... 12
        if (lane == 0) {
            const uint32_t base = smem_u32(smem);
            for (int k = 0; k < nst && !abort_flag; ++k) {
                const int blk = k / GDRAIN, kin = k % GDRAIN;
                if (kin == 0 && blk >= 1) {
                    if (!mbar_wait(smem_u32(&acce), (uint32_t)(blk - 1) & 1u)) {
                        gram_timeout(flags, 3, cta, k);
                        abort_flag = 1;
                        break;
                    }
                }
                const int slot = k % GNS;
                if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(k / GNS) & 1u)) {
                    gram_timeout(flags, 4, cta, k);
                    abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const uint32_t sa = base + slot * G_STAGE, sbb = sa + A_STAGE;
                // A piece s against the B pieces t = GS-1-s ... GS-1, which lie
                // consecutively in shared memory and so form one operand of
                // 64 (s + 1) rows whose products land on the consecutive
                // levels 0 ... s: ten MMAs of N <= 256 for the 28 pairs, each A
                // piece read once per MMA instead of once per pair. Piece GS-1
                // comes first and covers every level, so it alone starts a
                // drain block. The sums are exact integers, so the grouping
                // does not change them.
#pragma unroll
                for (int s = GS - 1; s >= 0; --s) {
                    const uint64_t da = tc_desc_lbo_sbo(sa + s * (GPIECE * 2), 128, 256);
#pragma unroll
                    for (int t0 = GS - 1 - s; t0 < GS; t0 += 4) {
                        const int np = GS - t0 < 4 ? GS - t0 : 4;  // B pieces of this MMA
                        const uint64_t db = tc_desc_lbo_sbo(sbb + t0 * B_PIECE, 128, 256);
                        const bool acc = kin > 0 || s < GS - 1;
                        mma_bf16(tmem + (uint32_t)(s + t0 - (GS - 1)) * GN, da, db, tc_idesc(GM, GN * np),
                                 acc ? 1u : 0u);
                    }
                }
                tc_commit(&empty[slot]);
                if (kin == GDRAIN - 1 || k == nst - 1) tc_commit(&accf);
            }
            tc_commit(&done);
            if (!mbar_wait(smem_u32(&done), 0u)) {
                gram_timeout(flags, 5, cta, nst);
                abort_flag = 1;
            }
        }
        __syncwarp();
    } else if (warp >= 4) {
        // drain: lanes 32 (warp % 4) ..., columns 32 h ... 32 h + 31
        const int q = warp & 3, h = (warp - 4) >> 2;
        Acc96 T[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) T[j] = Acc96{0, 0u};
        for (int blk = 0; blk < nblk; ++blk) {
            const bool got = mbar_wait(smem_u32(&accf), (uint32_t)blk & 1u);
            if (!got) gram_timeout(flags, 6, cta, blk * GDRAIN);
            const int bad = (!got || abort_flag) ? 1 : 0;
            int any;
            asm volatile(
                "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.or.pred q, 1, 256, p;\nselp.s32 %0, 1, 0, q;\n}\n"
                : "=r"(any)
                : "r"(bad));
            if (any) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const uint32_t lanes = tmem + ((uint32_t)(32 * q) << 16) + 32 * h;
#pragma unroll
            for (int c4 = 0; c4 < 32; c4 += 4) {
                float L[GS][4];
#pragma unroll
                for (int v = 0; v < GS; ++v) tc_ld4(lanes + v * GN + c4, L[v]);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // levels 9-12 and 6-8 by Horner in 64-bit integers (below
                    // 2^45 and 2^38), then T += t_hi 2^21 + t_lo
                    long long th = __float2int_rn(L[6][j]);
                    th = th * 128 + __float2int_rn(L[5][j]);
                    th = th * 128 + __float2int_rn(L[4][j]);
                    th = th * 128 + __float2int_rn(L[3][j]);
                    long long tl = __float2int_rn(L[2][j]);
                    tl = tl * 128 + __float2int_rn(L[1][j]);
                    tl = tl * 128 + __float2int_rn(L[0][j]);
                    acc_add(T[c4 + j], th >> 11, (uint32_t)th << 21);
                    acc_add(T[c4 + j], tl >> 32, (uint32_t)tl);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
            if (lane == 0) mbar_arrive(&acce);
        }
        if (!abort_flag) {
            const int r = GM * I + 32 * q + lane;
            if (r <= m) {
                const int er = col_exp(cmax[r]);
                double *out = part + (size_t)z * (m + 1) * m + (size_t)r * m;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int c = GN * J + 32 * h + j;
                    if (c < m && c <= r) {
                        const int ec = col_exp(cmax[c]);
                        double g = 0.0;
                        if (er > -1100 && ec > -1100) {
                            const double t = fma((double)T[j].hi, 4294967296.0, (double)T[j].lo);
                            g = ldexp(t, er + ec - GSCALE);
                        }
                        out[c] = g;
                    }
                }
            }
        }
    }
    if (threadIdx.x == 0 && abort_flag) gram_timeout(flags, 9, cta, 0);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512));
}

size_t slices_bytes(int l, int m) {
    const size_t ct = (size_t)ceil_div(m + 1, GM), npb = (size_t)ceil_div(std::max(l, 1), GBK);
    return ct * npb * GS * GPIECE * sizeof(__nv_bfloat16);
}

}  // namespace

// bf16 tensor-core flops issued by gram_tc_kernel since the last read (28
// digit-pair products per 128 x 64 x 16 step of every tile).
static double g_tc_flops = 0.0;
extern "C" double irwls_gram_tc_flops(int reset) {
    const double f = g_tc_flops;
    if (reset) g_tc_flops = 0.0;
    return f;
}

// Workspace of irwls_par_gram_tc for up to l active rows: the slices, then the
// m + 1 column maxima.
extern "C" size_t irwls_par_gram_tc_bytes(int l, int m) {
    return slices_bytes(l, m) + (size_t)(m + 1) * sizeof(unsigned long long) + 256;
}

// K1 (column-major, leading dimension ldK1, lower part) = KC + the Gram of
// the active rows, row m = K2, as irwls_par_gram gives; P bounds the
// split-K chunks (part holds at least P partials).
extern "C" int irwls_par_gram_tc(const double *d_KSC, int m, const int *d_act, int nact, const double *d_sd,
                                 const double *d_day, const double *d_KC, double *d_K1, int ldK1, double *d_part,
                                 int P, void *d_ws) {
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int ct = ceil_div(m + 1, GM), nt = ceil_div(m, GN);
    const int npb = ceil_div(std::max(nact, 1), GBK);
    __nv_bfloat16 *S = (__nv_bfloat16 *)d_ws;
    unsigned long long *cmax = (unsigned long long *)((char *)d_ws + slices_bytes(nact, m));
    // tiles of the lower part, and enough chunks to give every SM one CTA
    int tiles = 0;
    for (int I = 0; I < ct; ++I)
        for (int J = 0; J < nt; ++J)
            if (GN * J <= GM * I + GM - 1) ++tiles;
    int pz = std::max(1, std::min(P, sms / std::max(tiles, 1)));
    pz = std::min(pz, npb);
    const int spc = ceil_div(npb, pz);
    pz = ceil_div(npb, spc);
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_GRAM_SLICE);
    if (irwls_dev_memset(cmax, 0, (size_t)(m + 1) * sizeof(unsigned long long))) return -1;
    if (nact > 0) {
        gram_colmax_kernel<<<dim3(ceil_div(nact, GCM), ceil_div(m + 1, 1024)), 256, 0, irwls_stream()>>>(
            d_KSC, m, d_act, nact, d_sd, d_day, cmax);
        IRWLS_LAUNCH_CHECK("gram_colmax");
    }
    const long long items = (long long)ct * GM * npb * 2;
    gram_slice_kernel<<<(int)std::min<long long>(ceil_div(items, 256), 16LL * sms), 256, 0, irwls_stream()>>>(
        d_KSC, m, d_act, nact, d_sd, d_day, cmax, ct * GM, npb, S);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_GRAM_SLICE);
    IRWLS_LAUNCH_CHECK("gram_slice");
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_GRAM);
    const size_t smem = (size_t)GNS * G_STAGE + 1024;
    cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    gram_tc_kernel<<<dim3(nt, ct, pz), G_THREADS, smem, irwls_stream()>>>(S, npb, spc, m, cmax, d_part,
                                                                          irwls_dev_flags());
    g_tc_flops += (double)tiles * npb * GBK * GM * GN * 2.0 * GPAIRS;
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_GRAM);
    IRWLS_LAUNCH_CHECK("gram_tc");
    return irwls_par_gram_reduce(d_part, pz, m, d_KC, d_K1, ldK1);
}
