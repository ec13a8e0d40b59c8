// dev_budget.cu -- device steps of budgeted IRWLS: SGMA centroid selection
// (reference src/budgeted-train.c:114-309) and IRWLSpar (:324-505).
//
// SGMA keeps, per selected centroid s, the column KSC[:, s] = k(x_i, c_s)
// (column-major, l rows) and the lower Cholesky factor L of K_CC + jitter
// (row-major). One step scores 64 candidates:
//   z_c = (L L^T)^-1 k_C(c)      one CTA per candidate, blocked substitution
//   r_c = KSC z_c - k(c, .)      FP64 GEMM l x s x 64, the candidate kernel
//                                row is evaluated in the epilogue (never stored)
//   score_c = |r_c|^2 / eta_c    column norms reduced per CTA, then in a fixed
//                                order; strict ">" argmax, first index wins.
// IRWLSpar's Gram matrix K1 = KC + sum_i a_i a_i^T with a_i = sqrt(Da_i) KSC_i
// over active rows is a split-K SYRK on the lower triangle; the right-hand
// side K2 = sum_i a_i (sqrt(Da_i) y_i) is computed as the extra row m of the
// same product, which is exactly where the Cholesky solver wants it.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

#include "blocked_bf16.cuh"
#include "dev_common.cuh"

namespace {

constexpr int NCAND = 64;
constexpr int CT = 1024;

// --------------------------------------------------------------------------
// SGMA
// --------------------------------------------------------------------------

// Per candidate: KNC row, forward then backward substitution with L, eta.
// smem: v[s] (working vector), A row of the candidate (ld doubles).
__global__ void __launch_bounds__(256) sgma_cand_kernel(KView X, const int *__restrict__ cand,
                                                        const int *__restrict__ cent, int s,
                                                        const double *__restrict__ L, int ldL,
                                                        double *__restrict__ W, double *__restrict__ Z,
                                                        double *__restrict__ KN, int ldz,
                                                        double *__restrict__ eta) {
    extern __shared__ double sm[];
    double *v = sm;
    double *sA = sm + s;
    const int c = blockIdx.x, tid = threadIdx.x;
    const int gc = cand[c];
    for (int t = tid; t < X.ld; t += blockDim.x) sA[t] = X.X[(size_t)gc * X.ld + t];
    __syncthreads();
    const double qa = X.q[gc];
    for (int e = tid; e < s; e += blockDim.x) {
        const double kv = kentry(X, sA, qa, cent[e]);
        v[e] = kv;
        KN[(size_t)c * ldz + e] = kv;
    }
    __syncthreads();
    // forward: L w = v, 32-row blocks; the diagonal block is staged in Dg so
    // the serial sweep of warp 0 reads shared memory
    __shared__ double Dg[32][33];
    const int nblk = (s + 31) / 32;
    for (int b = 0; b < nblk; ++b) {
        const int r0 = b * 32, r1 = min(s, r0 + 32);
        for (int t = tid; t < 32 * 32; t += blockDim.x) {
            const int rr = t / 32, cc = t % 32;  // Dg[rr][cc] = L(r0 + rr, r0 + cc)
            Dg[rr][cc] = (r0 + rr < r1 && r0 + cc < r1) ? L[(size_t)(r0 + rr) * ldL + r0 + cc] : 0.0;
        }
        __syncthreads();
        if (tid < 32) {
            const int r = r0 + tid;
            double x = (r < r1) ? v[r] : 0.0;
            for (int cc = r0; cc < r1; ++cc) {
                double wc = 0.0;
                if (r == cc) wc = x / Dg[cc - r0][cc - r0];
                wc = __shfl_sync(0xffffffffu, wc, cc - r0);
                if (r == cc) x = wc;
                else if (r > cc && r < r1) x = fma(-Dg[tid][cc - r0], wc, x);
            }
            if (r < r1) v[r] = x;
        }
        __syncthreads();
        for (int r = r1 + tid; r < s; r += blockDim.x) {
            double x = v[r];
            const double *row = L + (size_t)r * ldL;
#pragma unroll 8
            for (int cc = r0; cc < r1; ++cc) x = fma(-row[cc], v[cc], x);
            v[r] = x;
        }
        __syncthreads();
    }
    for (int e = tid; e < s; e += blockDim.x) W[(size_t)c * ldz + e] = v[e];
    __syncthreads();
    // backward: L^T z = w
    for (int b = nblk - 1; b >= 0; --b) {
        const int r0 = b * 32, r1 = min(s, r0 + 32);
        for (int t = tid; t < 32 * 32; t += blockDim.x) {
            const int rr = t / 32, cc = t % 32;
            Dg[rr][cc] = (r0 + rr < r1 && r0 + cc < r1) ? L[(size_t)(r0 + rr) * ldL + r0 + cc] : 0.0;
        }
        __syncthreads();
        if (tid < 32) {
            const int r = r0 + tid;
            double x = (r < r1) ? v[r] : 0.0;
            for (int cc = r1 - 1; cc >= r0; --cc) {
                double zc = 0.0;
                if (r == cc) zc = x / Dg[cc - r0][cc - r0];
                zc = __shfl_sync(0xffffffffu, zc, cc - r0);
                if (r == cc) x = zc;
                else if (r < cc) x = fma(-Dg[cc - r0][tid], zc, x);
            }
            if (r < r1) v[r] = x;
        }
        __syncthreads();
        for (int r = tid; r < r0; r += blockDim.x) {
            double x = v[r];
#pragma unroll 8
            for (int cc = r0; cc < r1; ++cc) x = fma(-L[(size_t)cc * ldL + r], v[cc], x);
            v[r] = x;
        }
        __syncthreads();
    }
    for (int e = tid; e < s; e += blockDim.x) Z[(size_t)c * ldz + e] = v[e];
    if (tid == 0) {
        // eta = 1 - sum_e k_e z_e, left to right (src/budgeted-train.c:192-194)
        double val = 1.0;
        for (int e = 0; e < s; ++e) val = __dsub_rn(val, __dmul_rn(KN[(size_t)c * ldz + e], v[e]));
        eta[c] = val;
    }
}

// 8-byte asynchronous global->shared copy; src_bytes = 0 writes zeros.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---- precision form: candidate solves through the explicit inverse factor ----
//
// The reference keeps L^-1 beside L (invKC, src/budgeted-train.c:241-279); the
// precision form does the same so that the 64 candidate solves of a step,
// W = K_CN L^-T (FP64), are one split-K GEMM over all SMs instead of 64
// dependent substitutions. Linv is row-major (ldi), zero above the diagonal.

// KN[c][t] = k(cand_c, cent_t) for t < s, FP64 (the reference's kernel).
__global__ void __launch_bounds__(128) cand_rows_kernel(KView X, const int *__restrict__ cand,
                                                        const int *__restrict__ cent, int s, double *__restrict__ KN,
                                                        int ldz) {
    chain_wait();
    chain_open();
    extern __shared__ double sa[];
    const int c = blockIdx.y, gc = cand[c];
    for (int t = threadIdx.x; t < X.ld; t += blockDim.x) sa[t] = X.X[(size_t)gc * X.ld + t];
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < s) KN[(size_t)c * ldz + t] = kentry(X, sa, X.q[gc], cent[t]);
}

// Partial W^T over one chunk of WT columns of Linv: item (eb, tc) covers rows
// e in [WE eb, WE eb + WE) and t in [WT tc, WT tc + WT) (t <= e only, Linv is
// zero above); part[(tc * 64 + c) * ldp + e]. Rows of Linv and KN stream
// through a cp.async double buffer of WK columns. Four rows per item, one
// (row, candidate) sum per thread, so that the grid covers the SMs already
// at small orders; every sum runs over its chunk in increasing t whatever
// the item shape (the terms past the row's diagonal are zeros).
constexpr int WE = 4, WT = 64, WK = 16;
static_assert(WT % WE == 0, "row blocks must not straddle chunks");
__global__ void __launch_bounds__(256) w_gemm_kernel(const double *__restrict__ Linv, int ldi,
                                                     const double *__restrict__ KN, int ldz, int s,
                                                     double *__restrict__ part, int ldp) {
    chain_wait();
    chain_open();
    const int eb = blockIdx.x, tc = blockIdx.y;
    const int e0 = eb * WE, t0 = tc * WT;
    if (t0 > e0 + WE - 1) return;
    const int t1 = min(min(t0 + WT, e0 + WE), s);
    __shared__ __align__(16) double Ls[2][WE][WK + 1];
    __shared__ __align__(16) double Ks[2][NCAND][WK + 1];
    const int tid = threadIdx.x, c = tid & (NCAND - 1), ty = tid / NCAND;  // row e0 + ty, candidate c
    static_assert(WE * NCAND == 256, "one (row, candidate) per thread");
    double acc = 0.0;
    auto load = [&](int buf, int t) {
        for (int u = tid; u < (WE + NCAND) * WK; u += 256) {
            const int r = u / WK, k = u % WK;
            const int tt = t + k;
            if (r < WE) {
                const int e = e0 + r;
                const bool ok = e < s && tt < t1;
                cp_async8(&Ls[buf][r][k], ok ? (const void *)(Linv + (size_t)e * ldi + tt) : (const void *)Linv,
                          ok ? 8 : 0);
            } else {
                const int cr = r - WE;
                const bool ok = tt < t1;
                cp_async8(&Ks[buf][cr][k], ok ? (const void *)(KN + (size_t)cr * ldz + tt) : (const void *)KN,
                          ok ? 8 : 0);
            }
        }
        cp_async_commit();
    };
    if (t0 < t1) load(0, t0);
    int it = 0;
    for (int t = t0; t < t1; t += WK, ++it) {
        const int buf = it & 1;
        if (t + WK < t1) {
            load(buf ^ 1, t + WK);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < WK; ++k) acc = fma(Ls[buf][ty][k], Ks[buf][c][k], acc);
        __syncthreads();
    }
    const int e = e0 + ty;
    if (e < s) part[((size_t)tc * NCAND + c) * ldp + e] = acc;
}

// Per candidate c: w_e = sum of the chunks of row e in chunk order, W (FP64),
// eta = 1 - |w|^2 (fixed-order block reduction), and w as the bf16 hi/mid/lo
// pieces of its FP32 rounding in the blocked layout (zero up to the padded
// width kpad).
__global__ void __launch_bounds__(256) w_finish_kernel(const double *__restrict__ part, int ldp, int s,
                                                       double *__restrict__ W, int ldz, __nv_bfloat16 *Wb, int kpad,
                                                       double *__restrict__ eta) {
    chain_wait();
    chain_open();
    __shared__ double red[256];
    const int c = blockIdx.x;
    double ss = 0.0;
    for (int e = threadIdx.x; e < kpad; e += blockDim.x) {
        float xf = 0.f;
        if (e < s) {
            const int ntc = (e / WE * WE + WE - 1) / WT + 1;
            // the chunk partials loaded together, then summed in chunk order
            double pv[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) pv[u] = u < ntc ? part[((size_t)u * NCAND + c) * ldp + e] : 0.0;
            double w = 0.0;
#pragma unroll
            for (int u = 0; u < 16; ++u)
                if (u < ntc) w += pv[u];
            for (int tc = 16; tc < ntc; ++tc) w += part[((size_t)tc * NCAND + c) * ldp + e];
            W[(size_t)c * ldz + e] = w;
            ss = fma(w, w, ss);
            xf = (float)w;
        }
        __nv_bfloat16 pc[3];
        bf16_pieces3(xf, pc);
#pragma unroll
        for (int k = 0; k < QB_NP; ++k) Wb[wb_index(c, e, k)] = pc[k];
    }
    red[threadIdx.x] = ss;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) eta[c] = 1.0 - red[0];
}

// New row s of Linv from row s of L (l2, pivot L3):
//   Linv[s][t] = -(sum_{t <= e < s} l2_e Linv[e][t]) / L3,  Linv[s][s] = 1 / L3.
// Stage 1: partial sums over e-chunks of LE rows, part2[chunk][t].
constexpr int LE = 64;
__global__ void __launch_bounds__(128) linv_partial_kernel(const double *__restrict__ L, int ldL,
                                                           const double *__restrict__ Linv, int ldi, int s,
                                                           double *__restrict__ part2) {
    chain_wait();
    chain_open();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int e0 = blockIdx.y * LE, e1 = min(s, e0 + LE);
    if (t >= s) return;
    const double *l2 = L + (size_t)s * ldL;
    double acc = 0.0;
    // sixteen rows' loads in flight ahead of the (serial) sum, e increasing
    for (int e = max(e0, t); e < e1; e += 16) {
        double v[16], w[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const bool ok = e + u < e1;
            v[u] = ok ? Linv[(size_t)(e + u) * ldi + t] : 0.0;
            w[u] = ok ? l2[e + u] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 16; ++u)
            if (e + u < e1) acc = fma(w[u], v[u], acc);
    }
    part2[(size_t)blockIdx.y * s + t] = acc;
}

// Stage 2 (one CTA): the row of Linv in chunk order, and row s of L as FP32
// (l2, then 1 / L3) for the Q column update.
__global__ void __launch_bounds__(256) linv_finish_kernel(const double *__restrict__ L, int ldL,
                                                          double *__restrict__ Linv, int ldi, int s,
                                                          const double *__restrict__ part2, int nch,
                                                          float *__restrict__ lrow) {
    chain_wait();
    chain_open();
    const double L3 = L[(size_t)s * ldL + s];
    for (int t = threadIdx.x; t < s; t += blockDim.x) {
        // the chunk partials (at most 16 at order 1024) loaded together, then
        // summed in chunk order
        double pv[16];
        const int c0 = t / LE;
#pragma unroll
        for (int u = 0; u < 16; ++u) pv[u] = c0 + u < nch ? part2[(size_t)(c0 + u) * s + t] : 0.0;
        double acc = 0.0;
#pragma unroll
        for (int u = 0; u < 16; ++u)
            if (c0 + u < nch) acc += pv[u];
        for (int ch = c0 + 16; ch < nch; ++ch) acc += part2[(size_t)ch * s + t];
        Linv[(size_t)s * ldi + t] = -acc / L3;
        lrow[t] = __double2float_rn(L[(size_t)s * ldL + t]);
    }
    if (threadIdx.x == 0) {
        const double inv = 1.0 / L3;
        Linv[(size_t)s * ldi + s] = inv;
        lrow[s] = __double2float_rn(inv);
    }
}

// SGMA scores: for row tiles of GM rows and all 64 candidates,
// acc[i][c] = sum_k KSC[k*l + i] Z[c*ldz + k], r = acc - k(cand_c, x_i), and
// the sum of r^2 over the CTA's tiles goes to part[blockIdx.x][c].
// Persistent: CTA b takes tiles b, b + gridDim.x, ... (a fixed order, so the
// partial sums are deterministic); 32-row tiles keep the last round short.
// K-steps of GK are double-buffered with cp.async.
constexpr int GM = 32, GK = 16;
__global__ void __launch_bounds__(256, 2) sgma_gemm_kernel(KView X, int l, const int *__restrict__ cand, int s,
                                                           const double *__restrict__ KSC,
                                                           const double *__restrict__ Z, int ldz,
                                                           double *__restrict__ part) {
    __shared__ __align__(16) double As[2][GK][GM];
    __shared__ __align__(16) double Bs[2][GK][NCAND + 1];
    __shared__ double red[16][NCAND + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;  // tx: candidate group, ty: row group
    const int ntiles = (l + GM - 1) / GM;
    const int nk = (s + GK - 1) / GK;
    double ps[4] = {0.0, 0.0, 0.0, 0.0};
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i0 = tile * GM;
        double acc[2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
        auto load = [&](int buf, int k0) {
            for (int t = tid; t < GK * GM; t += 256) {
                const int kk = t / GM, r = t % GM;
                const int k = k0 + kk, i = i0 + r;
                const bool ok = (k < s && i < l);
                cp_async8(&As[buf][kk][r], ok ? (const void *)(KSC + (size_t)k * l + i) : (const void *)KSC,
                          ok ? 8 : 0);
            }
            for (int t = tid; t < GK * NCAND; t += 256) {
                const int c = t / GK, kk = t % GK;
                const int k = k0 + kk;
                const bool ok = k < s;
                cp_async8(&Bs[buf][kk][c], ok ? (const void *)(Z + (size_t)c * ldz + k) : (const void *)Z,
                          ok ? 8 : 0);
            }
            cp_async_commit();
        };
        if (nk > 0) load(0, 0);
        for (int kt = 0; kt < nk; ++kt) {
            const int buf = kt & 1;
            if (kt + 1 < nk) {
                load(buf ^ 1, (kt + 1) * GK);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < GK; ++kk) {
                double av[2], bv[4];
#pragma unroll
                for (int a = 0; a < 2; ++a) av[a] = As[buf][kk][ty + 16 * a];
#pragma unroll
                for (int b = 0; b < 4; ++b) bv[b] = Bs[buf][kk][tx + 16 * b];
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
            }
            __syncthreads();
        }
        // epilogue: subtract the candidate kernel value, square, accumulate
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gc = cand[tx + 16 * b];
            const double *arow = X.X + (size_t)gc * X.ld;
            const double qa = X.q[gc];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int i = i0 + ty + 16 * a;
                if (i < l) {
                    const double r = acc[a][b] - kentry(X, arow, qa, i);
                    ps[b] = fma(r, r, ps[b]);
                }
            }
        }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) red[ty][tx + 16 * b] = ps[b];
    __syncthreads();
    if (tid < NCAND) {
        double t = 0.0;
        for (int g = 0; g < 16; ++g) t += red[g][tid];
        part[(size_t)blockIdx.x * NCAND + tid] = t;
    }
}

// Fixed-order reduction of the partial norms, scores, argmax
// (src/budgeted-train.c:197-216).
__global__ void __launch_bounds__(NCAND) sgma_select_kernel(const double *__restrict__ part, int nblk,
                                                            const double *__restrict__ eta,
                                                            const int *__restrict__ cand, int s, int *cent,
                                                            int *best, double *bestval) {
    __shared__ double sc[NCAND];
    const int c = threadIdx.x;
    double v = 0.0;
    for (int b = 0; b < nblk; ++b) v += part[(size_t)b * NCAND + c];
    const double et = eta[c];
    sc[c] = (et > 0.0) ? __dmul_rn(__ddiv_rn(1.0, et), v) : 0.0;
    __syncthreads();
    if (c == 0) {
        double val = sc[0];
        int bb = 0;
        for (int i = 1; i < NCAND; ++i)
            if (sc[i] > val) {
                val = sc[i];
                bb = i;
            }
        cent[s] = cand[bb];
        best[0] = bb;
        bestval[s] = val;
    }
}

// Appends centroid s: KSC column (separate launch), and row s of L:
// L[s, :s] = L^-1 k_C(c_s) (the forward result of the winning candidate),
// L[s, s] = sqrt(k(c_s, c_s) + jitter - |L[s, :s]|^2)  (src/budgeted-train.c:247-279).
// tree = 1 (precision form): |L[s, :s]|^2 by a fixed-order block reduction
// instead of the reference's left-to-right sum.
__global__ void __launch_bounds__(128) sgma_factor_kernel(KView X, int s, const int *__restrict__ cent,
                                                          const int *__restrict__ best, const double *__restrict__ W,
                                                          int ldz, double *__restrict__ L, int ldL, int tree) {
    chain_wait();
    chain_open();
    extern __shared__ double sA[];
    __shared__ double red[128];
    const int gc = cent[s];
    for (int t = threadIdx.x; t < X.ld; t += blockDim.x) sA[t] = X.X[(size_t)gc * X.ld + t];
    __syncthreads();
    double ss = 0.0;
    if (s >= 2) {
        const int bb = best[0];
        for (int t = threadIdx.x; t < s; t += blockDim.x) {
            const double v = W[(size_t)bb * ldz + t];
            L[(size_t)s * ldL + t] = v;
            ss = fma(v, v, ss);
        }
    }
    red[threadIdx.x] = ss;
    __syncthreads();
    if (tree && s >= 2) {
        for (int o = 64; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const double kcc = kentry(X, sA, X.q[gc], gc);
            L[(size_t)s * ldL + s] = sqrt(__dsub_rn(__dadd_rn(kcc, 0.00001), red[0]));
        }
        return;
    }
    if (threadIdx.x == 0) {
        const double kcc = kentry(X, sA, X.q[gc], gc);
        if (s == 0) {
            L[0] = sqrt(__dadd_rn(kcc, 0.000001));
        } else {
            if (s == 1) {
                // L2 = (1 / L00) k(c0, c1) as the reference's inverse-factor product
                const double k01 = kentry(X, sA, X.q[gc], cent[0]);
                L[(size_t)1 * ldL + 0] = __dmul_rn(__ddiv_rn(1.0, L[0]), k01);
            }
            double l3 = __dadd_rn(kcc, 0.00001);
            for (int t = 0; t < s; ++t) {
                const double v = L[(size_t)s * ldL + t];
                l3 = __dsub_rn(l3, __dmul_rn(v, v));
            }
            L[(size_t)s * ldL + s] = sqrt(l3);
        }
    }
}

// --------------------------------------------------------------------------
// IRWLSpar
// --------------------------------------------------------------------------

__global__ void add_diag_kernel(double *KC, int m, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        KC[(size_t)i * m + i] = __dadd_rn(KC[(size_t)i * m + i], v);
}

// Partial Gram tiles. A' row p = [sd_p * KSC[act_p, :], day_p] (m + 1 values).
// Tile (bi, bj), bi >= bj, of the lower triangle of A'^T A' restricted to
// columns < m; chunk z of the active rows. part layout: [P][m+1 rows][m cols]
// row-major by output row. Row chunks of TK are copied with cp.async into a
// double buffer, then scaled in place (each thread scales the values it
// copied) so that the products use fl(sd * KSC) as the reference does.
constexpr int TT = 64, TK = 16;
__global__ void __launch_bounds__(256) gram_kernel(const double *__restrict__ KSC, int m, const int *__restrict__ act,
                                                   int nact, const double *__restrict__ sd,
                                                   const double *__restrict__ day, int chunk,
                                                   double *__restrict__ part) {
    const int bj = blockIdx.x, bi = blockIdx.y, z = blockIdx.z;
    if (bi < bj) return;
    const int r0 = bi * TT, c0 = bj * TT;  // output rows (0..m), output cols (0..m-1)
    const int p0 = z * chunk, p1 = min(nact, p0 + chunk);
    __shared__ __align__(16) double Ai[2][TK][TT + 1];
    __shared__ __align__(16) double Aj[2][TK][TT + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    auto load = [&](int buf, int p) {
        for (int t = tid; t < TK * TT; t += 256) {
            const int kk = t / TT, cc = t % TT;
            const int pp = p + kk;
            const int ci = r0 + cc, cj = c0 + cc;
            const double *si = KSC, *sj = KSC;
            int ni = 0, nj = 0;
            if (pp < p1) {
                const double *row = KSC + (size_t)act[pp] * m;
                if (ci < m) {
                    si = row + ci;
                    ni = 8;
                } else if (ci == m) {
                    si = day + pp;
                    ni = 8;
                }
                if (cj < m) {
                    sj = row + cj;
                    nj = 8;
                }
            }
            cp_async8(&Ai[buf][kk][cc], si, ni);
            cp_async8(&Aj[buf][kk][cc], sj, nj);
        }
        cp_async_commit();
    };
    auto scale = [&](int buf, int p) {
        for (int t = tid; t < TK * TT; t += 256) {
            const int kk = t / TT, cc = t % TT;
            const int pp = p + kk;
            if (pp < p1) {
                const double sc = sd[pp];
                if (r0 + cc < m) Ai[buf][kk][cc] = __dmul_rn(sc, Ai[buf][kk][cc]);
                if (c0 + cc < m) Aj[buf][kk][cc] = __dmul_rn(sc, Aj[buf][kk][cc]);
            }
        }
    };
    if (p0 < p1) load(0, p0);
    int it = 0;
    for (int p = p0; p < p1; p += TK, ++it) {
        const int buf = it & 1;
        if (p + TK < p1) {
            load(buf ^ 1, p + TK);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        scale(buf, p);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            double ai[4], aj[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) ai[a] = Ai[buf][kk][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) aj[b] = Aj[buf][kk][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(ai[a], aj[b], acc[a][b]);
        }
        __syncthreads();
    }
    double *out = part + (size_t)z * (m + 1) * m;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int r = r0 + ty + 16 * a;
        if (r > m) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int c = c0 + tx + 16 * b;
            if (c < m && c <= r) out[(size_t)r * m + c] = acc[a][b];
        }
    }
}

// K1 (column-major, leading dimension ld >= m + 1, lower part) = KC + sum_z
// part_z; row m = K2 = sum_z part_z[m][:].
__global__ void gram_reduce_kernel(const double *__restrict__ part, int P, int m, const double *__restrict__ KC,
                                   double *__restrict__ K1, int ld) {
    const long long total = (long long)(m + 1) * m;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(t / m), c = (int)(t % m);
        if (c > r) continue;
        double v = 0.0;
        for (int z = 0; z < P; ++z) v += part[(size_t)z * total + t];
        if (r < m) v = __dadd_rn(v, KC[(size_t)r * m + c]);
        K1[(size_t)c * ld + r] = v;
    }
}

// e = y - KSC beta, then Da (src/budgeted-train.c:431-457). A warp per row,
// two rows in flight (their loads interleaved); per row each lane's terms in
// increasing j, then a butterfly over the lanes.
__global__ void residual_kernel(const double *__restrict__ KSC, int l, int m, const double *__restrict__ beta,
                                const double *__restrict__ y, double C, double M, double *__restrict__ e,
                                double *__restrict__ Da) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i0 = warp; i0 < l; i0 += 2 * nw) {
        const int i1 = i0 + nw;
        const bool two = i1 < l;
        const double *r0 = KSC + (size_t)i0 * m, *r1 = KSC + (size_t)(two ? i1 : i0) * m;
        double a0 = 0.0, a1 = 0.0;
        int j = lane;
        for (; j + 32 < m; j += 64) {
            const double b0 = beta[j], b1 = beta[j + 32];
            const double x0 = r0[j], x1 = r1[j], y0 = r0[j + 32], y1 = r1[j + 32];
            a0 = fma(x0, b0, a0);
            a1 = fma(x1, b0, a1);
            a0 = fma(y0, b1, a0);
            a1 = fma(y1, b1, a1);
        }
        if (j < m) {
            const double b0 = beta[j];
            a0 = fma(r0[j], b0, a0);
            a1 = fma(r1[j], b0, a1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        }
        if (lane < 2 && (lane == 0 || two)) {
            const int i = lane == 0 ? i0 : i1;
            const double acc = lane == 0 ? a0 : a1;
            const double yi = y[i];
            const double ei = yi - acc;
            e[i] = ei;
            double d = (__dmul_rn(ei, yi) < 0.0) ? 0.0 : __ddiv_rn(__dmul_rn(1.0, C), __dmul_rn(yi, ei));
            if (d > M) d = M;
            Da[i] = d;
        }
    }
}

// Active rows (Da != 0) in ascending order with sqrt(Da) and sqrt(Da) y
// (src/budgeted-train.c:459-474), as an ordered compaction over blocks of WB
// rows: weights_count_kernel counts each block's active rows; each block of
// weights_write_kernel sums the counts before it and places its rows by
// warp-ballot prefixes, round by round in row order.
constexpr int WB = 2048;

__device__ __forceinline__ int block_sum256(int v, int *ws) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int k = 0; k < 8; ++k) t += ws[k];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(256) weights_count_kernel(const double *__restrict__ Da, int l,
                                                            int *__restrict__ cnt) {
    __shared__ int ws[8];
    const int r0 = blockIdx.x * WB, r1 = min(l, r0 + WB);
    int c = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += 256) c += Da[i] != 0.0;
    const int t = block_sum256(c, ws);
    if (threadIdx.x == 0) cnt[blockIdx.x] = t;
}

__global__ void __launch_bounds__(256) weights_write_kernel(const double *__restrict__ Da, const double *__restrict__ y,
                                                            int l, const int *__restrict__ cnt, int nb,
                                                            int *__restrict__ act, double *__restrict__ sd,
                                                            double *__restrict__ day, int *__restrict__ nact) {
    __shared__ int ws[8];
    __shared__ int woff[8];
    int part = 0;
    for (int k = threadIdx.x; k < (int)blockIdx.x; k += 256) part += cnt[k];
    int base = block_sum256(part, ws);
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) nact[0] = base + cnt[nb - 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = blockIdx.x * WB, r1 = min(l, r0 + WB);
    for (int i0 = r0; i0 < r1; i0 += 256) {
        const int i = i0 + threadIdx.x;
        const double d = i < r1 ? Da[i] : 0.0;
        const bool on = d != 0.0;
        const unsigned bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) ws[warp] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int k = 0; k < 8; ++k) {
                woff[k] = t;
                t += ws[k];
            }
            ws[0] = t;  // this round's total, read below after the barrier
        }
        __syncthreads();
        if (on) {
            const int pos = base + woff[warp] + __popc(bal & ((1u << lane) - 1u));
            act[pos] = i;
            const double r = sqrt(d);
            sd[pos] = r;
            day[pos] = __dmul_rn(r, y[i]);
        }
        base += ws[0];
        __syncthreads();
    }
}

// First IRWLSpar pass: every row, unscaled, with Day = y M (src/budgeted-train.c:348-352).
__global__ void first_weights_kernel(const double *__restrict__ y, int l, double M, int *act, double *sd,
                                     double *day) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l; i += gridDim.x * blockDim.x) {
        act[i] = i;
        sd[i] = 1.0;
        day[i] = __dmul_rn(y[i], M);
    }
}

// dW = |bnew - beta|^2, nW = |bnew|^2 (chunked, fixed order), beta <- bnew.
__global__ void __launch_bounds__(CT) delta_kernel(const double *__restrict__ bnew, double *beta, int m,
                                                   double *out2) {
    __shared__ double red[33];
    const int ch = (m + CT - 1) / CT;
    const int b = threadIdx.x * ch, e = min(m, b + ch);
    double vd = 0.0, vn = 0.0;
    for (int i = b; i < e; ++i) {
        const double d = __dsub_rn(bnew[i], beta[i]);
        vd = __dadd_rn(vd, __dmul_rn(d, d));
        vn = __dadd_rn(vn, __dmul_rn(bnew[i], bnew[i]));
    }
    const double dW = block_sum<CT>(vd, red);
    const double nW = block_sum<CT>(vn, red);
    __syncthreads();
    for (int i = b; i < e; ++i) beta[i] = bnew[i];
    if (threadIdx.x == 0) {
        out2[0] = dW;
        out2[1] = nW;
    }
}

}  // namespace

extern "C" int irwls_dev_kernel_block_t(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                                        const int *d_ib, int nB, double *d_out, long long ld_out, int trans);

// CTAs of the persistent score GEMM: two per SM (its launch bound), at most
// one per tile.
static int sgma_gemm_grid(int l) {
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int ntiles = ceil_div(l, GM);
    return ntiles < 2 * sms ? ntiles : 2 * sms;
}

extern "C" int irwls_sgma_first(const irwls_dev_set *X, int l, int *d_cent, double *d_L, int ldL, double *d_KSC) {
    // centroid 0 = row l (the positive class mean), set by the caller in d_cent
    if (irwls_dev_kernel_block_t(X, d_cent, 1, X, nullptr, l, d_KSC, l, 0)) return -2;
    const size_t smem = (size_t)X->ld * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(sgma_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    sgma_factor_kernel<<<1, 128, smem, irwls_stream()>>>(kview(X), 0, d_cent, nullptr, nullptr, 0, d_L, ldL, 0);
    IRWLS_LAUNCH_CHECK("sgma_factor");
    return 0;
}

extern "C" int irwls_sgma_score(const irwls_dev_set *X, int l, const int *d_cand, int ncand, const int *d_cent, int s,
                                const double *d_L, int ldL, const double *d_KSC, double *d_W, double *d_Z,
                                double *d_KN, int ldz, double *d_eta, double *d_part) {
    if (ncand != NCAND) {
        irwls_set_error(-7, "SGMA scores exactly %d candidates per step", NCAND);
        return -7;
    }
    const size_t smem = ((size_t)s + X->ld) * sizeof(double);
    if (smem > 200 * 1024) {
        irwls_set_error(-7, "SGMA budget %d with feature width %d exceeds the substitution tile", s, X->width);
        return -7;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(sgma_cand_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_SGMA_CAND);
    sgma_cand_kernel<<<NCAND, 256, smem, irwls_stream()>>>(kview(X), d_cand, d_cent, s, d_L, ldL, d_W, d_Z, d_KN, ldz,
                                                          d_eta);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_SGMA_CAND);
    IRWLS_LAUNCH_CHECK("sgma_cand");
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_SGMA_GEMM);
    sgma_gemm_kernel<<<sgma_gemm_grid(l), 256, 0, irwls_stream()>>>(kview(X), l, d_cand, s, d_KSC, d_Z, ldz,
                                                                     d_part);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_SGMA_GEMM);
    IRWLS_LAUNCH_CHECK("sgma_gemm");
    return 0;
}

extern "C" int irwls_sgma_partials(int l) { return sgma_gemm_grid(l); }

// Precision form: W = K_CN L^-T for the 64 candidates of step s, eta and the
// bf16 split of W. wpart: irwls_sgma_wpart_count(m) doubles.
extern "C" size_t irwls_sgma_wpart_count(int m) { return ((size_t)m / WT + 2) * NCAND * (size_t)(m > 0 ? m : 1); }
extern "C" size_t irwls_sgma_lpart_count(int m) { return ((size_t)ceil_div(m, LE) + 1) * (size_t)(m > 0 ? m : 1); }

extern "C" int irwls_sgma_cand_inv(const irwls_dev_set *X, const int *d_cand, const int *d_cent, int s,
                                   const double *d_Linv, int ldi, double *d_KN, int ldz, double *d_wpart, int ldp,
                                   double *d_W, void *Wb, int ldq, double *d_eta) {
    if (s < 1) return 0;
    const size_t smem = (size_t)X->ld * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(cand_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int kpad = ceil_div(s, 64) * 64;
    if (kpad > ldq) {
        irwls_set_error(-12, "candidate width %d exceeds the split leading dimension %d", kpad, ldq);
        return -12;
    }
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_SGMA_CAND);
    launch_chained(cand_rows_kernel, dim3(ceil_div(s, 128), NCAND), dim3(128), smem, kview(X), d_cand, d_cent, s, d_KN,
                   ldz);
    IRWLS_LAUNCH_CHECK("cand_rows");
    launch_chained(w_gemm_kernel, dim3(ceil_div(s, WE), ceil_div(s, WT)), dim3(256), 0, d_Linv, ldi, d_KN, ldz, s,
                   d_wpart, ldp);
    IRWLS_LAUNCH_CHECK("w_gemm");
    launch_chained(w_finish_kernel, dim3(NCAND), dim3(256), 0, d_wpart, ldp, s, d_W, ldz, (__nv_bfloat16 *)Wb, kpad,
                   d_eta);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_SGMA_CAND);
    IRWLS_LAUNCH_CHECK("w_finish");
    return 0;
}

// Row s of Linv from row s of L, and row s of L in FP32 (l2, 1 / L3) into lrow.
extern "C" int irwls_sgma_linv_update(const double *d_L, int ldL, double *d_Linv, int ldi, int s, double *d_lpart,
                                      float *d_lrow) {
    const int nch = ceil_div(s, LE);
    if (s > 0) {
        launch_chained(linv_partial_kernel, dim3(ceil_div(s, 128), nch), dim3(128), 0, d_L, ldL, d_Linv, ldi, s,
                       d_lpart);
        IRWLS_LAUNCH_CHECK("linv_partial");
    }
    launch_chained(linv_finish_kernel, dim3(1), dim3(256), 0, d_L, ldL, d_Linv, ldi, s, d_lpart, nch, d_lrow);
    IRWLS_LAUNCH_CHECK("linv_finish");
    return 0;
}

// Row s of the SGMA factor only (no K_nm column).
extern "C" int irwls_sgma_factor(const irwls_dev_set *X, int s, const int *d_cent, const int *d_best, const double *d_W,
                                 int ldz, double *d_L, int ldL) {
    const size_t smem = (size_t)X->ld * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(sgma_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    launch_chained(sgma_factor_kernel, dim3(1), dim3(128), smem, kview(X), s, d_cent, d_best, d_W, ldz, d_L, ldL, 1);
    IRWLS_LAUNCH_CHECK("sgma_factor");
    return 0;
}



extern "C" int irwls_sgma_select(const double *d_part, int l, const double *d_eta, const int *d_cand, int s,
                                 int *d_cent, int *d_best, double *d_bestval) {
    sgma_select_kernel<<<1, NCAND, 0, irwls_stream()>>>(d_part, sgma_gemm_grid(l), d_eta, d_cand, s, d_cent, d_best,
                                                        d_bestval);
    IRWLS_LAUNCH_CHECK("sgma_select");
    return 0;
}

extern "C" int irwls_sgma_extend(const irwls_dev_set *X, int l, int s, const int *d_cent, const int *d_best,
                                 const double *d_W, int ldz, double *d_L, int ldL, double *d_KSC) {
    if (irwls_dev_kernel_block_t(X, d_cent + s, 1, X, nullptr, l, d_KSC + (size_t)s * l, l, 0)) return -2;
    const size_t smem = (size_t)X->ld * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(sgma_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    sgma_factor_kernel<<<1, 128, smem, irwls_stream()>>>(kview(X), s, d_cent, d_best, d_W, ldz, d_L, ldL, 0);
    IRWLS_LAUNCH_CHECK("sgma_factor");
    return 0;
}

extern "C" int irwls_par_build(const irwls_dev_set *X, int l, const int *d_idx, int m, double *d_KC, double *d_KSC) {
    if (irwls_dev_kernel_block_t(X, d_idx, m, X, d_idx, m, d_KC, m, 0)) return -2;
    add_diag_kernel<<<ceil_div(m, 256), 256, 0, irwls_stream()>>>(d_KC, m, 0.00001);
    IRWLS_LAUNCH_CHECK("add_diag");
    // KSC row-major l x m: out[row * m + centroid]
    return irwls_dev_kernel_block_t(X, d_idx, m, X, nullptr, l, d_KSC, m, 1);
}

extern "C" int irwls_par_first(const double *d_y, int l, double M, int *d_act, double *d_sd, double *d_day) {
    first_weights_kernel<<<ceil_div(l, 256), 256, 0, irwls_stream()>>>(d_y, l, M, d_act, d_sd, d_day);
    IRWLS_LAUNCH_CHECK("first_weights");
    return 0;
}

extern "C" size_t irwls_par_gram_part_bytes(int m, int P) { return (size_t)P * (m + 1) * m * sizeof(double); }

// K1 = KC + the sum of P Gram partials (the last step of both Gram forms).
extern "C" int irwls_par_gram_reduce(const double *d_part, int P, int m, const double *d_KC, double *d_K1, int ldK1) {
    const long long tot = (long long)(m + 1) * m;
    gram_reduce_kernel<<<(int)std::min<long long>(ceil_div(tot, 256), 65535), 256, 0, irwls_stream()>>>(
        d_part, P, m, d_KC, d_K1, ldK1);
    IRWLS_LAUNCH_CHECK("gram_reduce");
    return 0;
}

extern "C" int irwls_par_gram(const double *d_KSC, int m, const int *d_act, int nact, const double *d_sd,
                              const double *d_day, const double *d_KC, double *d_K1, int ldK1, double *d_part, int P) {
    const int T = ceil_div(m + 1, TT);
    const int Tc = ceil_div(m, TT);
    const int chunk = nact > 0 ? ceil_div(nact, P) : 1;
    dim3 grid(Tc, T, P);
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_GRAM);
    gram_kernel<<<grid, 256, 0, irwls_stream()>>>(d_KSC, m, d_act, nact, d_sd, d_day, chunk, d_part);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_GRAM);
    IRWLS_LAUNCH_CHECK("gram");
    const long long total = (long long)(m + 1) * m;
    gram_reduce_kernel<<<(int)std::min<long long>(ceil_div(total, 256), 65535), 256, 0, irwls_stream()>>>(
        d_part, P, m, d_KC, d_K1, ldK1);
    IRWLS_LAUNCH_CHECK("gram_reduce");
    return 0;
}

extern "C" int irwls_par_residual(const double *d_KSC, int l, int m, const double *d_beta, const double *d_y, double C,
                                  double M, double *d_e, double *d_Da) {
    const int blocks = std::min(ceil_div(l, 8), 8 * (irwls_num_sms() > 0 ? irwls_num_sms() : 148));
    residual_kernel<<<blocks, 256, 0, irwls_stream()>>>(d_KSC, l, m, d_beta, d_y, C, M, d_e, d_Da);
    IRWLS_LAUNCH_CHECK("residual");
    return 0;
}

extern "C" int irwls_par_weights(const double *d_Da, const double *d_y, int l, int *d_act, double *d_sd,
                                 double *d_day, int *d_nact) {
    const int nb = std::max(1, ceil_div(l, WB));
    int *cnt = (int *)irwls_ctx_scratch(2, (size_t)nb * sizeof(int));
    if (!cnt) return -3;
    weights_count_kernel<<<nb, 256, 0, irwls_stream()>>>(d_Da, l, cnt);
    IRWLS_LAUNCH_CHECK("weights_count");
    weights_write_kernel<<<nb, 256, 0, irwls_stream()>>>(d_Da, d_y, l, cnt, nb, d_act, d_sd, d_day, d_nact);
    IRWLS_LAUNCH_CHECK("weights_write");
    return 0;
}

extern "C" int irwls_par_delta(const double *d_bnew, double *d_beta, int m, double *d_out2) {
    delta_kernel<<<1, CT, 0, irwls_stream()>>>(d_bnew, d_beta, m, d_out2);
    IRWLS_LAUNCH_CHECK("delta");
    return 0;
}
