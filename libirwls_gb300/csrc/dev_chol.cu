// dev_chol.cu -- blocked right-looking Cholesky factorization and solve in
// FP64 (reference src/ParallelAlgorithms.c:361-447, which ends in LAPACK
// dpotrf/dpotrs).
//
// M is column-major with leading dimension ld >= n + 1. The right-hand side b
// is carried as row n: the factorization then produces, in that row, the
// forward-substitution result z = L^-1 b, and one backward sweep gives x.
//
// Failed pivots keep LAPACK's behaviour: a pivot that is not positive is
// stored without its square root and reported (first failure, 1-based) in
// device flag 0. In full IRWLS the system matrix is bordered by the labels
// with a zero corner, so its last pivot fails by construction; the reference
// ignores that failure and solves with the stored negative Schur complement,
// and so does this code.
//
// Two factorizations with the same arithmetic per element (so the same
// bits): one cooperative launch scheduled by data flow (the default, below
// chol_df_kernel), and a multi-launch sequence per panel of 32 columns (a
// launch that solves the rows below the diagonal block against it, and a
// launch that applies the rank-32 update to the lower trailing matrix and
// factors the next diagonal block).
#include <math.h>

#include <atomic>

#include <cooperative_groups.h>

#include "dev_common.cuh"

namespace {

constexpr int NB = 32;

// Factors the nb x nb diagonal block at (k0, k0) held in D (shared, NB x NB,
// lower part valid), with LAPACK dpotrf's failed-pivot behaviour, leaving
// the reciprocal of each stored pivot in rp. Uses the whole CTA; ends synced.
// FP64 runs at a fraction of the FP32 rate on this part, so every dependent
// FP64 operation on this serial path costs tens of cycles: the pivot's
// reciprocal square root is formed once and the column is scaled by it (as
// dpotf2 scales by 1 / ajj).
__device__ void factor_block(double (*D)[NB + 1], double *rp, int nb, int k0, int *flags, int *failed_at) {
    const int tid = threadIdx.x;
    if (tid == 0) *failed_at = -1;
    __syncthreads();
    for (int c = 0; c < nb; ++c) {
        if (tid == 0) {
            const double s = D[c][c];
            if (s > 0.0) {
                const double r = rsqrt(s);
                D[c][c] = s * r;
                rp[c] = r;
            } else {
                if (*failed_at < 0) *failed_at = c;  // stored without its root, as dpotrf leaves it
                rp[c] = 1.0 / s;
            }
        }
        __syncthreads();
        const double r = rp[c];
        for (int rr = c + 1 + tid; rr < nb; rr += blockDim.x) D[rr][c] = D[rr][c] * r;
        __syncthreads();
        const int m = nb - c - 1;
        for (int t = tid; t < m * m; t += blockDim.x) {
            const int rr = c + 1 + t / m, j = c + 1 + t % m;
            if (j <= rr) D[rr][j] = fma(-D[rr][c], D[j][c], D[rr][j]);
        }
        __syncthreads();
    }
    if (tid == 0 && *failed_at >= 0) atomicCAS(flags, 0, k0 + *failed_at + 1);
}

// Inverse of the factored block (its reciprocal pivots in rp): each entry a
// dot product split over 8 lanes of a warp (column j by threads 8 j ..
// 8 j + 7), Di[c][j] = -(sum_{j <= t < c} D[c][t] Di[t][j]) rp[c].
// blockDim.x == 256; ends synced.
__device__ void invert_block(double (*D)[NB + 1], double (*Di)[NB + 1], const double *rp, int nb) {
    const int tid = threadIdx.x;
    for (int t = tid; t < NB * NB; t += blockDim.x) Di[t / NB][t % NB] = 0.0;
    __syncthreads();
    // (every lane of a warp runs the same iterations so that the shuffles
    // always see the whole warp)
    {
        const int j = tid >> 3, q = tid & 7;
        if (q == 0 && j < nb) Di[j][j] = rp[j];
        __syncwarp();
        for (int c = 1; c < NB; ++c) {
            const bool live = j < nb && c < nb && c > j;
            double acc = 0.0;
            if (live)
                for (int t = j + q; t < c; t += 8) acc = fma(D[c][t], Di[t][j], acc);
            acc += __shfl_xor_sync(0xffffffffu, acc, 4, 8);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2, 8);
            acc += __shfl_xor_sync(0xffffffffu, acc, 1, 8);
            if (live && q == 0) Di[c][j] = -acc * rp[c];
            __syncwarp();
        }
    }
    __syncthreads();
}

__device__ void factor_invert_block(double (*D)[NB + 1], double (*Di)[NB + 1], double *rp, int nb, int k0,
                                    int *flags, int *failed_at) {
    factor_block(D, rp, nb, k0, flags, failed_at);
    invert_block(D, Di, rp, nb);
}

// Panel solve of the rows r < nr of T (columns c < nb) against the factored
// diagonal block D with reciprocal pivots rp, in place, by forward
// substitution: x_c = (a_c - sum_{t < c} x_t D[c][t]) rp[c], the sum taken
// by FMAs in increasing t. Used by both factorizations, so they agree bit
// for bit. blockDim.x == 256; ends synced.
__device__ void subst_block(double (*T)[NB + 1], int nr, double (*D)[NB + 1], const double *rp, int nb) {
    const int tid = threadIdx.x;
    for (int t = 0; t < nb; ++t) {
        for (int r = tid; r < nr; r += blockDim.x) T[r][t] = T[r][t] * rp[t];
        __syncthreads();
        const int m = nb - t - 1;
        for (int e = tid; e < nr * m; e += blockDim.x) {
            const int r = e / m, c = t + 1 + e % m;
            T[r][c] = fma(-T[r][t], D[c][t], T[r][c]);
        }
        __syncthreads();
    }
}

__device__ void store_block(double *M, int ld, int k0, int nb, double (*D)[NB + 1], double (*Di)[NB + 1],
                            double *Dinv) {
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const int r = t / NB, c = t % NB;
        if (r < nb && c <= r) M[(size_t)(k0 + c) * ld + k0 + r] = D[r][c];
        Dinv[t] = Di[r][c];
    }
}

// First diagonal block (the others are factored by the trailing update of
// the previous panel).
__global__ void __launch_bounds__(256) chol_factor0_kernel(double *__restrict__ M, int n, int ld,
                                                           int *__restrict__ flags, double *__restrict__ Dinv) {
    __shared__ double D[NB][NB + 1], Di[NB][NB + 1];
    __shared__ double rp[NB];
    __shared__ int failed_at;
    const int nb = min(NB, n);
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const int r = t / NB, c = t % NB;
        D[r][c] = (r < nb && c <= r) ? M[(size_t)c * ld + r] : 0.0;
    }
    __syncthreads();
    factor_invert_block(D, Di, rp, nb, 0, flags, &failed_at);
    store_block(M, ld, 0, nb, D, Di, Dinv);
}

// Panel solve: rows i >= k0 + nb (and the right-hand-side row n when present)
// get L[i, k0:k0+nb] = A[i, k0:k0+nb] D^-T by forward substitution against
// the factored diagonal block (from M, its reciprocal pivots from the
// diagonal of the stored inverse). 8 rows per CTA.
__global__ void __launch_bounds__(256) chol_trsm_kernel(double *__restrict__ M, int ld, int k0, int nb, int nrows,
                                                        const double *__restrict__ Dinv) {
    __shared__ double D[NB][NB + 1];
    __shared__ double A[8][NB + 1];
    __shared__ double rp[NB];
    const int tid = threadIdx.x;
    const int i0 = k0 + nb + blockIdx.x * 8;
    for (int t = tid; t < NB * NB; t += 256) {
        const int r = t / NB, c = t % NB;
        D[r][c] = (r < nb && c <= r) ? M[(size_t)(k0 + c) * ld + k0 + r] : 0.0;
    }
    if (tid < NB) rp[tid] = Dinv[tid * (NB + 1)];
    {
        const int c = tid / 8, r = tid % 8;  // 256 = 32 columns x 8 rows
        const int i = i0 + r;
        A[r][c] = (c < nb && i < nrows) ? M[(size_t)(k0 + c) * ld + i] : 0.0;
    }
    __syncthreads();
    const int nr = min(8, nrows - i0);
    subst_block(A, nr, D, rp, nb);
    const int c = tid / 8, r = tid % 8;
    const int i = i0 + r;
    if (c < nb && i < nrows) M[(size_t)(k0 + c) * ld + i] = A[r][c];
}

// Trailing update of the lower part: M[i][j] -= sum_t L[i][t] L[j][t] over the
// panel columns t, for k1 <= j <= i < nrows, j < n. One 32x32 tile per CTA.
// The CTA of tile (0, 0) then factors and inverts that tile, which is the
// next panel's diagonal block.
__global__ void __launch_bounds__(256) chol_update_kernel(double *__restrict__ M, int n, int ld, int k0, int nb,
                                                          int nrows, int *__restrict__ flags,
                                                          double *__restrict__ Dinv_next) {
    const int bj = blockIdx.x, bi = blockIdx.y;
    if (bi < bj) return;
    const int k1 = k0 + nb;
    const int r0 = k1 + bi * 32, c0 = k1 + bj * 32;
    __shared__ double Li[32][NB + 1];
    __shared__ double Lj[32][NB + 1];
    __shared__ int failed_at;
    const int tid = threadIdx.x;
    for (int t = tid; t < 32 * NB; t += 256) {
        const int r = t % 32, k = t / 32;
        const int gi = r0 + r, gj = c0 + r;
        Li[r][k] = (k < nb && gi < nrows) ? M[(size_t)(k0 + k) * ld + gi] : 0.0;
        Lj[r][k] = (k < nb && gj < n) ? M[(size_t)(k0 + k) * ld + gj] : 0.0;
    }
    __syncthreads();
    const int r = tid % 32;
    for (int cc = tid / 32; cc < 32; cc += 8) {
        const int gi = r0 + r, gj = c0 + cc;
        if (gi >= nrows || gj >= n || gj > gi) continue;
        double acc = 0.0;
#pragma unroll 8
        for (int k = 0; k < NB; ++k) acc = fma(Li[r][k], Lj[cc][k], acc);
        double *p = M + (size_t)gj * ld + gi;
        *p = *p - acc;
    }
    if (bi != 0 || bj != 0) return;
    // next diagonal block: reuse Li / Lj as D / Di
    __syncthreads();
    const int nb2 = min(NB, n - k1);
    for (int t = tid; t < NB * NB; t += 256) {
        const int rr = t / NB, c = t % NB;
        Li[rr][c] = (rr < nb2 && c <= rr) ? M[(size_t)(k1 + c) * ld + k1 + rr] : 0.0;
    }
    __syncthreads();
    __shared__ double rp[NB];
    factor_invert_block(Li, Lj, rp, nb2, k1, flags, &failed_at);
    store_block(M, ld, k1, nb2, Li, Lj, Dinv_next);
}

// The two dot products of a backward-sweep block, shared by both sweeps so
// that they give the same bits: each as four interleaved partial FMA chains
// (the dependent chain of one FP64 FMA per term is four times shorter) added
// as (s0 + s1) + (s2 + s3).
// x_t = sum_{t <= c < nb} Di[c][t] yb[c]
__device__ __forceinline__ double sweep_dot(const double (*Di)[NB + 1], const double *yb, int t, int nb) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int c = t;
    for (; c + 3 < nb; c += 4) {
        a0 = fma(Di[c][t], yb[c], a0);
        a1 = fma(Di[c + 1][t], yb[c + 1], a1);
        a2 = fma(Di[c + 2][t], yb[c + 2], a2);
        a3 = fma(Di[c + 3][t], yb[c + 3], a3);
    }
    for (; c < nb; ++c) a0 = fma(Di[c][t], yb[c], a0);
    return (a0 + a1) + (a2 + a3);
}

// sum_{c < nb} col[c] xb[c]
__device__ __forceinline__ double sweep_row(const double *col, const double *xb, int nb) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int c = 0;
    for (; c + 3 < nb; c += 4) {
        a0 = fma(col[c], xb[c], a0);
        a1 = fma(col[c + 1], xb[c + 1], a1);
        a2 = fma(col[c + 2], xb[c + 2], a2);
        a3 = fma(col[c + 3], xb[c + 3], a3);
    }
    for (; c < nb; ++c) a0 = fma(col[c], xb[c], a0);
    return (a0 + a1) + (a2 + a3);
}

// Backward sweep L^T x = z, z in row n of M; one CTA, z in shared memory,
// 32-row blocks from the bottom: x_b = D_b^-T y_b (parallel dots with the
// stored inverse), then the rows above are updated.
__global__ void __launch_bounds__(256) chol_backsolve_kernel(const double *__restrict__ M, int n, int ld,
                                                             const double *__restrict__ Dinv,
                                                             double *__restrict__ x) {
    extern __shared__ double z[];
    __shared__ double Di[NB][NB + 1];
    __shared__ double yb[NB];
    const int tid = threadIdx.x;
    for (int c = tid; c < n; c += blockDim.x) z[c] = M[(size_t)c * ld + n];
    const int nblk = (n + NB - 1) / NB;
    for (int b = nblk - 1; b >= 0; --b) {
        const int r0 = b * NB, r1 = min(n, r0 + NB);
        for (int t = tid; t < NB * NB; t += blockDim.x) Di[t / NB][t % NB] = Dinv[(size_t)b * NB * NB + t];
        __syncthreads();
        if (tid < NB) yb[tid] = (r0 + tid < r1) ? z[r0 + tid] : 0.0;
        __syncthreads();
        if (tid < r1 - r0) z[r0 + tid] = sweep_dot(Di, yb, tid, r1 - r0);
        __syncthreads();
        for (int r = tid; r < r0; r += blockDim.x) z[r] = z[r] - sweep_row(M + (size_t)r * ld + r0, z + r0, r1 - r0);
        __syncthreads();
    }
    for (int c = tid; c < n; c += blockDim.x) x[c] = z[c];
}

__global__ void zero_upper_kernel(double *__restrict__ M, int n, int ld) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)n * n;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), r = (int)(t % n);
        if (r < c) M[(size_t)c * ld + r] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// The same factorization in one cooperative launch, scheduled by data flow.
//
// The lower blocked matrix (32 x 32 tiles (i, j), i >= j, the right-hand-side
// row n included as a row) is a list of tasks in column-major order; task t
// belongs to CTA t mod G, and each CTA runs its tasks in order, keeping its
// tile in shared memory. A tile takes the updates of panels k = 0 ... j - 1
// as soon as their tiles L(i, k) and L(j, k) are published, then either
// factors and inverts itself (i == j) or solves against the published inverse
// of diagonal block j; it then publishes itself (a release store of a ready
// word after its data; readers poll with acquire loads and read the data
// from L2). Every dependency of a task has a smaller index, and all CTAs are
// resident (cooperative launch), so the smallest unfinished task can always
// run: no wait is circular. There are no grid-wide barriers, so a panel's
// diagonal block is factored as soon as its last update lands while other
// CTAs are still applying earlier panels elsewhere.
//
// Every element gets the multi-launch path's operations in the same order:
// per panel, acc = sum over the panel's 32 columns by FMA from zero, then
// M - acc; the diagonal blocks through factor_block; the panel solves by
// forward substitution against the factored block (subst_block). The
// results are the same bits. A diagonal block's factor is published before
// its inverse is formed: only the backward sweep, after this launch, reads
// the inverse.
//
// The waits are bounded: one that runs out (which needs a fault in this
// schedule) sets the pivot status to -1 and the tensor-core status word to
// CHOL_WAIT_CODE, and the CTA stops; the others then run out too.
// ---------------------------------------------------------------------------
constexpr long long DF_WAIT_LIMIT = 1LL << 22;
constexpr int CHOL_WAIT_CODE = 0x40000000;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 polls *p until it is nonzero (or `abort` is set elsewhere); the
// CTA learns the outcome at the barrier. False if the wait ran out.
__device__ bool df_wait(const unsigned *p, const volatile int *abort, int *ok_sh) {
    if (threadIdx.x == 0) {
        int ok = 0;
        for (long long it = 0; it < DF_WAIT_LIMIT; ++it) {
            if (ld_acquire_u32(p)) {
                ok = 1;
                break;
            }
            if (*abort) break;
            __nanosleep(64);
        }
        *ok_sh = ok;
    }
    __syncthreads();
    return *ok_sh != 0;
}

// Publishes the tile just stored by the whole CTA.
__device__ __forceinline__ void df_publish(unsigned *p) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        st_release_u32(p, 1u);
    }
}

// ready: diag[j] at ready[j] (j < nbc), tile L(i, j) at ready[nbc + j * nbr + i].
__global__ void __launch_bounds__(256) chol_df_kernel(double *__restrict__ M, int n, int ld, int nrows,
                                                      int *__restrict__ flags, double *__restrict__ Dinv,
                                                      unsigned *__restrict__ ready, int *__restrict__ abort) {
    __shared__ double T[NB][NB + 1], Li[NB][NB + 1], Lj[NB][NB + 1];
    __shared__ double rp[NB];
    __shared__ int failed_at, ok_sh;
    const int tid = threadIdx.x;
    const int nbc = (n + NB - 1) / NB, nbr = (nrows + NB - 1) / NB;
    int t = 0;
    for (int j = 0; j < nbc; ++j) {
        for (int i = j; i < nbr; ++i, ++t) {
            if (t % (int)gridDim.x != (int)blockIdx.x) continue;
            const int r0 = NB * i, c0 = NB * j;
            const int nr = min(NB, nrows - r0), nc = min(NB, n - c0);
            for (int e = tid; e < NB * NB; e += 256) {
                const int r = e % NB, c = e / NB;
                T[r][c] = (r < nr && c < nc && (i != j || c <= r)) ? __ldcg(M + (size_t)(c0 + c) * ld + r0 + r) : 0.0;
            }
            for (int k = 0; k < j; ++k) {
                const int kc = NB * k;
                if (!df_wait(ready + nbc + (size_t)k * nbr + i, abort, &ok_sh) ||
                    !df_wait(ready + nbc + (size_t)k * nbr + j, abort, &ok_sh))
                    goto fail;
                for (int e = tid; e < NB * NB; e += 256) {
                    const int r = e % NB, kk = e / NB;
                    Li[r][kk] = r < nr ? __ldcg(M + (size_t)(kc + kk) * ld + r0 + r) : 0.0;
                    Lj[r][kk] = r < nc ? __ldcg(M + (size_t)(kc + kk) * ld + c0 + r) : 0.0;
                }
                __syncthreads();
                if (i != j) {
                    const int r = tid % NB;
                    for (int cc = tid / NB; cc < NB; cc += 8) {
                        if (r >= nr || cc >= nc) continue;
                        double acc = 0.0;
#pragma unroll 8
                        for (int kk = 0; kk < NB; ++kk) acc = fma(Li[r][kk], Lj[cc][kk], acc);
                        T[r][cc] = T[r][cc] - acc;
                    }
                } else {
                    // a diagonal tile needs only its lower triangle: threads
                    // take its NB (NB + 1) / 2 elements (the same FMAs per
                    // element), not the full tile's divergent columns, which
                    // halves this step on the factorization's critical path
                    for (int e = tid; e < NB * (NB + 1) / 2; e += 256) {
                        int r = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
                        while (r * (r + 1) / 2 > e) --r;
                        while ((r + 1) * (r + 2) / 2 <= e) ++r;
                        const int cc = e - r * (r + 1) / 2;
                        if (r >= nr || cc >= nc) continue;
                        double acc = 0.0;
#pragma unroll 8
                        for (int kk = 0; kk < NB; ++kk) acc = fma(Li[r][kk], Lj[cc][kk], acc);
                        T[r][cc] = T[r][cc] - acc;
                    }
                }
                __syncthreads();
            }
            if (i == j) {
                // rows >= n of this tile (the right-hand side) wait in Lj
                for (int e = tid; e < NB * NB; e += 256) {
                    const int r = e % NB, c = e / NB;
                    Lj[r][c] = (r >= nc && r < nr && c < nc) ? T[r][c] : 0.0;
                    if (r >= nc || c > r) T[r][c] = 0.0;
                }
                __syncthreads();
                factor_block(T, rp, nc, c0, flags, &failed_at);
                // the factor and its reciprocal pivots (the inverse's
                // diagonal) are all the panel solves read: publish them now
                for (int e = tid; e < NB * NB; e += 256) {
                    const int r = e / NB, c = e % NB;
                    if (r < nc && c <= r) M[(size_t)(c0 + c) * ld + c0 + r] = T[r][c];
                }
                if (tid < NB) Dinv[(size_t)j * NB * NB + tid * (NB + 1)] = tid < nc ? rp[tid] : 0.0;
                df_publish(ready + j);
                // the right-hand-side row, by the same substitution
                if (nr > nc) {
                    for (int e = tid; e < NB * NB; e += 256) {
                        const int r = e / NB, c = e % NB;
                        if (r < nr - nc) Li[r][c] = Lj[nc + r][c];
                    }
                    __syncthreads();
                    subst_block(Li, nr - nc, T, rp, nc);
                    for (int c = tid; c < nc; c += 256) M[(size_t)(c0 + c) * ld + r0 + nc] = Li[0][c];
                    df_publish(ready + nbc + (size_t)j * nbr + i);
                }
                // the inverse (for the backward sweep after this launch)
                invert_block(T, Lj, rp, nc);
                for (int e = tid; e < NB * NB; e += 256) Dinv[(size_t)j * NB * NB + e] = Lj[e / NB][e % NB];
            } else {
                if (!df_wait(ready + j, abort, &ok_sh)) goto fail;
                for (int e = tid; e < NB * NB; e += 256) {
                    const int r = e / NB, c = e % NB;
                    Li[r][c] = (r < nc && c <= r) ? __ldcg(M + (size_t)(c0 + c) * ld + c0 + r) : 0.0;
                }
                if (tid < NB) rp[tid] = __ldcg(Dinv + (size_t)j * NB * NB + tid * (NB + 1));
                __syncthreads();
                subst_block(T, nr, Li, rp, nc);
                for (int e = tid; e < NB * NB; e += 256) {
                    const int c = e / NB, r = e % NB;
                    if (c < nc && r < nr) M[(size_t)(c0 + c) * ld + r0 + r] = T[r][c];
                }
                df_publish(ready + nbc + (size_t)j * nbr + i);
            }
            __syncthreads();
        }
    }
    return;
fail:
    if (tid == 0) {
        *(volatile int *)abort = 1;
        atomicExch(flags, -1);
        atomicExch(flags + 1, CHOL_WAIT_CODE | (int)blockIdx.x);
    }
}

// CTAs of the data-flow factorization on the current device (one per SM at
// most, all resident), or 0 when a cooperative launch is not possible.
// Computed per device and published once, as for the backward sweep.
int df_capacity() {
    constexpr int kDevices = 64;
    static std::atomic<int> cap_plus1[kDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (dev < 0 || dev >= kDevices) return 0;
    int c = cap_plus1[dev].load(std::memory_order_acquire);
    if (c == 0) {
        int coop = 0, per_sm = 0, sms = 0, cap = 0;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_df_kernel, 256, 0) != cudaSuccess)
            cudaGetLastError();
        else if (coop && per_sm > 0)
            cap = sms;
        c = cap + 1;
        cap_plus1[dev].store(c, std::memory_order_release);
    }
    return c - 1;
}

int g_chol_path = 0;  // 0: data flow when possible, 1: multi-launch, 2: data flow only

// Words of the ready list for order n (with the right-hand-side row): one per
// diagonal block, one per tile, one abort word.
size_t df_ready_words(int n, int has_b) {
    const size_t nbc = (size_t)(n + NB - 1) / NB, nbr = (size_t)(n + has_b + NB - 1) / NB;
    return nbc + nbc * nbr + 1;
}

// Enqueues the whole factorization (and the solve when has_b) on `st`, with
// Dinv holding ceil(n/32) blocks of 32x32 doubles. Row n of M (the
// right-hand side) is scratch on return: which backward sweep runs decides
// what it holds.
// The same backward sweep on several CTAs (a cooperative launch): thread t
// of CTA k owns row 256 k + t of z, which is row n of M updated in place.
// Per 32-row block from the bottom, every CTA forms x_b = D_b^-T y_b in
// shared memory from the block's rows of z (final since the previous block),
// CTA 0 stores it, and the owners of the rows above subtract L_b^T x_b; every
// value takes the single-CTA sweep's FMAs in the same order, so the results
// are the same bits. A grid barrier closes each block; the next block's
// inverse is loaded into the other shared buffer before it.
__global__ void __launch_bounds__(256) chol_backsolve_coop_kernel(double *__restrict__ M, int n, int ld,
                                                                  const double *__restrict__ Dinv,
                                                                  double *__restrict__ x) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    __shared__ double Di[2][NB][NB + 1];  // this block's inverse and the next one's, loaded ahead
    __shared__ double yb[NB];
    __shared__ double xb[NB];
    const int tid = threadIdx.x;
    const int r = blockIdx.x * blockDim.x + tid;
    double *z = M + n;  // z[c] at z[c * ld]
    const int nblk = (n + NB - 1) / NB;
    for (int t = tid; t < NB * NB; t += blockDim.x)
        Di[(nblk - 1) & 1][t / NB][t % NB] = Dinv[(size_t)(nblk - 1) * NB * NB + t];
    for (int b = nblk - 1; b >= 0; --b) {
        const int r0 = b * NB, r1 = min(n, r0 + NB), u = b & 1;
        if (tid < NB) yb[tid] = (r0 + tid < r1) ? z[(size_t)(r0 + tid) * ld] : 0.0;
        __syncthreads();
        if (tid < r1 - r0) {
            const double v = sweep_dot(Di[u], yb, tid, r1 - r0);
            xb[tid] = v;
            if (blockIdx.x == 0) x[r0 + tid] = v;
        }
        __syncthreads();
        if (r < r0) z[(size_t)r * ld] = z[(size_t)r * ld] - sweep_row(M + (size_t)r * ld + r0, xb, r1 - r0);
        if (b > 0)
            for (int t = tid; t < NB * NB; t += blockDim.x)
                Di[u ^ 1][t / NB][t % NB] = Dinv[(size_t)(b - 1) * NB * NB + t];
        grid.sync();
    }
}

// CTAs of the cooperative sweep for order n on the current device, or 0 when
// they cannot all be resident at once (the single-CTA sweep is used then).
// The capacity is computed per device from the device's own attributes (the
// library context need not exist: the allocation-free solve runs without it)
// and published only once computed; concurrent first calls compute the same
// value. Only errors of these queries are cleared, never one the caller left.
int coop_backsolve_ctas(int n) {
    constexpr int kDevices = 64;
    static std::atomic<int> cap_plus1[kDevices];  // 0: not computed yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (dev < 0 || dev >= kDevices) return 0;
    int c = cap_plus1[dev].load(std::memory_order_acquire);
    if (c == 0) {
        int coop = 0, per_sm = 0, sms = 0, cap = 0;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_backsolve_coop_kernel, 256, 0) != cudaSuccess)
            cudaGetLastError();
        else if (coop)
            cap = per_sm * sms;
        c = cap + 1;
        cap_plus1[dev].store(c, std::memory_order_release);
    }
    const int g = (n + 255) / 256;
    return g <= c - 1 ? g : 0;
}

int chol_enqueue_panels(double *d_M, int n, int ld, int nrows, int *flags, double *Dinv, cudaStream_t st);
int chol_enqueue_backsolve(double *d_M, int n, int ld, double *d_x, double *Dinv, cudaStream_t st);

// ready: the data-flow path's list (df_ready_words words), or NULL for the
// multi-launch path.
int chol_enqueue(double *d_M, int n, int ld, double *d_x, int *flags, double *Dinv, cudaStream_t st,
                 unsigned *ready = nullptr) {
    const int has_b = d_x != nullptr;
    const int nrows = n + has_b;
    const int G = ready && g_chol_path != 1 ? df_capacity() : 0;
    if (G > 0) {
        // one cooperative launch of the data-flow factorization
        const size_t words = df_ready_words(n, has_b);
        cudaError_t e = cudaMemsetAsync(ready, 0, words * sizeof(unsigned), st);
        const int nbc = (n + NB - 1) / NB, nbr = (nrows + NB - 1) / NB;
        const int tasks = nbc * (2 * nbr - nbc + 1) / 2;
        int grid = std::min(G, tasks);
        int *abort = (int *)(ready + words - 1);
        void *args[] = {&d_M, &n, &ld, (void *)&nrows, &flags, &Dinv, &ready, &abort};
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void *)chol_df_kernel, dim3(grid), dim3(256), args, 0, st);
        if (e != cudaSuccess) {
            irwls_set_error(-2, "CUDA error in chol_df (cooperative): %s", cudaGetErrorString(e));
            return -2;
        }
        irwls_count_launch(1);
    } else if (g_chol_path == 2) {
        irwls_set_error(-2, "the data-flow Cholesky needs a cooperative launch");
        return -2;
    } else {
        const int rc = chol_enqueue_panels(d_M, n, ld, nrows, flags, Dinv, st);
        if (rc) return rc;
    }
    return has_b ? chol_enqueue_backsolve(d_M, n, ld, d_x, Dinv, st) : 0;
}

// The multi-launch factorization: per panel a solve launch and an update
// launch (whose tile (0, 0) factors the next diagonal block).
int chol_enqueue_panels(double *d_M, int n, int ld, int nrows, int *flags, double *Dinv, cudaStream_t st) {
    chol_factor0_kernel<<<1, 256, 0, st>>>(d_M, n, ld, flags, Dinv);
    IRWLS_LAUNCH_CHECK("chol_factor0");
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int nb = min(NB, n - k0);
        const int below = nrows - (k0 + nb);
        if (below <= 0) break;
        chol_trsm_kernel<<<ceil_div(below, 8), 256, 0, st>>>(d_M, ld, k0, nb, nrows,
                                                             Dinv + (size_t)(k0 / NB) * NB * NB);
        IRWLS_LAUNCH_CHECK("chol_trsm");
        if (k0 + nb < n) {
            dim3 g(ceil_div(n - (k0 + nb), 32), ceil_div(below, 32));
            chol_update_kernel<<<g, 256, 0, st>>>(d_M, n, ld, k0, nb, nrows, flags,
                                                  Dinv + (size_t)(k0 / NB + 1) * NB * NB);
            IRWLS_LAUNCH_CHECK("chol_update");
        }
    }
    return 0;
}

// The backward sweep L^T x = z (z in row n of M).
int chol_enqueue_backsolve(double *d_M, int n, int ld, double *d_x, double *Dinv, cudaStream_t st) {
    {
        const int g = coop_backsolve_ctas(n);
        if (g > 0) {
            void *args[] = {&d_M, &n, &ld, &Dinv, &d_x};
            const cudaError_t e = cudaLaunchCooperativeKernel((const void *)chol_backsolve_coop_kernel, dim3(g),
                                                              dim3(256), args, 0, st);
            if (e != cudaSuccess) {
                irwls_set_error(-2, "CUDA error in chol_backsolve (cooperative): %s", cudaGetErrorString(e));
                return -2;
            }
            irwls_count_launch(1);
            return 0;
        }
        const size_t smem = (size_t)n * sizeof(double);
        if (smem > 48 * 1024) {
            if (smem > 160 * 1024) {
                irwls_set_error(-6, "system of order %d exceeds the backward-solve tile", n);
                return -6;
            }
            cudaFuncSetAttribute(chol_backsolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        }
        chol_backsolve_kernel<<<1, 256, smem, st>>>(d_M, n, ld, Dinv, d_x);
        IRWLS_LAUNCH_CHECK("chol_backsolve");
    }
    return 0;
}


}  // namespace

extern "C" int irwls_dev_zero_upper(double *d_M, int n, int ld) {
    if (n <= 1) return 0;
    zero_upper_kernel<<<ceil_div((long long)n * n, 256) < 4096 ? ceil_div((long long)n * n, 256) : 4096, 256, 0,
                        irwls_stream()>>>(d_M, n, ld);
    IRWLS_LAUNCH_CHECK("zero_upper");
    return 0;
}

extern "C" int irwls_dev_chol_solve(double *d_M, int n, int ld, const double *d_b, double *d_x) {
    if (n <= 0) return 0;
    if (ld < n + 1) {
        irwls_set_error(-6, "Cholesky leading dimension %d < n + 1 = %d", ld, n + 1);
        return -6;
    }
    int *flags = irwls_dev_flags();
    if (irwls_dev_memset(flags, 0, sizeof(int))) return -2;
    if (d_b) {
        // b becomes row n: M[c*ld + n] = b[c]
        cudaError_t e = cudaMemcpy2DAsync(d_M + n, (size_t)ld * sizeof(double), d_b, sizeof(double), sizeof(double), n,
                                          cudaMemcpyDeviceToDevice, irwls_stream());
        if (e != cudaSuccess) {
            irwls_set_error(-2, "rhs copy: %s", cudaGetErrorString(e));
            return -2;
        }
    }
    const int npanel = ceil_div(n, NB);
    // factored diagonal blocks: the context's grow-only scratch slot 0
    double *diag = (double *)irwls_ctx_scratch(0, (size_t)npanel * NB * NB * sizeof(double));
    if (!diag) return -3;
    // ready list of the data-flow path: the context's grow-only slot 3
    unsigned *ready = (unsigned *)irwls_ctx_scratch(3, df_ready_words(n, d_x != nullptr) * sizeof(unsigned));
    if (!ready) return -3;
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_CHOL);
    int rc = chol_enqueue(d_M, n, ld, d_x, flags, diag, irwls_stream(), ready);
    if (rc) return rc;
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_CHOL);
    return 0;
}

extern "C" int irwls_chol_sweep_ctas(int n) { return coop_backsolve_ctas(n); }

// Test hook: 0 = the data-flow factorization where a cooperative launch is
// possible (default), 1 = the multi-launch factorization, 2 = data flow only.
extern "C" void irwls_debug_chol_path(int mode) { g_chol_path = mode >= 0 && mode <= 2 ? mode : 0; }

extern "C" int irwls_dev_pivot_status(int *info) {
    *info = 0;
    cudaError_t e = cudaMemcpyAsync(info, irwls_dev_flags(), sizeof(int), cudaMemcpyDeviceToHost, irwls_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(irwls_stream());
    if (e != cudaSuccess) {
        irwls_set_error(-2, "CUDA error reading the pivot status: %s", cudaGetErrorString(e));
        return -2;
    }
    return 0;
}

namespace {
// out = A v (trans = 0) or out = A^T v (trans = 1) for a column-major size x
// size matrix; one warp per output entry.
__global__ void gemv_kernel(const double *__restrict__ A, const double *__restrict__ v, double *__restrict__ out,
                            int size, int trans) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= size) return;
    double acc = 0.0;
    if (trans)
        for (int i = lane; i < size; i += 32) acc = fma(A[(size_t)w * size + i], v[i], acc);
    else
        for (int j = lane; j < size; j += 32) acc = fma(A[(size_t)j * size + w], v[j], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[w] = acc;
}
}  // namespace

extern "C" int irwls_dev_gemv(const double *d_A, const double *d_v, double *d_out, int size, int trans) {
    if (size <= 0) return 0;
    gemv_kernel<<<ceil_div((long long)size * 32, 256), 256, 0, irwls_stream()>>>(d_A, d_v, d_out, size, trans);
    IRWLS_LAUNCH_CHECK("gemv");
    return 0;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the Cholesky solve.
//
// Some callers cannot let a library allocate device memory while they run: a
// serving process that reserved the device's memory for its own pool
// allocator at start-up (a cudaMalloc in the middle of a request can fail, or
// force the pool to give memory back), or a latency-sensitive caller for whom
// cudaMalloc/cudaFree must not run because they can synchronize the whole
// device. irwls_chol_solve_noalloc serves them: the caller passes the matrix,
// the right-hand side and the output (all device memory the caller owns) and a
// stream, and the call itself allocates nothing. Its only scratch is the
// file-scope array below, which every GPU that loads this library holds until
// the process exits.
//
// The scratch keeps the inverted 32x32 diagonal blocks (one per panel), the
// status words and the ready list of the data-flow factorization, which
// sizes it for matrices of order up to IRWLS_NOALLOC_MAX_ORDER (4096: 1 MiB
// of blocks and 65 KiB of ready words, about 1.06 MiB in all).
// ---------------------------------------------------------------------------
#define IRWLS_NOALLOC_MAX_ORDER 4096
#define IRWLS_NOALLOC_PANELS (IRWLS_NOALLOC_MAX_ORDER / NB)
// ready words of the data-flow factorization at the largest order (with the
// right-hand-side row), rounded up to whole doubles
#define IRWLS_NOALLOC_READY (IRWLS_NOALLOC_PANELS + IRWLS_NOALLOC_PANELS * (IRWLS_NOALLOC_PANELS + 1) + 1)

static __device__ __align__(256) double
    g_noalloc_scratch[IRWLS_NOALLOC_PANELS * NB * NB + 32 + (IRWLS_NOALLOC_READY + 1) / 2];

#define IRWLS_NOALLOC_DEVICES 64
static double *g_noalloc_addr[IRWLS_NOALLOC_DEVICES];  // device address of the array, per device

extern "C" int irwls_chol_solve_noalloc(double *d_M, int n, int ld, const double *d_b, double *d_x, int *d_info,
                                        void *stream) {
    irwls_clear_error();
    // A CUDA error the caller left pending would be taken for one of this
    // call's launches (each launch is checked with cudaGetLastError, which
    // clears it): refuse instead, and leave the caller's error in place.
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        irwls_set_error(-14, "irwls_chol_solve_noalloc: a CUDA error is already pending (%s); not cleared",
                        cudaGetErrorString(pending));
        return -14;
    }
    if (n <= 0) return 0;
    if (n > IRWLS_NOALLOC_MAX_ORDER) {
        irwls_set_error(-11, "irwls_chol_solve_noalloc: order %d exceeds its limit of %d", n, IRWLS_NOALLOC_MAX_ORDER);
        return -11;
    }
    if (ld < n + 1) {
        irwls_set_error(-6, "irwls_chol_solve_noalloc: leading dimension %d < n + 1 = %d", ld, n + 1);
        return -6;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= IRWLS_NOALLOC_DEVICES) {
        irwls_set_error(-2, "irwls_chol_solve_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return -2;
    }
    // Set-up, once per device, with that device current: the host-side name
    // of the array is not a device address, so ask the runtime for it.
    if (!g_noalloc_addr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            irwls_set_error(-2, "irwls_chol_solve_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return -2;
        }
        g_noalloc_addr[dev] = p;
    }
    double *diag = g_noalloc_addr[dev];
    int *flags = (int *)(diag + IRWLS_NOALLOC_PANELS * NB * NB);
    unsigned *ready = (unsigned *)(diag + IRWLS_NOALLOC_PANELS * NB * NB + 32);
    cudaStream_t st = (cudaStream_t)stream;
    // the pivot status must start at zero; the diagonal blocks are fully
    // rewritten before they are read
    if ((e = cudaMemsetAsync(flags, 0, sizeof(int), st)) != cudaSuccess) {
        irwls_set_error(-2, "irwls_chol_solve_noalloc: %s", cudaGetErrorString(e));
        return -2;
    }
    if (d_b) {
        e = cudaMemcpy2DAsync(d_M + n, (size_t)ld * sizeof(double), d_b, sizeof(double), sizeof(double), n,
                              cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            irwls_set_error(-2, "irwls_chol_solve_noalloc: rhs copy: %s", cudaGetErrorString(e));
            return -2;
        }
    }
    // order <= 4096: the backward sweep's vector fits the default 48 KiB
    const int rc = chol_enqueue(d_M, n, ld, d_x, flags, diag, st, ready);
    if (rc) return rc;
    if (d_info && (e = cudaMemcpyAsync(d_info, flags, sizeof(int), cudaMemcpyDeviceToDevice, st)) != cudaSuccess) {
        irwls_set_error(-2, "irwls_chol_solve_noalloc: %s", cudaGetErrorString(e));
        return -2;
    }
    return 0;
}
