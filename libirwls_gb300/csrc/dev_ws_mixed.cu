// dev_ws_mixed.cu -- the precision form's working-set solve of full IRWLS:
// FP32 Cholesky in one thread-block cluster, FP64 iterative refinement.
//
// The reference solves the bordered system
//
//   [ H    y ] [ x  ]   [ r   ]
//   [ y^T  0 ] [ xn ] = [ r_n ]        (src/full-train.c:165-196)
//
// by dpotrf + dpotrs (src/ParallelAlgorithms.c:361-388). Its last pivot is
// -s with s = y^T H^-1 y > 0, which dpotrf stores without a root and
// reports; dpotrs then solves with that factor, i.e. with the matrix
// [H y; y^T s + s^2]. Written out by block elimination that solution is
//
//   u = H^-1 y,  v = H^-1 r,  s = y^T u,
//   xn = (r_n - y^T v) / s^2,   x = v - u xn,
//
// which this kernel computes with H itself SPD (H = K o y y^T + diag(1/a)).
// H's working-set systems are well conditioned (condition numbers below
// 10^3 on the full-IRWLS workloads), so an FP32 factor with FP64 residuals
// reaches FP64 accuracy in two refinement steps.
//
// One cluster of 16 CTAs (a 4 x 4 grid (p, q)) holds H in distributed shared
// memory as 32 x 32 FP32 blocks, block (i, j) (i >= j) on CTA
// (i mod 4, j mod 4). Per block column k:
//   F  the owner of (k, k) factors it (one warp, shuffles; LAPACK's
//      unblocked right-looking order);
//   P  the owners of (i, k), i > k, solve L_ik L_kk^T = A_ik by substitution;
//      the owners of row k of W = L^-1 scale it by L_kk^-1 (substitution);
//   U  every CTA copies the panel blocks it needs from their owners' shared
//      memory and applies A_ij -= L_ik L_jk^T (k < j <= i) and
//      W_ij -= L_ik W_kj (i > k, j <= k) to its own blocks; the owner of
//      (k + 1, k + 1) then factors it.
// A cluster barrier separates F/P and P/U. W = L^-1 is formed alongside the
// factor, so each solve with the factor is two block GEMVs (z = W b,
// x = W^T z) instead of two triangular sweeps. The refinement residuals
// b - H x are FP64 over H's FP64 entries in global memory.
//
// Every reduction has a fixed order, so the result does not depend on
// timing. All CTAs run the same sequence of cluster barriers (the control
// flow depends only on n1 and on values every CTA computes identically).
// The outcome is reported in device flag word 2: 0 solved, 1 an FP32 pivot
// was not positive, 2 the refinement did not converge; the caller then
// solves the system in FP64 instead.
#include <cooperative_groups.h>

#include <atomic>

#include "dev_common.cuh"
#include "tc_ptx.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int WB = 32;                     // block size
constexpr int WNB = 16;                    // blocks per dimension: order <= 512
constexpr int WP = 4, WQ = 4;              // CTA grid of the cluster
constexpr int WC = WP * WQ;                // cluster size
constexpr int WT = 512;                    // threads per CTA
constexpr int WWARPS = WT / 32;
constexpr int LDB = WB + 1;                // padded row of a stored block
constexpr int BLK = WB * LDB;              // floats per stored block
constexpr int SR = WNB / WP, SCOL = WNB / WQ;  // owned row / column blocks per CTA
constexpr int SLOTS = SR * (SR + 1) / 2;       // owned blocks of a CTA (at most 10: p >= q)
constexpr int MAXIT = 5;                   // refinement steps before giving up

// shared-memory layout (floats); the receive and send buffers come in two
// sets, used by steps of even and odd k
constexpr int PSET = SR * WB * WB + 2 * SCOL * BLK;  // one set of receive buffers
constexpr int OFF_A = 0;                       // A slots: the factor L
constexpr int OFF_W = OFF_A + SLOTS * BLK;     // W slots: L^-1
constexpr int OFF_PL = OFF_W + SLOTS * BLK;    // panel L_ik of my rows, transposed [t][r]
constexpr int OFF_PC = OFF_PL + SR * WB * WB;  // panel L_jk of my columns [c][t]
constexpr int OFF_PW = OFF_PC + SCOL * BLK;    // row k of W for my columns [t][c]
constexpr int OFF_DK = OFF_PL + 2 * PSET;      // L_kk, two buffers
constexpr int OFF_STG = OFF_DK + 2 * BLK;      // my panel blocks transposed, for sending (two sets)
constexpr int OFF_DI = OFF_STG + 2 * SR * WB * WB;  // 1 / L_kk[t][t]
constexpr int SMEM_FLOATS = OFF_DI + WB;
constexpr size_t SMEM_BYTES = (size_t)SMEM_FLOATS * sizeof(float);
static_assert(SMEM_BYTES + 256 <= 227 * 1024, "shared memory");

// after the factorization the A slots and the panel buffers hold the solve's
// vectors (same offsets in every CTA: partial sums are read remotely)
constexpr int NV = WNB * WB;                   // padded order
constexpr int OFF_VEC = OFF_PL;                // doubles: y, r, u, v
constexpr int OFF_BF = OFF_VEC + 2 * 4 * NV;   // floats: solve input [2][NV]
constexpr int OFF_CF = OFF_BF + 2 * NV;        // floats: solve output [2][NV]
constexpr int OFF_DP = OFF_CF + 2 * NV;        // doubles: per-slot row partials [SLOTS][2][WB]
constexpr int OFF_DPC = OFF_DP + 2 * SLOTS * 2 * WB;  // doubles: per-slot column partials
constexpr int OFF_VEND = OFF_DPC + 2 * SLOTS * 2 * WB;
constexpr int OFF_ZP = OFF_VEND;               // floats: z partials [SR][2][WB]
constexpr int OFF_ZF = OFF_ZP + SR * 2 * WB;   // floats: reduced z of my rows
constexpr int OFF_XP = OFF_ZF + SR * 2 * WB;   // floats: x partials [SCOL][2][WB]
constexpr int OFF_BP = OFF_XP + SCOL * 2 * WB; // floats: per-slot partials [SLOTS][2][WB]
constexpr int OFF_RR = OFF_BP + SLOTS * 2 * WB;        // doubles: row residual partials [SR][2][WB]
constexpr int OFF_RC = OFF_RR + 2 * SR * 2 * WB;       // doubles: column residual partials [SCOL][2][WB]
constexpr int OFF_PEND = OFF_RC + 2 * SCOL * 2 * WB;
static_assert(OFF_PEND <= OFF_DK, "solve vectors overflow the receive buffers");
static_assert((OFF_PL % 4) == 0 && (OFF_RR % 2) == 0 && (OFF_DP % 2) == 0, "alignment");

// Slot of block (i, j), j <= i, on its owner: the owner's blocks in order of
// (i / WP, j / WQ); a CTA with p >= q owns a + 1 of them in block row a, one
// with p < q owns a.
__device__ __forceinline__ int slot_of(int i, int j) {
    const int a = i / WP, b = j / WQ;
    return (i % WP >= j % WQ) ? a * (a + 1) / 2 + b : a * (a - 1) / 2 + b;
}
__device__ __forceinline__ int owner_of(int i, int j) { return (i % WP) * WQ + (j % WQ); }

// Factors the stored block in place (lane = row), LAPACK's unblocked
// right-looking order; the upper part is cleared. Returns true if every pivot
// was positive.
__device__ bool factor_warp(float *D, int lane) {
    float a[WB];
#pragma unroll
    for (int t = 0; t < WB; ++t) a[t] = D[lane * LDB + t];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < WB; ++k) {
        const float piv = __shfl_sync(0xffffffffu, a[k], k);
        ok = ok && (piv > 0.f);
        const float rs = rsqrtf(piv);
        const float l = a[k] * rs;
        a[k] = l;
#pragma unroll
        for (int j = k + 1; j < WB; ++j) {
            const float lj = __shfl_sync(0xffffffffu, l, j);
            a[j] = fmaf(-l, lj, a[j]);
        }
    }
#pragma unroll
    for (int t = 0; t < WB; ++t) D[lane * LDB + t] = t <= lane ? a[t] : 0.f;
    return ok;
}

// X L^T = B in place, lane = row of B (B stored [r][t]).
__device__ void subst_rows(float *B, const float *Dk, const float *dinv, int lane) {
    float a[WB];
#pragma unroll
    for (int t = 0; t < WB; ++t) a[t] = B[lane * LDB + t];
#pragma unroll
    for (int s = 0; s < WB; ++s) {
        a[s] *= dinv[s];
#pragma unroll
        for (int t = s + 1; t < WB; ++t) a[t] = fmaf(-a[s], Dk[t * LDB + s], a[t]);
    }
#pragma unroll
    for (int t = 0; t < WB; ++t) B[lane * LDB + t] = a[t];
}

// L X = B in place, lane = column of B (B stored [t][c]); B = I when `ident`.
__device__ void subst_cols(float *B, const float *Dk, const float *dinv, int lane, bool ident) {
    float b[WB];
#pragma unroll
    for (int t = 0; t < WB; ++t) b[t] = ident ? (t == lane ? 1.f : 0.f) : B[t * LDB + lane];
#pragma unroll
    for (int s = 0; s < WB; ++s) {
        b[s] *= dinv[s];
#pragma unroll
        for (int t = s + 1; t < WB; ++t) b[t] = fmaf(-Dk[t * LDB + s], b[s], b[t]);
    }
#pragma unroll
    for (int t = 0; t < WB; ++t) B[t * LDB + lane] = b[t];
}

// out[r][c] -= sum_t LT[t][r] R(t, c), lane = c; R(t, c) = R[c][t] (a block of
// L, `by_t` false) or R[t][c] (a block of W). Sum over t in increasing order.
__device__ void block_update(float *out, const float *LT, const float *R, bool by_t, int lane) {
    float acc[WB];
#pragma unroll
    for (int r = 0; r < WB; ++r) acc[r] = 0.f;
#pragma unroll 4
    for (int t = 0; t < WB; ++t) {
        const float rv = by_t ? R[t * LDB + lane] : R[lane * LDB + t];
        const float4 *l4 = (const float4 *)(LT + t * WB);
#pragma unroll
        for (int q = 0; q < WB / 4; ++q) {
            const float4 l = l4[q];
            acc[4 * q] = fmaf(l.x, rv, acc[4 * q]);
            acc[4 * q + 1] = fmaf(l.y, rv, acc[4 * q + 1]);
            acc[4 * q + 2] = fmaf(l.z, rv, acc[4 * q + 2]);
            acc[4 * q + 3] = fmaf(l.w, rv, acc[4 * q + 3]);
        }
    }
#pragma unroll
    for (int r = 0; r < WB; ++r) out[r * LDB + lane] -= acc[r];
}

constexpr long long WS_WAIT_LIMIT = 1LL << 22;  // polls of a data wait before it gives up

// The shared::cluster address, in CTA `rank`, of a local shared address (the
// layout is the same in every CTA).
__device__ __forceinline__ uint32_t cl_addr(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

// Sends `bytes` of this CTA's shared memory at src to the same offset dst in
// CTA `rank` with the bulk-copy engine; the copy completes on that CTA's
// mbarrier at offset bar. The caller has made the source visible to the
// async proxy (fence.proxy.async after the writes).
__device__ __forceinline__ void send(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar, int rank) {
    asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     cl_addr(dst, rank)),
                 "r"(src), "r"(bytes), "r"(cl_addr(bar, rank))
                 : "memory");
}

__device__ __forceinline__ void expect_bytes(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Bounded wait for the phase of parity `parity` of the mbarrier at bar.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity) {
    uint32_t done = 0;
    for (long long it = 0; it < WS_WAIT_LIMIT && !done; ++it)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    return done != 0;
}

__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// The two halves of a cluster barrier (every thread of every CTA calls them,
// alternately).
__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

// Panel blocks of step k that CTA (p, q) receives: L_ik of its row blocks
// i > k (transposed, 4 KB each), L_jk of its column blocks j > k and W_kj of
// its column blocks j <= k (4224 bytes each).
__device__ __forceinline__ uint32_t panel_bytes(int k, int NB, int p, int q) {
    const int i0 = k + 1 + ((p - (k + 1)) % WP + WP) % WP;
    const int j0 = k + 1 + ((q - (k + 1)) % WQ + WQ) % WQ;
    const int nPL = i0 < NB ? (NB - 1 - i0) / WP + 1 : 0;
    const int nPC = j0 < NB ? (NB - 1 - j0) / WQ + 1 : 0;
    const int nPW = q <= k ? (k - q) / WQ + 1 : 0;
    return (uint32_t)(nPL * WB * WB * 4 + (nPC + nPW) * BLK * 4);
}

__global__ void __launch_bounds__(WT, 1) ws_mixed_kernel(const double *__restrict__ H, int n1, int ld,
                                                       const double *__restrict__ rhs, double *__restrict__ x,
                                                       int *__restrict__ flags) {
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) float sm[];
    __shared__ int bad_sh, flag_sh;
    __shared__ float redf[WWARPS];
    __shared__ double xn_sh;
    // panel blocks received, L_kk received: one mbarrier per buffer set
    __shared__ __align__(8) uint64_t pan_bar[2], dk_bar[2];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int me = (int)cl.block_rank();
    const int p = me / WQ, q = me % WQ;
    const int NB = (n1 + WB - 1) / WB;
    float *A = sm + OFF_A, *W = sm + OFF_W, *PL = sm + OFF_PL, *PC = sm + OFF_PC, *PW = sm + OFF_PW;
    float *Dk = sm + OFF_DK, *STG = sm + OFF_STG, *dinv = sm + OFF_DI;
    const uint32_t dk_b0 = smem_u32(&dk_bar[0]), dk_b1 = smem_u32(&dk_bar[1]);
    if (tid == 0) {
        bad_sh = 0;
        mbar_init(&pan_bar[0], 1);
        mbar_init(&pan_bar[1], 1);
        mbar_init(&dk_bar[0], 1);
        mbar_init(&dk_bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }

    // ---- load my blocks of H (FP32, identity beyond n1) and W = I ----
    for (int ib = p; ib < NB; ib += WP)
        for (int jb = q; jb <= ib; jb += WQ) {
            float *a = A + slot_of(ib, jb) * BLK, *w = W + slot_of(ib, jb) * BLK;
            for (int e = tid; e < WB * WB; e += WT) {
                const int r = e & 31, c = e >> 5, gi = ib * WB + r, gj = jb * WB + c;
                float v;
                if (gi < n1 && gj < n1) v = gi >= gj ? __double2float_rn(H[(size_t)gj * ld + gi]) : 0.f;
                else v = gi == gj ? 1.f : 0.f;
                a[r * LDB + c] = v;
                w[r * LDB + c] = gi == gj ? 1.f : 0.f;
            }
        }
    __syncthreads();
    cl.sync();  // every CTA's mbarriers are initialized before anything is sent

    // L_kk (factored by its owner's warp 0) to the CTAs of block row and
    // block column k, into the Dk buffer of step parity k & 1; lane 0 sends
    auto send_dk = [&](int kk) {
        __syncwarp();
        if (lane == 0) {
            proxy_fence();
            const uint32_t src = smem_u32(A + slot_of(kk, kk) * BLK), dst = smem_u32(Dk + (kk & 1) * BLK);
            const uint32_t bar = (kk & 1) ? dk_b1 : dk_b0;
            for (int qq = 0; qq < WQ; ++qq) send(dst, src, BLK * 4, bar, (kk % WP) * WQ + qq);
            for (int pp = 0; pp < WP; ++pp)
                if (pp != kk % WP) send(dst, src, BLK * 4, bar, pp * WQ + kk % WQ);
        }
    };
    if (NB > 0 && owner_of(0, 0) == me && warp == 0) {
        if (!factor_warp(A + slot_of(0, 0) * BLK, lane) && lane == 0) bad_sh = 1;
        send_dk(0);
    }

    // ---- factorization with W = L^-1 alongside ----
    // Every block a step produces is sent by its owner to the CTAs whose
    // updates read it; a receiver waits on its mbarrier for the bytes it
    // expects. Steps of even and odd k use separate buffer sets (receive
    // buffers, send staging, L_kk, mbarriers), and a split cluster barrier
    // runs one step behind: a CTA arrives when it has finished step k and,
    // before it sends anything of step k + 2 into the set of step k (L_{k+2,
    // k+2} at the end of step k + 1, panel blocks in step k + 2), waits until
    // every CTA has arrived for step k. No CTA waits for the others' step
    // k + 1.
    int dk_n[2] = {0, 0};  // L_kk blocks received per buffer (the mbarrier phases)
    for (int k = 0; k < NB; ++k) {
        const int par = k & 1;
        float *PLk = PL + par * PSET, *PCk = PC + par * PSET, *PWk = PW + par * PSET;
        float *STGk = STG + par * SR * WB * WB;
        const uint32_t pan_b = smem_u32(&pan_bar[par]);
        const bool col_k = k % WQ == q, row_k = k % WP == p;
        if (col_k || row_k) {
            const uint32_t bar = (k & 1) ? dk_b1 : dk_b0;
            if (tid == 0) expect_bytes(bar, BLK * 4);
            if (!wait_phase(bar, (uint32_t)dk_n[k & 1] & 1u)) bad_sh = 3;
            ++dk_n[k & 1];
            const float *D = Dk + (k & 1) * BLK;
            if (tid < WB) dinv[tid] = __frcp_rn(D[tid * LDB + tid]);
            __syncthreads();
            // one warp per task: panel rows below k in column k, then row k
            // of W; each block is sent as soon as it is solved
            int task = 0;
            if (col_k)
                for (int ib = p; ib < NB; ib += WP) {
                    if (ib <= k || task++ % WWARPS != warp) continue;
                    float *blk = A + slot_of(ib, k) * BLK, *st = STGk + (ib / WP) * WB * WB;
                    subst_rows(blk, D, dinv, lane);
                    __syncwarp();
#pragma unroll 8
                    for (int t = 0; t < WB; ++t) st[t * WB + lane] = blk[lane * LDB + t];
                    __syncwarp();
                    if (lane == 0) {
                        proxy_fence();
                        for (int qq = 0; qq < WQ; ++qq)
                            send(smem_u32(PLk + (ib / WP) * WB * WB), smem_u32(st), WB * WB * 4, pan_b, p * WQ + qq);
                        for (int pp = 0; pp < WP; ++pp)
                            send(smem_u32(PCk + (ib / WQ) * BLK), smem_u32(blk), BLK * 4, pan_b, pp * WQ + ib % WQ);
                    }
                }
            if (row_k)
                for (int jb = q; jb <= k; jb += WQ) {
                    if (task++ % WWARPS != warp) continue;
                    float *blk = W + slot_of(k, jb) * BLK;
                    subst_cols(blk, D, dinv, lane, jb == k);
                    __syncwarp();
                    if (lane == 0) {
                        proxy_fence();
                        for (int pp = 0; pp < WP; ++pp)
                            send(smem_u32(PWk + (jb / WQ) * BLK), smem_u32(blk), BLK * 4, pan_b, pp * WQ + q);
                    }
                }
        }
        if (tid == 0) expect_bytes(pan_b, panel_bytes(k, NB, p, q));
        if (!wait_phase(pan_b, (uint32_t)(k >> 1) & 1u)) bad_sh = 3;
        __syncthreads();
        // the next diagonal block first, by warp 0, which then factors it
        // and sends it while the other warps apply the remaining updates
        const bool own_next = k + 1 < NB && owner_of(k + 1, k + 1) == me;
        int task = 0;
        for (int ib = p; ib < NB; ib += WP) {
            if (ib <= k) continue;
            for (int jb = q; jb <= ib; jb += WQ) {
                int w;
                if (own_next && ib == k + 1 && jb == k + 1) w = 0;
                else w = own_next ? 1 + task++ % (WWARPS - 1) : task++ % WWARPS;
                if (w != warp) continue;
                if (jb > k) block_update(A + slot_of(ib, jb) * BLK, PLk + (ib / WP) * WB * WB, PCk + (jb / WQ) * BLK, false, lane);
                else block_update(W + slot_of(ib, jb) * BLK, PLk + (ib / WP) * WB * WB, PWk + (jb / WQ) * BLK, true, lane);
            }
        }
        if (own_next && warp == 0) {
            __syncwarp();
            if (!factor_warp(A + slot_of(k + 1, k + 1) * BLK, lane) && lane == 0) bad_sh = 1;
        }
        proxy_fence();  // this CTA's reads of the receive buffers precede later sends into them
        __syncthreads();
        if (k >= 1) cluster_wait();  // every CTA has finished step k - 1
        if (own_next && warp == 0) send_dk(k + 1);
        cluster_arrive();  // this CTA has finished step k
    }
    if (NB > 0) cluster_wait();  // every CTA has finished the last step: no copy is in flight

    // ---- solves with W and FP64 refinement ----
    double *vy = (double *)(sm + OFF_VEC), *vr = vy + NV, *vu = vr + NV, *vv = vu + NV;
    float *bf = sm + OFF_BF, *cf = sm + OFF_CF, *zp = sm + OFF_ZP, *zf = sm + OFF_ZF, *xp = sm + OFF_XP,
          *bp = sm + OFF_BP;
    double *dp = (double *)(sm + OFF_DP), *dpc = (double *)(sm + OFF_DPC), *rr = (double *)(sm + OFF_RR),
           *rc = (double *)(sm + OFF_RC);
    for (int g = tid; g < NV; g += WT) {
        vy[g] = g < n1 ? H[(size_t)g * ld + n1] : 0.0;
        vr[g] = g < n1 ? rhs[g] : 0.0;
    }
    __syncthreads();

    // (cf[0], cf[1]) = W^T W (bf[0], bf[1]) in FP32
    auto solve = [&]() {
        for (int ib = p; ib < NB; ib += WP)
            for (int jb = q; jb <= ib; jb += WQ) {
                const int s = slot_of(ib, jb);
                if (s % WWARPS != warp) continue;
                const float *w = W + s * BLK;
                float a0 = 0.f, a1 = 0.f;
                for (int c = 0; c < WB; ++c) {
                    const float wv = w[lane * LDB + c];
                    a0 = fmaf(wv, bf[jb * WB + c], a0);
                    a1 = fmaf(wv, bf[NV + jb * WB + c], a1);
                }
                bp[(s * 2) * WB + lane] = a0;
                bp[(s * 2 + 1) * WB + lane] = a1;
            }
        __syncthreads();
        if (tid < SR * 2 * WB) {
            const int a = tid / (2 * WB), h = (tid / WB) & 1, r = tid % WB, ib = p + a * WP;
            float z = 0.f;
            if (ib < NB)
                for (int jb = q; jb <= ib; jb += WQ) z += bp[(slot_of(ib, jb) * 2 + h) * WB + r];
            zp[(a * 2 + h) * WB + r] = z;
        }
        __syncthreads();
        cl.sync();
        if (tid < SR * 2 * WB) {
            float z = 0.f;
            for (int qq = 0; qq < WQ; ++qq) z += cl.map_shared_rank(zp, p * WQ + qq)[tid];
            zf[tid] = z;
        }
        __syncthreads();
        for (int ib = p; ib < NB; ib += WP)
            for (int jb = q; jb <= ib; jb += WQ) {
                const int s = slot_of(ib, jb);
                if (s % WWARPS != warp) continue;
                const float *w = W + s * BLK, *z0 = zf + ((ib / WP) * 2) * WB, *z1 = z0 + WB;
                float a0 = 0.f, a1 = 0.f;
                for (int r = 0; r < WB; ++r) {
                    const float wv = w[r * LDB + lane];
                    a0 = fmaf(wv, z0[r], a0);
                    a1 = fmaf(wv, z1[r], a1);
                }
                bp[(s * 2) * WB + lane] = a0;
                bp[(s * 2 + 1) * WB + lane] = a1;
            }
        __syncthreads();
        if (tid < SCOL * 2 * WB) {
            const int b = tid / (2 * WB), h = (tid / WB) & 1, c = tid % WB, jb = q + b * WQ;
            float xs = 0.f;
            if (jb < NB)
                for (int ib = p; ib < NB; ib += WP)
                    if (ib >= jb) xs += bp[(slot_of(ib, jb) * 2 + h) * WB + c];
            xp[(b * 2 + h) * WB + c] = xs;
        }
        __syncthreads();
        cl.sync();
        for (int e = tid; e < 2 * NV; e += WT) {
            const int h = e / NV, g = e % NV, jb = g / WB, c = g % WB;
            float xs = 0.f;
            if (jb < NB)
                for (int pp = 0; pp < WP; ++pp)
                    xs += cl.map_shared_rank(xp, pp * WQ + jb % WQ)[((jb / WQ) * 2 + h) * WB + c];
            cf[h * NV + g] = xs;
        }
        __syncthreads();
    };

    // (y, r) - H (u, v) in FP64, rounded to FP32 into bf for the next solve
    auto residual = [&]() {
        for (int ib = p; ib < NB; ib += WP)
            for (int jb = q; jb <= ib; jb += WQ) {
                const int s = slot_of(ib, jb);
                if (s % WWARPS != warp) continue;
                // H is read in halves of 16 entries per lane, all loads of a
                // half in flight before its FMAs (in increasing index order)
                const int gi = ib * WB + lane;
                double a0 = 0.0, a1 = 0.0;
#pragma unroll
                for (int h0 = 0; h0 < WB; h0 += 16) {
                    double hv[16];
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        const int gj = jb * WB + h0 + c;
                        hv[c] = (gi < n1 && gj < n1) ? (gi >= gj ? H[(size_t)gj * ld + gi] : H[(size_t)gi * ld + gj])
                                                     : 0.0;
                    }
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        a0 = fma(hv[c], vu[jb * WB + h0 + c], a0);
                        a1 = fma(hv[c], vv[jb * WB + h0 + c], a1);
                    }
                }
                dp[(s * 2) * WB + lane] = a0;
                dp[(s * 2 + 1) * WB + lane] = a1;
                if (ib > jb) {
                    const int gj = jb * WB + lane;
                    double c0 = 0.0, c1 = 0.0;
#pragma unroll
                    for (int h0 = 0; h0 < WB; h0 += 16) {
                        double hv[16];
#pragma unroll
                        for (int r = 0; r < 16; ++r) {
                            const int gr = ib * WB + h0 + r;
                            hv[r] = (gr < n1 && gj < n1) ? H[(size_t)gj * ld + gr] : 0.0;
                        }
#pragma unroll
                        for (int r = 0; r < 16; ++r) {
                            c0 = fma(hv[r], vu[ib * WB + h0 + r], c0);
                            c1 = fma(hv[r], vv[ib * WB + h0 + r], c1);
                        }
                    }
                    dpc[(s * 2) * WB + lane] = c0;
                    dpc[(s * 2 + 1) * WB + lane] = c1;
                }
            }
        __syncthreads();
        if (tid < SR * 2 * WB) {
            const int a = tid / (2 * WB), h = (tid / WB) & 1, r = tid % WB, ib = p + a * WP;
            double t = 0.0;
            if (ib < NB)
                for (int jb = q; jb <= ib; jb += WQ) t += dp[(slot_of(ib, jb) * 2 + h) * WB + r];
            rr[(a * 2 + h) * WB + r] = t;
        } else if (tid < SR * 2 * WB + SCOL * 2 * WB) {
            const int u = tid - SR * 2 * WB;
            const int b = u / (2 * WB), h = (u / WB) & 1, c = u % WB, jb = q + b * WQ;
            double t = 0.0;
            if (jb < NB)
                for (int ib = p; ib < NB; ib += WP)
                    if (ib > jb) t += dpc[(slot_of(ib, jb) * 2 + h) * WB + c];
            rc[(b * 2 + h) * WB + c] = t;
        }
        __syncthreads();
        cl.sync();
        // the next solve reads the residual of this CTA's column blocks only
        const int ncq = q < NB ? (NB - 1 - q) / WQ + 1 : 0;
        for (int e = tid; e < 2 * ncq * WB; e += WT) {
            const int h = e / (ncq * WB), u = e % (ncq * WB), ib = q + (u / WB) * WQ, r = u % WB;
            const int g = ib * WB + r;
            double t = 0.0;
            for (int qq = 0; qq < WQ; ++qq)
                t += cl.map_shared_rank(rr, (ib % WP) * WQ + qq)[((ib / WP) * 2 + h) * WB + r];
            for (int pp = 0; pp < WP; ++pp)
                t += cl.map_shared_rank(rc, pp * WQ + q)[((ib / WQ) * 2 + h) * WB + r];
            bf[h * NV + g] = __double2float_rn((h ? vr : vy)[g] - t);
        }
        __syncthreads();
    };

    // max |v| over the first n1 entries of an FP32 vector (every CTA alike;
    // FP32 because every FP64 operation repeated by 512 threads costs about
    // 0.2 us on this part's FP64 pipe)
    auto maxabs_f = [&](const float *v) {
        float m = 0.f;
        for (int g = tid; g < n1; g += WT) m = fmaxf(m, fabsf(v[g]));
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        __syncthreads();
        if (lane == 0) redf[warp] = m;
        __syncthreads();
        float t = 0.f;
        for (int w = 0; w < WWARPS; ++w) t = fmaxf(t, redf[w]);
        return t;
    };

    for (int g = tid; g < NV; g += WT) {
        bf[g] = __double2float_rn(vy[g]);
        bf[NV + g] = __double2float_rn(vr[g]);
    }
    __syncthreads();
    solve();
    for (int g = tid; g < NV; g += WT) {
        vu[g] = (double)cf[g];
        vv[g] = (double)cf[NV + g];
    }
    // the first solve's sizes stand for |u| and |v| in the stop test
    const float nu = maxabs_f(cf), nv = maxabs_f(cf + NV);
    float last_u = nu, last_v = nv;
    bool converged = false;
    for (int it = 0; it < MAXIT && !converged; ++it) {
        residual();
        solve();
        for (int g = tid; g < NV; g += WT) {
            vu[g] += (double)cf[g];
            vv[g] += (double)cf[NV + g];
        }
        // the correction just applied, and the next one it predicts
        // (|c_k|^2 / |c_{k-1}| for a linearly converging iteration)
        const float cu = maxabs_f(cf), cv = maxabs_f(cf + NV);
        if (tid == 0) {
            const double tol = 0x1p-40;
            const bool ok_u = cu == 0.f || (cu <= 0.5f * last_u && (double)cu * cu <= tol * nu * last_u);
            const bool ok_v = cv == 0.f || (cv <= 0.5f * last_v && (double)cv * cv <= tol * nv * last_v);
            flag_sh = ok_u && ok_v;
        }
        __syncthreads();
        converged = flag_sh != 0;
        last_u = cu;
        last_v = cv;
        __syncthreads();
    }

    // ---- the bordered system's solution, and the status ----
    if (me == 0) {
        // s = y.u and y.v by warp 0: lane sums over a stride, then a fixed
        // shuffle tree
        if (warp == 0) {
            double s = 0.0, yv = 0.0;
            for (int g = lane; g < n1; g += 32) {
                s = fma(vy[g], vu[g], s);
                yv = fma(vy[g], vv[g], yv);
            }
            for (int o = 16; o > 0; o >>= 1) {
                s += __shfl_xor_sync(0xffffffffu, s, o);
                yv += __shfl_xor_sync(0xffffffffu, yv, o);
            }
            if (lane == 0) xn_sh = (rhs[n1] - yv) / (s * s);
        }
        __syncthreads();
        const double xn = xn_sh;
        for (int g = tid; g < n1; g += WT) x[g] = fma(-vu[g], xn, vv[g]);
        if (tid == 0) x[n1] = xn;
    }
    cl.sync();  // every remote read of this CTA's shared memory is done
    if (me == 0 && tid == 0) {
        int bad = 0;
        for (int r = 0; r < WC; ++r) bad |= *cl.map_shared_rank(&bad_sh, r);
        flags[2] = bad ? 1 : (converged ? 0 : 2);
    }
    cl.sync();
}

// Whether a 16-CTA cluster of this kernel can be resident on the current
// device (checked once per device).
bool cluster_ok() {
    constexpr int kDevices = 64;
    static std::atomic<int> state[kDevices];  // 0 unknown, 1 no, 2 yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) {
        cudaGetLastError();
        return false;
    }
    int s = state[dev].load(std::memory_order_acquire);
    if (s == 0) {
        bool ok = cudaFuncSetAttribute(ws_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) ==
                      cudaSuccess &&
                  cudaFuncSetAttribute(ws_mixed_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
        if (ok) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = WC;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(WC);
            cfg.blockDim = dim3(WT);
            cfg.dynamicSmemBytes = SMEM_BYTES;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nc = 0;
            ok = cudaOccupancyMaxActiveClusters(&nc, ws_mixed_kernel, &cfg) == cudaSuccess && nc >= 1;
        }
        cudaGetLastError();
        s = ok ? 2 : 1;
        state[dev].store(s, std::memory_order_release);
    }
    return s == 2;
}

}  // namespace

// Largest working set the cluster solve takes (0 when the device cannot run
// the cluster).
extern "C" int irwls_ws_mixed_max(void) { return cluster_ok() ? WNB * WB : 0; }

// The bordered working-set system of full IRWLS in the precision form: H's
// lower triangle (n1 x n1, column-major, leading dimension ld), the border
// y in row n1 of the same array, right-hand side rhs (n1 + 1 values); the
// solution goes to x (n1 + 1 values). Returns 0 when solved, 1 when the FP32
// factor or the refinement failed (x is then not written with a valid
// solution and the caller solves in FP64), a negative code on a launch error.
// Synchronizes the stream to read the outcome.
extern "C" int irwls_ws_solve_mixed(const double *d_H, int n1, int ld, const double *d_rhs, double *d_x) {
    if (n1 < 1 || n1 > WNB * WB || ld < n1 + 1 || !cluster_ok()) return 1;
    int *flags = irwls_dev_flags();
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = WC;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(WC);
    cfg.blockDim = dim3(WT);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.stream = irwls_stream();
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_CHOL);
    cudaError_t e = cudaLaunchKernelEx(&cfg, ws_mixed_kernel, d_H, n1, ld, d_rhs, d_x, flags);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_CHOL);
    if (e != cudaSuccess) {
        irwls_set_error(-2, "working-set cluster solve launch: %s", cudaGetErrorString(e));
        return -2;
    }
    IRWLS_LAUNCH_CHECK("ws_mixed");
    int st = -1;
    e = cudaMemcpyAsync(&st, flags + 2, sizeof(int), cudaMemcpyDeviceToHost, irwls_stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(irwls_stream());
    if (e != cudaSuccess) {
        irwls_set_error(-2, "working-set cluster solve: %s", cudaGetErrorString(e));
        return -2;
    }
    return st == 0 ? 0 : 1;
}
