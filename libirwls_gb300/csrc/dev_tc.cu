// dev_tc.cu -- split-BF16 GEMM on the 5th-generation tensor cores (tcgen05,
// sm_103a) for the precision form of the solvers.
//
//   C (M x N) = A (M x K) . B (N x K)^T,   A = Ahi + Alo, B = Bhi + Blo (bf16)
//   C ~= Ahi.Bhi + Ahi.Blo + Alo.Bhi      accumulated in FP32 in tensor memory
//
// An FP32 value x is split as hi = bf16(x), lo = bf16(x - hi): the pair
// carries 16 significant bits, and the dropped lo.lo product is 2^-16 of the
// product, so each term of the dot product has a relative error of about
// 1.5e-5; the accumulation itself is FP32.
//
// Operands are K-major (each row's K values contiguous) bf16 arrays in global
// memory with leading dimension ld (a multiple of 8 elements) and K padded
// with zeros to a multiple of 64. A CTA of 128 threads computes a 128 x BN
// tile (BN = 64 or 128): every K stage of 64 is copied with cp.async into the
// canonical K-major no-swizzle shared layout (8-row x 16-byte core matrices;
// LBO = 128 B between K-neighbouring core matrices, SBO = 1024 B between row
// groups), then thread 0 issues 4 x 3 tcgen05.mma (K = 16 each) and commits
// them to the stage's mbarrier. Two stages are in flight. The accumulator is
// a 128-lane x BN-column FP32 block of tensor memory; warp w reads lanes
// 32w..32w+31 with tcgen05.ld.
//
// Every mbarrier wait is bounded: if it runs out, the kernel records the
// failure in the device flag word 1, skips the rest of its work, and still
// releases its tensor memory.
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "blocked_bf16.cuh"
#include "dev_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TC_BM = 128, TC_BK = 64;
constexpr int TC_THREADS = 128;
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) { return tc_desc_lbo_sbo(saddr, 128, 1024); }

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void *gmem, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(gmem), "r"(src_bytes));
}

// Shared memory of one K stage: the P pieces of A (128 rows) then the P
// pieces of B (BN rows). P = 2 (hi, lo): three products; P = 3 (hi, mid,
// lo): six products (all terms down to 2^-24 of the product).
template <int BN, int P = 2>
struct TcStage {
    static constexpr int A_BYTES = TC_BM * TC_BK * 2;
    static constexpr int B_BYTES = BN * TC_BK * 2;
    static constexpr int BYTES = P * A_BYTES + P * B_BYTES;
};

// Copies K stage `ks` of the CTA's rows into stage buffer `sb` (cp.async).
// A[p] / B[p]: the P pieces of each operand.
template <int BN, int P = 2>
__device__ __forceinline__ void tc_load_stage_p(unsigned char *sb, const __nv_bfloat16 *const *A, int lda, int m0,
                                                int M, const __nv_bfloat16 *const *B, int ldb, int n0, int N, int ks) {
    using S = TcStage<BN, P>;
    const int k0 = ks * TC_BK;
    const uint32_t base = smem_u32(sb);
    for (int t = threadIdx.x; t < P * TC_BM * 8; t += TC_THREADS) {
        const int which = t / (TC_BM * 8), rem = t % (TC_BM * 8);
        const int r = rem / 8, c = rem % 8;
        const int gr = m0 + r;
        const __nv_bfloat16 *src = A[which] + (size_t)(gr < M ? gr : 0) * lda + k0 + c * 8;
        const uint32_t dst = base + which * S::A_BYTES + (r / 8) * 1024 + c * 128 + (r % 8) * 16;
        cp_async16(dst, src, gr < M ? 16 : 0);
    }
    for (int t = threadIdx.x; t < P * BN * 8; t += TC_THREADS) {
        const int which = t / (BN * 8), rem = t % (BN * 8);
        const int r = rem / 8, c = rem % 8;
        const int gr = n0 + r;
        const __nv_bfloat16 *src = B[which] + (size_t)(gr < N ? gr : 0) * ldb + k0 + c * 8;
        const uint32_t dst = base + P * S::A_BYTES + which * S::B_BYTES + (r / 8) * 1024 + c * 128 + (r % 8) * 16;
        cp_async16(dst, src, gr < N ? 16 : 0);
    }
    asm volatile("cp.async.commit_group;\n" ::);
}

template <int BN>
__device__ __forceinline__ void tc_load_stage(unsigned char *sb, const __nv_bfloat16 *Ahi, const __nv_bfloat16 *Alo,
                                              int lda, int m0, int M, const __nv_bfloat16 *Bhi,
                                              const __nv_bfloat16 *Blo, int ldb, int n0, int N, int ks) {
    const __nv_bfloat16 *A[2] = {Ahi, Alo}, *B[2] = {Bhi, Blo};
    tc_load_stage_p<BN, 2>(sb, A, lda, m0, M, B, ldb, n0, N, ks);
}

// Issues the MMAs of one K stage (thread 0 only): per 16-wide K step, the
// products of piece pairs (i, j) with i + j < P (3 for P = 2, 6 for P = 3).
template <int BN, int P = 2>
__device__ __forceinline__ void tc_mma_stage(unsigned char *sb, uint32_t tmem, bool first) {
    using S = TcStage<BN, P>;
    const uint32_t base = smem_u32(sb);
    constexpr uint32_t idesc = tc_idesc(TC_BM, BN);
#pragma unroll
    for (int kk = 0; kk < TC_BK / 16; ++kk) {
        const uint32_t off = kk * 256;  // 16 elements = 2 core matrices along K
        bool init = first && kk == 0;
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P - i; ++j) {
                const uint32_t a = base + i * S::A_BYTES + off, b = base + P * S::A_BYTES + j * S::B_BYTES + off;
                mma_bf16(tmem, tc_desc(a), tc_desc(b), idesc, init ? 0u : 1u);
                init = false;
            }
    }
}

// The main loop shared by the kernels below: accumulates the CTA's
// 128 x BN tile over K stages [ks0, ks1) into tensor memory. Returns false if
// a wait ran out. Stage i commits to mbar[i & 1]; `used` holds how many
// phases each barrier has completed before this call (0 for fresh barriers)
// and is advanced by the call, which waits for every commit it made, so a
// kernel can run the loop again on the same barriers and tensor memory.
template <int BN, int P>
__device__ bool tc_mainloop_p(unsigned char *smem, uint64_t *mbar, uint32_t tmem, const __nv_bfloat16 *const *A,
                              int lda, int m0, int M, const __nv_bfloat16 *const *B, int ldb, int n0, int N, int ks0,
                              int ks1, uint32_t *used) {
    constexpr int SB = TcStage<BN, P>::BYTES;
    const int nst = ks1 - ks0;
    bool ok = true;
    if (nst <= 0) return true;
    const uint32_t u0 = used ? used[0] : 0u, u1 = used ? used[1] : 0u;
    auto parity = [&](int stage) { return ((stage & 1 ? u1 : u0) + (uint32_t)(stage >> 1)) & 1u; };
    tc_load_stage_p<BN, P>(smem, A, lda, m0, M, B, ldb, n0, N, ks0);
    for (int i = 0; i < nst; ++i) {
        const int buf = i & 1;
        if (i + 1 < nst) {
            // the other buffer was last read by the MMAs of stage i - 1
            if (i >= 1 && !mbar_wait(smem_u32(&mbar[buf ^ 1]), parity(i - 1))) ok = false;
            tc_load_stage_p<BN, P>(smem + (buf ^ 1) * SB, A, lda, m0, M, B, ldb, n0, N, ks0 + i + 1);
            asm volatile("cp.async.wait_group 1;\n" ::);
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::);
        ok = __syncthreads_and(ok);  // CTA-uniform: every thread takes the same branch below
        if (!ok) break;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            tc_mma_stage<BN, P>(smem + buf * SB, tmem, i == 0);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&mbar[buf])));
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    // the last stage's commit covers all earlier MMAs; the one before it is
    // waited for too, so that both barriers end with every phase observed
    const int last = nst - 1;
    if (ok && !mbar_wait(smem_u32(&mbar[last & 1]), parity(last))) ok = false;
    if (ok && nst >= 2 && !mbar_wait(smem_u32(&mbar[(last - 1) & 1]), parity(last - 1))) ok = false;
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (used) {
        used[0] = u0 + (uint32_t)((nst + 1) / 2);
        used[1] = u1 + (uint32_t)(nst / 2);
    }
    return ok;
}

template <int BN>
__device__ bool tc_mainloop(unsigned char *smem, uint64_t *mbar, uint32_t tmem, const __nv_bfloat16 *Ahi,
                            const __nv_bfloat16 *Alo, int lda, int m0, int M, const __nv_bfloat16 *Bhi,
                            const __nv_bfloat16 *Blo, int ldb, int n0, int N, int ks0, int ks1,
                            uint32_t *used = nullptr) {
    const __nv_bfloat16 *A[2] = {Ahi, Alo}, *B[2] = {Bhi, Blo};
    return tc_mainloop_p<BN, 2>(smem, mbar, tmem, A, lda, m0, M, B, ldb, n0, N, ks0, ks1, used);
}

// ---- ring pipeline: NS stages of BK K-elements ------------------------------
//
// Stage layout as above with BK / 8 core matrices per row group: LBO = 128 B
// (next K core matrix), SBO = BK / 8 * 128 B (next 8-row group). Loads for
// stage i + NS - 1 are issued while the MMAs of stage i run, so NS - 1 stages
// of copies are in flight; a buffer is refilled only after the mbarrier of
// the MMAs that last read it has completed.
template <int BN, int P, int BK>
struct TcRing {
    static constexpr int A_BYTES = TC_BM * BK * 2;
    static constexpr int B_BYTES = BN * BK * 2;
    static constexpr int BYTES = P * A_BYTES + P * B_BYTES;
    static constexpr int SBO = BK / 8 * 128;
};

template <int BN, int P, int BK>
__device__ __forceinline__ void ring_load(unsigned char *sb, const __nv_bfloat16 *const *A, int lda, int m0, int M,
                                          const __nv_bfloat16 *const *B, int ldb, int n0, int N, int k0) {
    using S = TcRing<BN, P, BK>;
    constexpr int CH = BK / 8;  // 16-byte chunks per row
    const uint32_t base = smem_u32(sb);
    for (int t = threadIdx.x; t < P * TC_BM * CH; t += TC_THREADS) {
        const int which = t / (TC_BM * CH), rem = t % (TC_BM * CH);
        const int r = rem / CH, c = rem % CH;
        const int gr = m0 + r;
        const __nv_bfloat16 *src = A[which] + (size_t)(gr < M ? gr : 0) * lda + k0 + c * 8;
        cp_async16(base + which * S::A_BYTES + (r / 8) * S::SBO + c * 128 + (r % 8) * 16, src, gr < M ? 16 : 0);
    }
    for (int t = threadIdx.x; t < P * BN * CH; t += TC_THREADS) {
        const int which = t / (BN * CH), rem = t % (BN * CH);
        const int r = rem / CH, c = rem % CH;
        const int gr = n0 + r;
        const __nv_bfloat16 *src = B[which] + (size_t)(gr < N ? gr : 0) * ldb + k0 + c * 8;
        cp_async16(base + P * S::A_BYTES + which * S::B_BYTES + (r / 8) * S::SBO + c * 128 + (r % 8) * 16, src,
                   gr < N ? 16 : 0);
    }
}

template <int BN, int P, int BK>
__device__ __forceinline__ void ring_mma(unsigned char *sb, uint32_t tmem, bool first) {
    using S = TcRing<BN, P, BK>;
    const uint32_t base = smem_u32(sb);
    constexpr uint32_t idesc = tc_idesc(TC_BM, BN);
    bool init = first;
#pragma unroll
    for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t off = kk * 256;
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P - i; ++j) {
                const uint32_t a = base + i * S::A_BYTES + off, b = base + P * S::A_BYTES + j * S::B_BYTES + off;
                mma_bf16(tmem, tc_desc_sbo(a, S::SBO), tc_desc_sbo(b, S::SBO), idesc, init ? 0u : 1u);
                init = false;
            }
    }
}

// Accumulates the CTA's 128 x BN tile over K stages [ks0, ks1) (of BK
// elements) into tensor memory through an NS-stage ring. mbar: NS barriers;
// used[NS]: phases each has completed before the call, advanced by it. Every
// commit is waited for before returning. Returns false if a wait ran out.
template <int BN, int P, int BK, int NS>
__device__ bool tc_mainloop_ring(unsigned char *smem, uint64_t *mbar, uint32_t tmem, const __nv_bfloat16 *const *A,
                                 int lda, int m0, int M, const __nv_bfloat16 *const *B, int ldb, int n0, int N,
                                 int ks0, int ks1, uint32_t *used) {
    constexpr int SB = TcRing<BN, P, BK>::BYTES;
    const int nst = ks1 - ks0;
    if (nst <= 0) return true;
    auto parity = [&](int st) { return (used[st % NS] + (uint32_t)(st / NS)) & 1u; };
    bool ok = true;
    for (int i = 0; i < NS - 1; ++i) {
        if (i < nst) ring_load<BN, P, BK>(smem + i * SB, A, lda, m0, M, B, ldb, n0, N, (ks0 + i) * BK);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    for (int i = 0; i < nst; ++i) {
        const int j = i + NS - 1;  // the stage whose copies start now, into the buffer stage i - 1 used
        if (j < nst) {
            if (i >= 1 && !mbar_wait(smem_u32(&mbar[(i - 1) % NS]), parity(i - 1))) ok = false;
            ring_load<BN, P, BK>(smem + (j % NS) * SB, A, lda, m0, M, B, ldb, n0, N, (ks0 + j) * BK);
        }
        asm volatile("cp.async.commit_group;\n" ::);
        asm volatile("cp.async.wait_group %0;\n" ::"n"(NS - 1));  // stage i has landed
        asm volatile("fence.proxy.async.shared::cta;\n" ::);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            ring_mma<BN, P, BK>(smem + (i % NS) * SB, tmem, i == 0);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&mbar[i % NS])));
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    // the commits not yet waited for: the last NS stages at most
    for (int st = (nst > NS ? nst - NS : 0); st < nst && ok; ++st)
        if (!mbar_wait(smem_u32(&mbar[st % NS]), parity(st))) ok = false;
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    for (int b = 0; b < NS; ++b) used[b] += (uint32_t)((nst > b ? (nst - b + NS - 1) / NS : 0));
    return ok;
}

template <int NS>
__device__ __forceinline__ void ring_barriers_init(uint64_t *mbar) {
    if (threadIdx.x == 0) {
        for (int b = 0; b < NS; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[b])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
}

template <int BN>
__device__ __forceinline__ void tc_setup(uint64_t *mbar, uint32_t *tmem_slot) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
}

template <int BN, int NS>
__device__ __forceinline__ void tc_setup_ring(uint64_t *mbar, uint32_t *tmem_slot) {
    ring_barriers_init<NS>(mbar);
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
}

template <int BN>
__device__ __forceinline__ void tc_teardown(uint32_t tmem) {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

// Reads 8 accumulator columns of this thread's row (lane 32w + laneid).
__device__ __forceinline__ void tc_ld8(uint32_t tmem, int c0, float *v) {
    const int w = threadIdx.x >> 5;
    uint32_t r[8];
    const uint32_t addr = tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)c0;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// C tiles to global memory (FP32). grid: (ceil(N / BN), ceil(M / 128), splits);
// split z accumulates K stages [z*per, (z+1)*per) into C + z * zstride.
template <int BN>
__global__ void __launch_bounds__(TC_THREADS) tc_gemm_store_kernel(const __nv_bfloat16 *Ahi, const __nv_bfloat16 *Alo,
                                                                   int lda, int M, const __nv_bfloat16 *Bhi,
                                                                   const __nv_bfloat16 *Blo, int ldb, int N, int kst,
                                                                   int per, float *C, int ldc, long long zstride,
                                                                   int lower_only, int *flags) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    const int n0 = blockIdx.x * BN, m0 = blockIdx.y * TC_BM, z = blockIdx.z;
    if (lower_only && n0 >= m0 + TC_BM) return;  // whole tile above the diagonal
    // align the dynamic buffer to 1024 bytes
    unsigned char *smem = tc_smem + ((1024 - (smem_u32(tc_smem) & 1023)) & 1023);
    tc_setup<BN>(mbar, &tmem_slot);
    const uint32_t tmem = tmem_slot;
    const int ks0 = z * per, ks1 = min(kst, ks0 + per);
    const bool ok = tc_mainloop<BN>(smem, mbar, tmem, Ahi, Alo, lda, m0, M, Bhi, Blo, ldb, n0, N, ks0, ks1);
    if (!ok && threadIdx.x == 0) atomicExch(flags + 1, 1);
    const int row = m0 + threadIdx.x;
    float *out = C + z * zstride;
    if (ok) {
        for (int c0 = 0; c0 < BN; c0 += 8) {
            float v[8];
            if (ks1 > ks0) tc_ld8(tmem, c0, v);
            else
                for (int j = 0; j < 8; ++j) v[j] = 0.f;
            if (row < M)
                for (int j = 0; j < 8; ++j)
                    if (n0 + c0 + j < N) out[(size_t)row * ldc + n0 + c0 + j] = v[j];
        }
    }
    tc_teardown<BN>(tmem);
}

// hi/lo split of an FP32 (or FP64) matrix into two bf16 matrices.
template <class T>
__global__ void split_bf16_kernel(const T *__restrict__ X, long long rows, int cols, int ldx, __nv_bfloat16 *hi,
                                  __nv_bfloat16 *lo, int ldo) {
    const long long total = rows * (long long)ldo;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long r = t / ldo;
        const int c = (int)(t % ldo);
        const float x = (c < cols) ? (float)X[r * ldx + c] : 0.f;
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        hi[t] = h;
        lo[t] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

}  // namespace

extern "C" size_t irwls_tc_smem_bytes(int bn) {
    return (bn == 64 ? 2 * TcStage<64>::BYTES : 2 * TcStage<128>::BYTES) + 1024;
}

// C (M x N, FP32, row-major ldc) = A B^T from split operands; `splits` K
// partitions write to C + z * zstride. K must be a multiple of 64 (zero pad).
extern "C" int irwls_tc_gemm(const void *Ahi, const void *Alo, int lda, int M, const void *Bhi, const void *Blo,
                             int ldb, int N, int K, float *C, int ldc, int splits, long long zstride,
                             int lower_only, int bn) {
    if (K % TC_BK || lda % 8 || ldb % 8) {
        irwls_set_error(-12, "tensor-core GEMM needs K %% 64 == 0 and leading dimensions %% 8 == 0");
        return -12;
    }
    const int kst = K / TC_BK;
    if (splits < 1) splits = 1;
    const int per = (kst + splits - 1) / splits;
    int *flags = irwls_dev_flags();
    const size_t smem = irwls_tc_smem_bytes(bn);
    if (bn == 64) {
        cudaFuncSetAttribute(tc_gemm_store_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dim3 grid(ceil_div(N, 64), ceil_div(M, TC_BM), splits);
        tc_gemm_store_kernel<64><<<grid, TC_THREADS, smem, irwls_stream()>>>(
            (const __nv_bfloat16 *)Ahi, (const __nv_bfloat16 *)Alo, lda, M, (const __nv_bfloat16 *)Bhi,
            (const __nv_bfloat16 *)Blo, ldb, N, kst, per, C, ldc, zstride, lower_only, flags);
    } else {
        cudaFuncSetAttribute(tc_gemm_store_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dim3 grid(ceil_div(N, 128), ceil_div(M, TC_BM), splits);
        tc_gemm_store_kernel<128><<<grid, TC_THREADS, smem, irwls_stream()>>>(
            (const __nv_bfloat16 *)Ahi, (const __nv_bfloat16 *)Alo, lda, M, (const __nv_bfloat16 *)Bhi,
            (const __nv_bfloat16 *)Blo, ldb, N, kst, per, C, ldc, zstride, lower_only, flags);
    }
    IRWLS_LAUNCH_CHECK("tc_gemm");
    return 0;
}

extern "C" int irwls_split_bf16_f64(const double *X, long long rows, int cols, int ldx, void *hi, void *lo, int ldo) {
    const long long total = rows * (long long)ldo;
    const int blocks = (int)((total + 255) / 256 < 65535 ? (total + 255) / 256 : 65535);
    split_bf16_kernel<double><<<blocks, 256, 0, irwls_stream()>>>(X, rows, cols, ldx, (__nv_bfloat16 *)hi,
                                                                  (__nv_bfloat16 *)lo, ldo);
    IRWLS_LAUNCH_CHECK("split_bf16");
    return 0;
}

extern "C" int irwls_split_bf16_f32(const float *X, long long rows, int cols, int ldx, void *hi, void *lo, int ldo) {
    const long long total = rows * (long long)ldo;
    const int blocks = (int)((total + 255) / 256 < 65535 ? (total + 255) / 256 : 65535);
    split_bf16_kernel<float><<<blocks, 256, 0, irwls_stream()>>>(X, rows, cols, ldx, (__nv_bfloat16 *)hi,
                                                                 (__nv_bfloat16 *)lo, ldo);
    IRWLS_LAUNCH_CHECK("split_bf16");
    return 0;
}

// Reads (and clears) the tensor-core wait-failure flag: 0, or the nonzero
// code the failing kernel left (which wait of which CTA ran out).
extern "C" int irwls_tc_status(void) {
    int flags[8];
    cudaMemcpyAsync(flags, irwls_dev_flags(), sizeof flags, cudaMemcpyDeviceToHost, irwls_stream());
    cudaStreamSynchronize(irwls_stream());
    if (flags[1]) {
        int zero = 0;
        cudaMemcpyAsync(irwls_dev_flags() + 1, &zero, sizeof zero, cudaMemcpyHostToDevice, irwls_stream());
        cudaStreamSynchronize(irwls_stream());
        return flags[1];
    }
    return 0;
}

// ===========================================================================
// Precision form of SGMA.
//
// SGMA works on Q = K_nm L^-T (row i = the Nystrom features of sample i, all
// of norm <= 1) instead of K_nm: for a candidate c with w = L^-1 k_C(c),
// K_nm z = Q w, eta = 1 - |w|^2, and the residual is r = Q w - k(c, .). Q and
// w are bounded, which is what makes a product of bf16 pieces accurate here
// (the reference's K_nm z form multiplies K_nm by z = K_CC^-1 k_C, whose
// entries are large and cancel). Q is kept as three bf16 pieces per value
// (exactly its FP32 value), and the tensor cores take the six piece products
// down to 2^-24 of each term, so Q w has the accuracy of an FP32 dot
// product. A new centroid c_s adds the column
//   q_s = (k(., c_s) - Q l2) / L3,  l2 = L^-1 k_C(c_s) = w(c_s), L3 the pivot,
// which is minus the step's residual of the winning candidate over L3: the
// score kernel stores the 64 residuals of every row, and the column is read
// from them instead of from another pass over Q.
// ===========================================================================

namespace {

// FP32 mirror of a device set (dense rows, CSR values, norms), made once per
// precision-form run so that no kernel of that form converts from FP64 per
// entry: conversions and adds in FP64 run on this part's narrow FP64 pipe.
struct KViewF {
    int mode, width, ld;
    float ng;
    const float *__restrict__ X;
    const int *__restrict__ rp;
    const int *__restrict__ ci;
    const float *__restrict__ cv;
    const float *__restrict__ q;
};

struct F32Mirror {
    float *X, *cv, *q;
};

static inline KViewF kviewf(const irwls_dev_set *s, const F32Mirror *f) {
    KViewF v;
    v.mode = s->mode;
    v.width = s->width;
    v.ld = s->ld;
    v.ng = (float)s->neg_gamma;
    v.X = f->X;
    v.rp = s->rp;
    v.ci = s->ci;
    v.cv = f->cv;
    v.q = f->q;
    return v;
}

__global__ void to_f32_kernel(const double *__restrict__ in, long long n, float *__restrict__ out) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = __double2float_rn(in[t]);
}

// Candidate rows of the score kernel in shared memory, feature-major: the 64
// candidates' values of feature k at cat + k * CAT_LD, candidates contiguous
// (so one float4 load gives four candidates). The stride is 68 floats: 16-byte
// loads of lanes whose rows hold different features fall in different bank
// groups for features that differ mod 8.
constexpr int CAT_LD = 68;

// Scores of the precision form: per candidate, the tile sums in 16 strided
// groups with Kahan-compensated FP32 adds, the 16 group sums in FP64 in a
// fixed order, score = sum / eta; strict ">" argmax, first index wins.
__global__ void __launch_bounds__(1024) sgma_select_f32_kernel(const float *__restrict__ part, int nblk,
                                                              const double *__restrict__ eta,
                                                              const int *__restrict__ cand, int s, int *cent,
                                                              int *best, double *bestval, float *scores) {
    chain_wait();
    chain_open();
    __shared__ double grp[16][64];
    __shared__ double sc[64];
    const int c = threadIdx.x & 63, g = threadIdx.x >> 6;
    float sum = 0.f, comp = 0.f;
    for (int b = g; b < nblk; b += 16) {
        const float y = __fsub_rn(part[(size_t)b * 64 + c], comp);
        const float t = __fadd_rn(sum, y);
        comp = __fsub_rn(__fsub_rn(t, sum), y);
        sum = t;
    }
    grp[g][c] = (double)sum - (double)comp;
    __syncthreads();
    if (threadIdx.x < 64) {
        double v = 0.0;
        for (int k = 0; k < 16; ++k) v += grp[k][threadIdx.x];
        const double et = eta[threadIdx.x];
        sc[threadIdx.x] = (et > 0.0) ? v / et : 0.0;
        if (scores) scores[threadIdx.x] = (float)sc[threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double val = sc[0];
        int bb = 0;
        for (int i = 1; i < 64; ++i)
            if (sc[i] > val) {
                val = sc[i];
                bb = i;
            }
        cent[s] = cand[bb];
        best[0] = bb;
        bestval[s] = val;
    }
}

// ---- persistent warp-specialized score kernel --------------------------------
//
// One CTA per SM walks row tiles t = blockIdx.x, + gridDim.x, ...: warp 0
// streams the Q and W stages of every tile through an NS-deep ring
// (cp.async, each lane signalling the stage's "full" barrier when its copies
// land), lane 0 of warp 1 issues the MMAs into one of two tensor-memory
// accumulators and commits the ring stages ("empty") and the finished tile
// ("acc full"), and warps 4-11 run the epilogue of a tile while the next one
// accumulates in the other accumulator: warp w reads tensor-memory lanes
// 32 (w % 4) ... + 31 (its rows), warps 4-7 for candidates 0-31 and warps
// 8-11 for candidates 32-63. The candidate rows are loaded once per CTA.
// Every wait is bounded; on a timeout the flag word 1 is set and every role
// leaves its loop (the epilogue warps decide together at their named
// barrier), the MMA thread waits for its last commit and the producer for
// its copies before the tensor memory is released.
constexpr int WS_BK = 32;
// Epilogue groups: 2 (8 epilogue warps, 384 threads). Four groups (640
// threads, 96 registers) were measured at 200000 rows: 4 % faster at order
// 32, 3 % slower at orders 512-992, slower over a whole training -- the
// epilogue is bound by shared-memory traffic (staged rows and candidate
// gathers), which more warps do not reduce.
constexpr int WS_EG = 2;

__device__ __forceinline__ void cp_async4(uint32_t saddr, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(gmem));
}

// Row data of one 128-row tile staged in shared memory for the score
// epilogue, so that a lane's kernel entries read its row from there instead
// of walking it in global memory load after load. kind 1: the tile's CSR
// slice (column indices, values; rows are consecutive, so the slice is
// contiguous) with tile-relative row pointers; kind 2: the raw rows at an odd
// stride (conflict-free row-per-lane reads); kind 0: too large for the
// buffer, entries read from global memory.
struct TileRows {
    int kind, lds;
    const int *rp;
    const float *q;
    const int *ci;
    const float *cv;
    const float *x;
};

// Issues the staging copies of rows m0 ... m0 + nr - 1 (threads et = 0 ... 255
// of the epilogue); the caller waits for them (cp.async.wait_all + barrier).
__device__ __forceinline__ TileRows stage_tile_rows(const KViewF &X, int m0, int nr, unsigned char *buf, int buf_bytes,
                                                    int *srp, float *sq, int et, int nthr) {
    TileRows t;
    t.kind = 0;
    t.lds = 0;
    t.rp = srp;
    t.q = sq;
    if (X.mode == IRWLS_K_RAW_RBF) {
        const int lds = X.width | 1;
        float *x = (float *)buf;
        t.x = x;
        t.lds = lds;
        if (nr * lds * 4 <= buf_bytes) {
            t.kind = 2;
            const int n = nr * X.width;
            for (int k = et; k < n; k += nthr) {
                const int r = k / X.width, c = k - r * X.width;
                cp_async4(smem_u32(x + r * lds + c), X.X + (size_t)(m0 + r) * X.ld + c);
            }
        }
        return t;
    }
    const int p0 = X.rp[m0], p1 = X.rp[m0 + nr];
    const int nnz = p1 - p0;
    int *ci = (int *)buf;
    float *cv = (float *)(buf + (buf_bytes / 8) * 4);
    t.ci = ci;
    t.cv = cv;
    for (int k = et; k <= nr; k += nthr) srp[k] = X.rp[m0 + k] - p0;
    if (X.mode == IRWLS_K_NORM_RBF)
        for (int k = et; k < nr; k += nthr) sq[k] = X.q[m0 + k];
    if (nnz <= buf_bytes / 8) {
        t.kind = 1;
        for (int k = et; k < nnz; k += nthr) {
            cp_async4(smem_u32(ci + k), X.ci + p0 + k);
            cp_async4(smem_u32(cv + k), X.cv + p0 + k);
        }
    }
    return t;
}

// Kernel values of tile row r (global row jb) against 32 candidates, the
// candidates' values of feature k at a[k * CAT_LD + j]. The row is read once
// (from the staged tile rows, or from global memory when they were too large
// to stage) and every entry updates the 32 sums; per candidate the FMAs run
// in the row's entry order from 0, so the values do not depend on the
// staging.
__device__ __forceinline__ void kentry32_tile(const KViewF &B, const TileRows &T, const float *a, const float *qa,
                                              int r, int jb, float out[32]) {
    float acc[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j] = 0.f;
    if (B.mode == IRWLS_K_RAW_RBF) {
        const float *b = T.kind == 2 ? T.x + r * T.lds : B.X + (size_t)jb * B.ld;
        for (int t = 0; t < B.width; ++t) {
            const float bt = b[t];
            const float4 *ap = (const float4 *)(a + t * CAT_LD);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 av = ap[q];
                float d;
                d = av.x - bt;
                acc[4 * q] = fmaf(d, d, acc[4 * q]);
                d = av.y - bt;
                acc[4 * q + 1] = fmaf(d, d, acc[4 * q + 1]);
                d = av.z - bt;
                acc[4 * q + 2] = fmaf(d, d, acc[4 * q + 2]);
                d = av.w - bt;
                acc[4 * q + 3] = fmaf(d, d, acc[4 * q + 3]);
            }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) out[j] = __expf(B.ng * acc[j]);
        return;
    }
    const int *ci;
    const float *cv;
    int p0, p1;
    float qb;
    if (T.kind == 1) {
        ci = T.ci;
        cv = T.cv;
        p0 = T.rp[r];
        p1 = T.rp[r + 1];
        qb = B.mode == IRWLS_K_NORM_RBF ? T.q[r] : 0.f;
    } else {
        ci = B.ci;
        cv = B.cv;
        p0 = B.rp[jb];
        p1 = B.rp[jb + 1];
        qb = B.mode == IRWLS_K_NORM_RBF ? B.q[jb] : 0.f;
    }
    for (int p = p0; p < p1; ++p) {
        const float v = cv[p];
        const float4 *ap = (const float4 *)(a + ci[p] * CAT_LD);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 av = ap[q];
            acc[4 * q] = fmaf(v, av.x, acc[4 * q]);
            acc[4 * q + 1] = fmaf(v, av.y, acc[4 * q + 1]);
            acc[4 * q + 2] = fmaf(v, av.z, acc[4 * q + 2]);
            acc[4 * q + 3] = fmaf(v, av.w, acc[4 * q + 3]);
        }
    }
    if (B.mode == IRWLS_K_LINEAR) {
#pragma unroll
        for (int j = 0; j < 32; ++j) out[j] = acc[j];
        return;
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) out[j] = __expf(B.ng * fmaxf(qa[j] + qb - 2.f * acc[j], 0.f));
}

// Sums over the warp's 32 lanes of 32 values per lane (v[j] of every lane for
// j = 0 ... 31); on return lane j holds the sum for j in v[0]. At each step
// a lane keeps half of its values and passes the other half to the lane that
// differs in one index bit, so every sum is the tree that pairs lanes
// differing in bit 4, then bit 3, ..., bit 0 (31 shuffles instead of 160 for
// 32 separate butterflies). The adds are rounded explicitly.
__device__ __forceinline__ void warp_sum32_transposed(float v[32], int lane) {
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool up = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const float keep = up ? v[i + h] : v[i];
            const float send = up ? v[i] : v[i + h];
            v[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, h));
        }
    }
}

// Tensor-memory columns of one score accumulator: three 64-column sums
// S0 = sum Qhi Whi, S1 = sum (Qhi Wmid + Qmid Whi), S2 = sum (Qhi Wlo + Qmid
// Wmid + Qlo Whi), so that the small terms are not rounded against the large
// ones; Q w = S0 + (S1 + S2).
constexpr int SC_COLS = 192;

// The MMAs of one score stage (one thread): per 16-wide K step, Qhi against
// the W pieces hi, mid, lo stacked along N (N = 192, into S0 S1 S2), Qmid
// against hi, mid (N = 128, into S1 S2) and Qlo against hi (N = 64, into S2):
// three MMAs for the six products, each A piece read once.
__device__ __forceinline__ void score_mma_stage(unsigned char *sb, uint32_t tmem, bool first) {
    using S = TcRing<64, QB_NP, WS_BK>;
    const uint32_t base = smem_u32(sb), wbase = base + QB_NP * S::A_BYTES;
#pragma unroll
    for (int kk = 0; kk < WS_BK / 16; ++kk) {
        const uint32_t off = kk * 256;
        const uint64_t w = tc_desc_sbo(wbase + off, S::SBO);
#pragma unroll
        for (int i = 0; i < QB_NP; ++i) {
            const uint32_t idesc = tc_idesc(TC_BM, 64 * (QB_NP - i));
            mma_bf16(tmem + 64 * i, tc_desc_sbo(base + i * S::A_BYTES + off, S::SBO), w, idesc,
                     first && kk == 0 && i == 0 ? 0u : 1u);
        }
    }
}

// EG epilogue groups of four warps (warps 4 ... 4 EG + 3), each scoring 64 / EG
// of the candidates for all 128 rows of a tile.
template <int NS, int EG>
__global__ void __launch_bounds__(128 + 128 * EG, 1) sgma_tc_score_ws_kernel(
    KViewF X, int l, const int *__restrict__ cand, const __nv_bfloat16 *__restrict__ Qb, int kbn,
    const __nv_bfloat16 *__restrict__ Wb, int kst, float *__restrict__ part, float *__restrict__ resid, int xs_bytes,
    int *flags) {
    chain_wait();
    chain_open();
    using S = TcRing<64, QB_NP, WS_BK>;
    static_assert(S::A_BYTES == 2 * QB_PIECE && S::B_BYTES == 2 * WB_PIECE, "blocked pieces are stage images");
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full[NS], empty[NS], accf[2], acce[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ float qc[64];
    constexpr int EPI = 128 * EG, CPG = 64 / EG;  // epilogue threads, candidates per group
    static_assert(CPG == 32, "an epilogue warp scores 32 candidates");
    __shared__ float wred[4 * EG][CPG];
    __shared__ volatile int abort_flag;
    unsigned char *smem = tc_smem + ((1024 - (smem_u32(tc_smem) & 1023)) & 1023);
    float *cat = (float *)(smem + NS * S::BYTES);  // candidate rows, feature-major (CAT_LD)
    // two buffers of xs_bytes: the rows of the tile being scored and of the next
    unsigned char *xs = (unsigned char *)(cat + CAT_LD * X.ld);
    __shared__ int srp[2][TC_BM + 1];
    __shared__ float sq[2][TC_BM];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (l + TC_BM - 1) / TC_BM;
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        for (int b = 0; b < NS; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], 4 * EG);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
        abort_flag = 0;
    }
    for (int t = threadIdx.x; t < 64 * X.ld; t += blockDim.x) {
        const int c = t & 63, k = t >> 6;
        cat[k * CAT_LD + c] = X.X[(size_t)cand[c] * X.ld + k];
    }
    if (threadIdx.x < 64) qc[threadIdx.x] = X.q[cand[threadIdx.x]];
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
        // producer: one thread, two bulk copies per stage (the blocked Q and
        // W hold each stage's shared-memory image contiguously)
        if (lane == 0) {
            const uint32_t base = smem_u32(smem);
            int issued = 0;
            for (int j = 0; j < my_tiles && !abort_flag; ++j) {
                const size_t tile = (size_t)blockIdx.x + (size_t)j * gridDim.x;
                for (int k = 0; k < kst; ++k) {
                    const int u = j * kst + k, slot = u % NS;
                    if (u >= NS && !mbar_wait(smem_u32(&empty[slot]), (uint32_t)(u / NS - 1) & 1u)) abort_flag = 1;
                    if (abort_flag) break;
                    const uint32_t sb = base + slot * S::BYTES, fb = smem_u32(&full[slot]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb),
                                 "r"((uint32_t)S::BYTES));
                    bulk_g2s(sb, Qb + (tile * kbn + k) * (QB_NP * QB_PIECE), QB_NP * S::A_BYTES, fb);
                    bulk_g2s(sb + QB_NP * S::A_BYTES, Wb + (size_t)k * (QB_NP * WB_PIECE), QB_NP * S::B_BYTES, fb);
                    issued = u + 1;
                }
            }
            // no copy is left in flight: the last NS stages issued have landed
            for (int u = issued > NS ? issued - NS : 0; u < issued; ++u)
                if (!mbar_wait(smem_u32(&full[u % NS]), (uint32_t)(u / NS) & 1u)) abort_flag = 1;
        }
        __syncwarp();
    } else if (warp == 1) {
        // MMA issue
        if (lane == 0) {
            for (int j = 0; j < my_tiles && !abort_flag; ++j) {
                const int b = j & 1;
                if (j >= 2 && !mbar_wait(smem_u32(&acce[b]), (uint32_t)(j / 2 - 1) & 1u)) abort_flag = 1;
                for (int k = 0; k < kst && !abort_flag; ++k) {
                    const int u = j * kst + k, slot = u % NS;
                    if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(u / NS) & 1u)) {
                        abort_flag = 1;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;\n" ::);
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                    score_mma_stage(smem + slot * S::BYTES, tmem + b * SC_COLS, k == 0);
                    tc_commit(&empty[slot]);
                }
                if (!abort_flag) tc_commit(&accf[b]);
            }
            // every MMA issued has completed before the tensor memory is released
            tc_commit(&done);
            if (!mbar_wait(smem_u32(&done), 0u)) abort_flag = 1;
        }
        __syncwarp();
    } else if (warp >= 4) {
        // epilogue: rows 32 (warp % 4) + lane of each tile, candidates
        // 32 g ... 32 g + 31 of epilogue group g
        const int ew = warp & 3, g = (warp - 4) >> 2;
        const int et = threadIdx.x - 128;
        // the rows of tile j + 1 are copied in while tile j is scored
        auto stage = [&](int jt) {
            const int m0 = ((int)blockIdx.x + jt * (int)gridDim.x) * TC_BM;
            return stage_tile_rows(X, m0, min(TC_BM, l - m0), xs + (jt & 1) * xs_bytes, xs_bytes, srp[jt & 1],
                                   sq[jt & 1], et, EPI);
        };
        TileRows T = {};
        if (my_tiles > 0) T = stage(0);
        for (int j = 0; j < my_tiles; ++j) {
            const int b = j & 1, tile = (int)blockIdx.x + j * (int)gridDim.x;
            const int m0 = tile * TC_BM, r = 32 * ew + lane, row = m0 + r;
            const bool acc_ok = mbar_wait(smem_u32(&accf[b]), (uint32_t)(j / 2) & 1u);
            asm volatile("cp.async.wait_all;\n" ::);
            // one decision for all epilogue threads (an OR over them), so
            // that none is left at a named barrier that the others skip; the
            // barrier also publishes the staged rows
            const int bad = (!acc_ok || abort_flag) ? 1 : 0;
            int any;
            asm volatile(
                "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.or.pred q, 1, %2, p;\nselp.s32 %0, 1, 0, q;\n}\n"
                : "=r"(any)
                : "r"(bad), "r"(EPI));
            if (any) {
                abort_flag = 1;
                break;
            }
            // the other buffer was last read by tile j - 1, which every epilogue
            // thread finished before the barriers that closed it
            const TileRows Tn = j + 1 < my_tiles ? stage(j + 1) : T;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            {
                // this row's kernel values against the group's 32 candidates
                float v[32], acc[32];
                if (row < l) kentry32_tile(X, T, cat + CPG * g, qc + CPG * g, r, row, v);
                // Q w: the three accumulators (terms of order 1, 2^-8 and
                // 2^-16) added smallest first, eight candidates at a time
                const uint32_t tb = tmem + b * SC_COLS;
#pragma unroll
                for (int c8 = 0; c8 < 32; c8 += 8) {
                    float s1[8], s2[8];
                    tc_ld8_lanes(tb + 128, 32 * ew, CPG * g + c8, s2);
                    tc_ld8_lanes(tb + 64, 32 * ew, CPG * g + c8, s1);
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj) s2[jj] = __fadd_rn(s1[jj], s2[jj]);
                    tc_ld8_lanes(tb, 32 * ew, CPG * g + c8, s1);
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj) acc[c8 + jj] = __fadd_rn(s1[jj], s2[jj]);
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
                if (lane == 0) mbar_arrive(&acce[b]);  // this warp's reads of accumulator b are done
                // residuals r = Q w - k, then r^2 per candidate summed over the
                // warp's 32 rows
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) acc[jj] = __fsub_rn(acc[jj], v[jj]);
                if (row < l) {
                    // the residuals, from which the winner's column of Q is
                    // taken, candidate-major (a warp's stores are 128-byte lines)
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) resid[(size_t)(CPG * g + jj) * l + row] = acc[jj];
                }
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) v[jj] = row < l ? __fmul_rn(acc[jj], acc[jj]) : 0.f;
                warp_sum32_transposed(v, lane);
                wred[4 * g + ew][lane] = v[0];
            }
            asm volatile("bar.sync 1, %0;\n" ::"r"(EPI));
            if (et < 64) {
                // the candidate's four row-quarter sums, in a fixed order
                const float *w = &wred[4 * (et / CPG)][et % CPG];
                part[(size_t)tile * 64 + et] = (w[0] + w[CPG]) + (w[2 * CPG] + w[3 * CPG]);
            }
            asm volatile("bar.sync 1, %0;\n" ::"r"(EPI));
            T = Tn;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    // after the barrier: every role has finished, so a timeout any of them
    // met is in abort_flag
    if (threadIdx.x == 0 && abort_flag) atomicExch(flags + 1, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512));
}

// Q's column s written as its three pieces, and |Q_i|^2 updated.
__device__ __forceinline__ void put_q(int row, int s, float q, __nv_bfloat16 *Qb, int ldq, float *qn) {
    if (qn) qn[row] = fmaf(q, q, qn[row]);  // |Q_i|^2: the Nystrom residual of row i is k_ii - qn[i]
    __nv_bfloat16 pc[3];
    bf16_pieces3(q, pc);
#pragma unroll
    for (int k = 0; k < QB_NP; ++k) Qb[qb_index(row, s, ldq >> 5, k)] = pc[k];
}

// Column s of Q from the score step's residuals r = Q w - k of the winning
// candidate (slot best[0]; the residuals of candidate c at resid + c * l):
// q_i = -r_i / L3. lrow[s] holds 1 / L3.
__global__ void q_column_resid_kernel(int l, const float *__restrict__ resid, const int *__restrict__ best, int s,
                                      const float *__restrict__ lrow, __nv_bfloat16 *Qb, int ldq,
                                      float *__restrict__ qn) {
    chain_wait();
    chain_open();
    const int c = best[0];
    const float inv_l3 = lrow[s];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l; i += gridDim.x * blockDim.x)
        put_q(i, s, -resid[(size_t)c * l + i] * inv_l3, Qb, ldq, qn);
}

// Column s of Q directly, q_i = (k(x_i, c_s) - sum_{t<s} Q_it l2_t) / L3,
// one row per thread (Q from its pieces). Used for the first columns (the
// class-mean centroids), which no score step precedes. lrow holds l2 (s
// floats) then 1 / L3.
__global__ void __launch_bounds__(256) q_column_direct_kernel(KViewF X, int l, const int *__restrict__ cent, int s,
                                                              const float *__restrict__ lrow, __nv_bfloat16 *Qb,
                                                              int ldq, float *__restrict__ qn) {
    extern __shared__ float qsm[];
    float *sc = qsm;  // centroid row, X.ld floats
    const int gc = cent[s];
    for (int t = threadIdx.x; t < X.ld; t += blockDim.x) sc[t] = X.X[(size_t)gc * X.ld + t];
    __syncthreads();
    const float inv_l3 = lrow[s];
    const float qa = X.q[gc];
    const int kbn = ldq >> 5;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l; i += gridDim.x * blockDim.x) {
        float dot = 0.f;
        for (int t = 0; t < s; ++t)
            dot = fmaf(bf16_join3(Qb[qb_index(i, t, kbn, 0)], Qb[qb_index(i, t, kbn, 1)], Qb[qb_index(i, t, kbn, 2)]),
                       lrow[t], dot);
        float kd = 0.f, kv;
        if (X.mode == IRWLS_K_RAW_RBF) {
            const float *b = X.X + (size_t)i * X.ld;
            for (int t = 0; t < X.width; ++t) {
                const float d = sc[t] - b[t];
                kd = fmaf(d, d, kd);
            }
            kv = __expf(X.ng * kd);
        } else {
            for (int p = X.rp[i]; p < X.rp[i + 1]; ++p) kd = fmaf(X.cv[p], sc[X.ci[p]], kd);
            kv = X.mode == IRWLS_K_LINEAR ? kd : __expf(X.ng * fmaxf(qa + X.q[i] - 2.f * kd, 0.f));
        }
        put_q(i, s, (kv - dot) * inv_l3, Qb, ldq, qn);
    }
}

}  // namespace

extern "C" void *irwls_f32_mirror(const irwls_dev_set *X) {
    F32Mirror *f = (F32Mirror *)calloc(1, sizeof(F32Mirror));
    if (!f) return nullptr;
    const long long nx = (long long)X->n_rows * X->ld;
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&f->X, (size_t)(nx > 0 ? nx : 1) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&f->cv, (size_t)(X->nnz > 0 ? X->nnz : 1) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&f->q, (size_t)(X->n_rows > 0 ? X->n_rows : 1) * sizeof(float));
    if (!rc) {
        const int g = 4 * (irwls_num_sms() > 0 ? irwls_num_sms() : 148);
        const double *src[3] = {X->X, X->cv, X->q};
        float *dst[3] = {f->X, f->cv, f->q};
        const long long cnt[3] = {nx, X->nnz, X->n_rows};
        for (int k = 0; k < 3; ++k)
            if (cnt[k] > 0) {
                to_f32_kernel<<<g, 256, 0, irwls_stream()>>>(src[k], cnt[k], dst[k]);
                irwls_count_launch(1);
            }
        if (cudaPeekAtLastError() != cudaSuccess) rc = -1;
    }
    if (rc) {
        irwls_dev_free(f->X);
        irwls_dev_free(f->cv);
        irwls_dev_free(f->q);
        free(f);
        irwls_set_error(-3, "cannot create the FP32 copy of the dataset");
        return nullptr;
    }
    return f;
}

extern "C" void irwls_f32_mirror_view(const void *h, const float **X, const float **q) {
    const F32Mirror *f = (const F32Mirror *)h;
    *X = f->X;
    *q = f->q;
}

extern "C" void irwls_f32_mirror_free(void *h) {
    F32Mirror *f = (F32Mirror *)h;
    if (!f) return;
    irwls_dev_free(f->X);
    irwls_dev_free(f->cv);
    irwls_dev_free(f->q);
    free(f);
}

extern "C" int irwls_sgma_tc_score(const irwls_dev_set *X, const void *F, int l, const int *d_cand, const void *Qb,
                                   int ldq, const void *Wb, int s, float *d_part, float *d_resid) {
    constexpr size_t XS = 24 * 1024;  // largest row-staging buffer (one of two)
    const int kst = (s + WS_BK - 1) / WS_BK;
    if (kst * WS_BK > ldq || ldq % WS_BK) {
        irwls_set_error(-12, "Q leading dimension %d does not hold order %d in 32-column blocks", ldq, s);
        return -12;
    }
    // dynamic shared memory of a CTA: the device's opt-in limit less the
    // kernel's static shared memory (all instantiations have the same)
    static size_t limit = 0;
    if (!limit) {
        int dev = 0, optin = 0;
        cudaFuncAttributes fa;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, sgma_tc_score_ws_kernel<2, WS_EG>) != cudaSuccess) {
            cudaGetLastError();
            optin = 220 * 1024 + 4096;
            fa.sharedSizeBytes = 4096;
        }
        limit = (size_t)optin - fa.sharedSizeBytes;
    }
    const size_t fixed = 1024 + (size_t)CAT_LD * X->ld * sizeof(float);
    const size_t stage = TcRing<64, QB_NP, WS_BK>::BYTES;
    if (fixed + 2 * stage > limit) {
        irwls_set_error(-12, "feature width %d too wide for the precision-form SGMA tile", X->width);
        return -12;
    }
    // Row staging: what a typical tile needs (raw rows, or its CSR slice at the
    // set's mean row length plus a sixteenth; a tile above that reads its rows
    // from global memory), then as many ring stages as fit, then the rest of
    // the shared memory to the staging buffers (up to XS each).
    size_t need;
    if (X->mode == IRWLS_K_RAW_RBF) need = (size_t)TC_BM * (X->width | 1) * sizeof(float);
    else need = (size_t)(TC_BM * 8.0 * 1.0625 * (double)X->nnz / std::max(1, X->n_rows)) + 256;
    need = std::min((need + 127) / 128 * 128, XS);
    static const int kStages[] = {8, 6, 5, 4, 2};
    int ns = 2;
    size_t xs = 0;
    for (int c : kStages)
        if (fixed + 2 * need + (size_t)c * stage <= limit) {
            ns = c;
            xs = std::min(XS, (limit - fixed - (size_t)c * stage) / 2 / 128 * 128);
            break;
        }
    if (xs == 0)  // no staging: rows from global memory
        for (int c : kStages)
            if (fixed + (size_t)c * stage <= limit) {
                ns = c;
                break;
            }
    const size_t smem = fixed + 2 * xs + (size_t)ns * stage;
    const int ntiles = ceil_div(l, TC_BM);
    const int grid = std::max(1, std::min(ntiles, irwls_num_sms() > 0 ? irwls_num_sms() : 148));
    const KViewF kv = kviewf(X, (const F32Mirror *)F);
    const __nv_bfloat16 *qb = (const __nv_bfloat16 *)Qb, *wb = (const __nv_bfloat16 *)Wb;
    auto launch = [&](auto kern) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        launch_chained(kern, dim3(grid), dim3(128 + 128 * WS_EG), smem, kv, l, d_cand, qb, ldq / 32, wb, kst, d_part,
                       d_resid, (int)xs, irwls_dev_flags());
    };
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_SGMA_GEMM);
    switch (ns) {
        case 8: launch(sgma_tc_score_ws_kernel<8, WS_EG>); break;
        case 6: launch(sgma_tc_score_ws_kernel<6, WS_EG>); break;
        case 5: launch(sgma_tc_score_ws_kernel<5, WS_EG>); break;
        case 4: launch(sgma_tc_score_ws_kernel<4, WS_EG>); break;
        default: launch(sgma_tc_score_ws_kernel<2, WS_EG>); break;
    }
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_SGMA_GEMM);
    IRWLS_LAUNCH_CHECK("sgma_tc_score");
    return 0;
}

extern "C" int irwls_sgma_tc_partials(int l) { return ceil_div(l, TC_BM); }

extern "C" int irwls_sgma_tc_select(const float *d_part, int nblk, const double *d_eta, const int *d_cand, int s,
                                    int *d_cent, int *d_best, double *d_bestval, float *d_scores) {
    launch_chained(sgma_select_f32_kernel, dim3(1), dim3(1024), 0, d_part, nblk, d_eta, d_cand, s, d_cent, d_best,
                   d_bestval, d_scores);
    IRWLS_LAUNCH_CHECK("sgma_select_f32");
    return 0;
}

// lrow: row s of L in FP32 (s values, then 1 / L3), from irwls_sgma_linv_update.
// The direct form (the first columns, s small).
extern "C" int irwls_q_column(const irwls_dev_set *X, const void *F, int l, const int *d_cent, int s,
                              const float *lrow, void *Qb, int ldq, float *d_qn) {
    if (s >= ldq) {
        irwls_set_error(-12, "Q leading dimension %d below the order %d", ldq, s + 1);
        return -12;
    }
    const size_t smem = (size_t)X->ld * sizeof(float);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(q_column_direct_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int blocks = std::max(1, std::min(ceil_div(l, 256), 4 * (irwls_num_sms() > 0 ? irwls_num_sms() : 148)));
    q_column_direct_kernel<<<blocks, 256, smem, irwls_stream()>>>(kviewf(X, (const F32Mirror *)F), l, d_cent, s, lrow,
                                                                   (__nv_bfloat16 *)Qb, ldq, d_qn);
    IRWLS_LAUNCH_CHECK("q_column_direct");
    return 0;
}

// Column s from the residuals of the score step that chose centroid s.
extern "C" int irwls_q_column_resid(int l, const float *d_resid, const int *d_best, int s, const float *lrow, void *Qb,
                                    int ldq, float *d_qn) {
    if (s >= ldq) {
        irwls_set_error(-12, "Q leading dimension %d below the order %d", ldq, s + 1);
        return -12;
    }
    const int blocks = std::max(1, std::min(ceil_div(l, 256), 4 * (irwls_num_sms() > 0 ? irwls_num_sms() : 148)));
    launch_chained(q_column_resid_kernel, dim3(blocks), dim3(256), 0, l, d_resid, d_best, s, lrow, (__nv_bfloat16 *)Qb,
                   ldq, d_qn);
    IRWLS_LAUNCH_CHECK("q_column_resid");
    return 0;
}

// ===========================================================================
// Precision form of full IRWLS: the error update over every training row,
//   e_i <- (e_i - sum_j cb_j k(x_i, x_{b_j})) - tail,   j over the working set,
// with the kernel values from dot products on the tensor cores, then
// k = exp(-gamma (q_i + q_j - 2 x_i . x_j)) (RBF, the norm form) or x_i . x_j
// (linear). The update is incremental, so its per-entry error has to stay
// near FP32 rounding (a two-piece, 16-bit split moved errors across the
// classification threshold within a few updates). Two operand forms:
//  - P = 3 pieces: every value (rounded to FP32) is split into hi + mid + lo
//    bf16 (24 significant bits) and the six piece products down to 2^-24 of
//    the product are accumulated in FP32;
//  - P = 1 piece: when every value of the set is exactly a bf16 after a scale
//    S = 1 (binary data, small integers, values with <= 8 significant bits) or
//    S = 255 (8-bit data k / 255), the scaled values are the operands and
//    every product is exact; the dot product is multiplied by 1 / S^2.
// Both keep only the FP32 accumulation error.
//
// Layout: the dataset is copied once per training into a blocked array in
// which every (128-row tile, 32-column block) holds its P pieces as the
// shared-memory image of one tcgen05 operand stage (core matrices of 8 rows
// x 16 bytes, 128 bytes apart along K and 512 bytes apart along rows), and
// the working-set rows are gathered before each update into the same layout
// in 256-row chunks. A stage is then one bulk copy of the tile's block and P
// bulk copies of the chunk's rows.
//
// Kernel: persistent, one CTA per SM walking (tile, chunk) items; warp 0
// streams stages through an NS-deep ring, one thread of warp 1 issues the
// MMAs (M = 128 rows, N = the chunk's columns rounded to 16, K = 16) into
// one of two 256-column FP32 accumulators in tensor memory, and warps 4-11
// run the epilogue of the previous item: warp w reads lanes 32 (w % 4) ...
// (its rows), warps 4-7 the chunk's first 128 columns and warps 8-11 the
// rest, and each thread keeps a Kahan-compensated FP32 sum of its row over
// its columns in a fixed order; the two halves are added in FP64 at the end
// of the tile. Each A tile is read from memory once per 256 working-set
// columns. Every wait is bounded; on a timeout the device flag word 1 is
// set, every role leaves its loop, and no copy or MMA is in flight when the
// tensor memory is released.
// ===========================================================================

namespace {

constexpr int RS_BM = 128, RS_BN = 256, RS_BK = 32;
constexpr int RS_APIECE = RS_BM * RS_BK, RS_BPIECE = RS_BN * RS_BK;  // elements per piece of a stage
constexpr int RS_EPI = 256;                                          // epilogue threads (warps 4-11)
constexpr int RS_THREADS = 128 + RS_EPI;
constexpr long long RS_WAIT_DEFAULT = 1LL << 26;

// element offset of row r, column c (c < 32) inside one piece of a stage
__device__ __forceinline__ size_t rs_core(int r, int c) {
    return (size_t)(r >> 3) * 256 + (c >> 3) * 64 + (r & 7) * 8 + (c & 7);
}

template <int P>
struct RsStage {
    static constexpr int A_BYTES = P * RS_APIECE * 2;
    static constexpr int B_BYTES = P * RS_BPIECE * 2;
    static constexpr int BYTES = A_BYTES + B_BYTES;
};

template <int P>
constexpr int rs_stages() {
    return P == 1 ? 8 : 3;  // 192 KB and 216 KB of ring
}

__device__ __forceinline__ bool mbar_wait_lim(uint32_t mbar, uint32_t parity, long long limit) {
    uint32_t done = 0;
    for (long long it = 0; it < limit && !done; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity));
    }
    return done != 0;
}

// Operand-form check of a set's stored values (its CSR entries: zeros are
// exact in both forms). bad[0] |= some value is not exactly a bf16 (bit
// test: the low 45 mantissa bits zero, the exponent in bf16's normal range);
// bad[1] |= some value is not RN(k / 255) for an integer |k| <= 256. For the
// second, with k = rint(255 v), r = fma(v, 255, -k) = 255 v - k exactly (an
// integer multiple of ulp(v)), and v = RN(k / 255) exactly when
// |r| <= 127 ulp(v) (63 ulp when v is a power of two and k / 255 lies below
// it, where the binade below is finer); k / 255 is never halfway between two
// doubles unless it is an integer. A thread stops once both flags are set.
__global__ void rs_quant_check_kernel(const double *__restrict__ v, long long n, int *bad) {
    int b0 = 0, b1 = 0;
    const volatile int *vb = bad;
    long long it = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x, ++it) {
        if ((it & 63) == 0 && vb[0] && vb[1]) break;
        const double x = v[t];
        if (x == 0.0) continue;
        const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
        const int ex = (int)((bits >> 52) & 0x7ff);
        const unsigned long long man = bits & ((1ULL << 52) - 1);
        if ((man & ((1ULL << 45) - 1)) != 0 || ex < 1023 - 126 || ex > 1023 + 127) b0 = 1;
        const double k = rint(x * 255.0);
        if (!(fabs(k) <= 256.0) || ex < 64 || ex == 0x7ff) {
            b1 = 1;
            continue;
        }
        const double r = fma(x, 255.0, -k);
        const double ulp = __longlong_as_double((long long)((unsigned long long)(ex - 52) << 52));
        const double lim = (man == 0 && (r > 0.0) == (x > 0.0)) ? 63.0 : 127.0;
        if (fabs(r) > lim * ulp) b1 = 1;
    }
    b0 = __any_sync(0xffffffffu, b0);
    b1 = __any_sync(0xffffffffu, b1);
    if ((threadIdx.x & 31) == 0) {
        if (b0) atomicOr(bad, 1);
        if (b1) atomicOr(bad + 1, 1);
    }
}

// The blocked P-piece copy of rows x cols of a row-major FP64 matrix, scaled
// by `scale`; rows padded to tiles of 128 and columns to kbn blocks of 32
// with zeros. P = 3: hi, mid, lo of the FP32 value; P = 1: the value itself
// (exact by the check above).
template <int P>
__global__ void rs_split_kernel(const double *__restrict__ X, int rows, int cols, int ldx, int kbn, double scale,
                                __nv_bfloat16 *__restrict__ A) {
    const int ld = kbn * RS_BK;
    const long long total = (long long)((rows + RS_BM - 1) / RS_BM) * RS_BM * ld;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(t / ld), c = (int)(t % ld);
        const double v = (r < rows && c < cols) ? X[(size_t)r * ldx + c] * scale : 0.0;
        const size_t base = ((size_t)(r >> 7) * kbn + (c >> 5)) * P * RS_APIECE + rs_core(r & 127, c & 31);
        if (P == 1) {
            A[base] = __float2bfloat16_rn(__double2float_rn(v));
        } else {
            const float x = __double2float_rn(v);
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            const float r1 = x - __bfloat162float(h);
            const __nv_bfloat16 m = __float2bfloat16_rn(r1);
            A[base] = h;
            A[base + RS_APIECE] = m;
            A[base + 2 * RS_APIECE] = __float2bfloat16_rn(r1 - __bfloat162float(m));
        }
    }
}

// Working-set row j < *d_n becomes row j of the blocked B (256-row chunks):
// its 16-byte groups copied from the blocked A row idx[j]; qb[j] = q[idx[j]]
// and cbf[j] = (float)cb[j] (converted once here: FP64 conversions run on
// this part's narrow FP64 pipe, so the epilogue must not repeat them).
template <int P>
__global__ void rs_gather_kernel(const __nv_bfloat16 *__restrict__ A, int kbn, const float *__restrict__ q,
                                 const int *__restrict__ idx, const int *__restrict__ d_n, int nmax,
                                 __nv_bfloat16 *__restrict__ B, float *__restrict__ qb,
                                 const double *__restrict__ cb, float *__restrict__ cbf) {
    const int n = min(*d_n, nmax);
    const long long total = (long long)n * kbn * P * 4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(t & 3);
        long long rest = t >> 2;
        const int p = (int)(rest % P);
        rest /= P;
        const int k = (int)(rest % kbn);
        const int j = (int)(rest / kbn);
        const int i = idx[j];
        const size_t src = ((size_t)(i >> 7) * kbn + k) * P * RS_APIECE + (size_t)p * RS_APIECE + rs_core(i & 127, 8 * g);
        const size_t dst = ((size_t)(j >> 8) * kbn + k) * P * RS_BPIECE + (size_t)p * RS_BPIECE + rs_core(j & 255, 8 * g);
        *(uint4 *)(B + dst) = *(const uint4 *)(A + src);
        if (k == 0 && p == 0 && g == 0) {
            qb[j] = q[i];
            cbf[j] = __double2float_rn(cb[j]);
        }
    }
}

// MODE 0 (row sums): out_i = (init_i - sum_j cb_j k_ij) - tail[0].
// MODE 1 (prediction): out_i = bias + sum_j cb_j k_ij, or its sign (>= 0 ->
// +1) when `hard`.
template <int P, int NS, int MODE>
__global__ void __launch_bounds__(RS_THREADS, 1) tc_rowsum_ws_kernel(
    const __nv_bfloat16 *__restrict__ A, int M, int kbn, const float *__restrict__ qa,
    const __nv_bfloat16 *__restrict__ B, const int *__restrict__ d_n, int nmax, const float *__restrict__ qb,
    const float *__restrict__ cb, int rbf, float ng, float dscale, const double *init,
    const double *__restrict__ tail, double *out, double bias, int hard, int *flags, long long wait_limit,
    int stall) {
    using S = RsStage<P>;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full[NS], empty[NS], accf[2], acce[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ float2 half_sum[RS_BM];
    unsigned char *smem = tc_smem + ((1024 - (smem_u32(tc_smem) & 1023)) & 1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = max(0, min(*d_n, nmax));
    const int nch = (N + RS_BN - 1) / RS_BN;
    const int ntiles = (M + RS_BM - 1) / RS_BM;
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int items = my_tiles * nch;
    if (threadIdx.x == 0) {
        for (int b = 0; b < NS; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], RS_EPI / 32);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(2 * RS_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = tmem_slot;
    // columns of chunk h, rounded up to the MMA's N granularity
    auto chunk_rows = [&](int h) { return ((min(RS_BN, N - h * RS_BN) + 15) / 16) * 16; };

    if (warp == 0) {
        if (lane == 0) {
            const uint32_t base = smem_u32(smem);
            int u = 0;
            for (int it = 0; it < items && !abort_flag; ++it) {
                const int j = it / nch, h = it % nch;
                const size_t tile = (size_t)blockIdx.x + (size_t)j * gridDim.x;
                const uint32_t bbytes = (uint32_t)chunk_rows(h) * 64u;
                for (int k = 0; k < kbn; ++k, ++u) {
                    const int slot = u % NS;
                    if (u >= NS && !mbar_wait_lim(smem_u32(&empty[slot]), (uint32_t)(u / NS - 1) & 1u, wait_limit))
                        abort_flag = 1;
                    if (abort_flag) break;
                    const uint32_t sb = base + slot * S::BYTES, fb = smem_u32(&full[slot]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb),
                                 "r"((uint32_t)S::A_BYTES + P * bbytes));
                    bulk_g2s(sb, A + (tile * kbn + k) * P * RS_APIECE, S::A_BYTES, fb);
                    for (int p = 0; p < P; ++p)
                        bulk_g2s(sb + S::A_BYTES + p * RS_BPIECE * 2,
                                 B + (((size_t)h * kbn + k) * P + p) * RS_BPIECE, bbytes, fb);
                }
            }
            // no copy is left in flight: the last NS stages issued have landed
            for (int v = u > NS ? u - NS : 0; v < u; ++v)
                if (!mbar_wait_lim(smem_u32(&full[v % NS]), (uint32_t)(v / NS) & 1u, wait_limit)) abort_flag = 1;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            int u = 0;
            bool issued = false;  // tcgen05.commit only follows issued MMAs
            for (int it = 0; it < items && !abort_flag; ++it) {
                const int b = it & 1, h = it % nch;
                if (it >= 2 && !mbar_wait_lim(smem_u32(&acce[b]), (uint32_t)(it / 2 - 1) & 1u, wait_limit)) {
                    abort_flag = 1;
                    break;
                }
                const uint32_t idesc = tc_idesc(RS_BM, chunk_rows(h));
                for (int k = 0; k < kbn; ++k, ++u) {
                    const int slot = u % NS;
                    if (!mbar_wait_lim(smem_u32(&full[slot]), (uint32_t)(u / NS) & 1u, wait_limit)) {
                        abort_flag = 1;
                        break;
                    }
                    if (stall) {
                        // test mode: no MMA is issued and the accumulator is
                        // never completed, so the epilogue's wait runs out
                        mbar_arrive(&empty[slot]);
                        continue;
                    }
                    asm volatile("fence.proxy.async.shared::cta;\n" ::);
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                    const uint32_t sa = smem_u32(smem + slot * S::BYTES), sbb = sa + S::A_BYTES;
                    bool first = k == 0;
#pragma unroll
                    for (int kk = 0; kk < RS_BK / 16; ++kk)
#pragma unroll
                        for (int pi = 0; pi < P; ++pi)
#pragma unroll
                            for (int pj = 0; pj < P - pi; ++pj) {
                                mma_bf16(tmem + b * RS_BN, tc_desc_sbo(sa + pi * RS_APIECE * 2 + kk * 256, 512),
                                         tc_desc_sbo(sbb + pj * RS_BPIECE * 2 + kk * 256, 512), idesc, first ? 0u : 1u);
                                first = false;
                            }
                    tc_commit(&empty[slot]);
                    issued = true;
                }
                if (!abort_flag && !stall) tc_commit(&accf[b]);
            }
            // every MMA issued has completed before the tensor memory is released
            if (issued) tc_commit(&done);
            else mbar_arrive(&done);
            if (!mbar_wait_lim(smem_u32(&done), 0u, wait_limit)) abort_flag = 1;
        }
        __syncwarp();
    } else if (warp >= 4) {
        const int ew = warp & 3, g = (warp - 4) >> 2, r = 32 * ew + lane;
        int it = 0;
        bool aborted = false;
        for (int j = 0; j < my_tiles && !aborted; ++j) {
            const int row = ((int)blockIdx.x + j * (int)gridDim.x) * RS_BM + r;
            const float qi = row < M ? qa[row] : 0.f;
            float sum = 0.f, comp = 0.f;
            for (int h = 0; h < nch; ++h, ++it) {
                const int b = it & 1;
                const bool acc_ok = mbar_wait_lim(smem_u32(&accf[b]), (uint32_t)(it / 2) & 1u, wait_limit);
                // one decision for all epilogue threads (an OR over them)
                const int bad = (!acc_ok || abort_flag) ? 1 : 0;
                int any;
                asm volatile(
                    "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.or.pred q, 1, %2, p;\nselp.s32 %0, 1, 0, q;\n}\n"
                    : "=r"(any)
                    : "r"(bad), "r"(RS_EPI));
                if (any) {
                    abort_flag = 1;
                    aborted = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
                const int c_base = h * RS_BN + 128 * g;
                const int ncol = min(128, N - c_base);
                for (int c0 = 0; c0 < ncol; c0 += 32) {
                    float v[32];
                    tc_ld32_lanes(tmem + b * RS_BN + 128 * g, 32 * ew, c0, v);
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) {
                        const int c = c0 + jj;
                        if (c < ncol) {
                            const float dot = v[jj] * dscale;
                            const float k =
                                rbf ? expf(ng * fmaxf(qi + __ldg(qb + c_base + c) - 2.f * dot, 0.f)) : dot;
                            const float y = __fsub_rn(__fmul_rn(__ldg(cb + c_base + c), k), comp);
                            const float t = __fadd_rn(sum, y);
                            comp = __fsub_rn(__fsub_rn(t, sum), y);
                            sum = t;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
                if (lane == 0) mbar_arrive(&acce[b]);  // this warp's reads of accumulator b are done
            }
            if (aborted) break;
            // the two column halves of the row, added in FP64 in a fixed order
            if (g == 1) half_sum[r] = make_float2(sum, comp);
            asm volatile("bar.sync 2, %0;\n" ::"r"(RS_EPI));
            if (g == 0 && row < M) {
                const float2 o = half_sum[r];
                const double tot = ((double)sum - (double)comp) + ((double)o.x - (double)o.y);
                if (MODE == 0) {
                    out[row] = __dsub_rn(__dsub_rn(init[row], tot), tail ? tail[0] : 0.0);
                } else {
                    const double f = __dadd_rn(bias, tot);
                    out[row] = hard ? (f >= 0.0 ? 1.0 : -1.0) : f;
                }
            }
            asm volatile("bar.sync 2, %0;\n" ::"r"(RS_EPI));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    // after the barrier: every role has finished, so a timeout any of them
    // met is in abort_flag
    if (threadIdx.x == 0 && abort_flag) atomicExch(flags + 1, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * RS_BN));
}

struct TcSet {
    __nv_bfloat16 *A, *B;
    float *q, *qb, *cbf;
    int *bad;   // two words: the operand-form check, then the gathered-row count of a prediction
    int *nbuf;
    int rows, kbn, wmax, rbf, pieces;
    float ng, dscale;
    double kbound;
    // exact-integer mode (irwls_tc_exact_rowsum): whether it applies, the
    // operand scale, and its grow-only buffers (gathered rows, partial sums)
    int exact;
    double scale;
    __nv_bfloat16 *Ag;
    long long ag_cap;
    double *part;
    long long part_cap;
};

// max over rows of q (one CTA): |x_i . x_j| <= max q bounds linear kernel values.
__global__ void __launch_bounds__(1024) max_q_kernel(const float *__restrict__ q, int n, float *out) {
    __shared__ float red[1024];
    float m = 0.f;
    for (int i = threadIdx.x; i < n; i += 1024) m = fmaxf(m, q[i]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = 512; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

long long g_rs_wait_limit = RS_WAIT_DEFAULT;
int g_rs_stall = 0;
int g_rs_last_pieces = 0;

}  // namespace

// Test hook of the bounded waits of the full-IRWLS error update (no
// counterpart in the reference): the poll limit of every wait (<= 0: the
// default 2^26) and a stall switch with which the MMA thread issues nothing
// and never completes an accumulator, so that the epilogue's wait runs out
// with no copy or MMA in flight.
extern "C" void irwls_debug_tc_wait(long long limit, int stall) {
    g_rs_wait_limit = limit > 0 ? limit : RS_WAIT_DEFAULT;
    g_rs_stall = stall ? 1 : 0;
}
// Operand pieces of the last precision-form full-IRWLS set (1 or 3).
extern "C" int irwls_last_tc_pieces(void) { return g_rs_last_pieces; }

namespace {
// Operand-form flags of rows 0..rows-1 of a set: bad[0] (not every value is
// a bf16), bad[1] (not every value is k / 255 with |k| <= 256).
int rs_check(const irwls_dev_set *X, int rows, int *d_bad, int bad[2]) {
    bad[0] = bad[1] = 0;
    if (rows <= 0) return 0;
    int rc = irwls_dev_memset(d_bad, 0, 2 * sizeof(int));
    // the stored values of rows 0..rows-1: the first rp[rows] CSR entries
    int nnz = 0;
    rc |= irwls_dev_d2h(&nnz, X->rp + rows, sizeof(int));
    rc |= irwls_dev_sync();
    if (rc) return rc;
    const long long total = nnz;
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 8LL * sms));
    rs_quant_check_kernel<<<blocks, 256, 0, irwls_stream()>>>(X->cv, total, d_bad);
    irwls_count_launch(1);
    rc |= irwls_dev_d2h(bad, d_bad, 2 * sizeof(int));
    rc |= irwls_dev_sync();
    return rc;
}

// The operand form for flags of one or two sets: 1 piece with scale 1 or
// 255 when every value qualifies, else 3 pieces with scale 1.
void rs_form(const int *bad, int n, int *pieces, double *scale) {
    int b0 = 0, b1 = 0;
    for (int k = 0; k < n; ++k) {
        b0 |= bad[2 * k];
        b1 |= bad[2 * k + 1];
    }
    *pieces = (!b0 || !b1) ? 1 : 3;
    *scale = !b0 ? 1.0 : (!b1 ? 255.0 : 1.0);
}

// The blocked copy of rows 0..rows-1 in a given operand form, kbn blocks of
// 32 columns, with room for wmax gathered rows.
TcSet *rs_set_make(const irwls_dev_set *X, int rows, int wmax, int kbn, int P, double scale) {
    TcSet *t = (TcSet *)calloc(1, sizeof(TcSet));
    if (!t) return nullptr;
    t->rows = rows;
    t->kbn = kbn;
    t->wmax = wmax;
    t->rbf = X->mode != IRWLS_K_LINEAR;
    t->ng = (float)X->neg_gamma;
    t->pieces = P;
    t->scale = scale;
    t->dscale = (float)(1.0 / (scale * scale));
    int rc = irwls_dev_malloc((void **)&t->bad, 4 * sizeof(int));
    t->nbuf = t->bad + 2;
    const size_t ab = (size_t)ceil_div(rows > 0 ? rows : 1, RS_BM) * RS_BM * t->kbn * RS_BK * P * sizeof(__nv_bfloat16);
    const size_t bb = (size_t)ceil_div(wmax > 0 ? wmax : 1, RS_BN) * RS_BN * t->kbn * RS_BK * P * sizeof(__nv_bfloat16);
    rc |= irwls_dev_malloc((void **)&t->A, ab);
    rc |= irwls_dev_malloc((void **)&t->B, bb);
    rc |= irwls_dev_malloc((void **)&t->q, (size_t)(rows > 0 ? rows : 1) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&t->qb, (size_t)(wmax > 0 ? wmax : 1) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&t->cbf, (size_t)(wmax > 0 ? wmax : 1) * sizeof(float));
    if (!rc && rows > 0) {
        const long long total = (long long)ceil_div(rows, RS_BM) * RS_BM * t->kbn * RS_BK;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 65535);
        if (P == 1)
            rs_split_kernel<1><<<blocks, 256, 0, irwls_stream()>>>(X->X, rows, X->width, X->ld, t->kbn, scale, t->A);
        else
            rs_split_kernel<3><<<blocks, 256, 0, irwls_stream()>>>(X->X, rows, X->width, X->ld, t->kbn, scale, t->A);
        irwls_count_launch(1);
        to_f32_kernel<<<ceil_div(rows, 256), 256, 0, irwls_stream()>>>(X->q, rows, t->q);
        irwls_count_launch(1);
        if (cudaPeekAtLastError() != cudaSuccess) rc = -1;
    }
    t->kbound = 1.0;
    if (!rc && !t->rbf && rows > 0) {
        max_q_kernel<<<1, 1024, 0, irwls_stream()>>>(t->q, rows, t->qb);
        irwls_count_launch(1);
        float mq = 0.f;
        rc |= irwls_dev_d2h(&mq, t->qb, sizeof(float));
        rc |= irwls_dev_sync();
        t->kbound = 1.01 * (double)mq;
    }
    if (rc) {
        irwls_tc_set_free(t);
        irwls_set_error(-3, "cannot create the split copy of the dataset");
        return nullptr;
    }
    return t;
}
}  // namespace

namespace {
// bad[0] |= some stored value times `scale` is not an integer.
__global__ void rs_int_check_kernel(const double *__restrict__ v, long long n, double scale, int *bad) {
    int b = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double x = v[t] * scale;
        if (x != rint(x)) b = 1;
    }
    b = __any_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0 && b) atomicOr(bad, 1);
}

// Whether the exact-integer mode applies to a one-piece set (sets t->exact):
// every stored value times the scale an integer (true by construction for
// scale 255: the value is RN(k / 255) and the split rounds it to k), the
// kernel RBF in norm form or linear, and max_i ||scale x_i||^2 < 2^24, so that
// every partial sum of a dot product of two rows is an integer below 2^24.
int rs_exact_check(const irwls_dev_set *X, TcSet *t) {
    t->exact = 0;
    if (t->pieces != 1 || X->mode == IRWLS_K_RAW_RBF) return 0;
    int nnz = 0, bad = 0;
    int rc = irwls_dev_d2h(&nnz, X->rp + t->rows, sizeof(int));
    rc |= irwls_dev_sync();
    if (rc) return rc;
    if (t->scale == 1.0 && nnz > 0) {
        rc |= irwls_dev_memset(t->bad, 0, sizeof(int));
        const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
        const int blocks = (int)std::max<long long>(1, std::min<long long>((nnz + 255LL) / 256, 8LL * sms));
        rs_int_check_kernel<<<blocks, 256, 0, irwls_stream()>>>(X->cv, nnz, 1.0, t->bad);
        irwls_count_launch(1);
        rc |= irwls_dev_d2h(&bad, t->bad, sizeof(int));
        rc |= irwls_dev_sync();
        if (rc) return rc;
    }
    max_q_kernel<<<1, 1024, 0, irwls_stream()>>>(t->q, t->rows, t->qb);
    irwls_count_launch(1);
    float mq = 0.f;
    rc |= irwls_dev_d2h(&mq, t->qb, sizeof(float));
    rc |= irwls_dev_sync();
    if (rc) return rc;
    const double bound = 1.001 * (double)mq * t->scale * t->scale;
    t->exact = !bad && bound < 16777216.0;
    return 0;
}
}  // namespace

// Blocked copy of rows 0..rows-1 of a device set for the precision form, in
// the operand form its values allow, with room for `wmax` gathered rows.
extern "C" void *irwls_tc_set_create(const irwls_dev_set *X, int rows, int wmax) {
    int *d_bad = nullptr, bad[2] = {1, 1};
    if (irwls_dev_malloc((void **)&d_bad, 2 * sizeof(int))) return nullptr;
    const int rc = rs_check(X, rows, d_bad, bad);
    irwls_dev_free(d_bad);
    if (rc) return nullptr;
    int P;
    double scale;
    rs_form(bad, 1, &P, &scale);
    g_rs_last_pieces = P;
    TcSet *t = rs_set_make(X, rows, wmax, ceil_div(X->width, RS_BK), P, scale);
    if (t && rows > 0 && rs_exact_check(X, t)) {
        irwls_tc_set_free(t);
        return nullptr;
    }
    return t;
}

extern "C" double irwls_tc_set_kbound(void *h) { return ((TcSet *)h)->kbound; }

extern "C" void irwls_tc_set_free(void *h) {
    TcSet *t = (TcSet *)h;
    if (!t) return;
    irwls_dev_free(t->A);
    irwls_dev_free(t->B);
    irwls_dev_free(t->q);
    irwls_dev_free(t->qb);
    irwls_dev_free(t->cbf);
    irwls_dev_free(t->bad);
    irwls_dev_free(t->Ag);
    irwls_dev_free(t->part);
    free(t);
}

namespace {
// Gathers the rows idx[j < *d_n] into B, then runs the engine over the first
// M rows of the set in the given mode.
template <int P, int MODE>
int rs_launch(TcSet *t, int M, const int *d_idx, const int *d_n, const double *d_cb, const double *d_init,
              const double *d_tail, double *d_out, const TcSet *src = nullptr, double bias = 0.0, int hard = 0) {
    // B rows come from the set itself (error updates) or from another set of
    // the same layout (a model's support vectors)
    const TcSet *from = src ? src : t;
    const int gb = std::max(1, std::min(ceil_div((long long)t->wmax * t->kbn * P * 4, 256), 4096));
    rs_gather_kernel<P><<<gb, 256, 0, irwls_stream()>>>(from->A, t->kbn, from->q, d_idx, d_n, t->wmax, t->B, t->qb,
                                                        d_cb, t->cbf);
    IRWLS_LAUNCH_CHECK("tc_gather_rows");
    constexpr int NS = rs_stages<P>();
    const size_t smem = NS * RsStage<P>::BYTES + 1024;
    static_assert(NS * RsStage<P>::BYTES + 1024 <= 227 * 1024, "ring exceeds shared memory");
    cudaFuncSetAttribute(tc_rowsum_ws_kernel<P, NS, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int ntiles = ceil_div(M, RS_BM);
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int slot = MODE == 0 ? IRWLS_PROF_ROWSUM : IRWLS_PROF_PREDICT;
    if (irwls_prof_on()) irwls_prof_begin(slot);
    tc_rowsum_ws_kernel<P, NS, MODE><<<std::max(1, std::min(ntiles, sms)), RS_THREADS, smem, irwls_stream()>>>(
        t->A, M, t->kbn, t->q, t->B, d_n, t->wmax, t->qb, t->cbf, t->rbf, t->ng, t->dscale, d_init, d_tail, d_out, bias,
        hard, irwls_dev_flags(), g_rs_wait_limit, g_rs_stall);
    if (irwls_prof_on()) irwls_prof_end(slot);
    IRWLS_LAUNCH_CHECK(MODE == 0 ? "tc_kernel_rowsum" : "tc_predict");
    return 0;
}
}  // namespace

// out_i = (init_i - sum_{j < *d_n} cb_j k(x_i, x_{idx_j})) - tail[0] for every
// row of the set (init may alias out; tail may be NULL).
extern "C" int irwls_tc_kernel_rowsum(void *h, const int *d_idx, const int *d_n, const double *d_cb,
                                      const double *d_init, const double *d_tail, double *d_out) {
    TcSet *t = (TcSet *)h;
    if (t->rows <= 0) return 0;
    return t->pieces == 1 ? rs_launch<1, 0>(t, t->rows, d_idx, d_n, d_cb, d_init, d_tail, d_out)
                          : rs_launch<3, 0>(t, t->rows, d_idx, d_n, d_cb, d_init, d_tail, d_out);
}

namespace {
__global__ void iota_kernel(int *p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}
}  // namespace

// Precision-form prediction (src/LIBIRWLS-predict.c:56-131 computes
// f(x) = b + sum_j w_j k(x, sv_j) in FP64): the test rows T and the support
// vectors S in one blocked operand form (1 exact piece when both sets allow
// the same scale, else 3), f from the tensor-core dot products with an FP32
// exp and Kahan-compensated FP32 sums, bias added in FP64; the sign (>= 0 ->
// +1) when `hard`. T and S share the feature width.
extern "C" int irwls_tc_predict(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w,
                                double bias, int hard, double *d_out) {
    if (n <= 0) return 0;
    int *d_bad = nullptr, *d_idx = nullptr, bad[4] = {1, 1, 1, 1};
    int rc = irwls_dev_malloc((void **)&d_bad, 4 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_idx, (size_t)std::max(nSV, 1) * sizeof(int));
    if (!rc) rc |= rs_check(T, n, d_bad, bad);
    if (!rc) rc |= rs_check(S, nSV, d_bad + 2, bad + 2);
    TcSet *ts = nullptr, *ss = nullptr;
    if (!rc) {
        int P;
        double scale;
        rs_form(bad, 2, &P, &scale);
        const int kbn = ceil_div(std::max(T->width, S->width), RS_BK);
        ts = rs_set_make(T, n, nSV, kbn, P, scale);
        ss = ts ? rs_set_make(S, nSV, 0, kbn, P, scale) : nullptr;
        if (!ts || !ss) rc = -3;
    }
    if (!rc && nSV > 0) {
        iota_kernel<<<ceil_div(nSV, 256), 256, 0, irwls_stream()>>>(d_idx, nSV);
        irwls_count_launch(1);
        rc |= irwls_dev_h2d(ts->nbuf, &nSV, sizeof(int));
    }
    if (!rc) {
        if (nSV <= 0)
            rc = irwls_dev_memset(ts->nbuf, 0, sizeof(int));
        if (!rc)
            rc = ts->pieces == 1
                     ? rs_launch<1, 1>(ts, n, d_idx, ts->nbuf, d_w, nullptr, nullptr, d_out, ss, bias, hard)
                     : rs_launch<3, 1>(ts, n, d_idx, ts->nbuf, d_w, nullptr, nullptr, d_out, ss, bias, hard);
    }
    irwls_tc_set_free(ts);
    irwls_tc_set_free(ss);
    irwls_dev_free(d_bad);
    irwls_dev_free(d_idx);
    return rc;
}

// ---------------------------------------------------------------------------
// Exact-integer mode of the engine: FP64 kernel row sums over a row subset,
// with the dot products on the tensor cores.
//
// When every stored value times the set's scale s (1 or 255) is an integer
// and max_i ||s x_i||^2 < 2^24 (rs_exact_check), each one-piece bf16 product
// (s x_ik)(s x_jk) is an integer and every partial sum of a dot product is an
// integer of magnitude at most ||s x_i|| ||s x_j|| < 2^24: the FP32
// accumulation is exact in any order. The kernel value then follows in FP64,
// k_ij = exp(-gamma ((q_i + q_j) - 2 dot / s^2)) (RBF) or dot / s^2 (linear),
// within a few ulps of the reference's value, at about 25 FP64 operations
// per value instead of two per stored feature; so do the weighted sums
// (in a different order than the reference's left-to-right one).
//
// One CTA per item (a 128-row tile of the gathered rows x CW columns of the
// gathered list): warp 0 streams the operands through a 4-stage bulk-copy
// ring, warp 1 issues the MMAs into a 128 x CW FP32 accumulator in tensor
// memory, then all 8 warps form the item's partial row sums in FP64
// (rows by lane, columns split between two warp groups), written to
// part[h][row]; ex_combine_kernel adds the partials of each row in item
// order. Every wait is bounded; a wait that runs out sets device flag 1.
// ---------------------------------------------------------------------------
namespace {

constexpr int EX_THREADS = 256;
constexpr int EX_NS = 4;
std::atomic<long long> g_ex_calls{0};

// Rows ia[i < nA] of the full blocked copy A into the tile layout of the row
// subset Ag (16-byte groups of one core-matrix row at a time).
__global__ void rs_gather_rows_kernel(const __nv_bfloat16 *__restrict__ A, int kbn, const int *__restrict__ ia,
                                      int nA, __nv_bfloat16 *__restrict__ Ag) {
    const long long total = (long long)nA * kbn * 4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(t & 3);
        const long long rest = t >> 2;
        const int k = (int)(rest % kbn), i = (int)(rest / kbn), s = ia[i];
        const size_t src = ((size_t)(s >> 7) * kbn + k) * RS_APIECE + rs_core(s & 127, 8 * g);
        const size_t dst = ((size_t)(i >> 7) * kbn + k) * RS_APIECE + rs_core(i & 127, 8 * g);
        *(uint4 *)(Ag + dst) = *(const uint4 *)(A + src);
    }
}

// STORE: the kernel values themselves, out[j * ldp + i] = (k_ij sa_i) sb_j
// (a column-major block; with `lower`, items wholly above the diagonal are
// skipped), instead of partial row sums.
template <int CW, bool STORE>
__global__ void __launch_bounds__(EX_THREADS, 1) tc_exact_rowsum_kernel(
    const __nv_bfloat16 *__restrict__ A, int M, int kbn, const __nv_bfloat16 *__restrict__ B,
    const int *__restrict__ d_n, int nmax, int nchx, const double *__restrict__ q, const int *__restrict__ ia,
    const int *__restrict__ ib, int rbf, double ng, double dscale, const double *__restrict__ cb,
    const double *__restrict__ sa, const double *__restrict__ sb, double *__restrict__ part, long long ldp,
    int lower, int *flags, long long wait_limit) {
    static_assert(CW == 32 || CW == 64 || CW == 128, "column width");
    // columns per warp group in the epilogue (one group when CW is 32)
    constexpr int HALF = CW >= 64 ? CW / 2 : CW;
    constexpr uint32_t A_BYTES = RS_APIECE * 2, B_MAX = CW * RS_BK * 2;
    extern __shared__ __align__(1024) unsigned char ex_smem[];
    __shared__ __align__(8) uint64_t full[EX_NS], empty[EX_NS], accf;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ double half_sum[RS_BM];
    const int N = max(0, min(*d_n, nmax));
    const int tile = (int)blockIdx.x / nchx, h = (int)blockIdx.x % nchx, c0 = h * CW;
    if (c0 >= N) return;  // the list is shorter than this item's columns
    if (STORE && lower && c0 > tile * RS_BM + RS_BM - 1) return;  // above the diagonal
    unsigned char *smem = ex_smem + ((1024 - (smem_u32(ex_smem) & 1023)) & 1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ncols = min(CW, N - c0), nr16 = (ncols + 15) / 16 * 16;
    const uint32_t bbytes = (uint32_t)nr16 * RS_BK * 2;
    if (threadIdx.x == 0) {
        for (int b = 0; b < EX_NS; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        mbar_init(&accf, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(CW));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const uint32_t tmem = tmem_slot;
    const uint32_t stage_bytes = A_BYTES + B_MAX;
    if (warp == 0 && lane == 0) {
        // producer: the A tile and this item's B rows of each 32-wide K block
        const uint32_t base = smem_u32(smem);
        const __nv_bfloat16 *Bc = B + (size_t)(c0 >> 8) * kbn * RS_BPIECE + (size_t)((c0 & 255) >> 3) * 256;
        int issued = 0;
        for (int k = 0; k < kbn; ++k) {
            const int slot = k % EX_NS;
            if (k >= EX_NS && !mbar_wait_lim(smem_u32(&empty[slot]), (uint32_t)(k / EX_NS - 1) & 1u, wait_limit))
                abort_flag = 1;
            if (abort_flag) break;
            const uint32_t sb = base + slot * stage_bytes, fb = smem_u32(&full[slot]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(A_BYTES + bbytes));
            bulk_g2s(sb, A + ((size_t)tile * kbn + k) * RS_APIECE, A_BYTES, fb);
            bulk_g2s(sb + A_BYTES, Bc + (size_t)k * RS_BPIECE, bbytes, fb);
            issued = k + 1;
        }
        // no copy is left in flight
        for (int k = issued > EX_NS ? issued - EX_NS : 0; k < issued; ++k)
            if (!mbar_wait_lim(smem_u32(&full[k % EX_NS]), (uint32_t)(k / EX_NS) & 1u, wait_limit)) abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc_idesc(RS_BM, nr16);
        bool any = false;
        for (int k = 0; k < kbn && !abort_flag; ++k) {
            const int slot = k % EX_NS;
            if (!mbar_wait_lim(smem_u32(&full[slot]), (uint32_t)(k / EX_NS) & 1u, wait_limit)) {
                abort_flag = 1;
                break;
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::);
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
            const uint32_t sa_ = smem_u32(smem + slot * stage_bytes), sbb = sa_ + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < RS_BK / 16; ++kk)
                mma_bf16(tmem, tc_desc_sbo(sa_ + kk * 256, 512), tc_desc_sbo(sbb + kk * 256, 512), idesc,
                         (k > 0 || kk > 0) ? 1u : 0u);
            tc_commit(&empty[slot]);
            any = true;
        }
        // completes once every MMA issued has (or at once if none was)
        if (any) tc_commit(&accf);
        else mbar_arrive(&accf);
    }
    __syncwarp();
    const bool got = mbar_wait_lim(smem_u32(&accf), 0u, wait_limit);
    // one decision for the whole CTA (the epilogue has a named barrier)
    const bool ok = __syncthreads_and(got ? 1 : 0) && !abort_flag;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (ok) {
        const int ew = warp & 3, gh = warp >> 2, r = 32 * ew + lane, row = tile * RS_BM + r;
        const bool valid = row < M;
        const int gi = valid ? ia[row] : 0;
        const double qi = valid ? q[gi] : 0.0, sai = (valid && sa) ? sa[gi] : 1.0;
        double acc = 0.0;
        for (int cc = 0; cc < HALF; cc += 32) {
            const int cbase = gh * HALF + cc;
            if (cbase >= ncols) break;
            float v[32];
            tc_ld32_lanes(tmem, 32 * ew, cbase, v);
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
                const int c = cbase + jj;
                if (c < ncols) {
                    const int j = c0 + c, gj = ib[j];
                    const double dot = (double)v[jj] * dscale;
                    const double kv = rbf ? exp(ng * fma(-2.0, dot, qi + q[gj])) : dot;
                    double t = cb ? cb[j] * kv : kv;
                    if (sa) t *= sai;
                    if (sb) t *= sb[gj];
                    if (STORE) {
                        if (valid) part[(size_t)j * ldp + row] = t;
                    } else {
                        acc += t;
                    }
                }
            }
        }
        if (!STORE) {
            if (gh == 1) half_sum[r] = acc;
            asm volatile("bar.sync 1, %0;\n" ::"r"(EX_THREADS));
            if (gh == 0 && valid) part[(size_t)h * ldp + row] = acc + half_sum[r];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (threadIdx.x == 0 && !ok) atomicExch(flags + 1, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(CW));
}

// out_i = (init_i OP sum_h part[h][i]) - tail[0] over the items of the list
// that *d_n leaves, in item order (init may alias out; init, tail optional).
__global__ void ex_combine_kernel(const double *__restrict__ part, int ldp, int M, const int *__restrict__ d_n,
                                  int nmax, int cw, int op, const double *init, const double *__restrict__ tail,
                                  double *out) {
    const int N = max(0, min(*d_n, nmax)), nch = (N + cw - 1) / cw;
    const double tl = tail ? tail[0] : 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int h = 0; h < nch; ++h) s += part[(size_t)h * ldp + i];
        double acc = init ? init[i] : 0.0;
        acc = op > 0 ? acc + s : acc - s;
        out[i] = tail ? acc - tl : acc;
    }
}

__global__ void set_int_kernel(int *p, int v) { *p = v; }

template <int CW, bool STORE>
int ex_launch(TcSet *t, const irwls_dev_set *X, int nA, const int *d_ia, const int *d_ib, const int *d_n, int nmax,
              const double *d_cb, const double *d_sa, const double *d_sb, double *out, long long ldo, int lower) {
    const int ntiles = ceil_div(nA, RS_BM), nchx = ceil_div(nmax, CW);
    const size_t smem = (size_t)EX_NS * (RS_APIECE * 2 + CW * RS_BK * 2) + 1024;
    cudaFuncSetAttribute(tc_exact_rowsum_kernel<CW, STORE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    tc_exact_rowsum_kernel<CW, STORE><<<ntiles * nchx, EX_THREADS, smem, irwls_stream()>>>(
        t->Ag, nA, t->kbn, t->B, d_n, nmax, nchx, X->q, d_ia, d_ib, t->rbf, X->neg_gamma, 1.0 / (t->scale * t->scale),
        d_cb, d_sa, d_sb, out, ldo, lower, irwls_dev_flags(), g_rs_wait_limit);
    IRWLS_LAUNCH_CHECK(STORE ? "tc_exact_block" : "tc_exact_rowsum");
    return 0;
}

// Gathers the rows ia (nA) and the list entries ib (*d_n <= nmax) of the set.
int ex_gather(TcSet *t, const irwls_dev_set *X, const int *d_ia, int nA, const int *d_ib, const int *d_n, int nmax,
              const double *d_cb) {
    const long long rows_pad = (long long)ceil_div(nA, RS_BM) * RS_BM;
    if (rows_pad > t->ag_cap) {
        irwls_dev_free(t->Ag);
        t->Ag = nullptr;
        t->ag_cap = 0;
        if (irwls_dev_malloc((void **)&t->Ag, (size_t)rows_pad * t->kbn * RS_BK * sizeof(__nv_bfloat16))) return -3;
        t->ag_cap = rows_pad;
    }
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int gr = std::max(1, std::min(ceil_div((long long)nA * t->kbn * 4, 256), 8 * sms));
    rs_gather_rows_kernel<<<gr, 256, 0, irwls_stream()>>>(t->A, t->kbn, d_ia, nA, t->Ag);
    IRWLS_LAUNCH_CHECK("tc_exact_gather_rows");
    const int gb = std::max(1, std::min(ceil_div((long long)std::max(nmax, 1) * t->kbn * 4, 256), 4096));
    rs_gather_kernel<1><<<gb, 256, 0, irwls_stream()>>>(t->A, t->kbn, t->q, d_ib, d_n, t->wmax, t->B, t->qb,
                                                        d_cb ? d_cb : X->q, t->cbf);
    IRWLS_LAUNCH_CHECK("tc_exact_gather_cols");
    return 0;
}

}  // namespace

// FP64 kernel row sums with exact tensor-core dot products (the precision
// form's exact rows): for i < nA,
//   out_i = (init_i OP sum_{j < n} t_ij) - tail[0],
//   t_ij = ((cb_j k(x_ia[i], x_ib[j])) sa_ia[i]) sb_ib[j]   (cb, sa, sb optional),
// n = nB, or *d_nB when d_nB is given (then at most nbmax). The same values as
// irwls_dev_kernel_rowsum(_n) to within a few ulps of each kernel value and a
// different summation order. Returns 1 without doing anything when the set
// does not allow the exact mode or the list may exceed the set's gather room
// (the caller then uses the FP64 kernels), else 0 or an error.
extern "C" int irwls_tc_exact_rowsum(void *h, const irwls_dev_set *X, const int *d_ia, int nA, const int *d_ib,
                                     int nB, const int *d_nB, int nbmax, const double *d_cb, const double *d_sa,
                                     const double *d_sb, int op, const double *d_init, const double *d_tail,
                                     double *d_out) {
    TcSet *t = (TcSet *)h;
    if (!t || !t->exact) return 1;
    if (!d_nB) nbmax = nB;
    if (nbmax > t->wmax || nbmax < 0) return 1;
    if (nA <= 0) return 0;
    const int *d_n = d_nB;
    if (!d_nB) {
        set_int_kernel<<<1, 1, 0, irwls_stream()>>>(t->nbuf, nB);
        IRWLS_LAUNCH_CHECK("tc_exact_count");
        d_n = t->nbuf;
    }
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int ntiles = ceil_div(nA, RS_BM);
    // column width: enough items for every SM when the tiles are few
    int cw = 128;
    while (cw > 32 && (long long)ntiles * ceil_div(std::max(nbmax, 1), cw) < 2LL * sms) cw >>= 1;
    const long long need = (long long)ceil_div(std::max(nbmax, 1), cw) * nA;
    if (need > t->part_cap) {
        irwls_dev_free(t->part);
        t->part = nullptr;
        t->part_cap = 0;
        if (irwls_dev_malloc((void **)&t->part, (size_t)need * sizeof(double))) return -3;
        t->part_cap = need;
    }
    if (nbmax > 0) {
        int rc = ex_gather(t, X, d_ia, nA, d_ib, d_n, nbmax, d_cb);
        if (rc) return rc;
        if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_ROWSUM);
        rc = cw == 128  ? ex_launch<128, false>(t, X, nA, d_ia, d_ib, d_n, nbmax, d_cb, d_sa, d_sb, t->part, nA, 0)
             : cw == 64 ? ex_launch<64, false>(t, X, nA, d_ia, d_ib, d_n, nbmax, d_cb, d_sa, d_sb, t->part, nA, 0)
                        : ex_launch<32, false>(t, X, nA, d_ia, d_ib, d_n, nbmax, d_cb, d_sa, d_sb, t->part, nA, 0);
        if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_ROWSUM);
        if (rc) return rc;
    }
    ex_combine_kernel<<<std::max(1, std::min(ceil_div(nA, 256), 4 * sms)), 256, 0, irwls_stream()>>>(
        t->part, nA, nA, d_n, nbmax, cw, op, d_init, d_tail, d_out);
    IRWLS_LAUNCH_CHECK("tc_exact_combine");
    ++g_ex_calls;
    return 0;
}

// The kernel block itself in the exact-integer mode: out[j * ldo + i] =
// (k(x_ia[i], x_ib[j]) sa_ia[i]) sb_ib[j] for i < nA, j < nB (sa, sb
// optional); with `lower`, only the blocks on or below the diagonal (i >= j
// up to the 128 x 64 item grid; the rest of the upper part may be left
// unwritten). Returns 1 when the set does not allow it or nB exceeds its
// gather room.
extern "C" int irwls_tc_exact_block(void *h, const irwls_dev_set *X, const int *d_ia, int nA, const int *d_ib, int nB,
                                    const double *d_sa, const double *d_sb, double *d_out, long long ldo, int lower) {
    TcSet *t = (TcSet *)h;
    if (!t || !t->exact || nB > t->wmax || nB < 0) return 1;
    if (nA <= 0 || nB <= 0) return 0;
    set_int_kernel<<<1, 1, 0, irwls_stream()>>>(t->nbuf, nB);
    IRWLS_LAUNCH_CHECK("tc_exact_count");
    int rc = ex_gather(t, X, d_ia, nA, d_ib, t->nbuf, nB, nullptr);
    if (rc) return rc;
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_ROWSUM);
    rc = ex_launch<32, true>(t, X, nA, d_ia, d_ib, t->nbuf, nB, nullptr, d_sa, d_sb, d_out, ldo, lower);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_ROWSUM);
    if (rc) return rc;
    ++g_ex_calls;
    return 0;
}

// Whether a set made by irwls_tc_set_create allows the exact-integer mode.
extern "C" int irwls_tc_set_exact(void *h) { return h && ((TcSet *)h)->exact; }

// Row sums done in the exact-integer mode since the last reset.
extern "C" long long irwls_tc_exact_calls(int reset) {
    const long long n = g_ex_calls.load();
    if (reset) g_ex_calls = 0;
    return n;
}
