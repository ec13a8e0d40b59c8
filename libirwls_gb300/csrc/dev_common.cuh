// dev_common.cuh -- shared device helpers of the IRWLS kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "irwls_dev.h"

// The library's single stream (dev_context.cu).
cudaStream_t irwls_stream();
int irwls_check_launch(const char *what);
int irwls_num_sms();

#define IRWLS_LAUNCH_CHECK(what)                         \
    do {                                                 \
        irwls_count_launch(1);                           \
        int _rc = irwls_check_launch(what);              \
        if (_rc) return _rc;                             \
    } while (0)

// Chained launches (programmatic dependent launch): a kernel launched with
// launch_chained may be scheduled while the kernel before it on the stream
// is finishing, and starts with chain_wait(), which returns once that kernel
// has completed and its writes are visible; nothing before chain_wait() may
// touch global memory. chain_open() lets the next chained kernel be scheduled.
// Outside a chained launch both are no-ops.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void chain_open() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_chained(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = irwls_stream();
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// Device-side status words (dev_context.cu), a device array of 8 ints:
// [0] first failed Cholesky pivot of the last factorization (1-based, 0 if none).
int *irwls_dev_flags();

// ---------------------------------------------------------------------------
// Kernel entries. All arithmetic is FP64 with explicit round-to-nearest
// operations, so the values match the reference's x86 build
// (src/kernels.c:63-183) operation for operation: no multiply-add is
// contracted except the one in norm_sqdist, whose result is provably the
// reference's; exp() is CUDA's double-precision exponential.
// ---------------------------------------------------------------------------
struct KView {
    int mode;
    int width;
    int ld;
    double ng;  // -gamma
    const double *__restrict__ X;
    const int *__restrict__ rp;
    const int *__restrict__ ci;
    const double *__restrict__ cv;
    const double *__restrict__ q;
    const double *__restrict__ y;
};

static inline KView kview(const irwls_dev_set *s) {
    KView v;
    v.mode = s->mode;
    v.width = s->width;
    v.ld = s->ld;
    v.ng = s->neg_gamma;
    v.X = s->X;
    v.rp = s->rp;
    v.ci = s->ci;
    v.cv = s->cv;
    v.q = s->q;
    v.y = s->y;
    return v;
}

// Squared distance over `w` raw values (src/kernels.c:90-97).
__device__ __forceinline__ double raw_sqdist(const double *a, const double *b, int w) {
    double s = 0.0;
    for (int t = 0; t < w; ++t) {
        double d = __dsub_rn(a[t], b[t]);
        s = __dadd_rn(s, __dmul_rn(d, d));
    }
    return s;
}

// q_a + q_b, then "+ (-2 b_p) a[col_p]" over the stored entries of row b in
// index order (src/kernels.c:101-114). Entries whose partner value is zero
// add a signed zero, which leaves the sum unchanged, so iterating one row's
// entries against the other row's dense copy reproduces the merge-join.
// (-2 b) a rounds to -2 round(b a) (scaling by two is exact), so each entry
// is one multiply and one fused -2 t + s: the reference's value with two
// FP64 operations instead of three (the FP64 pipe bounds these kernels).
__device__ __forceinline__ double norm_sqdist(const double *a_dense, double qa, const KView &B, int jb) {
    double s = __dadd_rn(qa, B.q[jb]);
    const int p0 = B.rp[jb], p1 = B.rp[jb + 1];
    for (int p = p0; p < p1; ++p) s = __fma_rn(-2.0, __dmul_rn(B.cv[p], a_dense[B.ci[p]]), s);
    return s;
}

__device__ __forceinline__ double sparse_dot(const double *a_dense, const KView &B, int jb) {
    double s = 0.0;
    const int p0 = B.rp[jb], p1 = B.rp[jb + 1];
    for (int p = p0; p < p1; ++p) s = __dadd_rn(s, __dmul_rn(B.cv[p], a_dense[B.ci[p]]));
    return s;
}

// k(A row held densely in a_dense (shared memory), B row jb).
__device__ __forceinline__ double kentry(const KView &B, const double *a_dense, double qa, int jb) {
    if (B.mode == IRWLS_K_RAW_RBF) {
        return exp(__dmul_rn(B.ng, raw_sqdist(a_dense, B.X + (size_t)jb * B.ld, B.width)));
    } else if (B.mode == IRWLS_K_NORM_RBF) {
        return exp(__dmul_rn(B.ng, norm_sqdist(a_dense, qa, B, jb)));
    }
    return sparse_dot(a_dense, B, jb);
}

// Deterministic block-wide sum (fixed tree; every thread gets the result).
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = (lane < NT / 32) ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
