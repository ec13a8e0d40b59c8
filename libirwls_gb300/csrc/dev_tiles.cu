// dev_tiles.cu -- kernel-matrix tiles (reference src/kernels.c:63-183 applied
// to whole blocks of row pairs).
//
// Layout: the CTA stages its A rows densely in shared memory; B rows stream
// from global memory, as raw values (raw-RBF mode) or as CSR entries that are
// looked up against the dense A row, so stored zeros cost nothing. The work
// is FP64-ALU bound on GB300, so the design minimises FP64 instructions per
// kernel entry; memory traffic is a few bytes per entry and hits L1/L2.
#include "dev_common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr size_t kSmemBudget = 96 * 1024;

// Rows of A a CTA stages, given the dense width; 0 if even one row does not fit.
int rows_per_cta(int ld, int wanted) {
    size_t per = (size_t)ld * sizeof(double);
    int r = wanted;
    while (r > 1 && (size_t)r * per > kSmemBudget) r >>= 1;
    return ((size_t)r * per > kSmemBudget) ? 0 : r;
}

__device__ __forceinline__ void stage_rows(double *sA, double *sQ, const KView &A, const int *ia, int i0, int R,
                                           int nA) {
    for (int r = 0; r < R; ++r) {
        const int i = i0 + r;
        const int g = (i < nA) ? (ia ? ia[i] : i) : -1;
        for (int t = threadIdx.x; t < A.ld; t += blockDim.x) sA[r * A.ld + t] = (g >= 0) ? A.X[(size_t)g * A.ld + t] : 0.0;
        if (threadIdx.x == 0) sQ[r] = (g >= 0) ? A.q[g] : 0.0;
    }
    __syncthreads();
}

// out[i*ld_out + j] (or out[j*ld_out + i] when `trans`) = k(A_i, B_j).
// grid: (ceil(nB / 128), ceil(nA / R)); each thread owns one B column and
// R/2 rows of the CTA's R staged rows.
__global__ void __launch_bounds__(kThreads) kernel_block_kernel(KView A, const int *__restrict__ ia, int nA, KView B,
                                                                const int *__restrict__ ib, int nB, int R,
                                                                double *__restrict__ out, long long ld_out, int trans) {
    extern __shared__ double smem[];
    double *sA = smem;
    double *sQ = smem + (size_t)R * A.ld;
    const int i0 = blockIdx.y * R;
    stage_rows(sA, sQ, A, ia, i0, R, nA);
    const int j = blockIdx.x * 128 + (threadIdx.x & 127);
    if (j >= nB) return;
    const int jb = ib ? ib[j] : j;
    for (int r = threadIdx.x >> 7; r < R; r += 2) {
        const int i = i0 + r;
        if (i >= nA) break;
        const double kv = kentry(B, sA + (size_t)r * A.ld, sQ[r], jb);
        if (trans) out[(size_t)j * ld_out + i] = kv;
        else out[(size_t)i * ld_out + j] = kv;
    }
}

// Ordered row sums. CTA = R output rows x all B; B is swept in chunks of
// JB = 1024 / R columns: every thread evaluates 4 terms into shared memory,
// then one thread per row folds the chunk left to right.
__global__ void __launch_bounds__(kThreads) kernel_rowsum_kernel(KView A, const int *__restrict__ ia, int nA, KView B,
                                                                 const int *__restrict__ ib, int nB,
                                                                 const int *__restrict__ nBp, int R,
                                                                 const double *__restrict__ cb,
                                                                 const double *__restrict__ sa,
                                                                 const double *__restrict__ sb, int op,
                                                                 const double *init,  // may alias out
                                                                 const double *__restrict__ tail, double *out) {
    extern __shared__ double smem[];
    double *sA = smem;
    double *sQ = smem + (size_t)R * A.ld;
    double *sT = sQ + 8;  // R x JB terms
    const int JB = 1024 / R;
    if (nBp) nB = *nBp;
    const int i0 = blockIdx.x * R;
    stage_rows(sA, sQ, A, ia, i0, R, nA);
    double acc = 0.0;
    const int me = i0 + threadIdx.x;
    const bool folder = threadIdx.x < R && me < nA;
    if (folder) acc = init ? init[me] : 0.0;
    for (int j0 = 0; j0 < nB; j0 += JB) {
        const int jn = min(JB, nB - j0);
        for (int t = threadIdx.x; t < R * JB; t += kThreads) {
            const int r = t / JB, jj = t - r * JB;
            const int i = i0 + r;
            double term = 0.0;
            if (jj < jn && i < nA) {
                const int j = j0 + jj;
                const int jb = ib ? ib[j] : j;
                double kv = kentry(B, sA + (size_t)r * A.ld, sQ[r], jb);
                term = cb ? __dmul_rn(cb[j], kv) : kv;
                if (sa) term = __dmul_rn(term, sa[ia ? ia[i] : i]);
                if (sb) term = __dmul_rn(term, sb[jb]);
            }
            sT[t] = term;
        }
        __syncthreads();
        if (folder) {
            const double *row = sT + threadIdx.x * JB;
            if (op > 0)
                for (int jj = 0; jj < jn; ++jj) acc = __dadd_rn(acc, row[jj]);
            else
                for (int jj = 0; jj < jn; ++jj) acc = __dsub_rn(acc, row[jj]);
        }
        __syncthreads();
    }
    if (folder) out[me] = tail ? __dsub_rn(acc, tail[0]) : acc;
}

}  // namespace

extern "C" int irwls_dev_kernel_block_t(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                                        const int *d_ib, int nB, double *d_out, long long ld_out, int trans) {
    if (nA <= 0 || nB <= 0) return 0;
    const int R = rows_per_cta(A->ld, 16);
    if (R == 0) {
        irwls_set_error(-5, "feature width %d is too wide for the shared-memory tile", A->width);
        return -5;
    }
    const size_t smem = ((size_t)R * A->ld + 16) * sizeof(double);
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(ceil_div(nB, 128), ceil_div(nA, R));
    kernel_block_kernel<<<grid, kThreads, smem, irwls_stream()>>>(kview(A), d_ia, nA, kview(B), d_ib, nB, R, d_out,
                                                                   ld_out, trans);
    IRWLS_LAUNCH_CHECK("kernel_block");
    return 0;
}

extern "C" int irwls_dev_kernel_block(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                                      const int *d_ib, int nB, double *d_out, int ld_out) {
    return irwls_dev_kernel_block_t(A, d_ia, nA, B, d_ib, nB, d_out, ld_out, 0);
}

static int rowsum_launch(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B, const int *d_ib,
                         int nB, const int *d_nB, const double *d_cb, const double *d_sa, const double *d_sb, int op,
                         const double *d_init, const double *d_tail, double *d_out) {
    if (nA <= 0) return 0;
    // rows per CTA: enough CTAs to cover the SMs twice, at most 8
    int R = 8;
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    while (R > 1 && ceil_div(nA, R) < 2 * sms) R >>= 1;
    while (R > 1 && rows_per_cta(A->ld, R) < R) R >>= 1;
    if (rows_per_cta(A->ld, R) < R) {
        irwls_set_error(-5, "feature width %d is too wide for the shared-memory tile", A->width);
        return -5;
    }
    const size_t smem = ((size_t)R * A->ld + 8 + 1024) * sizeof(double);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(kernel_rowsum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_ROWSUM);
    kernel_rowsum_kernel<<<ceil_div(nA, R), kThreads, smem, irwls_stream()>>>(
        kview(A), d_ia, nA, kview(B), d_ib, nB > 0 ? nB : 0, d_nB, R, d_cb, d_sa, d_sb, op, d_init, d_tail, d_out);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_ROWSUM);
    IRWLS_LAUNCH_CHECK("kernel_rowsum");
    return 0;
}

extern "C" int irwls_dev_kernel_rowsum(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                                       const int *d_ib, int nB, const double *d_cb, const double *d_sa,
                                       const double *d_sb, int k_first, int op, const double *d_init,
                                       const double *d_tail, double *d_out) {
    (void)k_first;  // IEEE multiplication commutes: k*c and c*k round identically
    return rowsum_launch(A, d_ia, nA, B, d_ib, nB, nullptr, d_cb, d_sa, d_sb, op, d_init, d_tail, d_out);
}

extern "C" int irwls_dev_kernel_rowsum_n(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                                         const int *d_ib, const int *d_nB, const double *d_cb, const double *d_sa,
                                         const double *d_sb, int op, const double *d_init, const double *d_tail,
                                         double *d_out) {
    return rowsum_launch(A, d_ia, nA, B, d_ib, 0, d_nB, d_cb, d_sa, d_sb, op, d_init, d_tail, d_out);
}
