// dev_predict.cu -- batched prediction f(x_i) = bias + sum_j w_j k(x_i, sv_j)
// (reference src/LIBIRWLS-predict.c:56-131): an ordered kernel row sum, so
// every decision value accumulates its support vectors in the reference's
// order; the sign is taken on the device.
#include <algorithm>

#include "dev_common.cuh"

namespace {

__global__ void fill_kernel(double *p, int n, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

__global__ void sign_kernel(double *p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = (p[i] >= 0.0) ? 1.0 : -1.0;
}

// Linear-kernel fast path: W[c] = sum_j w_j sv_j[c]. Block b sums the
// support vectors of chunk b (LW_CHUNK of them, model order) for every
// feature c into part[b][c]; linear_w_reduce adds the chunks in order.
constexpr int LW_CHUNK = 64;
__global__ void linear_w_kernel(const double *__restrict__ X, int ld, int nsv, const double *__restrict__ w,
                                int width, double *__restrict__ part) {
    const int j0 = blockIdx.x * LW_CHUNK, j1 = min(nsv, j0 + LW_CHUNK);
    for (int c = threadIdx.x; c < width; c += blockDim.x) {
        double acc = 0.0;
        for (int j = j0; j < j1; ++j) acc = fma(w[j], X[(size_t)j * ld + c], acc);
        part[(size_t)blockIdx.x * width + c] = acc;
    }
}

__global__ void linear_w_reduce(const double *__restrict__ part, int nchunk, int width, double *__restrict__ W) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < width; c += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < nchunk; ++b) acc += part[(size_t)b * width + c];
        W[c] = acc;
    }
}

// f_i = bias + x_i . W, one warp per test row over its CSR entries (lane
// partial sums, then a fixed butterfly); the sign when hard.
__global__ void linear_dot_kernel(const int *__restrict__ rp, const int *__restrict__ ci,
                                  const double *__restrict__ cv, int n, const double *__restrict__ W, int wlen,
                                  double bias, int hard, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        double acc = 0.0;
        for (int p = rp[i] + lane; p < rp[i + 1]; p += 32) {
            const int c = ci[p];
            if (c < wlen) acc = fma(cv[p], W[c], acc);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const double f = bias + acc;
            out[i] = hard ? (f >= 0.0 ? 1.0 : -1.0) : f;
        }
    }
}

}  // namespace

// Prediction of a linear-kernel model through its primal weights
// W = sum_j w_j sv_j: one pass over the support vectors, then one sparse dot
// product per test row (instead of a kernel row sum over all support vectors).
// d_W: scratch of irwls_predict_linear_scratch(S->width, nSV) doubles.
extern "C" size_t irwls_predict_linear_scratch(int width, int nsv) {
    return (size_t)width * (1 + (size_t)ceil_div(std::max(nsv, 1), LW_CHUNK));
}

extern "C" int irwls_predict_linear(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w,
                                    double bias, int hard, double *d_W, double *d_out) {
    if (n <= 0) return 0;
    if (S->mode != IRWLS_K_LINEAR || T->mode != IRWLS_K_LINEAR) {
        irwls_set_error(-4, "the linear prediction path needs a linear-kernel model");
        return -4;
    }
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PREDICT);
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    const int nchunk = ceil_div(std::max(nSV, 1), LW_CHUNK);
    double *part = d_W + S->width;
    linear_w_kernel<<<nchunk, 128, 0, irwls_stream()>>>(S->X, S->ld, nSV, d_w, S->width, part);
    IRWLS_LAUNCH_CHECK("linear_w");
    linear_w_reduce<<<std::max(1, ceil_div(S->width, 128)), 128, 0, irwls_stream()>>>(part, nchunk, S->width, d_W);
    IRWLS_LAUNCH_CHECK("linear_w_reduce");
    linear_dot_kernel<<<std::min(ceil_div(n, 8), 16 * sms), 256, 0, irwls_stream()>>>(T->rp, T->ci, T->cv, n, d_W,
                                                                                     S->width, bias, hard, d_out);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PREDICT);
    IRWLS_LAUNCH_CHECK("linear_dot");
    return 0;
}

extern "C" int irwls_predict_soft(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w,
                                  double bias, int hard, double *d_out) {
    if (n <= 0) return 0;
    fill_kernel<<<ceil_div(n, 256), 256, 0, irwls_stream()>>>(d_out, n, bias);
    IRWLS_LAUNCH_CHECK("fill");
    if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PREDICT);
    int rc = irwls_dev_kernel_rowsum(T, nullptr, n, S, nullptr, nSV, d_w, nullptr, nullptr, 0, +1, d_out, nullptr,
                                     d_out);
    if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PREDICT);
    if (rc) return rc;
    if (hard) {
        sign_kernel<<<ceil_div(n, 256), 256, 0, irwls_stream()>>>(d_out, n);
        IRWLS_LAUNCH_CHECK("sign");
    }
    return 0;
}
