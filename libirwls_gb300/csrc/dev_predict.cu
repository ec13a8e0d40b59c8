// dev_predict.cu -- batched prediction f(x_i) = bias + sum_j w_j k(x_i, sv_j)
// (reference src/LIBIRWLS-predict.c:56-131): an ordered kernel row sum, so
// every decision value accumulates its support vectors in the reference's
// order; the sign is taken on the device.
#include "dev_common.cuh"

namespace {

__global__ void fill_kernel(double *p, int n, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

__global__ void sign_kernel(double *p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = (p[i] >= 0.0) ? 1.0 : -1.0;
}

}  // namespace

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
