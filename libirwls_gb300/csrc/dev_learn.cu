// dev_learn.cu -- learned-proposal form of SGMA: a small MLP (8 features ->
// 128 -> 128 -> 1, ReLU) scores a large pool of candidates per step, and the
// best 32 of each label go to the exact SGMA score (the reference's step draws
// 64 random candidates of alternating labels, src/budgeted-train.c:149-167).
//
// Features of a candidate c at step s (all cheap, and all relative to the
// current state so that they mean the same at any budget or dataset size):
//   d_c = k(c, c) - |Q_c|^2, the Nystrom residual of c (the exact score's
//         denominator), from the row norms of Q kept by the Q-column update,
//         relative to dbar, the mean residual of the probe rows;
//   rho_c  = mean over probe rows p of k(c, p)          (local density);
//   rhor_c = mean over probe rows p of d_p k(c, p)^2    (unexplained mass
//            near c, a proxy of the exact score's numerator), over dbar;
//   log dbar (the state) and the label.
// The network is trained on traces of the exact scores of random candidates
// (target: log score minus the step's mean log score) by the kernels below:
// layer forward with bias and ReLU fused, the three backward products, an
// MSE gradient and Adam, all FP32 with fixed summation orders. One training
// step is captured once as a CUDA graph and replayed.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "dev_common.cuh"

namespace {

constexpr int LF = 8, LH = 128;
constexpr int P_W1 = 0, P_B1 = P_W1 + LH * LF, P_W2 = P_B1 + LH, P_B2 = P_W2 + LH * LH, P_W3 = P_B2 + LH,
              P_B3 = P_W3 + LH, P_TOTAL = P_B3 + 1;

// ---- features --------------------------------------------------------------

// Features of 32 candidates per CTA (4 per warp): the probe rows are staged
// through shared memory in chunks of PCH rows and shared by the CTA's
// candidates; kernel values in the set's form (raw or norm; RBF only). All
// features are relative to the current state (dbar = mean residual of the
// probes), so that they mean the same at any budget and dataset size.
constexpr int PCH = 128, CPB = 32;
__global__ void __launch_bounds__(256) features_kernel(const float *__restrict__ X, int ld, int width, int raw,
                                                       const float *__restrict__ q, float ng,
                                                       const double *__restrict__ y, const int *__restrict__ cand,
                                                       int nc, const int *__restrict__ probe, int np,
                                                       const float *__restrict__ qn, float *__restrict__ F) {
    extern __shared__ float sm[];
    float *crow = sm;                // [CPB][ld] candidate rows
    float *prow = sm + CPB * ld;     // [PCH][ld] probe rows of the chunk
    float *pd = prow + PCH * ld;     // [PCH] probe residuals
    float *pq = pd + PCH;            // [PCH] probe norms
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = blockIdx.x * CPB;
    for (int t = threadIdx.x; t < CPB * ld; t += blockDim.x) {
        const int j = t / ld, k = t % ld;
        crow[t] = c0 + j < nc ? X[(size_t)cand[c0 + j] * ld + k] : 0.f;
    }
    float rho[4] = {0.f, 0.f, 0.f, 0.f}, rhor[4] = {0.f, 0.f, 0.f, 0.f}, dsum = 0.f;
    for (int p0 = 0; p0 < np; p0 += PCH) {
        const int npc = min(PCH, np - p0);
        __syncthreads();
        for (int t = threadIdx.x; t < npc * ld; t += blockDim.x) {
            const int j = t / ld, k = t % ld;
            prow[t] = X[(size_t)probe[p0 + j] * ld + k];
        }
        for (int j = threadIdx.x; j < npc; j += blockDim.x) {
            pd[j] = fmaxf(1.f - qn[probe[p0 + j]], 0.f);
            pq[j] = q[probe[p0 + j]];
        }
        __syncthreads();
        for (int j = lane; j < npc; j += 32) {
            const float *b = prow + j * ld;
            dsum += pd[j];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int ci = w * 4 + u;
                const float *a = crow + ci * ld;
                float d2;
                if (raw) {
                    d2 = 0.f;
                    for (int t = 0; t < width; ++t) {
                        const float d = a[t] - b[t];
                        d2 = fmaf(d, d, d2);
                    }
                } else {
                    float dot = 0.f;
                    for (int t = 0; t < width; ++t) dot = fmaf(a[t], b[t], dot);
                    const int c = c0 + ci < nc ? cand[c0 + ci] : 0;
                    d2 = fmaxf(q[c] + pq[j] - 2.f * dot, 0.f);
                }
                const float kv = expf(ng * d2);
                rho[u] += kv;
                rhor[u] = fmaf(pd[j] * kv, kv, rhor[u]);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            rho[u] += __shfl_xor_sync(0xffffffffu, rho[u], o);
            rhor[u] += __shfl_xor_sync(0xffffffffu, rhor[u], o);
        }
    }
    if (lane < 4) {
        const int ci = c0 + w * 4 + lane;
        if (ci < nc) {
            const int c = cand[ci];
            float r = rho[0], rr = rhor[0];
            if (lane == 1) { r = rho[1]; rr = rhor[1]; }
            if (lane == 2) { r = rho[2]; rr = rhor[2]; }
            if (lane == 3) { r = rho[3]; rr = rhor[3]; }
            const float dbar = dsum / (float)np + 1e-12f;
            const float dc = fmaxf(1.f - qn[c], 0.f);
            r /= (float)np;
            rr /= (float)np;
            float *f = F + (size_t)ci * LF;
            f[0] = dc / dbar;
            f[1] = logf(dc + 1e-9f) - logf(dbar);
            f[2] = logf(r + 1e-12f);
            f[3] = logf(rr + 1e-12f) - logf(dbar);
            f[4] = rr / (r * dbar + 1e-12f);
            f[5] = logf(dbar);
            f[6] = (float)y[c];
            f[7] = sqrtf(dc / dbar);
        }
    }
}

// ---- MLP layers ------------------------------------------------------------

// Y[n][out] = act(X[n][in] W^T + b) for W [out][in]; 16 rows per CTA, W
// transposed into shared memory.
template <bool RELU>
__global__ void __launch_bounds__(128) mlp_fwd_kernel(const float *__restrict__ X, int n, int in,
                                                      const float *__restrict__ W, const float *__restrict__ b,
                                                      int out, float *__restrict__ Y) {
    extern __shared__ float sm[];
    float *Wt = sm;             // [in][out]
    float *Xs = sm + in * out;  // [16][in]
    const int r0 = blockIdx.x * 16;
    for (int t = threadIdx.x; t < in * out; t += blockDim.x) {
        const int o = t / in, k = t % in;
        Wt[k * out + o] = W[t];
    }
    for (int t = threadIdx.x; t < 16 * in; t += blockDim.x) {
        const int r = t / in, k = t % in;
        Xs[t] = r0 + r < n ? X[(size_t)(r0 + r) * in + k] : 0.f;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < out; o += blockDim.x) {
        for (int r = 0; r < 16 && r0 + r < n; ++r) {
            float acc = b[o];
            for (int k = 0; k < in; ++k) acc = fmaf(Xs[r * in + k], Wt[k * out + o], acc);
            Y[(size_t)(r0 + r) * out + o] = RELU ? fmaxf(acc, 0.f) : acc;
        }
    }
}

// dW[o][k] = sum_r dY[r][o] X[r][k], db[o] = sum_r dY[r][o] (rows in order).
__global__ void mlp_wgrad_kernel(const float *__restrict__ dY, const float *__restrict__ X, int n, int in, int out,
                                 float *__restrict__ dW, float *__restrict__ db) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= out * (in + 1)) return;
    const int o = t / (in + 1), k = t % (in + 1);
    float acc = 0.f;
    if (k < in)
        for (int r = 0; r < n; ++r) acc = fmaf(dY[(size_t)r * out + o], X[(size_t)r * in + k], acc);
    else
        for (int r = 0; r < n; ++r) acc += dY[(size_t)r * out + o];
    if (k < in) dW[o * in + k] = acc;
    else db[o] = acc;
}

// dX[r][k] = (sum_o dY[r][o] W[o][k]) * (A[r][k] > 0), A the layer's input
// activation (the ReLU output of the layer before).
__global__ void mlp_xgrad_kernel(const float *__restrict__ dY, const float *__restrict__ W, int n, int in, int out,
                                 const float *__restrict__ A, float *__restrict__ dX) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * in) return;
    const int r = (int)(t / in), k = (int)(t % in);
    float acc = 0.f;
    for (int o = 0; o < out; ++o) acc = fmaf(dY[(size_t)r * out + o], W[o * in + k], acc);
    dX[t] = A[t] > 0.f ? acc : 0.f;
}

// dP = 2 (P - T) / n and the mean squared error (one CTA, fixed order).
__global__ void __launch_bounds__(256) mse_kernel(const float *__restrict__ P, const float *__restrict__ T, int n,
                                                  float *__restrict__ dP, float *__restrict__ loss) {
    __shared__ float red[256];
    float s = 0.f;
    for (int r = threadIdx.x; r < n; r += 256) {
        const float e = P[r] - T[r];
        dP[r] = 2.f * e / (float)n;
        s = fmaf(e, e, s);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)n;
}

// Adam with bias correction; step[0] is the number of earlier updates
// (advanced by step_kernel after this one).
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, const int *__restrict__ step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int t = step[0] + 1;
    const float mi = b1 * m[i] + (1.f - b1) * g[i];
    const float vi = b2 * v[i] + (1.f - b2) * g[i] * g[i];
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, (float)t)), vh = vi / (1.f - powf(b2, (float)t));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void step_kernel(int *step) { step[0] += 1; }

// Minibatch of the training set: rows perm[(step % nb) * B + r].
__global__ void gather_batch_kernel(const float *__restrict__ Xall, const float *__restrict__ Tall,
                                    const int *__restrict__ perm, int B, int nb, const int *__restrict__ step,
                                    float *__restrict__ Xb, float *__restrict__ Tb) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * LF) return;
    const int r = t / LF, k = t % LF;
    const int src = perm[(step[0] % nb) * B + r];
    Xb[t] = Xall[(size_t)src * LF + k];
    if (k == 0) Tb[r] = Tall[src];
}

// ---- proposals -------------------------------------------------------------

// Per label group g (0: label -1, 1: label +1) of `half` pool entries: the
// `keep` best predictions (ties to the lower pool index) then `nrand` pool
// entries taken in pool order (random draws), written to out[2 j + g] so that
// labels alternate as in the reference's draws.
__global__ void __launch_bounds__(1024) topk_kernel(const float *__restrict__ pred, const int *__restrict__ pool,
                                                    int half, int keep, int nrand, int *__restrict__ out) {
    __shared__ float key[2048];
    __shared__ int idx[2048];
    const int g = blockIdx.x;
    int n2 = 1;
    while (n2 < half) n2 <<= 1;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        key[t] = t < half ? pred[g * half + t] : -INFINITY;
        idx[t] = t;
    }
    __syncthreads();
    // bitonic sort, descending by key, ascending index on ties
    for (int k = 2; k <= n2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = threadIdx.x; t < n2; t += blockDim.x) {
                const int u = t ^ j;
                if (u > t) {
                    const bool before = key[t] > key[u] || (key[t] == key[u] && idx[t] < idx[u]);
                    const bool up = (t & k) == 0;
                    if (up ? !before : before) {
                        const float fk = key[t];
                        key[t] = key[u];
                        key[u] = fk;
                        const int fi = idx[t];
                        idx[t] = idx[u];
                        idx[u] = fi;
                    }
                }
            }
            __syncthreads();
        }
    for (int j = threadIdx.x; j < keep; j += blockDim.x) out[2 * j + g] = pool[g * half + idx[j]];
    for (int j = threadIdx.x; j < nrand; j += blockDim.x) out[2 * (keep + j) + g] = pool[g * half + j];
}

__global__ void residual_trace_kernel(const float *__restrict__ qn, int l, double *out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < l; i += 256) s += (double)fmaxf(1.f - qn[i], 0.f);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

struct Mlp {
    float *p, *g, *m, *v;  // parameters, gradients, Adam moments (P_TOTAL each)
    int *step;
    // forward/backward buffers for up to `cap` rows
    int cap;
    float *X, *T, *A1, *A2, *P, *dP, *dA2, *dA1, *loss;
};

int mlp_reserve(Mlp *M, int n) {
    if (n <= M->cap) return 0;
    float **b[] = {&M->X, &M->T, &M->A1, &M->A2, &M->P, &M->dP, &M->dA2, &M->dA1};
    for (float **q : b) {
        irwls_dev_free(*q);
        *q = nullptr;
    }
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&M->X, (size_t)n * LF * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->T, (size_t)n * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->A1, (size_t)n * LH * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->A2, (size_t)n * LH * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->P, (size_t)n * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->dP, (size_t)n * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->dA2, (size_t)n * LH * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->dA1, (size_t)n * LH * sizeof(float));
    M->cap = rc ? 0 : n;
    return rc;
}

int fwd_smem(int in, int out) { return (in * out + 16 * in) * (int)sizeof(float); }

// Forward of n rows held in M->X into M->P (hidden activations kept).
int mlp_forward(Mlp *M, const float *X, int n, float *P) {
    cudaStream_t st = irwls_stream();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(mlp_fwd_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_smem(LH, LH));
        cudaFuncSetAttribute(mlp_fwd_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_smem(LH, LH));
        attr = true;
    }
    const int g = ceil_div(n, 16);
    mlp_fwd_kernel<true><<<g, 128, fwd_smem(LF, LH), st>>>(X, n, LF, M->p + P_W1, M->p + P_B1, LH, M->A1);
    IRWLS_LAUNCH_CHECK("mlp_fwd1");
    mlp_fwd_kernel<true><<<g, 128, fwd_smem(LH, LH), st>>>(M->A1, n, LH, M->p + P_W2, M->p + P_B2, LH, M->A2);
    IRWLS_LAUNCH_CHECK("mlp_fwd2");
    mlp_fwd_kernel<false><<<g, 128, fwd_smem(LH, 1), st>>>(M->A2, n, LH, M->p + P_W3, M->p + P_B3, 1, P);
    IRWLS_LAUNCH_CHECK("mlp_fwd3");
    return 0;
}

// Loss gradient of n rows (X in M->X, T in M->T) into M->g.
int mlp_backward(Mlp *M, int n) {
    cudaStream_t st = irwls_stream();
    if (mlp_forward(M, M->X, n, M->P)) return -1;
    mse_kernel<<<1, 256, 0, st>>>(M->P, M->T, n, M->dP, M->loss);
    IRWLS_LAUNCH_CHECK("mse");
    mlp_wgrad_kernel<<<ceil_div(1 * (LH + 1), 128), 128, 0, st>>>(M->dP, M->A2, n, LH, 1, M->g + P_W3, M->g + P_B3);
    IRWLS_LAUNCH_CHECK("wgrad3");
    mlp_xgrad_kernel<<<ceil_div((long long)n * LH, 256), 256, 0, st>>>(M->dP, M->p + P_W3, n, LH, 1, M->A2, M->dA2);
    IRWLS_LAUNCH_CHECK("xgrad3");
    mlp_wgrad_kernel<<<ceil_div(LH * (LH + 1), 128), 128, 0, st>>>(M->dA2, M->A1, n, LH, LH, M->g + P_W2,
                                                                    M->g + P_B2);
    IRWLS_LAUNCH_CHECK("wgrad2");
    mlp_xgrad_kernel<<<ceil_div((long long)n * LH, 256), 256, 0, st>>>(M->dA2, M->p + P_W2, n, LH, LH, M->A1,
                                                                       M->dA1);
    IRWLS_LAUNCH_CHECK("xgrad2");
    mlp_wgrad_kernel<<<ceil_div(LH * (LF + 1), 128), 128, 0, st>>>(M->dA1, M->X, n, LF, LH, M->g + P_W1, M->g + P_B1);
    IRWLS_LAUNCH_CHECK("wgrad1");
    return 0;
}

unsigned lcg(unsigned &s) {
    s = s * 1664525u + 1013904223u;
    return s;
}

}  // namespace

extern "C" int irwls_mlp_param_count(void) { return P_TOTAL; }
extern "C" int irwls_mlp_feature_count(void) { return LF; }

// He-initialised network (weights N(0, 2 / fan_in) from a seeded Box-Muller
// stream, zero biases).
extern "C" void *irwls_mlp_create(unsigned seed) {
    if (irwls_dev_init()) return nullptr;
    Mlp *M = (Mlp *)calloc(1, sizeof(Mlp));
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&M->p, P_TOTAL * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->g, P_TOTAL * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->m, P_TOTAL * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->v, P_TOTAL * sizeof(float));
    rc |= irwls_dev_malloc((void **)&M->step, sizeof(int));
    rc |= irwls_dev_malloc((void **)&M->loss, sizeof(float));
    if (rc) {
        free(M);
        return nullptr;
    }
    std::vector<float> h(P_TOTAL, 0.f);
    unsigned s = seed * 2654435761u + 12345u;
    auto normal = [&]() {
        const double u1 = (lcg(s) + 1.0) / 4294967297.0, u2 = (lcg(s) + 1.0) / 4294967297.0;
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    };
    for (int i = 0; i < LH * LF; ++i) h[P_W1 + i] = (float)(normal() * sqrt(2.0 / LF));
    for (int i = 0; i < LH * LH; ++i) h[P_W2 + i] = (float)(normal() * sqrt(2.0 / LH));
    for (int i = 0; i < LH; ++i) h[P_W3 + i] = (float)(normal() * sqrt(2.0 / LH));
    rc |= irwls_dev_h2d(M->p, h.data(), P_TOTAL * sizeof(float));
    rc |= irwls_dev_memset(M->m, 0, P_TOTAL * sizeof(float));
    rc |= irwls_dev_memset(M->v, 0, P_TOTAL * sizeof(float));
    rc |= irwls_dev_memset(M->step, 0, sizeof(int));
    rc |= irwls_dev_sync();
    if (rc) return nullptr;
    return M;
}

extern "C" void irwls_mlp_free(void *h) {
    Mlp *M = (Mlp *)h;
    if (!M) return;
    void *b[] = {M->p, M->g, M->m, M->v, M->step, M->loss, M->X, M->T, M->A1, M->A2, M->P, M->dP, M->dA2, M->dA1};
    for (void *q : b) irwls_dev_free(q);
    irwls_dev_sync();
    free(M);
}

extern "C" int irwls_mlp_get_params(void *h, float *out) {
    Mlp *M = (Mlp *)h;
    if (irwls_dev_d2h(out, M->p, P_TOTAL * sizeof(float))) return -1;
    return irwls_dev_sync();
}

extern "C" int irwls_mlp_set_params(void *h, const float *in) {
    Mlp *M = (Mlp *)h;
    if (irwls_dev_h2d(M->p, in, P_TOTAL * sizeof(float))) return -1;
    return irwls_dev_sync();
}

// Mean squared error and its gradient (parameter layout) for n host rows.
extern "C" double irwls_mlp_loss_grad(void *h, const float *X, const float *T, int n, float *grad) {
    Mlp *M = (Mlp *)h;
    if (n <= 0 || mlp_reserve(M, n)) return -1.0;
    float loss = 0.f;
    if (irwls_dev_h2d(M->X, X, (size_t)n * LF * sizeof(float)) || irwls_dev_h2d(M->T, T, (size_t)n * sizeof(float)) ||
        mlp_backward(M, n) || irwls_dev_d2h(grad, M->g, P_TOTAL * sizeof(float)) ||
        irwls_dev_d2h(&loss, M->loss, sizeof(float)) || irwls_dev_sync())
        return -1.0;
    return loss;
}

extern "C" int irwls_mlp_predict_host(void *h, const float *X, int n, float *out) {
    Mlp *M = (Mlp *)h;
    if (n <= 0) return 0;
    if (mlp_reserve(M, n)) return -1;
    if (irwls_dev_h2d(M->X, X, (size_t)n * LF * sizeof(float)) || mlp_forward(M, M->X, n, M->P) ||
        irwls_dev_d2h(out, M->P, (size_t)n * sizeof(float)) || irwls_dev_sync())
        return -1;
    return 0;
}

// Adam on minibatches of `batch` rows of the host training set, `epochs`
// passes, each over a fresh seeded permutation; one training step is a CUDA
// graph (batch gather, forward, loss, backward, update, step count) captured
// once and replayed. Returns the mean loss of the last epoch.
extern "C" double irwls_mlp_train(void *h, const float *X, const float *T, int n, int epochs, int batch, float lr,
                                  unsigned seed) {
    Mlp *M = (Mlp *)h;
    const int B = std::max(1, std::min(batch, n));
    const int nb = n / B;
    if (nb <= 0 || mlp_reserve(M, B)) return -1.0;
    float *dX = nullptr, *dT = nullptr, *losses = nullptr;
    int *perm = nullptr;
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&dX, (size_t)n * LF * sizeof(float));
    rc |= irwls_dev_malloc((void **)&dT, (size_t)n * sizeof(float));
    rc |= irwls_dev_malloc((void **)&perm, (size_t)nb * B * sizeof(int));
    rc |= irwls_dev_malloc((void **)&losses, (size_t)nb * sizeof(float));
    if (rc) return -1.0;
    rc |= irwls_dev_h2d(dX, X, (size_t)n * LF * sizeof(float));
    rc |= irwls_dev_h2d(dT, T, (size_t)n * sizeof(float));
    rc |= irwls_dev_memset(M->step, 0, sizeof(int));
    rc |= irwls_dev_sync();
    // kernel attributes before capture
    mlp_forward(M, M->X, 1, M->P);
    rc |= irwls_dev_sync();
    cudaStream_t st = irwls_stream();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (!rc && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        gather_batch_kernel<<<ceil_div(B * LF, 256), 256, 0, st>>>(dX, dT, perm, B, nb, M->step, M->X, M->T);
        mlp_backward(M, B);
        adam_kernel<<<ceil_div(P_TOTAL, 256), 256, 0, st>>>(M->p, M->g, M->m, M->v, P_TOTAL, lr, M->step);
        step_kernel<<<1, 1, 0, st>>>(M->step);
        if (cudaStreamEndCapture(st, &graph) != cudaSuccess ||
            cudaGraphInstantiate(&exec, graph, nullptr, nullptr, 0) != cudaSuccess)
            rc = -1;
    } else {
        rc = -1;
    }
    std::vector<int> hp((size_t)nb * B);
    std::vector<float> hl(nb);
    double last = -1.0;
    unsigned s = seed;
    for (int e = 0; e < epochs && !rc; ++e) {
        std::vector<int> all(n);
        for (int i = 0; i < n; ++i) all[i] = i;
        for (int i = n - 1; i > 0; --i) std::swap(all[i], all[lcg(s) % (unsigned)(i + 1)]);
        for (int i = 0; i < nb * B; ++i) hp[i] = all[i];
        rc |= irwls_dev_h2d(perm, hp.data(), (size_t)nb * B * sizeof(int));
        for (int k = 0; k < nb && !rc; ++k) {
            if (cudaGraphLaunch(exec, st) != cudaSuccess) rc = -1;
            irwls_count_launch(12);
            cudaMemcpyAsync(losses + k, M->loss, sizeof(float), cudaMemcpyDeviceToDevice, st);
        }
        rc |= irwls_dev_d2h(hl.data(), losses, (size_t)nb * sizeof(float));
        rc |= irwls_dev_sync();
        double sum = 0.0;
        for (float v : hl) sum += v;
        last = sum / nb;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    void *b[] = {dX, dT, perm, losses};
    for (void *q : b) irwls_dev_free(q);
    irwls_dev_sync();
    return rc ? -1.0 : last;
}

// ---- device entry points used by the SGMA step (mixed.c) --------------------

extern "C" int irwls_learn_features(const float *X, int ld, int width, int raw, const float *q, float ng,
                                    const double *y, const int *d_cand, int nc, const int *d_probe, int np,
                                    const float *d_qn, float *d_F) {
    const int smem = ((CPB + PCH) * ld + 2 * PCH) * (int)sizeof(float);
    if (smem > 220 * 1024) {
        irwls_set_error(-12, "feature width %d too wide for the proposal features", width);
        return -12;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    features_kernel<<<ceil_div(nc, CPB), 256, smem, irwls_stream()>>>(X, ld, width, raw, q, ng, y, d_cand, nc,
                                                                      d_probe, np, d_qn, d_F);
    IRWLS_LAUNCH_CHECK("learn_features");
    return 0;
}

extern "C" int irwls_learn_predict(void *h, const float *d_F, int n, float *d_pred) {
    Mlp *M = (Mlp *)h;
    if (mlp_reserve(M, n)) return -1;
    return mlp_forward(M, d_F, n, d_pred);
}

extern "C" int irwls_learn_topk(const float *d_pred, const int *d_pool, int half, int keep, int nrand, int *d_out) {
    if (half > 2048 || keep > half || nrand > half) {
        irwls_set_error(-12, "proposal pool of %d per label (at most 2048) keeping %d + %d", half, keep, nrand);
        return -12;
    }
    topk_kernel<<<2, 1024, 0, irwls_stream()>>>(d_pred, d_pool, half, keep, nrand, d_out);
    IRWLS_LAUNCH_CHECK("learn_topk");
    return 0;
}

extern "C" int irwls_learn_residual_trace(const float *d_qn, int l, double *d_out) {
    residual_trace_kernel<<<1, 256, 0, irwls_stream()>>>(d_qn, l, d_out);
    IRWLS_LAUNCH_CHECK("residual_trace");
    return 0;
}
