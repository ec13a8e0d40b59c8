// dev_full.cu -- device steps of full IRWLS (reference src/full-train.c).
//
// The O(w) and O(l) bookkeeping (a_i weights, groups, list compaction,
// classification into working/inactive/candidate sets, convergence sums) runs
// in single-CTA kernels whose list orders and summation orders are the
// reference's: lists come out in ascending sample order, and the sums that
// feed convergence tests are accumulated left to right by one thread.
// Kernel tiles and solves are in dev_tiles.cu and dev_chol.cu.
#include <string.h>

#include <algorithm>
#include <atomic>

#include "dev_common.cuh"
#include "irwls_gpu.h"

// Working-set solves of the precision form: by the cluster solve, and
// handed to the FP64 factorization although their order fitted the cluster.
static std::atomic<long long> g_ws_mixed_solves{0}, g_ws_mixed_fallbacks{0};

extern "C" void irwls_ws_mixed_counts(long long *solves, long long *fallbacks, int reset) {
    if (solves) *solves = g_ws_mixed_solves.load();
    if (fallbacks) *fallbacks = g_ws_mixed_fallbacks.load();
    if (reset) {
        g_ws_mixed_solves = 0;
        g_ws_mixed_fallbacks = 0;
    }
}

namespace {

constexpr int CT = 1024;  // threads of the single-CTA bookkeeping kernels

// Exclusive scan of per-thread counts in shared memory; returns the total.
__device__ int block_exclusive_scan(int *s, int v) {
    const int t = threadIdx.x;
    s[t] = v;
    __syncthreads();
    for (int o = 1; o < CT; o <<= 1) {
        int x = (t >= o) ? s[t - o] : 0;
        __syncthreads();
        s[t] += x;
        __syncthreads();
    }
    const int incl = s[t];
    const int total = s[CT - 1];
    __syncthreads();
    s[t] = incl - v;
    __syncthreads();
    return total;
}

// Ordered compaction: writes, in ascending i, every i < n with pred(i) to
// out (through emit(pos, i)); returns the count (same in every thread).
template <class Pred, class Emit>
__device__ int block_compact(int n, Pred pred, Emit emit, int *s_scan) {
    const int ch = (n + CT - 1) / CT;
    const int b = threadIdx.x * ch, e = min(n, b + ch);
    int c = 0;
    for (int i = b; i < e; ++i) c += pred(i) ? 1 : 0;
    const int total = block_exclusive_scan(s_scan, c);
    int off = s_scan[threadIdx.x];
    for (int i = b; i < e; ++i)
        if (pred(i)) emit(off++, i);
    __syncthreads();
    return total;
}

// Deterministic CTA-wide sum of f(i), i < n: each thread adds its contiguous
// chunk left to right, then a fixed tree combines the threads. The result is
// returned to every thread.
template <class F>
__device__ double block_sum_ordered(int n, F f, double *red) {
    const int ch = (n + CT - 1) / CT;
    const int b = threadIdx.x * ch, e = min(n, b + ch);
    double v = 0.0;
    for (int i = b; i < e; ++i) v = __dadd_rn(v, f(i));
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = red[lane];
        for (int o = 16; o > 0; o >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

template <class F, class Op>
__device__ double block_reduce(int n, F f, Op op, double init, double *red) {
    double v = init;
    for (int i = threadIdx.x; i < n; i += CT) v = op(v, f(i));
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = red[lane];
        for (int o = 16; o > 0; o >>= 1) t = op(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

// --- inner IRWLS -----------------------------------------------------------

// a_i and groups at entry (src/full-train.c:131-155).
__global__ void __launch_bounds__(CT) sub_init_kernel(irwls_sub_ws ws, const double *__restrict__ yg, double C) {
    __shared__ int s_scan[CT];
    const int w = ws.w;
    for (int i = threadIdx.x; i < w; i += CT) {
        const double yi = yg[ws.map[i]];
        ws.y[i] = yi;
        const double ei = ws.e[i];
        const double ai = (ei * yi < 0) ? 0.0 : __ddiv_rn(__dmul_rn(1.0 * yi, C), ei);
        ws.a[i] = ai;
        ws.grp[i] = (ai == 0) ? 2 : ((ws.beta[i] == __dmul_rn(yi, C)) ? 3 : 1);
    }
    for (int i = threadIdx.x; i <= w; i += CT) ws.G13[i] = 0.0;
    __syncthreads();
    const int n1 = block_compact(w, [&](int i) { return ws.grp[i] == 1; },
                                 [&](int p, int i) { ws.S1[p] = i; ws.gl1[p] = ws.map[i]; }, s_scan);
    const int n3 = block_compact(w, [&](int i) { return ws.grp[i] == 3; },
                                 [&](int p, int i) { ws.S3[p] = i; ws.gl3[p] = ws.map[i]; }, s_scan);
    if (threadIdx.x == 0) {
        ws.stats->nS1 = n1;
        ws.stats->nS3 = n3;
        ws.stats->dW = 1e9;
        ws.stats->nW = 1.0;
        ws.stats->bmax = 0.0;
        ws.stats->bmin = 0.0;
    }
}

// H and its right-hand side (src/full-train.c:165-186). H is column-major
// with leading dimension ldH; only the lower triangle is read by the solver.
// grid: (ceil(n1 / 64), n1): CTA (bx, i) fills row i, columns bx*64 .. of the
// lower part; the A row (S1_i) is staged in shared memory.
__global__ void __launch_bounds__(64) build_H_kernel(irwls_sub_ws ws, KView X, int n1) {
    extern __shared__ double sA[];
    const int i = blockIdx.y;
    const int gi = ws.map[ws.S1[i]];
    for (int t = threadIdx.x; t < X.ld; t += 64) sA[t] = X.X[(size_t)gi * X.ld + t];
    __syncthreads();
    const double qa = X.q[gi];
    const double yi = ws.y[ws.S1[i]];
    const int j = blockIdx.x * 64 + threadIdx.x;
    if (j > i) return;
    const int lj = ws.S1[j];
    const double kv = kentry(X, sA, qa, ws.map[lj]);
    double h = __dmul_rn(__dmul_rn(kv, yi), ws.y[lj]);
    if (i == j) h = __dadd_rn(h, __ddiv_rn(1.0, ws.a[ws.S1[i]]));
    ws.H[(size_t)j * ws.ldH + i] = h;
}

// The diagonal's 1 / a_i after an exact-mode kernel block (the same
// operations as build_H_kernel's diagonal).
__global__ void build_H_diag_kernel(irwls_sub_ws ws, int n1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1) {
        double *h = ws.H + (size_t)i * ws.ldH + i;
        *h = __dadd_rn(*h, __ddiv_rn(1.0, ws.a[ws.S1[i]]));
    }
}

__global__ void build_border_kernel(irwls_sub_ws ws, int n1) {
    const int w = ws.w;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n1; i += gridDim.x * blockDim.x) {
        if (i < n1) {
            const int li = ws.S1[i];
            ws.H[(size_t)i * ws.ldH + n1] = ws.y[li];  // row n1, column i
            ws.rhs[i] = __dsub_rn(__dsub_rn(1.0, ws.G13[i]), ws.GIN[li]);
        } else {
            ws.H[(size_t)n1 * ws.ldH + n1] = 0.0;
            ws.rhs[n1] = __dsub_rn(-ws.G13[n1], ws.GIN[w]);
        }
    }
}

// New weights, convergence sums and the list of changed weights
// (src/full-train.c:205-230 and the skip test of :242).
__global__ void __launch_bounds__(CT) sub_update_kernel(irwls_sub_ws ws, double C, int n1, int n3) {
    __shared__ int s_scan[CT];
    const int w = ws.w;
    for (int i = threadIdx.x; i <= w; i += CT) ws.bnew[i] = 0.0;
    __syncthreads();
    for (int i = threadIdx.x; i < n1; i += CT) ws.bnew[ws.S1[i]] = __dmul_rn(ws.bsol[i], ws.y[ws.S1[i]]);
    for (int i = threadIdx.x; i < n3; i += CT) ws.bnew[ws.S3[i]] = __dmul_rn(C, ws.y[ws.S3[i]]);
    if (threadIdx.x == 0) ws.bnew[w] = ws.bsol[n1];
    __syncthreads();
    __shared__ double red[33];
    const double bmax = block_reduce(n1, [&](int i) { return ws.bsol[i]; },
                                     [](double a, double b) { return b > a ? b : a; }, 0.0, red);
    const double bmin = block_reduce(n1, [&](int i) { return ws.bsol[i]; },
                                     [](double a, double b) { return b < a ? b : a; }, 0.0, red);
    const double dW = block_sum_ordered(w + 1, [&](int i) {
        const double d = __dsub_rn(ws.bnew[i], ws.beta[i]);
        return __dmul_rn(d, d);
    }, red);
    const double nW = block_sum_ordered(w + 1, [&](int i) { return __dmul_rn(ws.beta[i], ws.beta[i]); }, red);
    if (threadIdx.x == 0) {
        ws.stats->bmax = bmax;
        ws.stats->bmin = bmin;
        ws.stats->dW = dW;
        ws.stats->nW = nW;
        ws.scal[0] = __dsub_rn(ws.bnew[w], ws.beta[w]);
    }
    const int nl = block_compact(w, [&](int j) { return ws.bnew[j] != ws.beta[j]; },
                                 [&](int p, int j) {
                                     ws.lst[p] = ws.map[j];
                                     ws.dlt[p] = __dsub_rn(ws.bnew[j], ws.beta[j]);
                                 },
                                 s_scan);
    if (threadIdx.x == 0) ws.cnt[0] = nl;
}

// a_i, groups, beta <- bnew, S1/S3 lists, G13[n1] (src/full-train.c:264-344).
__global__ void __launch_bounds__(CT) sub_groups_kernel(irwls_sub_ws ws, double C) {
    __shared__ int s_scan[CT];
    const int w = ws.w;
    for (int i = threadIdx.x; i < w; i += CT) {
        const double yi = ws.y[i], ei = ws.e[i];
        const double ey = __dmul_rn(ei, yi);
        double ai;
        if (ey < 0.0) ai = 0.0;
        else if (ey < (1.0 / 10000)) ai = __dmul_rn(C, 10000.0);
        else ai = __ddiv_rn(__dmul_rn(1.0 * yi, C), ei);
        ws.a[i] = ai;
        int g = ws.grp[i];
        if (ey < 0.0 && g != 2) g = 2;
        const double by = __dmul_rn(yi, ws.bnew[i]);
        if (g == 1 && by >= __dmul_rn(0.99, C) && by <= __dmul_rn(1.01, C)) g = 3;
        if (ai == 0.0 && g == 1) g = 2;
        if (g == 2 && ai != 0.0) g = 1;
        ws.grp[i] = g;
        ws.beta[i] = ws.bnew[i];
    }
    if (threadIdx.x == 0) ws.beta[w] = ws.bnew[w];
    __syncthreads();
    const int n1 = block_compact(w, [&](int i) { return ws.grp[i] == 1; },
                                 [&](int p, int i) {
                                     ws.S1[p] = i;
                                     ws.gl1[p] = ws.map[i];
                                 },
                                 s_scan);
    const int n3 = block_compact(w, [&](int i) { return ws.grp[i] == 3; },
                                 [&](int p, int i) {
                                     ws.S3[p] = i;
                                     ws.gl3[p] = ws.map[i];
                                     ws.rhs[p] = C;
                                 },
                                 s_scan);
    for (int i = threadIdx.x; i <= n1; i += CT) ws.G13[i] = 0.0;
    __syncthreads();
    __shared__ double red[33];
    const double g13 = block_sum_ordered(n3, [&](int o) { return __dmul_rn(ws.rhs[o], ws.y[ws.S3[o]]); }, red);
    if (threadIdx.x == 0) {
        if (n3 > 0) ws.G13[n1] = g13;
        ws.stats->nS1 = n1;
        ws.stats->nS3 = n3;
    }
}

// --- outer loop --------------------------------------------------------------

// Inactive samples with a non-zero weight, their weights, and GIN[nSW] =
// sum of the weights of every inactive sample (src/full-train.c:436-456).
__global__ void gather_ws_kernel(const int *__restrict__ SW, int nSW, const double *__restrict__ e,
                                 const double *__restrict__ beta, int l, double *esub, double *bsub) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nSW; i += gridDim.x * blockDim.x) {
        if (i < nSW) {
            esub[i] = e[SW[i]];
            bsub[i] = beta[SW[i]];
        } else {
            bsub[nSW] = beta[l];
        }
    }
}

// betaNew over the working set, the changed entries and the bias change
// (src/full-train.c:488-510).
__global__ void __launch_bounds__(CT) apply_ws_kernel(const int *__restrict__ SW, int nSW,
                                                      const double *__restrict__ bt, const double *__restrict__ beta,
                                                      int l, double *bnew, int *lst, double *cb, int *cnt,
                                                      double *dbias) {
    __shared__ int s_scan[CT];
    for (int i = threadIdx.x; i < nSW; i += CT) bnew[SW[i]] = bt[i];
    if (threadIdx.x == 0) {
        bnew[l] = bt[nSW];
        dbias[0] = __dsub_rn(bt[nSW], beta[l]);
    }
    __syncthreads();
    const int n = block_compact(nSW, [&](int j) { return bnew[SW[j]] != beta[SW[j]]; },
                                [&](int p, int j) {
                                    lst[p] = SW[j];
                                    cb[p] = __dsub_rn(bnew[SW[j]], beta[SW[j]]);
                                },
                                s_scan);
    if (threadIdx.x == 0) cnt[0] = n;
    // sum |beta change| (the precision form's error bound of this update)
    __shared__ double red[33];
    const double l1 = block_sum_ordered(n, [&](int p) { return fabs(cb[p]); }, red);
    if (threadIdx.x == 0) dbias[1] = l1;
}

// ---- ordered reductions of the outer loop over many CTAs --------------------
// block_sum_ordered splits [0, n) into CT chunks of ch = ceil(n / CT) (thread
// t: [t ch, min(n, (t + 1) ch))), sums each left to right, then combines the
// chunk sums by fixed shuffle trees. The chunk passes below compute the same
// chunk sums on CT threads spread over CT / PC CTAs (on one SM the FP64 pipe
// made these sums take 150 us); the final pass runs the same trees on one CTA
// of CT threads. The results are the single-CTA kernels' bits.
constexpr int PC = 128;  // threads per CTA of the chunk passes

__device__ double chunk_tree_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = red[lane];
        for (int o = 16; o > 0; o >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

// dW = sum (beta - bnew)^2 and nW = sum beta^2 (src/full-train.c:512-520).
__global__ void __launch_bounds__(PC) norms_chunk_kernel(const double *__restrict__ beta,
                                                         const double *__restrict__ bnew, int n, double *part) {
    const int t = blockIdx.x * PC + threadIdx.x, ch = (n + CT - 1) / CT, b = t * ch, e = min(n, b + ch);
    double v1 = 0.0, v2 = 0.0;
    for (int i = b; i < e; ++i) {
        const double d = __dsub_rn(beta[i], bnew[i]);
        v1 = __dadd_rn(v1, __dmul_rn(d, d));
        v2 = __dadd_rn(v2, __dmul_rn(beta[i], beta[i]));
    }
    part[t] = v1;
    part[CT + t] = v2;
}

__global__ void __launch_bounds__(CT) norms_final_kernel(const double *__restrict__ part, double *out2) {
    __shared__ double red[33];
    const double dW = chunk_tree_sum(part[threadIdx.x], red);
    const double nW = chunk_tree_sum(part[CT + threadIdx.x], red);
    if (threadIdx.x == 0) {
        out2[0] = dW;
        out2[1] = nW;
    }
}

// GIN's list (src/full-train.c:436-456): the entries of SIN with bnew != 0
// in ascending order with their weights, and GIN[nSW] = sum over SIN of bnew.
// Pass 1 counts and sums each chunk, pass 2 scans the counts and combines
// the sums, pass 3 writes each chunk's entries at its offset.
__global__ void __launch_bounds__(PC) gin_chunk_kernel(const int *__restrict__ SIN, int nSIN,
                                                       const double *__restrict__ bnew, int *ccount, double *csum) {
    const int t = blockIdx.x * PC + threadIdx.x, ch = (nSIN + CT - 1) / CT, b = t * ch, e = min(nSIN, b + ch);
    int c = 0;
    double v = 0.0;
    for (int o = b; o < e; ++o) {
        const double w = bnew[SIN[o]];
        c += w != 0.0 ? 1 : 0;
        v = __dadd_rn(v, w);
    }
    ccount[t] = c;
    csum[t] = v;
}

__global__ void __launch_bounds__(CT) gin_scan_kernel(int *ccount, const double *__restrict__ csum, int *cnt,
                                                      double *GIN, int nSW) {
    __shared__ int s_scan[CT];
    __shared__ double red[33];
    const int total = block_exclusive_scan(s_scan, ccount[threadIdx.x]);
    ccount[threadIdx.x] = s_scan[threadIdx.x];  // now the chunk's offset
    const double g = chunk_tree_sum(csum[threadIdx.x], red);
    if (threadIdx.x == 0) {
        cnt[0] = total;
        GIN[nSW] = g;
    }
}

__global__ void __launch_bounds__(PC) gin_write_kernel(const int *__restrict__ SIN, int nSIN,
                                                       const double *__restrict__ bnew,
                                                       const int *__restrict__ coffset, int *lst, double *cb) {
    const int t = blockIdx.x * PC + threadIdx.x, ch = (nSIN + CT - 1) / CT, b = t * ch, e = min(nSIN, b + ch);
    int off = coffset[t];
    for (int o = b; o < e; ++o) {
        const double w = bnew[SIN[o]];
        if (w != 0.0) {
            lst[off] = SIN[o];
            cb[off] = w;
            ++off;
        }
    }
}

// Classification of every sample after an outer iteration
// (src/full-train.c:540-615): the first violator of each (kind, label) slot
// joins the working set, other violators and all free weights become
// candidates, the rest stay inactive.
__device__ __forceinline__ int classify_one(double bi, double ei, double yi, double C, int *slot) {
    // returns 0: inactive, 1: candidate, 2: violator (slot set), -1: none
    const double thr = 0.001;
    const double by = __dmul_rn(bi, yi);
    int kind;
    bool viol;
    if (by == C) {
        kind = 0;
        viol = __dmul_rn(ei, yi) < -1.0 * thr;
        if (!viol) return 0;
    } else if (bi == 0.0) {
        kind = 1;
        viol = __dmul_rn(ei, yi) > thr;
        if (!viol) return 0;
    } else if (by != 0.0 && by != C) {
        kind = 2;
        viol = fabs(__dmul_rn(ei, yi)) > thr;
        if (!viol) return 1;
    } else {
        return -1;
    }
    *slot = (yi == -1) ? 2 * kind : ((yi == 1) ? 2 * kind + 1 : -1);
    return 2;
}

__global__ void __launch_bounds__(CT) classify_kernel(const double *__restrict__ bnew, const double *__restrict__ e,
                                                      const double *__restrict__ y, int l, double C, int *SW,
                                                      int *SC, int *SIN, irwls_outer_counts *counts) {
    __shared__ int s_scan[CT];
    __shared__ int first[6];
    if (threadIdx.x < 6) first[threadIdx.x] = 0x7fffffff;
    __syncthreads();
    for (int i = threadIdx.x; i < l; i += CT) {
        int slot = -1;
        if (classify_one(bnew[i], e[i], y[i], C, &slot) == 2 && slot >= 0) atomicMin(&first[slot], i);
    }
    __syncthreads();
    auto cat = [&](int i) {
        int slot = -1;
        const int c = classify_one(bnew[i], e[i], y[i], C, &slot);
        if (c == 2) return (slot >= 0 && first[slot] == i) ? 2 : 1;
        return c;  // 0 inactive, 1 candidate, -1 none
    };
    const int nsw = block_compact(l, [&](int i) { return cat(i) == 2; }, [&](int p, int i) { SW[p] = i; }, s_scan);
    const int nsc = block_compact(l, [&](int i) { return cat(i) == 1; }, [&](int p, int i) { SC[p] = i; }, s_scan);
    const int nin = block_compact(l, [&](int i) { return cat(i) == 0; }, [&](int p, int i) { SIN[p] = i; }, s_scan);
    if (threadIdx.x == 0) {
        counts->nSW = nsw;
        counts->nSC = nsc;
        counts->nSIN = nin;
    }
}

__global__ void fill_ws_kernel(int *SW, int nSW, int *SIN, int nSIN, const int *__restrict__ SC, int nSC,
                               const int *__restrict__ perm, int space) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nSC; i += gridDim.x * blockDim.x) {
        const int v = SC[perm ? perm[i] : i];
        if (i < space) SW[nSW + i] = v;
        else SIN[nSIN + (i - space)] = v;
    }
}


__global__ void gather_kernel(const double *__restrict__ src, const int *__restrict__ idx, int n,
                              double *__restrict__ dst) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = src[idx[k]];
}

__global__ void scatter_kernel(const double *__restrict__ src, const int *__restrict__ idx, int n,
                               double *__restrict__ dst) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[idx[k]] = src[k];
}

// Precision form: the support vectors (beta != 0 over the l samples) as a
// compact list with their weights, in index order.
__global__ void __launch_bounds__(CT) sv_list_kernel(const double *__restrict__ beta, int l, int *lst, double *cb,
                                                     int *cnt) {
    __shared__ int s_scan[CT];
    const int n = block_compact(l, [&](int i) { return beta[i] != 0.0; },
                                [&](int p, int i) {
                                    lst[p] = i;
                                    cb[p] = beta[i];
                                },
                                s_scan);
    if (threadIdx.x == 0) cnt[0] = n;
}

// ---- multi-block ordered compactions over all l rows ------------------------
//
// The outer classification and the precision form's exact set each split l
// rows into ordered lists. One CTA walking 100000 rows evaluated every row's
// FP64 tests several times on one SM (about 1 ms per call); here every row's
// list is decided once, by all SMs, and the lists are written in ascending
// row order by blocks of CB rows: a count pass per block, then a write pass
// in which each block adds the counts of the blocks before it and places its
// rows round by round with warp-ballot prefixes. The lists are the
// single-CTA kernels' lists, element for element.
constexpr int CB = 2048;

__device__ __forceinline__ int bsum256(int v, int *ws) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int k = 0; k < 8; ++k) t += ws[k];
    __syncthreads();
    return t;
}

// Writes the rows of one round (256 consecutive rows) that belong to list k
// (member[k]) at base[k] + their rank among the round's members, in row
// order; advances base[k] by the round's members. 256 threads.
template <int NL>
__device__ __forceinline__ void ordered_round(const bool (&member)[NL], int i, int *base, int *const (&out)[NL],
                                              int (*ws)[8]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned bal[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) {
        bal[k] = __ballot_sync(0xffffffffu, member[k]);
        if (lane == 0) ws[k][warp] = __popc(bal[k]);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NL; ++k) {
        int off = 0, tot = 0;
        for (int w = 0; w < 8; ++w) {
            off += w < warp ? ws[k][w] : 0;
            tot += ws[k][w];
        }
        if (member[k] && out[k]) out[k][base[k] + off + __popc(bal[k] & ((1u << lane) - 1u))] = i;
        base[k] += tot;
    }
    __syncthreads();
}

// Classification codes: 0 inactive, 1 candidate, 2 + slot a violator of
// type slot (its list is decided by first[slot]), 255 none.
__global__ void classify_code_kernel(const double *__restrict__ bnew, const double *__restrict__ e,
                                     const double *__restrict__ y, int l, double C, unsigned char *__restrict__ code,
                                     int *__restrict__ first) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l; i += gridDim.x * blockDim.x) {
        int slot = -1;
        const int c = classify_one(bnew[i], e[i], y[i], C, &slot);
        unsigned char v = 255;
        if (c == 2 && slot >= 0) {
            v = (unsigned char)(2 + slot);
            atomicMin(first + slot, i);
        } else if (c == 2 || c == 1) {
            v = 1;
        } else if (c == 0) {
            v = 0;
        }
        code[i] = v;
    }
}

// list of row i: 0 SW, 1 SC, 2 SIN, -1 none
__device__ __forceinline__ int classify_list(unsigned char v, int i, const int *first) {
    if (v >= 2 && v < 8) return first[v - 2] == i ? 0 : 1;
    return v == 1 ? 1 : (v == 0 ? 2 : -1);
}

__global__ void __launch_bounds__(256) classify_count_kernel(const unsigned char *__restrict__ code, int l,
                                                             const int *__restrict__ first, int *__restrict__ cnt) {
    __shared__ int ws[8];
    const int r0 = blockIdx.x * CB, r1 = min(l, r0 + CB);
    int c[3] = {0, 0, 0};
    for (int i = r0 + threadIdx.x; i < r1; i += 256) {
        const int k = classify_list(code[i], i, first);
        if (k >= 0) c[k] += 1;
    }
    for (int k = 0; k < 3; ++k) {
        const int t = bsum256(c[k], ws);
        if (threadIdx.x == 0) cnt[3 * blockIdx.x + k] = t;
    }
}

__global__ void __launch_bounds__(256) classify_write_kernel(const unsigned char *__restrict__ code, int l,
                                                             const int *__restrict__ first,
                                                             const int *__restrict__ cnt, int nb, int *SW, int *SC,
                                                             int *SIN, irwls_outer_counts *counts) {
    __shared__ int ws[3][8];
    int base[3];
    for (int k = 0; k < 3; ++k) {
        int part = 0;
        for (int b = threadIdx.x; b < (int)blockIdx.x; b += 256) part += cnt[3 * b + k];
        base[k] = bsum256(part, ws[0]);
    }
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) {
        counts->nSW = base[0] + cnt[3 * (nb - 1)];
        counts->nSC = base[1] + cnt[3 * (nb - 1) + 1];
        counts->nSIN = base[2] + cnt[3 * (nb - 1) + 2];
    }
    int *const out[3] = {SW, SC, SIN};
    const int r0 = blockIdx.x * CB, r1 = min(l, r0 + CB);
    for (int i0 = r0; i0 < r1; i0 += 256) {
        const int i = i0 + threadIdx.x;
        const int k = i < r1 ? classify_list(code[i], i, first) : -1;
        const bool m[3] = {k == 0, k == 1, k == 2};
        ordered_round<3>(m, i, base, out, ws);
    }
}

__global__ void fill_int_kernel(int *p, int n, int v) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

__global__ void mark_kernel(const int *__restrict__ SW, int nSW, int *__restrict__ mark, int v) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nSW; k += gridDim.x * blockDim.x) mark[SW[k]] = v;
}

// Precision form: the rows whose errors are kept exact (FP64 increments):
// support vectors, rows with |e_i y_i| < band, and the working set SW (marked
// in `mark`, l ints that are zero on entry and on exit). flag[i] says whether
// row i was exact before; rows entering the set are listed in Snew (their
// errors must be recomputed) unless `all_exact`.
__device__ __forceinline__ bool exact_in_set(const double *e, const double *y, const double *beta,
                                             const int *mark, double band, int i) {
    return beta[i] != 0.0 || fabs(e[i] * y[i]) < band || mark[i] != 0;
}

__global__ void __launch_bounds__(256) exact_count_kernel(const double *__restrict__ e, const double *__restrict__ y,
                                                          const double *__restrict__ beta, int l,
                                                          const int *__restrict__ mark, double band, int all_exact,
                                                          const int *__restrict__ flag, int *__restrict__ cnt) {
    __shared__ int ws[8];
    const int r0 = blockIdx.x * CB, r1 = min(l, r0 + CB);
    int cs = 0, cn = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += 256)
        if (exact_in_set(e, y, beta, mark, band, i)) {
            cs += 1;
            cn += (!all_exact && flag[i] == 0) ? 1 : 0;
        }
    cs = bsum256(cs, ws);
    cn = bsum256(cn, ws);
    if (threadIdx.x == 0) {
        cnt[2 * blockIdx.x] = cs;
        cnt[2 * blockIdx.x + 1] = cn;
    }
}

__global__ void __launch_bounds__(256) exact_write_kernel(const double *__restrict__ e, const double *__restrict__ y,
                                                          const double *__restrict__ beta, int l,
                                                          const int *__restrict__ mark, double band, int all_exact,
                                                          int *__restrict__ flag, const int *__restrict__ cnt, int nb,
                                                          int *S, int *Snew, int *counts) {
    __shared__ int ws[2][8];
    int base[2];
    for (int k = 0; k < 2; ++k) {
        int part = 0;
        for (int b = threadIdx.x; b < (int)blockIdx.x; b += 256) part += cnt[2 * b + k];
        base[k] = bsum256(part, ws[0]);
    }
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) {
        counts[0] = base[0] + cnt[2 * (nb - 1)];
        counts[1] = base[1] + cnt[2 * (nb - 1) + 1];
    }
    int *const out[2] = {S, Snew};
    const int r0 = blockIdx.x * CB, r1 = min(l, r0 + CB);
    for (int i0 = r0; i0 < r1; i0 += 256) {
        const int i = i0 + threadIdx.x;
        const bool in = i < r1 && exact_in_set(e, y, beta, mark, band, i);
        const bool m[2] = {in, in && !all_exact && flag[i] == 0};
        if (i < r1) flag[i] = in ? 1 : 0;  // each row's flag is read and written by its own thread only
        ordered_round<2>(m, i, base, out, ws);
    }
}

}  // namespace

// e = y - K(:, SV) beta_SV - b in FP64 over all l rows (the exact error
// vector that the incremental updates approximate).
extern "C" int irwls_full_exact_errors(const irwls_dev_set *X, int l, const double *d_beta, int *d_lst, double *d_cb,
                                       int *d_cnt, double *d_e) {
    sv_list_kernel<<<1, CT, 0, irwls_stream()>>>(d_beta, l, d_lst, d_cb, d_cnt);
    IRWLS_LAUNCH_CHECK("sv_list");
    return irwls_dev_kernel_rowsum_n(X, nullptr, l, X, d_lst, d_cnt, d_cb, nullptr, nullptr, -1, X->y, d_beta + l,
                                     d_e);
}

extern "C" int irwls_full_sv_list(const double *d_beta, int l, int *d_lst, double *d_cb, int *d_cnt) {
    sv_list_kernel<<<1, CT, 0, irwls_stream()>>>(d_beta, l, d_lst, d_cb, d_cnt);
    IRWLS_LAUNCH_CHECK("sv_list");
    return 0;
}

extern "C" int irwls_full_exact_set(const double *d_e, const double *d_y, const double *d_beta, int l,
                                    const int *d_SW, int nSW, double band, int all_exact, int *d_flag, int *d_mark,
                                    int *d_S, int *d_Snew, int *d_counts) {
    const int nb = std::max(1, ceil_div(l, CB));
    int *cnt = (int *)irwls_ctx_scratch(2, (size_t)2 * nb * sizeof(int));
    if (!cnt) return -3;
    if (nSW > 0) {
        mark_kernel<<<ceil_div(nSW, 256), 256, 0, irwls_stream()>>>(d_SW, nSW, d_mark, 1);
        IRWLS_LAUNCH_CHECK("exact_mark");
    }
    exact_count_kernel<<<nb, 256, 0, irwls_stream()>>>(d_e, d_y, d_beta, l, d_mark, band, all_exact, d_flag, cnt);
    IRWLS_LAUNCH_CHECK("exact_count");
    exact_write_kernel<<<nb, 256, 0, irwls_stream()>>>(d_e, d_y, d_beta, l, d_mark, band, all_exact, d_flag, cnt,
                                                       nb, d_S, d_Snew, d_counts);
    IRWLS_LAUNCH_CHECK("exact_write");
    if (nSW > 0) {
        mark_kernel<<<ceil_div(nSW, 256), 256, 0, irwls_stream()>>>(d_SW, nSW, d_mark, 0);
        IRWLS_LAUNCH_CHECK("exact_unmark");
    }
    return 0;
}

extern "C" int irwls_dev_gather(const double *d_src, const int *d_idx, int n, double *d_dst) {
    if (n <= 0) return 0;
    gather_kernel<<<std::min(ceil_div(n, 256), 1024), 256, 0, irwls_stream()>>>(d_src, d_idx, n, d_dst);
    IRWLS_LAUNCH_CHECK("gather");
    return 0;
}

extern "C" int irwls_dev_scatter(const double *d_src, const int *d_idx, int n, double *d_dst) {
    if (n <= 0) return 0;
    scatter_kernel<<<std::min(ceil_div(n, 256), 1024), 256, 0, irwls_stream()>>>(d_src, d_idx, n, d_dst);
    IRWLS_LAUNCH_CHECK("scatter");
    return 0;
}

extern "C" int irwls_sub_alloc(irwls_sub_ws *ws, int cap) {
    memset(ws, 0, sizeof *ws);
    ws->cap = cap;
    ws->ldH = cap + 2;
    const size_t nd = (size_t)cap + 2;
    int rc = 0;
    double **dbl[] = {&ws->a, &ws->e, &ws->beta, &ws->bnew, &ws->bsol, &ws->bbest, &ws->G13, &ws->rhs, &ws->GIN,
                      &ws->y, &ws->dlt, &ws->scal};
    for (double **p : dbl) rc |= irwls_dev_malloc((void **)p, nd * sizeof(double));
    int **ints[] = {&ws->grp, &ws->S1, &ws->S3, &ws->lst, &ws->gl1, &ws->gl3, &ws->cnt, &ws->mapbuf};
    for (int **p : ints) rc |= irwls_dev_malloc((void **)p, nd * sizeof(int));
    rc |= irwls_dev_malloc((void **)&ws->H, nd * nd * sizeof(double));
    rc |= irwls_dev_malloc((void **)&ws->stats, sizeof(irwls_sub_stats));
    rc |= irwls_dev_host_alloc((void **)&ws->h_stats, sizeof(irwls_sub_stats));
    ws->map = ws->mapbuf;
    return rc ? -3 : 0;
}

extern "C" void irwls_sub_release(irwls_sub_ws *ws) {
    irwls_dev_sync();
    void *ptrs[] = {ws->a, ws->e, ws->beta, ws->bnew, ws->bsol, ws->bbest, ws->G13, ws->rhs, ws->GIN, ws->y,
                    ws->dlt, ws->scal, ws->grp, ws->S1, ws->S3, ws->lst, ws->gl1, ws->gl3, ws->cnt, ws->mapbuf,
                    ws->H, ws->stats};
    for (void *p : ptrs) irwls_dev_free(p);
    irwls_dev_host_free(ws->h_stats);
    memset(ws, 0, sizeof *ws);
}

extern "C" int irwls_sub_init(irwls_sub_ws *ws, const irwls_dev_set *X, double C) {
    sub_init_kernel<<<1, CT, 0, irwls_stream()>>>(*ws, X->y, C);
    IRWLS_LAUNCH_CHECK("sub_init");
    return 0;
}

// G13 of the current S1/S3 lists (src/full-train.c:327-344). The reference
// computes it at the end of an iteration for use in the next one; it is
// issued here at the start of the next iteration, when n1/n3 are known.
extern "C" int irwls_sub_g13(irwls_sub_ws *ws, const irwls_dev_set *X, int n1, int n3) {
    if (n3 <= 0 || n1 <= 0) return 0;
    const int ex = irwls_tc_exact_rowsum(ws->tcs, X, ws->gl1, n1, ws->gl3, n3, nullptr, n3, ws->rhs, X->y, X->y, +1,
                                         nullptr, nullptr, ws->G13);
    if (ex != 1) return ex;
    return irwls_dev_kernel_rowsum(X, ws->gl1, n1, X, ws->gl3, n3, ws->rhs, X->y, X->y, 0, +1, nullptr, nullptr,
                                   ws->G13);
}

extern "C" int irwls_sub_iterate(irwls_sub_ws *ws, const irwls_dev_set *X, double C, int n1, int n3) {
    const int n = n1 + 1;
    KView kv = kview(X);
    if (n1 > 0) {
        // precision form on integer-valued data: the kernel block from exact
        // tensor-core dot products (FP64 exp), then the diagonal's 1 / a
        const int ex = irwls_tc_exact_block(ws->tcs, X, ws->gl1, n1, ws->gl1, n1, X->y, X->y, ws->H, ws->ldH, 1);
        if (ex < 0) return -2;
        if (ex == 0) {
            build_H_diag_kernel<<<ceil_div(n1, 256), 256, 0, irwls_stream()>>>(*ws, n1);
            IRWLS_LAUNCH_CHECK("build_H_diag");
        } else {
            dim3 grid(ceil_div(n1, 64), n1);
            const size_t smem = (size_t)X->ld * sizeof(double);
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(build_H_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            build_H_kernel<<<grid, 64, smem, irwls_stream()>>>(*ws, kv, n1);
            IRWLS_LAUNCH_CHECK("build_H");
        }
    }
    build_border_kernel<<<ceil_div(n1 + 1, 256), 256, 0, irwls_stream()>>>(*ws, n1);
    IRWLS_LAUNCH_CHECK("build_border");
    // precision form: FP32 factor + FP64 refinement in one cluster launch,
    // the FP64 factorization where that cannot run or does not converge
    int solve = 1;
    if (irwls_get_precision() == IRWLS_PRECISION_MIXED) {
        solve = irwls_ws_solve_mixed(ws->H, n1, ws->ldH, ws->rhs, ws->bsol);
        if (solve < 0) return -2;
        g_ws_mixed_solves += solve == 0;
        g_ws_mixed_fallbacks += solve == 1 && n1 >= 1 && n1 <= irwls_ws_mixed_max();
    }
    if (solve == 1 && irwls_dev_chol_solve(ws->H, n, ws->ldH, ws->rhs, ws->bsol)) return -2;
    sub_update_kernel<<<1, CT, 0, irwls_stream()>>>(*ws, C, n1, n3);
    IRWLS_LAUNCH_CHECK("sub_update");
    // e_i -= k(i, j) (bnew_j - beta_j) over changed j, then the bias change
    // (exact tensor-core dot products in the precision form where the data
    // allow them: at most w changed entries)
    const int ex = irwls_tc_exact_rowsum(ws->tcs, X, ws->map, ws->w, ws->lst, 0, ws->cnt, ws->w, ws->dlt, nullptr,
                                         nullptr, -1, ws->e, ws->scal, ws->e);
    if (ex < 0) return -2;
    if (ex == 1 && irwls_dev_kernel_rowsum_n(X, ws->map, ws->w, X, ws->lst, ws->cnt, ws->dlt, nullptr, nullptr, -1,
                                             ws->e, ws->scal, ws->e))
        return -2;
    sub_groups_kernel<<<1, CT, 0, irwls_stream()>>>(*ws, C);
    IRWLS_LAUNCH_CHECK("sub_groups");
    return 0;
}

extern "C" int irwls_full_gin(const irwls_dev_set *X, const int *d_SW, int nSW, const int *d_SIN, int nSIN,
                              const double *d_bnew, int *d_lst, double *d_cb, int *d_cnt, double *d_GIN) {
    // scratch slot 2: the chunk counts (then offsets) and chunk sums
    unsigned char *sc = (unsigned char *)irwls_ctx_scratch(2, (size_t)CT * (sizeof(int) + sizeof(double)));
    if (!sc) return -3;
    double *csum = (double *)sc;
    int *ccount = (int *)(sc + (size_t)CT * sizeof(double));
    gin_chunk_kernel<<<CT / PC, PC, 0, irwls_stream()>>>(d_SIN, nSIN, d_bnew, ccount, csum);
    IRWLS_LAUNCH_CHECK("gin_chunk");
    gin_scan_kernel<<<1, CT, 0, irwls_stream()>>>(ccount, csum, d_cnt, d_GIN, nSW);
    IRWLS_LAUNCH_CHECK("gin_scan");
    gin_write_kernel<<<CT / PC, PC, 0, irwls_stream()>>>(d_SIN, nSIN, d_bnew, ccount, d_lst, d_cb);
    IRWLS_LAUNCH_CHECK("gin_write");
    return irwls_dev_kernel_rowsum_n(X, d_SW, nSW, X, d_lst, d_cnt, d_cb, X->y, nullptr, +1, nullptr, nullptr,
                                     d_GIN);
}

extern "C" int irwls_full_gather_ws(const int *d_SW, int nSW, const double *d_e, const double *d_beta, int l,
                                    double *d_esub, double *d_bsub) {
    gather_ws_kernel<<<ceil_div(nSW + 1, 256), 256, 0, irwls_stream()>>>(d_SW, nSW, d_e, d_beta, l, d_esub, d_bsub);
    IRWLS_LAUNCH_CHECK("gather_ws");
    return 0;
}

extern "C" int irwls_full_apply_ws(const int *d_SW, int nSW, const double *d_bt, const double *d_beta, int l,
                                   double *d_bnew, int *d_lst, double *d_cb, int *d_cnt, double *d_dbias) {
    if (irwls_dev_d2d(d_bnew, d_beta, (size_t)(l + 1) * sizeof(double))) return -2;
    apply_ws_kernel<<<1, CT, 0, irwls_stream()>>>(d_SW, nSW, d_bt, d_beta, l, d_bnew, d_lst, d_cb, d_cnt, d_dbias);
    IRWLS_LAUNCH_CHECK("apply_ws");
    return 0;
}

extern "C" int irwls_full_norms(const double *d_beta, const double *d_bnew, int n, double *d_out2) {
    double *part = (double *)irwls_ctx_scratch(2, (size_t)2 * CT * sizeof(double));
    if (!part) return -3;
    norms_chunk_kernel<<<CT / PC, PC, 0, irwls_stream()>>>(d_beta, d_bnew, n, part);
    IRWLS_LAUNCH_CHECK("norms_chunk");
    norms_final_kernel<<<1, CT, 0, irwls_stream()>>>(part, d_out2);
    IRWLS_LAUNCH_CHECK("norms_final");
    return 0;
}

extern "C" int irwls_full_classify(const double *d_bnew, const double *d_e, const double *d_y, int l, double C,
                                   int *d_SW, int *d_SC, int *d_SIN, irwls_outer_counts *d_counts) {
    if (l < 4 * CB) {
        // small sets: one CTA is faster than four launches
        classify_kernel<<<1, CT, 0, irwls_stream()>>>(d_bnew, d_e, d_y, l, C, d_SW, d_SC, d_SIN, d_counts);
        IRWLS_LAUNCH_CHECK("classify");
        return 0;
    }
    const int nb = ceil_div(l, CB);
    // scratch slot 2: the per-block counts, then the six first-violator
    // slots, then one code byte per row
    const size_t cbytes = (size_t)3 * nb * sizeof(int), fbytes = 8 * sizeof(int);
    unsigned char *sc = (unsigned char *)irwls_ctx_scratch(2, cbytes + fbytes + (size_t)l);
    if (!sc) return -3;
    int *cnt = (int *)sc, *first = (int *)(sc + cbytes);
    unsigned char *code = sc + cbytes + fbytes;
    fill_int_kernel<<<1, 32, 0, irwls_stream()>>>(first, 6, 0x7fffffff);
    IRWLS_LAUNCH_CHECK("classify_first");
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    classify_code_kernel<<<std::min(ceil_div(l, 256), 8 * sms), 256, 0, irwls_stream()>>>(d_bnew, d_e, d_y, l, C,
                                                                                         code, first);
    IRWLS_LAUNCH_CHECK("classify_code");
    classify_count_kernel<<<nb, 256, 0, irwls_stream()>>>(code, l, first, cnt);
    IRWLS_LAUNCH_CHECK("classify_count");
    classify_write_kernel<<<nb, 256, 0, irwls_stream()>>>(code, l, first, cnt, nb, d_SW, d_SC, d_SIN, d_counts);
    IRWLS_LAUNCH_CHECK("classify_write");
    return 0;
}

extern "C" int irwls_full_fill_ws(int *d_SW, int nSW, int *d_SIN, int nSIN, const int *d_SC, int nSC,
                                  const int *d_perm, int space) {
    if (nSC <= 0) return 0;
    fill_ws_kernel<<<ceil_div(nSC, 256), 256, 0, irwls_stream()>>>(d_SW, nSW, d_SIN, nSIN, d_SC, nSC, d_perm, space);
    IRWLS_LAUNCH_CHECK("fill_ws");
    return 0;
}
