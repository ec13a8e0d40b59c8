// dev_model.cu -- models kept on the GPU: support-vector packing, the binary
// model file and batched prediction without host svm_sample arrays (the
// reference's calculateFULLModel / calculateBudgetedModel,
// src/full-train.c:779-839 and src/budgeted-train.c:519-570, and
// storeModel / readModel, src/IOStructures.c:773-825).
//
// A device model holds the header fields on the host and, on the device, its
// support vectors as a row set (CSR by feature index, the same rows densely
// by feature index, their norms) with their weights: the form the prediction
// kernels read. It is packed from a resident dataset (the rows with beta != 0
// in row order, or the given centroids), read from a model file (the file's
// svm_sample records go to the device as they are and are split into rows
// there), and stored as the byte layout storeModel writes.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "dev_common.cuh"
#include "irwls_gpu.h"

struct irwls_dmodel {
    double Kgamma, bias;
    int maxdim, kernelType, sparse, nSVs, nElem;
    irwls_dev_set S;  // the support vectors (mode: linear or norm-form RBF)
    double *d_w;      // weights, nSVs
};

extern "C" const irwls_dev_set *irwls_resident_devset(const irwls_resident *r);
extern "C" const svm_dataset *irwls_resident_dataset(const irwls_resident *r);

namespace {

constexpr int CB = 2048;  // rows per block of the ordered compactions

__device__ __forceinline__ int block_sum256(int v, int *ws) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int k = 0; k < 8; ++k) t += ws[k];
    __syncthreads();
    return t;
}

// Ordered selection of the indices i < n with pred(i): count per block, then
// every block places its indices after the counts of the blocks before it.
template <class Pred>
__global__ void __launch_bounds__(256) select_count_kernel(Pred pred, int n, int *__restrict__ cnt) {
    __shared__ int ws[8];
    const int r0 = blockIdx.x * CB, r1 = min(n, r0 + CB);
    int c = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += 256) c += pred(i) ? 1 : 0;
    const int t = block_sum256(c, ws);
    if (threadIdx.x == 0) cnt[blockIdx.x] = t;
}

template <class Pred>
__global__ void __launch_bounds__(256) select_write_kernel(Pred pred, int n, const int *__restrict__ cnt, int nb,
                                                           int *__restrict__ out, int *__restrict__ total) {
    __shared__ int ws[8], woff[8];
    int part = 0;
    for (int k = threadIdx.x; k < (int)blockIdx.x; k += 256) part += cnt[k];
    int base = block_sum256(part, ws);
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) total[0] = base + cnt[nb - 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = blockIdx.x * CB, r1 = min(n, r0 + CB);
    for (int i0 = r0; i0 < r1; i0 += 256) {
        const int i = i0 + threadIdx.x;
        const bool on = i < r1 && pred(i);
        const unsigned bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) ws[warp] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int k = 0; k < 8; ++k) {
                woff[k] = t;
                t += ws[k];
            }
            ws[0] = t;
        }
        __syncthreads();
        if (on) out[base + woff[warp] + __popc(bal & ((1u << lane) - 1u))] = i;
        base += ws[0];
        __syncthreads();
    }
}

struct NonZero {
    const double *v;
    __device__ bool operator()(int i) const { return v[i] != 0.0; }
};
struct Terminator {
    const svm_sample *r;
    __device__ bool operator()(int i) const { return r[i].index == -1; }
};

// Indices i < n with pred(i), in order, into out; returns their count.
template <class Pred>
int select(Pred pred, int n, int *out, int *count) {
    const int nb = std::max(1, ceil_div(n, CB));
    int *cnt = nullptr, *d_tot = nullptr;
    int rc = irwls_dev_malloc((void **)&cnt, (size_t)nb * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_tot, sizeof(int));
    if (!rc) {
        select_count_kernel<<<nb, 256, 0, irwls_stream()>>>(pred, n, cnt);
        irwls_count_launch(1);
        rc |= irwls_check_launch("select_count");
        select_write_kernel<<<nb, 256, 0, irwls_stream()>>>(pred, n, cnt, nb, out, d_tot);
        irwls_count_launch(1);
        rc |= irwls_check_launch("select_write");
        rc |= irwls_dev_d2h(count, d_tot, sizeof(int));
        rc |= irwls_dev_sync();
    }
    irwls_dev_free(cnt);
    irwls_dev_free(d_tot);
    return rc;
}

// Exclusive prefix of len[0, n) into off[0, n] (off[n] = total), in order.
__global__ void __launch_bounds__(256) scan_sum_kernel(const int *__restrict__ len, int n, int *__restrict__ bsum) {
    __shared__ int ws[8];
    const int r0 = blockIdx.x * CB, r1 = min(n, r0 + CB);
    int c = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += 256) c += len[i];
    const int t = block_sum256(c, ws);
    if (threadIdx.x == 0) bsum[blockIdx.x] = t;
}

__global__ void __launch_bounds__(256) scan_write_kernel(const int *__restrict__ len, int n,
                                                         const int *__restrict__ bsum, int nb, int *__restrict__ off) {
    __shared__ int ws[8], pre[256];
    int part = 0;
    for (int k = threadIdx.x; k < (int)blockIdx.x; k += 256) part += bsum[k];
    int base = block_sum256(part, ws);
    const int r0 = blockIdx.x * CB, r1 = min(n, r0 + CB);
    for (int i0 = r0; i0 < r1; i0 += 256) {
        const int i = i0 + threadIdx.x;
        const int v = i < r1 ? len[i] : 0;
        pre[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 256; o <<= 1) {
            const int x = threadIdx.x >= (unsigned)o ? pre[threadIdx.x - o] : 0;
            __syncthreads();
            pre[threadIdx.x] += x;
            __syncthreads();
        }
        if (i < r1) off[i] = base + pre[threadIdx.x] - v;
        base += pre[255];
        __syncthreads();
    }
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) off[n] = base;
}

int scan(const int *len, int n, int *off) {
    const int nb = std::max(1, ceil_div(n, CB));
    int *bs = nullptr;
    int rc = irwls_dev_malloc((void **)&bs, (size_t)nb * sizeof(int));
    if (!rc) {
        scan_sum_kernel<<<nb, 256, 0, irwls_stream()>>>(len, n, bs);
        irwls_count_launch(1);
        rc |= irwls_check_launch("scan_sum");
        scan_write_kernel<<<nb, 256, 0, irwls_stream()>>>(len, n, bs, nb, off);
        irwls_count_launch(1);
        rc |= irwls_check_launch("scan_write");
    }
    irwls_dev_free(bs);
    return rc;
}

// Rows src[k] of a device set (CSR by feature index): their lengths.
__global__ void pick_len_kernel(const int *__restrict__ rp, const int *__restrict__ src, int n, int *__restrict__ len) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        len[k] = rp[src[k] + 1] - rp[src[k]];
}

// Copies rows src[k] (CSR entries, norm) into the packed set; weights w[k] =
// wsrc[src[k]] (or wdir[k] when given); the largest index into *maxidx. One
// warp per row.
__global__ void pick_rows_kernel(const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ cv,
                                 const double *__restrict__ q, const int *__restrict__ src, int n,
                                 const int *__restrict__ prp, int *__restrict__ pci, double *__restrict__ pcv,
                                 double *__restrict__ pq, const double *__restrict__ wsrc,
                                 const double *__restrict__ wdir, double *__restrict__ w, int *__restrict__ maxidx) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int mx = -1;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += nw) {
        const int r = src[k], s0 = rp[r], len = rp[r + 1] - s0, d0 = prp[k];
        for (int t = lane; t < len; t += 32) {
            const int c = ci[s0 + t];
            pci[d0 + t] = c;
            pcv[d0 + t] = cv[s0 + t];
            mx = max(mx, c);
        }
        if (lane == 0) {
            pq[k] = q[r];
            w[k] = wdir ? wdir[k] : wsrc[r];
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && mx >= 0) atomicMax(maxidx, mx);
}

// Rows of a model file's svm_sample records: row k runs from the entry after
// terminator k - 1 up to terminator k.
__global__ void split_records_kernel(const svm_sample *__restrict__ rec, const int *__restrict__ term, int n,
                                     int *__restrict__ rp, int *__restrict__ ci, double *__restrict__ cv,
                                     int *__restrict__ maxidx) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int mx = -1;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += nw) {
        const int b = k == 0 ? 0 : term[k - 1] + 1, e = term[k];
        const int d0 = b - k;  // entries before row k: positions minus the k terminators before them
        if (lane == 0) rp[k] = d0;
        if (k == n - 1 && lane == 0) rp[n] = e - k;
        for (int t = lane; t < e - b; t += 32) {
            ci[d0 + t] = rec[b + t].index;
            cv[d0 + t] = rec[b + t].value;
            mx = max(mx, rec[b + t].index);
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && mx >= 0) atomicMax(maxidx, mx);
}

// Dense rows by feature index from the CSR rows (X zeroed first).
__global__ void dense_rows_kernel(const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ cv,
                                  int n, int ld, double *__restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += nw)
        for (int p = rp[k] + lane; p < rp[k + 1]; p += 32) X[(size_t)k * ld + ci[p]] = cv[p];
}

// The model file's records: each row's entries, then (-1, 0.0).
__global__ void records_kernel(const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ cv,
                               int n, svm_sample *__restrict__ rec) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += nw) {
        const int b = rp[k], e = rp[k + 1];
        for (int p = b + lane; p < e; p += 32) {
            rec[p + k].index = ci[p];
            rec[p + k].value = cv[p];
        }
        if (lane == 0) {
            rec[e + k].index = -1;
            rec[e + k].value = 0.0;
        }
    }
}

int grid_for(long long n, int per_block) {
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    return (int)std::max<long long>(1, std::min<long long>((n + per_block - 1) / per_block, 16LL * sms));
}

// Completes m->S from its CSR rows (rp, ci, cv, q already on the device):
// width, leading dimension, the dense rows, the mode.
int finish_set(irwls_dmodel *m, int maxidx, long long nnz) {
    irwls_dev_set &S = m->S;
    S.n_rows = m->nSVs;
    S.width = std::max(1, maxidx + 1);
    S.ld = (S.width + 1) & ~1;
    S.mode = m->kernelType == 0 ? IRWLS_K_LINEAR : IRWLS_K_NORM_RBF;
    S.neg_gamma = -m->Kgamma;
    S.nnz = nnz;
    const size_t xb = (size_t)std::max(1, m->nSVs) * S.ld * sizeof(double);
    int rc = irwls_dev_malloc((void **)&S.X, xb);
    rc |= irwls_dev_malloc((void **)&S.y, (size_t)std::max(1, m->nSVs) * sizeof(double));
    if (rc) return rc;
    rc |= irwls_dev_memset(S.X, 0, xb);
    rc |= irwls_dev_memset(S.y, 0, (size_t)std::max(1, m->nSVs) * sizeof(double));
    if (m->nSVs > 0) {
        dense_rows_kernel<<<grid_for((long long)m->nSVs * 32, 256), 256, 0, irwls_stream()>>>(S.rp, S.ci, S.cv, m->nSVs,
                                                                                            S.ld, S.X);
        irwls_count_launch(1);
        rc |= irwls_check_launch("dense_rows");
    }
    return rc;
}

irwls_dmodel *pack(const irwls_resident *r, properties props, const int *h_rows, int nrows_given, const double *beta,
                   const double *weights, double bias) {
    irwls_clear_error();
    const irwls_dev_set *X = irwls_resident_devset(r);
    const svm_dataset *ds = irwls_resident_dataset(r);
    irwls_dmodel *m = (irwls_dmodel *)calloc(1, sizeof *m);
    if (!m) return nullptr;
    m->Kgamma = props.Kgamma;
    m->bias = bias;
    m->maxdim = ds->maxdim;
    m->kernelType = props.kernelType;
    m->sparse = ds->sparse;
    int *d_src = nullptr, *d_len = nullptr, *d_max = nullptr;
    double *d_beta = nullptr, *d_wdir = nullptr;
    int rc = 0, n = 0;
    if (beta) {
        // the rows with beta != 0, in row order
        rc |= irwls_dev_malloc((void **)&d_beta, (size_t)(ds->l + 1) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_src, (size_t)std::max(1, ds->l) * sizeof(int));
        if (!rc) rc |= irwls_dev_h2d(d_beta, beta, (size_t)(ds->l + 1) * sizeof(double));
        if (!rc) rc |= select(NonZero{d_beta}, ds->l, d_src, &n);
    } else {
        n = nrows_given;
        rc |= irwls_dev_malloc((void **)&d_src, (size_t)std::max(1, n) * sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_wdir, (size_t)std::max(1, n) * sizeof(double));
        if (!rc && n) {
            rc |= irwls_dev_h2d(d_src, h_rows, (size_t)n * sizeof(int));
            rc |= irwls_dev_h2d(d_wdir, weights, (size_t)n * sizeof(double));
        }
    }
    m->nSVs = n;
    irwls_dev_set &S = m->S;
    int nnz = 0, maxidx = -1;
    if (!rc) {
        rc |= irwls_dev_malloc((void **)&d_len, (size_t)std::max(1, n) * sizeof(int));
        rc |= irwls_dev_malloc((void **)&S.rp, (size_t)(n + 1) * sizeof(int));
        rc |= irwls_dev_malloc((void **)&S.q, (size_t)std::max(1, n) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&m->d_w, (size_t)std::max(1, n) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_max, sizeof(int));
        rc |= irwls_dev_h2d(d_max, &maxidx, sizeof(int));
    }
    if (!rc && n > 0) {
        pick_len_kernel<<<grid_for(n, 256), 256, 0, irwls_stream()>>>(X->rp, d_src, n, d_len);
        irwls_count_launch(1);
        rc |= irwls_check_launch("pick_len");
        rc |= scan(d_len, n, S.rp);
        rc |= irwls_dev_d2h(&nnz, S.rp + n, sizeof(int));
        rc |= irwls_dev_sync();
    } else if (!rc) {
        rc |= irwls_dev_memset(S.rp, 0, sizeof(int));
    }
    if (!rc) {
        rc |= irwls_dev_malloc((void **)&S.ci, (size_t)std::max(1, nnz) * sizeof(int));
        rc |= irwls_dev_malloc((void **)&S.cv, (size_t)std::max(1, nnz) * sizeof(double));
    }
    if (!rc && n > 0) {
        pick_rows_kernel<<<grid_for((long long)n * 32, 256), 256, 0, irwls_stream()>>>(
            X->rp, X->ci, X->cv, X->q, d_src, n, S.rp, S.ci, S.cv, S.q, d_beta, d_wdir, m->d_w, d_max);
        irwls_count_launch(1);
        rc |= irwls_check_launch("pick_rows");
        rc |= irwls_dev_d2h(&maxidx, d_max, sizeof(int));
        rc |= irwls_dev_sync();
    }
    m->nElem = nnz + n;
    if (!rc) rc = finish_set(m, maxidx, nnz);
    void *bufs[] = {d_src, d_len, d_max, d_beta, d_wdir};
    for (void *p : bufs) irwls_dev_free(p);
    if (rc) {
        irwls_dmodel_free(m);
        return nullptr;
    }
    return m;
}

}  // namespace

extern "C" irwls_dmodel *irwls_dmodel_full(const irwls_resident *r, properties props, const double *beta) {
    if (!r || !beta) {
        irwls_set_error(-4, "a resident dataset and its weights are needed");
        return nullptr;
    }
    return pack(r, props, nullptr, 0, beta, nullptr, beta[irwls_resident_dataset(r)->l]);
}

extern "C" irwls_dmodel *irwls_dmodel_budgeted(const irwls_resident *r, properties props, const int *centroids,
                                               const double *weights) {
    if (!r || !centroids || !weights) {
        irwls_set_error(-4, "a resident dataset, centroids and weights are needed");
        return nullptr;
    }
    const irwls_dev_set *X = irwls_resident_devset(r);
    for (int i = 0; i < props.size; ++i)
        if (centroids[i] < 0 || centroids[i] >= X->n_rows) {
            irwls_set_error(-4, "centroid %d is row %d of a resident set of %d rows", i, centroids[i], X->n_rows);
            return nullptr;
        }
    return pack(r, props, centroids, props.size, nullptr, weights, 0.0);
}

extern "C" irwls_dmodel *irwls_dmodel_read(const char *path) {
    irwls_clear_error();
    if (irwls_dev_init()) return nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) {
        irwls_set_error(-5, "cannot open %s", path);
        return nullptr;
    }
    irwls_dmodel *m = (irwls_dmodel *)calloc(1, sizeof *m);
    size_t got = 0;
    got += fread(&m->Kgamma, sizeof(double), 1, f);
    got += fread(&m->bias, sizeof(double), 1, f);
    got += fread(&m->maxdim, sizeof(int), 1, f);
    got += fread(&m->kernelType, sizeof(int), 1, f);
    got += fread(&m->sparse, sizeof(int), 1, f);
    got += fread(&m->nSVs, sizeof(int), 1, f);
    got += fread(&m->nElem, sizeof(int), 1, f);
    const int n = m->nSVs, ne = m->nElem;
    void *h = nullptr;
    const size_t body = (size_t)n * 2 * sizeof(double) + (size_t)ne * sizeof(svm_sample);
    int rc = (got != 7 || n < 0 || ne < n) ? -5 : 0;
    if (!rc) rc = irwls_dev_host_alloc(&h, std::max<size_t>(body, 16));
    if (!rc && fread(h, 1, body, f) != body) rc = -5;
    fclose(f);
    if (rc) {
        if (h) irwls_dev_host_free(h);
        free(m);
        irwls_set_error(-5, "%s is not a complete model file", path);
        return nullptr;
    }
    double *hw = (double *)h, *hq = hw + n;
    const svm_sample *hrec = (const svm_sample *)(hq + n);
    svm_sample *d_rec = nullptr;
    int *d_term = nullptr, *d_max = nullptr;
    irwls_dev_set &S = m->S;
    int nterm = 0, maxidx = -1;
    rc |= irwls_dev_malloc((void **)&d_rec, (size_t)std::max(1, ne) * sizeof(svm_sample));
    rc |= irwls_dev_malloc((void **)&d_term, (size_t)std::max(1, ne) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&m->d_w, (size_t)std::max(1, n) * sizeof(double));
    rc |= irwls_dev_malloc((void **)&S.q, (size_t)std::max(1, n) * sizeof(double));
    rc |= irwls_dev_malloc((void **)&S.rp, (size_t)(n + 1) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&S.ci, (size_t)std::max(1, ne - n) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&S.cv, (size_t)std::max(1, ne - n) * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_max, sizeof(int));
    if (!rc) {
        rc |= irwls_dev_h2d(d_rec, hrec, (size_t)ne * sizeof(svm_sample));
        rc |= irwls_dev_h2d(m->d_w, hw, (size_t)n * sizeof(double));
        rc |= irwls_dev_h2d(S.q, hq, (size_t)n * sizeof(double));
        rc |= irwls_dev_h2d(d_max, &maxidx, sizeof(int));
        rc |= irwls_dev_memset(S.rp, 0, sizeof(int));
    }
    if (!rc && ne > 0) rc |= select(Terminator{d_rec}, ne, d_term, &nterm);
    if (!rc && nterm != n) {
        irwls_set_error(-5, "%s holds %d rows for %d support vectors", path, nterm, n);
        rc = -5;
    }
    if (!rc && n > 0) {
        split_records_kernel<<<grid_for((long long)n * 32, 256), 256, 0, irwls_stream()>>>(d_rec, d_term, n, S.rp, S.ci,
                                                                                         S.cv, d_max);
        irwls_count_launch(1);
        rc |= irwls_check_launch("split_records");
        rc |= irwls_dev_d2h(&maxidx, d_max, sizeof(int));
        rc |= irwls_dev_sync();
    }
    irwls_dev_host_free(h);
    irwls_dev_free(d_rec);
    irwls_dev_free(d_term);
    irwls_dev_free(d_max);
    if (!rc) rc = finish_set(m, maxidx, (long long)ne - n);
    if (rc) {
        irwls_dmodel_free(m);
        return nullptr;
    }
    return m;
}

extern "C" int irwls_dmodel_store(const irwls_dmodel *m, const char *path) {
    irwls_clear_error();
    const int n = m->nSVs, ne = m->nElem;
    svm_sample *d_rec = nullptr;
    void *h = nullptr;
    const size_t body = (size_t)n * 2 * sizeof(double) + (size_t)ne * sizeof(svm_sample);
    int rc = irwls_dev_malloc((void **)&d_rec, (size_t)std::max(1, ne) * sizeof(svm_sample));
    rc |= irwls_dev_host_alloc(&h, std::max<size_t>(body, 16));
    // zeroed first: the 4 padding bytes of every record are written as zeros, as
    // the reference's calloc'd records hold
    if (!rc) rc |= irwls_dev_memset(d_rec, 0, (size_t)std::max(1, ne) * sizeof(svm_sample));
    if (!rc && n > 0) {
        records_kernel<<<grid_for((long long)n * 32, 256), 256, 0, irwls_stream()>>>(m->S.rp, m->S.ci, m->S.cv, n,
                                                                                   d_rec);
        irwls_count_launch(1);
        rc |= irwls_check_launch("records");
        double *hw = (double *)h, *hq = hw + n;
        rc |= irwls_dev_d2h(hw, m->d_w, (size_t)n * sizeof(double));
        rc |= irwls_dev_d2h(hq, m->S.q, (size_t)n * sizeof(double));
        rc |= irwls_dev_d2h(hq + n, d_rec, (size_t)ne * sizeof(svm_sample));
        rc |= irwls_dev_sync();
    }
    irwls_dev_free(d_rec);
    FILE *f = rc ? nullptr : fopen(path, "wb");
    if (!rc && !f) {
        irwls_set_error(-5, "cannot write %s", path);
        rc = -5;
    }
    if (f) {
        size_t w = 0;
        w += fwrite(&m->Kgamma, sizeof(double), 1, f);
        w += fwrite(&m->bias, sizeof(double), 1, f);
        w += fwrite(&m->maxdim, sizeof(int), 1, f);
        w += fwrite(&m->kernelType, sizeof(int), 1, f);
        w += fwrite(&m->sparse, sizeof(int), 1, f);
        w += fwrite(&m->nSVs, sizeof(int), 1, f);
        w += fwrite(&m->nElem, sizeof(int), 1, f);
        if (body && fwrite(h, 1, body, f) != body) rc = -5;
        if (fclose(f) || w != 7) rc = -5;
        if (rc) irwls_set_error(-5, "cannot write %s", path);
    }
    if (h) irwls_dev_host_free(h);
    return rc;
}

// test (soft = 0) / softTest (soft = 1) of the reference with a device model.
extern "C" double *irwls_dmodel_predict(const irwls_dmodel *m, svm_dataset ds, predictProperties props, int soft) {
    irwls_clear_error();
    const int n = ds.l;
    double *out = (double *)malloc((size_t)std::max(1, n) * sizeof(double));
    if (!out) return nullptr;
    if (n > 0) {
        const int w = std::max(irwls_feature_width(&ds, n), m->S.width);
        irwls_dev_set T;
        const int fast = m->kernelType == 0 && irwls_get_linear_fast_path();
        int rc = fast ? irwls_dev_upload_csr(&ds, n, m->kernelType, m->Kgamma, w, &T)
                      : irwls_dev_upload(&ds, n, m->kernelType, m->Kgamma, 1, w, &T);
        if (rc) {
            free(out);
            return nullptr;
        }
        double *d_out = nullptr, *d_W = nullptr;
        rc |= irwls_dev_malloc((void **)&d_out, (size_t)n * sizeof(double));
        if (fast)
            rc |= irwls_dev_malloc((void **)&d_W, irwls_predict_linear_scratch(m->S.width, m->nSVs) * sizeof(double));
        if (!rc) {
            rc |= fast ? irwls_predict_linear(&T, n, &m->S, m->nSVs, m->d_w, m->bias, !soft, d_W, d_out)
                       : irwls_predict_soft(&T, n, &m->S, m->nSVs, m->d_w, m->bias, !soft, d_out);
            rc |= irwls_dev_d2h(out, d_out, (size_t)n * sizeof(double));
            rc |= irwls_dev_sync();
        }
        irwls_dev_free(d_out);
        irwls_dev_free(d_W);
        irwls_dev_release(&T);
        if (rc) {
            free(out);
            return nullptr;
        }
    }
    if (props.Labels == 1) {
        double hits = 0.0;
        for (int i = 0; i < n; i++) {
            if ((out[i] > 0) & (ds.y[i] > 0)) hits++;
            if ((out[i] <= 0) & (ds.y[i] <= 0)) hits++;
        }
        printf("Accuracy: %f\n", hits / (double)n);
    }
    return out;
}

extern "C" void irwls_dmodel_info(const irwls_dmodel *m, int *nSVs, int *nElem, double *bias) {
    if (nSVs) *nSVs = m->nSVs;
    if (nElem) *nElem = m->nElem;
    if (bias) *bias = m->bias;
}

extern "C" void irwls_dmodel_free(irwls_dmodel *m) {
    if (!m) return;
    irwls_dev_release(&m->S);
    irwls_dev_free(m->d_w);
    free(m);
}
