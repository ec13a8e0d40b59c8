// dev_context.cu -- device context of the library: the CUDA stream, error
// state, memory helpers, dataset upload and kernel timing.
//
// Every host thread works in an execution context: its stream, its device
// status words, its error slot, its grow-only scratch buffers and its random
// generator. The main thread uses the default context (whose generator is
// libc rand(), as in the reference); the batch driver gives each worker
// thread a context of its own (irwls_ctx_create / irwls_ctx_bind) so that
// trainings run concurrently on separate streams. Device memory is allocated
// stream-ordered (cudaMallocAsync / cudaFreeAsync on the context's stream),
// so that no thread's free waits for the whole device.
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "dev_common.cuh"

namespace {

constexpr int IRWLS_SCRATCH_SLOTS = 4;

// glibc's rand() generator (the additive feedback generator of degree 31 and
// separation 3 behind its random_r), restated so that a worker thread can
// reproduce exactly the numbers srand(seed) then rand() would give in a
// single-threaded run, without sharing libc's state.
struct Rand31 {
    int32_t r[31];
    int f, b;
    void seed(unsigned s) {
        int32_t w = (int32_t)(s == 0 ? 1u : s);
        r[0] = w;
        for (int i = 1; i < 31; ++i) {
            // 16807 * w mod (2^31 - 1) without overflow (Schrage's method)
            const int32_t hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            r[i] = w;
        }
        f = 3;
        b = 0;
        for (int i = 0; i < 310; ++i) next();
    }
    int next() {
        const uint32_t v = (uint32_t)r[f] + (uint32_t)r[b];
        r[f] = (int32_t)v;
        const int out = (int)(v >> 1);
        if (++f >= 31) f = 0;
        if (++b >= 31) b = 0;
        return out;
    }
};

struct Ctx {
    cudaStream_t stream = nullptr;
    int *flags = nullptr;  // device status words, see irwls_dev_flags()
    int err = 0;
    char msg[512] = "";
    void *scratch[IRWLS_SCRATCH_SLOTS] = {};
    size_t scratch_bytes[IRWLS_SCRATCH_SLOTS] = {};
    int own_rng = 0;
    Rand31 rng;
};

Ctx g_default;
thread_local Ctx *t_ctx = nullptr;
inline Ctx *cur() { return t_ctx ? t_ctx : &g_default; }

int g_inited = 0;
int g_num_sms = 0;
std::atomic<long long> g_launches{0};

}  // namespace

extern "C" void irwls_set_error(int code, const char *fmt, ...) {
    Ctx *c = cur();
    if (c->err < 0) return;  // keep the first error (an error replaces a warning)
    c->err = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->msg, sizeof c->msg, fmt, ap);
    va_end(ap);
}
// A warning (positive code): the call returns its result, and the condition
// is reported unless an error or an earlier warning is already recorded.
extern "C" void irwls_set_warning(int code, const char *fmt, ...) {
    Ctx *c = cur();
    if (c->err) return;
    c->err = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->msg, sizeof c->msg, fmt, ap);
    va_end(ap);
}
extern "C" int irwls_get_error(void) { return cur()->err; }
extern "C" const char *irwls_get_error_message(void) { return cur()->msg; }
extern "C" void irwls_clear_error(void) {
    cur()->err = 0;
    cur()->msg[0] = 0;
}

cudaStream_t irwls_stream() { return cur()->stream; }
int *irwls_dev_flags() { return cur()->flags; }
int irwls_num_sms() { return g_num_sms; }

extern "C" long long irwls_launch_count(void) { return g_launches.load(); }
extern "C" void irwls_count_launch(int n) { g_launches += n; }

static int cuda_fail(cudaError_t e, const char *what) {
    irwls_set_error(-2, "CUDA error in %s: %s", what, cudaGetErrorString(e));
    return -2;
}

int irwls_check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return 0;
}

static int ctx_open(Ctx *c) {
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamCreate");
    if ((e = cudaMalloc((void **)&c->flags, 8 * sizeof(int))) != cudaSuccess) return cuda_fail(e, "flags alloc");
    if ((e = cudaMemset(c->flags, 0, 8 * sizeof(int))) != cudaSuccess) return cuda_fail(e, "flags init");
    return 0;
}

extern "C" int irwls_dev_init(void) {
    if (g_inited) return 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        irwls_set_error(-1, "no CUDA device available (%s); this library has no CPU path",
                        e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        return -1;
    }
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if ((e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return cuda_fail(e, "cudaDeviceGetAttribute");
    if (ctx_open(&g_default)) return -2;
    g_inited = 1;
    return 0;
}

// Execution contexts of worker threads (the library must be initialised).
extern "C" void *irwls_ctx_create(void) {
    if (irwls_dev_init()) return nullptr;
    Ctx *c = new Ctx();
    if (ctx_open(c)) {
        delete c;
        return nullptr;
    }
    c->own_rng = 1;
    c->rng.seed(1);
    return c;
}
extern "C" void irwls_ctx_bind(void *h) { t_ctx = (Ctx *)h; }
extern "C" void irwls_ctx_destroy(void *h) {
    Ctx *c = (Ctx *)h;
    if (!c) return;
    cudaStreamSynchronize(c->stream);
    for (int k = 0; k < IRWLS_SCRATCH_SLOTS; ++k)
        if (c->scratch[k]) cudaFreeAsync(c->scratch[k], c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(c->flags);
    cudaStreamDestroy(c->stream);
    delete c;
}
// Error of a context (for the thread that created it, after a worker ended).
extern "C" int irwls_ctx_error(void *h, char *msg, int cap) {
    Ctx *c = (Ctx *)h;
    if (msg && cap > 0) snprintf(msg, (size_t)cap, "%s", c->msg);
    return c->err;
}

// The current context's random numbers: libc rand() in the default context,
// the context's own glibc-equivalent generator in worker contexts.
extern "C" void irwls_srand(unsigned seed) {
    Ctx *c = cur();
    if (c->own_rng) c->rng.seed(seed);
    else srand(seed);
}
extern "C" int irwls_rand(void) {
    Ctx *c = cur();
    return c->own_rng ? c->rng.next() : rand();
}
// n numbers of a private generator seeded with `seed` (tests compare them
// with libc's srand/rand).
extern "C" void irwls_rand_sequence(unsigned seed, int n, int *out) {
    Rand31 g;
    g.seed(seed);
    for (int i = 0; i < n; ++i) out[i] = g.next();
}

// Allocation-failure injection for tests of the error paths: armed with
// n > 0, the n-th device or pinned-host allocation of the library from then
// on fails as if the runtime had refused it (nothing is allocated).
static std::atomic<long long> g_fail_alloc{0};
extern "C" void irwls_debug_fail_alloc(long long n) { g_fail_alloc.store(n > 0 ? n : 0); }
static bool injected_alloc_failure() {
    long long v = g_fail_alloc.load();
    while (v > 0)
        if (g_fail_alloc.compare_exchange_weak(v, v - 1)) return v == 1;
    return false;
}

// Grow-only scratch buffer `slot` of the current context (stream-ordered).
extern "C" void *irwls_ctx_scratch(int slot, size_t bytes) {
    Ctx *c = cur();
    if (bytes > c->scratch_bytes[slot]) {
        if (c->scratch[slot]) cudaFreeAsync(c->scratch[slot], c->stream);
        c->scratch[slot] = nullptr;
        c->scratch_bytes[slot] = 0;
        if (injected_alloc_failure()) {
            irwls_set_error(-3, "device scratch of %zu bytes failed (injected failure)", bytes);
            return nullptr;
        }
        if (cudaMallocAsync(&c->scratch[slot], bytes, c->stream) != cudaSuccess) {
            cudaGetLastError();
            irwls_set_error(-3, "device scratch of %zu bytes failed", bytes);
            return nullptr;
        }
        c->scratch_bytes[slot] = bytes;
    }
    return c->scratch[slot];
}

extern "C" int irwls_dev_sync(void) {
    cudaError_t e = cudaStreamSynchronize(cur()->stream);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
    return 0;
}

extern "C" int irwls_dev_malloc(void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    if (injected_alloc_failure()) {
        irwls_set_error(-3, "device allocation of %zu bytes failed (injected failure)", bytes);
        return -3;
    }
    cudaError_t e = cudaMallocAsync(p, bytes, cur()->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        irwls_set_error(-3, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        *p = nullptr;
        return -3;
    }
    return 0;
}
extern "C" int irwls_dev_free(void *p) {
    if (p) cudaFreeAsync(p, cur()->stream);
    return 0;
}
extern "C" void irwls_count_bytes(long long h2d, long long d2h);
extern "C" int irwls_dev_h2d(void *d, const void *h, size_t bytes) {
    if (!bytes) return 0;
    irwls_count_bytes((long long)bytes, 0);
    cudaError_t e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, cur()->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "H2D copy");
}
extern "C" int irwls_dev_d2h(void *h, const void *d, size_t bytes) {
    if (!bytes) return 0;
    irwls_count_bytes(0, (long long)bytes);
    cudaError_t e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, cur()->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "D2H copy");
}
extern "C" int irwls_dev_d2d(void *d, const void *s, size_t bytes) {
    if (!bytes) return 0;
    cudaError_t e = cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, cur()->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "D2D copy");
}
extern "C" int irwls_dev_memset(void *d, int byte, size_t bytes) {
    if (!bytes) return 0;
    cudaError_t e = cudaMemsetAsync(d, byte, bytes, cur()->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "memset");
}
extern "C" int irwls_dev_host_alloc(void **p, size_t bytes) {
    if (injected_alloc_failure()) {
        *p = nullptr;
        irwls_set_error(-3, "pinned host allocation of %zu bytes failed (injected failure)", bytes);
        return -3;
    }
    cudaError_t e = cudaMallocHost(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMallocHost");
    }
    return 0;
}
extern "C" void irwls_dev_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

extern "C" int irwls_dev_workspace(size_t bytes, void **d_ws) {
    *d_ws = irwls_ctx_scratch(1, bytes);
    return *d_ws ? 0 : -3;
}
extern "C" void irwls_dev_release_workspace(void) {
    Ctx *c = cur();
    if (c->scratch[1]) cudaFreeAsync(c->scratch[1], c->stream);
    c->scratch[1] = nullptr;
    c->scratch_bytes[1] = 0;
}

// ---------------------------------------------------------------------------
// Dataset upload. Rows are walked on the host exactly as the reference walks
// its svm_sample lists; the device keeps a dense copy (raw values for the
// raw-RBF mode, values by feature index otherwise) plus CSR by feature index.
// ---------------------------------------------------------------------------
extern "C" int irwls_feature_width(const svm_dataset *ds, int n_rows) {
    int w = 1;
    for (int i = 0; i < n_rows; ++i)
        for (const svm_sample *p = ds->x[i]; p->index != -1; ++p)
            if (p->index + 1 > w) w = p->index + 1;
    return w;
}
extern "C" int irwls_model_feature_width(const model *m) {
    int w = 1;
    for (int i = 0; i < m->nSVs; ++i)
        for (const svm_sample *p = m->x[i]; p->index != -1; ++p)
            if (p->index + 1 > w) w = p->index + 1;
    return w;
}

// Training needs finite labels (prediction does not read them, so its
// datasets are not checked).
extern "C" int irwls_check_labels(const svm_dataset *ds, int n_rows) {
    for (int i = 0; i < n_rows; ++i)
        if (!isfinite(ds->y[i])) {
            irwls_set_error(-4, "non-finite label %g in row %d", ds->y[i], i);
            return -4;
        }
    return 0;
}

// csr_only: no dense copy X (for consumers that read the rows as CSR only).
static int upload_rows(svm_sample *const *rows, const double *q, const double *y, int n_rows, int mode,
                       double gamma, int raw_width, int width_hint, irwls_dev_set *out, int csr_only = 0) {
    memset(out, 0, sizeof *out);
    if (irwls_dev_init()) return -1;
    out->n_rows = n_rows;
    out->mode = mode;
    out->neg_gamma = -gamma;
    long long nnz = 0;
    int width = 1;
    for (int i = 0; i < n_rows; ++i)
        for (const svm_sample *p = rows[i]; p->index != -1; ++p) {
            ++nnz;
            if (p->index < 0) {
                irwls_set_error(-4, "negative feature index %d in row %d", p->index, i);
                return -4;
            }
            if (!isfinite(p->value)) {
                irwls_set_error(-4, "non-finite value %g of feature %d in row %d", p->value, p->index, i);
                return -4;
            }
            if (p->index + 1 > width) width = p->index + 1;
        }
    if (width_hint > width) width = width_hint;
    if (mode == IRWLS_K_RAW_RBF) width = raw_width > 0 ? raw_width : 1;
    out->width = width;
    out->ld = (width + 1) & ~1;
    out->nnz = nnz;
    if (nnz > 2147483647LL) {
        irwls_set_error(-4, "dataset has %lld stored entries; the device layout indexes them with int32", nnz);
        return -4;
    }
    const size_t xbytes = csr_only ? 0 : (size_t)n_rows * out->ld * sizeof(double);
    const size_t bytes = xbytes + (size_t)(n_rows + 1) * sizeof(int) + (size_t)nnz * (sizeof(int) + sizeof(double)) +
                         2 * (size_t)n_rows * sizeof(double);
    void *h = nullptr;
    if (irwls_dev_host_alloc(&h, bytes)) return -3;
    double *hX = (double *)h;
    double *hq = hX + xbytes / sizeof(double);
    double *hy = hq + n_rows;
    double *hcv = hy + n_rows;
    int *hrp = (int *)(hcv + nnz);
    int *hci = hrp + n_rows + 1;
    memset(hX, 0, xbytes);
    long long k = 0;
    for (int i = 0; i < n_rows; ++i) {
        hrp[i] = (int)k;
        double *row = csr_only ? nullptr : hX + (size_t)i * out->ld;
        if (row && mode == IRWLS_K_RAW_RBF) {
            // maxdim consecutive values from the row start, as src/kernels.c:93-97 reads them
            const svm_sample *p = rows[i];
            for (int t = 0; t < raw_width; ++t) row[t] = p[t].value;
        }
        for (const svm_sample *p = rows[i]; p->index != -1; ++p) {
            if (row && mode != IRWLS_K_RAW_RBF) row[p->index] = p->value;
            hci[k] = p->index;
            hcv[k] = p->value;
            ++k;
        }
        hq[i] = q ? q[i] : 0.0;
        hy[i] = y ? y[i] : 0.0;
    }
    hrp[n_rows] = (int)k;
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&out->X, xbytes);
    rc |= irwls_dev_malloc((void **)&out->q, n_rows * sizeof(double));
    rc |= irwls_dev_malloc((void **)&out->y, n_rows * sizeof(double));
    rc |= irwls_dev_malloc((void **)&out->rp, (n_rows + 1) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&out->ci, (nnz ? nnz : 1) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&out->cv, (nnz ? nnz : 1) * sizeof(double));
    if (!rc) {
        rc |= irwls_dev_h2d(out->X, hX, xbytes);
        rc |= irwls_dev_h2d(out->q, hq, n_rows * sizeof(double));
        rc |= irwls_dev_h2d(out->y, hy, n_rows * sizeof(double));
        rc |= irwls_dev_h2d(out->rp, hrp, (n_rows + 1) * sizeof(int));
        rc |= irwls_dev_h2d(out->ci, hci, nnz * sizeof(int));
        rc |= irwls_dev_h2d(out->cv, hcv, nnz * sizeof(double));
    }
    // the staging buffer is pinned: wait for the copies before freeing it
    rc |= irwls_dev_sync();
    irwls_dev_host_free(h);
    if (rc) {
        irwls_dev_release(out);
        return rc ? rc : -3;
    }
    return 0;
}

// The rows of ds as CSR only (no dense copy): for the linear prediction path.
extern "C" int irwls_dev_upload_csr(const svm_dataset *ds, int n_rows, int kernelType, double gamma, int width_hint,
                                    irwls_dev_set *out) {
    const int mode = kernelType == 0 ? IRWLS_K_LINEAR : IRWLS_K_NORM_RBF;
    return upload_rows(ds->x, ds->quadratic_value, ds->y, n_rows, mode, gamma, ds->maxdim, width_hint, out, 1);
}

extern "C" int irwls_dev_upload(const svm_dataset *ds, int n_rows, int kernelType, double gamma, int force_norm,
                                int width_hint, irwls_dev_set *out) {
    int mode = kernelType == 0 ? IRWLS_K_LINEAR
                               : ((ds->sparse == 0 && !force_norm) ? IRWLS_K_RAW_RBF : IRWLS_K_NORM_RBF);
    return upload_rows(ds->x, ds->quadratic_value, ds->y, n_rows, mode, gamma, ds->maxdim, width_hint, out);
}

extern "C" int irwls_dev_upload_model(const model *m, int width_hint, irwls_dev_set *out) {
    int mode = m->kernelType == 0 ? IRWLS_K_LINEAR : IRWLS_K_NORM_RBF;
    return upload_rows(m->x, m->quadratic_value, nullptr, m->nSVs, mode, m->Kgamma, m->maxdim, width_hint, out);
}

extern "C" void irwls_dev_release(irwls_dev_set *s) {
    if (!s) return;
    void *b[] = {s->X, s->q, s->y, s->rp, s->ci, s->cv};
    for (void *p : b) irwls_dev_free(p);
    memset(s, 0, sizeof *s);
}

// ---------------------------------------------------------------------------
// Timing of selected kernels with CUDA events on the library stream.
// ---------------------------------------------------------------------------
struct ProfSlot {
    std::vector<cudaEvent_t> pending;  // begin/end pairs not yet read
    std::vector<cudaEvent_t> pool;
    double ms = 0.0;
    long long launches = 0;
};
static ProfSlot g_prof[IRWLS_PROF_SLOTS];
static int g_prof_on = 0;

static cudaEvent_t prof_event(ProfSlot &s) {
    if (!s.pool.empty()) {
        cudaEvent_t e = s.pool.back();
        s.pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
// Kernel timing is recorded in the default context only.
extern "C" void irwls_prof_enable(int on) { g_prof_on = on; }
extern "C" int irwls_prof_on(void) { return g_prof_on && !t_ctx; }
extern "C" void irwls_prof_begin(int slot) {
    if (!irwls_prof_on()) return;
    ProfSlot &s = g_prof[slot];
    cudaEvent_t e = prof_event(s);
    cudaEventRecord(e, g_default.stream);
    s.pending.push_back(e);
}
extern "C" void irwls_prof_end(int slot) {
    if (!irwls_prof_on()) return;
    ProfSlot &s = g_prof[slot];
    cudaEvent_t e = prof_event(s);
    cudaEventRecord(e, g_default.stream);
    s.pending.push_back(e);
    if (s.pending.size() > 4096) irwls_prof_collect();
}
extern "C" int irwls_prof_collect(void) {
    cudaStreamSynchronize(g_default.stream);
    for (auto &s : g_prof) {
        for (size_t i = 0; i + 1 < s.pending.size(); i += 2) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, s.pending[i], s.pending[i + 1]);
            s.ms += ms;
            s.launches += 1;
            s.pool.push_back(s.pending[i]);
            s.pool.push_back(s.pending[i + 1]);
        }
        s.pending.clear();
    }
    return 0;
}
extern "C" void irwls_prof_read(int slot, double *ms, long long *launches) {
    *ms = g_prof[slot].ms;
    *launches = g_prof[slot].launches;
}
extern "C" void irwls_prof_reset(void) {
    irwls_prof_collect();
    for (auto &s : g_prof) {
        s.ms = 0.0;
        s.launches = 0;
    }
}

extern "C" int irwls_dev_chol_info(int *info) {
    int flags[8];
    cudaError_t e = cudaMemcpyAsync(flags, cur()->flags, sizeof flags, cudaMemcpyDeviceToHost, cur()->stream);
    if (e != cudaSuccess) return cuda_fail(e, "read flags");
    if (irwls_dev_sync()) return -2;
    *info = flags[0];
    return 0;
}

// ---------------------------------------------------------------------------
// Benchmark support: transfer counters, L2 flush, stream timers and a probe of
// the device's FP64 FMA throughput (the roofline denominator of the FP64
// kernels: chains of independent DFMAs, no memory traffic).
// ---------------------------------------------------------------------------
static std::atomic<long long> g_h2d{0}, g_d2h{0};
extern "C" void irwls_count_bytes(long long h2d, long long d2h) {
    g_h2d += h2d;
    g_d2h += d2h;
}
extern "C" void irwls_transfer_bytes(long long *h2d, long long *d2h) {
    *h2d = g_h2d.load();
    *d2h = g_d2h.load();
}

static void *g_flush = nullptr;
extern "C" int irwls_l2_flush(size_t bytes) {
    if (irwls_dev_init()) return -1;
    if (!g_flush && irwls_dev_malloc(&g_flush, bytes)) return -3;
    return irwls_dev_memset(g_flush, 0x5a, bytes);
}

static cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
extern "C" int irwls_timer_start(void) {
    if (irwls_dev_init()) return -1;
    if (!g_t0) {
        cudaEventCreate(&g_t0);
        cudaEventCreate(&g_t1);
    }
    cudaEventRecord(g_t0, cur()->stream);
    return 0;
}
extern "C" double irwls_timer_stop(void) {
    cudaEventRecord(g_t1, cur()->stream);
    cudaEventSynchronize(g_t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g_t0, g_t1);
    return ms;
}

namespace {
__global__ void fp64_probe_kernel(double *out, int iters) {
    double a[8];
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3 + k;
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0;
    for (int k = 0; k < 8; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void fp32_probe_kernel(float *out, int iters) {
    float a[8];
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3f + k;
    const float b = 0.9999f, c = 1e-4f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
    }
    float s = 0;
    for (int k = 0; k < 8; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

// FP32 FMA throughput in TFLOP/s (one FMA = 2 flops), best of `reps` timed
// launches: the FP32-issue ceiling reported beside the tensor-core kernels.
extern "C" double irwls_fp32_peak_tflops(int reps) {
    if (irwls_dev_init()) return 0.0;
    const int blocks = 4 * g_num_sms, threads = 256, iters = 100000;
    float *d = nullptr;
    if (irwls_dev_malloc((void **)&d, (size_t)blocks * threads * sizeof(float))) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    fp32_probe_kernel<<<blocks, threads, 0, cur()->stream>>>(d, iters);
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, cur()->stream);
        fp32_probe_kernel<<<blocks, threads, 0, cur()->stream>>>(d, iters);
        cudaEventRecord(e1, cur()->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    irwls_dev_free(d);
    irwls_dev_sync();
    return best;
}

// FP64 FMA throughput in TFLOP/s, best of `reps` timed launches.
extern "C" double irwls_fp64_peak_tflops(int reps) {
    if (irwls_dev_init()) return 0.0;
    const int blocks = 4 * g_num_sms, threads = 256, iters = 20000;
    double *d = nullptr;
    if (irwls_dev_malloc((void **)&d, (size_t)blocks * threads * sizeof(double))) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    fp64_probe_kernel<<<blocks, threads, 0, cur()->stream>>>(d, iters);
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, cur()->stream);
        fp64_probe_kernel<<<blocks, threads, 0, cur()->stream>>>(d, iters);
        cudaEventRecord(e1, cur()->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    irwls_dev_free(d);
    irwls_dev_sync();
    return best;
}
