// dev_parse.cu -- the libsvm reader on the GPU (reference readTrainFile,
// src/IOStructures.c:88-275): the text of the file is parsed on the device
// into exactly the svm_dataset the reference's reader builds.
//
// The reference reads each line with fgets into a 100000-byte buffer and
// tokenises it with strtok: a first pass (delimiters " \t" for the label,
// then ":" and " \t" alternately, stopping at a NULL token or one that starts
// with '\n') counts the entries and the largest index; the second pass takes
// the label with " \t\n", then index/value pairs until the value token is
// NULL, converting them with strtol and strtod and failing on a malformed
// number, a non-increasing index or a missing label. The device replays both
// passes per line (one thread per line) without modifying the text: a token
// is a [start, end) range, and the NUL that strtok writes over a delimiter is
// the end of that range.
//
// Numbers: strtod of the C library is correctly rounded, so the device
// conversion is exact too: the decimal is read as w * 10^q with up to 19
// significant digits; w <= 2^53 with |q| <= 22 takes one IEEE multiply or
// divide by an exact power of ten; everything else goes through big-integer
// arithmetic (w * 5^q, or a long division by 5^-q, rounded to nearest even
// at the precision of the result, subnormals included). A decimal with more
// than 19 significant digits is decided from its first 19 when both bounds
// of its interval round to the same double; when they do not, and for
// hexadecimal numbers and NaN payloads, the reader reports the line as
// unsupported instead of guessing.
//
// The O(bytes) work (line search, both passes, every conversion, the row
// norms) runs on the device; the class-mean rows and the row pointers, whose
// sums must follow the reference's row order, are assembled on the host from
// the parsed rows (irwls_dataset_assemble in io.c).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "dev_common.cuh"
#include "irwls_gpu.h"
#include "numparse.cuh"

extern "C" int irwls_dataset_alloc(svm_dataset *ds, int l, long long pass1_elements, int maxidx,
                                   long long row_entries);
extern "C" int irwls_dataset_finish(svm_dataset *ds, int l, int maxidx, int max_index, int sparse,
                                    long long row_entries, const long long *row_start, const double *y,
                                    const double *q);

namespace {

constexpr int LINE_CHARS = 100000 - 1;  // fgets(line, 100000, f) reads at most this many bytes

// ---- strtok over one line ----------------------------------------------------

enum { D_SPTAB = 1, D_SPTABNL = 2, D_COLON = 3 };

__device__ __forceinline__ bool is_delim(char c, int set) {
    if (set == D_COLON) return c == ':';
    if (set == D_SPTAB) return c == ' ' || c == '\t';
    return c == ' ' || c == '\t' || c == '\n';
}

// The next strtok token of the line b[.., le) from cursor pos (le: where the
// line's string ends). Returns false for NULL; else [ts, te) with the cursor
// past the delimiter that ended it (or at le).
__device__ bool next_tok(const char *b, int &pos, int le, int set, int &ts, int &te) {
    int p = pos;
    while (p < le && is_delim(b[p], set)) ++p;
    if (p >= le) {
        pos = le;
        return false;
    }
    ts = p;
    while (p < le && !is_delim(b[p], set)) ++p;
    te = p;
    pos = p < le ? p + 1 : le;
    return true;
}

// Where the line's C string ends: its first NUL, or its end.
__device__ int line_end(const char *b, int ls, int le) {
    for (int p = ls; p < le; ++p)
        if (b[p] == 0) return p;
    return le;
}

// ---- kernels -----------------------------------------------------------------

constexpr int CHUNK = 16384;  // bytes per block when searching newlines

// Newline bytes of a 4-byte word: __vcmpeq4 sets 0xff in each matching byte.
__device__ __forceinline__ int nl_in_word(uint32_t w) { return __popc(__vcmpeq4(w, 0x0a0a0a0au)) >> 3; }

// Newlines per chunk. A whole chunk on a 16-byte boundary is read in 16-byte
// loads; the last, partial chunk byte by byte, so no load passes the end of
// the text.
__global__ void nl_count_kernel(const char *__restrict__ b, long long len, int *__restrict__ cnt) {
    const long long c0 = (long long)blockIdx.x * CHUNK;
    int n = 0;
    if (len - c0 >= CHUNK && ((uintptr_t)(b + c0) & 15) == 0) {
        const uint4 *p4 = (const uint4 *)(b + c0);
        for (int j = threadIdx.x; j < CHUNK / 16; j += blockDim.x) {
            const uint4 v = p4[j];
            n += nl_in_word(v.x) + nl_in_word(v.y) + nl_in_word(v.z) + nl_in_word(v.w);
        }
    } else {
        for (long long p = c0 + threadIdx.x; p < min(len, c0 + CHUNK); p += blockDim.x) n += b[p] == '\n';
    }
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    __shared__ int ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += ws[k];
        cnt[blockIdx.x] = t;
    }
}

// Newline positions of each chunk, in order: thread k scans the chunk's k-th
// slice of CHUNK / blockDim bytes. A 64-byte slice inside the text (on a
// 16-byte boundary) is held in registers from four 16-byte loads; the slice
// holding the end of the text is read byte by byte.
__global__ void nl_write_kernel(const char *__restrict__ b, long long len, const long long *__restrict__ off,
                                long long *__restrict__ nl) {
    const int per = CHUNK / blockDim.x;
    const long long s0 = (long long)blockIdx.x * CHUNK + (long long)threadIdx.x * per;
    const bool whole = per == 64 && len - s0 >= 64 && ((uintptr_t)(b + s0) & 15) == 0;
    uint32_t wv[16];
    int n = 0;
    if (whole) {
        const uint4 *p4 = (const uint4 *)(b + s0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint4 v = p4[j];
            wv[4 * j] = v.x;
            wv[4 * j + 1] = v.y;
            wv[4 * j + 2] = v.z;
            wv[4 * j + 3] = v.w;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) n += nl_in_word(wv[j]);
    } else {
        for (long long p = s0; p < min(len, s0 + per); ++p) n += b[p] == '\n';
    }
    __shared__ int pre[1024];
    pre[threadIdx.x] = n;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        const int v = threadIdx.x >= (unsigned)o ? pre[threadIdx.x - o] : 0;
        __syncthreads();
        pre[threadIdx.x] += v;
        __syncthreads();
    }
    long long k = off[blockIdx.x] + pre[threadIdx.x] - n;
    if (whole) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            uint32_t m = __vcmpeq4(wv[j], 0x0a0a0a0au);  // little-endian: byte i is bits 8i .. 8i + 7
            while (m) {
                const int bit = __ffs(m) - 1;
                nl[k++] = s0 + 4 * j + (bit >> 3);
                m &= ~(0xffu << bit);
            }
        }
    } else {
        for (long long p = s0; p < min(len, s0 + per); ++p)
            if (b[p] == '\n') nl[k++] = p;
    }
}

struct LineSet {
    const char *b;
    const long long *nl;  // newline positions
    long long nnl;        // newlines
    long long len;
};

__device__ __forceinline__ void line_range(const LineSet &L, long long i, long long &ls, long long &le) {
    ls = i == 0 ? 0 : L.nl[i - 1] + 1;
    le = i < L.nnl ? L.nl[i] + 1 : L.len;  // the newline belongs to the line, as fgets keeps it
}

// Pass 1 of the reference (elements and the largest index) and the line
// length check. lcnt[i] = the line's index:value tokens, the slot that pass 2
// writes the line's entries into (pass 2 checks that the counts agree).
__global__ void pass1_kernel(LineSet L, long long nlines, unsigned long long *__restrict__ elements,
                             int *__restrict__ maxidx, int *__restrict__ err, int *__restrict__ lcnt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nlines;
         i += (long long)gridDim.x * blockDim.x) {
        long long ls, le0;
        line_range(L, i, ls, le0);
        if (le0 - ls > LINE_CHARS) {
            atomicMin(err, -3);  // the reference would split the line into several rows
            lcnt[i] = 0;
            continue;
        }
        const char *b = L.b + ls;
        const int le = line_end(b, 0, (int)(le0 - ls));
        int pos = 0, ts, te, is, ie;
        next_tok(b, pos, le, D_SPTAB, ts, te);
        unsigned long long el = 1;
        int mx = 0;
        for (;;) {
            const bool hi = next_tok(b, pos, le, D_COLON, is, ie);
            const bool ht = next_tok(b, pos, le, D_SPTAB, ts, te);
            if (!ht || b[ts] == '\n') break;
            int end;
            const int k = hi ? dev_strtol(b, is, ie, &end) : 0;
            mx = max(mx, k);
            ++el;
        }
        atomicAdd(elements, el);
        atomicMax(maxidx, mx);
        lcnt[i] = (int)min(el - 1, (unsigned long long)LINE_CHARS);
    }
}

// Pass 2 of the reference: the checks, the entry count per line, and (when
// rows != null) the entries, the label, the row norm and the row's largest
// index. err: the first failing line * 4 + kind (1 format, 2 unsupported).
// Line i's entries and terminator go to the slot [row_start[i],
// row_start[i + 1]); writes stay inside it, and a line whose entry count is
// not the slot's sets *mismatch (the rows are then laid out again from this
// pass's counts).
__global__ void pass2_kernel(LineSet L, long long nlines, const long long *__restrict__ row_start,
                             svm_sample *__restrict__ rows, double *__restrict__ y, double *__restrict__ q,
                             int *__restrict__ cnt, int *__restrict__ rmax, long long *__restrict__ err,
                             int *__restrict__ mismatch) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nlines;
         i += (long long)gridDim.x * blockDim.x) {
        long long ls, le0;
        line_range(L, i, ls, le0);
        const char *b = L.b + ls;
        const int le = line_end(b, 0, (int)(le0 - ls));
        int pos = 0, ts, te, is, ie;
        int kind = 0;
        if (!next_tok(b, pos, le, D_SPTABNL, ts, te)) kind = 1;
        double label = 0.0;
        if (!kind) {
            int un;
            const int end = dev_strtod(b, ts, te, &label, &un);
            if (end == ts || end != te) kind = 1;
            else if (un) kind = 2;
        }
        int n = 0, row_max = -1;
        double qq = 0.0;
        const long long base = rows ? row_start[i] : 0;
        const int cap = rows ? (int)(row_start[i + 1] - base - 1) : 0;
        while (!kind) {
            const bool hi = next_tok(b, pos, le, D_COLON, is, ie);
            if (!next_tok(b, pos, le, D_SPTAB, ts, te)) break;
            int end;
            const int k = hi ? dev_strtol(b, is, ie, &end) : 0;
            if (!hi || end == is || end != ie || k <= row_max) {
                kind = 1;
                break;
            }
            row_max = k;
            double v;
            int un;
            const int ve = dev_strtod(b, ts, te, &v, &un);
            if (ve == ts || (ve != te && !is_space(b[ve]))) {
                kind = 1;
                break;
            }
            if (un) {
                kind = 2;
                break;
            }
            qq = __dadd_rn(qq, __dmul_rn(v, v));
            if (rows && n < cap) {
                rows[base + n].index = k;
                rows[base + n].value = v;
            }
            ++n;
        }
        if (kind) {
            atomicMin((unsigned long long *)err, (unsigned long long)(i * 4 + kind));
            continue;
        }
        cnt[i] = n;
        if (rows) {
            if (n != cap) atomicExch(mismatch, 1);
            rows[base + min(n, cap)].index = -1;
            rows[base + min(n, cap)].value = 0.0;
            y[i] = label;
            q[i] = qq;
            rmax[i] = row_max;
        }
    }
}

// The reference's sparse flag: set when the entry at position dm of a row
// has another index than the entry at position dm of the whole array.
__global__ void sparse_kernel(const svm_sample *__restrict__ rows, const long long *__restrict__ row_start,
                              long long nlines, int *__restrict__ sparse) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nlines;
         i += (long long)gridDim.x * blockDim.x) {
        const long long j0 = row_start[i];
        for (long long j = j0; rows[j].index != -1; ++j)
            if (rows[j - j0].index != rows[j].index) {
                atomicExch(sparse, 1);
                break;
            }
    }
}

// Numbers one per line through dev_strtod (the conversion checks).
__global__ void parse_doubles_kernel(LineSet L, long long nlines, double *__restrict__ out, int *__restrict__ status) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nlines;
         i += (long long)gridDim.x * blockDim.x) {
        long long ls, le0;
        line_range(L, i, ls, le0);
        const char *b = L.b + ls;
        int le = line_end(b, 0, (int)(le0 - ls));
        if (le > 0 && b[le - 1] == '\n') --le;
        double v;
        int un;
        const int end = dev_strtod(b, 0, le, &v, &un);
        out[i] = v;
        status[i] = end == 0 ? -1 : (un ? 2 : (end == le ? 0 : 1));
    }
}

// Lines of a buffer already on the device: newline positions and the count.
int find_lines(const char *d_text, long long len, long long **d_nl, long long *nnl, long long *nlines) {
    const long long nch = len > 0 ? (len + CHUNK - 1) / CHUNK : 0;
    *d_nl = nullptr;
    *nnl = 0;
    *nlines = 0;
    if (nch == 0) return 0;
    int *d_cnt = nullptr;
    long long *d_off = nullptr;
    if (irwls_dev_malloc((void **)&d_cnt, nch * sizeof(int))) return -3;
    nl_count_kernel<<<(int)nch, 256, 0, irwls_stream()>>>(d_text, len, d_cnt);
    IRWLS_LAUNCH_CHECK("nl_count");
    std::vector<int> cnt(nch);
    std::vector<long long> off(nch);
    if (irwls_dev_d2h(cnt.data(), d_cnt, nch * sizeof(int)) || irwls_dev_sync()) return -1;
    long long t = 0;
    for (long long k = 0; k < nch; ++k) {
        off[k] = t;
        t += cnt[k];
    }
    *nnl = t;
    int rc = irwls_dev_malloc((void **)&d_off, nch * sizeof(long long));
    rc |= irwls_dev_malloc((void **)d_nl, (t > 0 ? t : 1) * sizeof(long long));
    if (rc) return -3;
    rc |= irwls_dev_h2d(d_off, off.data(), nch * sizeof(long long));
    nl_write_kernel<<<(int)nch, 256, 0, irwls_stream()>>>(d_text, len, d_off, *d_nl);
    IRWLS_LAUNCH_CHECK("nl_write");
    rc |= irwls_dev_sync();
    irwls_dev_free(d_cnt);
    irwls_dev_free(d_off);
    // a last line without a newline still counts, as fgets returns it
    long long last = -1;
    if (t > 0) rc |= irwls_dev_d2h(&last, *d_nl + (t - 1), sizeof(long long)) | irwls_dev_sync();
    *nlines = t + (last + 1 < len ? 1 : 0);
    return rc;
}

}  // namespace

// Parses the libsvm text buf[0, len) on the device into *ds, as the
// reference's readTrainFile parses a file with that content. Returns 0; or
// -20 (wrong file format, as the reference's "Wrong file format"), -21 (a
// number this reader does not convert exactly: hexadecimal, a NaN payload, an
// undecidable decimal of more than 19 digits), -22 (a line longer than the
// reference's 99999-byte line buffer), with the line number in the message.
extern "C" int irwls_parse_libsvm(const char *buf, size_t len, svm_dataset *ds) {
    irwls_clear_error();
    memset(ds, 0, sizeof *ds);
    if (irwls_dev_init()) return -1;
    const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
    char *d_text = nullptr;
    long long *d_nl = nullptr, *d_start = nullptr;
    unsigned long long *d_el = nullptr;
    int *d_maxidx = nullptr, *d_err1 = nullptr, *d_cnt = nullptr, *d_rmax = nullptr, *d_sparse = nullptr;
    int *d_mis = nullptr;
    long long *d_err2 = nullptr;
    svm_sample *d_rows = nullptr;
    double *d_y = nullptr, *d_q = nullptr;
    int rc = irwls_dev_malloc((void **)&d_text, len + 16);
    if (!rc && len) rc |= irwls_dev_h2d(d_text, buf, len);
    long long nnl = 0, n = 0;
    if (!rc) rc = find_lines(d_text, (long long)len, &d_nl, &nnl, &n);
    const LineSet L{d_text, d_nl, nnl, (long long)len};
    const int grid = (int)std::max<long long>(1, std::min<long long>((n + 127) / 128, 32LL * sms));
    unsigned long long elements = 0;
    int maxidx = 0, err1 = 0;
    long long err2 = 0x7fffffffffffffffLL;
    std::vector<int> cnt;
    std::vector<long long> start;
    if (!rc) {
        rc |= irwls_dev_malloc((void **)&d_el, sizeof(unsigned long long));
        rc |= irwls_dev_malloc((void **)&d_maxidx, sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_err1, sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_err2, sizeof(long long));
        rc |= irwls_dev_malloc((void **)&d_cnt, (n > 0 ? n : 1) * sizeof(int));
        rc |= irwls_dev_memset(d_el, 0, sizeof(unsigned long long));
        rc |= irwls_dev_memset(d_maxidx, 0, sizeof(int));
        rc |= irwls_dev_memset(d_err1, 0, sizeof(int));
        rc |= irwls_dev_h2d(d_err2, &err2, sizeof(long long));
    }
    if (!rc && n > 0) {
        if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PARSE);
        pass1_kernel<<<grid, 128, 0, irwls_stream()>>>(L, n, d_el, d_maxidx, d_err1, d_cnt);
        if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PARSE);
        irwls_count_launch(1);
        rc |= irwls_check_launch("pass1");
        cnt.resize(n);
        rc |= irwls_dev_d2h(&elements, d_el, sizeof elements);
        rc |= irwls_dev_d2h(&maxidx, d_maxidx, sizeof maxidx);
        rc |= irwls_dev_d2h(&err1, d_err1, sizeof err1);
        rc |= irwls_dev_d2h(cnt.data(), d_cnt, n * sizeof(int));
        rc |= irwls_dev_sync();
    }
    if (!rc && err1 < 0) {
        irwls_set_error(-22, "a line is longer than the reference's 99999-byte line buffer");
        rc = -22;
    }
    if (!rc) {
        rc |= irwls_dev_malloc((void **)&d_start, (n + 1) * sizeof(long long));
        rc |= irwls_dev_malloc((void **)&d_y, (n > 0 ? n : 1) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_q, (n > 0 ? n : 1) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_rmax, (n > 0 ? n : 1) * sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_sparse, sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_mis, sizeof(int));
        rc |= irwls_dev_memset(d_sparse, 0, sizeof(int));
    }
    // The rows are laid out from pass 1's entry counts and written by one
    // pass 2. On every line that pass 2 accepts the two passes stop at the
    // same token, so the counts agree; should a line's count differ all the
    // same, the layout is redone from pass 2's own counts (its count run,
    // then the write again).
    long long total = 0;
    for (int attempt = 0; !rc; ++attempt) {
        if (attempt == 1 && n > 0) {
            if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PARSE);
            pass2_kernel<<<grid, 128, 0, irwls_stream()>>>(L, n, nullptr, nullptr, nullptr, nullptr, d_cnt, nullptr,
                                                           d_err2, nullptr);
            if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PARSE);
            irwls_count_launch(1);
            rc |= irwls_check_launch("pass2 count");
            rc |= irwls_dev_d2h(cnt.data(), d_cnt, n * sizeof(int));
            rc |= irwls_dev_sync();
            if (rc) break;
        }
        start.assign(n + 1, 0);
        total = 0;
        for (long long i = 0; i < n; ++i) {
            start[i] = total;
            total += cnt[i] + 1;  // entries and the -1 terminator
        }
        start[n] = total;
        irwls_dev_free(d_rows);
        d_rows = nullptr;
        rc |= irwls_dev_malloc((void **)&d_rows, (total > 0 ? total : 1) * sizeof(svm_sample));
        rc |= irwls_dev_h2d(d_start, start.data(), (n + 1) * sizeof(long long));
        rc |= irwls_dev_memset(d_mis, 0, sizeof(int));
        if (rc || n == 0) break;
        int mis = 0;
        if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PARSE);
        pass2_kernel<<<grid, 128, 0, irwls_stream()>>>(L, n, d_start, d_rows, d_y, d_q, d_cnt, d_rmax, d_err2,
                                                       d_mis);
        if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PARSE);
        irwls_count_launch(1);
        rc |= irwls_check_launch("pass2 rows");
        rc |= irwls_dev_d2h(&err2, d_err2, sizeof err2);
        rc |= irwls_dev_d2h(&mis, d_mis, sizeof mis);
        rc |= irwls_dev_sync();
        if (rc || err2 != 0x7fffffffffffffffLL || !mis) break;
        if (attempt == 1) {
            irwls_set_error(-1, "libsvm reader: entry counts of pass 2 disagree between its two runs");
            rc = -1;
        }
    }
    if (!rc && err2 != 0x7fffffffffffffffLL) {
        const long long line = err2 / 4 + 1;
        if ((err2 & 3) == 1) {
            irwls_set_error(-20, "Wrong file format (line %lld)", line);
            rc = -20;
        } else {
            irwls_set_error(-21, "line %lld holds a number the device reader does not convert exactly", line);
            rc = -21;
        }
    }
    std::vector<double> y, q;
    std::vector<int> rmax;
    int sparse = 0;
    bool held = false;  // *ds holds host arrays
    if (!rc && n > 0) {
        if (irwls_prof_on()) irwls_prof_begin(IRWLS_PROF_PARSE);
        sparse_kernel<<<grid, 128, 0, irwls_stream()>>>(d_rows, d_start, n, d_sparse);
        if (irwls_prof_on()) irwls_prof_end(IRWLS_PROF_PARSE);
        irwls_count_launch(1);
        rc |= irwls_check_launch("sparse");
    }
    if (!rc) {
        // the rows go straight into the dataset's features array
        rc = irwls_dataset_alloc(ds, (int)n, (long long)elements, maxidx, total);
        held = rc == 0;
    }
    if (!rc && n > 0) {
        y.resize(n);
        q.resize(n);
        rmax.resize(n);
        rc |= irwls_dev_d2h(ds->features, d_rows, (size_t)total * sizeof(svm_sample));
        rc |= irwls_dev_d2h(y.data(), d_y, n * sizeof(double));
        rc |= irwls_dev_d2h(q.data(), d_q, n * sizeof(double));
        rc |= irwls_dev_d2h(rmax.data(), d_rmax, n * sizeof(int));
        rc |= irwls_dev_d2h(&sparse, d_sparse, sizeof(int));
        rc |= irwls_dev_sync();
    }
    void *bufs[] = {d_text, d_nl, d_start, d_el, d_maxidx, d_err1, d_cnt, d_rmax, d_sparse, d_err2, d_rows, d_y, d_q,
                    d_mis};
    for (void *p : bufs) irwls_dev_free(p);
    if (!rc) {
        int max_index = 0;
        for (long long i = 0; i < n; ++i) max_index = std::max(max_index, rmax[i]);
        rc = irwls_dataset_finish(ds, (int)n, maxidx, max_index, sparse, total, start.data(), y.data(), q.data());
    } else if (held) {
        freeDataset(*ds);
        memset(ds, 0, sizeof *ds);
    }
    return rc;
}

// readTrainFile on the device: the file's bytes are read once and parsed by
// irwls_parse_libsvm. On a format error it prints the reference's message
// and exits with status 2, as the reference's reader does.
extern "C" svm_dataset readTrainFileGPU(char filename[]) {
    svm_dataset ds;
    memset(&ds, 0, sizeof ds);
    FILE *f = fopen(filename, "rb");
    if (!f) {
        fprintf(stderr, "Error: file %s not found\n", filename);
        exit(2);
    }
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    void *h = nullptr;
    if (sz < 0 || irwls_dev_host_alloc(&h, (size_t)sz + 1)) {
        fclose(f);
        fprintf(stderr, "Error reading data file\n");
        exit(2);
    }
    const size_t got = fread(h, 1, (size_t)sz, f);
    fclose(f);
    const int rc = irwls_parse_libsvm((const char *)h, got, &ds);
    irwls_dev_host_free(h);
    if (rc == -20) {
        fprintf(stderr, "Wrong file format\n");
        exit(2);
    }
    if (rc) {
        fprintf(stderr, "%s\n", irwls_last_error_message());
        exit(2);
    }
    return ds;
}

// Numbers one per line (a trailing newline per line is allowed) converted by
// the device's strtod: out[i] the value, status[i] 0 (the whole line is the
// number), 1 (trailing text), -1 (no number), 2 (not converted exactly).
// Returns the number of lines, or a negative error.
extern "C" long long irwls_parse_doubles(const char *buf, size_t len, double *out, int *status, long long cap) {
    if (irwls_dev_init()) return -1;
    char *d_text = nullptr;
    long long *d_nl = nullptr;
    double *d_out = nullptr;
    int *d_st = nullptr;
    long long nnl = 0, n = 0;
    int rc = irwls_dev_malloc((void **)&d_text, len + 16);
    if (!rc && len) rc |= irwls_dev_h2d(d_text, buf, len);
    if (!rc) rc = find_lines(d_text, (long long)len, &d_nl, &nnl, &n);
    if (!rc && n > cap) {
        irwls_set_error(-4, "%lld lines for %lld outputs", n, cap);
        rc = -4;
    }
    if (!rc && n > 0) {
        rc |= irwls_dev_malloc((void **)&d_out, n * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_st, n * sizeof(int));
        const LineSet L{d_text, d_nl, nnl, (long long)len};
        const int sms = irwls_num_sms() > 0 ? irwls_num_sms() : 148;
        if (!rc) {
            parse_doubles_kernel<<<(int)std::min<long long>((n + 127) / 128, 32LL * sms), 128, 0, irwls_stream()>>>(
                L, n, d_out, d_st);
            irwls_count_launch(1);
        rc |= irwls_check_launch("parse_doubles");
            rc |= irwls_dev_d2h(out, d_out, n * sizeof(double));
            rc |= irwls_dev_d2h(status, d_st, n * sizeof(int));
            rc |= irwls_dev_sync();
        }
    }
    void *bufs[] = {d_text, d_nl, d_out, d_st};
    for (void *p : bufs) irwls_dev_free(p);
    return rc ? rc : n;
}
