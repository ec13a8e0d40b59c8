// numparse.cuh -- exact decimal-to-double (strtod) and strtol restated for
// the device libsvm reader (dev_parse.cu); host and device compile the same
// code, so the conversion can be checked against the C library on the host.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "pow5_table.cuh"

#ifdef __CUDACC__
#define NP_HD __host__ __device__
#else
#define NP_HD
#endif

NP_HD inline int np_clz(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __clz(v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}
NP_HD inline int np_clzll(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll(v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
NP_HD inline double np_bits_to_double(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}
// one IEEE multiply / divide, rounded to nearest even (never contracted)
NP_HD inline double np_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}
NP_HD inline double np_div(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    volatile double r = a / b;
    return r;
#endif
}

// ---- exact decimal to double ------------------------------------------------

constexpr int BL = 40;  // limbs (32-bit) of a big integer: 1280 bits

struct Big {
    uint32_t d[BL];
    int n;  // limbs in use; no leading zero limbs
};

NP_HD inline void bi_set(Big &a, uint64_t v) {
    a.d[0] = (uint32_t)v;
    a.d[1] = (uint32_t)(v >> 32);
    a.n = a.d[1] ? 2 : (a.d[0] ? 1 : 0);
}

NP_HD void bi_mul32(Big &a, uint32_t m) {
    uint64_t c = 0;
    for (int i = 0; i < a.n; ++i) {
        const uint64_t t = (uint64_t)a.d[i] * m + c;
        a.d[i] = (uint32_t)t;
        c = t >> 32;
    }
    if (c) a.d[a.n++] = (uint32_t)c;
}

NP_HD void bi_pow5_mul(Big &a, int k) {
    const uint32_t P13 = 1220703125u;  // 5^13
    while (k >= 13) {
        bi_mul32(a, P13);
        k -= 13;
    }
    uint32_t r = 1;
    while (k-- > 0) r *= 5;
    if (r > 1) bi_mul32(a, r);
}

NP_HD int bi_bitlen(const Big &a) { return a.n ? 32 * (a.n - 1) + (32 - np_clz(a.d[a.n - 1])) : 0; }

NP_HD void bi_shl(Big &a, int s) {
    if (!a.n || s <= 0) return;
    const int w = s >> 5, b = s & 31;
    int n = a.n + w + 1;
    for (int i = n - 1; i >= 0; --i) {
        const int src = i - w;
        uint32_t v = 0;
        if (src >= 0 && src < a.n) v = a.d[src] << b;
        if (b && src - 1 >= 0 && src - 1 < a.n) v |= a.d[src - 1] >> (32 - b);
        a.d[i] = v;
    }
    while (n > 0 && a.d[n - 1] == 0) --n;
    a.n = n;
}

NP_HD void bi_shr1(Big &a) {
    for (int i = 0; i < a.n; ++i) a.d[i] = (a.d[i] >> 1) | (i + 1 < a.n ? a.d[i + 1] << 31 : 0u);
    while (a.n > 0 && a.d[a.n - 1] == 0) --a.n;
}

NP_HD int bi_cmp(const Big &a, const Big &b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; --i)
        if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
}

NP_HD void bi_sub(Big &a, const Big &b) {  // a -= b, a >= b
    int64_t br = 0;
    for (int i = 0; i < a.n; ++i) {
        int64_t t = (int64_t)a.d[i] - (i < b.n ? (int64_t)b.d[i] : 0) - br;
        br = t < 0;
        a.d[i] = (uint32_t)(t + (br << 32));
    }
    while (a.n > 0 && a.d[a.n - 1] == 0) --a.n;
}

// Bits [sh, sh + 64) of a as an integer, the bit below them (half) and
// whether any bit below that is set (sticky).
NP_HD uint64_t bi_extract(const Big &a, int sh, int &half, int &sticky) {
    uint64_t v = 0;
    for (int k = 0; k < 64; ++k) {
        const int bit = sh + k;
        if (bit >= 0 && (bit >> 5) < a.n && ((a.d[bit >> 5] >> (bit & 31)) & 1u)) v |= 1ULL << k;
    }
    half = 0;
    sticky = 0;
    if (sh >= 1) {
        const int hb = sh - 1;
        half = (hb >> 5) < a.n ? (int)((a.d[hb >> 5] >> (hb & 31)) & 1u) : 0;
        for (int bit = 0; bit < hb && !sticky; ++bit)
            if ((bit >> 5) < a.n && ((a.d[bit >> 5] >> (bit & 31)) & 1u)) sticky = 1;
    }
    return v;
}

NP_HD inline int bitlen64(uint64_t v) { return v ? 64 - np_clzll(v) : 0; }

// ---- the interval step --------------------------------------------------------

// a * b as two 64-bit halves.
NP_HD inline void np_mul64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umul64hi(a, b);
#else
    const unsigned __int128 p = (unsigned __int128)a * b;
    lo = (uint64_t)p;
    hi = (uint64_t)(p >> 64);
#endif
}

// Y 2^k rounded to nearest even (subnormals and overflow included), Y the
// 256-bit integer y[3] .. y[0] with at least 54 significant bits. Returns
// false for a shorter Y.
NP_HD bool np_round_limbs(const uint64_t y[4], int k, double *out) {
    int L = 0;
    for (int i = 3; i >= 0 && !L; --i)
        if (y[i]) L = 64 * i + bitlen64(y[i]);
    if (L < 54) return false;
    int sh = L - 53;                       // lowest kept bit
    if (sh < -1074 - k) sh = -1074 - k;    // below the subnormal grid
    if (sh > L) {                          // under half the smallest subnormal
        *out = 0.0;
        return true;
    }
    const int i = sh >> 6, o = sh & 63;
    uint64_t m = i < 4 ? y[i] >> o : 0;
    if (o && i + 1 < 4) m |= y[i + 1] << (64 - o);
    const int hb = sh - 1, hi = hb >> 6, ho = hb & 63;
    const int half = (int)((y[hi] >> ho) & 1u);
    int sticky = (y[hi] & ((1ULL << ho) - 1)) != 0;
    for (int j = 0; j < hi && !sticky; ++j) sticky = y[j] != 0;
    if (half && (sticky || (m & 1))) ++m;
    *out = ldexp((double)m, sh + k);  // m <= 2^53: exact, or the overflow to infinity
    return true;
}

// w 10^q rounded to nearest even for w >= 1, through the table of 5^q:
// w 10^q = X 2^(q - lz + E_q - 127) with X = (w << lz) 5^q 2^(127 - E_q)
// (lz the leading zeros of w), and X lies in [A, A + (w << lz)), A =
// (w << lz) T_q, because 5^q 2^(127 - E_q) lies in [T_q, T_q + 1) (exactly
// T_q for 0 <= q <= 55). Rounding is monotone, so when both ends of that
// interval round to the same double, so does X. Returns false when they do
// not (X within 2^-73 of its rounding unit of a rounding boundary, or an
// exact tie) and for q outside the table.
NP_HD bool np_interval_round(uint64_t w, int q, double *out) {
    if (q < NP_POW5_QMIN || q > NP_POW5_QMAX) return false;
    const int t = q - NP_POW5_QMIN;
#ifdef __CUDA_ARCH__
    const uint64_t th = NP_POW5_D[t][0], tl = NP_POW5_D[t][1];
    const int e5 = NP_POW5_D_E[t];
#else
    const uint64_t th = NP_POW5_H[t][0], tl = NP_POW5_H[t][1];
    const int e5 = NP_POW5_H_E[t];
#endif
    const int lz = np_clzll(w);
    const uint64_t wn = w << lz;
    uint64_t p1h, p1l, p2h, p2l;
    np_mul64(wn, tl, p1h, p1l);
    np_mul64(wn, th, p2h, p2l);  // p2h <= 2^64 - 2
    uint64_t a[4], b[4];
    a[0] = p1l;
    a[1] = p1h + p2l;
    a[2] = p2h + (a[1] < p2l ? 1 : 0);
    a[3] = 0;
    const int k = q - lz + e5 - 127;
    double ra, rb;
    if (!np_round_limbs(a, k, &ra)) return false;
    if (q >= 0 && q <= 55) {  // T_q is 5^q 2^(127 - E_q) itself: X = A
        *out = ra;
        return true;
    }
    b[0] = a[0] + wn;
    uint64_t c = b[0] < wn ? 1 : 0;
    b[1] = a[1] + c;
    c = (c && b[1] == 0) ? 1 : 0;
    b[2] = a[2] + c;
    c = (c && b[2] == 0) ? 1 : 0;
    b[3] = c;
    if (!np_round_limbs(b, k, &rb) || ra != rb) return false;
    *out = ra;
    return true;
}

// w * 10^q rounded to nearest even (w >= 1), as a positive double: the
// exact-double product or quotient when w and 10^|q| are exact (Clinger's
// fast path), else the interval step, else big-integer arithmetic.
NP_HD double dec_to_double(uint64_t w, int q) {
    if (q > 310) return np_bits_to_double(0x7ff0000000000000LL);
    if (q < -380) return 0.0;
    if (w <= (1ULL << 53) && q >= -22 && q <= 22) {
        double p = 1.0;
        for (int k = 0; k < (q < 0 ? -q : q); ++k) p = np_mul(p, 10.0);  // 10^k < 2^53 * 2^k: exact
        return q < 0 ? np_div((double)w, p) : np_mul((double)w, p);
    }
    double r;
    if (np_interval_round(w, q, &r)) return r;
    if (q >= 0) {
        Big N;
        bi_set(N, w);
        bi_pow5_mul(N, q);
        const int L = bi_bitlen(N);
        int e2 = L - 1 + q;
        if (e2 > 1023) return np_bits_to_double(0x7ff0000000000000LL);
        if (L <= 53) return ldexp((double)(N.d[0] | ((uint64_t)(N.n > 1 ? N.d[1] : 0) << 32)), q);
        int sh = L - 53, half, sticky;
        uint64_t m = bi_extract(N, sh, half, sticky);  // the top 53 bits of N
        if (half && (sticky || (m & 1))) ++m;
        if (m == (1ULL << 53)) {
            m >>= 1;
            ++sh;
            ++e2;
        }
        if (e2 > 1023) return np_bits_to_double(0x7ff0000000000000LL);
        return ldexp((double)m, q + sh);
    }
    // q < 0: w / 5^-q * 2^q
    Big D, A;
    bi_set(D, 1);
    bi_pow5_mul(D, -q);
    const int Lw = bitlen64(w), LD = bi_bitlen(D);
    const int t = Lw - LD;
    int f;
    if (t >= 0) {
        Big Ds = D;
        bi_shl(Ds, t);
        bi_set(A, w);
        f = bi_cmp(A, Ds) >= 0 ? t : t - 1;
    } else {
        bi_set(A, w);
        bi_shl(A, -t);
        f = bi_cmp(A, D) >= 0 ? t : t - 1;
    }
    const int e2 = f + q;
    if (e2 < -1080) return 0.0;
    const int p = e2 - 52 > -1074 ? e2 - 52 : -1074;
    const int s = q - p;  // v / 2^p = w 2^s / D
    Big num, den = D;
    bi_set(num, w);
    if (s >= 0) bi_shl(num, s);
    else bi_shl(den, -s);
    Big dd = den;
    bi_shl(dd, 54);
    uint64_t m = 0;
    for (int k = 54; k >= 0; --k) {
        if (bi_cmp(num, dd) >= 0) {
            bi_sub(num, dd);
            m |= 1ULL << k;
        }
        bi_shr1(dd);
    }
    bi_shl(num, 1);  // twice the remainder against the divisor
    const int c = bi_cmp(num, den);
    if (c > 0 || (c == 0 && (m & 1))) ++m;
    return ldexp((double)m, p);
}

NP_HD inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}
NP_HD inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
NP_HD inline bool is_hex(char c) {
    return is_digit(c) || ((c | 32) >= 'a' && (c | 32) <= 'f');
}

// strtod on the NUL-terminated string b[s, e): returns the end offset (s when
// nothing converts), the value in *out, and *unsup = 1 for syntax this reader
// does not convert (hexadecimal, NaN payloads, undecidable long decimals).
NP_HD int dev_strtod(const char *b, int s, int e, double *out, int *unsup) {
    *unsup = 0;
    *out = 0.0;
    int p = s;
    while (p < e && is_space(b[p])) ++p;
    bool neg = false;
    if (p < e && (b[p] == '+' || b[p] == '-')) {
        neg = b[p] == '-';
        ++p;
    }
    const double sign = neg ? -1.0 : 1.0;
    auto match = [&](int at, const char *w) {
        for (int k = 0; w[k]; ++k)
            if (at + k >= e || (b[at + k] | 32) != w[k]) return false;
        return true;
    };
    if (p < e && (b[p] | 32) == 'i') {
        if (!match(p, "inf")) return s;
        p += 3;
        if (match(p, "inity")) p += 5;
        *out = np_bits_to_double(neg ? (long long)0xfff0000000000000ULL : 0x7ff0000000000000LL);
        return p;
    }
    if (p < e && (b[p] | 32) == 'n') {
        if (!match(p, "nan")) return s;
        p += 3;
        if (p < e && b[p] == '(') {
            *unsup = 1;  // a NaN payload: the token is taken whole, its value is not converted
            return e;
        }
        *out = np_bits_to_double(neg ? (long long)0xfff8000000000000ULL : 0x7ff8000000000000LL);
        return p;
    }
    if (p + 1 < e && b[p] == '0' && (b[p + 1] | 32) == 'x' &&
        ((p + 2 < e && is_hex(b[p + 2])) || (p + 3 < e && b[p + 2] == '.' && is_hex(b[p + 3])))) {
        *unsup = 1;  // hexadecimal: the token is taken whole, its value is not converted
        return e;
    }
    uint64_t w = 0;
    int nd = 0, q = 0;
    bool trunc = false, any = false;
    while (p < e && is_digit(b[p])) {
        const int c = b[p] - '0';
        any = true;
        if (nd < 19) {
            if (w || c) {
                w = w * 10 + c;
                ++nd;
            }
        } else {
            ++q;
            trunc |= c != 0;
        }
        ++p;
    }
    if (p < e && b[p] == '.') {
        ++p;
        while (p < e && is_digit(b[p])) {
            const int c = b[p] - '0';
            any = true;
            if (nd < 19) {
                if (w || c) {
                    w = w * 10 + c;
                    ++nd;
                }
                --q;
            } else {
                trunc |= c != 0;
            }
            ++p;
        }
    }
    if (!any) return s;
    if (p < e && (b[p] | 32) == 'e') {
        int x = p + 1;
        bool eneg = false;
        if (x < e && (b[x] == '+' || b[x] == '-')) {
            eneg = b[x] == '-';
            ++x;
        }
        if (x < e && is_digit(b[x])) {
            int ev = 0;
            while (x < e && is_digit(b[x])) {
                if (ev < 100000) ev = ev * 10 + (b[x] - '0');
                ++x;
            }
            q += eneg ? -ev : ev;
            p = x;
        }
    }
    if (w == 0) {
        *out = neg ? -0.0 : 0.0;
        return p;
    }
    const double r1 = dec_to_double(w, q);
    if (trunc && dec_to_double(w + 1, q) != r1) *unsup = 1;
    *out = sign * r1;
    return p;
}

// strtol(b + s, &end, 10) cast to int, on the NUL-terminated string b[s, e).
NP_HD int dev_strtol(const char *b, int s, int e, int *end) {
    int p = s;
    while (p < e && is_space(b[p])) ++p;
    bool neg = false;
    if (p < e && (b[p] == '+' || b[p] == '-')) {
        neg = b[p] == '-';
        ++p;
    }
    if (!(p < e && is_digit(b[p]))) {
        *end = s;
        return 0;
    }
    const uint64_t lim = neg ? 9223372036854775808ULL : 9223372036854775807ULL;
    uint64_t v = 0;
    bool over = false;
    while (p < e && is_digit(b[p])) {
        const uint64_t c = (uint64_t)(b[p] - '0');
        if (!over && (v > (lim - c) / 10)) over = true;
        if (!over) v = v * 10 + c;
        ++p;
    }
    *end = p;
    long long r = over ? (neg ? (long long)0x8000000000000000ULL : 0x7fffffffffffffffLL)
                       : (neg ? (long long)(0 - v) : (long long)v);
    return (int)(uint32_t)(uint64_t)r;  // the low 32 bits, as the host's (int) cast of a long
}

