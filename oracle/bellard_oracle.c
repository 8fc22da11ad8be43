/*
 * bellard_oracle.c - exact CPU oracle for the Bellard pi hex-digit series.
 *
 * TEST INFRASTRUCTURE ONLY (see bellard_oracle.h). Plain C with 128-bit
 * integers; OpenMP over k. Each function names the reference file:line whose
 * arithmetic it restates.
 */
#include "bellard_oracle.h"
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* KernelFuncs.as:9-12: numer 32,1,256,64,4,4,1; sign 1,1,0,1,1,1,0 (1 = minus);
 * den0 4,4,10,10,10,10,10; den1 1,3,1,3,5,7,9. */
const int      orc_numer_log2[7] = {5, 0, 8, 6, 2, 2, 0};
const int      orc_sign[7]       = {1, 1, 0, 1, 1, 1, 0};
const uint64_t orc_den0[7]       = {4, 4, 10, 10, 10, 10, 10};
const uint64_t orc_den1[7]       = {1, 3, 1, 3, 5, 7, 9};

/* Bellard_192.hsp:449-450 (limits) and :468-470 (d odd, needD re-derived). */
int orc_pos_to_d(uint64_t needD, uint64_t *d, uint64_t *needD_adj)
{
    if (needD <= 4 || needD > 999999999999999999ull) return -1;
    uint64_t dd = ((needD - 1) * 2 - 3) / 5;
    if (dd % 2 == 0) dd--;
    *d = dd;
    *needD_adj = (dd * 5 + 3) / 2 + 1;
    return 0;
}

int orc_hexpos_to_d(uint64_t p, uint64_t *d, int *shift)
{
    if (p < 3 || p > 999999999999999999ull) return -1;
    uint64_t B = 4 * (p - 1);          /* want frac(2^B * pi) */
    *d = (B - 6) / 10;
    *shift = (int)((B - 6) - 10 * *d);
    return 0;
}

/* ---- modular exponentiation ------------------------------------------------
 * Montgomery arithmetic with R = 2^64 for odd m < 2^63, restating the
 * Montgomery reduction of Bellard.cl:417-429 (MR64) on a base-2 left-to-right
 * ladder instead of the reference's window-3 table (Bellard.cl:433-461). */
static uint64_t neg_inv64(uint64_t m)
{
    uint64_t x = m;                         /* correct to 3 bits for odd m */
    for (int i = 0; i < 5; i++) x *= 2 - m * x;
    return (uint64_t)0 - x;                 /* -m^-1 mod 2^64 */
}

static inline uint64_t redc64(u128 t, uint64_t m, uint64_t mp)
{
    uint64_t u = (uint64_t)t * mp;
    u128 s = t + (u128)u * m;               /* < 2m*2^64 < 2^128 for m < 2^63 */
    uint64_t z = (uint64_t)(s >> 64);
    return z >= m ? z - m : z;
}

uint64_t orc_pow2mod(uint64_t e, uint64_t m)
{
    if (m == 1) return 0;
    uint64_t mp = neg_inv64(m);
    uint64_t one = ((uint64_t)0 - m) % m;   /* R mod m: Montgomery form of 1 */
    uint64_t x = one;
    /* Leading zero bits square the Montgomery one into itself: start at the top set bit. */
    int top = e ? 63 - __builtin_clzll(e) : -1;
    for (int b = top; b >= 0; b--) {
        x = redc64((u128)x * x, m, mp);
        if ((e >> b) & 1) { x += x; x = (x >= m) ? x - m : x; }   /* 2x < 2^64 */
    }
    return redc64((u128)x, m, mp);
}

uint64_t orc_pow2mod_plain(uint64_t e, uint64_t m)
{
    if (m == 1) return 0;
    uint64_t r = 1 % m, b = 2 % m;
    while (e) {
        if (e & 1) r = (uint64_t)(((u128)r * b) % m);
        b = (uint64_t)(((u128)b * b) % m);
        e >>= 1;
    }
    return r;
}

/* ---- fixed point ----------------------------------------------------------- */
/* floor(r * 2^(64W) / m), r < m: W-step long division (the exact quotient the
 * reference forms with divnby1, Bellard_div2by1.cl:195-211). */
static void frac_words(uint64_t r, uint64_t m, int W, uint64_t *q)
{
    u128 rem = r;
    for (int i = W - 1; i >= 0; i--) {
        u128 num = rem << 64;
        q[i] = (uint64_t)(num / m);
        rem = num - (u128)q[i] * m;
    }
}

static void add_words(uint64_t *acc, const uint64_t *x, int W)
{
    uint64_t c = 0;
    for (int i = 0; i < W; i++) {
        u128 s = (u128)acc[i] + x[i] + c;
        acc[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
}

static void shl_words(uint64_t *x, int W, int s)  /* mod 2^(64W), 0 <= s < 64 */
{
    if (s == 0) return;
    for (int i = W - 1; i > 0; i--) x[i] = (x[i] << s) | (x[i - 1] >> (64 - s));
    x[0] <<= s;
}

static void shr_words(uint64_t *x, int W, int s)  /* logical, any s >= 0 */
{
    int ws = s / 64, bs = s % 64;
    for (int i = 0; i < W; i++) {
        uint64_t lo = (i + ws < W) ? x[i + ws] : 0;
        uint64_t hi = (i + ws + 1 < W) ? x[i + ws + 1] : 0;
        x[i] = bs ? (lo >> bs) | (hi << (64 - bs)) : lo;
    }
}

/* Terms i = k-d with 10i <= 64W: 20 for W = 3 (i = 0..19, the reference's
 * 192-bit tail length, Bellard.cl:1164-1239), 26 for W = 4. */
int orc_tail_terms(int W) { return 64 * W / 10 + 1; }

/* Sign of term k of series f: (-1)^(k + sign_f), as in Bellard.cl:751 and
 * Bellard_div2by1.cl:335. Returns 1 for minus. */
static inline int term_neg(int f, uint64_t k) { return (int)((k + (uint64_t)orc_sign[f]) & 1); }

void orc_term(uint64_t d, int f, uint64_t k, int W, uint64_t *out)
{
    uint64_t m = orc_den0[f] * k + orc_den1[f];
    memset(out, 0, sizeof(uint64_t) * W);
    if (m == 1) return;                       /* x = 0 or 1: frac is 0 */
    if (k < d) {
        uint64_t r = orc_pow2mod(10 * (d - k), m);
        frac_words(r, m, W, out);
    } else {
        uint64_t i = k - d;                   /* 2^(-10i)/m: floor(2^N/m) >> 10i */
        frac_words(1, m, W, out);
        shr_words(out, W, i * 10 > (uint64_t)(64 * W) ? 64 * W : (int)(i * 10));
    }
    if (term_neg(f, k))
        for (int i = 0; i < W; i++) out[i] = ~out[i];
}

void orc_sum_range(uint64_t d, int f, uint64_t k0, uint64_t k1, int W, int nthreads, uint64_t *out)
{
    uint64_t total[8] = {0};
    if (k1 > k0) {
#ifdef _OPENMP
        int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
        {
            uint64_t acc[8] = {0}, t[8];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4096)
#endif
            for (long long kk = 0; kk < (long long)(k1 - k0); kk++) {
                orc_term(d, f, k0 + (uint64_t)kk, W, t);
                add_words(acc, t, W);
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            add_words(total, acc, W);
        }
    }
    (void)nthreads;
    memcpy(out, total, sizeof(uint64_t) * W);
}

void orc_series(uint64_t d, int f, int W, int nthreads, uint64_t *out)
{
    orc_sum_range(d, f, 0, d + (uint64_t)orc_tail_terms(W), W, nthreads, out);
}

/* The W = 3 and W = 4 sums of one series in one pass. The W = 3 long division
 * of r*2^192/m yields the first three quotient words of the W = 4 division of
 * r*2^256/m, so a W = 3 term is the W = 4 term's top three words (also for the
 * tail: floor(2^(256-10i)/m) >> 64 = floor(2^(192-10i)/m), and the sign fold
 * acts word by word). The W = 3 sum stops after its 20 tail terms. */
void orc_sum_range34(uint64_t d, int f, uint64_t k0, uint64_t k1, int nthreads, uint64_t *out3, uint64_t *out4)
{
    uint64_t total3[3] = {0}, total4[4] = {0};
    uint64_t k3end = d + (uint64_t)orc_tail_terms(3);
    if (k1 > k0) {
#ifdef _OPENMP
        int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
        {
            uint64_t acc3[3] = {0}, acc4[4] = {0}, t[4];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4096)
#endif
            for (long long kk = 0; kk < (long long)(k1 - k0); kk++) {
                uint64_t k = k0 + (uint64_t)kk;
                orc_term(d, f, k, 4, t);
                add_words(acc4, t, 4);
                if (k < k3end) add_words(acc3, t + 1, 3);
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            {
                add_words(total3, acc3, 3);
                add_words(total4, acc4, 4);
            }
        }
    }
    (void)nthreads;
    memcpy(out3, total3, sizeof total3);
    memcpy(out4, total4, sizeof total4);
}

void orc_result34(uint64_t d, int shift, int nthreads, uint64_t *out3, uint64_t *out4)
{
    uint64_t acc3[3] = {0}, acc4[4] = {0}, s3[3], s4[4];
    for (int f = 0; f < 7; f++) {
        orc_sum_range34(d, f, 0, d + (uint64_t)orc_tail_terms(4), nthreads, s3, s4);
        shl_words(s3, 3, orc_numer_log2[f] + shift);
        shl_words(s4, 4, orc_numer_log2[f] + shift);
        add_words(acc3, s3, 3);
        add_words(acc4, s4, 4);
    }
    memcpy(out3, acc3, sizeof acc3);
    memcpy(out4, acc4, sizeof acc4);
}

void orc_result(uint64_t d, int shift, int W, int nthreads, uint64_t *out)
{
    uint64_t acc[8] = {0}, s[8];
    for (int f = 0; f < 7; f++) {
        orc_series(d, f, W, nthreads, s);
        shl_words(s, W, orc_numer_log2[f] + shift);
        add_words(acc, s, W);
    }
    memcpy(out, acc, sizeof(uint64_t) * W);
}

void orc_to_hex(const uint64_t *w, int W, char *out)
{
    static const char hx[] = "0123456789abcdef";
    int p = 0;
    for (int i = W - 1; i >= 0; i--)
        for (int b = 60; b >= 0; b -= 4) out[p++] = hx[(w[i] >> b) & 15];
    out[p] = 0;
}

/* workmodeSum0_6.hsp:10-31: digit-wise add, least significant first, carry out
 * of the top digit dropped. */
int orc_hex48_sum(const char *const *hex, int n, char out[49])
{
    int acc[48] = {0};
    for (int j = 0; j < n; j++) {
        const char *s = hex[j];
        if (!s || strlen(s) < 48) return -1;
        int carry = 0;
        for (int i = 47; i >= 0; i--) {
            int c = (unsigned char)s[i], v;
            if (c >= '0' && c <= '9') v = c - '0';
            else if (c >= 'a' && c <= 'f') v = c - 'a' + 10;
            else if (c >= 'A' && c <= 'F') v = c - 'A' + 10;
            else return -1;
            int t = acc[i] + v + carry;
            acc[i] = t & 15;
            carry = t >> 4;
        }
    }
    static const char hx[] = "0123456789abcdef";
    for (int i = 0; i < 48; i++) out[i] = hx[acc[i]];
    out[48] = 0;
    return 0;
}

/* ---- double-double restatement of mode 0 ----------------------------------
 * Same quantities as Sglobal32mtg / Sglobal64mtg (Bellard.cl:729-763, 914-982):
 * per term (r/m) as a double-double, summed mod 1; the 10-term tail of
 * Sglobal_after (Bellard.cl:1118-1144); weighting by numer and frac as in Sum7
 * (Bellard.cl:1324-1353). Products use fma, which is exact, instead of the
 * reference's Dekker split. */
typedef struct { double hi, lo; } dd_t;

static inline dd_t two_sum(double a, double b)
{
    double s = a + b, bb = s - a;
    dd_t r = {s, (a - (s - bb)) + (b - bb)};
    return r;
}
static inline dd_t dd_add(dd_t a, dd_t b)
{
    dd_t s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return two_sum(s.hi, s.lo);
}
static inline dd_t dd_div_nn(double x, double y)   /* x/y to ~106 bits */
{
    double q1 = x / y;
    double rem = fma(-q1, y, x);                    /* exact for |x| < 2^53 */
    double q2 = rem / y;
    return two_sum(q1, q2);
}
static inline dd_t dd_frac(dd_t a)                   /* into (-1, 1) */
{
    double t = trunc(a.hi);
    if (t != 0.0) { dd_t s = two_sum(a.hi - t, a.lo); return s; }
    return a;
}

void orc_dd_result(uint64_t d, int nthreads, double *hi, double *lo)
{
    dd_t ans = {0.0, 0.0};
    for (int f = 0; f < 7; f++) {
        dd_t sum = {0.0, 0.0};
#ifdef _OPENMP
        int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
        {
            dd_t loc = {0.0, 0.0};
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (long long kk = 0; kk < (long long)d; kk++) {
                uint64_t k = (uint64_t)kk;
                uint64_t m = orc_den0[f] * k + orc_den1[f];
                uint64_t r = orc_pow2mod(10 * (d - k), m);
                dd_t t = dd_div_nn((double)r, (double)m);
                if (term_neg(f, k)) { t.hi = -t.hi; t.lo = -t.lo; }
                loc = dd_frac(dd_add(loc, t));
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            sum = dd_frac(dd_add(sum, loc));
        }
        (void)nthreads;
        double p = 1.0;                                /* tail, 10 terms */
        for (uint64_t i = 0; i < 10; i++) {
            uint64_t k = d + i;
            double m = (double)(orc_den0[f] * k + orc_den1[f]);
            dd_t t = dd_div_nn(p, m);
            if (term_neg(f, k)) { t.hi = -t.hi; t.lo = -t.lo; }
            sum = dd_add(sum, t);
            p /= 1024.0;
        }
        sum = dd_frac(sum);
        if (sum.hi < 0.0) sum = dd_add(sum, (dd_t){1.0, 0.0});
        double w = (double)(1 << orc_numer_log2[f]);
        sum.hi *= w; sum.lo *= w;
        sum = dd_frac(sum);
        ans = dd_frac(dd_add(ans, sum));
    }
    if (ans.hi < 0.0) ans = dd_add(ans, (dd_t){1.0, 0.0});
    *hi = ans.hi; *lo = ans.lo;
}
