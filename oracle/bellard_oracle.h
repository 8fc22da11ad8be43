/*
 * bellard_oracle.h - exact CPU oracle for the Bellard pi hex-digit series.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path in
 * clbellard_gb300/. Only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py may load it. The product library never links it
 * and has no CPU fallback.
 *
 * It restates, in plain C, the arithmetic of the reference's hot path:
 *   - formula table            KernelFuncs.as:9-12
 *   - needD -> d mapping       Bellard_192.hsp:468-470
 *   - per-term 2^(10(d-k)) mod m, Montgomery    Bellard.cl:380-461 (ExpMod32v4 / ExpMod64v4)
 *   - exact fixed-point quotient floor(r*2^N/m)  Bellard_div2by1.cl:339-347
 *   - tail terms k >= d                          Bellard.cl:1153-1253 (20 terms)
 *   - numer weighting by left shift, sum mod 1   Bellard.cl:1359-1398 (Sum7_192)
 *   - work-mode hex merge mod 16^48              workmodeSum0_6.hsp:10-31
 *
 * Fixed-point numbers are arrays of W little-endian 64-bit words holding
 * floor(x * 2^(64W)) mod 2^(64W) for a value x taken mod 1.
 *
 * Per-term contribution (the definition the CUDA kernels reproduce bit-exactly
 * when W = 3): for a signed term s*x with x = frac(2^(10(d-k))/m) (k < d) or
 * x = 2^(-10(k-d))/m (k >= d), the contribution is floor(s*x*2^N) mod 2^N.
 * For s = -1 and x not an integer multiple of 2^-N this is NOT(floor(x*2^N)),
 * the same value the reference gets from floor((m-r)*2^N/m).
 */
#ifndef BELLARD_ORACLE_H
#define BELLARD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* The 7 series of Bellard's formula (KernelFuncs.as:9-12). */
extern const int      orc_numer_log2[7]; /* numer = 32,1,256,64,4,4,1 as shifts */
extern const int      orc_sign[7];       /* 1 = minus */
extern const uint64_t orc_den0[7];
extern const uint64_t orc_den1[7];

/* needD -> (d, adjusted needD), Bellard_192.hsp:449-450,468-470.
 * Returns 0, or -1 for needD <= 4 or needD > 999999999999999999. */
int orc_pos_to_d(uint64_t needD, uint64_t *d, uint64_t *needD_adj);

/* 2^e mod m (m >= 1, m < 2^63). Montgomery ladder. */
uint64_t orc_pow2mod(uint64_t e, uint64_t m);
/* Same value by plain square-and-multiply with 128-bit remainder. */
uint64_t orc_pow2mod_plain(uint64_t e, uint64_t m);

/* One term of series f at index k (k < d: main body, k >= d: tail term
 * 2^(-10(k-d))/m), signed, as W words. */
void orc_term(uint64_t d, int f, uint64_t k, int W, uint64_t *out);

/* Sum of terms of series f for k in [k0, k1), as W words, mod 1.
 * k may run past d into the tail. nthreads <= 0 means all cores. */
void orc_sum_range(uint64_t d, int f, uint64_t k0, uint64_t k1, int W, int nthreads, uint64_t *out);

/* Number of tail terms the fixed-point path uses: 20 for W=3 (as the
 * reference's 192-bit tail), 26 for W=4. */
int orc_tail_terms(int W);

/* Full series partial S_f = sum over k in [0, d + tail) as W words. */
void orc_series(uint64_t d, int f, int W, int nthreads, uint64_t *out);

/* frac(2^(10d+6+shift) * pi) as W words: sum_f S_f << (numer_log2[f] + shift). */
void orc_result(uint64_t d, int shift, int W, int nthreads, uint64_t *out);

/* The W = 3 and W = 4 results (and one-series sums over [k0, k1)) from one
 * pass over k: the W = 3 words equal orc_result(.., 3, ..) and the W = 4 words
 * orc_result(.., 4, ..). */
void orc_sum_range34(uint64_t d, int f, uint64_t k0, uint64_t k1, int nthreads, uint64_t *out3, uint64_t *out4);
void orc_result34(uint64_t d, int shift, int nthreads, uint64_t *out3, uint64_t *out4);

/* General hex position p >= 3 (1-based digit after the point): d and shift with
 * 4(p-1) = 10d + 6 + shift, 0 <= shift < 10. Returns -1 if p < 3. */
int orc_hexpos_to_d(uint64_t p, uint64_t *d, int *shift);

/* W words -> 16W lowercase hex chars, most significant first, NUL-terminated. */
void orc_to_hex(const uint64_t *w, int W, char *out);

/* Work-mode merge: add n 48-digit hex strings mod 16^48 (workmodeSum0_6.hsp).
 * Returns 0, or -1 on a malformed string. */
int orc_hex48_sum(const char *const *hex, int n, char out[49]);

/* 106-bit double-double restatement of the reference's mode-0 sum
 * (Bellard.cl:729-763, 1118-1144, 1274-1353): returns the final (hi, lo)
 * in [0,1) for position d, with k-range [0,d) in one pass. */
void orc_dd_result(uint64_t d, int nthreads, double *hi, double *lo);

#ifdef __cplusplus
}
#endif
#endif
