// cbl_arith.cuh - integer arithmetic of one Bellard term on sm_103a.
//
// A term of series f at index k < d is x = frac(2^(10(d-k)) / m), m = den0*k + den1
// (Bellard.cl:739-749, Bellard_div2by1.cl:327-350). The reference computes
// r = 2^(10e) mod m by Montgomery exponentiation (Bellard.cl:380-461) and then
// forms the fraction r/m in double-double or by an exact 4-limb division
// (Bellard_div2by1.cl:339-341).
//
// Here one Montgomery ladder produces r6 = 2^(10e + 192) mod m, and the six
// 32-bit quotient digits of r/m fall out of six Montgomery reduction steps run
// downwards: with r_j = 2^(10e + 32j) mod m,
//     q_j = floor(r_{j-1} * 2^32 / m) = -r_j * m^-1 mod 2^32 = r_j * mp mod 2^32
//     r_{j-1} = (r_j + q_j * m) / 2^32
// (exact division by the odd m), so q_j is the Montgomery multiplier of the
// step and no division is ever executed. The chain ends at r_0 = 2^(10e) mod m.
//
// Six residue kinds:
//   width 1 (m < 2^28): R = 2^32, residues kept lazily in [0, 4m).
//   middle width 1 (2^28 <= m < 2^31): R = 2^32, residues in [0, m).
//   strict width 1 (2^28 <= m < 2^32): R = 2^32, residues in [0, m), carries kept.
//   short width 2 (2^32 <= m < 2^44): R = 2^48, residues in [0, 4m).
//   width 2 (2^28 <= m < 2^60): R = 2^64 by two word steps, residues in [0, 4m).
//   wide width 2 (2^60 <= m < 2^62): the same steps with residues in [0, 2m).
// The ladder step is y <- REDC(y^2) << b with b the next exponent bit; in the
// lazy kinds 16m < R keeps the result below 4m with no conditional subtraction.
#pragma once
#include <stdint.h>
#include "cbl_internal.h"

namespace cbl {

// -m^-1 mod 2^32 for odd m: (3m) xor 2 is an inverse to 5 bits; three Newton
// steps x <- x(2 - mx) take it to 40 bits.
__device__ __forceinline__ uint32_t neg_inv32(uint32_t m)
{
    uint32_t x = (m * 3u) ^ 2u;
    x *= 2u - m * x;
    x *= 2u - m * x;
    x *= 2u - m * x;
    return 0u - x;
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ------------------------------------------------------------ start values --
// The ladder starts from a value congruent to 2^(Rb+1) (the exponent's leading
// one already consumed). Two float-reciprocal quotient estimates with 32-bit
// conversions only: q1 = trunc(2^E0 / m) is off by at most 2^(E0-21)/m + 1, so
// r1 = 2^E0 - q1 m is small; q2 = rint(r1 / m) is then off by less than 1 and
// r1 - q2 m lies in (-m, m).

// trunc(x) for a positive float x < 2^63, as a 64-bit integer, from its bits.
__device__ __forceinline__ uint64_t float_to_u64_trunc(float x)
{
    const uint32_t bits = __float_as_uint(x);
    const int e = (int)((bits >> 23) & 0xffu) - 127;
    const uint64_t mant = (uint64_t)((bits & 0x7fffffu) | 0x800000u);
    return e >= 23 ? (mant << (e - 23)) : (mant >> (23 - e));
}

// Width 1 (3 <= m < 2^28): a value in (0, 2m) congruent to 2^33.
__device__ __forceinline__ uint32_t w1_start(uint32_t m)
{
    const float inv = rcp_approx(__uint2float_rn(m));
    const uint32_t q1 = __float2uint_rz(8589934592.0f * inv);          // < 2^32 for m >= 3
    const int32_t r1 = (int32_t)(0u - q1 * m);                          // 2^33 - q1 m, |r1| < 2^29
    const int32_t q2 = __float2int_rn(__int2float_rn(r1) * inv);
    return (uint32_t)(r1 + (1 - q2) * (int32_t)m);
}

// Width 2 (2^28 <= m < 2^62): a value in (0, 2m) congruent to 2^65.
__device__ __forceinline__ uint64_t w2_start(uint64_t m)
{
    const uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
    const float fm = __fmaf_rn(__uint2float_rn(m1), 4294967296.0f, __uint2float_rn(m0));
    const float inv = rcp_approx(fm);
    const uint64_t q1 = float_to_u64_trunc(36893488147419103232.0f * inv);   // 2^65 / m >= 2^5
    const int64_t r1 = (int64_t)(0ull - q1 * m);                               // |r1| <= 2^44 + m < 2^61
    const float fr1 = __fmaf_rn(__int2float_rn((int32_t)(r1 >> 32)), 4294967296.0f,
                                __uint2float_rn((uint32_t)r1));
    const int32_t q2 = __float2int_rn(fr1 * inv);                             // |r1/m| <= 2^16 + 1
    return (uint64_t)(r1 + (int64_t)(1 - q2) * (int64_t)m);
}

// ------------------------------------------------------------ exponent walk --
// Calls st.step(b) for every bit of Ep after its leading one, most significant
// first. When Ep >= 2^32 the 32 bits of the low word run fully unrolled.
template <typename State>
__device__ __forceinline__ void walk_bits(uint64_t Ep, State &st)
{
    const uint32_t hi = (uint32_t)(Ep >> 32), lo = (uint32_t)Ep;
    if (hi != 0) {
        const int nb = 32 - __clz(hi);
        uint32_t h = (hi << (32 - nb)) << 1;
        for (int i = 1; i < nb; ++i) {
            st.step(h >> 31);
            h <<= 1;
        }
#pragma unroll
        for (int i = 31; i >= 0; --i) st.step((lo >> i) & 1u);
    } else {
        const int nb = 32 - __clz(lo);
        uint32_t l = (lo << (32 - nb)) << 1;
        for (int i = 1; i < nb; ++i) {
            st.step(l >> 31);
            l <<= 1;
        }
    }
}

// Start from the leading up-to-NB bits of Ep at once (value p), then walk the
// rest; st.y is set by start(p).
template <int NB, typename State, typename Start>
__device__ __forceinline__ void walk_bits_start(uint64_t Ep, State &st, Start start)
{
    const uint32_t hi = (uint32_t)(Ep >> 32), lo = (uint32_t)Ep;
    if (hi != 0) {
        const int nb = 32 - __clz(hi);
        const int t = nb < NB ? nb : NB;
        start(st, hi >> (nb - t));
        uint32_t h = (nb - t) > 0 ? hi << (32 - (nb - t)) : 0u;
        for (int i = t; i < nb; ++i) {
            st.step(h >> 31);
            h <<= 1;
        }
#pragma unroll
        for (int i = 31; i >= 0; --i) st.step((lo >> i) & 1u);
    } else {
        const int nb = 32 - __clz(lo);
        const int t = nb < NB ? nb : NB;
        start(st, lo >> (nb - t));
        uint32_t l = (nb - t) > 0 ? lo << (32 - (nb - t)) : 0u;
        for (int i = t; i < nb; ++i) {
            st.step(l >> 31);
            l <<= 1;
        }
    }
}

// ------------------------------------------------- multiply-add chains --
// Every REDC word step below is written as a PTX carry chain of mad.lo.cc /
// madc.hi over 32-bit words. A 64-bit multiply-add (mad.wide with a 64-bit
// addend) issues more slowly on sm_103a than the two chained halves, and the
// carry out of the chain comes for free.

// hi(u m + (t0, t1)) mod 2^32, where u m + t0 = 0 mod 2^32 (a REDC word step).
__device__ __forceinline__ uint32_t redc_word(uint32_t u, uint32_t m, uint32_t t0, uint32_t t1)
{
    uint32_t r;
    asm("{\n\t.reg .u32 x;\n\t"
        "mad.lo.cc.u32 x, %1, %2, %3;\n\t"
        "madc.hi.u32 %0, %1, %2, %4;\n\t}"
        : "=r"(r)
        : "r"(u), "r"(m), "r"(t0), "r"(t1));
    return r;
}

// As redc_word, also returning the carry out of the high word in c (0 or 1).
__device__ __forceinline__ uint32_t redc_word_c(uint32_t u, uint32_t m, uint32_t t0, uint32_t t1, uint32_t &c)
{
    uint32_t r;
    asm("{\n\t.reg .u32 x;\n\t"
        "mad.lo.cc.u32 x, %2, %3, %4;\n\t"
        "madc.hi.cc.u32 %0, %2, %3, %5;\n\t"
        "addc.u32 %1, 0, 0;\n\t}"
        : "=r"(r), "=r"(c)
        : "r"(u), "r"(m), "r"(t0), "r"(t1));
    return r;
}

// ---------------------------------------------------------------- width 1 --
// y in [0,4m), m < 2^28: REDC_2^32(y^2) << b, again in [0,4m).
__device__ __forceinline__ uint32_t w1_sqr(uint32_t y, uint32_t m, uint32_t mp, uint32_t b)
{
    const uint64_t t = (uint64_t)y * y;                 // < 16 m^2 < 2^60
    const uint32_t u = (uint32_t)t * mp;
    return redc_word(u, m, (uint32_t)t, (uint32_t)(t >> 32)) << b;   // (t + u m) / 2^32 < 2m
}

struct W1State {
    uint32_t y, m, mp;
    __device__ __forceinline__ void step(uint32_t b) { y = w1_sqr(y, m, mp, b); }
};

// r6 = 2^E mod m in [0, m) for E >= 33 (m < 2^28, odd, >= 3).
__device__ __forceinline__ uint32_t w1_pow2(uint64_t E, uint32_t m, uint32_t mp)
{
    W1State st{w1_start(m), m, mp};                     // invariant y = 2^(32 + prefix of E - 32)
    walk_bits(E - 32, st);
    uint32_t y = st.y;
    y = min(y, y - 2u * m);                            // [0,4m) -> [0,2m)
    y = min(y, y - m);                                 //        -> [0,m)
    return y;
}

// Six quotient digits of r_0 / m from r6 (digit 0 least significant), and r_0.
// Valid for any odd m < 2^32.
__device__ __forceinline__ uint32_t w1_digits(uint32_t r, uint32_t m, uint32_t mp, uint32_t q[6])
{
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        q[j] = r * mp;
        r = redc_word(q[j], m, r, 0u);                  // (r + q m) / 2^32 < m
    }
    return r;
}

// --------------------------------------------------------- strict width 1 --
// 2^31 <= m < 2^32: R = 2^32, residues in [0, m). The doubling comes first,
// into the second multiplicand only: y2 = 2^b y, less m when the shift carries
// out of bit 31, is below 2^32 (not necessarily below m), so t = y y2 < m 2^32.
// u m + t can pass 2^64 once: the carry chain returns the carry c out of the
// high word, REDC = x + c 2^32 < 2m, and one conditional subtraction brings it
// below m. (Valid for 2^28 <= m < 2^32.)
__device__ __forceinline__ uint32_t w1s_sqr(uint32_t y, uint32_t m, uint32_t mp, uint32_t b)
{
    const uint32_t x2 = y << b;
    const uint32_t c2 = __funnelshift_l(y, 0u, b);                 // bit shifted out of y
    const uint32_t y2 = c2 ? x2 - m : x2;                          // 2^b y mod m, < 2^32
    const uint64_t t = (uint64_t)y * y2;
    const uint32_t u = (uint32_t)t * mp;
    uint32_t c;
    const uint32_t x = redc_word_c(u, m, (uint32_t)t, (uint32_t)(t >> 32), c);
    return c ? x - m : min(x, x - m);                              // REDC mod m, in [0, m)
}

struct W1SState {
    uint32_t y, m, mp;
    __device__ __forceinline__ void step(uint32_t b) { y = w1s_sqr(y, m, mp, b); }
};


// ------------------------------------------------------ middle width 1 --
// 2^28 <= m < 2^31: R = 2^32, residues in [0, m). The doubling comes first:
// t = y (2^b y) < 2m^2 < 2^63 and u m < 2^63, so the word step has no carry
// out and REDC(t) = REDC(y^2) 2^b mod m is below 2m; one min(z, z - m)
// brings it below m. (Two ALU operations fewer than reducing, then doubling
// and reducing again.)
__device__ __forceinline__ uint32_t w1m_sqr(uint32_t y, uint32_t m, uint32_t mp, uint32_t b)
{
    const uint64_t t = (uint64_t)y * (y << b);
    const uint32_t u = (uint32_t)t * mp;
    const uint32_t z = redc_word(u, m, (uint32_t)t, (uint32_t)(t >> 32));   // < 2m
    return min(z, z - m);
}

struct W1MState {
    uint32_t y, m, mp;
    __device__ __forceinline__ void step(uint32_t b) { y = w1m_sqr(y, m, mp, b); }
};

// 2^(32 + p) mod m in [0, m), 1 <= p <= 15, 2^28 <= m < 2^32: q1 <= 2^19 is
// off by at most one, so one correction either way suffices.
__device__ __forceinline__ uint32_t w1m_start(uint32_t m, uint32_t p)
{
    const float inv = rcp_approx(__uint2float_rn(m));
    const float scale = __int_as_float((int)((127u + 32u + p) << 23));
    const uint32_t q1 = __float2uint_rz(scale * inv);
    int64_t r = (int64_t)(1ull << (32 + p)) - (int64_t)q1 * (int64_t)m;   // in [-m, 2m)
    r += (r < 0) ? (int64_t)m : 0;
    r -= (r >= (int64_t)m) ? (int64_t)m : 0;
    return (uint32_t)r;
}

struct W1MStart {
    __device__ __forceinline__ void operator()(W1MState &st, uint32_t p) const { st.y = w1m_start(st.m, p); }
};

// r6 = 2^E mod m in [0, m) for E >= 33, 2^28 <= m < 2^31. The start value
// takes the leading up-to-four bits of E - 32 at once.
__device__ __forceinline__ uint32_t w1m_pow2(uint64_t E, uint32_t m, uint32_t mp)
{
    W1MState st{0, m, mp};
    walk_bits_start<4>(E - 32, st, W1MStart{});
    return st.y;
}

struct W1SStart {
    __device__ __forceinline__ void operator()(W1SState &st, uint32_t p) const { st.y = w1m_start(st.m, p); }
};

// r6 = 2^E mod m in [0, m) for E >= 33 (2^31 <= m < 2^32), from the same
// 4-bit start value.
__device__ __forceinline__ uint32_t w1s_pow2(uint64_t E, uint32_t m, uint32_t mp)
{
    W1SState st{0, m, mp};
    walk_bits_start<4>(E - 32, st, W1SStart{});
    return st.y;
}

// ---------------------------------------------------------------- width 2 --
// y = (y0,y1) in [0,4m), m = (m0,m1) with 2^28 <= m < 2^60 (so y1 < 2^30,
// m1 < 2^28, T + U m < 2^125): REDC_2^64(y^2) << b by two 32-bit word steps,
// again in [0,4m) because 16m < 2^64.
__device__ __forceinline__ void w2_sqr(uint32_t &y0, uint32_t &y1, uint32_t m0, uint32_t m1,
                                       uint32_t mp, uint32_t b)
{
    // T = y^2 = t0 + t1 2^32 + t2 2^64 + t3 2^96  (< 16 m^2 < 2^124)
    const uint64_t a = (uint64_t)y0 * y0;
    const uint64_t p = (uint64_t)y0 * (y1 << 1);        // y1 < 2^30
    const uint64_t s = (uint64_t)y1 * y1;
    const uint32_t t0 = (uint32_t)a;
    uint32_t t1, t2, t3;
    asm("add.cc.u32 %0, %3, %4;\n\t"
        "addc.cc.u32 %1, %5, %6;\n\t"
        "addc.u32 %2, %7, 0;"
        : "=r"(t1), "=r"(t2), "=r"(t3)
        : "r"((uint32_t)(a >> 32)), "r"((uint32_t)p), "r"((uint32_t)(p >> 32)), "r"((uint32_t)s),
          "r"((uint32_t)(s >> 32)));
    // word step 1: s = (T + u0 m) / 2^32 = (t1, t2, t3) + hi(u0 m0) + c + u0 m1,
    // c the carry out of u0 m0 + t0 (whose low word is 0)
    const uint32_t u0 = t0 * mp;
    uint32_t s0, s1, s2;
    asm("{\n\t.reg .u32 x, h, e2, e3;\n\t"
        "mad.lo.cc.u32 x, %3, %4, %5;\n\t"
        "madc.hi.cc.u32 h, %3, %4, %6;\n\t"
        "addc.cc.u32 e2, %7, 0;\n\t"
        "addc.u32 e3, %8, 0;\n\t"
        "mad.lo.cc.u32 %0, %3, %9, h;\n\t"
        "madc.hi.cc.u32 %1, %3, %9, e2;\n\t"
        "addc.u32 %2, e3, 0;\n\t}"
        : "=r"(s0), "=r"(s1), "=r"(s2)
        : "r"(u0), "r"(m0), "r"(t0), "r"(t1), "r"(t2), "r"(t3), "r"(m1));
    // word step 2: z = (s + u1 m) / 2^32 < 2m
    const uint32_t u1 = s0 * mp;
    uint32_t z0, z1;
    asm("{\n\t.reg .u32 x, h, e2;\n\t"
        "mad.lo.cc.u32 x, %2, %3, %4;\n\t"
        "madc.hi.cc.u32 h, %2, %3, %5;\n\t"
        "addc.u32 e2, %6, 0;\n\t"
        "mad.lo.cc.u32 %0, %2, %7, h;\n\t"
        "madc.hi.u32 %1, %2, %7, e2;\n\t}"
        : "=r"(z0), "=r"(z1)
        : "r"(u1), "r"(m0), "r"(s0), "r"(s1), "r"(s2), "r"(m1));
    y1 = __funnelshift_l(z0, z1, b);
    y0 = z0 << b;
}

struct W2State {
    uint32_t y0, y1, m0, m1, mp;
    __device__ __forceinline__ void step(uint32_t b) { w2_sqr(y0, y1, m0, m1, mp, b); }
};

// r6 = 2^E mod m in [0, m) for E >= 65 (2^28 <= m < 2^60).
__device__ __forceinline__ uint64_t w2_pow2(uint64_t E, uint64_t m, uint32_t mp)
{
    const uint64_t y = w2_start(m);
    W2State st{(uint32_t)y, (uint32_t)(y >> 32), (uint32_t)m, (uint32_t)(m >> 32), mp};
    walk_bits(E - 64, st);
    uint64_t r = ((uint64_t)st.y1 << 32) | st.y0;
    r = min(r, r - 2 * m);
    r = min(r, r - m);
    return r;
}

// --------------------------------------------------- width 2, m < 2^44 --
// 2^32 <= m < 2^44 (m1 < 2^12), y in [0,4m) (y1 < 2^14), R = 2^48: one 32-bit
// REDC word step and one 16-bit step. R > 16m^2/(3m) keeps the lazy residues
// in [0, 4m): REDC(y^2) < 16m^2/2^48 + m < 2m. y^2 = y0^2 + y0 (2 y1) 2^32 +
// y1^2 2^64 with y0 (2 y1) < 2^47 and y1^2 < 2^28, so word step 1 is
//   s = (y0^2 + u0 m0) / 2^32 + y1^2 2^32 + y0 (2 y1) + u0 m1 < 2^61,
// one carry chain whose carry out of the first multiply-add lands on y1^2
// (its high words stay below 2^29 and 2^30: no carry leaves the chain).
// The 16-bit step takes u1 = s0 mp mod 2^16, so u1 m1 < 2^28 is a single low
// multiply (a 32-bit step needs two words there): X = s + u1 m0 + u1 m1 2^32
// < 2^62 with its low 16 bits zero, and X / 2^16 < 2m. The doubling joins
// that shift: y = X >> (16 - b). 14 multiply halves per step instead of 15.
__device__ __forceinline__ void w2s_sqr(uint32_t &y0, uint32_t &y1, uint32_t m0, uint32_t m1, uint32_t mp,
                                        uint32_t b)
{
    const uint64_t A = (uint64_t)y0 * y0;
    const uint32_t a0 = (uint32_t)A, a1 = (uint32_t)(A >> 32);
    const uint32_t u0 = a0 * mp;
    const uint32_t ysq = y1 * y1;
    const uint32_t y2 = y1 << 1;
    uint32_t s0, s1;
    asm("{\n\t.reg .u32 x0, x1, w, t0, t1;\n\t"
        "mad.lo.cc.u32 x0, %2, %3, %4;\n\t"     // u0 m0 + y0^2: low word 0
        "madc.hi.cc.u32 x1, %2, %3, %5;\n\t"
        "addc.u32 w, %6, 0;\n\t"                // y1^2 + carry
        "mad.lo.cc.u32 t0, %7, %8, x1;\n\t"     // + y0 (2 y1)
        "madc.hi.u32 t1, %7, %8, w;\n\t"
        "mad.lo.cc.u32 %0, %2, %9, t0;\n\t"     // + u0 m1
        "madc.hi.u32 %1, %2, %9, t1;\n\t}"
        : "=r"(s0), "=r"(s1)
        : "r"(u0), "r"(m0), "r"(a0), "r"(a1), "r"(ysq), "r"(y0), "r"(y2), "r"(m1));
    const uint32_t u1 = (s0 * mp) & 0xffffu;
    uint32_t x0, x1;
    asm("mad.lo.cc.u32 %0, %2, %3, %4;\n\t"     // u1 m0 + s: low 16 bits 0
        "madc.hi.u32 %1, %2, %3, %5;\n\t"
        "mad.lo.u32 %1, %2, %6, %1;"              // + u1 m1 2^32
        : "=&r"(x0), "=&r"(x1)
        : "r"(u1), "r"(m0), "r"(s0), "r"(s1), "r"(m1));
    const uint32_t sh = 16u - b;
    y0 = __funnelshift_r(x0, x1, sh);
    y1 = x1 >> sh;
}

struct W2SState {
    uint32_t y0, y1, m0, m1, mp;
    __device__ __forceinline__ void step(uint32_t b) { w2s_sqr(y0, y1, m0, m1, mp, b); }
};

// A value in (0, 2m) congruent to 2^(48 + p), 1 <= p <= 15, for 2^32 <= m < 2^44:
// q1 = trunc(2^(48+p) / m) from a float reciprocal (q1 < 2^31) leaves
// |r1| <= 2^(27+p) + m; q2 = rint(r1 / m) (|r1 / m| < 2^11) is then off by at
// most a few thousandths, so r1 - q2 m lies in (-m/2, m/2) up to that slack and
// r1 + (1 - q2) m in (0, 2m). (Checked in float32 emulation over 4e5 moduli,
// every p, with reciprocals off by up to 2 ulps.)
__device__ __forceinline__ uint64_t w2s_start(uint64_t m, uint32_t p)
{
    const uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
    const float fm = __fmaf_rn(__uint2float_rn(m1), 4294967296.0f, __uint2float_rn(m0));
    const float inv = rcp_approx(fm);
    const float scale = __int_as_float((int)((127u + 48u + p) << 23));      // 2^(48+p)
    const uint64_t q1 = float_to_u64_trunc(scale * inv);
    const int64_t r1 = (int64_t)((1ull << (48 + p)) - q1 * m);
    const float fr1 = __fmaf_rn(__int2float_rn((int32_t)(r1 >> 32)), 4294967296.0f,
                                __uint2float_rn((uint32_t)r1));
    const int32_t q2 = __float2int_rn(fr1 * inv);
    return (uint64_t)(r1 + (int64_t)(1 - q2) * (int64_t)m);
}

// r6 = 2^E mod m in [0, m) for E >= 65, 2^32 <= m < 2^44. The ladder runs in
// Montgomery form with R = 2^48 on the bits of E - 48; the start value takes
// their leading up-to-four bits at once.
__device__ __forceinline__ uint64_t w2s_pow2(uint64_t E, uint64_t m, uint32_t mp)
{
    const uint64_t Ep = E - 48;
    const uint32_t hi = (uint32_t)(Ep >> 32), lo = (uint32_t)Ep;
    W2SState st{0, 0, (uint32_t)m, (uint32_t)(m >> 32), mp};
    if (hi != 0) {
        const int nb = 32 - __clz(hi);
        const int t = nb < 4 ? nb : 4;
        const uint64_t y = w2s_start(m, hi >> (nb - t));
        st.y0 = (uint32_t)y;
        st.y1 = (uint32_t)(y >> 32);
        uint32_t h = (nb - t) > 0 ? hi << (32 - (nb - t)) : 0u;   // remaining bits of hi, left-aligned
        for (int i = t; i < nb; ++i) {
            st.step(h >> 31);
            h <<= 1;
        }
#pragma unroll
        for (int i = 31; i >= 0; --i) st.step((lo >> i) & 1u);
    } else {
        const int nb = 32 - __clz(lo);
        const int t = nb < 4 ? nb : 4;
        const uint64_t y = w2s_start(m, lo >> (nb - t));
        st.y0 = (uint32_t)y;
        st.y1 = (uint32_t)(y >> 32);
        uint32_t l = (nb - t) > 0 ? lo << (32 - (nb - t)) : 0u;
        for (int i = t; i < nb; ++i) {
            st.step(l >> 31);
            l <<= 1;
        }
    }
    uint64_t r = ((uint64_t)st.y1 << 32) | st.y0;
    r = min(r, r - 2 * m);
    r = min(r, r - m);
    return r;
}

// ------------------------------------------------------- width 2, m >= 2^60 --
// 2^60 <= m < 2^62 (positions up to 999999999999999999): residues in [0, 2m).
// REDC(y^2) < 4m^2/2^64 + m < 2m still holds and T + U m < 2^127, so the
// two-word step of w2_sqr applies; only the doubling needs min(y, y - 2m).
struct W2XState {
    uint32_t y0, y1, m0, m1, mp;
    uint64_t m2;                                        // 2m
    __device__ __forceinline__ void step(uint32_t b)
    {
        w2_sqr(y0, y1, m0, m1, mp, b);                  // < 4m < 2^64
        uint64_t y = ((uint64_t)y1 << 32) | y0;
        y = min(y, y - m2);                             // < 2m
        y0 = (uint32_t)y;
        y1 = (uint32_t)(y >> 32);
    }
};

// r6 = 2^E mod m in [0, m) for E >= 65, 2^28 <= m < 2^62.
__device__ __forceinline__ uint64_t w2x_pow2(uint64_t E, uint64_t m, uint32_t mp)
{
    const uint64_t y = w2_start(m);                     // (0, 2m)
    W2XState st{(uint32_t)y, (uint32_t)(y >> 32), (uint32_t)m, (uint32_t)(m >> 32), mp, 2 * m};
    walk_bits(E - 64, st);
    uint64_t r = ((uint64_t)st.y1 << 32) | st.y0;
    r = min(r, r - m);
    return r;
}

// N REDC steps down from r < m (two-word m): q[j] are the quotient digits and
// the result is r 2^(-32 N) mod m.
template <int N>
__device__ __forceinline__ uint64_t w2_redc_down(uint64_t r, uint64_t m, uint32_t mp, uint32_t q[N])
{
    const uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
    uint32_t r0 = (uint32_t)r, r1 = (uint32_t)(r >> 32);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        q[j] = r0 * mp;
        // (r + q m) / 2^32 = hi(q m0 + r) + c 2^32 + q m1 < m, c the carry out
        asm("{\n\t.reg .u32 x, h, c;\n\t"
            "mad.lo.cc.u32 x, %2, %3, %4;\n\t"
            "madc.hi.cc.u32 h, %2, %3, %5;\n\t"
            "addc.u32 c, 0, 0;\n\t"
            "mad.lo.cc.u32 %0, %2, %6, h;\n\t"
            "madc.hi.u32 %1, %2, %6, c;\n\t}"
            : "=r"(r0), "=r"(r1)
            : "r"(q[j]), "r"(m0), "r"(r0), "r"(r1), "r"(m1));
    }
    return ((uint64_t)r1 << 32) | r0;
}

__device__ __forceinline__ uint64_t w2_digits(uint64_t r, uint64_t m, uint32_t mp, uint32_t q[6])
{
    return w2_redc_down<6>(r, m, mp, q);
}

// Two ladders at once (terms k and k+32 of one lane): when both exponents have
// the same bit length (in the same word) the steps interleave, giving the
// scheduler two independent chains; otherwise they run one after the other.
template <int NB, typename State, typename Start>
__device__ __forceinline__ void walk_bits_start_pair(uint64_t EpA, uint64_t EpB, State &A, State &B, Start start)
{
    const uint32_t ha = (uint32_t)(EpA >> 32), la = (uint32_t)EpA, hb = (uint32_t)(EpB >> 32), lb = (uint32_t)EpB;
    const uint32_t wa = ha ? ha : la, wb = hb ? hb : lb;         // word holding the leading bits
    const int nba = 32 - __clz(wa), nbb = 32 - __clz(wb);
    if ((ha == 0) != (hb == 0) || nba != nbb || nba < NB) {
        walk_bits_start<NB>(EpA, A, start);
        walk_bits_start<NB>(EpB, B, start);
        return;
    }
    start(A, wa >> (nba - NB));
    start(B, wb >> (nbb - NB));
    uint32_t ga = (nba - NB) > 0 ? wa << (32 - (nba - NB)) : 0u, gb = (nbb - NB) > 0 ? wb << (32 - (nbb - NB)) : 0u;
    for (int i = NB; i < nba; ++i) {
        A.step(ga >> 31);
        B.step(gb >> 31);
        ga <<= 1;
        gb <<= 1;
    }
    if (ha != 0) {
#pragma unroll
        for (int i = 31; i >= 0; --i) {
            A.step((la >> i) & 1u);
            B.step((lb >> i) & 1u);
        }
    }
}

struct W1Start1 {                                        // the single-bit start of the width-1 kind
    __device__ __forceinline__ void operator()(W1State &st, uint32_t) const { st.y = w1_start(st.m); }
};

struct W2SStart {
    __device__ __forceinline__ void operator()(W2SState &st, uint32_t p) const
    {
        const uint64_t y = w2s_start(((uint64_t)st.m1 << 32) | st.m0, p);
        st.y0 = (uint32_t)y;
        st.y1 = (uint32_t)(y >> 32);
    }
};

// ------------------------------------------------------------ fixed point --
// 192-bit accumulator as six 32-bit digits, digit 0 least significant.
struct Acc192 {
    uint32_t w[6];
};

__device__ __forceinline__ void acc_zero(Acc192 &a)
{
#pragma unroll
    for (int j = 0; j < 6; ++j) a.w[j] = 0;
}

__device__ __forceinline__ void acc_add(Acc192 &a, const uint32_t q[6])
{
    asm("add.cc.u32  %0, %0, %6;\n\t"
        "addc.cc.u32 %1, %1, %7;\n\t"
        "addc.cc.u32 %2, %2, %8;\n\t"
        "addc.cc.u32 %3, %3, %9;\n\t"
        "addc.cc.u32 %4, %4, %10;\n\t"
        "addc.u32    %5, %5, %11;"
        : "+r"(a.w[0]), "+r"(a.w[1]), "+r"(a.w[2]), "+r"(a.w[3]), "+r"(a.w[4]), "+r"(a.w[5])
        : "r"(q[0]), "r"(q[1]), "r"(q[2]), "r"(q[3]), "r"(q[4]), "r"(q[5]));
}

// a <- -a - c (mod 2^192): the sum of c negative terms NOT(q_i) = -q_i - 1.
__device__ __forceinline__ void acc_negate_minus(Acc192 &a, uint32_t c)
{
    // -a - c = ~a + (1 - c), with (1 - c) sign-extended to 192 bits.
#pragma unroll
    for (int j = 0; j < 6; ++j) a.w[j] = ~a.w[j];
    const uint32_t add = 1u - c;
    const uint32_t ext = (c > 1) ? 0xffffffffu : 0u;
    asm("add.cc.u32  %0, %0, %6;\n\t"
        "addc.cc.u32 %1, %1, %7;\n\t"
        "addc.cc.u32 %2, %2, %7;\n\t"
        "addc.cc.u32 %3, %3, %7;\n\t"
        "addc.cc.u32 %4, %4, %7;\n\t"
        "addc.u32    %5, %5, %7;"
        : "+r"(a.w[0]), "+r"(a.w[1]), "+r"(a.w[2]), "+r"(a.w[3]), "+r"(a.w[4]), "+r"(a.w[5])
        : "r"(add), "r"(ext));
}

}  // namespace cbl
