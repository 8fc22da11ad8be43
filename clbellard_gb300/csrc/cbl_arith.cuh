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
// Two residue widths:
//   width 1 (m < 2^28): R = 2^32, residues kept lazily in [0, 4m).
//   width 2 (2^28 <= m < 2^50): R = 2^64 by two word steps, residues in [0, 4m).
// The ladder step is y <- REDC(y^2) << b with b the next exponent bit; because
// 16m < R the result stays below 4m with no conditional subtraction.
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

// A value congruent to 2^E0 mod m in [0, 2m), for E0 = 33 (m < 2^28) or
// E0 = 65 (2^28 <= m < 2^50). Two float-reciprocal quotient estimates:
//   q1 = trunc(2^E0 / m) +- (2^(E0-21)/m + 1), so |r1| = |2^E0 - q1 m| <= 2^(E0-21) + m;
//   q2 = rint(r1 / m) is then off by less than 1 (|r1/m| <= 2^16 + 1 in both
//   uses), so r1 - q2 m lies in (-m, m) and adding m lands in (0, 2m).
template <int E0>
__device__ __forceinline__ uint64_t pow2_start(uint64_t m)
{
    const float fm = __ull2float_rn(m);
    const float inv = rcp_approx(fm);
    const float scale = __int_as_float((127 + E0) << 23);         // 2^E0
    const uint64_t q1 = __float2ull_rz(scale * inv);
    const uint64_t top = (E0 < 64) ? (1ull << (E0 & 63)) : 0ull;  // 2^E0 mod 2^64
    const int64_t r1 = (int64_t)(top - q1 * m);
    const int64_t q2 = __float2ll_rn(__ll2float_rn(r1) * inv);
    return (uint64_t)(r1 - (q2 - 1) * (int64_t)m);
}

// ---------------------------------------------------------------- width 1 --
// y in [0,4m), m < 2^28: REDC_2^32(y^2) << b, again in [0,4m).
__device__ __forceinline__ uint32_t w1_sqr(uint32_t y, uint32_t m, uint32_t mp, uint32_t b)
{
    const uint64_t t = (uint64_t)y * y;                 // < 16 m^2 < 2^60
    const uint32_t u = (uint32_t)t * mp;
    const uint64_t s = (uint64_t)u * m + t;             // low word is 0
    return (uint32_t)(s >> 32) << b;
}

// r6 = 2^E mod m in [0, m) for E >= 33 (m < 2^28, odd, >= 3).
__device__ __forceinline__ uint32_t w1_pow2(uint64_t E, uint32_t m, uint32_t mp)
{
    // Ladder on E' = E - 32: invariant y = 2^(32 + prefix of E').
    const uint64_t Ep = E - 32;
    const int nb = 64 - __clzll((long long)Ep);
    uint64_t bits = Ep << (64 - nb);                    // leading 1 at bit 63
    uint32_t y = (uint32_t)pow2_start<33>(m);           // prefix '1': 2^33
    bits <<= 1;
    for (int i = 1; i < nb; ++i) {
        const uint32_t b = (uint32_t)(bits >> 63);
        bits <<= 1;
        y = w1_sqr(y, m, mp, b);
    }
    y = min(y, y - 2u * m);                            // [0,4m) -> [0,2m)
    y = min(y, y - m);                                 //        -> [0,m)
    return y;
}

// Six quotient digits of r_0 / m from r6 (digit 0 least significant), and r_0.
__device__ __forceinline__ uint32_t w1_digits(uint32_t r, uint32_t m, uint32_t mp, uint32_t q[6])
{
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        q[j] = r * mp;
        r = (uint32_t)(((uint64_t)q[j] * m + r) >> 32);
    }
    return r;
}

// ---------------------------------------------------------------- width 2 --
// y = (y0,y1) in [0,4m), m = (m0,m1) with 2^28 <= m < 2^50:
// REDC_2^64(y^2) << b by two 32-bit word steps, again in [0,4m).
__device__ __forceinline__ void w2_sqr(uint32_t &y0, uint32_t &y1, uint32_t m0, uint32_t m1,
                                       uint32_t mp, uint32_t b)
{
    // T = y^2 = t0 + t1 2^32 + t2 2^64 + t3 2^96  (< 16 m^2 < 2^104)
    const uint64_t a = (uint64_t)y0 * y0;
    const uint64_t p = (uint64_t)y0 * (y1 << 1);        // y1 < 2^20
    const uint64_t s = (uint64_t)y1 * y1;
    const uint32_t t0 = (uint32_t)a;
    uint32_t t1, t2, t3;
    asm("add.cc.u32 %0, %3, %4;\n\t"
        "addc.cc.u32 %1, %5, %6;\n\t"
        "addc.u32 %2, %7, 0;"
        : "=r"(t1), "=r"(t2), "=r"(t3)
        : "r"((uint32_t)(a >> 32)), "r"((uint32_t)p), "r"((uint32_t)(p >> 32)), "r"((uint32_t)s),
          "r"((uint32_t)(s >> 32)));
    // word step 1: (T + u0 m) / 2^32 = t1 + t2 2^32 + t3 2^64 + h0 + u0 m1
    const uint32_t u0 = t0 * mp;
    const uint32_t h0 = (uint32_t)(((uint64_t)u0 * m0 + t0) >> 32);
    const uint64_t g = (uint64_t)u0 * m1 + h0;
    uint32_t s0, s1, s2;
    asm("add.cc.u32 %0, %3, %4;\n\t"
        "addc.cc.u32 %1, %5, %6;\n\t"
        "addc.u32 %2, %7, 0;"
        : "=r"(s0), "=r"(s1), "=r"(s2)
        : "r"(t1), "r"((uint32_t)g), "r"(t2), "r"((uint32_t)(g >> 32)), "r"(t3));
    // word step 2
    const uint32_t u1 = s0 * mp;
    const uint32_t h1 = (uint32_t)(((uint64_t)u1 * m0 + s0) >> 32);
    const uint64_t z = (((uint64_t)s2 << 32) | s1) + ((uint64_t)u1 * m1 + h1);   // < 2m
    const uint32_t z0 = (uint32_t)z, z1 = (uint32_t)(z >> 32);
    y1 = __funnelshift_l(z0, z1, b);
    y0 = z0 << b;
}

// r6 = 2^E mod m in [0, m) as (lo, hi) for E >= 65 (2^28 <= m < 2^50).
__device__ __forceinline__ uint64_t w2_pow2(uint64_t E, uint64_t m, uint32_t mp)
{
    const uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
    const uint64_t Ep = E - 64;
    const int nb = 64 - __clzll((long long)Ep);
    uint64_t bits = Ep << (64 - nb);
    const uint64_t y = pow2_start<65>(m);               // prefix '1': 2^65
    uint32_t y0 = (uint32_t)y, y1 = (uint32_t)(y >> 32);
    bits <<= 1;
    for (int i = 1; i < nb; ++i) {
        const uint32_t b = (uint32_t)(bits >> 63);
        bits <<= 1;
        w2_sqr(y0, y1, m0, m1, mp, b);
    }
    uint64_t r = ((uint64_t)y1 << 32) | y0;
    r = min(r, r - 2 * m);
    r = min(r, r - m);
    return r;
}

__device__ __forceinline__ uint64_t w2_digits(uint64_t r, uint64_t m, uint32_t mp, uint32_t q[6])
{
    const uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
    uint32_t r0 = (uint32_t)r, r1 = (uint32_t)(r >> 32);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        q[j] = r0 * mp;
        const uint32_t h = (uint32_t)(((uint64_t)q[j] * m0 + r0) >> 32);
        const uint64_t w = (uint64_t)q[j] * m1 + h + r1;   // < m
        r0 = (uint32_t)w;
        r1 = (uint32_t)(w >> 32);
    }
    return ((uint64_t)r1 << 32) | r0;
}

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
