// cbl_kernels.cu - sm_103a kernels of the Bellard hot path.
//
//   terms192_kernel  persistent, work-stealing over warp tiles of (position,
//                    series, k-range): the 192-bit integer term sum that
//                    replaces Sglobal32mtg_192 / Sglobal64mtg_192(_Refresh) /
//                    Sglobal_after_192 (Bellard.cl:771-823, 992-1092, 1153-1253;
//                    Bellard_div2by1.cl:313-359) and their shared-memory
//                    reductions (Bellard.cl:601-675).
//   combine_kernel   Ssum_192 + Sum7_192 for every position (Bellard.cl:1300-1398).
//   dd_*             the 106-bit double-double mode (Bellard.cl:729-763, 914-982,
//                    1118-1144, 1274-1353), the only FP64 on the GPU.
#include "cbl_arith.cuh"
#include "cbl_internal.h"

namespace cbl {

constexpr int kBlock192 = 256;

// numer of series f as a shift (KernelFuncs.as:9): 32,1,256,64,4,4,1
__device__ __forceinline__ int numer_log2(int f)
{
    return (int)((0x0226805u >> (4 * f)) & 15u);
}

// ---------------------------------------------------------------- helpers --
// q >>= s for s in [0, 192), on six 32-bit digits (digit 0 least significant),
// with static register indexing only.
__device__ __forceinline__ void shr192(uint32_t q[6], int s)
{
    if (s >= 192) {
#pragma unroll
        for (int j = 0; j < 6; ++j) q[j] = 0;
        return;
    }
    const int ws = s >> 5, bs = s & 31;
#pragma unroll
    for (int t = 0; t < 5; ++t) {
        if (t < ws) {
#pragma unroll
            for (int j = 0; j < 5; ++j) q[j] = q[j + 1];
            q[5] = 0;
        }
    }
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = __funnelshift_r(q[j], q[j + 1], bs);
    q[5] >>= bs;
}

// One term's six quotient digits: k < d gives frac(2^(10(d-k))/m), k >= d the
// tail value 2^(-10(k-d))/m (digits of 1/m shifted right by 10(k-d)).
// KIND: 1 = width 1 (m < 2^28), 5 = middle width 1 (2^28 <= m < 2^31),
// 3 = strict width 1 (2^28 <= m < 2^32), 4 = short width 2 (2^32 <= m < 2^44),
// 2 = width 2 (2^28 <= m < 2^60), 6 = wide width 2 (2^60 <= m < 2^62).
template <int KIND, bool TAIL>
__device__ __forceinline__ void term_digits(uint64_t d, uint64_t k, uint64_t m, uint32_t q[6])
{
    const uint32_t mp = neg_inv32((uint32_t)m);
    const uint64_t E = TAIL ? 192ull : 10ull * (d - k) + 192ull;
    if (KIND == 1) {
        const uint32_t r6 = w1_pow2(E, (uint32_t)m, mp);
        w1_digits(r6, (uint32_t)m, mp, q);
    } else if (KIND == 5) {
        const uint32_t r6 = w1m_pow2(E, (uint32_t)m, mp);
        w1_digits(r6, (uint32_t)m, mp, q);
    } else if (KIND == 3) {
        const uint32_t r6 = w1s_pow2(E, (uint32_t)m, mp);
        w1_digits(r6, (uint32_t)m, mp, q);
    } else if (KIND == 4) {
        const uint64_t r6 = w2s_pow2(E, m, mp);
        w2_digits(r6, m, mp, q);
    } else if (KIND == 6) {
        const uint64_t r6 = w2x_pow2(E, m, mp);
        w2_digits(r6, m, mp, q);
    } else {
        const uint64_t r6 = w2_pow2(E, m, mp);
        w2_digits(r6, m, mp, q);
    }
    if (TAIL) shr192(q, (int)(10 * (k - d)));
}

// Two terms (k and k+32) of a lane per iteration, their ladders interleaved
// (kinds 1, 3, 4, 5; the width-2 kinds above 2^44 run one term at a time).
// Same-box timings against one term per iteration, identical bits: 1e9
// 40.65 -> 38.55 ms, 1e10 841.0 -> 838.9 ms, batch 10.61 -> 10.08 s. Pairing
// only some kinds traded these against each other (the kernel's code layout
// and registers change with every instantiation), so all four are paired.
template <int KIND>
__device__ __forceinline__ void term_pair(uint64_t d, uint64_t ka, uint64_t ma, uint64_t mb, uint32_t qa[6],
                                          uint32_t qb[6])
{
    const uint32_t mpa = neg_inv32((uint32_t)ma), mpb = neg_inv32((uint32_t)mb);
    const uint64_t Ea = 10ull * (d - ka) + 192ull, Eb = Ea - 320ull;
    if (KIND == 4) {
        W2SState A{0, 0, (uint32_t)ma, (uint32_t)(ma >> 32), mpa}, B{0, 0, (uint32_t)mb, (uint32_t)(mb >> 32), mpb};
        walk_bits_start_pair<4>(Ea - 48, Eb - 48, A, B, W2SStart{});   // R = 2^48
        uint64_t ra = ((uint64_t)A.y1 << 32) | A.y0, rb = ((uint64_t)B.y1 << 32) | B.y0;
        ra = min(ra, ra - 2 * ma);
        ra = min(ra, ra - ma);
        rb = min(rb, rb - 2 * mb);
        rb = min(rb, rb - mb);
        w2_digits(ra, ma, mpa, qa);
        w2_digits(rb, mb, mpb, qb);
    } else if (KIND == 1) {
        W1State A{0, (uint32_t)ma, mpa}, B{0, (uint32_t)mb, mpb};
        walk_bits_start_pair<1>(Ea - 32, Eb - 32, A, B, W1Start1{});
        uint32_t ya = A.y, yb = B.y;
        ya = min(ya, ya - 2u * (uint32_t)ma);
        ya = min(ya, ya - (uint32_t)ma);
        yb = min(yb, yb - 2u * (uint32_t)mb);
        yb = min(yb, yb - (uint32_t)mb);
        w1_digits(ya, (uint32_t)ma, mpa, qa);
        w1_digits(yb, (uint32_t)mb, mpb, qb);
    } else if (KIND == 5) {
        W1MState A{0, (uint32_t)ma, mpa}, B{0, (uint32_t)mb, mpb};
        walk_bits_start_pair<4>(Ea - 32, Eb - 32, A, B, W1MStart{});
        w1_digits(A.y, (uint32_t)ma, mpa, qa);
        w1_digits(B.y, (uint32_t)mb, mpb, qb);
    } else {
        W1SState A{0, (uint32_t)ma, mpa}, B{0, (uint32_t)mb, mpb};
        walk_bits_start_pair<4>(Ea - 32, Eb - 32, A, B, W1SStart{});
        w1_digits(A.y, (uint32_t)ma, mpa, qa);
        w1_digits(B.y, (uint32_t)mb, mpb, qb);
    }
}

template <int KIND, bool TAIL>
__device__ __forceinline__ void run_tile(const Seg &s, uint64_t kb, uint64_t ke, int lane, Acc192 &acc,
                                         uint32_t &cnt)
{
    uint64_t k = kb + lane;
    if (!TAIL && (KIND == 1 || KIND == 3 || KIND == 4 || KIND == 5)) {
        for (; k + 32 < ke; k += 64) {                  // terms k and k+32 together
            const uint64_t ma = (uint64_t)s.den0 * k + s.den1, mb = ma + 32ull * s.den0;
            uint32_t qa[6], qb[6];
            term_pair<KIND>(s.d, k, ma, mb, qa, qb);
            acc_add(acc, qa);
            acc_add(acc, qb);
            cnt += 2;
        }
    }
    for (; k < ke; k += 32) {
        const uint64_t m = (uint64_t)s.den0 * k + s.den1;
        uint32_t q[6];
        term_digits<KIND, TAIL>(s.d, k, m, q);
        acc_add(acc, q);
        ++cnt;
    }
}

// Add v to element j of a slot (six 64-bit digit sums, element j weighing
// 2^(32j)), exactly mod 2^192 however many tiles land in the slot. An add that
// wraps element j past 2^64 drops 2^64 * 2^(32j) = one unit of element j+2, so
// that unit is added there (and again on the rare wrap of that add); from
// element 6 on the weight is >= 2^192 and vanishes. Each wrap is seen by
// exactly the atomic that crossed 2^64, so concurrent flushes stay exact.
__device__ __forceinline__ void slot_add(unsigned long long *slot6, int j, unsigned long long v)
{
    for (;;) {
        const unsigned long long old = atomicAdd(slot6 + j, v);
        if (old + v >= old) return;
        j += 2;
        v = 1ull;
        if (j >= 6) return;
    }
}

// Warp sum of the lanes' 192-bit values, normalised, added into a slot's six
// 64-bit digit sums. Each add is < 2^32, so a slot that receives fewer than
// 2^32 flushes from zero cannot wrap and takes plain fire-and-forget adds;
// with carry set (a slot that may receive 2^31 or more flushes, or a preset
// start value) slot_add carries the wraps, and the number of flushes per slot
// is unbounded.
__device__ __forceinline__ void warp_flush(const Acc192 &acc, int lane, unsigned long long *slot6, int carry)
{
    uint64_t S[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const uint32_t lo = __reduce_add_sync(0xffffffffu, acc.w[j] & 0xffffu);
        const uint32_t hi = __reduce_add_sync(0xffffffffu, acc.w[j] >> 16);
        S[j] = (uint64_t)lo + ((uint64_t)hi << 16);
    }
    if (lane == 0) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const uint64_t t = S[j] + c;
            const uint32_t dj = (uint32_t)t;
            c = t >> 32;
            if (dj) {
                if (carry) slot_add(slot6, j, (unsigned long long)dj);
                else atomicAdd(slot6 + j, (unsigned long long)dj);
            }
        }
    }
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------------- terms192 kernel --
// Fold a warp's accumulated terms of one segment and add them into its slot.
// Every k of a lane has the parity of seg.k0 + lane (tiles hold an even number
// of terms), so the lane's sign (-1)^(k + sign) is fixed for the segment.
__device__ __forceinline__ void flush_segment(const Seg &s, int lane, Acc192 &acc, uint32_t cnt,
                                              unsigned long long *slots, int carry)
{
    if (((s.k0 + (uint64_t)lane + (s.flags & kFlagSign)) & 1ull) != 0) acc_negate_minus(acc, cnt);
    warp_flush(acc, lane, slots + (size_t)s.slot * 6, carry);
}

// With budget_ns != 0 a warp takes no new tile once budget_ns have passed
// since it started. The deadline is checked before the tile counter is
// incremented, so every tile taken is finished and the finished tiles are
// exactly [0, counter): a later launch continues from there.
// A warp keeps its lanes' sums across consecutive tiles of one segment and
// flushes them when it moves to another segment, when a lane's term count
// reaches 2^30, and before it exits: one slot update per run of tiles
// instead of one per tile.
__global__ void __launch_bounds__(kBlock192) terms192_kernel(const Seg *__restrict__ segs, int nseg,
                                                             uint64_t ntiles, uint32_t tile_k,
                                                             unsigned long long *counter,
                                                             unsigned long long *slots, uint64_t budget_ns,
                                                             int carry)
{
    const int lane = threadIdx.x & 31;
    const uint64_t t_start = budget_ns ? global_ns() : 0;
    int cur = -1;                                   // segment of the sums held in acc
    Acc192 acc;
    acc_zero(acc);
    uint32_t cnt = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) {
            if (budget_ns && global_ns() - t_start > budget_ns) t = ~0ull;
            else t = atomicAdd(counter, 1ull);
        }
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntiles) break;
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].tile0 <= t) lo = mid; else hi = mid - 1;
        }
        if (lo != cur || __any_sync(0xffffffffu, cnt >= (1u << 30))) {
            if (cur >= 0) flush_segment(segs[cur], lane, acc, cnt, slots, carry);
            acc_zero(acc);
            cnt = 0;
            cur = lo;
        }
        const Seg s = segs[lo];
        const uint64_t kb = s.k0 + (t - s.tile0) * tile_k;
        const uint64_t ke = min(s.k1, kb + tile_k);
        const int width = (int)((s.flags >> 4) & 15u);
        const bool tail = kb >= s.d;
        if (tail) {
            if (width == 1) run_tile<1, true>(s, kb, ke, lane, acc, cnt);
            else if (width == 5) run_tile<5, true>(s, kb, ke, lane, acc, cnt);
            else if (width == 3) run_tile<3, true>(s, kb, ke, lane, acc, cnt);
            else if (width == 4) run_tile<4, true>(s, kb, ke, lane, acc, cnt);
            else if (width == 6) run_tile<6, true>(s, kb, ke, lane, acc, cnt);
            else run_tile<2, true>(s, kb, ke, lane, acc, cnt);
        } else {
            if (width == 1) run_tile<1, false>(s, kb, ke, lane, acc, cnt);
            else if (width == 5) run_tile<5, false>(s, kb, ke, lane, acc, cnt);
            else if (width == 3) run_tile<3, false>(s, kb, ke, lane, acc, cnt);
            else if (width == 4) run_tile<4, false>(s, kb, ke, lane, acc, cnt);
            else if (width == 6) run_tile<6, false>(s, kb, ke, lane, acc, cnt);
            else run_tile<2, false>(s, kb, ke, lane, acc, cnt);
        }
    }
    if (cur >= 0) flush_segment(segs[cur], lane, acc, cnt, slots, carry);
}

cudaError_t launch_terms192(const Seg *segs, int nseg, uint64_t ntiles, uint32_t tile_k,
                            unsigned long long *counter, unsigned long long *slots, int grid, int block,
                            cudaStream_t st, uint64_t budget_ns, bool carry)
{
    (void)block;
    terms192_kernel<<<grid, kBlock192, 0, st>>>(segs, nseg, ntiles, tile_k, counter, slots, budget_ns,
                                                carry ? 1 : 0);
    return cudaGetLastError();
}

int terms192_max_ctas_per_sm(int block)
{
    int n = 0;
    (void)block;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, terms192_kernel, kBlock192, 0) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

int device_sm_count(int device)
{
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    return n;
}

// ------------------------------------------------------ 192-bit combine --
// Six 64-bit digit sums (digit j weighs 2^(32j)) -> 192 bits as 3 little-endian words.
__device__ __forceinline__ void normalise6(const unsigned long long *s6, uint64_t w[3])
{
    uint32_t dgt[6];
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const uint64_t v = s6[j];
        const uint64_t lo = (v & 0xffffffffull) + c;
        dgt[j] = (uint32_t)lo;
        c = (v >> 32) + (lo >> 32);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = ((uint64_t)dgt[2 * i + 1] << 32) | dgt[2 * i];
}

__device__ __forceinline__ void shl192(uint64_t w[3], int s)   // 0 <= s < 64, mod 2^192
{
    if (s == 0) return;
    w[2] = (w[2] << s) | (w[1] >> (64 - s));
    w[1] = (w[1] << s) | (w[0] >> (64 - s));
    w[0] <<= s;
}

__device__ __forceinline__ void add192(uint64_t a[3], const uint64_t b[3])
{
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const uint64_t s = a[i] + b[i];
        const uint64_t c1 = s < a[i];
        a[i] = s + c;
        c = c1 | (a[i] < s);
    }
}

// Every slot's six digit sums <- preset[0..6) (a test hook: presets near 2^64
// make the sums wrap within a few tiles).
__global__ void slot_fill_kernel(unsigned long long *slots, int nslot, const unsigned long long *preset)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nslot * 6) slots[i] = preset[i % 6];
}

cudaError_t launch_slot_fill(unsigned long long *slots, int nslot, const unsigned long long *preset,
                             cudaStream_t st)
{
    const int b = 256;
    slot_fill_kernel<<<(nslot * 6 + b - 1) / b, b, 0, st>>>(slots, nslot, preset);
    return cudaGetLastError();
}

__global__ void combine_kernel(const unsigned long long *slots, int npos, const int *shift, uint64_t *out3,
                               uint64_t *partial7)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npos) return;
    uint64_t ans[3] = {0, 0, 0};
    const int sh = shift ? shift[i] : 0;
    for (int f = 0; f < 7; ++f) {
        uint64_t w[3];
        normalise6(slots + ((size_t)i * 7 + f) * 6, w);
        shl192(w, numer_log2(f) + sh);
        if (partial7) {
            uint64_t *p = partial7 + ((size_t)i * 7 + f) * 3;
            p[0] = w[2]; p[1] = w[1]; p[2] = w[0];
        }
        add192(ans, w);
    }
    out3[3 * (size_t)i + 0] = ans[2];
    out3[3 * (size_t)i + 1] = ans[1];
    out3[3 * (size_t)i + 2] = ans[0];
}

cudaError_t launch_combine(const unsigned long long *slots, int npos, const int *shift, uint64_t *out3,
                           uint64_t *partial7, cudaStream_t st)
{
    const int b = 128;
    combine_kernel<<<(npos + b - 1) / b, b, 0, st>>>(slots, npos, shift, out3, partial7);
    return cudaGetLastError();
}

__global__ void ssum192_kernel(const unsigned long long *slots, uint64_t *partial)
{
    uint64_t w[3];
    normalise6(slots, w);
    partial[0] = w[2]; partial[1] = w[1]; partial[2] = w[0];
}

cudaError_t launch_ssum192(const unsigned long long *slots, uint64_t *partial, cudaStream_t st)
{
    ssum192_kernel<<<1, 1, 0, st>>>(slots, partial);
    return cudaGetLastError();
}

__global__ void sum7_192_kernel(uint64_t *partial, uint64_t *ans, int sh)
{
    uint64_t w[3] = {partial[2], partial[1], partial[0]};
    shl192(w, sh);
    partial[0] = w[2]; partial[1] = w[1]; partial[2] = w[0];
    uint64_t a[3] = {ans[2], ans[1], ans[0]};
    add192(a, w);
    ans[0] = a[2]; ans[1] = a[1]; ans[2] = a[0];
}

cudaError_t launch_sum7_192(uint64_t *partial, uint64_t *ans, int numer_log2, cudaStream_t st)
{
    sum7_192_kernel<<<1, 1, 0, st>>>(partial, ans, numer_log2);
    return cudaGetLastError();
}

// ---------------------------------------------------------- per-term kernel --
__global__ void terms_each_kernel(uint64_t d, uint32_t den0, uint32_t den1, int sign, const uint64_t *ks, int n,
                                  uint64_t *out3n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = ks[i];
    const uint64_t m = (uint64_t)den0 * k + den1;
    uint32_t q[6] = {0, 0, 0, 0, 0, 0};
    if (m != 1) {
        if (k < d) {
            if (m < kW1Max) term_digits<1, false>(d, k, m, q);
            else if (m < kW1MMax) term_digits<5, false>(d, k, m, q);
            else if (m < kW1SMax) term_digits<3, false>(d, k, m, q);
            else if (m < kW2SMax) term_digits<4, false>(d, k, m, q);
            else if (m < kW2Max) term_digits<2, false>(d, k, m, q);
            else term_digits<6, false>(d, k, m, q);
        } else {
            if (m < kW1Max) term_digits<1, true>(d, k, m, q);
            else if (m < kW1MMax) term_digits<5, true>(d, k, m, q);
            else if (m < kW1SMax) term_digits<3, true>(d, k, m, q);
            else if (m < kW2SMax) term_digits<4, true>(d, k, m, q);
            else if (m < kW2Max) term_digits<2, true>(d, k, m, q);
            else term_digits<6, true>(d, k, m, q);
        }
        if ((k + (uint64_t)sign) & 1ull)
            for (int j = 0; j < 6; ++j) q[j] = ~q[j];
    }
    out3n[3 * (size_t)i + 0] = ((uint64_t)q[5] << 32) | q[4];
    out3n[3 * (size_t)i + 1] = ((uint64_t)q[3] << 32) | q[2];
    out3n[3 * (size_t)i + 2] = ((uint64_t)q[1] << 32) | q[0];
}

cudaError_t launch_terms_each(uint64_t d, uint32_t den0, uint32_t den1, int sign, const uint64_t *k, int n,
                              uint64_t *out3n, cudaStream_t st)
{
    const int b = 128;
    terms_each_kernel<<<(n + b - 1) / b, b, 0, st>>>(d, den0, den1, sign, k, n, out3n);
    return cudaGetLastError();
}

// ------------------------------------------------------ double-double mode --
struct DD {
    double hi, lo;
};

__device__ __forceinline__ DD two_sum(double a, double b)
{
    const double s = a + b;
    const double bb = s - a;
    return DD{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ DD dd_add(DD a, DD b)
{
    DD s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return two_sum(s.hi, s.lo);
}

// Into (-1, 1): drop the integer part of hi (sumfix2, Bellard.cl:472-488).
__device__ __forceinline__ DD dd_frac(DD a)
{
    const double t = trunc(a.hi);
    return (t != 0.0) ? two_sum(a.hi - t, a.lo) : a;
}

// x / y to ~106 bits (nn_div, Bellard.cl:99-106), with an exact fma residual.
__device__ __forceinline__ DD dd_div_nn(double x, double y)
{
    const double q1 = x / y;
    const double rem = fma(-q1, y, x);
    const double q2 = rem / y;
    return two_sum(q1, q2);
}

// An integer 0 <= x < 2^63 as an exact double-double: hi = x rounded to 53
// bits, lo = the (small, signed) rest.
__device__ __forceinline__ DD dd_from_u64(uint64_t x)
{
    const double hi = __ull2double_rn(x);
    const int64_t rest = (int64_t)(x - __double2ull_rn(hi));
    return DD{hi, (double)rest};
}

// a / b for exact double-doubles a >= 0, b > 0 of integers (the OVERDOUBLE case
// m >= 2^53 of Bellard.cl:937-945, 1040-1047): q1 = a.hi / b.hi, the remainder
// a - q1 b formed with an exact product (fma) and a single rounding of the
// q1 b.lo term, then one correction quotient. For b ~ 2^e the remainder is
// ~2^(e-53) and carries errors ~2^(e-106), so the quotient keeps ~104 bits.
__device__ __forceinline__ DD dd_div_dd(DD a, DD b)
{
    const double q1 = a.hi / b.hi;
    const double p_hi = q1 * b.hi;
    const double p_lo = fma(q1, b.hi, -p_hi);            // q1 b.hi = p_hi + p_lo exactly
    double e = a.hi - p_hi;                               // exact: p_hi is within a factor 2 of a.hi
    e += a.lo - p_lo;
    e = fma(-q1, b.lo, e);
    const double q2 = e / b.hi;
    return two_sum(q1, q2);
}

constexpr int kBlockDD = 256;

__device__ __forceinline__ DD block_reduce_dd(DD v)
{
    __shared__ double sh_hi[kBlockDD], sh_lo[kBlockDD];
    const int t = threadIdx.x;
    sh_hi[t] = v.hi;
    sh_lo[t] = v.lo;
    for (int i = kBlockDD / 2; i > 0; i >>= 1) {
        __syncthreads();
        if (t < i) {
            const DD a = dd_frac(dd_add(DD{sh_hi[t], sh_lo[t]}, DD{sh_hi[t + i], sh_lo[t + i]}));
            sh_hi[t] = a.hi;
            sh_lo[t] = a.lo;
        }
    }
    __syncthreads();
    return DD{sh_hi[0], sh_lo[0]};
}

__global__ void __launch_bounds__(kBlockDD) dd_terms_kernel(double2 *bigsum, uint64_t k0, uint64_t k1, uint64_t d,
                                                            int sign, uint32_t den0, uint32_t den1)
{
    const uint64_t gsize = (uint64_t)gridDim.x * blockDim.x;
    DD sum{0.0, 0.0};
    for (uint64_t k = k0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gsize) {
        const uint64_t m = (uint64_t)den0 * k + den1;
        if (m == 1) continue;
        const uint32_t mp = neg_inv32((uint32_t)m);
        // r = 2^(10(d-k)) mod m: the ladder to 2^(10(d-k) + 32 j) and j REDC
        // steps down (j = 1 one word, 2 two words); no quotient digits.
        const uint64_t e = 10ull * (d - k);
        uint64_t r;
        if (m < kW1SMax) {
            uint32_t y;
            if (m < kW1Max) y = w1_pow2(e + 32, (uint32_t)m, mp);
            else if (m < kW1MMax) y = w1m_pow2(e + 32, (uint32_t)m, mp);
            else y = w1s_pow2(e + 32, (uint32_t)m, mp);
            r = redc_word(y * mp, (uint32_t)m, y, 0u);
        } else {
            uint64_t y;
            if (m < kW2SMax) y = w2s_pow2(e + 64, m, mp);
            else if (m < kW2Max) y = w2_pow2(e + 64, m, mp);
            else y = w2x_pow2(e + 64, m, mp);
            uint32_t q[2];
            r = w2_redc_down<2>(y, m, mp, q);
        }
        // r and m are exact doubles below 2^53; above, exact double-doubles
        DD t = (m < kDDMax) ? dd_div_nn((double)r, (double)m) : dd_div_dd(dd_from_u64(r), dd_from_u64(m));
        if ((k + (uint64_t)sign) & 1ull) { t.hi = -t.hi; t.lo = -t.lo; }
        sum = dd_frac(dd_add(sum, t));
    }
    const DD b = block_reduce_dd(sum);
    if (threadIdx.x == 0) {
        const double2 o = bigsum[blockIdx.x];
        const DD s = dd_frac(dd_add(DD{o.x, o.y}, b));
        bigsum[blockIdx.x] = make_double2(s.hi, s.lo);
    }
}

cudaError_t launch_dd_terms(double2 *bigsum, int nblk, int block, uint64_t k0, uint64_t k1, uint64_t d, int sign,
                            uint32_t den0, uint32_t den1, cudaStream_t st)
{
    (void)block;
    dd_terms_kernel<<<nblk, kBlockDD, 0, st>>>(bigsum, k0, k1, d, sign, den0, den1);
    return cudaGetLastError();
}

__global__ void dd_tail_kernel(double2 *bigsum, uint64_t d, int sign, uint32_t den0, uint32_t den1)
{
    DD sum{0.0, 0.0};
    double p = 1.0;
    for (int i = 0; i < kTailDD; ++i) {
        const uint64_t k = d + (uint64_t)i;
        const uint64_t m = (uint64_t)den0 * k + den1;
        if (m != 1) {
            DD t = (m < kDDMax) ? dd_div_nn(p, (double)m) : dd_div_dd(DD{p, 0.0}, dd_from_u64(m));
            if ((k + (uint64_t)sign) & 1ull) { t.hi = -t.hi; t.lo = -t.lo; }
            sum = dd_add(sum, t);
        }
        p *= 0.0009765625;   // 2^-10
    }
    const double2 o = bigsum[0];
    const DD s = dd_frac(dd_add(DD{o.x, o.y}, sum));
    bigsum[0] = make_double2(s.hi, s.lo);
}

cudaError_t launch_dd_tail(double2 *bigsum, uint64_t d, int sign, uint32_t den0, uint32_t den1, cudaStream_t st)
{
    dd_tail_kernel<<<1, 1, 0, st>>>(bigsum, d, sign, den0, den1);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(kBlockDD) dd_ssum_kernel(const double2 *bigsum, int nblk, double2 *partial)
{
    DD s{0.0, 0.0};
    for (int i = threadIdx.x; i < nblk; i += kBlockDD) s = dd_frac(dd_add(s, DD{bigsum[i].x, bigsum[i].y}));
    const DD b = block_reduce_dd(s);
    if (threadIdx.x == 0) *partial = make_double2(b.hi, b.lo);
}

cudaError_t launch_dd_ssum(const double2 *bigsum, int nblk, double2 *partial, cudaStream_t st)
{
    dd_ssum_kernel<<<1, kBlockDD, 0, st>>>(bigsum, nblk, partial);
    return cudaGetLastError();
}

__device__ __forceinline__ DD dd_unit(DD a)   // into [0, 1)
{
    a = dd_frac(a);
    if (a.hi < 0.0 || (a.hi == 0.0 && a.lo < 0.0)) a = dd_add(a, DD{1.0, 0.0});
    if (a.hi >= 1.0) a = dd_add(a, DD{-1.0, 0.0});
    return a;
}

// Sum7 (Bellard.cl:1324-1353): weight by numer, keep the fraction, write back,
// add into the answer.
__global__ void dd_sum7_kernel(double2 *partial, double2 *ans, int numer)
{
    DD a = dd_unit(DD{partial->x, partial->y});
    a.hi *= (double)numer;
    a.lo *= (double)numer;
    a = dd_unit(a);
    *partial = make_double2(a.hi, a.lo);
    const DD s = dd_unit(dd_add(DD{ans->x, ans->y}, a));
    *ans = make_double2(s.hi, s.lo);
}

cudaError_t launch_dd_sum7(double2 *partial, double2 *ans, int numer, cudaStream_t st)
{
    dd_sum7_kernel<<<1, 1, 0, st>>>(partial, ans, numer);
    return cudaGetLastError();
}

}  // namespace cbl

namespace cbl {

// ------------------------------------------------------------ IMAD probe --
// 16 independent dependent chains of mad.lo.u32 per thread, one multiply half
// per instruction: the full issue rate of the FMA-heavy pipe, which is the
// peak of the term kernels' algorithmic work unit (a multiply half).
__global__ void __launch_bounds__(256) probe_imad_kernel(uint32_t *sink, int iters)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x[16], a[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        a[j] = t * 2654435761u + 7919u * j;
        x[j] = (t ^ (0x9e3779b9u * (j + 1))) | 1u;
    }
    const uint32_t k1 = 0x7feb352du;
    // 16 independent chains x = x k1 + a: each multiply needs the previous
    // one's result, so none can be hoisted out of the loop, and 16 chains per
    // thread hide the latency: the issue rate of mad.lo.u32 (one multiply half
    // each) is measured. A full 32x32 product (two halves) issues at half this
    // rate, so the rate of halves is the same for wide products.
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[j]) : "r"(k1), "r"(a[j]));
    }
    uint32_t r = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) r ^= x[j];
    sink[t] = r;
}

int probe_imad_grid(int sm_count)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, probe_imad_kernel, 256, 0) != cudaSuccess || n < 1) n = 1;
    return sm_count * n;
}

cudaError_t launch_probe_imad(uint32_t *sink, int grid, int block, int iters, uint64_t *ops, cudaStream_t st)
{
    (void)block;
    probe_imad_kernel<<<grid, 256, 0, st>>>(sink, iters);
    if (ops) *ops = (uint64_t)grid * block * (uint64_t)iters * 16ull;   // one half per mad.lo
    return cudaGetLastError();
}

}  // namespace cbl
