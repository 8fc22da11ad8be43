// cbl_internal.h - shared between the kernels (cbl_kernels.cu) and the host
// library (cbl_host.cu). Not part of the public ABI.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include <new>

// Every int-returning entry point runs inside this guard, so no C++ exception
// crosses the C ABI: a failed host allocation returns CBL_E_NOMEM, anything
// else CBL_E_ARG.
#define CBL_GUARD_BEGIN try {
#define CBL_GUARD_END                                                                   \
    }                                                                                   \
    catch (const std::bad_alloc &) { return CBL_E_NOMEM; }                              \
    catch (...) { return CBL_E_ARG; }

namespace cbl {

// The 7 series (KernelFuncs.as:9-12).
constexpr int kNumer[7] = {32, 1, 256, 64, 4, 4, 1};
constexpr int kNumerLog2[7] = {5, 0, 8, 6, 2, 2, 0};
constexpr int kSign[7] = {1, 1, 0, 1, 1, 1, 0};      // 1 = minus
constexpr uint32_t kDen0[7] = {4, 4, 10, 10, 10, 10, 10};
constexpr uint32_t kDen1[7] = {1, 3, 1, 3, 5, 7, 9};

// Residue-width limits of the term kernels (m odd, m >= 3).
constexpr uint64_t kW1Max = 1ull << 28;   // width 1 (one 32-bit word) for m < 2^28
constexpr uint64_t kW1MMax = 1ull << 31;  // middle width 1 for 2^28 <= m < 2^31
constexpr uint64_t kW1SMax = 1ull << 32;  // strict width 1 for 2^31 <= m < 2^32
constexpr uint64_t kW2SMax = 1ull << 44;  // short width 2 for 2^32 <= m < 2^44
constexpr uint64_t kW2Max = 1ull << 60;   // width 2 (two words, residues < 4m) for m < 2^60
constexpr uint64_t kW2XMax = 1ull << 62;  // wide width 2 (residues < 2m) for 2^60 <= m < 2^62
constexpr uint64_t kDDMax = 1ull << 53;   // double-double mode: m and r exact as doubles below, double-doubles above

constexpr int kTail192 = 20;   // tail terms k = d..d+19 (Bellard.cl:1164-1239)
constexpr int kTailDD = 10;    // tail terms k = d..d+9  (Bellard.cl:1125)

// One contiguous k-range of one series at one position, within one residue
// width. Tiles of `tile_k` consecutive k are handed to warps in order of the
// global tile index; tile0 is this segment's first tile.
struct Seg {
    uint64_t d;
    uint64_t k0, k1;       // [k0, k1); k >= d are tail terms 2^(-10(k-d))/m
    uint64_t tile0;
    uint32_t den0, den1;
    uint32_t slot;         // accumulator slot (6 x u64 digit sums)
    uint32_t flags;        // bit 0: series sign (1 = minus), bits 4-7: residue kind 1..6
};
static_assert(sizeof(Seg) == 48, "Seg layout");

constexpr uint32_t kFlagSign = 1u;
inline uint32_t seg_flags(int sign, int width) { return (uint32_t)(sign & 1) | ((uint32_t)width << 4); }

// Launch wrappers (cbl_kernels.cu).
// budget_ns = 0: run to the end; else warps stop taking tiles after budget_ns
// and the finished tiles are [0, *counter).
// carry: the slots' digit sums may wrap past 2^64 (a slot can receive 2^31 or
// more flushes since it was zeroed, or it started from a preset); the flushes
// then carry each wrap into the digit sum two places up (exact mod 2^192).
// A slot receives at most one flush per tile, so slot_needs_carry() decides it
// from the tile counts.
cudaError_t launch_terms192(const Seg *segs, int nseg, uint64_t ntiles, uint32_t tile_k,
                            unsigned long long *counter, unsigned long long *slots, int grid, int block,
                            cudaStream_t st, uint64_t budget_ns, bool carry);
constexpr uint64_t kCarryTiles = 1ull << 31;
inline bool slot_needs_carry(uint64_t max_tiles_per_slot) { return max_tiles_per_slot >= kCarryTiles; }
// slots (nslot x 6 digit sums) of position i, series f = slots[(slot_base[i] + f) * 6 ..]:
// out3[3i..3i+2] (word 0 most significant) = sum_f (S_f << (numer_log2[f] + shift[i])).
// If partial7 != nullptr it also receives the 7 weighted partials per position.
cudaError_t launch_combine(const unsigned long long *slots, int npos, const int *shift,
                           uint64_t *out3, uint64_t *partial7, cudaStream_t st);
// slots[0 .. 6*nslot) <- preset[j % 6] (device array of 6), instead of zero.
cudaError_t launch_slot_fill(unsigned long long *slots, int nslot, const unsigned long long *preset,
                             cudaStream_t st);
// Reference-style single-series pieces on 192-bit buffers:
//  normalise slot 0 into partial[3] (Ssum_192)
cudaError_t launch_ssum192(const unsigned long long *slots, uint64_t *partial, cudaStream_t st);
//  partial <- partial << log2(numer); ans += partial (Sum7_192)
cudaError_t launch_sum7_192(uint64_t *partial, uint64_t *ans, int numer_log2, cudaStream_t st);
// Per-term evaluation (diagnostics and per-term parity).
cudaError_t launch_terms_each(uint64_t d, uint32_t den0, uint32_t den1, int sign, const uint64_t *k,
                              int n, uint64_t *out3n, cudaStream_t st);

// Double-double (mode 0) kernels.
cudaError_t launch_dd_terms(double2 *bigsum, int nblk, int block, uint64_t k0, uint64_t k1,
                            uint64_t d, int sign, uint32_t den0, uint32_t den1, cudaStream_t st);
cudaError_t launch_dd_tail(double2 *bigsum, uint64_t d, int sign, uint32_t den0, uint32_t den1,
                           cudaStream_t st);
cudaError_t launch_dd_ssum(const double2 *bigsum, int nblk, double2 *partial, cudaStream_t st);
cudaError_t launch_dd_sum7(double2 *partial, double2 *ans, int numer, cudaStream_t st);

// Throughput probe: grid x block threads each run `iters` rounds of 16
// independent dependent mad.lo.u32 chains; *ops = multiply halves issued.
cudaError_t launch_probe_imad(uint32_t *sink, int grid, int block, int iters, uint64_t *ops, cudaStream_t st);
int probe_imad_grid(int sm_count);   // one full wave of probe CTAs

int device_sm_count(int device);
int terms192_max_ctas_per_sm(int block);

}  // namespace cbl
