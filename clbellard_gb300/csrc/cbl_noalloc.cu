// cbl_noalloc.cu - an entry point for callers that may not allocate device
// memory: cbl_batch_noalloc. It evaluates up to CBL_NOALLOC_MAX_POSITIONS
// reference positions in 192-bit mode with the same persistent term kernel
// and combine kernel as cbl_batch, but every piece of scratch those kernels
// need (tile counter, per-series digit sums, per-position shifts, the tile
// table) lives in one fixed-size array defined in this file. The caller passes
// the positions and a device output buffer it already owns.
//
// The positions travel to the GPU as a kernel parameter, and a one-block
// kernel builds the tile table in the array, so a call issues no host-to-device
// copy: it enqueues a memset and three kernels on the caller's stream and
// returns without waiting for them.
#include "../../include/clbellard.h"
#include "cbl_internal.h"

#include <mutex>

using namespace cbl;

namespace {

constexpr int kMaxPos = CBL_NOALLOC_MAX_POSITIONS;
// One series covers k in [0, d + 20), cut at d (main body / tail) and at the
// five residue-kind boundaries m = 2^28, 2^31, 2^32, 2^44, 2^60: at most 7 pieces.
constexpr int kMaxPieces = 7;
constexpr int kMaxSegs = kMaxPos * 7 * kMaxPieces;
constexpr int kBuckets = 12;                      // (main, tail) x 6 residue kinds, costliest first
constexpr uint64_t kTileTerms = 2048;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCounter = 0;                                          // 8 bytes
constexpr size_t kOffSlots = 256;                                          // 7 x 6 digit sums per position
constexpr size_t kOffShift = align256(kOffSlots + (size_t)kMaxPos * 7 * 6 * 8);
constexpr size_t kOffSegs = align256(kOffShift + (size_t)kMaxPos * sizeof(int));
constexpr size_t kScratchBytes = align256(kOffSegs + (size_t)kMaxSegs * sizeof(Seg));
static_assert(kScratchBytes == CBL_NOALLOC_SCRATCH_BYTES, "scratch size documented in clbellard.h");

typedef unsigned __int128 u128;

// The 7 series (KernelFuncs.as:9-12) packed for host and device code alike.
__host__ __device__ __forceinline__ uint32_t series_den0(int f) { return f < 2 ? 4u : 10u; }
__host__ __device__ __forceinline__ uint32_t series_den1(int f) { return (0x9753131u >> (4 * f)) & 15u; }
__host__ __device__ __forceinline__ int series_sign(int f) { return (0x3Bu >> f) & 1u; }

struct Piece {
    uint64_t k0, k1;
    uint32_t kind;     // residue kind 1..6 (cbl_internal.h)
};

// The pieces of series f at position d, in increasing k. k = 0 of a series
// with den1 = 1 has m = 1 and contributes exactly 0, so it is left out.
__host__ __device__ inline int series_pieces(uint64_t d, int f, Piece out[kMaxPieces])
{
    const uint64_t den0 = series_den0(f), den1 = series_den1(f);
    const uint64_t k0 = den1 == 1 ? 1 : 0, k1 = d + kTail192;
    const uint64_t cut[6] = {d,
                             (kW1Max - den1 + den0 - 1) / den0,     // first k with m >= 2^28
                             (kW1MMax - den1 + den0 - 1) / den0,    // 2^31
                             (kW1SMax - den1 + den0 - 1) / den0,    // 2^32
                             (kW2SMax - den1 + den0 - 1) / den0,    // 2^44
                             (kW2Max - den1 + den0 - 1) / den0};    // 2^60
    uint64_t pts[8] = {k0, k1};
    for (int i = 0; i < 6; ++i) pts[2 + i] = cut[i] < k0 ? k0 : (cut[i] > k1 ? k1 : cut[i]);
    for (int i = 1; i < 8; ++i)                                      // insertion sort
        for (int j = i; j > 0 && pts[j - 1] > pts[j]; --j) {
            const uint64_t t = pts[j];
            pts[j] = pts[j - 1];
            pts[j - 1] = t;
        }
    int n = 0;
    for (int i = 0; i + 1 < 8; ++i) {
        const uint64_t a = pts[i], b = pts[i + 1];
        if (b <= a) continue;
        const uint32_t kind = a >= cut[5] ? 6 : a >= cut[4] ? 2 : a >= cut[3] ? 4 : a >= cut[2] ? 3 : a >= cut[1] ? 5 : 1;
        out[n++] = Piece{a, b, kind};
    }
    return n;
}

// Bucket of a piece: main body before tail, then the costlier residue kind
// first (wide width 2, width 2, short width 2, strict, middle, width 1).
__host__ __device__ __forceinline__ int piece_bucket(const Piece &p, uint64_t d)
{
    const int order = p.kind == 6 ? 0 : p.kind == 2 ? 1 : p.kind == 4 ? 2 : p.kind == 3 ? 3 : p.kind == 5 ? 4 : 5;
    return (p.k0 >= d ? 6 : 0) + order;
}

__host__ __device__ __forceinline__ uint64_t piece_tiles(const Piece &p)
{
    return (p.k1 - p.k0 + kTileTerms - 1) / kTileTerms;
}

struct PositionArgs {
    uint64_t d[kMaxPos];
    int n;
};

}  // namespace

// The scratch array. Every GPU that loads this library holds it until the
// process exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// One block of kMaxPos threads, thread i for position i. The table is ordered
// costliest tiles first: by bucket, then by d (larger first, ties by position
// index), then by series; a series has at most one piece per bucket. Thread i
// counts its pieces and tiles per bucket under its rank in that d order, one
// thread turns the counts into offsets, then every thread writes its segments.
__global__ void __launch_bounds__(kMaxPos) noalloc_table_kernel(PositionArgs a, Seg *segs)
{
    __shared__ uint32_t seg_off[kBuckets][kMaxPos];
    __shared__ uint64_t tile_off[kBuckets][kMaxPos];
    const int i = threadIdx.x;
    for (int b = 0; b < kBuckets; ++b) {
        seg_off[b][i] = 0;
        tile_off[b][i] = 0;
    }
    __syncthreads();
    int rank = 0;
    uint64_t d = 0;
    Piece p[kMaxPieces];
    if (i < a.n) {
        d = a.d[i];
        for (int j = 0; j < a.n; ++j)
            if (a.d[j] > d || (a.d[j] == d && j < i)) ++rank;
        for (int f = 0; f < 7; ++f) {
            const int np = series_pieces(d, f, p);
            for (int q = 0; q < np; ++q) {
                const int b = piece_bucket(p[q], d);
                seg_off[b][rank] += 1;
                tile_off[b][rank] += piece_tiles(p[q]);
            }
        }
    }
    __syncthreads();
    if (i == 0) {                                           // exclusive scan, bucket-major then rank
        uint32_t s = 0;
        uint64_t t = 0;
        for (int b = 0; b < kBuckets; ++b)
            for (int r = 0; r < a.n; ++r) {
                const uint32_t cs = seg_off[b][r];
                const uint64_t ct = tile_off[b][r];
                seg_off[b][r] = s;
                tile_off[b][r] = t;
                s += cs;
                t += ct;
            }
    }
    __syncthreads();
    if (i >= a.n) return;
    for (int f = 0; f < 7; ++f) {
        const int np = series_pieces(d, f, p);
        for (int q = 0; q < np; ++q) {
            const int b = piece_bucket(p[q], d);
            Seg s;
            s.d = d;
            s.k0 = p[q].k0;
            s.k1 = p[q].k1;
            s.tile0 = tile_off[b][rank];
            s.den0 = series_den0(f);
            s.den1 = series_den1(f);
            s.slot = (uint32_t)(i * 7 + f);
            s.flags = (uint32_t)series_sign(f) | (p[q].kind << 4);
            segs[seg_off[b][rank]] = s;
            seg_off[b][rank] += 1;                          // this (bucket, rank) cell is this thread's alone
            tile_off[b][rank] += piece_tiles(p[q]);
        }
    }
}

namespace {

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch on this device
    int grid = 0;
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Once per device, with that device current: resolve the array's device
// address (the host-side name is only a stand-in), size the persistent grid,
// and load the table kernel, so later calls only enqueue work.
int setup_device(int dev, DeviceSetup **out)
{
    if (dev < 0 || dev >= kMaxDevices) return CBL_E_NODEVICE;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceSetup &s = g_setup[dev];
    if (!s.ready) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return CBL_E_CUDA;
        const int sms = device_sm_count(dev);
        if (sms <= 0) return CBL_E_CUDA;
        cudaFuncAttributes attr;
        if (cudaFuncGetAttributes(&attr, noalloc_table_kernel) != cudaSuccess) return CBL_E_CUDA;
        s.scratch = static_cast<unsigned char *>(p);
        s.grid = sms * terms192_max_ctas_per_sm(256);
        s.ready = true;
    }
    *out = &s;
    return CBL_OK;
}

}  // namespace

extern "C" int cbl_batch_noalloc(const uint64_t *pos, int n, uint64_t *d_out3n, void *stream)
{
    CBL_GUARD_BEGIN
    if (n < 0 || (n > 0 && (!pos || !d_out3n))) return CBL_E_ARG;
    if (n > kMaxPos) return CBL_E_LIMIT;
    if (n == 0) return CBL_OK;
    // positions as a kernel parameter; segment and tile counts from the same
    // piece arithmetic the table kernel runs
    PositionArgs args;
    args.n = n;
    int nseg = 0;
    uint64_t ntiles = 0, max_series_tiles = 0;
    for (int i = 0; i < n; ++i) {
        uint64_t d = 0;
        const int rc = cbl_pos_to_d(pos[i], &d, nullptr);
        if (rc) return rc;
        if ((u128)10 * (d + kTail192 - 1) + 9 >= (u128)kW2XMax) return CBL_E_POSITION;
        args.d[i] = d;
        Piece p[kMaxPieces];
        for (int f = 0; f < 7; ++f) {
            const int np = series_pieces(d, f, p);
            nseg += np;
            uint64_t series_tiles = 0;
            for (int q = 0; q < np; ++q) series_tiles += piece_tiles(p[q]);
            ntiles += series_tiles;
            max_series_tiles = max_series_tiles > series_tiles ? max_series_tiles : series_tiles;
        }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CBL_E_NODEVICE;
    DeviceSetup *ds = nullptr;
    const int rc = setup_device(dev, &ds);
    if (rc) return rc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = ds->scratch;
    auto *counter = reinterpret_cast<unsigned long long *>(base + kOffCounter);
    auto *slots = reinterpret_cast<unsigned long long *>(base + kOffSlots);
    auto *shift = reinterpret_cast<int *>(base + kOffShift);
    auto *dsegs = reinterpret_cast<Seg *>(base + kOffSegs);
    // the array keeps the previous call's contents: zero the counter, the digit
    // sums and the shifts; the table kernel overwrites the first nseg segments
    if (cudaMemsetAsync(base, 0, kOffSegs, st) != cudaSuccess) return CBL_E_CUDA;
    noalloc_table_kernel<<<1, kMaxPos, 0, st>>>(args, dsegs);
    if (cudaGetLastError() != cudaSuccess) return CBL_E_CUDA;
    if (launch_terms192(dsegs, nseg, ntiles, (uint32_t)kTileTerms, counter, slots, ds->grid, 256, st, 0,
                        slot_needs_carry(max_series_tiles)) != cudaSuccess)
        return CBL_E_CUDA;
    if (launch_combine(slots, n, shift, d_out3n, nullptr, st) != cudaSuccess) return CBL_E_CUDA;
    return CBL_OK;
    CBL_GUARD_END
}
