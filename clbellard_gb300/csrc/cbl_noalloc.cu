// cbl_noalloc.cu - an entry point for callers that may not allocate device
// memory: cbl_batch_noalloc. It evaluates up to CBL_NOALLOC_MAX_POSITIONS
// reference positions in 192-bit mode with the same persistent term kernel
// and combine kernel as cbl_batch, but every piece of scratch those kernels
// need (tile counter, per-series digit sums, per-position shifts, the tile
// table) lives in one fixed-size array defined in this file. The caller passes
// the positions and a device output buffer it already owns.
#include "../../include/clbellard.h"
#include "cbl_internal.h"

#include <algorithm>
#include <mutex>

using namespace cbl;

namespace {

constexpr int kMaxPos = CBL_NOALLOC_MAX_POSITIONS;
constexpr int kSegsPerSeries = 4;                 // width-1/width-2 main range, width-1/width-2 tail
constexpr int kMaxSegs = kMaxPos * 7 * kSegsPerSeries;
constexpr int kTileTerms = 2048;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCounter = 0;                                          // 8 bytes
constexpr size_t kOffSlots = 256;                                          // 7 x 6 digit sums per position
constexpr size_t kOffShift = align256(kOffSlots + (size_t)kMaxPos * 7 * 6 * 8);
constexpr size_t kOffSegs = align256(kOffShift + (size_t)kMaxPos * sizeof(int));
constexpr size_t kScratchBytes = align256(kOffSegs + (size_t)kMaxSegs * sizeof(Seg));
static_assert(kScratchBytes == CBL_NOALLOC_SCRATCH_BYTES, "scratch size documented in clbellard.h");

typedef unsigned __int128 u128;

}  // namespace

// The scratch array. Every GPU that loads this library holds it until the
// process exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

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
// address (the host-side name is only a stand-in) and size the persistent grid.
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
        s.scratch = static_cast<unsigned char *>(p);
        s.grid = sms * terms192_max_ctas_per_sm(256);
        s.ready = true;
    }
    *out = &s;
    return CBL_OK;
}

// The k-ranges of one series (main [0,d) and tail [d,d+20)), split at the
// width boundary m = 2^28, written into a fixed array; m = 1 (k = 0 of a
// series with den1 = 1) contributes 0 and is left out.
int put_series(Seg *segs, int &nseg, uint64_t d, int f, uint32_t slot)
{
    const uint32_t den0 = kDen0[f], den1 = kDen1[f];
    const uint64_t kw = (kW1Max - den1 + den0 - 1) / den0;
    const uint64_t kend = d + kTail192;
    if ((u128)den0 * (kend - 1) + den1 >= (u128)kW2Max) return CBL_E_POSITION;
    const uint64_t k0 = (den1 == 1) ? 1 : 0;
    const uint64_t cut[4] = {k0, std::min(std::max(kw, k0), d), d, std::max(std::min(std::max(kw, d), kend), d)};
    // pieces: [k0, cut1) w1 main, [cut1, d) w2 main, [d, cut3) w1 tail, [cut3, kend) w2 tail
    const uint64_t lo[4] = {cut[0], cut[1], std::max(d, k0), cut[3]};
    const uint64_t hi[4] = {cut[1], d, cut[3], kend};
    for (int i = 0; i < 4; ++i) {
        const uint64_t a = std::max(lo[i], k0), b = hi[i];
        if (b <= a) continue;
        Seg s{};
        s.d = d;
        s.k0 = a;
        s.k1 = b;
        s.den0 = den0;
        s.den1 = den1;
        s.slot = slot;
        s.flags = seg_flags(kSign[f], (i == 1 || i == 3) ? 2 : 1);
        segs[nseg++] = s;
    }
    return CBL_OK;
}

}  // namespace

extern "C" int cbl_batch_noalloc(const uint64_t *pos, int n, uint64_t *d_out3n, void *stream)
{
    if (n < 0 || (n > 0 && (!pos || !d_out3n))) return CBL_E_ARG;
    if (n > kMaxPos) return CBL_E_LIMIT;
    if (n == 0) return CBL_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CBL_E_NODEVICE;
    DeviceSetup *ds = nullptr;
    int rc = setup_device(dev, &ds);
    if (rc) return rc;

    Seg segs[kMaxSegs];                 // host staging on the stack
    int nseg = 0;
    for (int i = 0; i < n; ++i) {
        uint64_t d = 0;
        rc = cbl_pos_to_d(pos[i], &d, nullptr);
        for (int f = 0; f < 7 && !rc; ++f) rc = put_series(segs, nseg, d, f, (uint32_t)(i * 7 + f));
        if (rc) return rc;
    }
    // costlier tiles first: main before tail, width 2 before width 1, larger d first
    std::sort(segs, segs + nseg, [](const Seg &a, const Seg &b) {
        const bool ta = a.k0 >= a.d, tb = b.k0 >= b.d;
        if (ta != tb) return !ta;
        const uint32_t wa = (a.flags >> 4) & 15u, wb = (b.flags >> 4) & 15u;
        if (wa != wb) return wa > wb;
        if (a.d != b.d) return a.d > b.d;
        if (a.slot != b.slot) return a.slot < b.slot;
        return a.k0 < b.k0;
    });
    uint64_t ntiles = 0;
    for (int i = 0; i < nseg; ++i) {
        segs[i].tile0 = ntiles;
        ntiles += (segs[i].k1 - segs[i].k0 + kTileTerms - 1) / kTileTerms;
    }

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = ds->scratch;
    auto *counter = reinterpret_cast<unsigned long long *>(base + kOffCounter);
    auto *slots = reinterpret_cast<unsigned long long *>(base + kOffSlots);
    auto *shift = reinterpret_cast<int *>(base + kOffShift);
    auto *dsegs = reinterpret_cast<Seg *>(base + kOffSegs);
    // the array keeps the previous call's contents: zero the counter, the digit
    // sums and the shifts, then replace the tile table
    if (cudaMemsetAsync(base, 0, kOffSegs, st) != cudaSuccess) return CBL_E_CUDA;
    if (cudaMemcpyAsync(dsegs, segs, sizeof(Seg) * nseg, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return CBL_E_CUDA;
    if (launch_terms192(dsegs, nseg, ntiles, kTileTerms, counter, slots, ds->grid, 256, st) != cudaSuccess)
        return CBL_E_CUDA;
    if (launch_combine(slots, n, shift, d_out3n, nullptr, st) != cudaSuccess) return CBL_E_CUDA;
    return CBL_OK;
}
