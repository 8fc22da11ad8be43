// cbl_host.cu - the C ABI of include/clbellard.h: context, launch
// orchestration (KernelFuncs.as), job model and work-mode files
// (Bellard_192.hsp), and the workmodeSum merge (workmodeSum0_6.hsp).
#include "../../include/clbellard.h"
#include "cbl_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include <sys/stat.h>
#include <unistd.h>
#include <sys/types.h>
#include <new>


using namespace cbl;

namespace {

constexpr uint64_t kMaxNeedD = 999999999999999999ull;   // Bellard_192.hsp:450
constexpr int kDDBlocks = 4096;                         // dd per-block partials (bigSum)
constexpr int kDefaultTile = 32 * 64;                   // terms per warp tile

typedef unsigned __int128 u128;

}  // namespace

struct cbl_ctx {
    int device = 0;
    int precision = 1;
    int sm_count = 0;
    cudaStream_t st = nullptr;
    char devname[256] = {0};
    int64_t launches = 0;
    int tile_k = kDefaultTile;
    int ctas_per_sm = 0;
    // 192-bit buffers
    Seg *d_segs = nullptr;
    Seg *h_segs = nullptr;
    int seg_cap = 0;
    unsigned long long *d_counter = nullptr;
    unsigned long long *d_slots = nullptr;   // nslot x 6 digit sums; slot 0 is bigSum
    int slot_cap = 0;
    uint64_t *d_partial = nullptr;           // 3 words, most significant first
    uint64_t *d_ans = nullptr;               // 3 words
    int *d_shift = nullptr;
    uint64_t *d_out3 = nullptr;
    uint64_t *h_out3 = nullptr;
    int pos_cap = 0;
    uint64_t *d_kbuf = nullptr;
    int kbuf_cap = 0;
    // prepared multi-position run (cbl_prepare / cbl_run_prepared)
    int prep_npos = 0;
    int prep_nseg = 0;
    uint64_t prep_ntiles = 0;
    uint64_t prep_terms = 0;
    bool prep_carry = false;                         // a prepared slot may take >= 2^31 flushes
    uint64_t slot0_tiles = 0;                        // tiles added into slot 0 since it was zeroed
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;   // around the term kernel of the last prepared run
    bool ev_valid = false;
    cudaGraphExec_t graph = nullptr;                 // captured prepared pass
    bool use_graph = true;
    int partial = 0;                                 // a budgeted run is in progress
    uint64_t seg_hash = 0;                           // identity of the prepared tile table
    std::vector<Seg> prep_segs;                      // host copy of the prepared segments
    std::vector<int> prep_shift;
    // double-double buffers
    double2 *d_bigsum = nullptr;
    double2 *d_ddpartial = nullptr;
    double2 *d_ddans = nullptr;
    // scratch host
    uint64_t *h_small = nullptr;              // pinned, 8 words
    // test hook: initial digit sums of the prepared passes' slots (null = zero)
    unsigned long long *d_preset = nullptr;
};

extern "C" {
static int upload_prepared(cbl_ctx *c);
}

#define CK(x)                                     \
    do {                                          \
        cudaError_t e_ = (x);                     \
        if (e_ != cudaSuccess) return CBL_E_CUDA; \
    } while (0)

namespace {

bool is192(const cbl_ctx *c) { return c->precision != 0; }

void drop_graph(cbl_ctx *c)
{
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
}

int ensure_segs(cbl_ctx *c, int n)
{
    if (n <= c->seg_cap) return CBL_OK;
    int cap = std::max(n, 2 * c->seg_cap);
    if (c->d_segs) cudaFree(c->d_segs);
    if (c->h_segs) cudaFreeHost(c->h_segs);
    c->d_segs = nullptr;
    c->h_segs = nullptr;
    c->seg_cap = 0;
    if (cudaMalloc(&c->d_segs, sizeof(Seg) * cap) != cudaSuccess) return CBL_E_NOMEM;
    if (cudaMallocHost(&c->h_segs, sizeof(Seg) * cap) != cudaSuccess) return CBL_E_NOMEM;
    c->seg_cap = cap;
    return CBL_OK;
}

int ensure_slots(cbl_ctx *c, int nslot)
{
    if (nslot <= c->slot_cap) return CBL_OK;
    int cap = std::max(nslot, 2 * c->slot_cap);
    unsigned long long *p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned long long) * 6 * cap) != cudaSuccess) return CBL_E_NOMEM;
    if (c->d_slots) {
        cudaMemcpyAsync(p, c->d_slots, sizeof(unsigned long long) * 6 * c->slot_cap, cudaMemcpyDeviceToDevice, c->st);
        cudaStreamSynchronize(c->st);
        cudaFree(c->d_slots);
    }
    c->d_slots = p;
    c->slot_cap = cap;
    return CBL_OK;
}

int ensure_pos(cbl_ctx *c, int n)
{
    if (n <= c->pos_cap) return CBL_OK;
    int cap = std::max(n, 2 * c->pos_cap);
    if (c->d_shift) cudaFree(c->d_shift);
    if (c->d_out3) cudaFree(c->d_out3);
    if (c->h_out3) cudaFreeHost(c->h_out3);
    c->d_shift = nullptr;
    c->d_out3 = nullptr;
    c->h_out3 = nullptr;
    c->pos_cap = 0;
    if (cudaMalloc(&c->d_shift, sizeof(int) * cap) != cudaSuccess) return CBL_E_NOMEM;
    if (cudaMalloc(&c->d_out3, sizeof(uint64_t) * 3 * cap) != cudaSuccess) return CBL_E_NOMEM;
    if (cudaMallocHost(&c->h_out3, sizeof(uint64_t) * 3 * cap) != cudaSuccess) return CBL_E_NOMEM;
    c->pos_cap = cap;
    return CBL_OK;
}

bool formula_ok(int f) { return f >= 0 && f < 7; }

// Moduli den0*k+den1 must be odd: den0 even, den1 odd (true for the 7 series).
bool series_ok(uint64_t den0, uint64_t den1)
{
    return den0 >= 2 && den0 < (1ull << 31) && (den0 & 1) == 0 && (den1 & 1) == 1 && den1 < (1ull << 31);
}

// Append the segments covering k in [k0, k1) of one series, split at d (main
// vs tail) and at the residue-kind boundaries m = 2^28, 2^31, 2^32, 2^44 and 2^60. k = 0 with
// den1 = 1 (m = 1) contributes exactly 0 and is left out.
int add_segments(std::vector<Seg> &v, uint64_t d, uint32_t den0, uint32_t den1, int sign, uint32_t slot,
                 uint64_t k0, uint64_t k1)
{
    if (k0 == 0 && den1 == 1) k0 = 1;
    if (k1 <= k0) return CBL_OK;
    if ((u128)den0 * (k1 - 1) + den1 >= (u128)kW2XMax) return CBL_E_POSITION;
    const uint64_t kw1 = (kW1Max - den1 + den0 - 1) / den0;    // first k with m >= 2^28
    const uint64_t kw1m = (kW1MMax - den1 + den0 - 1) / den0;  // first k with m >= 2^31
    const uint64_t kw1s = (kW1SMax - den1 + den0 - 1) / den0;  // first k with m >= 2^32
    const uint64_t kw2s = (kW2SMax - den1 + den0 - 1) / den0;  // first k with m >= 2^44
    const uint64_t kw2 = (kW2Max - den1 + den0 - 1) / den0;    // first k with m >= 2^60
    std::vector<uint64_t> pts = {k0, k1};
    for (uint64_t c : {d, kw1, kw1m, kw1s, kw2s, kw2}) pts.push_back(std::min(std::max(c, k0), k1));
    std::sort(pts.begin(), pts.end());
    for (size_t i = 0; i + 1 < pts.size(); ++i) {
        const uint64_t a = pts[i], b = pts[i + 1];
        if (b <= a) continue;
        Seg s{};
        s.d = d;
        s.k0 = a;
        s.k1 = b;
        s.den0 = den0;
        s.den1 = den1;
        s.slot = slot;
        s.flags = seg_flags(sign, a >= kw2 ? 6 : a >= kw2s ? 2 : (a >= kw1s ? 4 : (a >= kw1m ? 3 : (a >= kw1 ? 5 : 1))));
        v.push_back(s);
    }
    return CBL_OK;
}

// Cost rank of a residue kind: wide width 2 > width 2 > short width 2 >
// strict width 1 > middle width 1 > width 1.
int kind_rank(uint32_t flags)
{
    switch ((flags >> 4) & 15u) {
    case 6: return 5;
    case 2: return 4;
    case 4: return 3;
    case 3: return 2;
    case 5: return 1;
    default: return 0;
    }
}

// Costlier tiles first (width 2, then large d), tails last; then tile prefixes.
uint64_t order_and_number(std::vector<Seg> &v, uint32_t tile_k)
{
    std::stable_sort(v.begin(), v.end(), [](const Seg &a, const Seg &b) {
        const bool ta = a.k0 >= a.d, tb = b.k0 >= b.d;
        if (ta != tb) return !ta;
        const int ra = kind_rank(a.flags), rb = kind_rank(b.flags);
        if (ra != rb) return ra > rb;
        return a.d > b.d;
    });
    uint64_t t = 0;
    for (Seg &s : v) {
        s.tile0 = t;
        t += (s.k1 - s.k0 + tile_k - 1) / tile_k;
    }
    return t;
}

int grid_192(cbl_ctx *c)
{
    int per = c->ctas_per_sm > 0 ? c->ctas_per_sm : terms192_max_ctas_per_sm(256);
    return std::max(1, c->sm_count * per);
}

// Upload segments and run the persistent term kernel (accumulates into slots).
int run_segments(cbl_ctx *c, std::vector<Seg> &v)
{
    if (v.empty()) return CBL_OK;
    const uint64_t ntiles = order_and_number(v, (uint32_t)c->tile_k);
    int rc = ensure_segs(c, (int)v.size());
    if (rc) return rc;
    // the pinned staging buffer may still feed an earlier async copy
    CK(cudaStreamSynchronize(c->st));
    std::memcpy(c->h_segs, v.data(), sizeof(Seg) * v.size());
    CK(cudaMemcpyAsync(c->d_segs, c->h_segs, sizeof(Seg) * v.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), c->st));
    // slot 0 collects every launch since cbl_Set0mem: carry once it may have
    // taken 2^31 flushes (at most one per tile)
    c->slot0_tiles = std::min<uint64_t>(c->slot0_tiles + ntiles, kCarryTiles);
    CK(launch_terms192(c->d_segs, (int)v.size(), ntiles, (uint32_t)c->tile_k, c->d_counter, c->d_slots,
                       grid_192(c), 256, c->st, 0, slot_needs_carry(c->slot0_tiles)));
    c->launches++;
    return CBL_OK;
}

int dd_range(cbl_ctx *c, uint64_t k0, uint64_t k1, uint64_t d, int sign, uint32_t den0, uint32_t den1)
{
    if (k1 > k0 && (u128)den0 * (k1 - 1) + den1 >= (u128)kW2XMax) return CBL_E_POSITION;
    // chunks of 2^30 terms keep each launch to a bounded time
    const uint64_t chunk = 1ull << 30;
    for (uint64_t a = k0; a < k1; a += chunk) {
        const uint64_t b = std::min(k1, a + chunk);
        CK(launch_dd_terms(c->d_bigsum, kDDBlocks, 256, a, b, d, sign, den0, den1, c->st));
        c->launches++;
    }
    return CBL_OK;
}

int sync(cbl_ctx *c)
{
    CK(cudaStreamSynchronize(c->st));
    return CBL_OK;
}

void to_hex192(const uint64_t w[3], char out[49])
{
    static const char hx[] = "0123456789abcdef";
    int p = 0;
    for (int i = 0; i < 3; ++i)
        for (int b = 60; b >= 0; b -= 4) out[p++] = hx[(w[i] >> b) & 15];
    out[48] = 0;
}

// floor(|x| * 2^128) for a double |x| < 1.
u128 fixed128_abs(double x)
{
    if (x == 0.0) return 0;
    int e;
    const double m = std::frexp(std::fabs(x), &e);                  // |x| = m 2^e, m in [0.5,1)
    const uint64_t mi = (uint64_t)std::ldexp(m, 53);                 // exact 53-bit integer
    const int sh = e - 53 + 128;                                     // |x| 2^128 = mi 2^sh
    if (sh >= 0) return (u128)mi << sh;
    return (sh > -64) ? (u128)(mi >> (-sh)) : 0;
}

// Mode-0 hex: the double-double value mod 1 to 28 hex digits (14 bytes, as
// hexadecimal_dd, hexsademical.as:21-101) and 20 trailing zeros. A negative
// value is first lifted by 1.0 with the reference's own double-double add
// (hexsademical.as:3-19, 25-31: two-sum, the low words added in order, two-sum),
// whose rounding of the low word the printed bytes keep; then the sum is formed
// mod 2^128, exactly, and truncated. The reference's byte loop is exact except
// for its borrow branch (hexsademical.as:73-97), which leaves every later byte
// 00; this truncation prints those bytes' true values.
void dd_to_hex(double hi, double lo, char out[49])
{
    if (hi < 0.0) {
        const double x = hi + 1.0, t = x - hi;
        double y = (hi - (x - t)) + (1.0 - t);
        y = y + lo + 0.0;
        const double x2 = x + y, t2 = x2 - x;
        lo = (x - (x2 - t2)) + (y - t2);
        hi = x2;
    }
    u128 u = hi < 0 ? (u128)0 - fixed128_abs(hi) : fixed128_abs(hi);
    u += lo < 0 ? (u128)0 - fixed128_abs(lo) : fixed128_abs(lo);
    const uint64_t top = (uint64_t)(u >> 64), low = (uint64_t)u;
    const uint64_t w[3] = {top, low & ~0xffffull, 0};                // keep 112 bits
    to_hex192(w, out);
}

int hexval(int c)
{
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}

int mkdir_p(const std::string &path)
{
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur.push_back(path[i]);
        if (path[i] == '/' || i + 1 == path.size()) {
            if (cur == "/") continue;
            if (mkdir(cur.c_str(), 0777) != 0) {
                struct stat st;
                if (stat(cur.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) return -1;
            }
        }
    }
    return 0;
}

std::string job_path(const char *workdir, int s, uint64_t b)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "/%d/%d_%llu.txt", s, s, (unsigned long long)b);
    return std::string(workdir) + buf;
}

}  // namespace

extern "C" {

const char *cbl_strerror(int code)
{
    switch (code) {
    case CBL_OK: return "ok";
    case CBL_SKIPPED: return "job skipped: k_start > d";
    case CBL_E_ARG: return "invalid argument";
    case CBL_E_POSITION:
        return "invalid position (outside [5, 999999999999999999])";
    case CBL_E_NODEVICE: return "no CUDA device";
    case CBL_E_CUDA: return "CUDA runtime error";
    case CBL_E_TIMEOUT: return "timed out waiting for the device";
    case CBL_E_RANGE: return "k-range outside this entry point's modulus range";
    case CBL_E_NOMEM: return "out of memory";
    case CBL_E_PRECISION: return "call not valid for this precision";
    case CBL_E_IO: return "file I/O error";
    case CBL_E_FORMAT: return "malformed input";
    case CBL_E_LIMIT: return "request exceeds a fixed limit (at most CBL_NOALLOC_MAX_POSITIONS positions)";
    default: return "unknown error";
    }
}

int cbl_hex_dd(double hi, double lo, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!hex || !std::isfinite(hi) || !std::isfinite(lo) || std::fabs(hi) >= 1.0 || std::fabs(lo) >= 1.0)
        return CBL_E_ARG;
    dd_to_hex(hi, lo, hex);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_formula(int f, uint64_t *numer, int64_t *numesign, uint64_t *den0, uint64_t *den1)
{
    CBL_GUARD_BEGIN
    if (!formula_ok(f)) return CBL_E_ARG;
    if (numer) *numer = (uint64_t)kNumer[f];
    if (numesign) *numesign = kSign[f];
    if (den0) *den0 = kDen0[f];
    if (den1) *den1 = kDen1[f];
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_pos_to_d(uint64_t needD, uint64_t *d, uint64_t *needD_adj)
{
    CBL_GUARD_BEGIN
    if (needD <= 4 || needD > kMaxNeedD) return CBL_E_POSITION;
    uint64_t dd = ((needD - 1) * 2 - 3) / 5;
    if (dd % 2 == 0) dd--;
    if (d) *d = dd;
    if (needD_adj) *needD_adj = (dd * 5 + 3) / 2 + 1;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_create(int device, int precision, cbl_ctx **out)
{
    CBL_GUARD_BEGIN
    if (!out || precision < 0 || precision > 2) return CBL_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CBL_E_NODEVICE;
    if (device < 0 || device >= n) return CBL_E_NODEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return CBL_E_CUDA;
    cbl_ctx *c = new cbl_ctx();
    c->device = device;
    c->precision = precision;
    c->sm_count = device_sm_count(device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess)
        std::snprintf(c->devname, sizeof c->devname, "%s", prop.name);
    int rc = CBL_OK;
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) rc = CBL_E_CUDA;
    if (!rc && cudaMalloc(&c->d_counter, sizeof(unsigned long long)) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMalloc(&c->d_partial, sizeof(uint64_t) * 3) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMalloc(&c->d_ans, sizeof(uint64_t) * 3) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMalloc(&c->d_bigsum, sizeof(double2) * kDDBlocks) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMalloc(&c->d_ddpartial, sizeof(double2)) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMalloc(&c->d_ddans, sizeof(double2)) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaMallocHost(&c->h_small, sizeof(uint64_t) * 8) != cudaSuccess) rc = CBL_E_NOMEM;
    if (!rc && cudaEventCreate(&c->ev_k0) != cudaSuccess) rc = CBL_E_CUDA;
    if (!rc && cudaEventCreate(&c->ev_k1) != cudaSuccess) rc = CBL_E_CUDA;
    if (!rc) rc = ensure_slots(c, 8);
    if (!rc) rc = ensure_segs(c, 64);
    if (!rc) rc = ensure_pos(c, 1);
    if (!rc) {
        cudaMemsetAsync(c->d_slots, 0, sizeof(unsigned long long) * 6 * c->slot_cap, c->st);
        cudaMemsetAsync(c->d_partial, 0, sizeof(uint64_t) * 3, c->st);
        cudaMemsetAsync(c->d_ans, 0, sizeof(uint64_t) * 3, c->st);
        cudaMemsetAsync(c->d_bigsum, 0, sizeof(double2) * kDDBlocks, c->st);
        cudaMemsetAsync(c->d_ddpartial, 0, sizeof(double2), c->st);
        cudaMemsetAsync(c->d_ddans, 0, sizeof(double2), c->st);
        if (cudaStreamSynchronize(c->st) != cudaSuccess) rc = CBL_E_CUDA;
    }
    if (rc) {
        cbl_destroy(c);
        return rc;
    }
    *out = c;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_destroy(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    cudaFree(c->d_segs);
    cudaFreeHost(c->h_segs);
    cudaFree(c->d_counter);
    cudaFree(c->d_slots);
    cudaFree(c->d_partial);
    cudaFree(c->d_ans);
    cudaFree(c->d_shift);
    cudaFree(c->d_out3);
    cudaFreeHost(c->h_out3);
    cudaFree(c->d_kbuf);
    cudaFree(c->d_bigsum);
    cudaFree(c->d_ddpartial);
    cudaFree(c->d_ddans);
    cudaFreeHost(c->h_small);
    cudaFree(c->d_preset);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->ev_k0) cudaEventDestroy(c->ev_k0);
    if (c->ev_k1) cudaEventDestroy(c->ev_k1);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_precision(const cbl_ctx *c) { return c ? c->precision : CBL_E_ARG; }
void *cbl_stream(cbl_ctx *c) { return c ? (void *)c->st : nullptr; }
int64_t cbl_launch_count(const cbl_ctx *c) { return c ? c->launches : CBL_E_ARG; }

int cbl_device_name(const cbl_ctx *c, char *buf, int len)
{
    CBL_GUARD_BEGIN
    if (!c || !buf || len <= 0) return CBL_E_ARG;
    std::snprintf(buf, (size_t)len, "%s", c->devname);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_set_tuning(cbl_ctx *c, int tile_terms, int ctas_per_sm)
{
    CBL_GUARD_BEGIN
    if (!c || tile_terms < 32 || tile_terms % 32 != 0 || ctas_per_sm < 0) return CBL_E_ARG;
    if (c->partial) return CBL_E_ARG;                 // a budgeted run depends on the tile numbering
    const bool renumber = tile_terms != c->tile_k && c->prep_npos > 0;
    c->tile_k = tile_terms;
    c->ctas_per_sm = ctas_per_sm;
    drop_graph(c);
    if (renumber) {
        cudaSetDevice(c->device);
        return upload_prepared(c);
    }
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_set_slot_preset(cbl_ctx *c, const uint64_t preset[6])
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->st));
    if (!preset) {
        cudaFree(c->d_preset);
        c->d_preset = nullptr;
    } else {
        if (!c->d_preset && cudaMalloc(&c->d_preset, sizeof(unsigned long long) * 6) != cudaSuccess) {
            c->d_preset = nullptr;
            return CBL_E_NOMEM;
        }
        CK(cudaMemcpy(c->d_preset, preset, sizeof(unsigned long long) * 6, cudaMemcpyHostToDevice));
    }
    drop_graph(c);                                        // the captured pass clears the slots
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_set_graph(cbl_ctx *c, int enable)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    c->use_graph = enable != 0;
    drop_graph(c);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_Set0mem(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) {
        CK(cudaMemsetAsync(c->d_slots, 0, sizeof(unsigned long long) * 6, c->st));
        c->slot0_tiles = 0;
    } else {
        CK(cudaMemsetAsync(c->d_bigsum, 0, sizeof(double2) * kDDBlocks, c->st));
    }
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_Set0ans(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) CK(cudaMemsetAsync(c->d_ans, 0, sizeof(uint64_t) * 3, c->st));
    else CK(cudaMemsetAsync(c->d_ddans, 0, sizeof(double2), c->st));
    return CBL_OK;
    CBL_GUARD_END
}

static int sglobal(cbl_ctx *c, uint64_t offset, uint64_t d, uint64_t k_max, int64_t numesign, uint64_t den0,
                   uint64_t den1, uint64_t mlimit)
{
    if (!c || !series_ok(den0, den1) || (numesign != 0 && numesign != 1)) return CBL_E_ARG;
    if (k_max <= offset) return CBL_OK;
    if (k_max > d) return CBL_E_RANGE;
    if ((u128)den0 * (k_max - 1) + den1 >= (u128)mlimit) return CBL_E_RANGE;
    cudaSetDevice(c->device);
    if (is192(c)) {
        std::vector<Seg> v;
        int rc = add_segments(v, d, (uint32_t)den0, (uint32_t)den1, (int)numesign, 0, offset, k_max);
        if (rc) return rc == CBL_E_POSITION ? CBL_E_RANGE : rc;
        return run_segments(c, v);
    }
    return dd_range(c, offset, k_max, d, (int)numesign, (uint32_t)den0, (uint32_t)den1);
}

int cbl_Sglobal32mtg(cbl_ctx *c, uint64_t offset, uint64_t d, uint64_t k_max, int64_t numesign, uint64_t den0,
                     uint64_t den1)
{
    CBL_GUARD_BEGIN
    return sglobal(c, offset, d, k_max, numesign, den0, den1, 1ull << 32);
    CBL_GUARD_END
}

int cbl_Sglobal64mtg(cbl_ctx *c, uint64_t offset, uint64_t d, uint64_t k_max, int64_t numesign, uint64_t den0,
                     uint64_t den1)
{
    CBL_GUARD_BEGIN
    return sglobal(c, offset, d, k_max, numesign, den0, den1, kW2XMax);
    CBL_GUARD_END
}

int cbl_Sglobal_after(cbl_ctx *c, uint64_t d, int64_t numesign, uint64_t den0, uint64_t den1)
{
    CBL_GUARD_BEGIN
    if (!c || !series_ok(den0, den1) || (numesign != 0 && numesign != 1)) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) {
        std::vector<Seg> v;
        int rc = add_segments(v, d, (uint32_t)den0, (uint32_t)den1, (int)numesign, 0, d, d + kTail192);
        if (rc) return rc;
        return run_segments(c, v);
    }
    CK(launch_dd_tail(c->d_bigsum, d, (int)numesign, (uint32_t)den0, (uint32_t)den1, c->st));
    c->launches++;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_Ssum(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) CK(launch_ssum192(c->d_slots, c->d_partial, c->st));
    else CK(launch_dd_ssum(c->d_bigsum, kDDBlocks, c->d_ddpartial, c->st));
    c->launches++;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_Sum7(cbl_ctx *c, uint64_t numer)
{
    CBL_GUARD_BEGIN
    if (!c || numer == 0 || (numer & (numer - 1)) != 0 || numer > 256) return CBL_E_ARG;
    cudaSetDevice(c->device);
    int sh = 0;
    while ((1ull << sh) != numer) ++sh;
    if (is192(c)) CK(launch_sum7_192(c->d_partial, c->d_ans, sh, c->st));
    else CK(launch_dd_sum7(c->d_ddpartial, c->d_ddans, (int)numer, c->st));
    c->launches++;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_BatchCalc(cbl_ctx *c, uint64_t k_start, uint64_t k_end, int f, uint64_t d)
{
    CBL_GUARD_BEGIN
    if (!c || !formula_ok(f)) return CBL_E_ARG;
    cudaSetDevice(c->device);
    const uint64_t kend = std::min(k_end, d);
    // the reference's offset after its two loops is max(k_start, min(k_end, d));
    // the tail runs when that equals d (KernelFuncs.as:27-59)
    const uint64_t offset = std::max(k_start, kend);
    const bool tail = offset == d;
    if (is192(c)) {
        std::vector<Seg> v;
        int rc = CBL_OK;
        if (k_start < kend) rc = add_segments(v, d, kDen0[f], kDen1[f], kSign[f], 0, k_start, kend);
        if (!rc && tail) rc = add_segments(v, d, kDen0[f], kDen1[f], kSign[f], 0, d, d + kTail192);
        if (rc) return rc;
        rc = run_segments(c, v);
        if (rc) return rc;
    } else {
        if (k_start < kend) {
            int rc = dd_range(c, k_start, kend, d, kSign[f], kDen0[f], kDen1[f]);
            if (rc) return rc;
        }
        if (tail) {
            if ((u128)kDen0[f] * (d + kTailDD) + kDen1[f] >= (u128)kW2XMax) return CBL_E_POSITION;
            CK(launch_dd_tail(c->d_bigsum, d, kSign[f], kDen0[f], kDen1[f], c->st));
            c->launches++;
        }
    }
    return cbl_Ssum(c);
    CBL_GUARD_END
}

int cbl_AddAns(cbl_ctx *c, int f)
{
    CBL_GUARD_BEGIN
    if (!formula_ok(f)) return CBL_E_ARG;
    return cbl_Sum7(c, (uint64_t)kNumer[f]);
    CBL_GUARD_END
}

int cbl_read_partial(cbl_ctx *c, void *out)
{
    CBL_GUARD_BEGIN
    if (!c || !out) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) CK(cudaMemcpyAsync(c->h_small, c->d_partial, 24, cudaMemcpyDeviceToHost, c->st));
    else CK(cudaMemcpyAsync(c->h_small, c->d_ddpartial, 16, cudaMemcpyDeviceToHost, c->st));
    int rc = sync(c);
    if (rc) return rc;
    std::memcpy(out, c->h_small, is192(c) ? 24 : 16);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_read_ans(cbl_ctx *c, void *out)
{
    CBL_GUARD_BEGIN
    if (!c || !out) return CBL_E_ARG;
    cudaSetDevice(c->device);
    if (is192(c)) CK(cudaMemcpyAsync(c->h_small, c->d_ans, 24, cudaMemcpyDeviceToHost, c->st));
    else CK(cudaMemcpyAsync(c->h_small, c->d_ddans, 16, cudaMemcpyDeviceToHost, c->st));
    int rc = sync(c);
    if (rc) return rc;
    std::memcpy(out, c->h_small, is192(c) ? 24 : 16);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_query(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    const cudaError_t e = cudaStreamQuery(c->st);
    if (e == cudaSuccess) return 0;
    if (e == cudaErrorNotReady) {
        cudaGetLastError();
        return 1;
    }
    return CBL_E_CUDA;
    CBL_GUARD_END
}

int cbl_wait(cbl_ctx *c, int timeout_ms)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const int q = cbl_query(c);
        if (q <= 0) return q;
        if (timeout_ms >= 0) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0);
            if (ms.count() >= timeout_ms) return CBL_E_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    CBL_GUARD_END
}

static uint64_t fnv1a(const void *p, size_t n, uint64_t h = 1469598103934665603ull)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

// Number the prepared segments' tiles for the current tile size and upload
// them with the per-position shifts (again after a tile-size change).
static int upload_prepared(cbl_ctx *c)
{
    std::vector<Seg> &v = c->prep_segs;
    const int n = c->prep_npos;
    const uint64_t ntiles = order_and_number(v, (uint32_t)c->tile_k);
    std::vector<uint64_t> slot_tiles((size_t)7 * n, 0);
    uint64_t max_slot_tiles = 0;
    for (const Seg &sg : v) {
        uint64_t &t = slot_tiles[sg.slot];
        t += (sg.k1 - sg.k0 + c->tile_k - 1) / c->tile_k;
        max_slot_tiles = std::max(max_slot_tiles, t);
    }
    c->prep_carry = slot_needs_carry(max_slot_tiles);
    int rc = ensure_segs(c, (int)v.size());
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->st));
    std::memcpy(c->h_segs, v.data(), sizeof(Seg) * v.size());
    CK(cudaMemcpyAsync(c->d_segs, c->h_segs, sizeof(Seg) * v.size(), cudaMemcpyHostToDevice, c->st));
    std::memcpy(c->h_out3, c->prep_shift.data(), sizeof(int) * n);      // pinned staging for the shifts
    CK(cudaMemcpyAsync(c->d_shift, c->h_out3, sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    drop_graph(c);
    c->prep_nseg = (int)v.size();
    c->prep_ntiles = ntiles;
    c->partial = 0;
    c->seg_hash = fnv1a(c->prep_shift.data(), sizeof(int) * n, fnv1a(v.data(), sizeof(Seg) * v.size()));
    return CBL_OK;
}

// Build and upload the segments of all 7 series of n positions (d[i],
// shift[i]); slots i*7+f. Nothing is launched.
static int prepare_positions(cbl_ctx *c, const uint64_t *d, const int *shift, int n)
{
    int rc = ensure_slots(c, 7 * n);
    if (!rc) rc = ensure_pos(c, n);
    if (rc) return rc;
    std::vector<Seg> v;
    v.reserve((size_t)n * 7 * 4);
    uint64_t terms = 0;
    for (int i = 0; i < n && !rc; ++i) {
        terms += 7 * d[i];
        for (int f = 0; f < 7 && !rc; ++f)
            rc = add_segments(v, d[i], kDen0[f], kDen1[f], kSign[f], (uint32_t)(i * 7 + f), 0, d[i] + kTail192);
    }
    if (rc) return rc;
    c->prep_segs.swap(v);
    c->prep_shift.assign(shift, shift + n);
    c->prep_npos = n;
    c->prep_terms = terms;
    return upload_prepared(c);
}

// A prepared pass carries digit-sum wraps when a slot may take 2^31 or more
// flushes or starts from a preset.
static bool prepared_carry(const cbl_ctx *c) { return c->prep_carry || c->d_preset != nullptr; }

// Zero the first nslot slots, or set them to the test preset. Slot 0 is then
// no longer a known count of flushes from zero for the kernel-by-kernel calls
// (until cbl_Set0mem).
static cudaError_t clear_slots(cbl_ctx *c, int nslot)
{
    c->slot0_tiles = kCarryTiles;
    if (c->d_preset) return launch_slot_fill(c->d_slots, nslot, c->d_preset, c->st);
    return cudaMemsetAsync(c->d_slots, 0, sizeof(unsigned long long) * 6 * nslot, c->st);
}

// Enqueue the prepared pass: zero slots and tile counter, the persistent term
// kernel between two events, the combine kernel. The first pass after a
// prepare is captured into a CUDA graph and every later pass replays it.
static int enqueue_prepared(cbl_ctx *c, bool capturing)
{
    // inside a capture the events must be external records so that the graph
    // records them when it is replayed; outside a capture that flag is refused
    const unsigned int evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    const int n = c->prep_npos;
    CK(clear_slots(c, 7 * n));
    CK(cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), c->st));
    CK(cudaEventRecordWithFlags(c->ev_k0, c->st, evf));
    CK(launch_terms192(c->d_segs, c->prep_nseg, c->prep_ntiles, (uint32_t)c->tile_k, c->d_counter, c->d_slots,
                       grid_192(c), 256, c->st, 0, prepared_carry(c)));
    CK(cudaEventRecordWithFlags(c->ev_k1, c->st, evf));
    CK(launch_combine(c->d_slots, n, c->d_shift, c->d_out3, nullptr, c->st));
    return CBL_OK;
}

static int launch_prepared(cbl_ctx *c)
{
    if (c->prep_npos <= 0) return CBL_E_ARG;
    c->partial = 0;
    if (c->use_graph) {
        if (!c->graph) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue_prepared(c, true);
            const cudaError_t e = cudaStreamEndCapture(c->st, &g);
            if (rc || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return rc ? rc : CBL_E_CUDA;
            }
            const cudaError_t ei = cudaGraphInstantiate(&c->graph, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                c->graph = nullptr;
                return CBL_E_CUDA;
            }
        }
        CK(cudaGraphLaunch(c->graph, c->st));
    } else {
        const int rc = enqueue_prepared(c, false);
        if (rc) return rc;
    }
    c->ev_valid = true;
    c->launches += 2;
    return CBL_OK;
}

static int run_positions(cbl_ctx *c, const uint64_t *d, const int *shift, int n)
{
    int rc = prepare_positions(c, d, shift, n);
    return rc ? rc : launch_prepared(c);
}

static int compute_d(cbl_ctx *c, uint64_t d, int shift, char hex[49])
{
    if (is192(c)) {
        int rc = run_positions(c, &d, &shift, 1);
        if (rc) return rc;
        CK(cudaMemcpyAsync(c->d_ans, c->d_out3, 24, cudaMemcpyDeviceToDevice, c->st));
        CK(cudaMemcpyAsync(c->h_out3, c->d_out3, 24, cudaMemcpyDeviceToHost, c->st));
        rc = sync(c);
        if (rc) return rc;
        to_hex192(c->h_out3, hex);
        return CBL_OK;
    }
    if (shift != 0) return CBL_E_PRECISION;
    int rc = cbl_Set0ans(c);
    for (int f = 0; f < 7 && !rc; ++f) {
        rc = cbl_Set0mem(c);
        if (!rc) rc = cbl_BatchCalc(c, 0, d, f, d);
        if (!rc) rc = cbl_AddAns(c, f);
    }
    if (rc) return rc;
    double a[2];
    rc = cbl_read_ans(c, a);
    if (rc) return rc;
    dd_to_hex(a[0], a[1], hex);
    return CBL_OK;
}

int cbl_compute(cbl_ctx *c, uint64_t needD, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!c || !hex) return CBL_E_ARG;
    uint64_t d;
    int rc = cbl_pos_to_d(needD, &d, nullptr);
    if (rc) return rc;
    cudaSetDevice(c->device);
    return compute_d(c, d, 0, hex);
    CBL_GUARD_END
}

int cbl_compute_hexpos(cbl_ctx *c, uint64_t p, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!c || !hex) return CBL_E_ARG;
    if (p < 3 || p > kMaxNeedD) return CBL_E_POSITION;
    const uint64_t B = 4 * (p - 1);
    const uint64_t d = (B - 6) / 10;
    const int shift = (int)((B - 6) - 10 * d);
    cudaSetDevice(c->device);
    return compute_d(c, d, shift, hex);
    CBL_GUARD_END
}

int cbl_run_job(cbl_ctx *c, uint64_t needD, int s, uint64_t b, uint64_t batchsize, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!c || !hex || !formula_ok(s) || batchsize == 0) return CBL_E_ARG;
    uint64_t d;
    int rc = cbl_pos_to_d(needD, &d, nullptr);
    if (rc) return rc;
    if ((u128)batchsize * (b + 1) > (u128)UINT64_MAX) return CBL_E_ARG;
    const uint64_t k_start = batchsize * b, k_end = batchsize * (b + 1);
    if (k_start > d) return CBL_SKIPPED;                       // Bellard_192.hsp:306
    cudaSetDevice(c->device);
    rc = cbl_Set0mem(c);
    if (!rc) rc = cbl_BatchCalc(c, k_start, k_end, s, d);
    if (!rc) rc = cbl_AddAns(c, s);
    if (rc) return rc;
    if (is192(c)) {
        uint64_t w[3];
        rc = cbl_read_partial(c, w);
        if (!rc) to_hex192(w, hex);
    } else {
        double a[2];
        rc = cbl_read_partial(c, a);
        if (!rc) dd_to_hex(a[0], a[1], hex);
    }
    return rc;
    CBL_GUARD_END
}

// ---- balanced work-mode planning
// Relative cost of one ladder step per residue kind, from each kind's measured
// term time on its own k-range (GB300; 0.6e8-4.6e8 terms per range, divided by
// bitlen(10(d-k)) + 8 and scaled to W1 = 7): W1 7, W1M 5.9, W1S 8.2, W2S 14.5,
// W2 16.8, W2X 24.3.
static double step_cost(uint64_t m)
{
    if (m < kW1Max) return 7.0;
    if (m < kW1MMax) return 5.9;
    if (m < kW1SMax) return 8.2;
    if (m < kW2SMax) return 14.5;
    if (m < kW2Max) return 16.8;
    return 24.3;
}

// Estimated cost of terms k in [k0, k1) of series f at position d (k < d):
// (bitlen(10(d - k)) + 8) steps per term (the 8 stands for the start value and
// the six digit steps) times the kind's step cost; piecewise constant between
// the powers of two of 10(d - k) and the kind boundaries.
static double range_cost(uint64_t d, int f, uint64_t k0, uint64_t k1)
{
    const uint64_t den0 = kDen0[f], den1 = kDen1[f];
    double total = 0.0;
    uint64_t k = k0;
    while (k < k1) {
        const uint64_t e10 = 10 * (d - k);
        const int bl = 64 - __builtin_clzll(e10);
        // next k where bitlen(10(d-k)) drops: 10(d-k) < 2^(bl-1)  <=>  k > d - 2^(bl-1)/10
        const uint64_t lim = (uint64_t)1 << (bl - 1);
        uint64_t knext = d - (lim - 1) / 10;                 // first k with 10(d-k) < 2^(bl-1)
        if (knext <= k) knext = k + 1;
        const uint64_t m = den0 * k + den1;
        const uint64_t bounds[5] = {kW1Max, kW1MMax, kW1SMax, kW2SMax, kW2Max};
        for (uint64_t b : bounds)
            if (m < b) {
                const uint64_t kb = (b - den1 + den0 - 1) / den0;
                if (kb < knext) knext = kb;
                break;
            }
        if (knext > k1) knext = k1;
        if (knext <= k) knext = k + 1;
        total += (double)(knext - k) * (bl + 8) * step_cost(m);
        k = knext;
    }
    return total;
}

int cbl_plan_jobs(uint64_t needD, int njobs, int *out_s, uint64_t *out_k0, uint64_t *out_k1, int cap)
{
    CBL_GUARD_BEGIN
    if (njobs < 7 || cap < njobs || !out_s || !out_k0 || !out_k1) return CBL_E_ARG;
    uint64_t d;
    int rc = cbl_pos_to_d(needD, &d, nullptr);
    if (rc) return rc;
    double cost[7], total = 0;
    for (int f = 0; f < 7; ++f) total += cost[f] = range_cost(d, f, 0, d) + 1.0;
    // jobs per series: one each, then each further job to the series whose cost
    // per job is largest (this minimises the largest job for a fixed count)
    // (at most d jobs per series: each job keeps at least one term below d)
    const int maxper = (int)std::min<uint64_t>(d, (uint64_t)njobs);
    int per[7], used = 7;
    for (int f = 0; f < 7; ++f) per[f] = 1;
    while (used < njobs) {
        int best = -1;
        for (int f = 0; f < 7; ++f)
            if (per[f] < maxper && (best < 0 || cost[f] / per[f] > cost[best] / per[best])) best = f;
        if (best < 0) break;
        ++per[best];
        ++used;
    }
    int n = 0;
    for (int f = 0; f < 7; ++f) {
        uint64_t k = 0;
        for (int j = 0; j < per[f]; ++j) {
            uint64_t kend = d;
            if (j + 1 < per[f]) {                           // cost target by bisection on k
                const double target = cost[f] * (j + 1) / per[f];
                uint64_t lo = k, hi = d;
                while (lo + 1 < hi) {
                    const uint64_t mid = lo + (hi - lo) / 2;
                    if (range_cost(d, f, 0, mid) < target) lo = mid; else hi = mid;
                }
                // a job that reaches d also runs the tail (cbl_BatchCalc), so all
                // but the last job of a series end below d, each with >= 1 term
                kend = std::min(std::max(hi, k + 1), d - (uint64_t)(per[f] - 1 - j));
            }
            out_s[n] = f;
            out_k0[n] = k;
            out_k1[n] = j + 1 < per[f] ? kend : d + kTail192;   // the last job of a series takes the tail
            ++n;
            k = kend;
        }
    }
    return n;
    CBL_GUARD_END
}

int cbl_run_job_range(cbl_ctx *c, uint64_t needD, int s, uint64_t k0, uint64_t k1, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!c || !hex || !formula_ok(s) || k1 < k0) return CBL_E_ARG;
    uint64_t d;
    int rc = cbl_pos_to_d(needD, &d, nullptr);
    if (rc) return rc;
    if (k0 > d) return CBL_SKIPPED;
    cudaSetDevice(c->device);
    rc = cbl_Set0mem(c);
    if (!rc) rc = cbl_BatchCalc(c, k0, k1, s, d);
    if (!rc) rc = cbl_AddAns(c, s);
    if (rc) return rc;
    if (is192(c)) {
        uint64_t w[3];
        rc = cbl_read_partial(c, w);
        if (!rc) to_hex192(w, hex);
    } else {
        double a[2];
        rc = cbl_read_partial(c, a);
        if (!rc) dd_to_hex(a[0], a[1], hex);
    }
    return rc;
    CBL_GUARD_END
}

int cbl_workmode_sum(const char *const *hex48, int n, char out[49])
{
    CBL_GUARD_BEGIN
    if (!out || n < 0 || (n > 0 && !hex48)) return CBL_E_ARG;
    int acc[48] = {0};
    for (int j = 0; j < n; ++j) {
        const char *s = hex48[j];
        if (!s) return CBL_E_ARG;
        for (int i = 0; i < 48; ++i)
            if (hexval((unsigned char)s[i]) < 0) return CBL_E_FORMAT;   // also stops at a short string's NUL
        int carry = 0;
        for (int i = 47; i >= 0; --i) {
            const int t = acc[i] + hexval((unsigned char)s[i]) + carry;
            acc[i] = t & 15;
            carry = t >> 4;                                          // out of digit 0: dropped
        }
    }
    static const char hx[] = "0123456789abcdef";
    for (int i = 0; i < 48; ++i) out[i] = hx[acc[i]];
    out[48] = 0;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_job_write(const char *workdir, int s, uint64_t b, const char *hex, int deviceno, const char *devname,
                  int64_t ms)
{
    CBL_GUARD_BEGIN
    if (!workdir || !hex || !formula_ok(s)) return CBL_E_ARG;
    char dir[32];
    std::snprintf(dir, sizeof dir, "/%d", s);
    if (mkdir_p(std::string(workdir) + dir) != 0) return CBL_E_IO;
    const std::string p = job_path(workdir, s, b);
    // Written to a temporary name in the same directory and renamed into place,
    // so a process killed mid-write leaves no partial job file: the job then
    // simply counts as not done. (The reference writes the file in place,
    // Bellard_192.hsp:514-533.)
    char suffix[48];
    std::snprintf(suffix, sizeof suffix, ".tmp%ld", (long)getpid());
    const std::string tmp = p + suffix;
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return CBL_E_IO;
    // HSP writes "\n" as CR LF; the layout is hex / device no TAB name / ms "ms"
    const int w = std::fprintf(f, "%.48s\r\n%d\t%s\r\n%lldms", hex, deviceno, devname ? devname : "",
                               (long long)ms);
    const int cl = std::fclose(f);
    if (w < 0 || cl != 0 || std::rename(tmp.c_str(), p.c_str()) != 0) {
        std::remove(tmp.c_str());
        return CBL_E_IO;
    }
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_job_read(const char *workdir, int s, uint64_t b, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!workdir || !hex || !formula_ok(s)) return CBL_E_ARG;
    const std::string p = job_path(workdir, s, b);
    FILE *f = std::fopen(p.c_str(), "rb");
    if (!f) return CBL_E_IO;
    char line[256] = {0};
    const char *ok = std::fgets(line, sizeof line, f);
    std::fclose(f);
    if (!ok) return CBL_E_FORMAT;
    for (int i = 0; i < 48; ++i)
        if (hexval((unsigned char)line[i]) < 0) return CBL_E_FORMAT;
    std::memcpy(hex, line, 48);
    hex[48] = 0;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_workdir_sum(const char *workdir, char out[49], int counts[7])
{
    CBL_GUARD_BEGIN
    if (!workdir || !out) return CBL_E_ARG;
    std::vector<std::string> hs;
    for (int s = 0; s < 7; ++s) {
        int cnt = 0;
        for (uint64_t b = 0;; ++b) {
            char h[49];
            const std::string p = job_path(workdir, s, b);
            struct stat st;
            if (stat(p.c_str(), &st) != 0) break;                   // first gap ends the series
            const int rc = cbl_job_read(workdir, s, b, h);
            if (rc) return rc;
            hs.emplace_back(h);
            ++cnt;
        }
        if (counts) counts[s] = cnt;
    }
    std::vector<const char *> ptrs;
    for (auto &h : hs) ptrs.push_back(h.c_str());
    return cbl_workmode_sum(ptrs.data(), (int)ptrs.size(), out);
    CBL_GUARD_END
}

int cbl_batch(cbl_ctx *c, const uint64_t *pos, int n, uint64_t *out3n)
{
    CBL_GUARD_BEGIN
    if (!c || (n > 0 && (!pos || !out3n)) || n < 0) return CBL_E_ARG;
    if (!is192(c)) return CBL_E_PRECISION;
    if (n == 0) return CBL_OK;
    std::vector<uint64_t> d(n);
    std::vector<int> sh(n, 0);
    for (int i = 0; i < n; ++i) {
        const int rc = cbl_pos_to_d(pos[i], &d[i], nullptr);
        if (rc) return rc;
    }
    cudaSetDevice(c->device);
    int rc = run_positions(c, d.data(), sh.data(), n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->h_out3, c->d_out3, sizeof(uint64_t) * 3 * n, cudaMemcpyDeviceToHost, c->st));
    rc = sync(c);
    if (rc) return rc;
    std::memcpy(out3n, c->h_out3, sizeof(uint64_t) * 3 * n);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_terms(cbl_ctx *c, uint64_t d, int f, const uint64_t *k, int n, uint64_t *out3n)
{
    CBL_GUARD_BEGIN
    if (!c || !formula_ok(f) || n < 0 || (n > 0 && (!k || !out3n))) return CBL_E_ARG;
    if (n == 0) return CBL_OK;
    for (int i = 0; i < n; ++i)
        if ((u128)kDen0[f] * k[i] + kDen1[f] >= (u128)kW2XMax) return CBL_E_RANGE;
    cudaSetDevice(c->device);
    if (n > c->kbuf_cap) {
        cudaFree(c->d_kbuf);
        c->d_kbuf = nullptr;
        c->kbuf_cap = 0;
        if (cudaMalloc(&c->d_kbuf, sizeof(uint64_t) * 4 * (size_t)n) != cudaSuccess) return CBL_E_NOMEM;
        c->kbuf_cap = n;
    }
    uint64_t *d_out = c->d_kbuf + n;
    CK(cudaMemcpyAsync(c->d_kbuf, k, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, c->st));
    CK(launch_terms_each(d, kDen0[f], kDen1[f], kSign[f], c->d_kbuf, n, d_out, c->st));
    c->launches++;
    CK(cudaMemcpyAsync(out3n, d_out, sizeof(uint64_t) * 3 * n, cudaMemcpyDeviceToHost, c->st));
    return sync(c);
    CBL_GUARD_END
}

int cbl_prepare(cbl_ctx *c, const uint64_t *pos, int n)
{
    CBL_GUARD_BEGIN
    if (!c || n <= 0 || !pos) return CBL_E_ARG;
    if (!is192(c)) return CBL_E_PRECISION;
    std::vector<uint64_t> d(n);
    std::vector<int> sh(n, 0);
    for (int i = 0; i < n; ++i) {
        const int rc = cbl_pos_to_d(pos[i], &d[i], nullptr);
        if (rc) return rc;
    }
    cudaSetDevice(c->device);
    return prepare_positions(c, d.data(), sh.data(), n);
    CBL_GUARD_END
}

int cbl_run_prepared(cbl_ctx *c)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    cudaSetDevice(c->device);
    return launch_prepared(c);
    CBL_GUARD_END
}

int cbl_read_results(cbl_ctx *c, uint64_t *out3n)
{
    CBL_GUARD_BEGIN
    if (!c || !out3n || c->prep_npos <= 0) return CBL_E_ARG;
    cudaSetDevice(c->device);
    const size_t bytes = sizeof(uint64_t) * 3 * c->prep_npos;
    CK(cudaMemcpyAsync(c->h_out3, c->d_out3, bytes, cudaMemcpyDeviceToHost, c->st));
    const int rc = sync(c);
    if (rc) return rc;
    std::memcpy(out3n, c->h_out3, bytes);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_prepared_info(const cbl_ctx *c, uint64_t *terms, uint64_t *tiles, int *segments, int *grid)
{
    CBL_GUARD_BEGIN
    if (!c) return CBL_E_ARG;
    if (terms) *terms = c->prep_terms;
    if (tiles) *tiles = c->prep_ntiles;
    if (segments) *segments = c->prep_nseg;
    if (grid) *grid = grid_192(const_cast<cbl_ctx *>(c));
    return CBL_OK;
    CBL_GUARD_END
}

// ---- autotuning: tile size x persistent CTAs per SM, timed on the caller's
// positions, cached per (device name, SM count, positions) in a text file.
static std::string tune_cache_path()
{
    if (const char *p = std::getenv("CBL_TUNE_CACHE")) return p;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/clbellard_tune.txt";
}

static bool tune_cache_lookup(const std::string &key, int *tile, int *ctas)
{
    FILE *f = std::fopen(tune_cache_path().c_str(), "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (std::fgets(line, sizeof line, f)) {
        char k[400];
        int t, c;
        if (std::sscanf(line, "%399s %d %d", k, &t, &c) == 3 && key == k) {
            *tile = t;
            *ctas = c;
            found = true;                                    // the last entry wins
        }
    }
    std::fclose(f);
    return found;
}

static void tune_cache_store(const std::string &key, int tile, int ctas)
{
    const std::string p = tune_cache_path();
    const size_t slash = p.rfind('/');
    if (slash != std::string::npos) mkdir_p(p.substr(0, slash));
    if (FILE *f = std::fopen(p.c_str(), "a")) {
        std::fprintf(f, "%s %d %d\n", key.c_str(), tile, ctas);
        std::fclose(f);
    }
}

int cbl_autotune(cbl_ctx *c, const uint64_t *pos, int n, int force, int *best_tile, int *best_ctas, double *best_ms)
{
    CBL_GUARD_BEGIN
    if (!c || !pos || n <= 0) return CBL_E_ARG;
    if (!is192(c)) return CBL_E_PRECISION;
    cudaSetDevice(c->device);
    char key[400];
    std::snprintf(key, sizeof key, "%s|sm%d|n%d|h%016llx", c->devname, c->sm_count, n,
                  (unsigned long long)fnv1a(pos, sizeof(uint64_t) * n));
    for (char *q = key; *q; ++q)
        if (*q == ' ') *q = '_';
    int tile = 0, ctas = 0;
    double ms_best = -1.0;
    if (!force && tune_cache_lookup(key, &tile, &ctas)) {
        int rc = cbl_set_tuning(c, tile, ctas);
        if (rc) return rc;
    } else {
        const int occ = terms192_max_ctas_per_sm(256);
        const int tiles[] = {512, 1024, 2048, 4096, 8192};
        ms_best = 1e300;
        for (int t : tiles) {
            for (int cc = occ; cc >= 1 && cc >= occ - 2; --cc) {
                int rc = cbl_set_tuning(c, t, cc);
                if (!rc) rc = cbl_prepare(c, pos, n);
                if (!rc) rc = cbl_run_prepared(c);                 // warm-up and graph capture
                if (!rc) rc = cbl_run_prepared(c);
                float ms = 0;
                if (!rc) rc = cbl_kernel_ms(c, &ms);
                if (rc) return rc;
                if (ms < ms_best) {
                    ms_best = ms;
                    tile = t;
                    ctas = cc;
                }
            }
        }
        int rc = cbl_set_tuning(c, tile, ctas);
        if (rc) return rc;
        tune_cache_store(key, tile, ctas);
    }
    if (best_tile) *best_tile = tile;
    if (best_ctas) *best_ctas = ctas;
    if (best_ms) *best_ms = ms_best;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_run_prepared_budget(cbl_ctx *c, double budget_ms, uint64_t *tiles_done, uint64_t *tiles_total)
{
    CBL_GUARD_BEGIN
    if (!c || budget_ms <= 0 || c->prep_npos <= 0) return CBL_E_ARG;
    cudaSetDevice(c->device);
    const int n = c->prep_npos;
    if (!c->partial) {                                    // a fresh pass
        CK(clear_slots(c, 7 * n));
        CK(cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), c->st));
        c->partial = 1;
    }
    const uint64_t budget_ns = (uint64_t)(budget_ms * 1e6) + 1;
    CK(launch_terms192(c->d_segs, c->prep_nseg, c->prep_ntiles, (uint32_t)c->tile_k, c->d_counter, c->d_slots,
                       grid_192(c), 256, c->st, budget_ns, prepared_carry(c)));
    c->launches++;
    CK(cudaMemcpyAsync(c->h_small, c->d_counter, sizeof(uint64_t), cudaMemcpyDeviceToHost, c->st));
    int rc = sync(c);
    if (rc) return rc;
    const uint64_t done = std::min<uint64_t>(c->h_small[0], c->prep_ntiles);
    if (done >= c->prep_ntiles) {
        CK(launch_combine(c->d_slots, n, c->d_shift, c->d_out3, nullptr, c->st));
        c->launches++;
        c->partial = 0;
    }
    if (tiles_done) *tiles_done = done;
    if (tiles_total) *tiles_total = c->prep_ntiles;
    return CBL_OK;
    CBL_GUARD_END
}

// Checkpoint of a budgeted run: header, tiles done, the slots' digit sums.
struct CkptHeader {
    uint64_t magic, hash, npos, ntiles, done;
};
static const uint64_t kCkptMagic = 0x31544b50434c4243ull;   // "CBLCPKT1"

int64_t cbl_checkpoint_size(const cbl_ctx *c)
{
    if (!c || c->prep_npos <= 0) return CBL_E_ARG;
    return (int64_t)(sizeof(CkptHeader) + sizeof(unsigned long long) * 6 * 7 * c->prep_npos);
}

int cbl_checkpoint_save(cbl_ctx *c, void *buf, int64_t size)
{
    CBL_GUARD_BEGIN
    if (!c || !buf || c->prep_npos <= 0 || size < cbl_checkpoint_size(c)) return CBL_E_ARG;
    cudaSetDevice(c->device);
    int rc = sync(c);
    if (rc) return rc;
    CkptHeader h{kCkptMagic, c->seg_hash, (uint64_t)c->prep_npos, c->prep_ntiles, 0};
    if (c->partial) {
        CK(cudaMemcpy(&h.done, c->d_counter, sizeof(uint64_t), cudaMemcpyDeviceToHost));
        h.done = std::min<uint64_t>(h.done, c->prep_ntiles);
    }
    std::memcpy(buf, &h, sizeof h);
    if (c->partial)
        CK(cudaMemcpy(static_cast<char *>(buf) + sizeof h, c->d_slots, sizeof(unsigned long long) * 6 * 7 * c->prep_npos,
                      cudaMemcpyDeviceToHost));
    else
        std::memset(static_cast<char *>(buf) + sizeof h, 0, sizeof(unsigned long long) * 6 * 7 * c->prep_npos);
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_checkpoint_load(cbl_ctx *c, const void *buf, int64_t size)
{
    CBL_GUARD_BEGIN
    if (!c || !buf || c->prep_npos <= 0 || size < cbl_checkpoint_size(c)) return CBL_E_ARG;
    CkptHeader h;
    std::memcpy(&h, buf, sizeof h);
    if (h.magic != kCkptMagic) return CBL_E_FORMAT;
    if (h.hash != c->seg_hash || h.npos != (uint64_t)c->prep_npos || h.ntiles != c->prep_ntiles || h.done > h.ntiles)
        return CBL_E_FORMAT;                               // not a checkpoint of this prepared run
    cudaSetDevice(c->device);
    CK(cudaMemcpy(c->d_slots, static_cast<const char *>(buf) + sizeof h,
                  sizeof(unsigned long long) * 6 * 7 * c->prep_npos, cudaMemcpyHostToDevice));
    const unsigned long long done = h.done;
    CK(cudaMemcpy(c->d_counter, &done, sizeof done, cudaMemcpyHostToDevice));
    c->partial = 1;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_kernel_ms(cbl_ctx *c, float *ms)
{
    CBL_GUARD_BEGIN
    if (!c || !ms || !c->ev_valid) return CBL_E_ARG;
    cudaSetDevice(c->device);
    CK(cudaEventSynchronize(c->ev_k1));
    CK(cudaEventElapsedTime(ms, c->ev_k0, c->ev_k1));
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_probe_imad(cbl_ctx *c, int iters, double *ops_per_s, double *ms)
{
    CBL_GUARD_BEGIN
    if (!c || iters <= 0) return CBL_E_ARG;
    cudaSetDevice(c->device);
    uint32_t *d_sink = nullptr;
    const int grid = probe_imad_grid(c->sm_count), block = 256;
    if (cudaMalloc(&d_sink, sizeof(uint32_t) * grid * block) != cudaSuccess) return CBL_E_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = CBL_OK;
    double best = 1e30;
    uint64_t ops = 0;
    for (int rep = 0; rep < 4 && !rc; ++rep) {
        cudaEventRecord(e0, c->st);
        if (launch_probe_imad(d_sink, grid, block, iters, &ops, c->st) != cudaSuccess) rc = CBL_E_CUDA;
        cudaEventRecord(e1, c->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = CBL_E_CUDA;
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0) best = std::min(best, (double)t);
        c->launches++;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_sink);
    if (rc) return rc;
    if (ms) *ms = best;
    if (ops_per_s) *ops_per_s = (double)ops / (best * 1e-3);
    return CBL_OK;
    CBL_GUARD_END
}

// ---- HSP-friendly pointer forms
int cbl_pos_to_d_p(const int64_t *needD, int64_t *d, int64_t *needD_adj)
{
    CBL_GUARD_BEGIN
    if (!needD || *needD < 0) return CBL_E_ARG;
    uint64_t a, b;
    const int rc = cbl_pos_to_d((uint64_t)*needD, &a, &b);
    if (rc) return rc;
    if (d) *d = (int64_t)a;
    if (needD_adj) *needD_adj = (int64_t)b;
    return CBL_OK;
    CBL_GUARD_END
}

int cbl_compute_p(cbl_ctx *c, const int64_t *needD, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!needD || *needD < 0) return CBL_E_ARG;
    return cbl_compute(c, (uint64_t)*needD, hex);
    CBL_GUARD_END
}

int cbl_BatchCalc_p(cbl_ctx *c, const int64_t *k_start, const int64_t *k_end, int f, const int64_t *d)
{
    CBL_GUARD_BEGIN
    if (!k_start || !k_end || !d || *k_start < 0 || *k_end < 0 || *d < 0) return CBL_E_ARG;
    return cbl_BatchCalc(c, (uint64_t)*k_start, (uint64_t)*k_end, f, (uint64_t)*d);
    CBL_GUARD_END
}

int cbl_run_job_p(cbl_ctx *c, const int64_t *needD, int s, const int64_t *b, const int64_t *batchsize, char hex[49])
{
    CBL_GUARD_BEGIN
    if (!needD || !b || !batchsize || *needD < 0 || *b < 0 || *batchsize <= 0) return CBL_E_ARG;
    return cbl_run_job(c, (uint64_t)*needD, s, (uint64_t)*b, (uint64_t)*batchsize, hex);
    CBL_GUARD_END
}

}  // extern "C"
