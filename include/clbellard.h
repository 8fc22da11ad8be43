/*
 * clbellard.h - C ABI of the GB300 Bellard pi hex-digit library (libclbellard.so).
 *
 * The library evaluates the 7-term Bellard series for pi at a hex position on
 * one NVIDIA GB300 with hand-written CUDA kernels (sm_103a). Each entry point
 * below replaces one piece of the reference CLBellard host/kernel interface;
 * the reference location is cited beside it (paths inside the CLBellard tree).
 *
 * Conventions
 *  - Every function returns an int status: 0 on success, a negative CBL_E_*
 *    code on failure, CBL_SKIPPED (1) where the reference silently skips a job.
 *    No exceptions, aborts or exit() cross this boundary.
 *  - Precision (Bellard_192.hsp:64): 0 = "106bit" double-double,
 *    1 = "192bit", 2 = "192bit(beta)". Modes 1 and 2 both run the exact 192-bit
 *    integer fixed-point kernels (exact quotients for every modulus).
 *  - 192-bit values cross the ABI as uint64_t[3] with element 0 the MOST
 *    significant word, the reference's bigSum[0..2] / dev_ans order
 *    (Bellard.cl:1359-1398, Bellard_192.hsp:350-361). Double-double values cross
 *    as double[2] = {hi, lo} (the reference's double2 .x/.y).
 *  - Hex strings are 48 lowercase hex digits plus NUL (char[49]), the
 *    reference's printed form (hexsademical.as:104-127). In mode 0 the last 20
 *    digits are '0' as in hexadecimal_dd (hexsademical.as:21-101).
 *  - Ownership: the library owns all device memory; callers own every host
 *    buffer they pass. Nothing returned outlives cbl_destroy.
 *  - Threading: one context per host thread; calls on one context are
 *    serialised by the caller. Several contexts may share a GPU.
 *  - Every call on a context is asynchronous on the context's stream except the
 *    cbl_read_* / cbl_compute / cbl_run_job / cbl_batch family, which
 *    synchronise before returning (like HCLReadBuffer).
 */
#ifndef CLBELLARD_H
#define CLBELLARD_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CBL_OK            0
#define CBL_SKIPPED       1   /* job not run: k_start > d (Bellard_192.hsp:306) */
#define CBL_E_ARG        -1   /* bad argument (null pointer, bad formula index) */
#define CBL_E_POSITION   -2   /* position outside [5, 999999999999999999] (Bellard_192.hsp:449-450) */
#define CBL_E_NODEVICE   -3   /* no CUDA device / bad device index */
#define CBL_E_CUDA       -4   /* a CUDA runtime call failed */
#define CBL_E_TIMEOUT    -5   /* cbl_wait gave up */
#define CBL_E_RANGE      -6   /* k-range outside the entry point's modulus range */
#define CBL_E_NOMEM      -7   /* allocation failed */
#define CBL_E_PRECISION  -8   /* call not valid for the context's precision */
#define CBL_E_IO         -9   /* file read/write failed */
#define CBL_E_FORMAT    -10   /* malformed hex string / worklist */
#define CBL_E_LIMIT     -11   /* request larger than a fixed limit (cbl_batch_noalloc) */

typedef struct cbl_ctx cbl_ctx;

/* ---- context (replaces HCLinit / HCLSetDev / *GlobalMemSet, Bellard_192.hsp:16,250,408-420) */
int cbl_create(int device, int precision, cbl_ctx **out);
int cbl_destroy(cbl_ctx *ctx);
int cbl_precision(const cbl_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time with events. */
void *cbl_stream(cbl_ctx *ctx);
/* Device name (CL_DEVICE_NAME in the reference, Bellard_192.hsp:41,528). */
int cbl_device_name(const cbl_ctx *ctx, char *buf, int len);

/* ---- reference kernel entry points (Bellard.cl / Bellard_div2by1.cl __kernels) */
/* FillBuffer8 over bigSum: Set0memUlong3 / Set0memdd (KernelFuncs.as:15-23). */
int cbl_Set0mem(cbl_ctx *ctx);
/* Zero the running answer dev_ans (Bellard_192.hsp:413-419). */
int cbl_Set0ans(cbl_ctx *ctx);
/* Sglobal32mtg / Sglobal32mtg_192 (Bellard.cl:729-823): add the terms
 * k in [offset, k_max) of the series (numesign, den0, den1) at position d into
 * bigSum. Every modulus den0*k+den1 must be < 2^32, else CBL_E_RANGE. */
int cbl_Sglobal32mtg(cbl_ctx *ctx, uint64_t offset, uint64_t d, uint64_t k_max,
                     int64_t numesign, uint64_t den0, uint64_t den1);
/* Sglobal64mtg / Sglobal64mtg_192 / Sglobal64mtg_192_Refresh (Bellard.cl:914-1092,
 * Bellard_div2by1.cl:313-359): same contract for any modulus below 2^62. In
 * mode 0, moduli from 2^53 up take the OVERDOUBLE route (Bellard.cl:937-945):
 * r and m as exact double-doubles and a double-double division. */
int cbl_Sglobal64mtg(cbl_ctx *ctx, uint64_t offset, uint64_t d, uint64_t k_max,
                     int64_t numesign, uint64_t den0, uint64_t den1);
/* Sglobal_after / Sglobal_after_192 (Bellard.cl:1118-1253): the tail terms
 * k >= d (10 in mode 0, 20 in modes 1-2). */
int cbl_Sglobal_after(cbl_ctx *ctx, uint64_t d, int64_t numesign, uint64_t den0, uint64_t den1);
/* Ssum / Ssum_192 (Bellard.cl:1274-1315): reduce bigSum to the partial. */
int cbl_Ssum(cbl_ctx *ctx);
/* Sum7 / Sum7_192 (Bellard.cl:1324-1398): weight the partial by numer
 * (1,4,32,64,256), write the weighted partial back, add it into dev_ans. */
int cbl_Sum7(cbl_ctx *ctx, uint64_t numer);

/* ---- launch orchestration (KernelFuncs.as) */
/* numer_denom_init (KernelFuncs.as:3-13): series f = 0..6. */
int cbl_formula(int f, uint64_t *numer, int64_t *numesign, uint64_t *den0, uint64_t *den1);
/* BatchCalc (KernelFuncs.as:25-66): terms k in [k_start, min(k_end, d)) of
 * series formulano, the tail when that range reaches d, then Ssum. */
int cbl_BatchCalc(cbl_ctx *ctx, uint64_t k_start, uint64_t k_end, int formulano, uint64_t d);
/* AddAns (KernelFuncs.as:68-74): Sum7 with numer[formulano]. */
int cbl_AddAns(cbl_ctx *ctx, int formulano);

/* ---- readback and completion (HCLReadBuffer / HCLGetEventStatus / HCLFinish) */
/* Partial (bigSum[0..]) and answer (dev_ans): uint64_t[3] in modes 1-2, double[2] in mode 0. */
int cbl_read_partial(cbl_ctx *ctx, void *out);
int cbl_read_ans(cbl_ctx *ctx, void *out);
/* 0 when all queued work is complete (CL_COMPLETE), 1 while running, <0 on error. */
int cbl_query(cbl_ctx *ctx);
/* Wait for queued work; timeout_ms < 0 waits forever. CBL_E_TIMEOUT on expiry. */
int cbl_wait(cbl_ctx *ctx, int timeout_ms);

/* ---- application level (Bellard_192.hsp) */
/* needD -> d (Bellard_192.hsp:449-450,468-470): d odd, needD_adj = (5d+3)/2+1. */
int cbl_pos_to_d(uint64_t needD, uint64_t *d, uint64_t *needD_adj);
/* Normal mode (*Allloop, Bellard_192.hsp:264-296): 48 hex digits of pi starting
 * at hex position needD_adj (1-based), i.e. frac(2^(10d+6) pi). */
int cbl_compute(cbl_ctx *ctx, uint64_t needD, char hex[49]);
/* Any hex position p >= 3 (not limited to multiples of 5): frac(16^(p-1) pi).
 * The low `shift` bits (shift = 4(p-1)-6 mod 10 <= 9) of the 192 are zero. */
int cbl_compute_hexpos(cbl_ctx *ctx, uint64_t p, char hex[49]);
/* Mode-0 result printer (replaces hexadecimal_dd, hexsademical.as:21-101): a
 * double-double hi + lo (|hi|, |lo| < 1) taken mod 1, as 28 hex digits (112
 * bits) and 20 zeros. A negative value is lifted by 1.0 with the reference's
 * own double-double add, then truncated exactly: the reference's bytes, except
 * after a negative intermediate byte (hexsademical.as:73-97), where the
 * reference keeps x + 256 as the remainder and prints every later byte as 00;
 * here those bytes are the value's own. Host only. */
int cbl_hex_dd(double hi, double lo, char hex[49]);
/* Work-mode job (s, b) (*Batchloop body, Bellard_192.hsp:304-333): terms
 * k in [b*batchsize, (b+1)*batchsize) of series s, weighted by numer; hex is
 * line 0 of the reference's work/<s>/<s>_<b>.txt. CBL_SKIPPED if b*batchsize > d. */
int cbl_run_job(cbl_ctx *ctx, uint64_t needD, int s, uint64_t b, uint64_t batchsize, char hex[49]);
/* Work-mode job over an explicit k-range [k0, k1) of series s (the tail is
 * included when the range reaches d), weighted by numer; as cbl_run_job. */
int cbl_run_job_range(cbl_ctx *ctx, uint64_t needD, int s, uint64_t k0, uint64_t k1, char hex[49]);
/* Balanced work-mode plan (instead of the reference's fixed 2^37-term batches,
 * Bellard_192.hsp:19): njobs >= 7 jobs of about equal estimated device time,
 * from a per-term model (ladder steps x the residue kind's step cost). Job i is
 * series out_s[i], k in [out_k0[i], out_k1[i]); the ranges of one series tile
 * [0, d + 20), and only the last one reaches d. At most d jobs per series.
 * Returns the number of jobs (<= njobs <= cap) or a negative code. */
int cbl_plan_jobs(uint64_t needD, int njobs, int *out_s, uint64_t *out_k0, uint64_t *out_k1, int cap);
/* workmodeSum0_6.hsp:10-49: sum of n 48-digit hex strings mod 16^48. */
int cbl_workmode_sum(const char *const *hex48, int n, char out[49]);
/* Write / read a job file in the reference layout (Bellard_192.hsp:514-533):
 * <dir>/<s>/<s>_<b>.txt = hex, '\n', device no '\t' device name, '\n', ms "ms". */
int cbl_job_write(const char *workdir, int s, uint64_t b, const char *hex, int deviceno,
                  const char *devname, int64_t ms);
int cbl_job_read(const char *workdir, int s, uint64_t b, char hex[49]);
/* Merge every existing <dir>/s/s_b.txt (s = 0..6, b = 0,1,... until a gap),
 * as workmodeSum does; counts[7] receives the files found per series. */
int cbl_workdir_sum(const char *workdir, char out[49], int counts[7]);

/* ---- batched positions (one persistent launch over all positions) */
/* out3n[3*i .. 3*i+2] = 192-bit result for reference position pos[i] (modes 1-2). */
int cbl_batch(cbl_ctx *ctx, const uint64_t *pos, int n, uint64_t *out3n);

/* ---- prepared runs (the timed device pass of a benchmark) */
/* Build and upload the tile table for reference positions pos[0..n). */
int cbl_prepare(cbl_ctx *ctx, const uint64_t *pos, int n);
/* Enqueue one full pass over the prepared positions (no host sync). */
int cbl_run_prepared(cbl_ctx *ctx);
/* Copy the prepared positions' results (3 words each, most significant first). */
int cbl_read_results(cbl_ctx *ctx, uint64_t *out3n);
/* Bounded-time pass (the reference's "GPU 99% load" launch splitting,
 * Bellard_192.hsp:74, KernelFuncs.as:36-51): starts a pass over the prepared
 * positions, or continues the one in progress, for about budget_ms of device
 * time, waits, and reports the warp tiles finished so far. When
 * tiles_done == tiles_total the results are ready for cbl_read_results.
 * Resumed passes give the same bits as an uninterrupted one. */
int cbl_run_prepared_budget(cbl_ctx *ctx, double budget_ms, uint64_t *tiles_done, uint64_t *tiles_total);
/* Checkpoint of a pass in progress (on-device 192-bit partial sums and the
 * tiles finished): size, save to a host buffer, load into a context that has
 * prepared the same positions (CBL_E_FORMAT otherwise), then continue with
 * cbl_run_prepared_budget. */
int64_t cbl_checkpoint_size(const cbl_ctx *ctx);
int cbl_checkpoint_save(cbl_ctx *ctx, void *buf, int64_t size);
int cbl_checkpoint_load(cbl_ctx *ctx, const void *buf, int64_t size);
/* cbl_run_prepared replays a CUDA graph captured on its first call after
 * cbl_prepare (enable = 1, the default); 0 launches the kernels directly. */
int cbl_set_graph(cbl_ctx *ctx, int enable);
/* Device time of the term kernel in the last cbl_run_prepared (CUDA events on
 * the context's stream around that launch); waits for it to finish. */
int cbl_kernel_ms(cbl_ctx *ctx, float *ms);
/* Terms (7*d summed, tail excluded), warp tiles, segments and persistent grid of the prepared run. */
int cbl_prepared_info(const cbl_ctx *ctx, uint64_t *terms, uint64_t *tiles, int *segments, int *grid);

/* ---- diagnostics */
/* Peak rate of 32-bit multiply halves on this GPU (dependent mad.lo.u32
 * chains, one half per instruction): the denominator of the term kernels'
 * roofline. */
int cbl_probe_imad(cbl_ctx *ctx, int iters, double *ops_per_s, double *ms);
/* Individual signed 192-bit terms (the per-term check of the oracle):
 * out3n[3*i..] = term k[i] of series f at position d; k >= d gives tail terms. */
int cbl_terms(cbl_ctx *ctx, uint64_t d, int f, const uint64_t *k, int n, uint64_t *out3n);
/* Kernel launches issued on this context since creation (counts every kernel). */
int64_t cbl_launch_count(const cbl_ctx *ctx);
/* Autotuner: times one pass over pos[0..n) for each warp-tile size
 * (512..8192 terms) and persistent CTAs per SM (the occupancy limit and two
 * below it), keeps the fastest (cbl_set_tuning) and appends it to a cache
 * file ($CBL_TUNE_CACHE, default ~/.cache/clbellard_tune.txt) keyed by device,
 * SM count and positions; a cached entry is reused unless force != 0
 * (*best_ms is then -1). Leaves the context prepared for pos. */
int cbl_autotune(cbl_ctx *ctx, const uint64_t *pos, int n, int force, int *best_tile, int *best_ctas,
                 double *best_ms);
/* Test hook (no counterpart in the reference): the six digit sums every slot of
 * later prepared passes (cbl_compute, cbl_batch, cbl_run_prepared) starts from,
 * instead of zero; NULL restores zero. A slot's value is sum_j preset[j]*2^(32j)
 * mod 2^192, so each series partial grows by that value and the result by
 * sum_f (value << log2(numer_f)). Presets near 2^64 make the digit sums wrap
 * within a few tiles, which exercises the carry that keeps results exact however
 * many tiles land in one slot (positions beyond 2^32 tiles per series). */
int cbl_set_slot_preset(cbl_ctx *ctx, const uint64_t preset[6]);
/* Tuning: terms per warp tile (multiple of 32) and persistent CTAs per SM (0 = auto). */
int cbl_set_tuning(cbl_ctx *ctx, int tile_terms, int ctas_per_sm);
const char *cbl_strerror(int code);

/* ---- allocation-free evaluation (no counterpart in the reference)
 * For callers that must not allocate GPU memory themselves: programs whose
 * device memory is owned by another allocator or fixed budget (a framework's
 * caching allocator, a long-running service that allocates only at start-up),
 * or pipelines that cannot absorb the device-wide synchronisation that
 * cudaMalloc / cudaFree may cause. cbl_batch_noalloc evaluates up to
 * CBL_NOALLOC_MAX_POSITIONS reference positions in 192-bit mode on the CURRENT
 * device and stream and calls no cudaMalloc, cudaFree or other allocating
 * routine. The caller passes pos[0..n) (host) and d_out3n, a device buffer it
 * owns of 3*n uint64_t; d_out3n[3i..3i+2] receives position i's result (most
 * significant word first), bit-identical to cbl_batch, once `stream` (a
 * cudaStream_t, 0 for the legacy default stream) reaches that point. The
 * positions go to the GPU as a kernel argument and the tile table is built on
 * the device, so the call makes no host-to-device copy: it enqueues a memset
 * and three kernels and returns without waiting for them.
 * The kernels' scratch is one static device array of CBL_NOALLOC_SCRATCH_BYTES
 * (about 169 KiB) that every GPU loading this library holds until the process
 * exits. The first call on each device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current; make that first call before
 * any stream capture. All calls on a device share the array and each call
 * clears it before use, so calls whose work overlaps on the GPU (different
 * streams, or several host threads) race and corrupt each other's results:
 * serialise them. n > CBL_NOALLOC_MAX_POSITIONS returns CBL_E_LIMIT; positions
 * are validated as in cbl_compute (CBL_E_POSITION). */
#define CBL_NOALLOC_MAX_POSITIONS 64
#define CBL_NOALLOC_SCRATCH_BYTES 172544
int cbl_batch_noalloc(const uint64_t *pos, int n, uint64_t *d_out3n, void *stream);

/* ---- HSP-friendly variants: 64-bit arguments by pointer (HSP passes int64 vars
 * by address; #uselib/#func cannot pass 64-bit values directly). */
int cbl_pos_to_d_p(const int64_t *needD, int64_t *d, int64_t *needD_adj);
int cbl_compute_p(cbl_ctx *ctx, const int64_t *needD, char hex[49]);
int cbl_BatchCalc_p(cbl_ctx *ctx, const int64_t *k_start, const int64_t *k_end, int formulano,
                    const int64_t *d);
int cbl_run_job_p(cbl_ctx *ctx, const int64_t *needD, int s, const int64_t *b,
                  const int64_t *batchsize, char hex[49]);

#ifdef __cplusplus
}
#endif
#endif
