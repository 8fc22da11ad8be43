/*
 * harness.cpp - runs the reference's own OpenCL kernels (Bellard.cl,
 * Bellard_div2by1.cl, compiled as C++ through shim.h) on the CPU with the
 * reference's launch sequence (KernelFuncs.as:15-74, Bellard_192.hsp:264-296,
 * 376-420, 468-470). TEST INFRASTRUCTURE: the reference run here, used to pin
 * the oracle and as a CPU baseline. Work-groups of 256 work-items run as
 * ucontext fibers (barrier() = yield to the group scheduler), one work-group
 * per OS thread at a time (OpenMP over groups).
 *
 *   ref_bellard <needD> <precision 0|1|2> [groups=64] [threads=all] [k0 k1 chunks]
 *   prints: d, the 48-hex result (mode 0: double-double hi lo), seconds, terms/s
 * With k0 k1 chunks: a timing sample instead of a full position: for every
 * series, `chunks` ranges of (k1-k0) terms spread evenly over [0, d) run as the
 * reference's BatchCalc main loops (no tail); terms/s counts those terms.
 *
 *   ref_bellard range <needD> <precision> <f> <k0> <k1> [groups=64] [threads=all]
 *   prints: d, and the series-f partial over k in [k0, min(k1, d)) plus the
 *   tail when the range reaches d, after Ssum and before Sum7 (the reference's
 *   BatchCalc for one series: bigSum[0..2] as 48 hex, or the dd pair).
 */
#include "shim.h"

#include <omp.h>
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>
#include <chrono>

thread_local WorkItem cl_wi;

namespace bellard {
#include "Bellard.cl"
}
namespace div2by1 {
#include "Bellard_div2by1.cl"
}

// ---------------------------------------------------------------- fibers --
namespace {
constexpr int kLocal = 256;                  // LOCAL_WORK_SIZE (Bellard_192.hsp:6)
constexpr size_t kStack = 64 * 1024;

struct Group {
    ucontext_t sched;
    ucontext_t ctx[kLocal];
    std::vector<char> stacks;
    bool done[kLocal];
    WorkItem wi[kLocal];
    int current;
    const std::function<void()> *body;
};
thread_local Group *cur_group = nullptr;

void fiber_entry()
{
    Group *g = cur_group;
    (*g->body)();
    g->done[g->current] = true;
    // returning goes to uc_link (the scheduler)
}
}  // namespace

void barrier(int)
{
    Group *g = cur_group;
    swapcontext(&g->ctx[g->current], &g->sched);
    cl_wi = g->wi[g->current];
}

// Run one work-group: every work-item runs `body` until its next barrier, in
// rounds, so all of them pass each barrier together.
static void run_group(Group &g, ulong group_id, ulong global_size, int local_size, const std::function<void()> &body)
{
    g.body = &body;
    if (g.stacks.empty()) g.stacks.resize(kStack * kLocal);
    cur_group = &g;
    for (int i = 0; i < local_size; ++i) {
        g.done[i] = false;
        g.wi[i] = WorkItem{group_id * (ulong)local_size + i, (ulong)i, group_id, global_size};
        getcontext(&g.ctx[i]);
        g.ctx[i].uc_stack.ss_sp = g.stacks.data() + kStack * i;
        g.ctx[i].uc_stack.ss_size = kStack;
        g.ctx[i].uc_link = &g.sched;
        makecontext(&g.ctx[i], fiber_entry, 0);
    }
    for (;;) {
        bool any = false;
        for (int i = 0; i < local_size; ++i) {
            if (g.done[i]) continue;
            any = true;
            g.current = i;
            cl_wi = g.wi[i];
            swapcontext(&g.sched, &g.ctx[i]);
        }
        if (!any) break;
    }
}

// HCLDoKrn1 kernel, global, local: all groups of an NDRange, groups spread over threads
static void launch(ulong global, int local, const std::function<void()> &body, int threads)
{
    const long ngroups = (long)(global / (ulong)local);
#pragma omp parallel num_threads(threads)
    {
        Group *g = new Group();
#pragma omp for schedule(dynamic, 1)
        for (long gi = 0; gi < ngroups; ++gi) run_group(*g, (ulong)gi, global, local, body);
        delete g;
    }
}

int main(int argc, char **argv)
{
    const bool range = argc > 1 && !strcmp(argv[1], "range");
    if (range) {
        if (argc < 7) {
            fprintf(stderr, "usage: ref_bellard range needD precision f k0 k1 [groups] [threads]\n");
            return 2;
        }
        ++argv;                                          // the rest reads like the position form
        --argc;
    }
    if (argc < 3) {
        fprintf(stderr, "usage: ref_bellard needD precision [groups] [threads]\n");
        return 2;
    }
    long long needD = atoll(argv[1]);
    const int precision = atoi(argv[2]);
    const int rf = range ? atoi(argv[3]) : -1;
    const ulong rk0 = range ? strtoull(argv[4], nullptr, 10) : 0, rk1 = range ? strtoull(argv[5], nullptr, 10) : 0;
    if (range) {                                         // groups / threads follow the range arguments
        argv += 3;
        argc -= 3;
        if (rf < 0 || rf > 6 || rk1 < rk0) return 2;
    }
    const int groups = argc > 3 ? atoi(argv[3]) : 64;
    const int threads = argc > 4 && atoi(argv[4]) > 0 ? atoi(argv[4]) : omp_get_max_threads();
    const bool sample = !range && argc > 7;
    const long long slen = sample ? atoll(argv[6]) - atoll(argv[5]) : 0;
    const int nchunks = sample ? atoi(argv[7]) : 1;
    if (needD <= 4) return 2;
    // Bellard_192.hsp:468-470
    long long d = ((needD - 1) * 2 - 3) / 5;
    if (d % 2 == 0) d--;
    const ulong GWS = (ulong)groups * kLocal;            // GLOBAL_WORK_SIZE with `groups` work-groups
    const ulong BIGSUM = (ulong)groups;                  // one bigSum entry per work-group
    // KernelFuncs.as:9-12
    const long long numer[7] = {32, 1, 256, 64, 4, 4, 1}, nsign[7] = {1, 1, 0, 1, 1, 1, 0};
    const long long den0[7] = {4, 4, 10, 10, 10, 10, 10}, den1[7] = {1, 3, 1, 3, 5, 7, 9};
    const int words = precision == 0 ? 2 : 3;
    std::vector<ulong> bigSum(BIGSUM * words + 256 * 3, 0), smallSum(256 * 3, 0), dev_ans(3, 0);
    double *bigD = reinterpret_cast<double *>(bigSum.data());
    double *ansD = reinterpret_cast<double *>(dev_ans.data());
    auto t0 = std::chrono::steady_clock::now();
    long long sample_terms = 0;
    for (int fc = 0; fc < 7 * nchunks; ++fc) {
        const int f = range ? rf : fc / nchunks;
        if (range && fc > 0) break;
        std::fill(bigSum.begin(), bigSum.end(), 0);              // Set0memUlong3 / Set0memdd
        // BatchCalc k_start, k_end, f (KernelFuncs.as:25-66); the whole of [0, d) unless sampling
        ulong k_start = 0, k_end = (ulong)d;
        if (range) {
            k_start = std::min(rk0, (ulong)d);
            k_end = std::min(rk1, (ulong)d);
        }
        if (sample) {
            k_start = (ulong)((long double)d * (fc % nchunks) / nchunks);
            k_end = std::min((ulong)d, k_start + (ulong)slen);
            sample_terms += (long long)(k_end - k_start);
        }
        ulong k_max = k_start, offset = k_start;
        if (range && rk0 > (ulong)d) offset = rk0;               // past d: nothing runs (Bellard_192.hsp:306)
        ulong loopmax32 = (((ulong)1 << 32) - den1[f] - 1) / den0[f] + 1;
        if (loopmax32 > (ulong)d) loopmax32 = d;
        if (loopmax32 > k_end) loopmax32 = k_end;
        while (offset < loopmax32) {
            k_max = std::min(k_max + GWS * 16, loopmax32);
            const ulong o = offset, km = k_max;
            if (precision == 0)
                launch(GWS, kLocal, [&, o, km] { bellard::Sglobal32mtg((double2 *)bigD, o, d, km, nsign[f], den0[f], den1[f]); }, threads);
            else
                launch(GWS, kLocal, [&, o, km] { bellard::Sglobal32mtg_192(bigSum.data(), o, d, km, nsign[f], den0[f], den1[f]); }, threads);
            offset = k_max;
        }
        while (offset < k_end) {
            k_max = std::min(k_max + GWS * 32, k_end);
            const ulong o = offset, km = k_max;
            if (precision == 0)
                launch(GWS, kLocal, [&, o, km] { bellard::Sglobal64mtg((double2 *)bigD, o, d, km, nsign[f], den0[f], den1[f]); }, threads);
            else if (precision == 1)
                launch(GWS, kLocal, [&, o, km] { bellard::Sglobal64mtg_192(bigSum.data(), o, d, km, nsign[f], den0[f], den1[f]); }, threads);
            else
                launch(GWS, kLocal, [&, o, km] { div2by1::Sglobal64mtg_192_Refresh(bigSum.data(), o, d, km, nsign[f], den0[f], den1[f]); }, threads);
            offset = k_max;
        }
        if (sample) continue;
        if (offset == (ulong)d) {                                // KernelFuncs.as: the tail when the loops reach d
            if (precision == 0)
                launch(1, 1, [&] { bellard::Sglobal_after((double2 *)bigD, d, nsign[f], den0[f], den1[f]); }, 1);
            else
                launch(1, 1, [&] { bellard::Sglobal_after_192(bigSum.data(), d, nsign[f], den0[f], den1[f]); }, 1);
        }
        // Ssum: the reference reduces 65536 -> 256 -> 1; here the group
        // partials (padded with zeros to 256 entries) go through one 256-wide pass
        if (precision == 0) {
            launch(256, kLocal, [&] { bellard::Ssum((const double2 *)bigD, (double2 *)smallSum.data()); }, 1);
            bigD[0] = ((double *)smallSum.data())[0];
            bigD[1] = ((double *)smallSum.data())[1];
            if (range) break;
            launch(1, 1, [&] { bellard::Sum7((double2 *)ansD, (double2 *)bigD, numer[f]); }, 1);
        } else {
            launch(256, kLocal, [&] { bellard::Ssum_192(bigSum.data(), smallSum.data()); }, 1);
            bigSum[0] = smallSum[0];
            bigSum[1] = smallSum[1];
            bigSum[2] = smallSum[2];
            if (range) break;
            launch(1, 1, [&] { bellard::Sum7_192(dev_ans.data(), bigSum.data(), numer[f]); }, 1);
        }
    }
    if (range) {
        printf("d %lld\n", d);
        if (precision == 0)
            printf("partial_dd %.17g %.17g\n", bigD[0], bigD[1]);
        else
            printf("partial %016llx%016llx%016llx\n", (unsigned long long)bigSum[0], (unsigned long long)bigSum[1],
                   (unsigned long long)bigSum[2]);
        return 0;
    }
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("d %lld\n", d);
    if (precision == 0)
        printf("dd %.17g %.17g\n", ansD[0], ansD[1]);
    else
        printf("hex %016llx%016llx%016llx\n", (unsigned long long)dev_ans[0], (unsigned long long)dev_ans[1],
               (unsigned long long)dev_ans[2]);
    printf("seconds %.3f\nterms_per_s %.4g\nthreads %d\n", sec, (sample ? (double)sample_terms : 7.0 * d) / sec,
           threads);
    return 0;
}
