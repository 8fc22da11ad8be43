/*
 * cbl_main.c - command-line driver over libclbellard.so, taking the roles of
 * CLBellard.exe (normal mode and work mode, Bellard_192.hsp) and
 * workmodeSum0_6.exe (workmodeSum0_6.hsp) without the GUI.
 *
 *   cbl normal <digits> [precision 0|1|2] [device] [--json] [--check]
 *       --json   one JSON line: position, d, mode, terms, seconds, terms/s, hex
 *       --check  also computes hex position P-8 and reports how many of the
 *                overlapping hex digits agree (192-bit modes)
 *   cbl work   <worklist.txt> [workdir] [device]
 *   cbl sum    [workdir]
 *   cbl hexpos <p> [device]            any hex position p >= 3
 *   cbl plan   <digits> <jobs> [precision]   balanced worklist on stdout
 */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "clbellard.h"

static const uint64_t kBatchSize = 137438953472ull; /* 2^37, Bellard_192.hsp:19 */

static int64_t now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (int64_t)ts.tv_sec * 1000 + ts.tv_nsec / 1000000;
}

static int fail(int rc, const char *what)
{
    fprintf(stderr, "%s: %s (%d)\n", what, cbl_strerror(rc), rc);
    return 1;
}

/* "digits=..." with ',', ' ', '-' removed (Bellard_192.hsp:179-182, 444-447). */
static uint64_t parse_digits(const char *s)
{
    uint64_t v = 0;
    int any = 0;
    for (; *s; ++s) {
        if (isdigit((unsigned char)*s)) {
            if (v > 99999999999999999ull) return 999999999999999999ull + 1; /* clamp above the limit */
            v = v * 10 + (uint64_t)(*s - '0');
            any = 1;
        }
    }
    return any ? v : 0;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int cmd_normal(int argc, char **argv)
{
    int json = 0, check = 0, npos = 0;
    const char *pos[3] = {NULL, NULL, NULL};              /* digits, precision, device */
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--json")) json = 1;
        else if (!strcmp(argv[i], "--check")) check = 1;
        else if (npos < 3) pos[npos++] = argv[i];
    }
    if (!pos[0]) return fprintf(stderr, "usage: cbl normal <digits> [precision] [device] [--json] [--check]\n"), 2;
    uint64_t needD = parse_digits(pos[0]), d, adj;
    int precision = pos[1] ? atoi(pos[1]) : 1, device = pos[2] ? atoi(pos[2]) : 0;
    int rc = cbl_pos_to_d(needD, &d, &adj);
    if (rc) return fail(rc, "invalid digits");
    cbl_ctx *c;
    if ((rc = cbl_create(device, precision, &c))) return fail(rc, "cbl_create");
    char name[256], hex[49], hex8[49];
    cbl_device_name(c, name, sizeof name);
    if (!json) printf("%s\ndigits=%llu\nloopnum=%llu\n", name, (unsigned long long)adj, (unsigned long long)d);
    const double t0 = now_s();
    rc = cbl_compute(c, needD, hex);
    const double t1 = now_s();
    if (rc) return cbl_destroy(c), fail(rc, "cbl_compute");
    /* overlap: hex digit i of position P is digit i+8 of position P-8 */
    int overlap = -1;
    if (check && precision != 0 && adj > 10) {
        rc = cbl_compute_hexpos(c, adj - 8, hex8);
        if (rc) return cbl_destroy(c), fail(rc, "cbl_compute_hexpos");
        overlap = 0;
        while (overlap < 40 && hex[overlap] == hex8[overlap + 8]) ++overlap;
    }
    if (json) {
        printf("{\"position\": %llu, \"d\": %llu, \"mode\": %d, \"terms\": %llu, \"seconds\": %.6f, "
               "\"terms_per_s\": %.6g, \"hex\": \"%s\", \"device\": \"%s\"",
               (unsigned long long)adj, (unsigned long long)d, precision, (unsigned long long)(7 * d), t1 - t0,
               7.0 * (double)d / (t1 - t0), hex, name);
        if (overlap >= 0) printf(", \"overlap_digits\": %d", overlap);
        printf("}\n");
    } else {
        printf("All calc time %lldms\nPI value output -> \n%s\n", (long long)((t1 - t0) * 1000.0), hex);
        if (overlap >= 0) printf("hex digits agreeing with position %llu: %d\n", (unsigned long long)(adj - 8), overlap);
    }
    cbl_destroy(c);
    return 0;
}

static int cmd_work(int argc, char **argv)
{
    if (argc < 3) return fprintf(stderr, "usage: cbl work <worklist> [workdir] [device]\n"), 2;
    const char *workdir = argc > 3 ? argv[3] : "work";
    int device = argc > 4 ? atoi(argv[4]) : 0;
    FILE *f = fopen(argv[2], "rb");
    if (!f) return fail(CBL_E_IO, argv[2]);
    char line[512];
    uint64_t needD = 0;
    int precision = -1, ln = 0, rc;
    cbl_ctx *c = NULL;
    char name[256] = "";
    while (fgets(line, sizeof line, f)) {
        if (ln == 0) {
            needD = parse_digits(line); /* Bellard_192.hsp:178-182 */
        } else if (ln == 1) {
            const char *p = strchr(line, '='); /* first character after "precision=" (:184-189) */
            p = p ? p + 1 : line;
            while (*p == ' ') ++p;
            precision = (*p >= '0' && *p <= '2') ? *p - '0' : -1;
            if (needD < 5 || needD > 999999999999999999ull || precision < 0) {
                fclose(f);
                return fail(CBL_E_FORMAT, "worklist header"); /* Bellard_192.hsp:222-226 */
            }
            if ((rc = cbl_create(device, precision, &c))) {
                fclose(f);
                return fail(rc, "cbl_create");
            }
            cbl_device_name(c, name, sizeof name);
        } else {
            /* "s_b" (Bellard_192.hsp:238-244), or "s_b k0 k1" for an explicit k-range */
            if (!isdigit((unsigned char)line[0]) || line[1] != '_') { ++ln; continue; }
            int s = line[0] - '0';
            char *end = NULL;
            uint64_t b = strtoull(line + 2, &end, 10);
            unsigned long long k0 = 0, k1 = 0;
            const int ranged = end && sscanf(end, "%llu %llu", &k0, &k1) == 2;
            char hex[49];
            if (cbl_job_read(workdir, s, b, hex) == CBL_OK) { ++ln; continue; } /* done before (:307-308) */
            const int64_t t0 = now_ms();
            rc = ranged ? cbl_run_job_range(c, needD, s, k0, k1, hex) : cbl_run_job(c, needD, s, b, kBatchSize, hex);
            const int64_t ms = now_ms() - t0;
            if (rc == CBL_SKIPPED) { ++ln; continue; }
            if (rc) { fclose(f); cbl_destroy(c); return fail(rc, "cbl_run_job"); }
            rc = cbl_job_write(workdir, s, b, hex, device, name, ms);
            if (rc) { fclose(f); cbl_destroy(c); return fail(rc, "cbl_job_write"); }
            printf("%d_%llu : time=%lldms\n%s\n", s, (unsigned long long)b, (long long)ms, hex);
        }
        ++ln;
    }
    fclose(f);
    if (c) cbl_destroy(c);
    printf("end\n");
    return 0;
}

static int cmd_sum(int argc, char **argv)
{
    const char *workdir = argc > 2 ? argv[2] : "work";
    char out[49];
    int counts[7];
    int rc = cbl_workdir_sum(workdir, out, counts);
    if (rc) return fail(rc, "workmode sum");
    printf("file num\n");
    for (int s = 0; s < 7; ++s) printf("%d:%d\n", s, counts[s]);
    printf("\n%s\n", out);
    return 0;
}

static int cmd_hexpos(int argc, char **argv)
{
    if (argc < 3) return fprintf(stderr, "usage: cbl hexpos <p> [device]\n"), 2;
    uint64_t p = strtoull(argv[2], NULL, 10);
    cbl_ctx *c;
    int rc = cbl_create(argc > 3 ? atoi(argv[3]) : 0, 1, &c);
    if (rc) return fail(rc, "cbl_create");
    char hex[49];
    rc = cbl_compute_hexpos(c, p, hex);
    cbl_destroy(c);
    if (rc) return fail(rc, "cbl_compute_hexpos");
    printf("%s\n", hex);
    return 0;
}

static int cmd_plan(int argc, char **argv)
{
    if (argc < 4) return fprintf(stderr, "usage: cbl plan <digits> <jobs> [precision]\n"), 2;
    const uint64_t needD = parse_digits(argv[2]);
    const int njobs = atoi(argv[3]);
    const int precision = argc > 4 ? atoi(argv[4]) : 1;
    if (njobs < 7 || njobs > 100000) return fail(CBL_E_ARG, "jobs");
    int *s = malloc(sizeof(int) * njobs);
    uint64_t *k0 = malloc(sizeof(uint64_t) * njobs), *k1 = malloc(sizeof(uint64_t) * njobs);
    int count[7] = {0};
    const int n = cbl_plan_jobs(needD, njobs, s, k0, k1, njobs);
    if (n < 0) return free(s), free(k0), free(k1), fail(n, "cbl_plan_jobs");
    uint64_t adj = 0, d = 0;
    cbl_pos_to_d(needD, &d, &adj);
    printf("digits=%llu\nprecision=%d (0=106bit , 1=192bit)\n", (unsigned long long)adj, precision);
    for (int i = 0; i < n; ++i)
        printf("%d_%d %llu %llu\n", s[i], count[s[i]]++, (unsigned long long)k0[i], (unsigned long long)k1[i]);
    free(s); free(k0); free(k1);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc >= 2 && !strcmp(argv[1], "normal")) return cmd_normal(argc, argv);
    if (argc >= 2 && !strcmp(argv[1], "work")) return cmd_work(argc, argv);
    if (argc >= 2 && !strcmp(argv[1], "sum")) return cmd_sum(argc, argv);
    if (argc >= 2 && !strcmp(argv[1], "hexpos")) return cmd_hexpos(argc, argv);
    if (argc >= 2 && !strcmp(argv[1], "plan")) return cmd_plan(argc, argv);
    fprintf(stderr, "usage: cbl normal|work|sum|hexpos|plan ...\n");
    return 2;
}
