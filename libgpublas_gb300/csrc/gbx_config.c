/*
 * gbx_config.c — BLAS2CUDA_OPTIONS parsing.
 *
 * Same variable and syntax as the reference (blas2cuda.c:46-124): options
 * chained with ';'.  Kept: help, debug_execfail, debug_exec, trace_copy,
 * heuristic=random|true|false|oracle:<file> (the allocation placement policy;
 * read by the allocation interposer).  Added:
 *   precision=fp64|ozaki[:<tol>]  route dgemm_/zgemm_/dsyrk_ to the Ozaki
 *                                 split-precision path (default fp64)
 *   prefetch=on|off               prefetch managed operands (default on)
 *   errors=abort|return           on a CUDA failure inside a Fortran call,
 *                                 abort (the reference's behaviour) or print
 *                                 and return (default abort)
 * Unlike the reference, the environment string is copied before tokenising.
 */
#include "gbx_internal.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static gbx_config g_cfg = {0, 1e-14, 1, 1, 0, 0, 0, {0}, {0}, 0, {0}};
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

static const char help_text[] =
          "gbxblas options (set BLAS2CUDA_OPTIONS, chain with ';'):\n"
          "   help                      -- print help\n"
          "   debug_execfail            -- accepted for compatibility\n"
          "   debug_exec                -- accepted for compatibility\n"
          "   trace_copy                -- accepted for compatibility\n"
          "   heuristic=<val>           -- one of: 'random', 'true', 'false', or\n"
          "                                'oracle:<filename>' (allocation placement)\n"
          "   precision=fp64|ozaki[:t]  -- FP64 or Ozaki split products (target error t)\n"
          "   prefetch=on|off           -- prefetch managed operands to the GPU\n"
          "   errors=abort|return       -- behaviour on a device failure\n"
          "   serve=on|off              -- route Level-3 calls through the serving loop\n"
          "   managed_min=<bytes>       -- smaller allocations stay on the host\n"
          "   statistics[=<file>]       -- write call/placement counters at exit\n"
          "   trace=<file>              -- (preload library) write the allocation/call trace\n";

static void print_help(void) { fputs(help_text, stderr); }

/* The option help without stdio (usable from the program entry point). */
void gbx_print_options(int fd)
{
    if (write(fd, help_text, sizeof help_text - 1) < 0) { /* nothing to do */ }
}

static void parse(void)
{
    const char *env = getenv("BLAS2CUDA_OPTIONS");
    if (!env || !*env) return;
    char *copy = strdup(env);
    if (!copy) return;
    char *save = NULL;
    int helped = 0;
    for (char *opt = strtok_r(copy, ";", &save); opt; opt = strtok_r(NULL, ";", &save)) {
        if (strcmp(opt, "help") == 0) {
            if (!helped) print_help();
            helped = 1;
        } else if (strcmp(opt, "debug_execfail") == 0 || strcmp(opt, "debug_exec") == 0 ||
                   strcmp(opt, "trace_copy") == 0) {
            /* parsed but unused in the reference as well */
        } else if (strncmp(opt, "heuristic=", 10) == 0) {
            const char *h = opt + 10;
            if (strncmp(h, "random", 6) == 0) g_cfg.heuristic = 2;
            else if (strncmp(h, "true", 4) == 0) g_cfg.heuristic = 1;
            else if (strncmp(h, "false", 5) == 0) g_cfg.heuristic = 0;
            else if (strncmp(h, "oracle:", 7) == 0) {
                g_cfg.heuristic = 3;
                snprintf(g_cfg.oracle_file, sizeof g_cfg.oracle_file, "%s", h + 7);
            } else fprintf(stderr, "gbxblas: unsupported heuristic '%s'\n", h);
        } else if (strncmp(opt, "managed_min=", 12) == 0) {
            g_cfg.managed_min = (size_t)strtoull(opt + 12, NULL, 10);
        } else if (strcmp(opt, "statistics") == 0) {
            snprintf(g_cfg.stats_file, sizeof g_cfg.stats_file, "statistics.csv");
        } else if (strncmp(opt, "statistics=", 11) == 0) {
            snprintf(g_cfg.stats_file, sizeof g_cfg.stats_file, "%s", opt + 11);
        } else if (strncmp(opt, "precision=", 10) == 0) {
            const char *p = opt + 10;
            if (strncmp(p, "ozaki", 5) == 0) {
                g_cfg.precision_ozaki = 1;
                if (p[5] == ':') {
                    double t = atof(p + 6);
                    if (t > 0.0) g_cfg.ozaki_tol = t;
                }
            } else if (strcmp(p, "fp64") == 0) {
                g_cfg.precision_ozaki = 0;
            } else {
                fprintf(stderr, "gbxblas: unknown precision '%s'\n", p);
            }
        } else if (strncmp(opt, "serve=", 6) == 0) {
            g_cfg.serve = strcmp(opt + 6, "on") == 0;
        } else if (strncmp(opt, "prefetch=", 9) == 0) {
            g_cfg.prefetch = strcmp(opt + 9, "off") != 0;
        } else if (strncmp(opt, "errors=", 7) == 0) {
            g_cfg.abort_on_error = strcmp(opt + 7, "return") != 0;
        } else if (strncmp(opt, "trace=", 6) == 0) {
            g_cfg.trace = 1;
            snprintf(g_cfg.trace_file, sizeof g_cfg.trace_file, "%s", opt + 6);
        } else {
            fprintf(stderr, "gbxblas: unknown option '%s'. Set BLAS2CUDA_OPTIONS=help.\n", opt);
        }
    }
    free(copy);
}

const gbx_config *gbx_get_config(void)
{
    pthread_once(&g_once, parse);
    return &g_cfg;
}
