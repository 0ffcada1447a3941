/*
 * tracker_prog.c — test program for the allocation interposer
 * (libgbxblas_preload.so), run under LD_PRELOAD by tests/test_tracker.py.
 *
 *   tracker_prog seq        allocate a fixed sequence; print per object:
 *                           "<nth> <managed> <aligned256>"
 *   tracker_prog realloc    realloc/calloc/free semantics on managed objects
 *   tracker_prog threads    8 threads x 20000 malloc/free of random sizes
 *   tracker_prog blas <n>   (GPU) dgemm_ on managed operands; prints the
 *                           placement counters
 *   tracker_prog fwd        dgemm_, dsymm_, ddot_, idamax_ on host arrays
 *                           (run with OBJTRACKER_OPTIONS=blas_libs=...: the
 *                           calls go to that library); prints the results
 *   tracker_prog churn      300000 managed malloc/free pairs with up to 1000
 *                           live objects; prints the side table's use and
 *                           longest probe run
 *   tracker_prog align      posix_memalign / memalign alignment rules
 * Output uses write(2) on a stack buffer so the program itself makes no
 * hidden allocations between the counted ones.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <malloc.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static int (*is_managed)(const void *);
static void (*counters)(uint64_t *, uint64_t *, uint64_t *, uint64_t *);

static void out(const char *fmt, unsigned long long a, unsigned long long b, unsigned long long c)
{
    char buf[128];
    int n = snprintf(buf, sizeof buf, fmt, a, b, c);
    if (write(1, buf, (size_t)n) < 0) _exit(3);
}

static uint64_t nth_now(void)
{
    uint64_t v;
    counters(&v, NULL, NULL, NULL);
    return v;
}

static int seq(void)
{
    static const size_t sizes[] = {16, 300, 4096, 100000, 3 << 20, 64, 1 << 20, 777, 5000, 65536};
    void *p[10];
    for (int i = 0; i < 10; i++) {
        const uint64_t nth = nth_now();
        p[i] = (i % 3 == 2) ? calloc(1, sizes[i]) : malloc(sizes[i]);
        if (!p[i]) return 1;
        memset(p[i], 0x5a, sizes[i]);
        out("%llu %llu %llu\n", (unsigned long long)nth, (unsigned long long)is_managed(p[i]),
            (unsigned long long)(((uintptr_t)p[i] & 255) == 0));
    }
    for (int i = 0; i < 10; i++) free(p[i]);
    uint64_t objs;
    counters(NULL, &objs, NULL, NULL);
    out("objects_after_free %llu %llu %llu\n", objs, 0, 0);
    /* posix_memalign */
    void *q = NULL;
    if (posix_memalign(&q, 128, 10000) != 0) return 2;
    out("memalign %llu %llu %llu\n", (unsigned long long)is_managed(q), ((uintptr_t)q & 127) == 0, 0);
    free(q);
    return 0;
}

static int realloc_case(void)
{
    unsigned char *a = (unsigned char *)calloc(1000, 8);
    int zero = 1;
    for (int i = 0; i < 8000; i++) zero &= a[i] == 0;
    for (int i = 0; i < 8000; i++) a[i] = (unsigned char)i;
    const int m0 = is_managed(a);
    unsigned char *b = (unsigned char *)realloc(a, 100000);
    int same = 1;
    for (int i = 0; i < 8000; i++) same &= b[i] == (unsigned char)i;
    const int m1 = is_managed(b);
    unsigned char *c = (unsigned char *)realloc(b, 100);
    int same2 = 1;
    for (int i = 0; i < 100; i++) same2 &= c[i] == (unsigned char)i;
    out("realloc %llu %llu %llu\n", (unsigned long long)(zero * 100 + m0 * 10 + m1),
        (unsigned long long)(same * 10 + same2), (unsigned long long)is_managed(c));
    /* reuse: a freed block of a size class comes back */
    void *x = malloc(3000);
    free(x);
    void *y = malloc(3000);
    out("reuse %llu %llu %llu\n", (unsigned long long)(x == y), (unsigned long long)is_managed(y), 0);
    free(y);
    free(c);
    void *z = realloc(NULL, 500);
    out("realloc_null %llu %llu %llu\n", (unsigned long long)(z != NULL), 0, 0);
    free(z);
    return 0;
}

static void *worker(void *arg)
{
    uint64_t s = (uint64_t)(uintptr_t)arg * 0x9E3779B97F4A7C15ull + 1;
    void *live[64] = {0};
    for (int it = 0; it < 20000; it++) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const int k = (int)(s % 64);
        if (live[k]) {
            free(live[k]);
            live[k] = NULL;
        } else {
            const size_t n = 1 + (size_t)((s >> 8) % 200000);
            live[k] = malloc(n);
            if (!live[k]) return (void *)1;
            ((char *)live[k])[0] = 1;
            ((char *)live[k])[n - 1] = 2;
        }
    }
    for (int k = 0; k < 64; k++) free(live[k]);
    return NULL;
}

static int threads(void)
{
    pthread_t t[8];
    uint64_t objs0;
    counters(NULL, &objs0, NULL, NULL);
    for (int i = 0; i < 8; i++) pthread_create(&t[i], NULL, worker, (void *)(uintptr_t)(i + 1));
    int bad = 0;
    for (int i = 0; i < 8; i++) {
        void *r;
        pthread_join(t[i], &r);
        bad |= r != NULL;
    }
    /* the C library keeps small per-thread records (thread vectors) of the
     * joined threads; everything the workers allocated must be back */
    uint64_t objs, bytes;
    counters(NULL, &objs, &bytes, NULL);
    out("threads %llu %llu %llu\n", (unsigned long long)bad, objs - objs0, bytes);
    return bad;
}

static int many(void)
{
    static void *p[2000];
    unsigned long long managed = 0;
    for (int i = 0; i < 2000; i++) {
        p[i] = malloc(1024);
        managed += (unsigned long long)is_managed(p[i]);
    }
    for (int i = 0; i < 2000; i++) free(p[i]);
    out("many %llu %llu %llu\n", managed, 2000, 0);
    return 0;
}

typedef void (*dgemm_fn)(const char *, const char *, const int *, const int *, const int *, const double *,
                         const double *, const int *, const double *, const int *, const double *, double *,
                         const int *);

static int blas(int n)
{
    dgemm_fn dgemm = (dgemm_fn)dlsym(RTLD_DEFAULT, "dgemm_");
    void (*stats)(uint64_t *, uint64_t *, uint64_t *, uint64_t *, uint64_t *) =
        (void (*)(uint64_t *, uint64_t *, uint64_t *, uint64_t *, uint64_t *))dlsym(RTLD_DEFAULT, "gbx_stats");
    double *a = (double *)malloc(sizeof(double) * n * n);
    double *b = (double *)malloc(sizeof(double) * n * n);
    double *c = (double *)malloc(sizeof(double) * n * n);
    for (int i = 0; i < n * n; i++) { a[i] = (i % 7) - 3; b[i] = (i % 5) - 2; c[i] = 0; }
    const double one = 1.0, zero = 0.0;
    dgemm("N", "N", &n, &n, &n, &one, a, &n, b, &n, &zero, c, &n);
    /* check one entry on the host */
    double want = 0;
    for (int l = 0; l < n; l++) want += a[l * n + 1] * b[2 * n + l];
    uint64_t calls, hits, misses, h2d, d2h;
    stats(&calls, &hits, &misses, &h2d, &d2h);
    out("blas managed %llu %llu %llu\n", (unsigned long long)is_managed(a), (unsigned long long)is_managed(c),
        (unsigned long long)(c[2 * n + 1] == want));
    out("blas stats %llu %llu %llu\n", (unsigned long long)hits, (unsigned long long)misses,
        (unsigned long long)(h2d + d2h));
    free(a);
    free(b);
    free(c);
    return 0;
}

/* six 8x8 matrices; dgemm_ names objects 1, 3 (through an interior pointer)
 * and 4; prints "<index> <managed>" for each object.  Without a GPU the
 * call reports its device failure and returns (errors=return); the trace
 * lines are written before that. */
static int blas_note(void)
{
    dgemm_fn dgemm = (dgemm_fn)dlsym(RTLD_DEFAULT, "dgemm_");
    double *p[6];
    for (int i = 0; i < 6; i++) {
        p[i] = (double *)malloc(sizeof(double) * 80);
        for (int j = 0; j < 80; j++) p[i][j] = 1.0;
    }
    int n = 8, ld = 8;
    const double one = 1.0, zero = 0.0;
    dgemm("N", "N", &n, &n, &n, &one, p[1], &ld, p[3] + 8, &ld, &zero, p[4], &ld);
    for (int i = 0; i < 6; i++) out("%llu %llu %llu\n", (unsigned long long)i, (unsigned long long)is_managed(p[i]), 0);
    for (int i = 0; i < 6; i++) free(p[i]);
    return 0;
}

typedef void (*dsymm_fn)(const char *, const char *, const int *, const int *, const double *, const double *,
                         const int *, const double *, const int *, const double *, double *, const int *);

static int fwd(void)
{
    dgemm_fn dgemm = (dgemm_fn)dlsym(RTLD_DEFAULT, "dgemm_");
    dsymm_fn dsymm = (dsymm_fn)dlsym(RTLD_DEFAULT, "dsymm_");
    double (*ddot)(const int *, const double *, const int *, const double *, const int *) =
        (double (*)(const int *, const double *, const int *, const double *, const int *))dlsym(RTLD_DEFAULT, "ddot_");
    int (*idamax)(const int *, const double *, const int *) =
        (int (*)(const int *, const double *, const int *))dlsym(RTLD_DEFAULT, "idamax_");
    const int n = 4, one_i = 1;
    double *a = (double *)malloc(sizeof(double) * 16), *b = (double *)malloc(sizeof(double) * 16);
    double *c = (double *)malloc(sizeof(double) * 16);
    for (int i = 0; i < 16; i++) { a[i] = i + 1; b[i] = (i % 3) - 1; c[i] = 1; }
    const double one = 1.0, half = 0.5;
    dgemm("N", "N", &n, &n, &n, &one, a, &n, b, &n, &half, c, &n);
    double want = 0.5;
    for (int l = 0; l < n; l++) want += a[l * n + 2] * b[3 * n + l];   /* C(2,3) */
    out("dgemm %llu %llu %llu\n", (unsigned long long)(c[3 * n + 2] == want), 0, 0);
    for (int i = 0; i < 16; i++) c[i] = 0;
    dsymm("L", "U", &n, &n, &one, a, &n, b, &n, &one, c, &n);
    want = 0;   /* C(1,0) with A symmetric from its upper triangle */
    for (int l = 0; l < n; l++) want += (l >= 1 ? a[l * n + 1] : a[1 * n + l]) * b[0 * n + l];
    out("dsymm %llu %llu %llu\n", (unsigned long long)(c[1] == want), 0, 0);
    const double d = ddot(&n, a, &one_i, a, &one_i);
    out("ddot %llu %llu %llu\n", (unsigned long long)d, 0, 0);     /* 1+4+9+16 = 30 */
    a[2] = -99;
    out("idamax %llu %llu %llu\n", (unsigned long long)idamax(&n, a, &one_i), 0, 0);
    free(a);
    free(b);
    free(c);
    return 0;
}

static int churn(void)
{
    void (*table)(uint64_t *, uint64_t *) = (void (*)(uint64_t *, uint64_t *))dlsym(RTLD_DEFAULT,
                                                                                   "gbx_tracker_table_stats");
    if (!table) return 7;
    enum { LIVE = 1000, ROUNDS = 300000 };
    void *live[LIVE] = {0};
    uint64_t x = 88172645463325252ull, bad = 0;
    for (int r = 0; r < ROUNDS; r++) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        const int i = (int)(x % LIVE);
        if (live[i]) {
            if (!is_managed(live[i])) bad++;
            free(live[i]);
        }
        live[i] = malloc(64 + (x >> 40) % 4000);
        /* a pointer that is in the managed range but is not an object start */
        if (live[i] && is_managed((char *)live[i] + 8)) bad++;
    }
    uint64_t used, longest;
    table(&used, &longest);
    int count = 0;
    for (int i = 0; i < LIVE; i++) count += live[i] != NULL;
    out("live %llu %llu %llu\n", (unsigned long long)count, (unsigned long long)used, (unsigned long long)bad);
    for (int i = 0; i < LIVE; i++) free(live[i]);
    table(&used, &longest);
    out("after %llu %llu %llu\n", (unsigned long long)used, (unsigned long long)longest, 0);
    return 0;
}

static int align_case(void)
{
    void *p = NULL;
    const int e24 = posix_memalign(&p, 24, 100), e4 = posix_memalign(&p, 4, 100);
    void *q = NULL;
    const int ok = posix_memalign(&q, 64, 100);
    out("posix_memalign %llu %llu %llu\n", (unsigned long long)e24, (unsigned long long)e4,
        (unsigned long long)(ok == 0 && ((uintptr_t)q & 63) == 0));
    void *m = memalign(48, 100);   /* rounded up to 64 */
    out("memalign %llu %llu %llu\n", (unsigned long long)(m != NULL), (unsigned long long)(((uintptr_t)m & 63) == 0), 0);
    free(q);
    free(m);
    return 0;
}

int main(int argc, char **argv)
{
    is_managed = (int (*)(const void *))dlsym(RTLD_DEFAULT, "gbx_tracker_is_managed");
    counters = (void (*)(uint64_t *, uint64_t *, uint64_t *, uint64_t *))dlsym(RTLD_DEFAULT,
                                                                               "gbx_tracker_counters");
    if (!is_managed || !counters) {
        out("interposer not loaded %llu %llu %llu\n", 0, 0, 0);
        return 9;
    }
    if (argc < 2) return 8;
    if (!strcmp(argv[1], "seq")) return seq();
    if (!strcmp(argv[1], "realloc")) return realloc_case();
    if (!strcmp(argv[1], "threads")) return threads();
    if (!strcmp(argv[1], "many")) return many();
    if (!strcmp(argv[1], "blas_note")) return blas_note();
    if (!strcmp(argv[1], "blas")) return blas(argc > 2 ? atoi(argv[2]) : 512);
    if (!strcmp(argv[1], "fwd")) return fwd();
    if (!strcmp(argv[1], "churn")) return churn();
    if (!strcmp(argv[1], "align")) return align_case();
    return 8;
}
