/*
 * preload_tracker.c — allocation interposer of libgbxblas_preload.so.
 *
 * Replaces the reference's object tracker (lib/obj_tracker.c:789-982
 * malloc/calloc/realloc/free, placement policy 226-242, oracle file
 * lib/oracle.c:14-73): chosen heap allocations of the application are served
 * from CUDA managed memory, so BLAS operands that live there need no copy
 * (the BLAS layer treats them as resident and prefetches them).
 *
 * Same contract: BLAS2CUDA_OPTIONS=heuristic=false|true|random|oracle:<file>
 * decides, per counted malloc/calloc (the n-th allocation, 0-based, counting
 * malloc, calloc and realloc calls made by the application), whether the
 * object is managed; an oracle file holds "D #<n> ..." (managed) and
 * "H #<n> ..." (host) records.  Differences, all deliberate:
 *   * managed objects come from a pool: 64 MiB managed slabs cut into
 *     power-of-two blocks (256 B .. 1 MiB), larger objects get their own
 *     allocation; metadata lives in a side table, so pointers keep 256-byte
 *     alignment (the reference's inline size header returns base+8,
 *     blas2cuda.c:145-147);
 *   * slabs are advised to prefer the GPU and to be accessible by the host;
 *   * the decision uses the object's own index (the reference passes the
 *     already-incremented counter, obj_tracker.c:824), the oracle bitset is
 *     sized in bytes correctly (oracle.c:61-62), and heuristic=random is a
 *     fair coin (random()/LONG_MAX > 0.5 is never true on LP64,
 *     obj_tracker.c:236);
 *   * managed_min=<bytes> keeps smaller objects on the host (default 0);
 *   * if managed memory cannot be had, the object is served from the host
 *     heap (the BLAS layer then stages it) instead of aborting;
 *   * statistics[=<file>] writes the call/placement counters at exit (the
 *     reference always writes statistics.csv, blas2cuda.c:266-273).
 * Allocations made by the CUDA libraries and by this library itself (its
 * text contains the statically linked CUDA runtime) bypass tracking, as the
 * reference does for libcuda/nvidia (blas2cuda.c:232, obj_tracker.c:409-424).
 */
#define _GNU_SOURCE
#include "gbx_internal.h"
#include "../../include/gbxblas_f77.h"

#include <dlfcn.h>
#include <errno.h>
#include <fcntl.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

void *gbx_tracker_slab_alloc(size_t bytes, int (*host_alloc)(void **, size_t, size_t));
void gbx_tracker_slab_free(void *p, void (*host_free)(void *));

typedef void *(*fn_malloc)(size_t);
typedef void *(*fn_calloc)(size_t, size_t);
typedef void *(*fn_realloc)(void *, size_t);
typedef void (*fn_free)(void *);
typedef int (*fn_posix_memalign)(void **, size_t, size_t);
typedef size_t (*fn_usable)(void *);

static fn_malloc r_malloc;
static fn_calloc r_calloc;
static fn_realloc r_realloc;
static fn_free r_free;
static fn_posix_memalign r_posix_memalign;
static fn_usable r_usable;

static __thread int t_in;   /* inside the interposer: pass through */

/* ---- bootstrap arena for allocations made while dlsym resolves ---------- */
static _Alignas(64) char g_boot[1 << 16];
static atomic_size_t g_boot_used;
static atomic_int g_ready;  /* 0 unresolved, 1 resolving, 2 ready */

static int in_boot(const void *p)
{
    return (const char *)p >= g_boot && (const char *)p < g_boot + sizeof g_boot;
}

/* sizes of the first bootstrap allocations (OBJTRACKER_OPTIONS=debug_uninit) */
#define BOOT_LOG 64
static size_t g_boot_log[BOOT_LOG];
static atomic_int g_boot_calls;

static void *boot_alloc(size_t n)
{
    const int k = atomic_fetch_add(&g_boot_calls, 1);
    if (k < BOOT_LOG) g_boot_log[k] = n;
    n = (n + 63) & ~(size_t)63;
    size_t off = atomic_fetch_add(&g_boot_used, n);
    if (off + n > sizeof g_boot) return NULL;
    return g_boot + off;
}

static void resolve(void)
{
    int expect = 0;
    if (!atomic_compare_exchange_strong(&g_ready, &expect, 1)) {
        while (atomic_load(&g_ready) != 2) { /* another thread is resolving */ }
        return;
    }
    r_malloc = (fn_malloc)dlsym(RTLD_NEXT, "malloc");
    r_calloc = (fn_calloc)dlsym(RTLD_NEXT, "calloc");
    r_realloc = (fn_realloc)dlsym(RTLD_NEXT, "realloc");
    r_free = (fn_free)dlsym(RTLD_NEXT, "free");
    r_posix_memalign = (fn_posix_memalign)dlsym(RTLD_NEXT, "posix_memalign");
    r_usable = (fn_usable)dlsym(RTLD_NEXT, "malloc_usable_size");
    atomic_store(&g_ready, 2);
}

static inline int ready(void)
{
    if (atomic_load_explicit(&g_ready, memory_order_acquire) == 2) return 1;
    if (atomic_load(&g_ready) == 1) return 0;   /* dlsym in progress: bootstrap */
    resolve();
    return atomic_load(&g_ready) == 2;
}

/* ---- excluded text ranges (CUDA libraries and this library) ------------- */
#define MAX_EXCL 128
static uintptr_t g_excl_lo[MAX_EXCL], g_excl_hi[MAX_EXCL];
static atomic_int g_nexcl;
static pthread_mutex_t g_excl_mu = PTHREAD_MUTEX_INITIALIZER;

static int excluded(const void *ret)
{
    const uintptr_t a = (uintptr_t)ret;
    const int n = atomic_load_explicit(&g_nexcl, memory_order_acquire);
    for (int i = 0; i < n; i++)
        if (a >= g_excl_lo[i] && a < g_excl_hi[i]) return 1;
    return 0;
}

static int path_excluded(const char *path)
{
    return strstr(path, "libcuda") || strstr(path, "libnvidia") || strstr(path, "libgbxblas") ||
           strstr(path, "libcudart") || strstr(path, "libnvrtc");
}

/* Rescan /proc/self/maps with raw reads (no allocation). */
void gbx_tracker_refresh(void)
{
    static char buf[1 << 18];
    pthread_mutex_lock(&g_excl_mu);
    int fd = open("/proc/self/maps", O_RDONLY | O_CLOEXEC);
    if (fd >= 0) {
        size_t len = 0;
        ssize_t r;
        while (len < sizeof buf - 1 && (r = read(fd, buf + len, sizeof buf - 1 - len)) > 0) len += (size_t)r;
        close(fd);
        buf[len] = '\0';
        int n = 0;
        for (char *line = buf; line && *line && n < MAX_EXCL;) {
            char *nl = strchr(line, '\n');
            if (nl) *nl = '\0';
            unsigned long lo, hi;
            char perms[8];
            if (sscanf(line, "%lx-%lx %7s", &lo, &hi, perms) == 3 && perms[2] == 'x') {
                const char *path = strchr(line, '/');
                if (path && path_excluded(path)) {
                    g_excl_lo[n] = lo;
                    g_excl_hi[n] = hi;
                    n++;
                }
            }
            line = nl ? nl + 1 : NULL;
        }
        atomic_store_explicit(&g_nexcl, n, memory_order_release);
    }
    pthread_mutex_unlock(&g_excl_mu);
}

/* ---- placement policy ------------------------------------------------------ */
static int g_tracking;
static atomic_ullong g_nth;
static uint8_t *g_dec;           /* oracle bitset */
static uint64_t g_ndec;          /* number of decision bits */
static size_t g_min_bytes;
static atomic_ullong g_rng = 0x9E3779B97F4A7C15ull;
static atomic_ullong g_managed_objects, g_managed_bytes, g_managed_fail;

static int coin(void)
{
    /* SplitMix64 step on a shared state: a fair coin per decision */
    uint64_t z = atomic_fetch_add(&g_rng, 0x9E3779B97F4A7C15ull) + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (int)((z ^ (z >> 31)) >> 63);
}

static int decide(uint64_t nth, size_t bytes)
{
    if (bytes < g_min_bytes) return 0;
    switch (gbx_get_config()->heuristic) {
    case 1: return 1;
    case 2: return coin();
    case 3: return nth < g_ndec && ((g_dec[nth >> 3] >> (nth & 7)) & 1u);
    default: return 0;
    }
}

/* Parse "D #<n> ..." / "H #<n> ..." records (analyze_trace.py:40,95-97). */
int gbx_tracker_load_oracle(const char *path)
{
    FILE *f = fopen(path, "r");
    if (!f) return 0;
    char line[512];
    uint64_t cap = 0, maxn = 0;
    uint8_t *bits = NULL;
    while (fgets(line, sizeof line, f)) {
        char c;
        unsigned long long n;
        if (sscanf(line, " %c #%llu", &c, &n) != 2 || (c != 'D' && c != 'H')) continue;
        if (n + 1 > maxn) maxn = n + 1;
        if ((n >> 3) >= cap) {
            uint64_t ncap = cap ? cap : 1024;
            while ((n >> 3) >= ncap) ncap *= 2;
            uint8_t *nb = (uint8_t *)r_realloc(bits, ncap);
            if (!nb) { fclose(f); r_free(bits); return 0; }
            memset(nb + cap, 0, ncap - cap);
            bits = nb;
            cap = ncap;
        }
        if (c == 'D') bits[n >> 3] |= (uint8_t)(1u << (n & 7));
        else bits[n >> 3] &= (uint8_t)~(1u << (n & 7));
    }
    fclose(f);
    g_dec = bits;
    g_ndec = maxn;
    return 1;
}

/* ---- managed pool ------------------------------------------------------------ */
#define NCLASS 13                      /* 256 B << 0..12 = 256 B .. 1 MiB */
#define SLAB_BYTES ((size_t)64 << 20)
#define LARGE_ALIGN ((size_t)2 << 20)
#define TAB_BITS 20
#define TAB_SIZE ((size_t)1 << TAB_BITS)

struct cls {
    char *cur, *end;
    void **freelist;
    size_t nfree, cap;
};
struct ent {
    uintptr_t p;
    size_t size;
    int cls;
};
static struct cls g_cls[NCLASS];
static struct ent g_tab[TAB_SIZE];
static size_t g_tab_used;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static atomic_uintptr_t g_env_lo = UINTPTR_MAX, g_env_hi = 0;

static size_t slot(uintptr_t p) { return (size_t)((p >> 8) * 0x9E3779B97F4A7C15ull >> (64 - TAB_BITS)); }

static struct ent *tab_find(uintptr_t p)
{
    for (size_t i = slot(p), k = 0; k < TAB_SIZE; i = (i + 1) & (TAB_SIZE - 1), k++) {
        if (g_tab[i].p == p) return &g_tab[i];
        if (g_tab[i].p == 0) return NULL;
    }
    return NULL;
}

static int tab_insert(uintptr_t p, size_t size, int cls)
{
    if (g_tab_used >= TAB_SIZE - TAB_SIZE / 8) return 0;
    for (size_t i = slot(p);; i = (i + 1) & (TAB_SIZE - 1)) {
        if (g_tab[i].p == 0) {
            g_tab[i].p = p;
            g_tab[i].size = size;
            g_tab[i].cls = cls;
            g_tab_used++;
            return 1;
        }
    }
}

/* Removes e by backward-shift deletion (Knuth, TAOCP vol. 3, 6.4,
 * Algorithm R): later entries of the same probe run move into the hole
 * unless their home slot lies cyclically in (hole, their slot].  No
 * tombstones are left, so lookups stay short under any allocate/free churn
 * and every run still ends at an empty slot. */
static void tab_erase(struct ent *e)
{
    const size_t mask = TAB_SIZE - 1;
    size_t hole = (size_t)(e - g_tab);
    g_tab[hole].p = 0;
    g_tab_used--;
    for (size_t j = (hole + 1) & mask; g_tab[j].p != 0; j = (j + 1) & mask) {
        const size_t home = slot(g_tab[j].p);
        /* the entry may stay iff home is in the cyclic interval (hole, j] */
        const int stays = hole <= j ? (home > hole && home <= j) : (home > hole || home <= j);
        if (stays) continue;
        g_tab[hole] = g_tab[j];
        g_tab[j].p = 0;
        hole = j;
    }
}

static void envelope(uintptr_t lo, uintptr_t hi)
{
    uintptr_t cur = atomic_load(&g_env_lo);
    while (lo < cur && !atomic_compare_exchange_weak(&g_env_lo, &cur, lo)) {}
    cur = atomic_load(&g_env_hi);
    while (hi > cur && !atomic_compare_exchange_weak(&g_env_hi, &cur, hi)) {}
}

static int class_of(size_t n)
{
    int c = 0;
    size_t b = 256;
    while (b < n) { b <<= 1; c++; }
    return c;
}

/* caller holds g_mu */
static void *pool_alloc(size_t n)
{
    void *p = NULL;
    int c = -1;
    if (n > ((size_t)256 << (NCLASS - 1))) {
        size_t sz = (n + LARGE_ALIGN - 1) & ~(LARGE_ALIGN - 1);
        p = gbx_tracker_slab_alloc(sz, r_posix_memalign);
        if (!p) return NULL;
        envelope((uintptr_t)p, (uintptr_t)p + sz);
    } else {
        c = class_of(n);
        struct cls *k = &g_cls[c];
        const size_t bs = (size_t)256 << c;
        if (k->nfree) {
            p = k->freelist[--k->nfree];
        } else {
            if (!k->cur || k->cur + bs > k->end) {
                char *s = (char *)gbx_tracker_slab_alloc(SLAB_BYTES, r_posix_memalign);
                if (!s) return NULL;
                envelope((uintptr_t)s, (uintptr_t)s + SLAB_BYTES);
                k->cur = s;
                k->end = s + SLAB_BYTES;
            }
            p = k->cur;
            k->cur += bs;
        }
    }
    if (!tab_insert((uintptr_t)p, n, c)) {
        if (c < 0) gbx_tracker_slab_free(p, r_free);
        else {
            struct cls *k = &g_cls[c];
            if (k->nfree < k->cap) k->freelist[k->nfree++] = p;
        }
        return NULL;
    }
    atomic_fetch_add(&g_managed_objects, 1);
    atomic_fetch_add(&g_managed_bytes, n);
    return p;
}

/* caller holds g_mu; e was found in the table */
static void pool_free(struct ent *e)
{
    void *p = (void *)e->p;
    const int c = e->cls;
    atomic_fetch_sub(&g_managed_objects, 1);
    atomic_fetch_sub(&g_managed_bytes, e->size);
    tab_erase(e);
    if (c < 0) {
        gbx_tracker_slab_free(p, r_free);
        return;
    }
    struct cls *k = &g_cls[c];
    if (k->nfree == k->cap) {
        size_t ncap = k->cap ? 2 * k->cap : 1024;
        void **nf = (void **)r_realloc(k->freelist, ncap * sizeof(void *));
        if (!nf) return;   /* block leaks into the slab; still correct */
        k->freelist = nf;
        k->cap = ncap;
    }
    k->freelist[k->nfree++] = p;
}

static int maybe_managed(const void *p)
{
    const uintptr_t a = (uintptr_t)p;
    return a >= atomic_load_explicit(&g_env_lo, memory_order_relaxed) &&
           a < atomic_load_explicit(&g_env_hi, memory_order_relaxed);
}

/* managed size of p, or 0 when p is not a managed object */
static size_t managed_size(const void *p)
{
    if (!p || !maybe_managed(p)) return 0;
    pthread_mutex_lock(&g_mu);
    struct ent *e = tab_find((uintptr_t)p);
    size_t s = e ? (e->size ? e->size : 1) : 0;
    pthread_mutex_unlock(&g_mu);
    return s;
}

static void *managed_alloc(size_t n)
{
    pthread_mutex_lock(&g_mu);
    void *p = pool_alloc(n);
    pthread_mutex_unlock(&g_mu);
    if (!p) atomic_fetch_add(&g_managed_fail, 1);
    return p;
}

static int managed_release(void *p)
{
    if (!maybe_managed(p)) return 0;
    pthread_mutex_lock(&g_mu);
    struct ent *e = tab_find((uintptr_t)p);
    if (e) pool_free(e);
    pthread_mutex_unlock(&g_mu);
    return e != NULL;
}

/* ---- OBJTRACKER_OPTIONS --------------------------------------------------------
 * The reference's standalone tracker options (lib/obj_tracker.c:246-321),
 * same variable and syntax (chained with ';'), for the trace mode here:
 *   help              print these options
 *   only_print_calls  write only the BLAS-call lines ("C"): each names the
 *                     object's allocation index, size and address, which is
 *                     all the decision file needs
 *   debug_uninit      report the allocations served before the interposer
 *                     was ready (from its bootstrap arena)
 *   blas_libs=a,b,... load these libraries, in order; every Fortran BLAS
 *                     call is then forwarded to the first of them that
 *                     defines the routine, so the traced program computes on
 *                     the CPU BLAS as it would without this library
 *                     (lib/blas_tracker.c:65-93, 100-116) */
static int g_only_calls, g_debug_uninit;
#define MAX_BLAS_LIBS 16
static void *g_blas_handles[MAX_BLAS_LIBS];
static int g_nblas;

static const char objtracker_help[] =
    "object tracker options (set OBJTRACKER_OPTIONS, chain with ';'):\n"
    "   help               -- print this help\n"
    "   only_print_calls   -- trace only the BLAS calls that use objects\n"
    "   blas_libs=<a,b,..> -- comma-separated libraries to load, in order; the\n"
    "                         BLAS calls are forwarded to the first that defines\n"
    "                         each routine (the traced program runs on that BLAS)\n"
    "   debug_uninit       -- report allocations made before the tracker was ready\n";

void gbx_tracker_print_options(void)
{
    if (write(STDERR_FILENO, objtracker_help, sizeof objtracker_help - 1) < 0) { /* nothing to do */ }
}

/* caller has t_in set (allocations pass through) */
static void parse_objtracker_options(void)
{
    const char *env = getenv("OBJTRACKER_OPTIONS");
    if (!env || !*env) return;
    char *copy = strdup(env);
    if (!copy) return;
    char *save = NULL;
    int helped = 0;
    for (char *opt = strtok_r(copy, ";", &save); opt; opt = strtok_r(NULL, ";", &save)) {
        if (strcmp(opt, "help") == 0) {
            if (!helped) gbx_tracker_print_options();
            helped = 1;
        } else if (strcmp(opt, "only_print_calls") == 0) {
            g_only_calls = 1;
        } else if (strcmp(opt, "debug_uninit") == 0) {
            g_debug_uninit = 1;
        } else if (strncmp(opt, "blas_libs=", 10) == 0) {
            char *save2 = NULL;
            for (char *lib = strtok_r(opt + 10, ",", &save2); lib; lib = strtok_r(NULL, ",", &save2)) {
                if (g_nblas == MAX_BLAS_LIBS) {
                    fprintf(stderr, "objtracker: at most %d BLAS libraries; '%s' ignored\n", MAX_BLAS_LIBS, lib);
                    continue;
                }
                void *h = dlopen(lib, RTLD_NOW | RTLD_LOCAL);
                if (!h) {
                    fprintf(stderr, "objtracker: dlopen(%s): %s\n", lib, dlerror());
                    abort();   /* the reference aborts too: the run would not be the one asked for */
                }
                g_blas_handles[g_nblas++] = h;
            }
            if (!g_nblas) fprintf(stderr, "objtracker: blas_libs= names no library. Set OBJTRACKER_OPTIONS=help.\n");
        } else {
            fprintf(stderr, "objtracker: unknown option '%s'. Set OBJTRACKER_OPTIONS=help.\n", opt);
        }
    }
    free(copy);
}

/* Forwarding target of a Fortran BLAS routine (NULL: run it here).  Looked
 * up once per name in the blas_libs= libraries, in order. */
#define FWD_CACHE 256
static struct { const char *name; void *fn; } g_fwd[FWD_CACHE];
static atomic_int g_nfwd;
static pthread_mutex_t g_fwd_mu = PTHREAD_MUTEX_INITIALIZER;

void *gbx_tracker_forward(const char *sym)
{
    if (!g_nblas) return NULL;
    int n = atomic_load_explicit(&g_nfwd, memory_order_acquire);
    for (int i = 0; i < n; i++)
        if (g_fwd[i].name == sym || strcmp(g_fwd[i].name, sym) == 0) return g_fwd[i].fn;
    const int saved = t_in;
    t_in = 1;
    pthread_mutex_lock(&g_fwd_mu);
    void *fn = NULL;
    n = atomic_load(&g_nfwd);
    for (int i = 0; i < n && !fn; i++)
        if (strcmp(g_fwd[i].name, sym) == 0) fn = g_fwd[i].fn;
    for (int i = 0; i < g_nblas && !fn; i++) fn = dlsym(g_blas_handles[i], sym);
    if (!fn) fprintf(stderr, "objtracker: no library in blas_libs= defines '%s'; it runs on the GPU\n", sym);
    if (n < FWD_CACHE) {
        g_fwd[n].name = sym;
        g_fwd[n].fn = fn;
        atomic_store_explicit(&g_nfwd, n + 1, memory_order_release);
    }
    pthread_mutex_unlock(&g_fwd_mu);
    t_in = saved;
    return fn;
}

/* ---- trace mode (trace=<file>): the producer side of the allocation-file
 * workflow.  Same line grammar as the reference's standalone tracker
 * (obj_tracker.c:426-483, blas_tracker.c:24-31):
 *   T #<nth> [<ptr>] fun=[malloc] reqsize=[<n>] tid=[<tid>] time=[<s>s+<ns>ns] uid=[<uid>]
 *   U #<nth> [<ptr>] fun=[free] ...         (object freed)
 *   C #<nth> [<ptr>] fun=[dgemm_] ...       (a BLAS call names the object)
 * analyze_trace.py turns it into the H/D decision file of heuristic=oracle.
 * Every counted allocation is kept in a search tree keyed by address range,
 * so interior pointers passed to BLAS resolve to their object. */
#include <search.h>
#include <sys/syscall.h>
#include <time.h>

struct tobj {
    uintptr_t base;
    size_t size;
    uint64_t nth, uid;
    const char *fun;
};
static int g_trace_fd = -1;
static void *g_troot;
static atomic_ullong g_uid;
static pthread_mutex_t g_tmu = PTHREAD_MUTEX_INITIALIZER;

static int tcmp(const void *a, const void *b)
{
    const struct tobj *x = (const struct tobj *)a, *y = (const struct tobj *)b;
    /* ranges that overlap compare equal: a 1-byte probe finds its container */
    if (x->base + (x->size ? x->size : 1) <= y->base) return -1;
    if (y->base + (y->size ? y->size : 1) <= x->base) return 1;
    return 0;
}

static void trace_line(char c, const struct tobj *o, const char *fun)
{
    if (g_only_calls && c != 'C') return;
    char buf[256];
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC_RAW, &ts);
    const long tid = (long)syscall(SYS_gettid);
    int n = snprintf(buf, sizeof buf, "%c #%llu [%p] fun=[%s] reqsize=[%zu] tid=[%ld] time=[%llds+%ldns] uid=[%llu]\n",
                     c, (unsigned long long)o->nth, (void *)o->base, fun, o->size, tid, (long long)ts.tv_sec,
                     ts.tv_nsec, (unsigned long long)o->uid);
    if (n > 0 && write(g_trace_fd, buf, (size_t)(n < (int)sizeof buf ? n : (int)sizeof buf - 1)) < 0) { /* ignore */ }
}

/* caller has t_in set */
static void trace_alloc(void *p, size_t n, uint64_t nth, const char *fun)
{
    if (g_trace_fd < 0 || !p) return;
    struct tobj *o = (struct tobj *)r_malloc(sizeof *o);
    if (!o) return;
    o->base = (uintptr_t)p;
    o->size = n;
    o->nth = nth;
    o->uid = atomic_fetch_add(&g_uid, 1);
    o->fun = fun;
    pthread_mutex_lock(&g_tmu);
    void *r = tsearch(o, &g_troot, tcmp);
    if (r && *(struct tobj **)r == o) trace_line('T', o, fun);
    else r_free(o);   /* stale overlapping record: keep the tree consistent */
    pthread_mutex_unlock(&g_tmu);
}

/* caller has t_in set */
static void trace_free(void *p)
{
    if (g_trace_fd < 0 || !p) return;
    struct tobj key = {(uintptr_t)p, 1, 0, 0, NULL};
    pthread_mutex_lock(&g_tmu);
    void *r = tfind(&key, &g_troot, tcmp);
    if (r) {
        struct tobj *o = *(struct tobj **)r;
        if (o->base == (uintptr_t)p) {
            trace_line('U', o, "free");
            tdelete(o, &g_troot, tcmp);
            r_free(o);
        }
    }
    pthread_mutex_unlock(&g_tmu);
}

void gbx_tracker_note(const char *fun, const void *ptr)
{
    if (g_trace_fd < 0 || !ptr) return;
    const int saved = t_in;
    t_in = 1;
    struct tobj key = {(uintptr_t)ptr, 1, 0, 0, NULL};
    pthread_mutex_lock(&g_tmu);
    void *r = tfind(&key, &g_troot, tcmp);
    if (r) trace_line('C', *(struct tobj **)r, fun);
    pthread_mutex_unlock(&g_tmu);
    t_in = saved;
}

/* ---- the interposed entry points -------------------------------------------- */
static inline int bypass(const void *ret)
{
    return t_in || !g_tracking || excluded(ret);
}

void *malloc(size_t n)
{
    if (!ready()) return boot_alloc(n);
    if (bypass(__builtin_return_address(0))) return r_malloc(n);
    const uint64_t nth = atomic_fetch_add(&g_nth, 1);
    t_in = 1;
    void *p = (n && decide(nth, n)) ? managed_alloc(n) : NULL;
    if (!p) p = r_malloc(n);
    trace_alloc(p, n, nth, "malloc");
    t_in = 0;
    return p;
}

void *calloc(size_t nm, size_t sz)
{
    if (!ready()) {
        if (sz && nm > SIZE_MAX / sz) return NULL;
        void *p = boot_alloc(nm * sz);
        if (p) memset(p, 0, nm * sz);
        return p;
    }
    if (bypass(__builtin_return_address(0))) return r_calloc(nm, sz);
    const uint64_t nth = atomic_fetch_add(&g_nth, 1);
    if (sz && nm > SIZE_MAX / sz) {
        errno = ENOMEM;
        return NULL;
    }
    const size_t n = nm * sz;
    t_in = 1;
    void *p = (n && decide(nth, n)) ? managed_alloc(n) : NULL;
    if (p) memset(p, 0, n);
    else p = r_calloc(nm, sz);
    trace_alloc(p, n, nth, "calloc");
    t_in = 0;
    return p;
}

void free(void *p)
{
    if (!p || in_boot(p)) return;
    if (!ready()) return;
    if (g_trace_fd >= 0 && !t_in) {
        t_in = 1;
        trace_free(p);
        t_in = 0;
    }
    if (managed_release(p)) return;
    r_free(p);
}

void *realloc(void *p, size_t n)
{
    if (!ready() || in_boot(p)) {
        void *q = ready() ? malloc(n) : boot_alloc(n);
        if (q && p) {
            const size_t avail = (size_t)(g_boot + sizeof g_boot - (char *)p);
            memcpy(q, p, n < avail ? n : avail);
        }
        return q;
    }
    const size_t old = managed_size(p);
    const int counted = !bypass(__builtin_return_address(0));
    const uint64_t nth = counted ? atomic_fetch_add(&g_nth, 1) : 0;
    if (!old) {
        if (!counted || g_trace_fd < 0) return r_realloc(p, n);
        t_in = 1;
        trace_free(p);
        void *q = r_realloc(p, n);
        trace_alloc(q, n, nth, "realloc");
        t_in = 0;
        return q;
    }
    if (counted && g_trace_fd >= 0) {
        t_in = 1;
        trace_free(p);
        t_in = 0;
    }
    if (n == 0) {
        managed_release(p);
        return NULL;
    }
    /* a managed object stays managed */
    const int saved = t_in;
    t_in = 1;
    void *q = managed_alloc(n);
    if (!q) q = r_malloc(n);
    if (q && counted) trace_alloc(q, n, nth, "realloc");
    t_in = saved;
    if (!q) return NULL;
    memcpy(q, p, old < n ? old : n);
    managed_release(p);
    return q;
}

int posix_memalign(void **out, size_t align, size_t n)
{
    /* POSIX: the alignment must be a power of two multiple of sizeof(void *) */
    if (align < sizeof(void *) || (align & (align - 1)) != 0) return EINVAL;
    if (!ready()) {
        void *p = boot_alloc(n + align);
        if (!p) return ENOMEM;
        *out = (void *)(((uintptr_t)p + align - 1) & ~(uintptr_t)(align - 1));
        return 0;
    }
    if (!bypass(__builtin_return_address(0)) && align <= 256 && n &&
        gbx_get_config()->heuristic == 1 && n >= g_min_bytes) {
        t_in = 1;
        void *p = managed_alloc(n);
        t_in = 0;
        if (p) {
            *out = p;
            return 0;
        }
    }
    return r_posix_memalign(out, align, n);
}

void *aligned_alloc(size_t align, size_t n)
{
    void *p = NULL;
    return posix_memalign(&p, align < sizeof(void *) ? sizeof(void *) : align, n) == 0 ? p : NULL;
}

void *memalign(size_t align, size_t n)
{
    /* like glibc: an alignment that is not a power of two is rounded up */
    size_t a = sizeof(void *);
    while (a < align) a <<= 1;
    return aligned_alloc(a, n);
}

size_t malloc_usable_size(void *p)
{
    if (!p || in_boot(p)) return 0;
    const size_t s = managed_size(p);
    if (s) return s;
    return r_usable ? r_usable(p) : 0;
}

/* ---- introspection (tests, statistics) ------------------------------------- */
int gbx_tracker_is_managed(const void *p) { return managed_size(p) != 0; }

/* Entries in the side table and the longest run of occupied slots (the
 * worst lookup length). */
void gbx_tracker_table_stats(uint64_t *used, uint64_t *longest_run)
{
    pthread_mutex_lock(&g_mu);
    size_t run = 0, best = 0, first = 0;
    while (first < TAB_SIZE && g_tab[first].p != 0) first++;   /* start after an empty slot */
    for (size_t k = 1; k <= TAB_SIZE; k++) {
        const size_t i = (first + k) & (TAB_SIZE - 1);
        run = g_tab[i].p ? run + 1 : 0;
        if (run > best) best = run;
    }
    if (used) *used = g_tab_used;
    if (longest_run) *longest_run = best;
    pthread_mutex_unlock(&g_mu);
}

void gbx_tracker_counters(uint64_t *nth, uint64_t *objects, uint64_t *bytes, uint64_t *failures)
{
    if (nth) *nth = atomic_load(&g_nth);
    if (objects) *objects = atomic_load(&g_managed_objects);
    if (bytes) *bytes = atomic_load(&g_managed_bytes);
    if (failures) *failures = atomic_load(&g_managed_fail);
}

__attribute__((constructor(101))) static void tracker_init(void)
{
    t_in = 1;
    ready();
    gbx_tracker_refresh();
    parse_objtracker_options();
    if (g_debug_uninit) {
        const int calls = atomic_load(&g_boot_calls);
        fprintf(stderr, "objtracker: %d allocation(s) before initialisation, %zu bytes of the bootstrap arena\n",
                calls, atomic_load(&g_boot_used));
        for (int i = 0; i < calls && i < BOOT_LOG; i++)
            fprintf(stderr, "objtracker:   before initialisation: allocation of %zu bytes\n", g_boot_log[i]);
    }
    const gbx_config *cfg = gbx_get_config();
    g_min_bytes = cfg->managed_min;
    if (cfg->heuristic == 3 && !gbx_tracker_load_oracle(cfg->oracle_file)) {
        fprintf(stderr, "gbxblas: failed to load allocation oracle '%s': %s\n", cfg->oracle_file,
                strerror(errno));
        abort();
    }
    if (cfg->trace_file[0]) {
        g_trace_fd = open(cfg->trace_file, O_WRONLY | O_CREAT | O_TRUNC | O_APPEND | O_CLOEXEC, 0644);
        if (g_trace_fd < 0) fprintf(stderr, "gbxblas: cannot open trace file '%s'\n", cfg->trace_file);
    }
    g_tracking = 1;
    t_in = 0;
}

__attribute__((destructor)) static void tracker_fini(void)
{
    const gbx_config *cfg = gbx_get_config();
    if (!cfg->stats_file[0]) return;
    t_in = 1;
    uint64_t calls, hits, misses, h2d, d2h;
    gbx_stats(&calls, &hits, &misses, &h2d, &d2h);
    FILE *f = fopen(cfg->stats_file, "w");
    if (f) {
        fprintf(f, "calls,hits,misses,bytes_h2d,bytes_d2h,counted_allocs,managed_objects,managed_bytes,"
                   "managed_failures\n");
        fprintf(f, "%llu,%llu,%llu,%llu,%llu,%llu,%llu,%llu,%llu\n", (unsigned long long)calls,
                (unsigned long long)hits, (unsigned long long)misses, (unsigned long long)h2d,
                (unsigned long long)d2h, (unsigned long long)atomic_load(&g_nth),
                (unsigned long long)atomic_load(&g_managed_objects),
                (unsigned long long)atomic_load(&g_managed_bytes),
                (unsigned long long)atomic_load(&g_managed_fail));
        fclose(f);
    }
    t_in = 0;
}
