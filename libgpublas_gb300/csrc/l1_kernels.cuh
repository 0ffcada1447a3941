// l1_kernels.cuh — device code of the Level-1 routines (included by l1.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// The kernels are static: this header is included by more than one
// translation unit.
namespace gbx_l1 {

constexpr int L1_THREADS = 256;
constexpr int L1_BLOCKS_PER_SM = 4;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum: fixed shuffle tree inside each warp, then warp 0
// adds the per-warp results in warp order.  Valid in thread 0.
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double s_warp[L1_THREADS / 32];
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) s_warp[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = l < L1_THREADS / 32 ? s_warp[l] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

__device__ __forceinline__ double2 ldg2(const double2 *p) { return __ldg(p); }

static __global__ void zero_result(double *res) { *res = 0.0; }
static __global__ void zero_index(int *res) { *res = 0; }

// ---------------------------------------------------------------- daxpy ---
// Unit stride.  When x and y have the same 16-byte phase the body runs on
// double2 (128-bit) accesses after peeling one leading element; otherwise it
// falls back to 64-bit accesses.
static __global__ void __launch_bounds__(L1_THREADS)
axpy_unit(int n, double a, const double *__restrict__ x, double *__restrict__ y)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const unsigned px = (unsigned)((uintptr_t)x & 15), py = (unsigned)((uintptr_t)y & 15);
    if (px == py) {
        const int peel = px ? 1 : 0;
        if (peel && tid == 0) y[0] = fma(a, x[0], y[0]);
        const long long n2 = (long long)(n - peel) >> 1;
        const double2 *x2 = (const double2 *)(x + peel);
        double2 *y2 = (double2 *)(y + peel);
        long long i = tid;
        for (; i + stride < n2; i += 2 * stride) {
            double2 xa = ldg2(x2 + i), xb = ldg2(x2 + i + stride);
            double2 ya = y2[i], yb = y2[i + stride];
            ya.x = fma(a, xa.x, ya.x); ya.y = fma(a, xa.y, ya.y);
            yb.x = fma(a, xb.x, yb.x); yb.y = fma(a, xb.y, yb.y);
            y2[i] = ya; y2[i + stride] = yb;
        }
        for (; i < n2; i += stride) {
            double2 xa = ldg2(x2 + i), ya = y2[i];
            ya.x = fma(a, xa.x, ya.x); ya.y = fma(a, xa.y, ya.y);
            y2[i] = ya;
        }
        if (((n - peel) & 1) && tid == 0) y[n - 1] = fma(a, x[n - 1], y[n - 1]);
    } else {
        for (long long i = tid; i < n; i += stride) y[i] = fma(a, __ldg(x + i), y[i]);
    }
}

// Any increments; x and y point at element 0 of the logical vectors.
static __global__ void __launch_bounds__(L1_THREADS)
axpy_strided(int n, double a, const double *__restrict__ x, int incx, double *__restrict__ y, int incy)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double *yp = y + i * incy;
        *yp = fma(a, x[i * incx], *yp);
    }
}

static __global__ void __launch_bounds__(L1_THREADS)
scal_kernel(int n, double a, double *__restrict__ x, int incx)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        x[i * incx] = (a == 0.0) ? 0.0 : a * x[i * incx];
}

// ----------------------------------------------------------------- ddot ---
static __global__ void __launch_bounds__(L1_THREADS)
dot_partial(int n, const double *__restrict__ x, int incx, const double *__restrict__ y, int incy,
            double *__restrict__ part)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double s0 = 0.0, s1 = 0.0;
    const unsigned px = (unsigned)((uintptr_t)x & 15), py = (unsigned)((uintptr_t)y & 15);
    if (incx == 1 && incy == 1 && px == py) {
        const int peel = px ? 1 : 0;
        if (peel && tid == 0) s0 = x[0] * y[0];
        const long long n2 = (long long)(n - peel) >> 1;
        const double2 *x2 = (const double2 *)(x + peel), *y2 = (const double2 *)(y + peel);
        long long i = tid;
        for (; i + stride < n2; i += 2 * stride) {
            double2 xa = ldg2(x2 + i), xb = ldg2(x2 + i + stride);
            double2 ya = ldg2(y2 + i), yb = ldg2(y2 + i + stride);
            s0 = fma(xa.x, ya.x, s0); s1 = fma(xa.y, ya.y, s1);
            s0 = fma(xb.x, yb.x, s0); s1 = fma(xb.y, yb.y, s1);
        }
        for (; i < n2; i += stride) {
            double2 xa = ldg2(x2 + i), ya = ldg2(y2 + i);
            s0 = fma(xa.x, ya.x, s0); s1 = fma(xa.y, ya.y, s1);
        }
        if (((n - peel) & 1) && tid == 0) s1 = fma(x[n - 1], y[n - 1], s1);
    } else {
        for (long long i = tid; i < n; i += stride) s0 = fma(x[i * incx], y[i * incy], s0);
    }
    double b = block_sum(s0 + s1);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
}

static __global__ void __launch_bounds__(L1_THREADS)
sum_partials(const double *__restrict__ part, int g, double *__restrict__ res)
{
    double s = 0.0;
    for (int i = threadIdx.x; i < g; i += blockDim.x) s += part[i];
    double b = block_sum(s);
    if (threadIdx.x == 0) *res = b;
}

// ---------------------------------------------------------------- dnrm2 ---
// Three-accumulator scaled sum of squares: Blue (ACM TOMS 4(1), 1978), in the
// form of Anderson, "Algorithm 978: Safe Scaling in the Level 1 BLAS" (ACM
// TOMS 44(1), 2017).  The thresholds follow from the binary64 format
// (minimum exponent -1021, maximum exponent 1024, 53 digits):
//   tsml = 2^ceil((-1021-1)/2) = 2^-511     tbig = 2^floor((1024-53+1)/2) = 2^486
//   ssml = 2^-floor((-1021-53)/2) = 2^537   sbig = 2^-ceil((1024+53-1)/2) = 2^-538
struct Blue {
    static constexpr double tsml = 0x1p-511, tbig = 0x1p+486;
    static constexpr double ssml = 0x1p+537, sbig = 0x1p-538;
};

// High word of the bit pattern of |v|, taken in PTX.  Integer compares on
// the bits of a double written in C are folded back into FP64 compares by
// the compiler, and on this part every FP64 instruction per element costs as
// much as the element's load: the streaming kernels below keep their range
// and NaN tests on the integer pipe through these two helpers.
__device__ __forceinline__ unsigned abs_hi_word(double v)
{
    unsigned h;
    asm("{\n\t.reg .b32 lo;\n\tmov.b64 {lo, %0}, %1;\n\tand.b32 %0, %0, 0x7FFFFFFF;\n\t}"
        : "=r"(h) : "l"(__double_as_longlong(v)));
    return h;
}

// Bit pattern of |v| (monotone in |v| for non-NaN values), taken in PTX.
__device__ __forceinline__ unsigned long long abs_bits(double v)
{
    unsigned long long b;
    asm("and.b64 %0, %1, 0x7FFFFFFFFFFFFFFF;" : "=l"(b) : "l"(__double_as_longlong(v)));
    return b;
}

// Warp-uniform fast path: when the high word of |v| puts every lane's
// element in 2^-511 <= |v| < 2^486·(1 + 2^-20) the warp executes the single
// DFMA only (a predicated if-conversion of the three branches would issue
// all three FP64 sequences for every element).  Against the exact thresholds
// this keeps the elements in [2^486, 2^486·(1 + 2^-20)) in the unscaled
// accumulator, where their squares (< 2^973) still cannot overflow a sum of
// 2^31 terms; the result differs from the exact-threshold sum by rounding
// only.  A warp holding any other element (zeros included) classifies each
// lane with the exact thresholds; NaN fails both compares and lands in the
// unscaled accumulator, from where it propagates (netlib's rule).
__device__ __forceinline__ void blue_acc(double v, double &asml, double &amed, double &abig)
{
    constexpr unsigned kBigHi = (unsigned)(486 + 1023) << 20;   // high word of tbig
    constexpr unsigned kSmlHi = (unsigned)(1023 - 511) << 20;   // high word of tsml
    const unsigned h = abs_hi_word(v);
    if (!__any_sync(__activemask(), h - kSmlHi > kBigHi - kSmlHi)) {
        amed = fma(v, v, amed);
        return;
    }
    const double ax = fabs(v);
    if (ax > Blue::tbig) { const double t = ax * Blue::sbig; abig = fma(t, t, abig); }
    else if (ax < Blue::tsml) { const double t = ax * Blue::ssml; asml = fma(t, t, asml); }
    else amed = fma(v, v, amed);
}

// Exact sum of squares on the integer pipe, for one element in four of the
// warps whose elements all lie in the medium range.  One DFMA per element
// would cap the kernel at the FP64 pipe's 2 lanes per clock per SM (about
// 5 TB/s of operands); moving a quarter of the squares to the integer pipe
// lifts that cap above the HBM rate.  A medium-range x is m 2^(e - 1075)
// with the 53-bit significand m, so x^2 = m^2 2^(2e - 2150); the
// accumulator is the unsigned 128-bit integer sum of m^2 2^(2(e - eref) -
// 12), eref the largest exponent seen so far: an element at eref adds
// m^2 >> 12 < 2^94 (2^34 of them fit), a smaller one drops only its bits
// below 2^-94 of the largest square, and a larger exponent shifts the sum
// down first.  The truncation is far below the FP64 rounding of the DFMA
// partials it is added to.
struct SqFix {
    unsigned long long lo, hi;
    int eref;
    __device__ __forceinline__ void init() { lo = 0ull; hi = 0ull; eref = 0; }
    __device__ __forceinline__ void shift_down(int d)
    {
        if (d >= 128) { lo = 0ull; hi = 0ull; }
        else if (d >= 64) { lo = hi >> (d - 64); hi = 0ull; }
        else if (d > 0) { lo = (lo >> d) | (hi << (64 - d)); hi >>= d; }
    }
    // v: a finite normal double (the medium range guarantees it)
    __device__ __forceinline__ void add(double v)
    {
        const unsigned long long b = abs_bits(v);
        const int e = (int)(b >> 52);
        const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
        if (e > eref) {
            shift_down(2 * (e - eref));
            eref = e;
        }
        const int sh = 12 + 2 * (eref - e);   // >= 12
        const unsigned long long plo = m * m, phi = __umul64hi(m, m);   // m^2 < 2^106
        const int s1 = min(sh, 63), s2 = min(max(sh - 64, 0), 63);
        unsigned long long clo = sh < 64 ? (plo >> s1) | (phi << (64 - s1)) : (phi >> s2);
        unsigned long long chi = sh < 64 ? (phi >> s1) : 0ull;
        if (sh >= 106) { clo = 0ull; chi = 0ull; }
        lo += clo;
        hi += chi + (lo < clo ? 1ull : 0ull);
    }
    // the sum as a double: acc * 2^(2 eref - 2150 + 12)
    __device__ __forceinline__ double value() const
    {
        if ((lo | hi) == 0ull) return 0.0;
        return ldexp(fma((double)hi, 0x1p64, (double)lo), 2 * eref - 2138);
    }
};

// True when every active lane's four elements lie in the medium range
// (integer tests on the high words, as in blue_acc).
__device__ __forceinline__ bool all_medium4(double a, double b, double c, double d)
{
    constexpr unsigned kBigHi = (unsigned)(486 + 1023) << 20;
    constexpr unsigned kSmlHi = (unsigned)(1023 - 511) << 20;
    const bool out = (abs_hi_word(a) - kSmlHi > kBigHi - kSmlHi) | (abs_hi_word(b) - kSmlHi > kBigHi - kSmlHi) |
                     (abs_hi_word(c) - kSmlHi > kBigHi - kSmlHi) | (abs_hi_word(d) - kSmlHi > kBigHi - kSmlHi);
    return !__any_sync(__activemask(), out);
}

static __global__ void __launch_bounds__(L1_THREADS)
nrm2_partial(int n, const double *__restrict__ x, int incx, double *__restrict__ part)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double asml = 0.0, amed = 0.0, abig = 0.0;
    if (incx == 1 && (((uintptr_t)x & 15) == 0)) {
        const long long n2 = (long long)n >> 1;
        const double2 *x2 = (const double2 *)x;
        long long i = tid;
        // four independent accumulator chains per thread (the DFMA latency
        // would otherwise serialise the loop)
        double s1 = 0.0, m1 = 0.0, b1 = 0.0, s2 = 0.0, m2 = 0.0, b2 = 0.0, s3 = 0.0, m3 = 0.0, b3 = 0.0;
        SqFix fx;
        fx.init();
        for (; i + stride < n2; i += 2 * stride) {
            double2 a = ldg2(x2 + i), b = ldg2(x2 + i + stride);
            if (all_medium4(a.x, a.y, b.x, b.y)) {
                // three squares on the FP64 pipe, the fourth on the integer pipe
                amed = fma(a.x, a.x, amed);
                m1 = fma(a.y, a.y, m1);
                m2 = fma(b.x, b.x, m2);
                fx.add(b.y);
            } else {
                blue_acc(a.x, asml, amed, abig); blue_acc(a.y, s1, m1, b1);
                blue_acc(b.x, s2, m2, b2); blue_acc(b.y, s3, m3, b3);
            }
        }
        asml += (s1 + s2) + s3;
        amed += ((m1 + m2) + m3) + fx.value();
        abig += (b1 + b2) + b3;
        for (; i < n2; i += stride) {
            double2 a = ldg2(x2 + i);
            blue_acc(a.x, asml, amed, abig); blue_acc(a.y, asml, amed, abig);
        }
        if ((n & 1) && tid == 0) blue_acc(x[n - 1], asml, amed, abig);
    } else {
        for (long long i = tid; i < n; i += stride) blue_acc(x[i * incx], asml, amed, abig);
    }
    double s = block_sum(asml);
    double m = block_sum(amed);
    double b = block_sum(abig);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = s;
        part[3 * blockIdx.x + 1] = m;
        part[3 * blockIdx.x + 2] = b;
    }
}

__device__ __forceinline__ double blue_finish(double asml, double amed, double abig)
{
    double scl, sumsq;
    if (abig > 0.0) {
        if (amed > 0.0 || isnan(amed)) abig = fma(amed * Blue::sbig, Blue::sbig, abig);
        scl = 1.0 / Blue::sbig;
        sumsq = abig;
    } else if (asml > 0.0) {
        if (amed > 0.0 || isnan(amed)) {
            const double am = sqrt(amed), as = sqrt(asml) / Blue::ssml;
            const double ymin = as > am ? am : as, ymax = as > am ? as : am;
            scl = 1.0;
            const double r = ymin / ymax;
            sumsq = ymax * ymax * (1.0 + r * r);
        } else {
            scl = 1.0 / Blue::ssml;
            sumsq = asml;
        }
    } else {
        scl = 1.0;
        sumsq = amed;
    }
    return scl * sqrt(sumsq);
}

static __global__ void __launch_bounds__(L1_THREADS)
nrm2_finish(const double *__restrict__ part, int g, double *__restrict__ res)
{
    double s = 0.0, m = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < g; i += blockDim.x) {
        s += part[3 * i]; m += part[3 * i + 1]; b += part[3 * i + 2];
    }
    s = block_sum(s);
    m = block_sum(m);
    b = block_sum(b);
    if (threadIdx.x == 0) *res = blue_finish(s, m, b);
}

// ------------------------------------------------------- idamax / idamin ---
// Bit-exact arg-max of |x_i| with the first index winning ties.  The key of
// an element is the bit pattern of |x_i| (monotone in |x_i| for non-NaN
// values); for the arg-min the key is its complement.  NaN gets key 0 and
// never beats a number, which is netlib's rule (a NaN never compares greater
// or smaller) except when x_1 itself is NaN: netlib then returns 1, handled in
// the finishing kernel.
template <bool IS_MIN>
__device__ __forceinline__ unsigned long long amax_key(double v)
{
    // integer pipe only: |v| is the bit pattern without the sign bit
    const unsigned long long bits = abs_bits(v);
    if (bits > 0x7FF0000000000000ull) return 0ull;   // NaN
    return IS_MIN ? ~bits : bits;
}

__device__ __forceinline__ bool better(unsigned long long k1, long long i1, unsigned long long k2, long long i2)
{
    return k1 > k2 || (k1 == k2 && i1 < i2);
}

__device__ __forceinline__ void warp_best(unsigned long long &k, long long &i)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
        long long i2 = __shfl_xor_sync(0xffffffffu, i, o);
        if (better(k2, i2, k, i)) { k = k2; i = i2; }
    }
}

__device__ __forceinline__ void block_best(unsigned long long &k, long long &i)
{
    __shared__ unsigned long long s_k[L1_THREADS / 32];
    __shared__ long long s_i[L1_THREADS / 32];
    warp_best(k, i);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s_k[w] = k; s_i[w] = i; }
    __syncthreads();
    if (w == 0) {
        k = l < L1_THREADS / 32 ? s_k[l] : 0ull;
        i = l < L1_THREADS / 32 ? s_i[l] : 0x7fffffffffffffffll;
        warp_best(k, i);
    }
    __syncthreads();
}

template <bool IS_MIN>
static __global__ void __launch_bounds__(L1_THREADS)
iamax_partial(int n, const double *__restrict__ x, int incx, unsigned long long *__restrict__ keys,
              long long *__restrict__ idx)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long bk = 0ull;
    long long bi = 0x7fffffffffffffffll;
    if (incx == 1 && (((uintptr_t)x & 15) == 0)) {
        const long long n2 = (long long)n >> 1;
        const double2 *x2 = (const double2 *)x;
        long long i = tid;
        // four loads in flight per thread; elements are visited in increasing
        // index order within the thread, so the first index keeps winning ties
        for (; i + 3 * stride < n2; i += 4 * stride) {
            double2 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = ldg2(x2 + i + u * stride);
            // pairwise tree over the 8 elements (short dependency chains),
            // then one merge into the running best; ties resolve to the
            // smaller index at every level
            unsigned long long k[8];
            long long e[8];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                k[2 * u] = amax_key<IS_MIN>(v[u].x);
                k[2 * u + 1] = amax_key<IS_MIN>(v[u].y);
                e[2 * u] = 2 * (i + u * stride);
                e[2 * u + 1] = e[2 * u] + 1;
            }
#pragma unroll
            for (int w = 1; w < 8; w *= 2)
#pragma unroll
                for (int a = 0; a < 8; a += 2 * w)
                    if (better(k[a + w], e[a + w], k[a], e[a])) { k[a] = k[a + w]; e[a] = e[a + w]; }
            if (better(k[0], e[0], bk, bi)) { bk = k[0]; bi = e[0]; }
        }
        for (; i < n2; i += stride) {
            double2 v = ldg2(x2 + i);
            unsigned long long k0 = amax_key<IS_MIN>(v.x), k1 = amax_key<IS_MIN>(v.y);
            if (better(k0, 2 * i, bk, bi)) { bk = k0; bi = 2 * i; }
            if (better(k1, 2 * i + 1, bk, bi)) { bk = k1; bi = 2 * i + 1; }
        }
        if ((n & 1) && tid == 0) {
            unsigned long long k = amax_key<IS_MIN>(x[n - 1]);
            if (better(k, n - 1, bk, bi)) { bk = k; bi = n - 1; }
        }
    } else {
        for (long long i = tid; i < n; i += stride) {
            unsigned long long k = amax_key<IS_MIN>(x[i * incx]);
            if (better(k, i, bk, bi)) { bk = k; bi = i; }
        }
    }
    block_best(bk, bi);
    if (threadIdx.x == 0) { keys[blockIdx.x] = bk; idx[blockIdx.x] = bi; }
}

template <bool IS_MIN>
static __global__ void __launch_bounds__(L1_THREADS)
iamax_finish(const double *__restrict__ x, const unsigned long long *__restrict__ keys,
             const long long *__restrict__ idx, int g, int *__restrict__ res)
{
    unsigned long long bk = 0ull;
    long long bi = 0x7fffffffffffffffll;
    for (int i = threadIdx.x; i < g; i += blockDim.x)
        if (better(keys[i], idx[i], bk, bi)) { bk = keys[i]; bi = idx[i]; }
    block_best(bk, bi);
    if (threadIdx.x == 0) *res = isnan(x[0]) ? 1 : (int)(bi + 1);
}

}  // namespace gbx_l1
