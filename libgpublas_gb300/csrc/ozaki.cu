// ozaki.cu — Ozaki split-precision DGEMM / ZGEMM / DSYRK on tcgen05 FP8
// tensor cores (opt-in; the reference has no counterpart: it calls
// cublasDgemm, blas_level3/gemm.cc:174).
//
// Method (Ozaki scheme I with exact low-precision products):
//   * every row i of op(A) is scaled by 2^-e_i (e_i: smallest e with
//     max_k |A_ik| < 2^e) and written as balanced base-32 digits
//         A_ik = 2^(e_i-4) * sum_s d_s(i,k) * 2^(-5 s),   |d_s| <= 16;
//     the columns of op(B) likewise with exponents f_j.  Integers with
//     |d| <= 16 are exact in FP8 E4M3, so each slice is an E4M3 matrix;
//   * slice products d_s * g_t are integers <= 256 and a tcgen05 FP32
//     accumulator stays exact while the accumulated K extent is <= 65536
//     (all partial sums are integers below 2^24), so every product of
//     slices is exact;
//   * products with the same s + t = q share one TMEM accumulator (and one
//     power-of-two weight 2^-5q); only q <= S-1 are formed (S(S+1)/2 slice
//     products); the diagonal sums are combined by Horner's rule, largest
//     weight first: in the wide-tile kernel as one FP64 value per element
//     (rounded once per step, relative to the partial value), in the
//     small-K kernel exactly in two 64-bit integers; the result is scaled by
//     2^(e_i+f_j-8-5(S-1)) and written as C = alpha*sum + beta*C;
//   * S is chosen on the device from the operands' exponent statistics for a
//     target relative Frobenius error (or forced by the caller).
// The scaling, the final recombination and alpha/beta are FP64.
//
// Kernel layout: persistent, one CTA per SM, 320 threads: warp 0 issues TMA
// loads of 128x128-byte (A) and BNx128-byte (B, BN = 256 or 128) slice tiles
// into a shared-memory ring; warp 1 allocates all 512 TMEM columns and
// issues the tcgen05.mma.kind::f8f6f4 (M=128, N=BN, K=32) into one of
// 512/BN accumulators; warps 2-9 drain the others.  Large full products run
// in clusters of two CTAs on vertically adjacent tiles that multicast their
// shared B tile to each other, and the tiles of a last wave that would fill
// at most half the SMs run as half-width tiles.
#include "gbx_internal.h"
#include "gemm_host.h"
#include "tc_ptx.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

using namespace gbx_tc;

namespace {

// Tile: OZ_BM rows by OZ_BN (256) or 128 columns (oz_gemm_kernel<BN>), K in
// blocks of OZ_BK digits.
constexpr int OZ_BM = 128, OZ_BN = 256, OZ_BK = 128;
constexpr int OZ_SMAX = 14;
constexpr int OZ_KEXT_MAX = 65536;   // 2^24 / 16^2
constexpr int OZ_A_BYTES = OZ_BM * OZ_BK;

inline cudaStream_t S_(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }
inline long long rup(long long v, long long m) { return (v + m - 1) / m * m; }

// ---------------------------------------------------------------------------
// operand statistics and slicing
// ---------------------------------------------------------------------------
// Logical rows x K source X: element (r, k) is X[r*ld + k] (row_k) or
// X[k*ld + r] (col_k).  For complex sources (cplx != 0) the element is the
// real part, the imaginary part, or its negation/conjugate of an interleaved
// pair, selected by 'part': 0 re, 1 im, 2 -im; for concatenated operands the
// k range [0, K) is split at Ksplit between two such views.
struct SrcView {
    const double *X;
    long long ld;
    int row_k;      // 1: X[r*ld + k]; 0: X[k*ld + r]
    int cplx;       // 1: interleaved complex
    int part0;      // part for k <  Ksplit
    int part1;      // part for k >= Ksplit
    int Ksplit;     // (complex concatenation) columns of the first view
    int conj;       // conjugate the complex element before taking parts
};

__device__ __forceinline__ double src_get(const SrcView &v, int r, int k)
{
    int kk = k, part = v.part0;
    if (k >= v.Ksplit) { kk = k - v.Ksplit; part = v.part1; }
    const long long idx = v.row_k ? (long long)r * v.ld + kk : (long long)kk * v.ld + r;
    if (!v.cplx) return v.X[idx];
    const double re = v.X[2 * idx], im = v.conj ? -v.X[2 * idx + 1] : v.X[2 * idx + 1];
    return part == 0 ? re : (part == 1 ? im : -im);
}

// ---- operand statistics on the binary64 bit patterns --------------------
// GB300 runs FP64 at ~1.2 TFLOP/s, so the statistics and the slicing work on
// the integer pipe: row maxima are integer maxima of |x| bit patterns, and
// the sum of squares (used only to choose the slice count) is an FP32
// estimate built from the exponent and top mantissa bits.
constexpr int OZ_NONFINITE = 5;   // status word: an operand holds Inf/NaN

// Bit pattern of |x|, taken in PTX: integer tests on a double's bits written
// in C are folded back into FP64 compares, one FP64-pipe slot per element.
__device__ __forceinline__ unsigned long long abs_bits(double x)
{
    unsigned long long b;
    asm("and.b64 %0, %1, 0x7FFFFFFFFFFFFFFF;" : "=l"(b) : "l"(__double_as_longlong(x)));
    return b;
}

// frexp exponent e (|x| < 2^e, |x| >= 2^(e-1)) of a finite |x| bit pattern.
__device__ __forceinline__ int expo_of_bits(unsigned long long b)
{
    if (b == 0) return 0;
    const int E = (int)(b >> 52);
    if (E == 0) return (64 - __clzll((long long)b)) - 1074;   // subnormal
    return E - 1022;
}

// Running max and scaled sum of squares: ss = sum (|x| / 2^(mref-1023))^2
// over the elements seen, mref the largest biased exponent seen.
struct SsAcc {
    unsigned long long maxb;
    int mref;
    float ss;
    __device__ __forceinline__ void init() { maxb = 0ull; mref = 0; ss = 0.f; }
    // v * 2^(2*d) for d <= 0 (exact power-of-two factor; tiny -> 0)
    static __device__ __forceinline__ float scale(float v, int d)
    {
        return d < -60 ? 0.f : v * __int_as_float((127 + 2 * d) << 23);
    }
    __device__ __forceinline__ void add(unsigned long long b)
    {
        maxb = b > maxb ? b : maxb;
        const int E = (int)(b >> 52);
        if (E == 0) return;   // zeros and subnormals do not move the estimate
        if (E > mref) { ss = scale(ss, mref - E); mref = E; }
        const int d = mref - E;
        if (d > 60) return;
        const float y = __int_as_float(((127 - d) << 23) | (int)((b >> 29) & 0x7FFFFFull));
        ss = fmaf(y, y, ss);
    }
    // the same with selects instead of branches, so that a thread's elements
    // are not separated by control flow (more instructions, more overlap:
    // faster where a few blocks run alone, slower where the SMs are full)
    __device__ __forceinline__ void add_sel(unsigned long long b)
    {
        maxb = b > maxb ? b : maxb;
        const int E = (int)(b >> 52);   // zeros and subnormals (E = 0) do not move the estimate
        const bool up = E > mref;       // never for E = 0 (mref >= 0)
        ss = up ? scale(ss, mref - E) : ss;
        mref = up ? E : mref;
        const int d = mref - E;
        const float y = __int_as_float(((127 - min(d, 64)) << 23) | (int)((b >> 29) & 0x7FFFFFull));
        const float t = fmaf(y, y, ss);
        ss = (E == 0 || d > 60) ? ss : t;
    }
    __device__ __forceinline__ void merge(const SsAcc &o)
    {
        maxb = o.maxb > maxb ? o.maxb : maxb;
        if (o.mref > mref) { ss = scale(ss, mref - o.mref) + o.ss; mref = o.mref; }
        else ss += scale(o.ss, o.mref - mref);
    }
    // expo = e of the row max; ss of x * 2^-e (a factor 1/4 from the
    // definition of mref for normal maxima)
    __device__ __forceinline__ void finish(int &e, double &s) const
    {
        e = expo_of_bits(maxb);
        s = (maxb >> 52) ? 0.25 * (double)ss : 0.0;
    }
};

__device__ __forceinline__ void flag_nonfinite(unsigned long long b, int *status)
{
    if ((b >> 52) == 0x7FFull) atomicCAS(status, 0, OZ_NONFINITE);
}

// ---- per-call operand preparation, fused over both operands ----------------
// One call of the Ozaki product prepares op(A) (rows M) and op(B)^T (rows N)
// in three launches: statistics of both operands, the combination of the
// statistics with the scale exponents and (in the last CTA to finish) the
// slice count, and the slicing of both operands.  Small products (the
// trailing updates of a blocked factorization) are dominated by per-launch
// cost, not by these kernels' bytes.
struct OzPrepOp {
    SrcView v;
    int rows, K, Rp, Kp;
    int kch, nkb, rblocks;   // col_k statistics: 32-row blocks x kch-wide K chunks
    int stat_blocks;         // CTAs of the statistics launch (0: no statistics)
    int split_blocks;        // CTAs of the slicing launch: (Kp/128) x (Rp/OZ_SPLIT_ROWS)
    SsAcc *part;             // col_k partials [nkb][rows]
    int *expo;               // frexp exponent of each row's max |x|
    double *ss;              // scaled sum of squares per row
    int *scale;              // Rp scale exponents e-4 (padded rows 0)
    int *scale2;             // optional second copy over Rp2 rows (symmetric rank-k)
    int Rp2;
    uint8_t *X8;             // S digit planes [s][Rp][Kp]
    float *gpart;            // one-launch path: (emax, num, den) per 16-row block
};

__device__ __forceinline__ void oz_stats_rowk_block(const SrcView &v, int rows, int K, int blk, int *expo,
                                                    double *ss, int *status)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blk * 8 + warp;   // one warp per row, 8 rows per CTA
    if (r >= rows) return;
    SsAcc a;
    a.init();
    for (int k = lane; k < K; k += 32) {
        const unsigned long long b = abs_bits(src_get(v, r, k));
        flag_nonfinite(b, status);
        a.add(b);
    }
    for (int o = 16; o; o >>= 1) {
        SsAcc t;
        t.maxb = __shfl_xor_sync(0xffffffffu, a.maxb, o);
        t.mref = __shfl_xor_sync(0xffffffffu, a.mref, o);
        t.ss = __shfl_xor_sync(0xffffffffu, a.ss, o);
        a.merge(t);
    }
    if (lane == 0) a.finish(expo[r], ss[r]);
}

// col_k sources (rows contiguous): 32 rows x 8 k-lanes per CTA over one K
// chunk; partials merged in oz_prep_finish.
__device__ __forceinline__ void oz_stats_colk_block(const SrcView &v, int rows, int K, int kch, int rblocks,
                                                    int blk, SsAcc *part, int *status)
{
    __shared__ SsAcc s_acc[8][32];
    const int rr = threadIdx.x & 31, kl = threadIdx.x >> 5;
    const int r = (blk % rblocks) * 32 + rr, kb = blk / rblocks;
    const int k0 = kb * kch, k1 = min(K, k0 + kch);
    SsAcc a;
    a.init();
    if (r < rows)
        for (int k = k0 + kl; k < k1; k += 8) {
            const unsigned long long b = abs_bits(src_get(v, r, k));
            flag_nonfinite(b, status);
            a.add(b);
        }
    s_acc[kl][rr] = a;
    __syncthreads();
    if (kl == 0 && r < rows) {
        for (int q = 1; q < 8; q++) a.merge(s_acc[q][rr]);
        part[(size_t)kb * rows + r] = a;
    }
}

__global__ void __launch_bounds__(256)
oz_prep_stats(OzPrepOp a, OzPrepOp b, int *status, unsigned *counter)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) *counter = 0u;   // for oz_prep_finish (next launch)
    int blk = blockIdx.x;
    if (blk < a.stat_blocks) {
        if (a.v.row_k) oz_stats_rowk_block(a.v, a.rows, a.K, blk, a.expo, a.ss, status);
        else oz_stats_colk_block(a.v, a.rows, a.K, a.kch, a.rblocks, blk, a.part, status);
    } else {
        blk -= a.stat_blocks;
        if (b.v.row_k) oz_stats_rowk_block(b.v, b.rows, b.K, blk, b.expo, b.ss, status);
        else oz_stats_colk_block(b.v, b.rows, b.K, b.kch, b.rblocks, blk, b.part, status);
    }
}

// Per row: merge col_k partials into (expo, ss), then the scale exponent.
__device__ __forceinline__ void oz_finish_row(const OzPrepOp &o, int r)
{
    int e = 0;
    if (r < o.rows) {
        if (!o.v.row_k) {
            SsAcc acc = o.part[r];
            for (int q = 1; q < o.nkb; q++) acc.merge(o.part[(size_t)q * o.rows + r]);
            acc.finish(o.expo[r], o.ss[r]);
            e = o.expo[r] - 4;
        } else {
            e = o.expo[r] - 4;
        }
    }
    if (r < o.Rp) o.scale[r] = e;
    if (o.scale2 && r < o.Rp2) o.scale2[r] = e;
}

// Block-wide reductions for 256 threads (fixed order: deterministic); every
// thread gets the result.
__device__ __forceinline__ int oz_block_max(int v)
{
    __shared__ int s[8];
#pragma unroll
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    v = s[0];
#pragma unroll
    for (int i = 1; i < 8; i++) v = max(v, s[i]);
    __syncthreads();
    return v;
}

__device__ __forceinline__ double oz_block_sum(double v)
{
    __shared__ double s[8];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    v = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
    __syncthreads();
    return v;
}

// Slice count: relative Frobenius error ~ c * 2^(-5S) * gamma_A * gamma_B with
// gamma^2 = (sum_i 2^(2 e_i)) / (sum_i 2^(2 e_i) * ss_i / K): the ratio of the
// squared row maxima to the squared row norms (1 <= gamma <= sqrt(K)).  The
// statistics were written by other CTAs of the same launch: read through L2,
// four rows per thread in flight.  The logarithm is one thread's (FP64
// transcendental work by a whole CTA costs microseconds on this part).
__device__ __forceinline__ double oz_gamma_finish(double num, double den, int K)
{
    __shared__ double g;
    num = oz_block_sum(num);
    den = oz_block_sum(den);
    if (threadIdx.x == 0) g = den > 0.0 ? 0.5 * log2(num * (double)K / den) : 0.0;
    __syncthreads();
    const double r = g;
    __syncthreads();   // g is reused by the next call
    return r;
}

// 2^(2d) for d <= 0 from the exponent field (0 below the normal range)
__device__ __forceinline__ double oz_pow4(int d)
{
    return 2 * d < -1022 ? 0.0 : __longlong_as_double((long long)(1023 + 2 * d) << 52);
}

__device__ double oz_log2_gamma(const int *expo, const double *ss, int rows, int K)
{
    int emax = -100000;
#pragma unroll 4
    for (int i = threadIdx.x; i < rows; i += blockDim.x) emax = max(emax, __ldcg(expo + i));
    emax = oz_block_max(emax);
    double num = 0.0, den = 0.0;
#pragma unroll 4
    for (int i = threadIdx.x; i < rows; i += blockDim.x) {
        const double w = oz_pow4(__ldcg(expo + i) - emax);
        num += w;
        den += w * __ldcg(ss + i);
    }
    return oz_gamma_finish(num, den, K);
}

// Finishes the statistics of both operands (b_stats: b has its own) and, in
// the last CTA to finish, chooses the slice count:
//   error ~ c * 2^(-5S) * gamma_A * gamma_B; c = 2^1.5 covers the truncated
//   cross terms and the FP64 recombination (measured c ~ 1.4 against the
//   double-double oracle on uniform inputs).
__global__ void __launch_bounds__(256)
oz_prep_finish(OzPrepOp a, OzPrepOp b, int b_stats, double tol, int forced, unsigned *counter, int *S_dev)
{
    const int na = max(a.Rp, a.scale2 ? a.Rp2 : 0);
    const int nb = b_stats ? b.Rp : 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < na + nb; t += gridDim.x * blockDim.x) {
        if (t < na) oz_finish_row(a, t);
        else oz_finish_row(b, t - na);
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double ga = oz_log2_gamma(a.expo, a.ss, a.rows, a.K);
    const double gb = b_stats ? oz_log2_gamma(b.expo, b.ss, b.rows, b.K) : ga;
    if (threadIdx.x == 0) {
        int S;
        if (forced > 0) S = forced;
        else S = (int)ceil((-log2(tol) + ga + gb + 1.5) / 5.0);
        S_dev[0] = max(1, min(OZ_SMAX, S));
    }
}

// E4M3 byte of an integer digit |d| <= 16 (exact).
__device__ __forceinline__ uint32_t e4m3_of_digit(int d)
{
    const int a = d < 0 ? -d : d;
    if (a == 0) return 0u;
    const int E = 31 - __clz(a);
    const int mant = ((a << 3) >> E) - 8;
    return ((d < 0) ? 0x80u : 0u) | (uint32_t)((E + 7) << 3) | (uint32_t)mant;
}

// Slices one 16-row x 128-k tile of an operand: S digit planes X8[s][r][k]
// (K-major, rows padded to Rp, k to Kp), OZ_SPLIT_PER consecutive k per
// thread; padding gets digit 0.  The tile is staged through shared memory so
// col_k sources are read coalesced.
constexpr int OZ_SPLIT_ROWS = 16, OZ_SPLIT_PER = 8;
// the one-launch preparation: 256 threads per 16-row block (16 per row for
// the statistics, 8 k per thread for the digits), or 512 (4 k per thread for
// the digits) when the blocks fit on the SMs at once: the digit split is then
// the block's longest step, and more warps per block shorten it (with more
// blocks than SMs, 512-thread blocks measured slower)
constexpr int OZ_SMALL_THREADS = 256;

// PER consecutive k per thread (blockDim = 16 * 128 / PER); pre: the same
// tile already staged by the caller (one-launch path, K <= 128); expo_s: the
// 16 rows' exponents in the caller's shared memory (one-launch path), else
// they are read from expo
template <int PER, bool SEL = false>
__device__ __forceinline__ void oz_split_tile(const SrcView &v, int rows, int K, int Rp, int Kp, const int *expo,
                                              int S, uint8_t *X8, int blk, const double (*pre)[129] = nullptr,
                                              const int *expo_s = nullptr)
{
    static_assert(PER == 4 || PER == 8, "split width");
    __shared__ double tile[OZ_SPLIT_ROWS][129];
    // E4M3 byte of the digit c - 16 at [c] and of 16 - c at [40 + c], c in
    // [0, 32]: a negative element reads the second table (no per-digit sign)
    __shared__ uint32_t e4m3_tbl[80];
    const int kblocks = Kp / 128;
    const int r0 = (blk / kblocks) * OZ_SPLIT_ROWS, k0 = (blk % kblocks) * 128;
    __syncthreads();   // a previous call's readers of tile are done
    if (threadIdx.x < 33) {
        e4m3_tbl[threadIdx.x] = e4m3_of_digit((int)threadIdx.x - 16);
        e4m3_tbl[40 + threadIdx.x] = e4m3_of_digit(16 - (int)threadIdx.x);
    }
    // load: col_k -> threads along rows; row_k -> threads along k
    if (!pre)
        for (int t = threadIdx.x; t < OZ_SPLIT_ROWS * 128; t += blockDim.x) {
            int rr, kk;
            if (v.row_k) { kk = t & 127; rr = t >> 7; }
            else         { rr = t % OZ_SPLIT_ROWS; kk = t / OZ_SPLIT_ROWS; }
            const int r = r0 + rr, k = k0 + kk;
            tile[rr][kk] = (r < rows && k < K) ? src_get(v, r, k) : 0.0;
        }
    const double (*T)[129] = pre ? pre : tile;
    __syncthreads();
    constexpr int TPR = 128 / PER;   // threads per row
    const int rr = threadIdx.x / TPR, kq = (threadIdx.x % TPR) * PER;
    const int r = r0 + rr;
    if (r >= Rp) return;
    const int e = r < rows ? (expo_s ? expo_s[rr] : expo[r]) : 0;
    // N_j = round(|x_j| * 2^(4 - e + 5(S-1))) as a 128-bit integer hi:lo.
    // |x| < 2^e bounds N_j by 16 * 32^(S-1) <= 2^69.  Integer pipe only.
    const int top = 4 - e + 5 * (S - 1);
    unsigned long long lo[PER], hi[PER];
    unsigned neg = 0u;
    // (SEL: with selects instead of branches, so that the elements of a
    // thread are not separated by control flow and their integer chains
    // overlap; more instructions, so only where few blocks run)
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(T[rr][kq + j]);
        neg |= (unsigned)(b >> 63) << j;
        const int E = (int)((b >> 52) & 0x7FF);
        const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (E ? (1ull << 52) : 0ull);
        const int sh = (E ? E : 1) - 1075 + top;
        if constexpr (!SEL) {
            if (M == 0ull || sh <= -54) { lo[j] = 0ull; hi[j] = 0ull; }
            else if (sh < 0) { lo[j] = (M + (1ull << (-sh - 1))) >> (-sh); hi[j] = 0ull; }
            else if (sh == 0) { lo[j] = M; hi[j] = 0ull; }
            else if (sh < 64) { lo[j] = M << sh; hi[j] = M >> (64 - sh); }
            else { lo[j] = 0ull; hi[j] = M << (sh - 64); }
            continue;
        }
        // sh < 0: M * 2^sh rounded half up (0 for sh <= -54; M = 0 gives 0);
        // sh >= 0: M << sh in 128 bits (sh <= 69)
        const int rs = max(1, min(-sh, 63));
        const unsigned long long mr = sh < 0 ? (sh <= -54 ? 0ull : (M + (1ull << (rs - 1))) >> rs) : M;
        const int ls = max(sh, 0);
        lo[j] = ls < 64 ? mr << (ls & 63) : 0ull;
        hi[j] = ls == 0 ? 0ull : (ls < 64 ? mr >> ((64 - ls) & 63) : mr << ((ls - 64) & 63));
    }
    // Balanced base-32 digits d_s in [-16, 16] with N = sum_s d_s 32^(S-1-s):
    // adding C = 16 * sum_{s<S} 32^s once turns every 5-bit chunk c of N + C
    // into the digit c - 16 (the carries are resolved by the one addition);
    // the top chunk is taken unmasked (N <= 16 * 32^(S-1) bounds it by 32).
    unsigned long long clo = 0ull, chi = 0ull;
    for (int s = 0; s < S; s++) {
        const int b = 5 * s + 4;
        if (b < 64) clo |= 1ull << b;
        else chi |= 1ull << (b - 64);
    }
    // N + C as three 32-bit words (N + C < 2^71)
    uint32_t w0[PER], w1[PER], w2[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const unsigned long long nl = lo[j] + clo;
        const unsigned long long nh = hi[j] + chi + (nl < clo ? 1ull : 0ull);
        w0[j] = (uint32_t)nl;
        w1[j] = (uint32_t)(nl >> 32);
        w2[j] = (uint32_t)nh;
    }
    const uint32_t *tb[PER];   // each element's table (by its sign)
#pragma unroll
    for (int j = 0; j < PER; j++) tb[j] = e4m3_tbl + (((neg >> j) & 1u) ? 40 : 0);
    // chunk t (bit 5t, from the low end) is the digit of plane S - 1 - t;
    // unrolled over t so that its word and bit offset are constants (one
    // funnel shift per chunk)
#pragma unroll
    for (int t = 0; t < OZ_SMAX; t++) {
        if (t >= S) break;
        const int sh = 5 * t, wk = sh >> 5, off = sh & 31;
        const uint32_t mask = t == S - 1 ? 63u : 31u;
        uint32_t w[PER / 4] = {};
#pragma unroll
        for (int j = 0; j < PER; j++) {
            uint32_t c = wk == 0 ? __funnelshift_r(w0[j], w1[j], off)
                                 : (wk == 1 ? __funnelshift_r(w1[j], w2[j], off) : w2[j] >> off);
            c &= mask;
            // the digit of x = sign(x) * (c - 16) as an E4M3 byte
            w[j >> 2] |= tb[j][c] << (8 * (j & 3));
        }
        uint8_t *dst = X8 + ((size_t)(S - 1 - t) * Rp + r) * Kp + k0 + kq;
        if constexpr (PER == 8) *(uint2 *)dst = make_uint2(w[0], w[PER / 4 - 1]);
        else *(uint32_t *)dst = w[0];
    }
}

__global__ void __launch_bounds__(256)
oz_prep_split(OzPrepOp a, OzPrepOp b, const int *__restrict__ S_dev)
{
    const int S = *S_dev;
    if ((int)blockIdx.x < a.split_blocks)
        oz_split_tile<OZ_SPLIT_PER>(a.v, a.rows, a.K, a.Rp, a.Kp, a.expo, S, a.X8, blockIdx.x);
    else
        oz_split_tile<OZ_SPLIT_PER>(b.v, b.rows, b.K, b.Rp, b.Kp, b.expo, S, b.X8, blockIdx.x - a.split_blocks);
}

// ---- small K: the whole preparation in one launch ---------------------------
// Each CTA owns 16 complete rows of one operand: a first pass over their K
// extent gives the row statistics (maximum and sum of squares), a second
// writes P digit planes, P the largest slice count the tolerance can call
// for (the slice count itself is not known yet; the leading S planes of the
// P-digit balanced expansion represent the row to within 16.5 * 2^(-5S) of
// its maximum, the same bound as rounding at S digits); every CTA leaves a partial of the slice-count statistic,
// from which the product kernel chooses S.  One launch instead of three:
// small products are dominated by per-launch cost.
template <int THREADS>
__device__ __forceinline__ void oz_prep_rows(const SrcView &v, int rows, int K, int Rp, int Kp, int *expo, double *ss,
                                             int *scale, uint8_t *X8, float *gpart, int planes, int rblk,
                                             int *status)
{
    static_assert(THREADS == 256 || THREADS == 512, "the statistics map 16 threads to a row of a 16-row block");
    constexpr int PER = OZ_SPLIT_ROWS * 128 / THREADS;   // k per thread in the digit split
    __shared__ double tile[OZ_SPLIT_ROWS][129];
    __shared__ int s_ex[OZ_SPLIT_ROWS];       // the rows' exponents and sums of squares, also kept here
    __shared__ double s_ss[OZ_SPLIT_ROWS];    // for the partial and the split (no global round trip)
    const int r0 = rblk * OZ_SPLIT_ROWS;
    const int rr = threadIdx.x >> 4, lane16 = threadIdx.x & 15;   // 16 threads per row
    SsAcc acc;
    acc.init();
    for (int k0 = 0; k0 < K; k0 += 128) {
        if (!v.cplx && v.Ksplit >= K && r0 + OZ_SPLIT_ROWS <= rows && k0 + 128 <= K) {
            // a full 16 x 128 block of a real operand (uniform): strided
            // pointers, every load issued before the first store
            constexpr int N = OZ_SPLIT_ROWS * 128 / THREADS;
            double x[N];
            if (v.row_k) {   // X[r * ld + k]: 128 consecutive k per row
                constexpr int RS = THREADS / 128;
                const int tr = threadIdx.x >> 7, kk = threadIdx.x & 127;
                const double *src = v.X + (long long)(r0 + tr) * v.ld + k0 + kk;
#pragma unroll
                for (int i = 0; i < N; i++) x[i] = src[(long long)i * RS * v.ld];
#pragma unroll
                for (int i = 0; i < N; i++) tile[tr + i * RS][kk] = x[i];
            } else {         // X[k * ld + r]: 16 consecutive rows per k
                constexpr int KS = THREADS / OZ_SPLIT_ROWS;
                const int tr = threadIdx.x & (OZ_SPLIT_ROWS - 1), kk = threadIdx.x / OZ_SPLIT_ROWS;
                const double *src = v.X + (long long)(k0 + kk) * v.ld + r0 + tr;
#pragma unroll
                for (int i = 0; i < N; i++) x[i] = src[(long long)i * KS * v.ld];
#pragma unroll
                for (int i = 0; i < N; i++) tile[tr][kk + i * KS] = x[i];
            }
        } else {
            for (int t = threadIdx.x; t < OZ_SPLIT_ROWS * 128; t += blockDim.x) {
                int tr, kk;
                if (v.row_k) { kk = t & 127; tr = t >> 7; }
                else         { tr = t % OZ_SPLIT_ROWS; kk = t / OZ_SPLIT_ROWS; }
                const int r = r0 + tr, k = k0 + kk;
                tile[tr][kk] = (r < rows && k < K) ? src_get(v, r, k) : 0.0;
            }
        }
        __syncthreads();
        if (threadIdx.x < 256) {   // warp-uniform: the first eight warps
            bool nonfinite = false;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const unsigned long long b = abs_bits(tile[rr][lane16 + 16 * j]);
                nonfinite |= (b >> 52) == 0x7FFull;
                if constexpr (THREADS == 512) acc.add_sel(b);
                else acc.add(b);
            }
            if (nonfinite) atomicCAS(status, 0, OZ_NONFINITE);
        }
        __syncthreads();
    }
    if (threadIdx.x < 256) {
#pragma unroll
        for (int o = 8; o; o >>= 1) {   // the 16 threads of a row are one half-warp
            SsAcc t;
            t.maxb = __shfl_xor_sync(0xffffffffu, acc.maxb, o);
            t.mref = __shfl_xor_sync(0xffffffffu, acc.mref, o);
            t.ss = __shfl_xor_sync(0xffffffffu, acc.ss, o);
            acc.merge(t);
        }
    }
    const int r = r0 + rr;
    if (threadIdx.x < 256 && lane16 == 0 && r < Rp) {
        int ex = 0;
        double sv = 0.0;
        if (r < rows) {
            acc.finish(ex, sv);
            expo[r] = ex;
            ss[r] = sv;
            scale[r] = ex - 4;
        } else {
            scale[r] = 0;
        }
        s_ex[rr] = ex;
        s_ss[rr] = sv;
    }
    __syncthreads();   // the row exponents are visible to the whole CTA
    if (gpart && threadIdx.x < 32) {
        // this block's partial of the slice-count statistic (oz_choose_S):
        // (emax_c, sum 2^(2(e_i - emax_c)), sum 2^(2(e_i - emax_c)) ss_i)
        const int rg = r0 + (threadIdx.x & 15);
        const bool valid = threadIdx.x < 16 && rg < rows;
        const int e = valid ? s_ex[threadIdx.x & 15] : -100000;
        int em = e;
#pragma unroll
        for (int o = 16; o; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
        const int d = 2 * (e - em);
        const float w = (!valid || d < -126) ? 0.f : __int_as_float((127 + d) << 23);
        float nu = w, de = valid ? w * (float)s_ss[threadIdx.x & 15] : 0.f;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            nu += __shfl_xor_sync(0xffffffffu, nu, o);
            de += __shfl_xor_sync(0xffffffffu, de, o);
        }
        if (threadIdx.x == 0) {
            gpart[3 * rblk] = (float)em;
            gpart[3 * rblk + 1] = nu;
            gpart[3 * rblk + 2] = de;
        }
    }
    const int kblocks = Kp / 128;
    if (kblocks == 1)   // the statistics pass left this block's only tile in shared memory
        oz_split_tile<PER, THREADS == 512>(v, rows, K, Rp, Kp, expo, planes, X8, rblk, tile, s_ex);
    else
        for (int kb = 0; kb < kblocks; kb++)
            oz_split_tile<PER, THREADS == 512>(v, rows, K, Rp, Kp, expo, planes, X8, rblk * kblocks + kb, nullptr,
                                               s_ex);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS == 256 ? 4 : 1)
oz_prep_small(OzPrepOp a, OzPrepOp b, int planes, int *status)
{
    // the product kernel may be scheduled now: its set-up needs none of this
    // launch's results, and it waits for them (griddepcontrol.wait)
    asm volatile("griddepcontrol.launch_dependents;");
    const int na = a.Rp / OZ_SPLIT_ROWS;
    if ((int)blockIdx.x < na)
        oz_prep_rows<THREADS>(a.v, a.rows, a.K, a.Rp, a.Kp, a.expo, a.ss, a.scale, a.X8, a.gpart, planes, blockIdx.x,
                              status);
    else
        oz_prep_rows<THREADS>(b.v, b.rows, b.K, b.Rp, b.Kp, b.expo, b.ss, b.scale, b.X8, b.gpart, planes, blockIdx.x - na,
                     status);
}

// ---------------------------------------------------------------------------
// the tensor-core kernel
// ---------------------------------------------------------------------------
struct OzParams {
    int M, N, Mp, Np, Kp;
    int tiles_m, tiles_n;
    int t_split, nunits;       // wide-tile kernel: units below t_split are whole tiles, the rest
                               // half tiles (two per tile t_split + (u - t_split) / 2)
    int *S;                    // slice count (written by the small-K kernel, read by the others)
    const int *row_exp;        // Mp: e_i - 4
    const int *col_exp;        // Np: f_j - 4
    long long *W;              // Mp x Np running sums, column-major: two 64-bit words per element
                               // (exact drain) or one double (Horner drain)
    double *C;
    long long ldc;
    double alpha, beta;
    int c_part;                // 0 full, 1 lower (row >= col), 2 upper
    int *status;               // the context's status word (zero while nothing failed)
    int *status_host;          // its mapped host mirror
    // small-K kernel: the slice count is chosen in the kernel from the
    // preparation's per-block partials (and written to *S by CTA 0)
    const float *gpa, *gpb;    // partials of op(A) and op(B)^T
    int npa, npb;              // their counts
    int K;
    float tol_bits;            // -log2(tol)
    int forced;                // fixed slice count, or 0
    int smax;                  // digit planes prepared (upper bound of S)
    int s_lo;                  // lower bound of S from the tolerance alone (small-K kernel)
};

// The small-K product kernel's slice count, computed by every CTA from the
// preparation's per-block partials of both operands (the same data in the
// same order in every CTA: one S per call) with the model oz_prep_finish
// applies, clamped to the planes the preparation wrote; CTA 0 records it.
// Returns 0 for a call to skip (the status word is set: a non-finite operand
// or an earlier kernel's expired wait); every thread gets the same answer
// before any copy or MMA is issued.  The status and up to two partials per
// thread and operand are read in one round of loads (a round costs about a
// microsecond at the start of a call of a few tens of microseconds).
__device__ int oz_choose_S(const OzParams &p)
{
    constexpr int R = 2;   // partials per thread and operand held in registers
    __shared__ int s_e[2][32];
    __shared__ float s_v[4][32];
    __shared__ int s_S;
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nt = blockDim.x;
    const int st = threadIdx.x == 0 ? *(volatile int *)p.status : 0;
    if (p.forced > 0) {
        if (threadIdx.x == 0) {
            s_S = st ? 0 : min(p.forced, p.smax);
            if (blockIdx.x == 0 && s_S) *p.S = s_S;
        }
        __syncthreads();
        return s_S;
    }
    // the partial i is handled by thread i mod nt, in increasing i: the
    // same sums in the same order whichever branch runs
    const bool regs = p.npa <= R * nt && p.npb <= R * nt;   // uniform
    float pa[R][3], pb[R][3];
    int ea = -100000, eb = -100000;
    if (regs) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = threadIdx.x + r * nt;
            const bool va = i < p.npa, vb = i < p.npb;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                pa[r][c] = va ? __ldcg(p.gpa + 3 * i + c) : 0.f;
                pb[r][c] = vb ? __ldcg(p.gpb + 3 * i + c) : 0.f;
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = threadIdx.x + r * nt;
            if (i < p.npa) ea = max(ea, (int)pa[r][0]);
            if (i < p.npb) eb = max(eb, (int)pb[r][0]);
        }
    } else {
        for (int i = threadIdx.x; i < p.npa; i += nt) ea = max(ea, (int)__ldcg(p.gpa + 3 * i));
        for (int i = threadIdx.x; i < p.npb; i += nt) eb = max(eb, (int)__ldcg(p.gpb + 3 * i));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        ea = max(ea, __shfl_xor_sync(0xffffffffu, ea, o));
        eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, o));
    }
    if (lane == 0) { s_e[0][warp] = ea; s_e[1][warp] = eb; }
    __syncthreads();
    ea = lane < nw ? s_e[0][lane] : -100000;   // nw <= 32
    eb = lane < nw ? s_e[1][lane] : -100000;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        ea = max(ea, __shfl_xor_sync(0xffffffffu, ea, o));
        eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, o));
    }
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    auto weight = [](int e, int em) {
        const int d = 2 * (e - em);
        return d < -126 ? 0.f : __int_as_float((127 + d) << 23);
    };
    if (regs) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = threadIdx.x + r * nt;
            if (i < p.npa) {
                const float w = weight((int)pa[r][0], ea);
                v[0] = fmaf(w, pa[r][1], v[0]);
                v[1] = fmaf(w, pa[r][2], v[1]);
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = threadIdx.x + r * nt;
            if (i < p.npb) {
                const float w = weight((int)pb[r][0], eb);
                v[2] = fmaf(w, pb[r][1], v[2]);
                v[3] = fmaf(w, pb[r][2], v[3]);
            }
        }
    } else {
        for (int i = threadIdx.x; i < p.npa; i += nt) {
            const float w = weight((int)__ldcg(p.gpa + 3 * i), ea);
            v[0] = fmaf(w, __ldcg(p.gpa + 3 * i + 1), v[0]);
            v[1] = fmaf(w, __ldcg(p.gpa + 3 * i + 2), v[1]);
        }
        for (int i = threadIdx.x; i < p.npb; i += nt) {
            const float w = weight((int)__ldcg(p.gpb + 3 * i), eb);
            v[2] = fmaf(w, __ldcg(p.gpb + 3 * i + 1), v[2]);
            v[3] = fmaf(w, __ldcg(p.gpb + 3 * i + 2), v[3]);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
#pragma unroll
        for (int o = 16; o; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
        if (lane == 0) s_v[j][warp] = v[j];
    }
    __syncthreads();
    if (warp == 0) {
        float t[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            t[j] = lane < nw ? s_v[j][lane] : 0.f;
#pragma unroll
            for (int o = 16; o; o >>= 1) t[j] += __shfl_xor_sync(0xffffffffu, t[j], o);
        }
        if (lane == 0) {
            const float ga = t[1] > 0.f ? 0.5f * __log2f(t[0] * (float)p.K / t[1]) : 0.f;
            const float gb = t[3] > 0.f ? 0.5f * __log2f(t[2] * (float)p.K / t[3]) : 0.f;
            int S = (int)ceilf((p.tol_bits + ga + gb + 1.5f) / 5.0f);
            // never below s_lo: the kernel requested that many A slices early
            S = max(max(1, p.s_lo), min(p.smax, S));
            s_S = st ? 0 : S;
            if (blockIdx.x == 0 && !st) *p.S = S;
        }
    }
    __syncthreads();
    return s_S;
}

// A call whose operands were found non-finite (or whose earlier kernel gave
// up a wait) skips the product kernel: every thread of the CTA takes the
// same decision before any copy or MMA is issued, so no asynchronous work is
// left behind.
__device__ __forceinline__ bool oz_skip_kernel(const OzParams &p)
{
    __shared__ int s_st;
    if (threadIdx.x == 0) s_st = *(volatile int *)p.status;
    __syncthreads();
    return s_st != 0;
}

// A nonzero status is copied to the host mirror as the CTA finishes (the
// host reads the mirror after its stream synchronisation).
__device__ __forceinline__ void oz_report(const OzParams &p)
{
    if (threadIdx.x == 0) {
        const int st = *(volatile int *)p.status;
        if (st) *(volatile int *)p.status_host = st;
    }
}

// Group enumeration shared by the three roles.  Items are (pair, k chunk);
// a group is a run of consecutive items of one diagonal whose K extent stays
// within the exact-accumulation bound.  A diagonal of n items is cut into
// ceil(n / items_per_group) groups of near-equal size (K = 8192: nine items
// as 5 + 4, not 8 + 1): the MMAs of a short group cannot hide the drain of
// the group before it, so the tensor pipe waited on every one-item group.
struct GroupPlan {
    int S, nkb, kch_blocks, nchunks, items_per_group;
    __device__ void init(int S_, int Kp, int bk = OZ_BK)
    {
        S = S_;
        nkb = Kp / bk;
        const int kch = min(Kp, OZ_KEXT_MAX);
        kch_blocks = kch / bk;
        nchunks = (nkb + kch_blocks - 1) / kch_blocks;
        items_per_group = max(1, OZ_KEXT_MAX / (kch_blocks * bk));
    }
    __device__ int ngroups(int nitems) const { return (nitems + items_per_group - 1) / items_per_group; }
    // first item of group g of ng (g = ng gives nitems); every group holds at
    // most ceil(nitems / ng) <= items_per_group items
    __device__ int gbegin(int nitems, int ng, int g) const { return g * nitems / ng; }
};

__device__ __forceinline__ bool tile_needed(const OzParams &p, int tm, int tn, int bm = OZ_BM, int bn = OZ_BN)
{
    if (p.c_part == 0) return true;
    const int r0 = tm * bm, r1 = r0 + bm - 1, c0 = tn * bn, c1 = c0 + bn - 1;
    return p.c_part == 1 ? (r1 >= c0) : (r0 <= c1);
}

// Whether element (grow, gcol) of C is written: inside N and, for DSYRK, in
// the stored triangle.
__device__ __forceinline__ bool oz_c_keep(const OzParams &p, int grow, int gcol)
{
    return gcol < p.N && (p.c_part == 0 || (p.c_part == 1 ? grow >= gcol : grow <= gcol));
}

template <int CH>
__device__ __forceinline__ void tmem_ld_chunk(uint32_t taddr, uint32_t (&r)[CH]);
template <>
__device__ __forceinline__ void tmem_ld_chunk<8>(uint32_t taddr, uint32_t (&r)[8]) { tmem_ld_32x32b_x8(taddr, r); }
template <>
__device__ __forceinline__ void tmem_ld_chunk<4>(uint32_t taddr, uint32_t (&r)[4]) { tmem_ld_32x32b_x4(taddr, r); }

// V (128-bit) as a double: the exact integer rounded once to 53 bits when it
// fits 64 bits, else hi * 2^64 + lo (the low word rounded first, within one
// unit of the last place).
__device__ __forceinline__ double oz_to_double(unsigned long long lo, long long hi)
{
    if (hi == ((long long)lo >> 63)) return (double)(long long)lo;
    return fma((double)hi, 0x1p64, (double)lo);
}

// alpha * 2^e, exact: the exponent field moved on the integer pipe when the
// result stays a normal number, ldexp otherwise.  Then alpha * (V * 2^e) is
// one FP64 multiply of V by this factor.
__device__ __forceinline__ double oz_alpha_pow2(double alpha, int e)
{
    const long long b = __double_as_longlong(alpha);
    const int ea = (int)((b >> 52) & 0x7FF);
    if (ea != 0 && ea != 0x7FF && ea + e >= 1 && ea + e <= 2046)
        return __longlong_as_double(b + ((long long)e << 52));
    return ldexp(alpha, e);
}

// An FP32 accumulator value (an integer, so zero or normal) widened to
// double by re-biasing its exponent field on the integer pipe: the FP32 to
// FP64 conversion instruction issues to the FP64 pipe, which the Horner
// step already keeps half busy.  Exact, like the conversion it replaces.
__device__ __forceinline__ double oz_f32_to_f64(uint32_t b)
{
    const unsigned long long mag = b & 0x7FFFFFFFu;
    const unsigned long long bits =
        ((unsigned long long)(b & 0x80000000u) << 32) | (mag ? (mag + (896ull << 23)) << 29 : 0ull);
    return __longlong_as_double((long long)bits);
}

// FP32 accumulator values are integers.  Float-to-integer conversion
// instructions issue to the FP64 pipe, which on this part retires two lanes
// per clock per SM (one drain of a 128 x 32 tile with ten diagonals spent
// 20k cycles there), so the drains decode the value on the FMA and integer
// pipes instead.
//   |v| < 2^22: adding 1.5 * 2^23 (exact, round to nearest) leaves v in the
//   low mantissa bits, bits = 0x4B400000 + v.
__device__ __forceinline__ int oz_f2i22(float v)
{
    return __float_as_int(__fadd_rn(v, 12582912.0f)) - 0x4B400000;
}

// The signed 128-bit integer (hi:lo) times 2^e as a double, rounded to
// nearest even, built on the integer pipe: magnitude, leading-zero count,
// normalisation, rounding of the 75 discarded bits, exponent field.  ok is
// false when the result would not be a normal number (the caller then takes
// the FP64 route); zero is exact.
__device__ __forceinline__ double oz_i128_ldexp(unsigned long long lo, long long hi, int e, bool &ok)
{
    const unsigned long long s = (unsigned long long)(hi >> 63);
    const unsigned long long ml = (lo ^ s) - s;
    const unsigned long long mh = ((unsigned long long)hi ^ s) + (s & (ml == 0ull ? 1ull : 0ull));
    if ((mh | ml) == 0ull) {
        ok = true;
        return 0.0;
    }
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
    unsigned long long nh, nl;
    if (lz >= 64) {
        nh = ml << (lz - 64);
        nl = 0ull;
    } else if (lz == 0) {
        nh = mh;
        nl = ml;
    } else {
        nh = (mh << lz) | (ml >> (64 - lz));
        nl = ml << lz;
    }
    unsigned long long mant = nh >> 11;   // 53 bits, the leading one at bit 52
    const unsigned long long rem = nh & 0x7FFull;
    if (rem > 0x400ull || (rem == 0x400ull && (nl != 0ull || (mant & 1ull)))) mant++;
    const int eb = 127 - lz + e + 1023;   // biased exponent (a rounding carry adds one through mant)
    ok = eb >= 1 && eb <= 2045;
    return __longlong_as_double((long long)((((unsigned long long)(eb - 1)) << 52) + mant) |
                                (long long)(s & 0x8000000000000000ull));
}

// alpha as +-2^ea when it is a power of two (folded into the exponent on the
// integer pipe), else kept for one FP64 multiply; and whether beta is
// nonzero, decided once per thread (an FP64 compare per element costs a slot
// on the 2-lane FP64 pipe like any FP64 instruction).
struct OzAlpha {
    bool pow2;
    bool beta_on;
    int ea;
    unsigned long long sign;
};
__device__ __forceinline__ OzAlpha oz_alpha_split(double alpha, double beta)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(alpha);
    const int ex = (int)((b >> 52) & 0x7FF);
    OzAlpha a;
    a.pow2 = (b & 0xFFFFFFFFFFFFFull) == 0ull && ex != 0 && ex != 0x7FF;
    a.beta_on = beta != 0.0;
    a.ea = ex - 1023;
    a.sign = b & 0x8000000000000000ull;
    return a;
}

// One Horner step v = 32 v + D for each element of a drain thread's row segment
// (D: FP32 accumulator values below 2^22, decoded off the FP64 pipe).
template <int N>
__device__ __forceinline__ void oz_horner(long long (&v)[N], const uint32_t (&r)[N])
{
#pragma unroll
    for (int j = 0; j < N; j++)
        v[j] = (long long)(((unsigned long long)v[j] << 5) +
                           (unsigned long long)(long long)oz_f2i22(__uint_as_float(r[j])));
}

// Two Horner steps at once, v = 1024 v + (32 D_a + D_b): the pair is formed
// in 32-bit arithmetic (|32 D_a + D_b| < 2^28; the decode's offsets cancel
// modulo 2^32), so the 64-bit shift-add runs once per two diagonals.
template <int N>
__device__ __forceinline__ void oz_horner2(long long (&v)[N], const uint32_t (&ra)[N], const uint32_t (&rb)[N])
{
#pragma unroll
    for (int j = 0; j < N; j++) {
        const uint32_t ba = __float_as_uint(__fadd_rn(__uint_as_float(ra[j]), 12582912.0f));
        const uint32_t bb = __float_as_uint(__fadd_rn(__uint_as_float(rb[j]), 12582912.0f));
        const int g = (int)(ba * 32u + bb - 33u * 0x4B400000u);
        v[j] = (long long)(((unsigned long long)v[j] << 10) + (unsigned long long)(long long)g);
    }
}

// v * 2^e as a double for |v| < 2^53 (exact), built on the integer pipe;
// eb receives the biased exponent of the result (1023 for v = 0), which the
// caller checks against the normal range.
__device__ __forceinline__ double oz_i53_ldexp(long long v, int e, int &eb)
{
    const unsigned long long s = (unsigned long long)(v >> 63);
    const unsigned long long m = ((unsigned long long)v ^ s) - s;
    const int lz = __clzll((long long)m);   // >= 11; 64 for v = 0
    eb = m ? 1086 - lz + e : 1023;
    const unsigned long long bits = ((unsigned long long)(eb - 1) << 52) + (m << (lz - 11));
    return __longlong_as_double((long long)((m ? bits : 0ull) | (s & 0x8000000000000000ull)));
}

// The output value alpha * V * 2^e + beta * cold for the signed 128-bit V:
// one rounding of V * 2^e (exact scaling), then one multiply-add with beta.
__device__ __forceinline__ double oz_result(unsigned long long lo, long long hi, int e, double alpha,
                                            const OzAlpha &as, double beta, double cold)
{
    bool ok;
    double r;
    if (as.pow2) {
        r = oz_i128_ldexp(lo, hi, e + as.ea, ok);
        r = __longlong_as_double(__double_as_longlong(r) ^ (long long)as.sign);
    } else {
        r = alpha * oz_i128_ldexp(lo, hi, e, ok);
    }
    if (!ok) r = oz_alpha_pow2(alpha, e) * oz_to_double(lo, hi);
    return as.beta_on ? fma(beta, cold, r) : r;
}

// The same for V = vh * 2^lsh + vl with |vh|, |vl| < 2^53 (0 <= lsh < 64):
// both parts convert exactly on the integer pipe and one FP64 addition
// rounds their sum once, so V * 2^e is correctly rounded with two FP64
// instructions per element (the addition and the beta multiply-add) and no
// 128-bit normalisation.  Parts outside the normal range take the 128-bit
// route.
__device__ __forceinline__ double oz_result_split(long long vh, long long vl, int lsh, int e, double alpha,
                                                  const OzAlpha &as, double beta, double cold)
{
    const int ee = as.pow2 ? e + as.ea : e;
    int ebh, ebl;
    double dh = oz_i53_ldexp(vh, ee + lsh, ebh);
    double dl = oz_i53_ldexp(vl, ee, ebl);
    if (ebh >= 1 && ebh <= 2045 && ebl >= 1 && ebl <= 2045) {
        double r;
        if (as.pow2) {
            dh = __longlong_as_double(__double_as_longlong(dh) ^ (long long)as.sign);
            dl = __longlong_as_double(__double_as_longlong(dl) ^ (long long)as.sign);
            r = dh + dl;
        } else {
            r = alpha * (dh + dl);
        }
        return as.beta_on ? fma(beta, cold, r) : r;
    }
    unsigned long long lo;
    long long hi;
    if (lsh == 0) {
        lo = (unsigned long long)vh;
        hi = vh >> 63;
    } else {
        lo = (unsigned long long)vh << lsh;
        hi = vh >> (64 - lsh);
    }
    const unsigned long long nlo = lo + (unsigned long long)vl;
    hi = hi + (vl >> 63) + (nlo < lo ? 1 : 0);
    return oz_result(nlo, hi, e, alpha, as, beta, cold);
}

// The drain conversion of a row segment of N elements (V = vh * 2^lsh + vl
// each, scale 2^(erow + ecol[j])): the common case of oz_result_split with
// no control flow inside, for a given alpha form (POW2) and beta (BETA), so
// that the FP64 chains of the N elements (addition, then beta multiply-add:
// about 64 cycles each) overlap; with a branch in each element they ran one
// after another, and the row took twice as long.  Returns true when some
// part left the normal range: the caller then converts the segment again by
// oz_result_split, whose 128-bit route handles it.
template <bool POW2, bool BETA, int N>
__device__ __forceinline__ bool oz_convert_segment(double *res, const long long *vh, const long long *vl, int lsh,
                                                   int erow, const int *ecol, double alpha, const OzAlpha &as,
                                                   double beta, const double *cold)
{
    bool bad = false;
#pragma unroll
    for (int j = 0; j < N; j++) {
        const int e = erow + ecol[j] + (POW2 ? as.ea : 0);
        int ebh, ebl;
        double dh = oz_i53_ldexp(vh[j], e + lsh, ebh);
        double dl = oz_i53_ldexp(vl[j], e, ebl);
        bad |= (unsigned)(ebh - 1) > 2044u || (unsigned)(ebl - 1) > 2044u;
        double r;
        if constexpr (POW2) {
            dh = __longlong_as_double(__double_as_longlong(dh) ^ (long long)as.sign);
            dl = __longlong_as_double(__double_as_longlong(dl) ^ (long long)as.sign);
            r = dh + dl;
        } else {
            r = alpha * (dh + dl);
        }
        res[j] = BETA ? fma(beta, cold[j], r) : r;
    }
    return bad;
}

// oz_result_split out of line, for the rare segments oz_convert_segment
// leaves (inlined at each element of a drain thread, the 128-bit route
// raised the register count past the small-K kernel's budget)
__device__ __noinline__ double oz_result_split_slow(long long vh, long long vl, int lsh, int e, double alpha,
                                                    OzAlpha as, double beta, double cold)
{
    return oz_result_split(vh, vl, lsh, e, alpha, as, beta, cold);
}

// Tile order of the wide-tile kernel: groups of OZ_GROUP_M row tiles, the
// row tile fastest within a group, so the 152 tiles resident at once form an
// 8 x 19 block (at 8192^2) instead of all 64 row tiles of two or three
// column tiles.  The slice tiles that block streams per K step are about a
// third fewer, and each A tile is shared by 19 CTAs instead of two or three
// (the CTAs progress through K at about the same pace, so shared tiles are
// read from L2).
constexpr int OZ_GROUP_M = 8;
__device__ __forceinline__ void oz_tile_coords(int t, int tiles_m, int tiles_n, int &tm, int &tn)
{
    const int per_group = OZ_GROUP_M * tiles_n;
    const int g = t / per_group, r = t - g * per_group;
    const int rows = min(OZ_GROUP_M, tiles_m - g * OZ_GROUP_M);   // the last group may be shorter
    tm = g * OZ_GROUP_M + r % rows;
    tn = r / rows;
}

// Work unit u of the wide-tile kernel: whole tiles in the grouped order,
// then the tiles of the last, partial wave cut into two half-width tiles, so
// that wave runs on twice the SMs for half the time (2048 tiles of 128 x 256
// on 152 SMs: 13 full waves and one of 144 half tiles instead of a 14th wave
// of 72 tiles).  With B multicast (mrows = 2) a unit is a pair of vertically
// adjacent tiles and CTA rank r of the cluster takes row tile 2 tm + r.
// col_off: first column of the unit within its column tile.
__device__ __forceinline__ void oz_unit(const OzParams &p, int u, int bn, int mrows, int rank, int &tm, int &tn,
                                        int &col_off, bool &narrow)
{
    int t = u;
    narrow = u >= p.t_split;
    col_off = 0;
    if (narrow) {
        const int v = u - p.t_split;
        t = p.t_split + (v >> 1);
        col_off = (v & 1) * (bn / 2);
    }
    oz_tile_coords(t, p.tiles_m / mrows, p.tiles_n, tm, tn);
    tm = tm * mrows + rank;
}

__device__ __forceinline__ bool oz_unit_needed(const OzParams &p, int tm, int tn, int col_off, bool narrow, int bn)
{
    return narrow ? tile_needed(p, tm, 2 * tn + (col_off ? 1 : 0), OZ_BM, bn / 2) : tile_needed(p, tm, tn, OZ_BM, bn);
}

// Drain of the wide-tile kernel: diagonals arrive in ascending q (largest
// weight first) and each element's running value is one double, combined by
// Horner's rule: v = 32 v + D_q at the first accumulation group of diagonal
// q, v += D for that diagonal's further groups (D: the group's FP32 sum, an
// integer below 2^24, exact in a double).  The last group scales v by
// 2^(e_i + f_j - 8 - 5(S-1)) and writes C = alpha v 2^e + beta C.  Keeping v
// in 8 bytes instead of the exact 128-bit integer halves the running-sum
// traffic between diagonals, the kernel's largest DRAM stream (the sums of
// 152 resident 128 x 256 tiles do not stay in L2 next to the slices); each
// Horner step rounds once, relative to the partial value, so the result
// carries about S units of roundoff of |C| -- far below the target error of
// the slice truncation.
//
// One row (grow) and NCOL columns from gcol0 per call, walked in CH-column
// chunks and software-pipelined: the global loads of chunk c+1 (running
// values, and C on the last pass) are issued before chunk c is combined and
// stored.  Loads and stores are never interleaved element by element: the
// compiler cannot prove that W and C do not overlap, and a load/add/store
// per element serialised one L2 round trip per element.
template <int NCOL, int CH>
__device__ __forceinline__ void oz_drain_row_h(const OzParams &p, uint32_t taddr, int grow, int gcol0, int S,
                                               int rexp, bool first, bool new_diag, bool last)
{
    constexpr int NCH = NCOL / CH;
    const int erow = rexp - 5 * (S - 1);   // scale of v without the column part
    const bool row_ok = grow < p.M;
    const bool need_c = last && row_ok && p.beta != 0.0;
    const double *wrow = (const double *)p.W + (size_t)gcol0 * p.Mp + grow;
    double *crow = p.C + (size_t)gcol0 * p.ldc + grow;
    double wn[CH], cn[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) { wn[j] = 0.0; cn[j] = 0.0; }
    if (!first) {
#pragma unroll
        for (int j = 0; j < CH; j++) wn[j] = __ldcg(wrow + (size_t)j * p.Mp);
    }
    if (need_c) {
#pragma unroll
        for (int j = 0; j < CH; j++) cn[j] = oz_c_keep(p, grow, gcol0 + j) ? crow[(size_t)j * p.ldc] : 0.0;
    }
#pragma unroll 1
    for (int c = 0; c < NCH; c++) {
        double wc[CH], cc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) { wc[j] = wn[j]; cc[j] = cn[j]; }
        const int nc = (c + 1) * CH;
        if (c + 1 < NCH) {
            if (!first) {
#pragma unroll
                for (int j = 0; j < CH; j++) wn[j] = __ldcg(wrow + (size_t)(nc + j) * p.Mp);
            }
            if (need_c) {
#pragma unroll
                for (int j = 0; j < CH; j++)
                    cn[j] = oz_c_keep(p, grow, gcol0 + nc + j) ? crow[(size_t)(nc + j) * p.ldc] : 0.0;
            }
        }
        uint32_t r[CH];
        tmem_ld_chunk<CH>(taddr + (uint32_t)(c * CH), r);
        tmem_ld_wait();
        const int cb = c * CH;
#pragma unroll
        for (int j = 0; j < CH; j++) {
            const double d = oz_f32_to_f64(r[j]);
            wc[j] = first ? d : (new_diag ? fma(wc[j], 32.0, d) : wc[j] + d);
        }
        if (!last) {
            double *wdst = (double *)p.W + (size_t)(gcol0 + cb) * p.Mp + grow;
#pragma unroll
            for (int j = 0; j < CH; j++) __stcg(wdst + (size_t)j * p.Mp, wc[j]);
        } else if (row_ok) {
            const bool beta_on = p.beta != 0.0;
#pragma unroll
            for (int j = 0; j < CH; j++) {
                const int gcol = gcol0 + cb + j;
                if (!oz_c_keep(p, grow, gcol)) continue;
                const int e = erow + __ldg(p.col_exp + gcol);
                // alpha 2^e exactly (an exponent-field add) when it stays normal,
                // else scale v itself first (results near the underflow threshold)
                const double r0 = (e >= -1000 && e <= 1000) ? oz_alpha_pow2(p.alpha, e) * wc[j]
                                                             : p.alpha * ldexp(wc[j], e);
                crow[(size_t)(cb + j) * p.ldc] = beta_on ? fma(p.beta, cc[j], r0) : r0;
            }
        }
    }
}

// 1-CTA MMA kernel, BM = 128 rows by BN = 256 or 128 columns.  Warp 0
// issues the TMA loads, warp 1 the MMAs, warps 2..9 drain: two warps per
// TMEM lane quarter (a warp may only read the 32 TMEM lanes of its rank
// within its warpgroup), each taking half of the tile's columns.  TMEM holds
// 512/BN accumulator buffers, so the MMAs run up to that many diagonal
// groups ahead of the drain.
//
// MC (B multicast): CTAs run in clusters of two on vertically adjacent
// tiles that share their B slice tile.  Each CTA loads its own A tile and
// half of the B tile, multicast into both CTAs' shared memory, so an SM
// pulls 32 KB from L2 per K step instead of 48 KB; the tensor pipe of the
// one-CTA form waited on its loads about 30 % of the time.  A stage is free
// again once both CTAs' MMAs have read it (each MMA commit arrives on both
// CTAs' empty barrier).
constexpr int OZ_WBK = 128;   // K block of the wide-tile kernel, in digits (bytes per tile row)
template <int BN>
struct OzCfg {
    static constexpr int NBUF = 512 / BN;
    static constexpr int BK = OZ_WBK;
    static constexpr int A_BYTES = OZ_BM * BK;
    static constexpr int B_BYTES = BN * BK;
    static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
    // as many stages as the opt-in shared memory holds (the loads in flight
    // are what hide the L2/DRAM latency: three stages ran 10 % slower than four)
    static constexpr int STAGES = (227 * 1024 - 1024 - 512) / STAGE_BYTES < 16
                                      ? (227 * 1024 - 1024 - 512) / STAGE_BYTES : 16;
    static constexpr int EPI_WARPS = 8;
    static constexpr int THREADS = 64 + 32 * EPI_WARPS;
    static constexpr int DRAIN_COLS = BN / 2;
    static constexpr int DRAIN_CH = 8;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024 /*align*/ + 512 /*barriers*/;
    static_assert((2 * STAGES + 2 * NBUF) * 8 + 4 <= 512, "barriers and the TMEM slot fit their region");
    static_assert(SMEM <= 227 * 1024, "opt-in shared memory");
};

template <int BN, bool MC>
__global__ void __launch_bounds__(OzCfg<BN>::THREADS, 1)
oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               const __grid_constant__ CUtensorMap tmBh, OzParams p)
{
    if (oz_skip_kernel(p)) {
        oz_report(p);
        return;
    }
    using Cfg = OzCfg<BN>;
    constexpr int STAGES = Cfg::STAGES, NBUF = Cfg::NBUF, STAGE_BYTES = Cfg::STAGE_BYTES;
    constexpr int MROWS = MC ? 2 : 1;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + STAGES;
    uint64_t *tfull = bars + 2 * STAGES, *tempty = tfull + NBUF;
    uint32_t *tmem_slot = (uint32_t *)(tempty + NBUF);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rank = MC ? (int)(cluster_ctarank() & 1u) : 0;
    const int unit0 = MC ? (int)blockIdx.x >> 1 : (int)blockIdx.x;
    const int ustep = MC ? (int)gridDim.x >> 1 : (int)gridDim.x;
    volatile int *status = p.status;

    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; i++) { mbar_init(&full[i], 1); mbar_init(&empty[i], MROWS); }
        for (int i = 0; i < NBUF; i++) { mbar_init(&tfull[i], 1); mbar_init(&tempty[i], 32 * Cfg::EPI_WARPS); }
        fence_barrier_init();
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmB);
        prefetch_tmap(&tmBh);
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    if (MC) cluster_sync();   // the peer's barriers are initialised before any multicast reaches them
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    GroupPlan gp;
    gp.init(*p.S, p.Kp, Cfg::BK);

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int u = unit0; u < p.nunits && ok; u += ustep) {
                int tm, tn, col_off;
                bool narrow;
                oz_unit(p, u, BN, MROWS, rank, tm, tn, col_off, narrow);
                if (!MC && !oz_unit_needed(p, tm, tn, col_off, narrow, BN)) continue;
                const CUtensorMap *mb = narrow ? &tmBh : &tmB;
                const int bytes = Cfg::A_BYTES + (narrow ? Cfg::B_BYTES / 2 : Cfg::B_BYTES);
                // with MC each CTA brings this share of the unit's B rows to both CTAs
                const int b_rows = (narrow ? BN / 2 : BN) / MROWS;
                for (int q = 0; q < gp.S && ok; q++) {
                    const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                    const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                    for (int it = 0; it < nitems && ok; it++) {
                        const int s = s_lo + it / gp.nchunks, t2 = q - s, ch = it % gp.nchunks;
                        const int kb0 = ch * gp.kch_blocks, kb1 = min(gp.nkb, kb0 + gp.kch_blocks);
                        for (int kb = kb0; kb < kb1; kb++) {
                            if (!mbar_wait(&empty[stage], phase ^ 1u, status, TC_TIMEOUT_EMPTY)) { ok = false; break; }
                            uint8_t *sa = smem + stage * STAGE_BYTES;
                            mbar_arrive_expect_tx(&full[stage], (uint32_t)bytes);
                            tma_load_2d(sa, &tmA, &full[stage], kb * Cfg::BK, s * p.Mp + tm * OZ_BM);
                            if (MC)
                                tma_load_2d_mc(sa + Cfg::A_BYTES + rank * b_rows * Cfg::BK, mb, &full[stage],
                                               kb * Cfg::BK, t2 * p.Np + tn * BN + col_off + rank * b_rows,
                                               (uint16_t)3u);
                            else
                                tma_load_2d(sa + Cfg::A_BYTES, mb, &full[stage], kb * Cfg::BK,
                                            t2 * p.Np + tn * BN + col_off);
                            if (++stage == STAGES) { stage = 0; phase ^= 1u; }
                        }
                    }
                }
            }
            // drain: wait (bounded) until every issued load has landed and, with
            // MC, both CTAs' MMAs are done with every stage
            for (int i = 0; i < STAGES; i++) {
                mbar_wait(&empty[stage], phase ^ 1u, status, TC_TIMEOUT_EMPTY);
                if (++stage == STAGES) { stage = 0; phase ^= 1u; }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int stage = 0, buf = 0;
            uint32_t phase = 0, tphase = 0;
            bool ok = true;
            const uint32_t smem_base = smem_u32(smem);
            for (int u = unit0; u < p.nunits && ok; u += ustep) {
                int tm, tn, col_off;
                bool narrow;
                oz_unit(p, u, BN, MROWS, rank, tm, tn, col_off, narrow);
                if (!MC && !oz_unit_needed(p, tm, tn, col_off, narrow, BN)) continue;
                const uint32_t idesc = narrow ? idesc_e4m3_f32(OZ_BM, BN / 2) : idesc_e4m3_f32(OZ_BM, BN);
                for (int q = 0; q < gp.S && ok; q++) {
                    const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                    const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                    const int ng = gp.ngroups(nitems);
                    for (int g = 0; g < ng && ok; g++) {
                        const int g0 = gp.gbegin(nitems, ng, g), g1 = gp.gbegin(nitems, ng, g + 1);
                        if (!mbar_wait(&tempty[buf], tphase ^ 1u, status, TC_TIMEOUT_TMEM_EMPTY)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
                        uint32_t acc = 0;
                        for (int it = g0; it < g1 && ok; it++) {
                            const int ch = it % gp.nchunks;
                            const int kb0 = ch * gp.kch_blocks, kb1 = min(gp.nkb, kb0 + gp.kch_blocks);
                            for (int kb = kb0; kb < kb1; kb++) {
                                if (!mbar_wait(&full[stage], phase, status, TC_TIMEOUT_FULL)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t a_addr = smem_base + stage * STAGE_BYTES;
                                // descriptors built once per stage, advanced by 32 bytes
                                // (2 in the address field) per k step
                                const uint64_t a_d = smem_desc_kmaj<Cfg::BK>(a_addr);
                                const uint64_t b_d = smem_desc_kmaj<Cfg::BK>(a_addr + Cfg::A_BYTES);
#pragma unroll
                                for (int kk = 0; kk < Cfg::BK / 32; kk++) {
                                    mma_f8f6f4(d_tmem, a_d + 2 * kk, b_d + 2 * kk, idesc, acc);
                                    acc = 1;
                                }
                                if (MC) mma_commit_mc(&empty[stage], (uint16_t)3u);
                                else mma_commit(&empty[stage]);
                                if (++stage == STAGES) { stage = 0; phase ^= 1u; }
                            }
                        }
                        mma_commit(&tfull[buf]);
                        if (++buf == NBUF) { buf = 0; tphase ^= 1u; }
                    }
                }
            }
        }
    } else {
        // ---------------- drain (warps 2..9) ----------------
        const int quarter = warp & 3;               // TMEM lane window of this warp
        const int half = (warp - 2) >> 2;           // which half of the unit's columns
        const int row = quarter * 32 + lane;
        int buf = 0;
        uint32_t tphase = 0;
        bool ok = true;
        for (int u = unit0; u < p.nunits && ok; u += ustep) {
            int tm, tn, col_off;
            bool narrow;
            oz_unit(p, u, BN, MROWS, rank, tm, tn, col_off, narrow);
            if (!MC && !oz_unit_needed(p, tm, tn, col_off, narrow, BN)) continue;
            const int dcols = narrow ? Cfg::DRAIN_COLS / 2 : Cfg::DRAIN_COLS;
            const int grow = tm * OZ_BM + row;
            const int rexp = p.row_exp[grow];
            bool first = true;
            for (int q = 0; q < gp.S && ok; q++) {
                const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                const int ng = gp.ngroups(nitems);
                for (int g = 0; g < ng && ok; g++) {
                    const bool last = (q == gp.S - 1) && (g == ng - 1);
                    // warp-uniform outcome: tcgen05.ld below is .sync.aligned
                    ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tphase, status, TC_TIMEOUT_TMEM_FULL));
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t taddr = tmem_base + ((uint32_t)(quarter * 32) << 16) +
                                           (uint32_t)(buf * BN + half * dcols);
                    const int gcol0 = tn * BN + col_off + half * dcols;
                    if (narrow)
                        oz_drain_row_h<Cfg::DRAIN_COLS / 2, Cfg::DRAIN_CH>(p, taddr, grow, gcol0, gp.S, rexp, first,
                                                                          g == 0, last);
                    else
                        oz_drain_row_h<Cfg::DRAIN_COLS, Cfg::DRAIN_CH>(p, taddr, grow, gcol0, gp.S, rexp, first,
                                                                      g == 0, last);
                    tc_fence_before();
                    mbar_arrive(&tempty[buf]);
                    first = false;
                    if (++buf == NBUF) { buf = 0; tphase ^= 1u; }
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (MC) cluster_sync();   // no CTA leaves while its peer may still write to it
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
    oz_report(p);
}

// ---------------------------------------------------------------------------
// Small-K kernel: every diagonal accumulator resident in TMEM
// ---------------------------------------------------------------------------
// For Kp <= 1024 each diagonal sum over the whole K extent is an integer of
// magnitude below 14 * 1024 * 16 * 16 < 2^22, exact in one FP32 accumulator,
// so a 128 x 32 tile keeps all S (<= 14) diagonal sums in TMEM at once:
// diagonal q in columns [32q, 32q + 32).  One drain per tile combines the S
// sums exactly in registers and writes C: no running-sum traffic and no
// per-diagonal hand-off between the MMA issuer and the drain.
//
// The B slices of one k block are loaded side by side, B_0..B_{S-1} as the
// rows 32t..32t+31 of one S*32 x 128-byte stage.  Then a single MMA of
// N = 32(S - s) columns multiplies A_s by B_0..B_{S-1-s} at once and writes
// A_s B_t into columns 32(s + t): exactly diagonal s + t's accumulator.  A
// tcgen05.mma costs the issuing thread about 70 cycles whatever its N up to
// 128 (N = 256: 128 cycles; measured by gbx_diag_mma_issue), so S(S+1)/2 products of
// N = 32 would leave the tensor pipe three quarters idle; concatenated, a
// 128-wide k block of a tile is sum_s ceil(32(S - s) / 256) * 4 MMAs (48 for
// S = 10 instead of 220).  The A slices (16 KB each) stream through a ring
// of up to eight stages: an A slice whose product has a narrow N is used
// up in a few hundred cycles, so with K > 128 the ring depth, not the tensor
// pipe, set the pace at four stages.  The B stage is double-buffered so the
// next k block's (or tile's) slices load under the current MMAs.  A TMA
// request costs the issuing thread about 80 ns, so a B stage (all P
// prepared planes, of which the MMAs read the first S) is one 3-D request,
// and the first tile's B stage and first A slices are requested before the
// slice count is chosen (S >= s_lo from the tolerance alone).
//
// The drain prefetches its row's C values and scale exponents while the
// MMAs run, then decodes each FP32 sum on the FMA and integer pipes (oz_f2i22)
// and folds diagonals by Horner's rule, V = (...(D_0 * 32 + D_1) * 32 ...) +
// D_{S-1}, in two signed 64-bit halves (diagonals 0..g-1 and g..S-1, g =
// ceil(S/2): at most seven each, |half| < 2^22 * 32^6 * 1.04 < 2^53); each
// half converts exactly to a double on the integer pipe and one FP64 addition
// rounds V once (oz_result_split).  Tiles are ordered column-fastest so the
// CTAs sharing an A row block run together and its slices come from L2.
// Warp 0: TMA; warp 1: MMA issuer; warps 2..17: drain (four per TMEM lane
// quarter, BN/4 columns each: the per-element conversion work of one tile is
// what bounds a CTA with several tiles, so it gets most of the warps).  The
// accumulators are released before C is written, so the next tile's MMAs
// overlap that work.
// Tiles are 128 x BN, BN = 32, or 16 when the 32-wide tiles would occupy at
// most half the SMs: a call that small is one tile per CTA, and its time is
// the tile's chain (loads, MMAs, drain); half-width tiles halve the drain
// (the longest step: 8 conversions per thread) and double the CTAs at work.
constexpr int OZS_BN = 32, OZS_AMAX = 8, OZS_BSTG = 2, OZS_DRAIN_WARPS = 16;
constexpr int OZS_B_BYTES = OZS_BN * OZ_BK;                 // 4 KB: one slice's 32 rows (BN = 32)
constexpr int OZS_THREADS = 64 + 32 * OZS_DRAIN_WARPS;
// Dynamic shared memory: the two B stages (S x 4 KB each) and as many 16 KB
// A stages as fit (8 for S <= 10, 6 for S = 14), barriers at the end.
constexpr size_t OZS_SMEM = 220 * 1024;
constexpr size_t OZS_DATA = OZS_SMEM - 1024 - 512;   // alignment slack, barriers
static_assert(OZS_DATA >= 2 * OZ_SMAX * OZS_B_BYTES + 4 * (size_t)OZ_A_BYTES, "small-K stages");
constexpr int OZS_KMAX = 1024;
static_assert((long long)OZ_SMAX * OZS_KMAX * 256 < (1LL << 22), "small-K diagonal sums must stay below 2^22");
static_assert(OZ_SMAX * OZS_BN <= 512, "small-K accumulators must fit TMEM");

template <int BN>
__global__ void __launch_bounds__(OZS_THREADS, 1)
oz_gemm_sk_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, OzParams p)
{
    static_assert(BN == 16 || BN == 32, "tile width: MMA N = BN (S - s) must be a multiple of 16");
    constexpr int DCOLS = BN / (OZS_DRAIN_WARPS / 4);   // columns per drain thread
    constexpr int B_BYTES = BN * OZ_BK;                 // one slice's BN rows
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + OZS_DATA);
    uint64_t *fullA = bars, *emptyA = fullA + OZS_AMAX;
    uint64_t *fullB = emptyA + OZS_AMAX, *emptyB = fullB + OZS_BSTG;
    uint64_t *tfull = emptyB + OZS_BSTG, *tempty = tfull + 2;   // two accumulator sets
    uint32_t *tmem_slot = (uint32_t *)(tempty + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int *status = p.status;

    if (threadIdx.x == 0) {
        for (int i = 0; i < OZS_AMAX; i++) { mbar_init(&fullA[i], 1); mbar_init(&emptyA[i], 1); }
        for (int i = 0; i < OZS_BSTG; i++) { mbar_init(&fullB[i], 1); mbar_init(&emptyB[i], 1); }
        for (int i = 0; i < 2; i++) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 32 * OZS_DRAIN_WARPS);
        }
        fence_barrier_init();
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmB);
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // Launched as a programmatic dependent of the preparation: the set-up
    // above overlaps its tail; its slices, scales and S are complete and
    // visible after this wait (a no-op for an ordinary launch).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int P = p.smax;   // digit planes prepared: S <= P
    const int nkb = p.Kp / OZ_BK;
    // B stages first (all P slices of BN rows each: a stage can be requested
    // before S is known; the MMAs read the first S), then the A ring
    const int bstage = P * B_BYTES;
    uint8_t *sB = smem;
    uint8_t *sA = smem + OZS_BSTG * bstage;
    const int nA = min(OZS_AMAX, (int)((OZS_DATA - (size_t)OZS_BSTG * bstage) / OZ_A_BYTES));
    const int ntiles = p.tiles_m * p.tiles_n;
    // The first tile's first B stage and A slices 0..spec-1 (S >= p.s_lo, a
    // bound from the tolerance alone) are requested before the slice count
    // is chosen, so that these loads overlap the choice.
    int t_first = -1, spec = 0;
    if (warp == 0 && lane == 0) {
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
            if (tile_needed(p, t / p.tiles_n, t % p.tiles_n, OZ_BM, BN)) { t_first = t; break; }
        if (t_first >= 0) {
            const int tm = t_first / p.tiles_n, tn = t_first % p.tiles_n;
            spec = min(min(nA, p.s_lo), 3);   // a TMA request costs the thread ~80 ns
            mbar_arrive_expect_tx(&fullB[0], (uint32_t)(P * B_BYTES));
            tma_load_3d(sB, &tmB, &fullB[0], 0, tn * BN, 0);
            for (int sa = 0; sa < spec; sa++) {
                mbar_arrive_expect_tx(&fullA[sa], OZ_A_BYTES);
                tma_load_2d(sA + sa * OZ_A_BYTES, &tmA, &fullA[sa], 0, sa * p.Mp + tm * OZ_BM);
            }
        }
    }
    const int S = oz_choose_S(p);   // 0: skip this call
    if (S == 0) {
        // the early loads land before the CTA leaves (a wait bounded by time
        // only: the status word is set on this path)
        if (warp == 0 && lane == 0 && t_first >= 0) {
            const uint64_t t0 = globaltimer();
            while (!mbar_try_wait(&fullB[0], 0u) && globaltimer() - t0 < WAIT_LIMIT_NS) {}
            for (int sa = 0; sa < spec; sa++)
                while (!mbar_try_wait(&fullA[sa], 0u) && globaltimer() - t0 < WAIT_LIMIT_NS) {}
        }
        if (warp == 1) {
            tc_fence_after();
            tmem_dealloc(tmem_base, 512);
        }
        __syncthreads();
        oz_report(p);
        return;
    }
    // Accumulator sets in TMEM: two of 256 columns when a tile's S diagonals
    // fit (S * BN <= 256: always for BN = 16), so that a tile's MMAs run while
    // the previous tile's sums are read out; else one
    const int nbuf = S * BN <= 256 ? 2 : 1;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            int as = 0, bs = 0;
            uint32_t ap = 0, bp = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int tm = t / p.tiles_n, tn = t % p.tiles_n;
                if (!tile_needed(p, tm, tn, OZ_BM, BN)) continue;
                for (int kb = 0; kb < nkb && ok; kb++) {
                    // requested before the slice count was chosen
                    const bool early = t == t_first && kb == 0;
                    // the B stage: slices 0..P-1 of the tile's BN columns, side by side
                    if (!early) {
                        if (!mbar_wait(&emptyB[bs], bp ^ 1u, status, TC_TIMEOUT_EMPTY)) { ok = false; break; }
                        mbar_arrive_expect_tx(&fullB[bs], (uint32_t)(P * B_BYTES));
                        tma_load_3d(sB + bs * bstage, &tmB, &fullB[bs], kb * OZ_BK, tn * BN, 0);   // P planes
                    }
                    if (++bs == OZS_BSTG) { bs = 0; bp ^= 1u; }
                    // then the A slices
                    for (int sa = 0; sa < S; sa++) {
                        if (!(early && sa < spec)) {
                            if (!mbar_wait(&emptyA[as], ap ^ 1u, status, TC_TIMEOUT_EMPTY)) { ok = false; break; }
                            mbar_arrive_expect_tx(&fullA[as], OZ_A_BYTES);
                            tma_load_2d(sA + as * OZ_A_BYTES, &tmA, &fullA[as], kb * OZ_BK, sa * p.Mp + tm * OZ_BM);
                        }
                        if (++as == nA) { as = 0; ap ^= 1u; }
                    }
                }
            }
            // wait (bounded) until every issued load has been consumed
            for (int i = 0; i < nA; i++) {
                mbar_wait(&emptyA[as], ap ^ 1u, status, TC_TIMEOUT_EMPTY);
                if (++as == nA) { as = 0; ap ^= 1u; }
            }
            for (int i = 0; i < OZS_BSTG; i++) {
                mbar_wait(&emptyB[bs], bp ^ 1u, status, TC_TIMEOUT_EMPTY);
                if (++bs == OZS_BSTG) { bs = 0; bp ^= 1u; }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int as = 0, bs = 0, tbuf = 0;
            uint32_t ap = 0, bp = 0, tp = 0;
            bool ok = true;
            const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int tm = t / p.tiles_n, tn = t % p.tiles_n;
                if (!tile_needed(p, tm, tn, OZ_BM, BN)) continue;
                // this accumulator set's previous sums have been read out of TMEM
                if (!mbar_wait(&tempty[tbuf], tp ^ 1u, status, TC_TIMEOUT_TMEM_EMPTY)) { ok = false; break; }
                tc_fence_after();
                for (int kb = 0; kb < nkb && ok; kb++) {
                    if (!mbar_wait(&fullB[bs], bp, status, TC_TIMEOUT_FULL)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t b_addr = b_base + bs * bstage;
                    for (int sa = 0; sa < S; sa++) {
                        if (!mbar_wait(&fullA[as], ap, status, TC_TIMEOUT_FULL)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t a_addr = a_base + as * OZ_A_BYTES;
                        // A_s against B_0..B_{S-1-s}: columns BN s.. of TMEM, N <= 256 per MMA.
                        // Descriptors are built once per stage and advanced by 32 bytes
                        // (2 in the address field) per k step: the issuing thread shares
                        // its SMSP with four drain warps, so its instructions are few.
                        const uint64_t a_d = smem_desc_k128(a_addr);
                        // the first k block's s = 0 products start every diagonal
                        const uint32_t acc0 = (kb == 0 && sa == 0) ? 0u : 1u;
                        const int ntot = BN * (S - sa);
                        for (int c0 = 0; c0 < ntot; c0 += 256) {
                            const int n = min(256, ntot - c0);
                            const uint32_t idesc = idesc_e4m3_f32(OZ_BM, n);
                            const uint32_t d_tmem = tmem_base + (uint32_t)(tbuf * 256 + BN * sa + c0);
                            const uint64_t b_d = smem_desc_k128(b_addr + (uint32_t)c0 * OZ_BK);
#pragma unroll
                            for (int kk = 0; kk < OZ_BK / 32; kk++)
                                mma_f8f6f4(d_tmem, a_d + 2 * kk, b_d + 2 * kk, idesc, kk == 0 ? acc0 : 1u);
                        }
                        mma_commit(&emptyA[as]);
                        if (++as == nA) { as = 0; ap ^= 1u; }
                    }
                    if (!ok) break;
                    mma_commit(&emptyB[bs]);
                    if (++bs == OZS_BSTG) { bs = 0; bp ^= 1u; }
                }
                if (!ok) break;
                mma_commit(&tfull[tbuf]);
                if (++tbuf == nbuf) { tbuf = 0; tp ^= 1u; }
            }
        }
    } else {
        // ---------------- drain (warps 2..17) ----------------
        const int quarter = warp & 3;               // TMEM lane window of this warp
        const int cg = (warp - 2) >> 2;             // columns cg*DCOLS .. of the tile
        const int row = quarter * 32 + lane;
        const OzAlpha as = oz_alpha_split(p.alpha, p.beta);
        const int g = (S + 1) >> 1;                 // diagonals of the high half
        const int lsh = 5 * (S - g);                // weight of the high half over the low one
        uint32_t tp = 0;
        int tbuf = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            const int tm = t / p.tiles_n, tn = t % p.tiles_n;
            if (!tile_needed(p, tm, tn, OZ_BM, BN)) continue;
            // this row's C values and scale exponents, loaded while the MMAs run
            const int grow = tm * OZ_BM + row;
            const bool row_ok = grow < p.M;
            const int gc0 = tn * BN + cg * DCOLS;
            double *cp = p.C + (size_t)gc0 * p.ldc + grow;
            double cold[DCOLS];
            int ecol[DCOLS];
#pragma unroll
            for (int j = 0; j < DCOLS; j++) {
                cold[j] = (row_ok && as.beta_on && oz_c_keep(p, grow, gc0 + j)) ? cp[(size_t)j * p.ldc] : 0.0;
                ecol[j] = __ldg(p.col_exp + gc0 + j);
            }
            const int erow = row_ok ? p.row_exp[grow] - 5 * (S - 1) : 0;

            ok = __all_sync(0xffffffffu, mbar_wait(&tfull[tbuf], tp, status, TC_TIMEOUT_TMEM_FULL));
            if (!ok) break;
            tc_fence_after();
            const int cur = tbuf;
            if (++tbuf == nbuf) { tbuf = 0; tp ^= 1u; }
            long long vh[DCOLS], vl[DCOLS];
#pragma unroll
            for (int j = 0; j < DCOLS; j++) { vh[j] = 0; vl[j] = 0; }
            const uint32_t tbase =
                tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(cur * 256 + cg * DCOLS);
            // diagonals qa and qa + 1 into the halves (q < g: high)
            auto fold2 = [&](int qa, const uint32_t (&ra)[DCOLS], const uint32_t (&rb)[DCOLS]) {
                if (qa + 1 < g) {
                    oz_horner2(vh, ra, rb);
                } else if (qa >= g) {
                    if (qa + 1 < S) oz_horner2(vl, ra, rb);
                    else if (qa < S) oz_horner(vl, ra);
                } else {   // qa = g - 1
                    oz_horner(vh, ra);
                    if (qa + 1 < S) oz_horner(vl, rb);
                }
            };
            // G diagonals per TMEM round trip (as many as the registers allow);
            // q < g folds into the high half
            if constexpr (DCOLS <= 4) {
                constexpr int G = 4;
                for (int q = 0; q < S; q += G) {
                    uint32_t r[G][DCOLS];
#pragma unroll
                    for (int i = 0; i < G; i++)
                        if (q + i < S) tmem_ld_chunk<DCOLS>(tbase + (uint32_t)((q + i) * BN), r[i]);   // uniform
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < G; i += 2) fold2(q + i, r[i], r[i + 1]);
                }
            } else {
                for (int q = 0; q < S; q += 2) {
                    uint32_t r0[DCOLS], r1[DCOLS];
                    tmem_ld_chunk<DCOLS>(tbase + (uint32_t)(q * BN), r0);
                    if (q + 1 < S) tmem_ld_chunk<DCOLS>(tbase + (uint32_t)((q + 1) * BN), r1);
                    tmem_ld_wait();
                    fold2(q, r0, r1);
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[cur]);   // this set free: a later tile's MMAs may use it
            // The next tile's C segment goes into L1 now: its MMAs overlap
            // this tile's conversion, so at its turn the loads of C would
            // otherwise wait on L2 with nothing to overlap them.
            if (as.beta_on && t + (int)gridDim.x < ntiles) {
                const int t2 = t + (int)gridDim.x;
                const int grow2 = (t2 / p.tiles_n) * OZ_BM + row;
                const int gc2 = (t2 % p.tiles_n) * BN + cg * DCOLS;
                if (grow2 < p.M) {
                    const double *cp2 = p.C + (size_t)gc2 * p.ldc + grow2;
#pragma unroll
                    for (int j = 0; j < DCOLS; j++)
                        if (oz_c_keep(p, grow2, gc2 + j))
                            asm volatile("prefetch.global.L1 [%0];" ::"l"(cp2 + (size_t)j * p.ldc));
                }
            }
            if (row_ok) {
                // V = vh * 2^lsh + vl, converted and stored four elements at a
                // time (fewer values live at once: no spills at 96 registers)
                constexpr int SEG = DCOLS < 4 ? DCOLS : 4;
#pragma unroll
                for (int h = 0; h < DCOLS; h += SEG) {
                    double res[SEG];
                    bool bad;
                    if (as.pow2)
                        bad = as.beta_on ? oz_convert_segment<true, true, SEG>(res, vh + h, vl + h, lsh, erow, ecol + h,
                                                                              p.alpha, as, p.beta, cold + h)
                                         : oz_convert_segment<true, false, SEG>(res, vh + h, vl + h, lsh, erow, ecol + h,
                                                                               p.alpha, as, p.beta, cold + h);
                    else
                        bad = as.beta_on ? oz_convert_segment<false, true, SEG>(res, vh + h, vl + h, lsh, erow, ecol + h,
                                                                               p.alpha, as, p.beta, cold + h)
                                         : oz_convert_segment<false, false, SEG>(res, vh + h, vl + h, lsh, erow,
                                                                                ecol + h, p.alpha, as, p.beta, cold + h);
                    if (bad) {   // a part outside the normal range: the 128-bit route
#pragma unroll
                        for (int j = 0; j < SEG; j++)
                            res[j] = oz_result_split_slow(vh[h + j], vl[h + j], lsh, erow + ecol[h + j], p.alpha, as,
                                                          p.beta, cold[h + j]);
                    }
#pragma unroll
                    for (int j = 0; j < SEG; j++)
                        if (oz_c_keep(p, grow, gc0 + h + j)) cp[(size_t)(h + j) * p.ldc] = res[j];
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
    oz_report(p);
}

// ---------------------------------------------------------------------------
// CTA-pair variant (tcgen05 cta_group::2): a cluster of two CTAs on two SMs
// computes a 256x256 tile with M=256 MMAs issued by the even CTA.  Each CTA
// loads its own 128 rows of the A slice and its own 128 rows of the B slice
// (half of N), so every SM moves 32 KB per k-block instead of 48 KB for the
// same tensor work, and seven stages fit in shared memory.  Each CTA's TMEM
// holds its 128 rows x 256 columns of the accumulator (two buffers); eight
// drain warps per CTA take them as the one-CTA kernel does (two warps per
// TMEM lane quarter, each half of the columns), with the same Horner drain,
// diagonals in ascending order and the same grouped tile order.
//   full[s]   (even CTA): its producer arrives expecting both CTAs' 64 KB;
//             both CTAs' TMA loads complete on it (cta_group::2 TMA)
//   empty[s]  (each CTA): arrived by the MMA commit, multicast to both CTAs
//   tfull[b]  (each CTA): arrived by the MMA commit, multicast to both CTAs
//   tempty[b] (even CTA): the 512 drain threads of both CTAs arrive
// ---------------------------------------------------------------------------
constexpr int OZ2_BM = 256, OZ2_STAGES = 7;

// Whether a unit of the CTA-pair kernel (a 256-row tile or half of one) has
// any element in the written part of C.
__device__ __forceinline__ bool oz_pair_unit_needed(const OzParams &p, int tm, int tn, int col_off, bool narrow)
{
    return narrow ? tile_needed(p, tm, 2 * tn + (col_off ? 1 : 0), OZ2_BM, OZ_BN / 2)
                  : tile_needed(p, tm, tn, OZ2_BM, OZ_BN);
}
constexpr int OZ2_HALF = 128 * OZ_BK;                // 16 KB: 128 rows x 128 bytes
constexpr int OZ2_STAGE_BYTES = 2 * OZ2_HALF;        // A half + B half
constexpr int OZ2_EPI_WARPS = 8;
constexpr int OZ2_THREADS = 64 + 32 * OZ2_EPI_WARPS;
constexpr size_t OZ2_SMEM = (size_t)OZ2_STAGES * OZ2_STAGE_BYTES + 1024 + 256;
static_assert(OZ2_SMEM <= 227 * 1024, "CTA-pair stages must fit the opt-in shared memory");

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(OZ2_THREADS, 1)
oz_gemm2_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const __grid_constant__ CUtensorMap tmBh, OzParams p)
{
    if (oz_skip_kernel(p)) {
        oz_report(p);
        return;
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + OZ2_STAGES * OZ2_STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + OZ2_STAGES;
    uint64_t *tfull = bars + 2 * OZ2_STAGES, *tempty = tfull + 2;
    uint32_t *tmem_slot = (uint32_t *)(tempty + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();
    const bool leader = (rank & 1u) == 0u;
    volatile int *status = p.status;

    if (threadIdx.x == 0) {
        for (int i = 0; i < OZ2_STAGES; i++) { mbar_init(&full[i], 1); mbar_init(&empty[i], 1); }
        for (int i = 0; i < 2; i++) { mbar_init(&tfull[i], 1); mbar_init(&tempty[i], 2 * 32 * OZ2_EPI_WARPS); }
        fence_barrier_init();
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmB);
        prefetch_tmap(&tmBh);
    }
    if (warp == 1) {
        tmem_alloc_pair(tmem_slot, 512);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    __syncthreads();
    cluster_sync();   // peers' barriers are initialised before any remote arrive
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const uint32_t leader_rank = rank & ~1u;

    GroupPlan gp;
    gp.init(*p.S, p.Kp);
    const int pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;

    if (warp == 0) {
        // ---------------- TMA producer (both CTAs) ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int u = pair; u < p.nunits && ok; u += npairs) {
                int tm, tn, col_off;
                bool narrow;
                oz_unit(p, u, OZ_BN, 1, 0, tm, tn, col_off, narrow);
                if (!oz_pair_unit_needed(p, tm, tn, col_off, narrow)) continue;
                const CUtensorMap *mb = narrow ? &tmBh : &tmB;
                const int b_rows = narrow ? OZ_BN / 4 : OZ_BN / 2;     // this CTA's share of the unit's B
                const uint32_t bytes = (uint32_t)(OZ2_HALF + b_rows * OZ_BK);
                for (int q = 0; q < gp.S && ok; q++) {
                    const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                    const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                    for (int it = 0; it < nitems && ok; it++) {
                        const int s = s_lo + it / gp.nchunks, t2 = q - s, ch = it % gp.nchunks;
                        const int kb0 = ch * gp.kch_blocks, kb1 = min(gp.nkb, kb0 + gp.kch_blocks);
                        for (int kb = kb0; kb < kb1; kb++) {
                            if (!mbar_wait_cl(&empty[stage], phase ^ 1u, status, TC_TIMEOUT_EMPTY)) { ok = false; break; }
                            uint8_t *sa = smem + stage * OZ2_STAGE_BYTES;
                            const uint32_t fbar = mapa_cluster(smem_u32(&full[stage]), leader_rank);
                            // only the even CTA arrives, expecting both CTAs' bytes: a
                            // remote arrive from the odd CTA per stage cut the load
                            // rate to a third
                            if (leader) mbar_arrive_expect_tx(&full[stage], 2u * bytes);
                            tma_load_2d_pair(sa, &tmA, fbar, kb * OZ_BK,
                                             s * p.Mp + tm * OZ2_BM + (int)(rank & 1u) * 128);
                            tma_load_2d_pair(sa + OZ2_HALF, mb, fbar, kb * OZ_BK,
                                             t2 * p.Np + tn * OZ_BN + col_off + (int)(rank & 1u) * b_rows);
                            if (++stage == OZ2_STAGES) { stage = 0; phase ^= 1u; }
                        }
                    }
                }
            }
            for (int i = 0; i < OZ2_STAGES; i++) {
                mbar_wait_cl(&empty[stage], phase ^ 1u, status, TC_TIMEOUT_EMPTY);
                if (++stage == OZ2_STAGES) { stage = 0; phase ^= 1u; }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (even CTA only) ----------------
        if (leader && lane == 0) {
            int stage = 0, buf = 0;
            uint32_t phase = 0, tphase = 0;
            bool ok = true;
            const uint32_t smem_base = smem_u32(smem);
            for (int u = pair; u < p.nunits && ok; u += npairs) {
                int tm, tn, col_off;
                bool narrow;
                oz_unit(p, u, OZ_BN, 1, 0, tm, tn, col_off, narrow);
                if (!oz_pair_unit_needed(p, tm, tn, col_off, narrow)) continue;
                const uint32_t idesc = narrow ? idesc_e4m3_f32(OZ2_BM, OZ_BN / 2) : idesc_e4m3_f32(OZ2_BM, OZ_BN);
                for (int q = 0; q < gp.S && ok; q++) {
                    const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                    const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                    const int ng = gp.ngroups(nitems);
                    for (int g = 0; g < ng && ok; g++) {
                        const int g0 = gp.gbegin(nitems, ng, g), g1 = gp.gbegin(nitems, ng, g + 1);
                        if (!mbar_wait_cl(&tempty[buf], tphase ^ 1u, status, TC_TIMEOUT_TMEM_EMPTY)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t d_tmem = tmem_base + (uint32_t)(buf * OZ_BN);
                        uint32_t acc = 0;
                        for (int it = g0; it < g1 && ok; it++) {
                            const int ch = it % gp.nchunks;
                            const int kb0 = ch * gp.kch_blocks, kb1 = min(gp.nkb, kb0 + gp.kch_blocks);
                            for (int kb = kb0; kb < kb1; kb++) {
                                if (!mbar_wait_cl(&full[stage], phase, status, TC_TIMEOUT_FULL)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t a_addr = smem_base + stage * OZ2_STAGE_BYTES;
                                const uint64_t a_d = smem_desc_k128(a_addr);
                                const uint64_t b_d = smem_desc_k128(a_addr + OZ2_HALF);
#pragma unroll
                                for (int kk = 0; kk < OZ_BK / 32; kk++) {
                                    mma_f8f6f4_pair(d_tmem, a_d + 2 * kk, b_d + 2 * kk, idesc, acc);
                                    acc = 1;
                                }
                                mma_commit_pair_mc(&empty[stage], (uint16_t)(3u << leader_rank));
                                if (++stage == OZ2_STAGES) { stage = 0; phase ^= 1u; }
                            }
                        }
                        mma_commit_pair_mc(&tfull[buf], (uint16_t)(3u << leader_rank));
                        if (++buf == 2) { buf = 0; tphase ^= 1u; }
                    }
                }
            }
        }
    } else {
        // ---------------- drain (warps 2..9, both CTAs) ----------------
        const int quarter = warp & 3;               // TMEM lane window of this warp
        const int half = (warp - 2) >> 2;           // which half of the tile's columns
        const int row = quarter * 32 + lane;
        int buf = 0;
        uint32_t tphase = 0;
        bool ok = true;
        const uint32_t tempty_cl0 = mapa_cluster(smem_u32(&tempty[0]), leader_rank);
        const uint32_t tempty_cl1 = mapa_cluster(smem_u32(&tempty[1]), leader_rank);
        for (int u = pair; u < p.nunits && ok; u += npairs) {
            int tm, tn, col_off;
            bool narrow;
            oz_unit(p, u, OZ_BN, 1, 0, tm, tn, col_off, narrow);
            if (!oz_pair_unit_needed(p, tm, tn, col_off, narrow)) continue;
            const int dcols = narrow ? OZ_BN / 4 : OZ_BN / 2;
            const int grow = tm * OZ2_BM + (int)(rank & 1u) * 128 + row;
            const int rexp = p.row_exp[grow];
            bool first = true;
            for (int q = 0; q < gp.S && ok; q++) {
                const int s_lo = max(0, q - (gp.S - 1)), s_hi = min(q, gp.S - 1);
                const int nitems = (s_hi - s_lo + 1) * gp.nchunks;
                const int ng = gp.ngroups(nitems);
                for (int g = 0; g < ng && ok; g++) {
                    const bool last = (q == gp.S - 1) && (g == ng - 1);
                    // warp-uniform outcome: tcgen05.ld below is .sync.aligned
                    ok = __all_sync(0xffffffffu, mbar_wait_cl(&tfull[buf], tphase, status, TC_TIMEOUT_TMEM_FULL));
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t taddr = tmem_base + ((uint32_t)(quarter * 32) << 16) +
                                           (uint32_t)(buf * OZ_BN + half * dcols);
                    const int gcol0 = tn * OZ_BN + col_off + half * dcols;
                    if (narrow)
                        oz_drain_row_h<OZ_BN / 4, 8>(p, taddr, grow, gcol0, gp.S, rexp, first, g == 0, last);
                    else
                        oz_drain_row_h<OZ_BN / 2, 8>(p, taddr, grow, gcol0, gp.S, rexp, first, g == 0, last);
                    tc_fence_before();
                    mbar_arrive_cluster(buf ? tempty_cl1 : tempty_cl0);
                    first = false;
                    if (++buf == 2) { buf = 0; tphase ^= 1u; }
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    cluster_sync();   // no CTA leaves while its peer may still signal its barriers
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc_pair(tmem_base, 512);
    }
    oz_report(p);
}

// complex combine: C = alpha*(Wr + i Wi) + beta*C
__global__ void oz_complex_combine(int M, int N, const double *__restrict__ Wr, const double *__restrict__ Wi,
                                   long long ldw, double ar, double ai, double br, double bi, double *C,
                                   long long ldc)
{
    const long long total = (long long)M * N;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % M), j = (int)(t / M);
        const double xr = Wr[(size_t)j * ldw + i], xi = Wi[(size_t)j * ldw + i];
        double *cp = C + 2 * ((size_t)j * ldc + i);
        double rr = ar * xr - ai * xi, ri = ar * xi + ai * xr;
        if (br != 0.0 || bi != 0.0) {
            const double cr = cp[0], ci = cp[1];
            rr += br * cr - bi * ci;
            ri += br * ci + bi * cr;
        }
        cp[0] = rr;
        cp[1] = ri;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

// 2-D byte tensor [rows][Kp] with a (box_rows x 128-byte) box, 128B swizzle.
bool make_map_uncached(CUtensorMap *map, void *base, long long rows, long long Kp, int box_rows, int inner)
{
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kp};
    cuuint32_t box[2] = {(cuuint32_t)inner, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               inner == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The digit planes as a 3-D tensor (k, row, plane): one load brings a
// box_rows-row block of box_planes consecutive planes (the small-K kernel's
// B stage in one request instead of one per plane).
bool make_map3_uncached(CUtensorMap *map, void *base, long long rows, long long Kp, int box_rows, int box_planes)
{
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)OZ_SMAX};
    cuuint64_t strides[2] = {(cuuint64_t)Kp, (cuuint64_t)(rows * Kp)};
    cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, (cuuint32_t)box_planes};
    cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, base, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The digit planes live in workspace slots that persist across calls, so a
// calling thread sees the same few (base, rows, K, box) over and over: the
// encoded maps are kept per thread (8 entries, round robin) instead of
// re-encoding two per call on the host.
bool make_map(CUtensorMap *map, void *base, long long rows, long long Kp, int box_rows, int inner = OZ_BK)
{
    struct Entry {
        void *base;
        long long rows, Kp;
        int box, inner;
        CUtensorMap map;
    };
    thread_local Entry cache[8] = {};
    thread_local int next = 0;
    for (auto &e : cache)
        if (e.base == base && e.rows == rows && e.Kp == Kp && e.box == box_rows && e.inner == inner) {
            *map = e.map;
            return true;
        }
    // box_rows < 0 asks for the 3-D form: -box_rows = rows x 256 + planes
    const bool three = box_rows < 0;
    if (three ? !make_map3_uncached(map, base, rows, Kp, (-box_rows) >> 8, (-box_rows) & 255)
              : !make_map_uncached(map, base, rows, Kp, box_rows, inner))
        return false;
    Entry &e = cache[next];
    next = (next + 1) & 7;
    e.base = base;
    e.rows = rows;
    e.Kp = Kp;
    e.box = box_rows;
    e.inner = inner;
    e.map = *map;
    return true;
}

// B multicast between cluster pairs of the wide-tile kernel is the default;
// GBX_OZAKI_MC=0 turns it off.
bool oz_use_mc()
{
    static int env = [] {
        const char *s = getenv("GBX_OZAKI_MC");
        return s ? atoi(s) : 1;
    }();
    return env != 0;
}

// Clusters of two of the wide-tile kernel resident at once on the context's
// device (clusters must fit in a GPC), once per device and tile width; the
// shared-memory attribute of the cluster instantiations is set then too.
int oz_mc_clusters(gbx_ctx *ctx, int bn)
{
    static std::mutex mu;
    static int cached[64][2] = {};
    const int dev = gbx_ctx_device(ctx), w = bn == 128 ? 0 : 1;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && cached[dev][w]) return cached[dev][w];
    const void *fn = bn == 128 ? (const void *)oz_gemm_kernel<128, true> : (const void *)oz_gemm_kernel<256, true>;
    const int smem = (int)(bn == 128 ? OzCfg<128>::SMEM : OzCfg<256>::SMEM);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * (unsigned)std::max(1, gbx_ctx_sms(ctx) / 2));
    cfg.blockDim = dim3(bn == 128 ? OzCfg<128>::THREADS : OzCfg<256>::THREADS);
    cfg.dynamicSmemBytes = (size_t)smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, fn, &cfg) != cudaSuccess || nc < 1) {
        cudaGetLastError();
        nc = gbx_ctx_sms(ctx) / 2;
    }
    if (dev >= 0 && dev < 64) cached[dev][w] = nc;
    return nc;
}

// Small-K products (the rank-nb updates of blocked factorizations) take the
// kernel with every diagonal in TMEM; GBX_OZAKI_SMALLK=0 turns it off.
bool oz_small_k(int K)
{
    static int env = [] {
        const char *s = getenv("GBX_OZAKI_SMALLK");
        return s ? atoi(s) : 1;
    }();
    return env != 0 && K <= 1024;
}

// The CTA-pair kernel takes the products (K > 1024) of at most four waves of
// its 256 x 256 tiles: measured one after another on one GB300 it ran 2048^3
// in 0.50 ms against 0.70 ms and 4096^3 in 2.90 against 3.07 ms of the
// one-CTA kernel; from 8192 on (calls of 20 ms and more under the power
// cap) it draws more power, the SM clock falls further, and it ties (8192)
// or loses (16384: 185-194 against 163 ms).  GBX_OZAKI_PAIR=1 selects it
// for every product with more than one 128-row tile (small K included),
// GBX_OZAKI_PAIR=0 never.
bool oz_use_pair(int M, int N, int K, int sms)
{
    static int env = [] {
        const char *s = getenv("GBX_OZAKI_PAIR");
        return s ? atoi(s) : -1;
    }();
    if (env == 0 || M <= OZ_BM) return false;
    if (env > 0) return true;
    if (rup(std::max(K, 1), OZ_BK) <= OZS_KMAX && oz_small_k(K)) return false;
    const long long tiles = (long long)((M + OZ2_BM - 1) / OZ2_BM) * ((N + OZ_BN - 1) / OZ_BN);
    return tiles <= 4LL * std::max(1, sms / 2);
}

// Column tile: 128 when N fits in it (the rank-nb updates of blocked
// factorizations have N = nb = 128) or when 256-wide tiles would leave most
// SMs idle; 256 otherwise (half the A-tile reloads per output column).  The
// CTA-pair kernel always uses 256.
int oz_tile_n(int M, int N, int sms, bool pair)
{
    if (pair) return OZ_BN;
    if (N <= 128) return 128;
    const long long tiles256 = ((M + OZ_BM - 1) / OZ_BM) * (long long)((N + OZ_BN - 1) / OZ_BN);
    return tiles256 < sms ? 128 : OZ_BN;
}

// Workspace layout for one Ozaki product.
struct OzBuffers {
    uint8_t *A8, *B8;
    int *ea, *eb, *S;
    int *rsa, *csb;   // scale exponents e-4 (rows of op(A), columns of op(B))
    double *ssa, *ssb;
    long long *W;     // nW planes of Mp x Np 128-bit running sums
    float *gpart;     // (Mp + Np) / 16 slice-count partials of the one-launch preparation
    int *status;      // the context's status words
    int *status_host; // device address of their host mirror
};

gbx_status oz_buffers(gbx_ctx *ctx, int Mp, int Np, int Kp, int nW, OzBuffers &b)
{
    gbx_status st;
    void *p;
    if ((st = gbx_ws(ctx, GBX_WS_OZ0, (size_t)OZ_SMAX * Mp * Kp, &p)) != GBX_OK) return st;
    b.A8 = (uint8_t *)p;
    if ((st = gbx_ws(ctx, GBX_WS_OZ1, (size_t)OZ_SMAX * Np * Kp, &p)) != GBX_OK) return st;
    b.B8 = (uint8_t *)p;
    if ((st = gbx_ws(ctx, GBX_WS_OZ2, 2 * sizeof(long long) * (size_t)Mp * Np * nW, &p)) != GBX_OK) return st;
    b.W = (long long *)p;
    const size_t small = 256 + sizeof(int) * (size_t)(Mp + Np) + sizeof(double) * 4 * (size_t)(Mp + Np) + 1024 +
                         3 * sizeof(double) * (size_t)((Mp + Np) / 16 + 2);
    if ((st = gbx_ws(ctx, GBX_WS_OZ3, small, &p)) != GBX_OK) return st;
    uint8_t *q = (uint8_t *)p;
    if ((st = gbx_ctx_status(ctx, &b.status, &b.status_host)) != GBX_OK) return st;
    q += 64;
    b.S = (int *)q; q += 64;
    b.ssa = (double *)q; q += sizeof(double) * Mp;
    b.ssb = (double *)q; q += sizeof(double) * Np;
    b.rsa = (int *)q; q += sizeof(double) * Mp;
    b.csb = (int *)q; q += sizeof(double) * Np;
    b.ea = (int *)q; q += sizeof(int) * Mp;
    b.eb = (int *)q; q += sizeof(int) * Np;
    q = (uint8_t *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
    b.gpart = (float *)q;
    return GBX_OK;
}

// col_k statistics partition: K chunk per CTA of at most OZ_STATS_KCH,
// smaller when the 32-row blocks alone would leave SMs idle.
constexpr int OZ_STATS_KCH = 1024;

OzPrepOp oz_prep_op(gbx_ctx *ctx, const SrcView &v, int rows, int K, int Rp, int Kp, int *expo, double *ss,
                    int *scale, uint8_t *X8, bool stats)
{
    OzPrepOp o{};
    o.v = v; o.rows = rows; o.K = K; o.Rp = Rp; o.Kp = Kp;
    o.expo = expo; o.ss = ss; o.scale = scale; o.X8 = X8;
    o.rblocks = (rows + 31) / 32;
    o.kch = OZ_STATS_KCH;
    if (!v.row_k)
        while (o.kch > 64 && (long long)o.rblocks * ((K + o.kch - 1) / o.kch) < 2LL * gbx_ctx_sms(ctx)) o.kch >>= 1;
    o.nkb = (K + o.kch - 1) / o.kch;
    o.stat_blocks = !stats ? 0 : (v.row_k ? (rows + 7) / 8 : o.rblocks * o.nkb);
    o.split_blocks = (Kp / 128) * (Rp / OZ_SPLIT_ROWS);
    return o;
}

// The three preparation launches (statistics, finish + slice count, slicing)
// for op(A) and, unless it is op(A) itself, op(B)^T.
gbx_status oz_prepare(gbx_ctx *ctx, OzPrepOp &a, OzPrepOp &b, bool b_stats, double tol, int forced, int *status,
                      unsigned *counter, int *S_dev)
{
    cudaStream_t s = S_(ctx);
    const size_t pa = a.v.row_k ? 0 : (size_t)a.nkb * a.rows, pb = (!b_stats || b.v.row_k) ? 0 : (size_t)b.nkb * b.rows;
    if (pa + pb) {
        void *p;
        gbx_status st = gbx_ws(ctx, GBX_WS_TMP2, sizeof(SsAcc) * (pa + pb), &p);
        if (st != GBX_OK) return st;
        a.part = (SsAcc *)p;
        b.part = (SsAcc *)p + pa;
    }
    if (!b_stats) b.stat_blocks = 0;
    const long long nstat = (long long)a.stat_blocks + b.stat_blocks;
    const long long nsplit = (long long)a.split_blocks + b.split_blocks;
    if (nstat > 0x7fffffffLL || nsplit > 0x7fffffffLL)
        return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki: operands too large");
    oz_prep_stats<<<(unsigned)nstat, 256, 0, s>>>(a, b, status, counter);
    const long long rows = (long long)std::max(a.Rp, a.scale2 ? a.Rp2 : 0) + (b_stats ? b.Rp : 0);
    const int fin = (int)std::max(1LL, std::min<long long>(2LL * gbx_ctx_sms(ctx), (rows + 255) / 256));
    oz_prep_finish<<<fin, 256, 0, s>>>(a, b, b_stats ? 1 : 0, tol, forced, counter, S_dev);
    oz_prep_split<<<(unsigned)nsplit, 256, 0, s>>>(a, b, S_dev);
    gbx_count_launch(ctx, 3);
    return gbx_check_launch(ctx, "ozaki prepare");
}

struct OzProblem {
    int M, N, K;
    SrcView a, b;    // op(A) rows M, op(B)^T rows N (both "rows x K")
    double alpha, beta;
    double *C;
    long long ldc;
    int c_part;
    bool same_ab;    // op(B)^T == op(A) (symmetric rank-k): slice once
};

gbx_status run_ozaki(gbx_ctx *ctx, const OzProblem &pr, double tol, int forced, int *slices_used,
                     OzBuffers *keep = nullptr, int nW = 1, int w_index = 0)
{
    if (pr.K > 0x3fffffff) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki: K too large");
    const bool pair = oz_use_pair(pr.M, pr.N, pr.K, gbx_ctx_sms(ctx));
    const bool small_k = !pair && rup(std::max(pr.K, 1), OZ_BK) <= OZS_KMAX && oz_small_k(pr.K);
    const long long sk_tiles = ((long long)pr.M + OZ_BM - 1) / OZ_BM * (((long long)pr.N + OZS_BN - 1) / OZS_BN);
    const int bn = small_k ? (2 * sk_tiles <= gbx_ctx_sms(ctx) ? OZS_BN / 2 : OZS_BN)
                           : oz_tile_n(pr.M, pr.N, gbx_ctx_sms(ctx), pair);
    const int Mp = (int)rup(pr.M, pair ? OZ2_BM : OZ_BM), Np = (int)rup(pr.N, bn);
    const int Kp = (int)rup(std::max(pr.K, 1), OZ_BK);
    // wide tiles in clusters of two sharing (multicasting) their B tile: full
    // products whose row tiles pair up and that fill every SM at least twice
    const bool mc = !small_k && !pair && pr.c_part == 0 && (Mp / OZ_BM) % 2 == 0 && oz_use_mc() &&
                    (long long)(Mp / OZ_BM) * (Np / bn) >= 2LL * gbx_ctx_sms(ctx);
    if (tol <= 0.0) tol = 1e-14;
    // small K: the digit planes to prepare, the largest S the tolerance can
    // call for (gamma <= 2 sqrt(K) per operand in the slice-count model)
    const int planes = forced > 0 ? forced
                                  : std::max(1, std::min(OZ_SMAX, (int)ceil((-log2(tol) + 2.0 +
                                                                             log2((double)std::max(pr.K, 1)) +
                                                                             1.5) / 5.0)));
    OzBuffers b;
    gbx_status st;
    if (keep) b = *keep;
    else if ((st = oz_buffers(ctx, Mp, Np, Kp, nW, b)) != GBX_OK) return st;
    cudaStream_t s = S_(ctx);

    gbx_timer_begin(ctx, GBX_TIMER_OZAKI_SPLIT);
    // op(A): statistics and slices; op(B)^T: its own, or for a symmetric
    // rank-k update the A slices themselves (re-sliced into the Np-row layout
    // of the B tiles when Np != Mp, with scales mirrored from op(A)'s rows)
    OzPrepOp oa = oz_prep_op(ctx, pr.a, pr.M, pr.K, Mp, Kp, b.ea, b.ssa, b.rsa, b.A8, true);
    OzPrepOp ob{};
    uint8_t *B8 = b.B8;
    const int *csb = b.csb;
    bool b_stats = false;
    if (!pr.same_ab) {
        ob = oz_prep_op(ctx, pr.b, pr.N, pr.K, Np, Kp, b.eb, b.ssb, b.csb, b.B8, true);
        b_stats = true;
    } else if (Np != Mp) {
        ob = oz_prep_op(ctx, pr.a, pr.M, pr.K, Np, Kp, b.ea, b.ssa, b.csb, b.B8, false);
        oa.scale2 = b.csb;
        oa.Rp2 = Np;
    } else {
        B8 = b.A8;
        csb = b.rsa;
    }
    if (small_k) {
        // one launch; both operands carry their own statistics (for a
        // symmetric rank-k update the second copy repeats op(A)'s)
        if (pr.same_ab) {
            ob = oz_prep_op(ctx, pr.a, pr.M, pr.K, Np, Kp, b.eb, b.ssb, b.csb, b.B8, true);
            oa.scale2 = nullptr;
            B8 = b.B8;
            csb = b.csb;
        }
        const long long blocks = (long long)Mp / OZ_SPLIT_ROWS + (long long)Np / OZ_SPLIT_ROWS;
        if (blocks > 0x7fffffffLL) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki: operands too large");
        oa.gpart = b.gpart;
        ob.gpart = b.gpart + 3 * (size_t)(Mp / OZ_SPLIT_ROWS);
        if (blocks <= gbx_ctx_sms(ctx))
            oz_prep_small<2 * OZ_SMALL_THREADS><<<(unsigned)blocks, 2 * OZ_SMALL_THREADS, 0, s>>>(oa, ob, planes, b.status);
        else
            oz_prep_small<OZ_SMALL_THREADS><<<(unsigned)blocks, OZ_SMALL_THREADS, 0, s>>>(oa, ob, planes, b.status);
        gbx_count_launch(ctx, 1);
        if ((st = gbx_check_launch(ctx, "ozaki prepare")) != GBX_OK) return st;
    } else if ((st = oz_prepare(ctx, oa, ob, b_stats, tol, forced, b.status, (unsigned *)(b.S + 4), b.S)) !=
               GBX_OK) {
        return st;
    }
    gbx_timer_end(ctx);

    CUtensorMap tmA, tmB, tmBh;
    // small K: op(B)^T's planes as a 3-D map, the B stage of a tile in one load;
    // wide tiles: also a half-width B box for the half tiles of the last wave
    const bool wide = !small_k && !pair;
    const int inner = wide ? OZ_WBK : OZ_BK;
    if (!make_map(&tmA, b.A8, (long long)OZ_SMAX * Mp, Kp, OZ_BM, inner) ||
        !(small_k ? make_map(&tmB, B8, Np, Kp, -(bn * 256 + planes))
                  : make_map(&tmB, B8, (long long)OZ_SMAX * Np, Kp, pair ? 128 : (mc ? bn / 2 : bn), inner)) ||
        (wide && !make_map(&tmBh, B8, (long long)OZ_SMAX * Np, Kp, mc ? bn / 4 : bn / 2, inner)) ||
        (pair && !make_map(&tmBh, B8, (long long)OZ_SMAX * Np, Kp, OZ_BN / 4)))
        return gbx_fail(ctx, GBX_ERR_CUDA, "ozaki: cuTensorMapEncodeTiled failed");

    OzParams p{};
    p.M = pr.M; p.N = pr.N; p.Mp = Mp; p.Np = Np; p.Kp = Kp;
    p.tiles_m = Mp / (pair ? OZ2_BM : OZ_BM); p.tiles_n = Np / bn;
    int mc_clusters = 0;
    {
        // wide tiles: a last wave filling at most half the SMs (cluster pairs
        // with B multicast) runs as half tiles
        const int per = mc ? 2 : 1;
        if (mc && (mc_clusters = oz_mc_clusters(ctx, bn)) < 1) return gbx_fail(ctx, GBX_ERR_CUDA, "ozaki: clusters");
        const int nt = p.tiles_m / per * p.tiles_n;
        const int slots = mc ? mc_clusters : (pair ? std::max(1, gbx_ctx_sms(ctx) / 2) : gbx_ctx_sms(ctx));
        const int g = std::min(nt, slots), r = nt % g;
        p.t_split = ((wide || pair) && r > 0 && 2 * r <= g) ? nt - r : nt;
        p.nunits = p.t_split + 2 * (nt - p.t_split);
    }
    p.S = b.S;
    p.row_exp = b.rsa;
    p.col_exp = csb;
    p.W = b.W + 2 * (size_t)w_index * Mp * Np;
    p.C = pr.C; p.ldc = pr.ldc;
    p.alpha = pr.alpha; p.beta = pr.beta;
    p.c_part = pr.c_part;
    p.status = b.status;
    p.status_host = b.status_host;
    p.gpa = b.gpart;
    p.gpb = b.gpart + 3 * (size_t)(Mp / OZ_SPLIT_ROWS);
    p.npa = Mp / OZ_SPLIT_ROWS;
    p.npb = Np / OZ_SPLIT_ROWS;
    p.K = pr.K;
    p.tol_bits = (float)(-log2(tol));
    p.forced = forced;
    p.smax = planes;
    // S >= ceil((-log2 tol + 1.5) / 5) (gamma >= 1 per operand); one less
    // for the FP32 arithmetic of the device's choice
    p.s_lo = forced > 0 ? std::min(forced, planes)
                        : std::max(1, std::min(planes, (int)ceil((-log2(tol) + 1.5) / 5.0) - 1));

    // kernel attributes (per device) and the resident CTA-pair count; calls
    // arrive from many host threads
    static std::mutex attr_mu;
    static int max_pairs_of[64] = {0};
    const int dev = gbx_ctx_device(ctx);
    int max_pairs;
    {
        std::lock_guard<std::mutex> lk(attr_mu);
        max_pairs = (dev >= 0 && dev < 64) ? max_pairs_of[dev] : 0;
        if (max_pairs == 0) {
            if (cudaFuncSetAttribute(oz_gemm_sk_kernel<OZS_BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)OZS_SMEM) != cudaSuccess ||
                cudaFuncSetAttribute(oz_gemm_sk_kernel<OZS_BN / 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)OZS_SMEM) != cudaSuccess ||
                cudaFuncSetAttribute(oz_gemm_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)OzCfg<256>::SMEM) != cudaSuccess ||
                cudaFuncSetAttribute(oz_gemm_kernel<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)OzCfg<128>::SMEM) != cudaSuccess ||
                cudaFuncSetAttribute(oz_gemm2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)OZ2_SMEM) != cudaSuccess)
                return gbx_fail(ctx, GBX_ERR_CUDA, "ozaki: shared memory attribute");
            // how many CTA pairs can be resident at once (clusters must fit in a GPC)
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(2 * (unsigned)std::max(1, gbx_ctx_sms(ctx) / 2));
            cfg.blockDim = dim3(OZ2_THREADS);
            cfg.dynamicSmemBytes = OZ2_SMEM;
            int nc = 0;
            if (cudaOccupancyMaxActiveClusters(&nc, oz_gemm2_kernel, &cfg) != cudaSuccess || nc < 1) {
                cudaGetLastError();
                nc = gbx_ctx_sms(ctx) / 2;
            }
            max_pairs = std::max(1, nc);
            if (dev >= 0 && dev < 64) max_pairs_of[dev] = max_pairs;
        }
    }
    const int ntiles = p.tiles_m * p.tiles_n;
    gbx_timer_begin(ctx, GBX_TIMER_OZAKI_MMA);
    if (pair) {
        const int npairs = std::max(1, std::min(ntiles, max_pairs));
        oz_gemm2_kernel<<<2 * npairs, OZ2_THREADS, OZ2_SMEM, s>>>(tmA, tmB, tmBh, p);
    } else {
        const int grid = std::min(ntiles, gbx_ctx_sms(ctx));
        if (small_k) {
            // a programmatic dependent of the one-launch preparation before it
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)grid);
            cfg.blockDim = dim3(OZS_THREADS);
            cfg.dynamicSmemBytes = OZS_SMEM;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            const cudaError_t le = bn == OZS_BN ? cudaLaunchKernelEx(&cfg, oz_gemm_sk_kernel<OZS_BN>, tmA, tmB, p)
                                                : cudaLaunchKernelEx(&cfg, oz_gemm_sk_kernel<OZS_BN / 2>, tmA, tmB, p);
            if (le != cudaSuccess) {
                cudaGetLastError();
                return gbx_fail(ctx, GBX_ERR_CUDA, "ozaki gemm: %s", cudaGetErrorString(le));
            }
        } else if (mc) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(2 * (unsigned)std::min(p.nunits, mc_clusters));
            cfg.blockDim = dim3(bn == 128 ? OzCfg<128>::THREADS : OzCfg<256>::THREADS);
            cfg.dynamicSmemBytes = bn == 128 ? OzCfg<128>::SMEM : OzCfg<256>::SMEM;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = 2;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            const cudaError_t le = bn == 128 ? cudaLaunchKernelEx(&cfg, oz_gemm_kernel<128, true>, tmA, tmB, tmBh, p)
                                             : cudaLaunchKernelEx(&cfg, oz_gemm_kernel<256, true>, tmA, tmB, tmBh, p);
            if (le != cudaSuccess) {
                cudaGetLastError();
                return gbx_fail(ctx, GBX_ERR_CUDA, "ozaki gemm: %s", cudaGetErrorString(le));
            }
        } else if (bn == 128)
            oz_gemm_kernel<128, false><<<grid, OzCfg<128>::THREADS, OzCfg<128>::SMEM, s>>>(tmA, tmB, tmBh, p);
        else
            oz_gemm_kernel<256, false><<<grid, OzCfg<256>::THREADS, OzCfg<256>::SMEM, s>>>(tmA, tmB, tmBh, p);
    }
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    if ((st = gbx_check_launch(ctx, "ozaki gemm")) != GBX_OK) return st;
    if (slices_used) {
        int h = 0;
        cudaMemcpyAsync(&h, b.S, sizeof(int), cudaMemcpyDeviceToHost, s);
        if ((st = gbx_ctx_sync(ctx)) != GBX_OK) return st;
        *slices_used = h;
    }
    if (keep) *keep = b;
    return GBX_OK;
}

SrcView view_real(const double *X, int ld, bool row_k)
{
    SrcView v{};
    v.X = X; v.ld = ld; v.row_k = row_k ? 1 : 0; v.Ksplit = 0x7fffffff;
    return v;
}

}  // namespace

extern "C" gbx_status gbx_dgemm_ozaki(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                                      const double *A, int lda, const double *B, int ldb, double beta,
                                      double *C, int ldc, double tol, int slices, int *slices_used)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_gemm_args(ta, tb, m, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DGEMM parameter %d", info);
    if (slices < 0 || slices > OZ_SMAX) return gbx_fail(ctx, GBX_ERR_ARG, "ozaki: slices must be 0..%d", OZ_SMAX);
    if (slices_used) *slices_used = 0;
    if (m == 0 || n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return GBX_OK;
    if (alpha == 0.0 || k == 0) return gbx_gemm::scale_matrix<double>(ctx, m, n, beta, C, ldc, 0);
    OzProblem pr{};
    pr.M = m; pr.N = n; pr.K = k;
    // op(A)(i,k): 'N' -> A[k*lda + i] (col_k); 'T' -> A[i*lda + k] (row_k)
    pr.a = view_real(A, lda, !gbx_lsame(ta, 'N'));
    // op(B)^T(j,k) = op(B)(k,j): 'N' -> B[j*ldb + k] (row_k); 'T' -> B[k*ldb + j] (col_k)
    pr.b = view_real(B, ldb, gbx_lsame(tb, 'N'));
    pr.alpha = alpha; pr.beta = beta; pr.C = C; pr.ldc = ldc; pr.c_part = 0;
    return run_ozaki(ctx, pr, tol, slices, slices_used);
}

extern "C" gbx_status gbx_dsyrk_ozaki(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                                      const double *A, int lda, double beta, double *C, int ldc, double tol,
                                      int slices, int *slices_used)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_syrk_args(uplo, trans, n, k, lda, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DSYRK parameter %d", info);
    if (slices < 0 || slices > OZ_SMAX) return gbx_fail(ctx, GBX_ERR_ARG, "ozaki: slices must be 0..%d", OZ_SMAX);
    if (slices_used) *slices_used = 0;
    const int part = gbx_lsame(uplo, 'U') ? 2 : 1;
    if (n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return GBX_OK;
    if (alpha == 0.0 || k == 0) return gbx_gemm::scale_matrix<double>(ctx, n, n, beta, C, ldc, part);
    OzProblem pr{};
    pr.M = n; pr.N = n; pr.K = k;
    // 'N': C = A A^T, rows of A (col_k); 'T': C = A^T A, columns of A (row_k)
    pr.a = view_real(A, lda, !gbx_lsame(trans, 'N'));
    pr.b = pr.a;
    pr.same_ab = true;
    pr.alpha = alpha; pr.beta = beta; pr.C = C; pr.ldc = ldc; pr.c_part = part;
    return run_ozaki(ctx, pr, tol, slices, slices_used);
}

// DTRSM via the inverse: X = op(A)^-1 is formed in FP64 (the FP64 DTRSM of
// the identity: the diagonal-block solves stay FP64), then B is multiplied
// by it as one Ozaki product (B := alpha X B or alpha B X).  For the
// well-conditioned diagonal blocks of a Cholesky factorization the extra
// error of applying the inverse is a factor cond(op(A)) on the rounding of X.
namespace {
// Inverse of a triangular matrix of order n <= 256 in FP64, one warp per
// column of the inverse.  An upper triangle U is handled as the lower
// triangle L' = P U P (P the order-reversing permutation; U^-1 = P L'^-1 P).
// Column j of W = L'^-1 solves L' w = e_j by forward substitution, lane l
// holding rows l, l + 32, ...: at step i the owner lane scales w_i by the
// inverse diagonal entry, broadcasts it, and every lane subtracts
// w_i L'(r, i) from its rows r > i.  The columns of L' stream through shared
// memory 16 at a time.  Each step costs one FP64 warp instruction per
// 32-row slot still below the pivot, and an FP64 warp instruction occupies
// the SM's 2-lane FP64 pipe for 16 cycles whatever its predicate: CTAs of 2
// warps spread the columns over as many SMs as possible, and slots above
// the pivot are skipped.  The FP64 DTRSM of the identity this replaces ran
// its small GEMM updates on one or two SMs (~270 µs for n = 128).
// X = W, or W^T for op = 'T'/'C'.
constexpr int OZ_TI_WARPS = 2, OZ_TI_PANEL = 16, OZ_TI_NMAX = 256;

__global__ void __launch_bounds__(OZ_TI_WARPS * 32)
oz_trinv_kernel(int n, const double *__restrict__ T, long long ldt, int lower, int unit, int trans,
                double *__restrict__ X, long long ldx)
{
    __shared__ double sT[OZ_TI_PANEL][OZ_TI_NMAX];
    __shared__ double sR[OZ_TI_NMAX];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // L'(r, c) for r >= c
    auto tget = [&](int r, int c) -> double {
        const int rr = lower ? r : n - 1 - r, cc = lower ? c : n - 1 - c;
        return T[(long long)cc * ldt + rr];
    };
    for (int i = threadIdx.x; i < n; i += blockDim.x) sR[i] = unit ? 1.0 : 1.0 / tget(i, i);
    const int jfirst = blockIdx.x * OZ_TI_WARPS;
    const int j = jfirst + warp;   // this warp's column of L'^-1
    double w[OZ_TI_NMAX / 32];
#pragma unroll
    for (int s = 0; s < OZ_TI_NMAX / 32; s++) w[s] = (s * 32 + lane == j) ? 1.0 : 0.0;
    for (int p0 = jfirst / OZ_TI_PANEL * OZ_TI_PANEL; p0 < n; p0 += OZ_TI_PANEL) {
        __syncthreads();   // the previous panel is consumed (and sR written)
        const int rows = n - p0;
        for (int t = threadIdx.x; t < OZ_TI_PANEL * rows; t += blockDim.x) {
            const int c = t / rows, r = p0 + t % rows;
            sT[c][r] = (p0 + c < n && r >= p0 + c) ? tget(r, p0 + c) : 0.0;
        }
        __syncthreads();
        if (j >= n) continue;
        for (int c = 0; c < OZ_TI_PANEL; c++) {
            const int i = p0 + c;
            if (i >= n) break;
            if (i < j) continue;   // uniform over the warp
            const int slot = i >> 5;
            double wo = 0.0;
#pragma unroll
            for (int s = 0; s < OZ_TI_NMAX / 32; s++)
                if (s == slot) wo = w[s];
            const double wi = __shfl_sync(0xffffffffu, wo * sR[i], i & 31);
#pragma unroll
            for (int s = 0; s < OZ_TI_NMAX / 32; s++) {
                if (s < slot || s * 32 >= n) continue;   // warp-uniform: no FP64 issue
                const int r = s * 32 + lane;
                if (r > i && r < n) w[s] = fma(-sT[c][r], wi, w[s]);
                else if (r == i) w[s] = wi;
            }
        }
    }
    if (j >= n) return;
#pragma unroll
    for (int s = 0; s < OZ_TI_NMAX / 32; s++) {
        const int r = s * 32 + lane;
        if (r >= n) continue;
        const double v = r >= j ? w[s] : 0.0;
        const int R = lower ? r : n - 1 - r, J = lower ? j : n - 1 - j;   // entry (R, J) of T^-1
        if (trans) X[(long long)R * ldx + J] = v;
        else X[(long long)J * ldx + R] = v;
    }
}

__global__ void oz_set_identity(int n, double *X, long long ldx)
{
    const long long total = (long long)n * n;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n), j = (int)(t / n);
        X[(long long)j * ldx + i] = i == j ? 1.0 : 0.0;
    }
}
}  // namespace

extern "C" gbx_status gbx_dtrsm_ozaki(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                      double alpha, const double *A, int lda, double *B, int ldb, double tol,
                                      int slices, int *slices_used)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_trxm_args(side, uplo, ta, diag, m, n, lda, ldb);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DTRSM parameter %d", info);
    if (slices < 0 || slices > OZ_SMAX) return gbx_fail(ctx, GBX_ERR_ARG, "ozaki: slices must be 0..%d", OZ_SMAX);
    if (slices_used) *slices_used = 0;
    if (m == 0 || n == 0) return GBX_OK;
    const bool lside = gbx_lsame(side, 'L');
    const int na = lside ? m : n;
    if (alpha == 0.0 || na > 1024) return gbx_dtrsm(ctx, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb);
    gbx_status st;
    void *px;
    if ((st = gbx_ws(ctx, GBX_WS_TRSM_X, sizeof(double) * (size_t)na * na, &px)) != GBX_OK) return st;
    double *X = (double *)px;
    cudaStream_t s = S_(ctx);
    if (na <= OZ_TI_NMAX) {
        // X = op(A)^-1 by the warp-per-column substitution kernel
        oz_trinv_kernel<<<(na + OZ_TI_WARPS - 1) / OZ_TI_WARPS, OZ_TI_WARPS * 32, 0, s>>>(
            na, A, lda, gbx_lsame(uplo, 'L') ? 1 : 0, gbx_lsame(diag, 'U') ? 1 : 0, gbx_lsame(ta, 'N') ? 0 : 1, X, na);
        gbx_count_launch(ctx, 1);
        if ((st = gbx_check_launch(ctx, "dtrsm_ozaki inverse")) != GBX_OK) return st;
    } else {
        // X = op(A)^-1 I by the FP64 DTRSM
        const long long total = (long long)na * na;
        oz_set_identity<<<(int)std::min<long long>((total + 255) / 256, (long long)gbx_ctx_sms(ctx) * 4), 256, 0,
                          s>>>(na, X, na);
        gbx_count_launch(ctx, 1);
        if ((st = gbx_check_launch(ctx, "dtrsm_ozaki identity")) != GBX_OK) return st;
        if ((st = gbx_dtrsm(ctx, 'L', uplo, ta, diag, na, na, 1.0, A, lda, X, na)) != GBX_OK) return st;
    }
    // B is both an operand and the result: the Ozaki product reads its FP64
    // operands only in the preparation launches, which complete before the
    // product kernel writes C, and with beta = 0 it never reads C.
    if (lside)
        return gbx_dgemm_ozaki(ctx, 'N', 'N', m, n, m, alpha, X, na, B, ldb, 0.0, B, ldb, tol, slices, slices_used);
    return gbx_dgemm_ozaki(ctx, 'N', 'N', m, n, n, alpha, B, ldb, X, na, 0.0, B, ldb, tol, slices, slices_used);
}

// ZGEMM: Re = [Ar | Ai] x [Br ; -Bi],  Im = [Ar | Ai] x [Bi ; Br]  (K' = 2K),
// both real Ozaki products into FP64 workspace, then C = alpha*(Re + i Im) +
// beta*C.  Conjugation ('C') negates the imaginary part while slicing.
extern "C" gbx_status gbx_zgemm_ozaki(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, const double *alpha,
                                      const double *A, int lda, const double *B, int ldb, const double *beta,
                                      double *C, int ldc, double tol, int slices, int *slices_used)
{
    if (!ctx || !alpha || !beta) return GBX_ERR_ARG;
    int info = gbx_check_gemm_args(ta, tb, m, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "ZGEMM parameter %d", info);
    if (slices < 0 || slices > OZ_SMAX) return gbx_fail(ctx, GBX_ERR_ARG, "ozaki: slices must be 0..%d", OZ_SMAX);
    if (slices_used) *slices_used = 0;
    const bool alpha0 = alpha[0] == 0.0 && alpha[1] == 0.0, beta1 = beta[0] == 1.0 && beta[1] == 0.0;
    if (m == 0 || n == 0 || ((alpha0 || k == 0) && beta1)) return GBX_OK;
    if (alpha0 || k == 0) {
        gbx_gemm::dcplx be{beta[0], beta[1]};
        return gbx_gemm::scale_matrix<gbx_gemm::dcplx>(ctx, m, n, be, (gbx_gemm::dcplx *)C, ldc, 0);
    }
    if (2LL * k > 0x3fffffffLL) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki: K too large");
    const int K2 = 2 * k;
    const int Mp = (int)rup(m, oz_use_pair(m, n, K2, gbx_ctx_sms(ctx)) ? OZ2_BM : OZ_BM), Np = (int)rup(n, OZ_BN);
    const int Kp = (int)rup(K2, OZ_BK);
    OzBuffers b;
    gbx_status st = oz_buffers(ctx, Mp, Np, Kp, 2, b);
    if (st != GBX_OK) return st;

    OzProblem pr{};
    pr.M = m; pr.N = n; pr.K = K2;
    pr.a.X = A; pr.a.ld = lda; pr.a.row_k = !gbx_lsame(ta, 'N'); pr.a.cplx = 1;
    pr.a.conj = gbx_lsame(ta, 'C'); pr.a.part0 = 0; pr.a.part1 = 1; pr.a.Ksplit = k;
    pr.b.X = B; pr.b.ld = ldb; pr.b.row_k = gbx_lsame(tb, 'N'); pr.b.cplx = 1;
    pr.b.conj = gbx_lsame(tb, 'C'); pr.b.part0 = 0; pr.b.part1 = 2; pr.b.Ksplit = k;   // [Br ; -Bi]
    pr.alpha = 1.0; pr.beta = 0.0; pr.c_part = 0;
    // W holds two planes of 16 bytes per element: the first takes each
    // product's running values, the second keeps Re (Mp x n doubles) while
    // the imaginary product runs
    double *Wre = (double *)(b.W + 2 * (size_t)Mp * Np);
    pr.C = Wre; pr.ldc = Mp;
    int used_re = 0, used_im = 0;
    // real part: Re = Ar Br - Ai Bi, one real product of [Ar Ai] and [Br ; -Bi]
    if ((st = run_ozaki(ctx, pr, tol, slices, slices_used ? &used_re : nullptr, &b, 2, 0)) != GBX_OK) return st;
    // imaginary part: Im = Ar Bi + Ai Br, [Ar Ai] times [Bi ; Br], into its
    // own workspace slot; its running values reuse W's first plane
    double *Wim;
    void *p;
    if ((st = gbx_ws(ctx, GBX_WS_TMP1, sizeof(double) * (size_t)Mp * n, &p)) != GBX_OK) return st;
    Wim = (double *)p;
    pr.b.part0 = 1; pr.b.part1 = 0;
    pr.C = Wim; pr.ldc = Mp;
    if ((st = run_ozaki(ctx, pr, tol, slices, slices_used ? &used_im : nullptr, &b, 2, 0)) != GBX_OK) return st;
    const long long total = (long long)m * n;
    const int g = (int)std::min<long long>((total + 255) / 256, (long long)gbx_ctx_sms(ctx) * 8);
    oz_complex_combine<<<g, 256, 0, S_(ctx)>>>(m, n, Wre, Wim, Mp, alpha[0], alpha[1], beta[0], beta[1], C, ldc);
    gbx_count_launch(ctx, 1);
    if (slices_used) *slices_used = std::max(used_re, used_im);
    return gbx_check_launch(ctx, "ozaki zgemm combine");
}
