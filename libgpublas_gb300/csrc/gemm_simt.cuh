// gemm_simt.cuh — GEMM core on the SIMT FMA pipes, for the four BLAS
// element types (float, double, complex float, complex double).
//
// Measured on GB300: SIMT DFMA sustains about 1.2 TFLOP/s per GPU, the legacy
// FP64 tensor path (mma.sync.m8n8k4.f64) about 1.05 TFLOP/s, so the plain
// FP64 GEMM-class routines run on DFMA.  At 2 DFMA lanes per clock per SM the
// kernel is compute-bound at any sane tile size: a 64x64 block tile with
// 4x4 register tiles moves 8 KB of operands per 32k FMAs, so operand staging
// through shared memory with register prefetch is all the memory pipeline
// needs; what counts is keeping the pipe fed across the barriers of each
// K step, which two resident CTAs per SM do better than one large one.
//
// One kernel template serves xGEMM, xSYRK/xHERK and xSYR2K/xHER2K (triangular
// tile grid), xSYMM/xHEMM (an operand read from one stored triangle), xTRMM
// (triangular operand masking) and the xTRSM updates, for S, D, C and Z.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbx_gemm {

struct dcplx { double x, y; };
struct fcplx { float x, y; };

// Complex quotient a / b by Smith's algorithm (R. L. Smith, "Algorithm 116:
// Complex division", CACM 5(8), 1962): scales by the larger component of b
// so that no intermediate overflows where the quotient does not.
template <typename C, typename R>
__device__ __forceinline__ C smith_div(C a, C b)
{
    if (fabs(b.y) <= fabs(b.x)) {
        const R r = b.y / b.x, d = b.x + b.y * r;
        return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
    }
    const R r = b.x / b.y, d = b.y + b.x * r;
    return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
}

template <typename T> struct Ops;
template <> struct Ops<double> {
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ double one() { return 1.0; }
    static __device__ __forceinline__ void fma_acc(double &acc, double a, double b) { acc = fma(a, b, acc); }
    static __device__ __forceinline__ double conj(double a) { return a; }
    static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    // a x + b y with the rounding spelled out (x a rounded, then one FMA), so
    // that every instantiation of the GEMM core gives the same bits whatever
    // the compiler would contract
    static __device__ __forceinline__ double axpby(double a, double x, double b, double y)
    {
        return __fma_rn(b, y, __dmul_rn(a, x));
    }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __device__ __forceinline__ double neg(double a) { return -a; }
    static __device__ __forceinline__ double real_only(double a) { return a; }
    static __device__ __forceinline__ bool is_zero(double a) { return a == 0.0; }
};
template <> struct Ops<float> {
    static __device__ __forceinline__ float zero() { return 0.0f; }
    static __device__ __forceinline__ float one() { return 1.0f; }
    static __device__ __forceinline__ void fma_acc(float &acc, float a, float b) { acc = fmaf(a, b, acc); }
    static __device__ __forceinline__ float conj(float a) { return a; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float axpby(float a, float x, float b, float y)
    {
        return __fmaf_rn(b, y, __fmul_rn(a, x));
    }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float neg(float a) { return -a; }
    static __device__ __forceinline__ float real_only(float a) { return a; }
    static __device__ __forceinline__ bool is_zero(float a) { return a == 0.0f; }
};
template <> struct Ops<fcplx> {
    static __device__ __forceinline__ fcplx zero() { return {0.0f, 0.0f}; }
    static __device__ __forceinline__ fcplx one() { return {1.0f, 0.0f}; }
    static __device__ __forceinline__ void fma_acc(fcplx &acc, fcplx a, fcplx b)
    {
        acc.x = fmaf(a.x, b.x, acc.x);
        acc.x = fmaf(-a.y, b.y, acc.x);
        acc.y = fmaf(a.x, b.y, acc.y);
        acc.y = fmaf(a.y, b.x, acc.y);
    }
    static __device__ __forceinline__ fcplx conj(fcplx a) { return {a.x, -a.y}; }
    static __device__ __forceinline__ fcplx mul(fcplx a, fcplx b)
    {
        // rounding spelled out (one product rounded, one FMA), so that the
        // result does not depend on what the compiler contracts
        return {__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x))};
    }
    static __device__ __forceinline__ fcplx add(fcplx a, fcplx b) { return {a.x + b.x, a.y + b.y}; }
    static __device__ __forceinline__ fcplx axpby(fcplx a, fcplx x, fcplx b, fcplx y)
    {
        const fcplx u = mul(a, x), v = mul(b, y);
        return {__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y)};
    }
    static __device__ __forceinline__ fcplx div(fcplx a, fcplx b) { return smith_div<fcplx, float>(a, b); }
    static __device__ __forceinline__ fcplx neg(fcplx a) { return {-a.x, -a.y}; }
    static __device__ __forceinline__ fcplx real_only(fcplx a) { return {a.x, 0.0f}; }
    static __device__ __forceinline__ bool is_zero(fcplx a) { return a.x == 0.0f && a.y == 0.0f; }
};
template <> struct Ops<dcplx> {
    static __device__ __forceinline__ dcplx zero() { return {0.0, 0.0}; }
    static __device__ __forceinline__ dcplx one() { return {1.0, 0.0}; }
    static __device__ __forceinline__ void fma_acc(dcplx &acc, dcplx a, dcplx b)
    {
        acc.x = fma(a.x, b.x, acc.x);
        acc.x = fma(-a.y, b.y, acc.x);
        acc.y = fma(a.x, b.y, acc.y);
        acc.y = fma(a.y, b.x, acc.y);
    }
    static __device__ __forceinline__ dcplx conj(dcplx a) { return {a.x, -a.y}; }
    static __device__ __forceinline__ dcplx mul(dcplx a, dcplx b)
    {
        // rounding spelled out (one product rounded, one FMA), so that the
        // result does not depend on what the compiler contracts
        return {__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)), __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x))};
    }
    static __device__ __forceinline__ dcplx add(dcplx a, dcplx b) { return {a.x + b.x, a.y + b.y}; }
    static __device__ __forceinline__ dcplx axpby(dcplx a, dcplx x, dcplx b, dcplx y)
    {
        const dcplx u = mul(a, x), v = mul(b, y);
        return {__dadd_rn(u.x, v.x), __dadd_rn(u.y, v.y)};
    }
    static __device__ __forceinline__ dcplx div(dcplx a, dcplx b) { return smith_div<dcplx, double>(a, b); }
    static __device__ __forceinline__ dcplx neg(dcplx a) { return {-a.x, -a.y}; }
    static __device__ __forceinline__ dcplx real_only(dcplx a) { return {a.x, 0.0}; }
    static __device__ __forceinline__ bool is_zero(dcplx a) { return a.x == 0.0 && a.y == 0.0; }
};

// Triangular description of an operand (op() already applied):
//   TRI_NONE, or TRI_LOWER / TRI_UPPER optionally | TRI_UNIT.
enum { TRI_NONE = 0, TRI_LOWER = 1, TRI_UPPER = 2, TRI_UNIT = 4 };
// Which part of C is written.
enum { C_FULL = 0, C_LOWER = 1, C_UPPER = 2 };
// Symmetric / Hermitian operand (xSYMM, xHEMM): which triangle is stored;
// the other is read from its mirror (conjugated for Hermitian, whose
// diagonal is taken as real).
enum { SYM_NONE = 0, SYM_LOWER = 1, SYM_UPPER = 2, SYM_HERM = 4 };

template <typename T>
struct GemmArgs {
    int m, n, k;
    const T *A; long long lda; int ta; int conja;   // ta: op(A) = A^T (A stored k x m)
    const T *B; long long ldb; int tb; int conjb;   // tb: op(B) = B^T (B stored n x k)
    T alpha, beta;
    T *C; long long ldc;
    int tri_a, tri_b;   // triangular masks of op(A) (m x m) / op(B) (n x n)
    int sym_a, sym_b;   // symmetric / Hermitian operand (square; op() ignored)
    int c_part;         // C_FULL / C_LOWER / C_UPPER (symmetric rank-k update)
    int c_herm;         // Hermitian C: the diagonal's imaginary part is set to zero
    int tiles_m, tiles_n;
};

constexpr int GEMM_THREADS = 256;

// Load the (MN x BK) panel of op(X) starting at (mn0, k0) into registers.
// contig_mn: X is stored with the MN index contiguous (i.e. op(X) = X for A,
// op(X) = X^T for B); otherwise the k index is contiguous.
template <typename T, int MN, int BK>
struct PanelLoader {
    static constexpr int PER = MN * BK / GEMM_THREADS;
    T r[PER];

    __device__ __forceinline__ void load(const T *__restrict__ X, long long ld, bool contig_mn,
                                         int mn0, int mn_lim, int k0, int k_lim, int conj, int tri,
                                         bool is_a, int sym)
    {
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int idx = threadIdx.x + q * GEMM_THREADS;
            int mn, kk;
            if (contig_mn) { mn = idx % MN; kk = idx / MN; }
            else           { kk = idx % BK; mn = idx / BK; }
            const int gm = mn0 + mn, gk = k0 + kk;
            T v = Ops<T>::zero();
            if (sym) {
                if (gm < mn_lim && gk < k_lim) {
                    const int row = is_a ? gm : gk, col = is_a ? gk : gm;
                    const bool stored = (sym & SYM_LOWER) ? row >= col : row <= col;
                    v = stored ? X[(long long)col * ld + row] : X[(long long)row * ld + col];
                    if (sym & SYM_HERM) {
                        if (!stored) v = Ops<T>::conj(v);
                        if (row == col) v = Ops<T>::real_only(v);
                    }
                }
            } else if (gm < mn_lim && gk < k_lim) {
                bool keep = true, unit_diag = false;
                if (tri) {
                    // element of op(X) at (row, col): for A rows are mn, for B rows are k
                    const int row = is_a ? gm : gk, col = is_a ? gk : gm;
                    keep = (tri & TRI_LOWER) ? (col <= row) : (col >= row);
                    unit_diag = (tri & TRI_UNIT) && row == col;
                }
                if (unit_diag) v = Ops<T>::one();
                else if (keep) {
                    v = contig_mn ? X[(long long)gk * ld + gm] : X[(long long)gm * ld + gk];
                    if (conj) v = Ops<T>::conj(v);
                }
            }
            r[q] = v;
        }
    }
    __device__ __forceinline__ void store(T (*S)[MN], bool contig_mn)
    {
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int idx = threadIdx.x + q * GEMM_THREADS;
            int mn, kk;
            if (contig_mn) { mn = idx % MN; kk = idx / MN; }
            else           { kk = idx % BK; mn = idx / BK; }
            S[kk][mn] = r[q];
        }
    }
};

// Triangular-tile decode for C_LOWER/C_UPPER grids: t -> (bi, bj), bi >= bj.
__device__ __forceinline__ void tri_decode(int t, int &bi, int &bj)
{
    int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)(i + 1) * (i + 2) / 2 <= t) i++;
    while ((long long)i * (i + 1) / 2 > t) i--;
    bi = i;
    bj = t - i * (i + 1) / 2;
}

// Row (col) of a thread's i-th register-tile entry within the block tile:
// with TM >= 2 a thread holds TM/2 adjacent rows in each half of the tile
// (conflict-free shared-memory reads); with TM == 1 one row.
template <int TM>
__device__ __forceinline__ int frag_pos(int t, int i)
{
    if constexpr (TM == 1) return t;
    else return i < TM / 2 ? t * (TM / 2) + i : 8 * TM + t * (TM / 2) + (i - TM / 2);
}

// One BM x BN tile of C (tile index: column-major over the tile grid, or the
// triangular enumeration for C_LOWER / C_UPPER), computed by the whole CTA
// of GEMM_THREADS threads.  The launch kernel below runs one tile per CTA;
// the serving loop's persistent kernel calls it for the tiles it takes.
// Every output element is one FMA chain over K in increasing order,
// whatever the tile size (TM = TN = 1, a 16 x 16 tile with one element per
// thread, needs BK = 16 so that a panel has one element per thread).
template <typename T, int TM, int TN, int BK>
__device__ __forceinline__ void gemm_simt_tile(const GemmArgs<T> &p, int tile)
{
    constexpr int BM = 16 * TM, BN = 16 * TN;
    static_assert((TM == 1 || TM % 2 == 0) && (TN == 1 || TN % 2 == 0), "register tile");
    static_assert(BM * BK % GEMM_THREADS == 0 && BN * BK % GEMM_THREADS == 0, "panel per thread");
    __shared__ __align__(16) T As[2][BK][BM];
    __shared__ __align__(16) T Bs[2][BK][BN];

    int bi, bj;
    if (p.c_part == C_FULL) {
        // groups of 16 row tiles, row tile fastest: the 304 tiles resident at
        // once share their A panels 19 ways and their B panels 16 ways (in
        // column order 2.4 and 128), so fewer operand lines come from DRAM
        constexpr int GM = 16;
        const int per_group = GM * p.tiles_n;
        const int g = tile / per_group, r = tile - g * per_group;
        const int rows = min(GM, p.tiles_m - g * GM);
        bi = g * GM + r % rows;
        bj = r / rows;
    } else {
        int r, c;
        tri_decode(tile, r, c);
        if (p.c_part == C_LOWER) { bi = r; bj = c; } else { bi = c; bj = r; }
    }
    const int m0 = bi * BM, n0 = bj * BN;

    // K range that can contribute given triangular operands
    int kbeg = 0, kend = p.k;
    if (p.tri_a & TRI_LOWER) kend = min(kend, m0 + BM);
    if (p.tri_a & TRI_UPPER) kbeg = max(kbeg, m0);
    if (p.tri_b & TRI_LOWER) kbeg = max(kbeg, n0);
    if (p.tri_b & TRI_UPPER) kend = min(kend, n0 + BN);
    kbeg = (kbeg / BK) * BK;

    const bool a_contig_mn = !p.ta;   // A (m x k) column-major: m contiguous
    const bool b_contig_mn = p.tb;    // B^T stored n x k: n contiguous

    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = Ops<T>::zero();

    PanelLoader<T, BM, BK> la;
    PanelLoader<T, BN, BK> lb;
    int cur = 0;
    if (kbeg < kend) {
        la.load(p.A, p.lda, a_contig_mn, m0, p.m, kbeg, p.k, p.conja, p.tri_a, true, p.sym_a);
        lb.load(p.B, p.ldb, b_contig_mn, n0, p.n, kbeg, p.k, p.conjb, p.tri_b, false, p.sym_b);
        la.store(As[0], a_contig_mn);
        lb.store(Bs[0], b_contig_mn);
    }
    __syncthreads();

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        const bool more = k0 + BK < kend;
        if (more) {
            la.load(p.A, p.lda, a_contig_mn, m0, p.m, k0 + BK, p.k, p.conja, p.tri_a, true, p.sym_a);
            lb.load(p.B, p.ldb, b_contig_mn, n0, p.n, k0 + BK, p.k, p.conjb, p.tri_b, false, p.sym_b);
        }
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            T a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; i++) a[i] = As[cur][kk][frag_pos<TM>(ty, i)];
#pragma unroll
            for (int j = 0; j < TN; j++) b[j] = Bs[cur][kk][frag_pos<TN>(tx, j)];
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) Ops<T>::fma_acc(acc[i][j], a[i], b[j]);
        }
        if (more) {
            la.store(As[cur ^ 1], a_contig_mn);
            lb.store(Bs[cur ^ 1], b_contig_mn);
        }
        __syncthreads();
        cur ^= 1;
    }

    // epilogue: C = alpha*acc + beta*C ; beta == 0 overwrites C
    const bool beta0 = Ops<T>::is_zero(p.beta);
#pragma unroll
    for (int j = 0; j < TN; j++) {
        const int col = n0 + frag_pos<TN>(tx, j);
        if (col >= p.n) continue;
#pragma unroll
        for (int i = 0; i < TM; i++) {
            const int row = m0 + frag_pos<TM>(ty, i);
            if (row >= p.m) continue;
            if (p.c_part == C_LOWER && row < col) continue;
            if (p.c_part == C_UPPER && row > col) continue;
            T *cp = p.C + (long long)col * p.ldc + row;
            T v = beta0 ? Ops<T>::mul(p.alpha, acc[i][j]) : Ops<T>::axpby(p.alpha, acc[i][j], p.beta, *cp);
            if (p.c_herm && row == col) v = Ops<T>::real_only(v);
            *cp = v;
        }
    }
}

template <typename T, int TM, int TN, int BK>
__global__ void __launch_bounds__(GEMM_THREADS)
gemm_simt_kernel(GemmArgs<T> p)
{
    gemm_simt_tile<T, TM, TN, BK>(p, blockIdx.x);
}

}  // namespace gbx_gemm
