// gemm.cu — the host side of the GEMM core shared by every Level-3 routine:
// the beta-scaling kernel, the tile-size choice and launch, and the netlib
// argument checks.  The BLAS entry points themselves are in level3.cu.
//
// Argument checks use the netlib INFO numbering that the reference's wrappers
// replicate (blas_level3/gemm.cc:87-127, syrk.cc:78-146, trmm.cc:82-137); on
// the device layer an invalid argument returns GBX_ERR_ARG and the position
// is recorded in the context's error text.
#include "gbx_internal.h"
#include "gemm_simt.cuh"
#include "gemm_host.h"

#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <type_traits>

using namespace gbx_gemm;

namespace {

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

template <typename T>
__global__ void scale_matrix_kernel(int m, int n, T beta, T *C, long long ldc, int part, int herm)
{
    const long long total = (long long)m * n;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % m), j = (int)(t / m);
        if (part == C_LOWER && i < j) continue;
        if (part == C_UPPER && i > j) continue;
        T *cp = C + (long long)j * ldc + i;
        T v = Ops<T>::is_zero(beta) ? Ops<T>::zero() : Ops<T>::mul(beta, *cp);
        if (herm && i == j) v = Ops<T>::real_only(v);
        *cp = v;
    }
}

}  // namespace

namespace gbx_gemm {

template <typename T>
gbx_status scale_matrix(gbx_ctx *ctx, int m, int n, T beta, T *C, long long ldc, int part, int herm)
{
    if (m <= 0 || n <= 0) return GBX_OK;
    long long total = (long long)m * n;
    long long g = std::min<long long>((total + 255) / 256, (long long)gbx_ctx_sms(ctx) * 8);
    scale_matrix_kernel<T><<<(int)g, 256, 0, S(ctx)>>>(m, n, beta, C, ldc, part, herm);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "scale_matrix");
}
template gbx_status scale_matrix<float>(gbx_ctx *, int, int, float, float *, long long, int, int);
template gbx_status scale_matrix<double>(gbx_ctx *, int, int, double, double *, long long, int, int);
template gbx_status scale_matrix<fcplx>(gbx_ctx *, int, int, fcplx, fcplx *, long long, int, int);
template gbx_status scale_matrix<dcplx>(gbx_ctx *, int, int, dcplx, dcplx *, long long, int, int);

template <typename T, int TM>
gbx_status launch_gemm_tile(gbx_ctx *ctx, GemmArgs<T> p, const char *what)
{
    constexpr int TN = TM, BK = TM == 1 ? 16 : 8;
    constexpr int BM = 16 * TM, BN = 16 * TN;
    p.tiles_m = (p.m + BM - 1) / BM;
    p.tiles_n = (p.n + BN - 1) / BN;
    long long blocks;
    if (p.c_part == C_FULL) blocks = (long long)p.tiles_m * p.tiles_n;
    else {
        if (p.m != p.n) return gbx_fail(ctx, GBX_ERR_ARG, "%s: triangular C must be square", what);
        blocks = (long long)p.tiles_m * (p.tiles_m + 1) / 2;
    }
    if (blocks > 0x7fffffffLL) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "%s: grid too large", what);
    gbx_timer_begin(ctx, GBX_TIMER_GEMM_FP64);
    gemm_simt_kernel<T, TM, TN, BK><<<(unsigned)blocks, GEMM_THREADS, 0, S(ctx)>>>(p);
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, what);
}

// Tile choice.  Real double: the tile (64x64, 32x32 or 16x16 with one
// element per thread) with the best product of its kernel's efficiency and
// the fill of its last wave.  At 2 FP64 lanes per clock per SM each SM works
// through its share of tiles one after another, so a launch takes
// ceil(tiles / SMs) tile times: 512 tiles of 64x64 (DGEMM 2048x1024x2048, a
// DTRSM update) take four tile times on 152 SMs for 3.37 tiles' work (0.84),
// the same product as 8192 tiles of 16x16 runs at 0.98.  Measured DGEMM
// rates with the other shapes equal: 64x64 1.249, 32x32 1.247, 16x16 1.23
// TFLOP/s; 2048x1024x2048 takes 8.25 / 7.17 / 6.96 ms on the three tiles,
// 1024^3 2.11 / 1.80 / 1.75 ms, 4096x1024x4096 28.7 / 27.6 / 27.8 ms.  Two
// CTAs of 124 registers per SM keep the DFMA pipe fed across each CTA's
// barriers, so 64x64 beats 128x128 (DGEMM 8192^3 881 against 901 ms).
// Other types: the largest tile that still gives every SM two tiles,
// 128x128 for float and complex float (their faster FMA pipe needs the
// operand reuse), 64x64 and 32x32 for complex double (its 8x8 register tile
// would not fit), then smaller for the skinny and small products.
template <typename T>
gbx_status launch_gemm(gbx_ctx *ctx, GemmArgs<T> p, const char *what)
{
    if (p.m <= 0 || p.n <= 0) return GBX_OK;
    const long long want = 2LL * gbx_ctx_sms(ctx);
    auto tiles = [&](int bm) {
        const long long tm = (p.m + bm - 1) / bm, tn = (p.n + bm - 1) / bm;
        return p.c_part == C_FULL ? tm * tn : tm * (tm + 1) / 2;
    };
    if constexpr (std::is_same<T, double>::value) {
        const int bm = gbx_dgemm_tile_choice(p.m, p.n, p.c_part != C_FULL, gbx_ctx_sms(ctx));
        if (bm == 64) return launch_gemm_tile<T, 4>(ctx, p, what);
        if (bm == 32) return launch_gemm_tile<T, 2>(ctx, p, what);
        return launch_gemm_tile<T, 1>(ctx, p, what);
    } else if constexpr (sizeof(T) <= 8) {
        if (tiles(128) >= want) return launch_gemm_tile<T, 8>(ctx, p, what);
        if (tiles(64) >= want) return launch_gemm_tile<T, 4>(ctx, p, what);
        if (tiles(32) >= want) return launch_gemm_tile<T, 2>(ctx, p, what);
        return launch_gemm_tile<T, 1>(ctx, p, what);
    } else {
        if (tiles(64) >= want) return launch_gemm_tile<T, 4>(ctx, p, what);
        return launch_gemm_tile<T, 2>(ctx, p, what);
    }
}
template gbx_status launch_gemm<float>(gbx_ctx *, GemmArgs<float>, const char *);
template gbx_status launch_gemm<double>(gbx_ctx *, GemmArgs<double>, const char *);
template gbx_status launch_gemm<fcplx>(gbx_ctx *, GemmArgs<fcplx>, const char *);
template gbx_status launch_gemm<dcplx>(gbx_ctx *, GemmArgs<dcplx>, const char *);

}  // namespace gbx_gemm

// The FP64 block tile (64, 32 or 16) for an m x n output (its lower or upper
// triangle when triangular) on `sms` SMs: the best product of the kernel's
// own efficiency and the fill of its last wave (see launch_gemm).
extern "C" int gbx_dgemm_tile_choice(int m, int n, int triangular, int sms)
{
    if (m <= 0 || n <= 0 || sms <= 0) return 16;
    auto score = [&](int bm, double eff) {
        const long long tm = (m + bm - 1) / bm, tn = (n + bm - 1) / bm;
        const double w = (double)(triangular ? tm * (tm + 1) / 2 : tm * tn) / sms;
        return eff * w / std::ceil(w);
    };
    const double s64 = score(64, 1.0), s32 = score(32, 0.998), s16 = score(16, 0.985);
    if (s64 >= s32 && s64 >= s16) return 64;
    return s32 >= s16 ? 32 : 16;
}

// ------------------------------------------------------------------ checks
extern "C" int gbx_check_gemm_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc)
{
    const int nota = gbx_lsame(ta, 'N'), notb = gbx_lsame(tb, 'N');
    const int nrowa = nota ? m : k, nrowb = notb ? k : n;
    if (!nota && !gbx_lsame(ta, 'C') && !gbx_lsame(ta, 'T')) return 1;
    if (!notb && !gbx_lsame(tb, 'C') && !gbx_lsame(tb, 'T')) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (k < 0) return 5;
    if (lda < std::max(1, nrowa)) return 8;
    if (ldb < std::max(1, nrowb)) return 10;
    if (ldc < std::max(1, m)) return 13;
    return 0;
}

extern "C" int gbx_check_syrk_args(char uplo, char trans, int n, int k, int lda, int ldc)
{
    const int nrowa = gbx_lsame(trans, 'N') ? n : k;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (!gbx_lsame(trans, 'N') && !gbx_lsame(trans, 'T') && !gbx_lsame(trans, 'C')) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < std::max(1, nrowa)) return 7;
    if (ldc < std::max(1, n)) return 10;
    return 0;
}

extern "C" int gbx_check_trxm_args(char side, char uplo, char ta, char diag, int m, int n, int lda,
                                   int ldb)
{
    const int lside = gbx_lsame(side, 'L');
    const int nrowa = lside ? m : n;
    if (!lside && !gbx_lsame(side, 'R')) return 1;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 2;
    if (!gbx_lsame(ta, 'N') && !gbx_lsame(ta, 'T') && !gbx_lsame(ta, 'C')) return 3;
    if (!gbx_lsame(diag, 'U') && !gbx_lsame(diag, 'N')) return 4;
    if (m < 0) return 5;
    if (n < 0) return 6;
    if (lda < std::max(1, nrowa)) return 9;
    if (ldb < std::max(1, m)) return 11;
    return 0;
}

// Rank-k and rank-2k updates: which transposition letters a routine takes
// (real: N, T, C; complex symmetric: N, T; Hermitian: N, C).
extern "C" int gbx_trans_ok(char trans, int allowed)
{
    return (gbx_lsame(trans, 'N') && (allowed & GBX_TR_N)) || (gbx_lsame(trans, 'T') && (allowed & GBX_TR_T)) ||
           (gbx_lsame(trans, 'C') && (allowed & GBX_TR_C));
}

// xSYRK / xHERK (netlib numbering: uplo 1, trans 2, n 3, k 4, lda 7, ldc 10)
extern "C" int gbx_check_rank_k_args(char uplo, char trans, int allowed, int n, int k, int lda, int ldc)
{
    const int nrowa = gbx_lsame(trans, 'N') ? n : k;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (!gbx_trans_ok(trans, allowed)) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < std::max(1, nrowa)) return 7;
    if (ldc < std::max(1, n)) return 10;
    return 0;
}

// xSYR2K / xHER2K (uplo 1, trans 2, n 3, k 4, lda 7, ldb 9, ldc 12)
extern "C" int gbx_check_rank_2k_args(char uplo, char trans, int allowed, int n, int k, int lda, int ldb,
                                      int ldc)
{
    const int nrowa = gbx_lsame(trans, 'N') ? n : k;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (!gbx_trans_ok(trans, allowed)) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < std::max(1, nrowa)) return 7;
    if (ldb < std::max(1, nrowa)) return 9;
    if (ldc < std::max(1, n)) return 12;
    return 0;
}

// xSYMM / xHEMM (side 1, uplo 2, m 3, n 4, lda 7, ldb 9, ldc 12)
extern "C" int gbx_check_symm_args(char side, char uplo, int m, int n, int lda, int ldb, int ldc)
{
    const int nrowa = gbx_lsame(side, 'L') ? m : n;
    if (!gbx_lsame(side, 'L') && !gbx_lsame(side, 'R')) return 1;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (lda < std::max(1, nrowa)) return 7;
    if (ldb < std::max(1, m)) return 9;
    if (ldc < std::max(1, m)) return 12;
    return 0;
}

// ------------------------------------------------------ triangular operands
// Effective triangle of op(A): transposing swaps lower and upper.
extern "C" int gbx_op_tri(char uplo, char transa, char diag)
{
    const bool lower = gbx_lsame(uplo, 'L');
    const bool notr = gbx_lsame(transa, 'N');
    int t = (lower == notr) ? TRI_LOWER : TRI_UPPER;
    if (gbx_lsame(diag, 'U')) t |= TRI_UNIT;
    return t;
}

