// gb_trsm.cu -- triangular solve with multiple right-hand sides for sm_103a
// (bli_trsm_ex, frame/3/bli_l3_oapi_ex.c:692-801).
//
// The reference's blocked variant (frame/3/trsm/bli_trsm_blk_var1.c:37-189)
// solves a KC x KC diagonal block, then updates the rest of B with gemm;
// its macro-kernel walks MR-row panels serially (bli_trsm_ll_ker_var2.c).
// On a GPU the serial part must stay small, so the solve is recursive:
//     X1 = inv(L11) B1;  B2 -= L21 X1;  X2 = inv(L22) B2
// down to diagonal blocks of at most 64 rows, which one kernel solves by
// substitution on a shared-memory panel, one thread per right-hand side
// (or 8 lanes per right-hand side when there are few of them; FP64,
// diagonal pre-inverted as with BLIS_ENABLE_TRSM_PREINVERSION,
// ref_kernels/3/bli_trsm_ref.c:110-134).
// Nearly all m^2 n flops land in the off-diagonal gemm updates, which run
// on the native FP64 kernel or, in the precision form, on the Ozaki kernel.
// Right-side solves are turned into left-side ones by swapping B's strides
// and transposing A, the reduction of frame/3/bli_l3_oapi_ex.c:753-758.
#include <stdlib.h>

#include "gb_internal.h"

namespace gb {
namespace {

constexpr int TRSM_NB = 64;

// Solves op(A11) X = B1 in place for an nb x nb diagonal block.
// op(A)(i, l) = a[i*ars + l*acs]; B(i, j) = b[i*brs + j*bcs].  A CTA owns
// TRSM_COLS right-hand sides, one per thread: the triangle and the CTA's
// nb x TRSM_COLS panel of B are staged in shared memory (coalesced along B's
// contiguous direction), each thread runs forward / backward substitution on
// its column with four independent partial sums per row (a dependent chain
// of i/4 FMAs instead of i) and the pre-inverted diagonal, and the panel is
// written back.  One thread per column issues the fewest FP64 instructions,
// which is what bounds this kernel on GB300's narrow FP64 pipe.
constexpr int TRSM_COLS = 64, TRSM_THREADS = TRSM_COLS;

__global__ void __launch_bounds__(TRSM_THREADS) trsm_diag_kernel(int nb, int lower, int unit,
                                                                 const double* __restrict__ a, int64_t ars,
                                                                 int64_t acs, double* __restrict__ b,
                                                                 int64_t brs, int64_t bcs, int64_t ncols)
{
    extern __shared__ double trsm_smem[];
    constexpr int LL = TRSM_NB + 1, LX = TRSM_COLS + 1;
    double* L = trsm_smem;                 // [TRSM_NB][LL]
    double* dinv = L + TRSM_NB * LL;       // [TRSM_NB]
    double* X = dinv + TRSM_NB;            // [TRSM_NB][LX]
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * TRSM_COLS;
    const int cols = (ncols - j0 < TRSM_COLS) ? (int)(ncols - j0) : TRSM_COLS;
#pragma unroll 8
    for (int e = t; e < nb * nb; e += TRSM_THREADS) {
        const int i = e % nb, l = e / nb;
        const bool in_tri = lower ? (l <= i) : (l >= i);
        L[i * LL + l] = in_tri ? a[i * ars + l * acs] : 0.0;
    }
    const bool rows_fast = (brs == 1);
#pragma unroll 8
    for (int e = t; e < nb * TRSM_COLS; e += TRSM_THREADS) {
        const int i = rows_fast ? e % nb : e / TRSM_COLS, c = rows_fast ? e / nb : e % TRSM_COLS;
        X[i * LX + c] = (c < cols) ? b[i * brs + (j0 + c) * bcs] : 0.0;
    }
    __syncthreads();
    if (t < nb) dinv[t] = unit ? 1.0 : 1.0 / L[t * LL + t];
    __syncthreads();
    for (int step = 0; step < nb; ++step) {
        const int i = lower ? step : nb - 1 - step;
        const int l0 = lower ? 0 : i + 1, l1 = lower ? i : nb;
        double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
        int l = l0;
        for (; l + 3 < l1; l += 4) {
            p0 = fma(L[i * LL + l], X[l * LX + t], p0);
            p1 = fma(L[i * LL + l + 1], X[(l + 1) * LX + t], p1);
            p2 = fma(L[i * LL + l + 2], X[(l + 2) * LX + t], p2);
            p3 = fma(L[i * LL + l + 3], X[(l + 3) * LX + t], p3);
        }
        for (; l < l1; ++l) p0 = fma(L[i * LL + l], X[l * LX + t], p0);
        X[i * LX + t] = (X[i * LX + t] - ((p0 + p1) + (p2 + p3))) * dinv[i];
    }
    __syncthreads();
#pragma unroll 8
    for (int e = t; e < nb * TRSM_COLS; e += TRSM_THREADS) {
        const int i = rows_fast ? e % nb : e / TRSM_COLS, cc = rows_fast ? e / nb : e % TRSM_COLS;
        if (cc < cols) b[i * brs + (j0 + cc) * bcs] = X[i * LX + cc];
    }
}

// The same solve with 8 lanes per right-hand side, for few right-hand sides
// (fewer than one 64-column CTA per SM): each row's dot product is split over
// the lanes (lane g takes l = g, g + 8, ...) and combined with shuffles.  It
// spends more FP64 issue slots per column but keeps more SMs busy.
constexpr int TRSM_SCOLS = 32, TRSM_LANES = 8, TRSM_STHREADS = TRSM_SCOLS * TRSM_LANES;

__global__ void __launch_bounds__(TRSM_STHREADS) trsm_diag_split_kernel(int nb, int lower, int unit,
                                                                        const double* __restrict__ a, int64_t ars,
                                                                        int64_t acs, double* __restrict__ b,
                                                                        int64_t brs, int64_t bcs, int64_t ncols)
{
    extern __shared__ double trsm_smem[];
    constexpr int LL = TRSM_NB + 1, LX = TRSM_SCOLS + 1;
    double* L = trsm_smem;
    double* dinv = L + TRSM_NB * LL;
    double* X = dinv + TRSM_NB;
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * TRSM_SCOLS;
    const int cols = (ncols - j0 < TRSM_SCOLS) ? (int)(ncols - j0) : TRSM_SCOLS;
#pragma unroll 8
    for (int e = t; e < nb * nb; e += TRSM_STHREADS) {
        const int i = e % nb, l = e / nb;
        const bool in_tri = lower ? (l <= i) : (l >= i);
        L[i * LL + l] = in_tri ? a[i * ars + l * acs] : 0.0;
    }
    const bool rows_fast = (brs == 1);
#pragma unroll 8
    for (int e = t; e < nb * TRSM_SCOLS; e += TRSM_STHREADS) {
        const int i = rows_fast ? e % nb : e / TRSM_SCOLS, c = rows_fast ? e / nb : e % TRSM_SCOLS;
        X[i * LX + c] = (c < cols) ? b[i * brs + (j0 + c) * bcs] : 0.0;
    }
    __syncthreads();
    if (t < nb) dinv[t] = unit ? 1.0 : 1.0 / L[t * LL + t];
    __syncthreads();
    const int c = t / TRSM_LANES, g = t % TRSM_LANES;  // the 8 lanes of a column share a warp
    for (int step = 0; step < nb; ++step) {
        const int i = lower ? step : nb - 1 - step;
        const int l0 = lower ? 0 : i + 1, l1 = lower ? i : nb;
        double part = 0.0;
#pragma unroll 4
        for (int l = l0 + g; l < l1; l += TRSM_LANES) part = fma(L[i * LL + l], X[l * LX + c], part);
#pragma unroll
        for (int off = TRSM_LANES / 2; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
        if (g == 0) X[i * LX + c] = (X[i * LX + c] - part) * dinv[i];
        __syncwarp();
    }
    __syncthreads();
#pragma unroll 8
    for (int e = t; e < nb * TRSM_SCOLS; e += TRSM_STHREADS) {
        const int i = rows_fast ? e % nb : e / TRSM_SCOLS, cc = rows_fast ? e / nb : e % TRSM_SCOLS;
        if (cc < cols) b[i * brs + (j0 + cc) * bcs] = X[i * LX + cc];
    }
}

constexpr size_t TRSM_SSMEM = sizeof(double) * (TRSM_NB * (TRSM_NB + 1) + TRSM_NB + TRSM_NB * (TRSM_SCOLS + 1));

constexpr size_t TRSM_SMEM = sizeof(double) * (TRSM_NB * (TRSM_NB + 1) + TRSM_NB + TRSM_NB * (TRSM_COLS + 1));

// Multiply-adds below which a TRSM update runs natively in the precision form
// (GB_TRSM_OZAKI_MIN_FMA; default 0: measured on GB300, even the 64 x n x 64
// updates at the bottom of the recursion are faster in the Ozaki form).
double trsm_ozaki_min_fma()
{
    static double v = -1.0;
    if (v < 0.0) {
        const char* e = getenv("GB_TRSM_OZAKI_MIN_FMA");
        v = e ? atof(e) : 0.0;
        if (v < 0.0) v = 0.0;
    }
    return v;
}

struct TrsmCtx {
    int lower, unit, slices;
    const double* a;
    int64_t ars, acs;
    double* b;
    int64_t brs, bcs;
    int64_t n;
    cudaStream_t s;
};

int update(const TrsmCtx& t, int64_t r0, int64_t rcount, int64_t c0, int64_t ccount)
{
    // B[r0:r0+rcount, :] -= op(A)[r0:.., c0:c0+ccount] * X[c0:c0+ccount, :]
    const double* ap = t.a + r0 * t.ars + c0 * t.acs;
    const double* xp = t.b + c0 * t.brs;
    double* bp = t.b + r0 * t.brs;
    if (t.slices > 0 && (double)rcount * (double)ccount * (double)t.n >= trsm_ozaki_min_fma())
        return dgemm_ozaki(rcount, t.n, ccount, -1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp,
                           t.brs, t.bcs, t.slices, t.s);
    return dgemm_native(rcount, t.n, ccount, -1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp,
                        t.brs, t.bcs, t.s);
}

int solve(const TrsmCtx& t, int64_t r0, int64_t mm)
{
    if (mm <= TRSM_NB) {
        static bool attr = false;
        if (!attr) {
            int rc0 = check_cuda(cudaFuncSetAttribute(trsm_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)TRSM_SMEM), "trsm smem attr");
            if (!rc0)
                rc0 = check_cuda(cudaFuncSetAttribute(trsm_diag_split_kernel,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRSM_SSMEM),
                                 "trsm smem attr");
            if (rc0) return rc0;
            attr = true;
        }
        const int sms = sm_count() > 0 ? sm_count() : 148;
        const int64_t blocks = (t.n + TRSM_COLS - 1) / TRSM_COLS;
        LaunchScope ls("trsm_diag", t.s);
        if (blocks >= sms) {
            if (blocks > INT32_MAX) return set_error(GB_ERR_ARG, "dtrsm", "too many right-hand sides");
            trsm_diag_kernel<<<(unsigned)blocks, TRSM_THREADS, TRSM_SMEM, t.s>>>(
                (int)mm, t.lower, t.unit, t.a + r0 * t.ars + r0 * t.acs, t.ars, t.acs, t.b + r0 * t.brs, t.brs,
                t.bcs, t.n);
        } else {
            const int64_t sblocks = (t.n + TRSM_SCOLS - 1) / TRSM_SCOLS;
            trsm_diag_split_kernel<<<(unsigned)sblocks, TRSM_STHREADS, TRSM_SSMEM, t.s>>>(
                (int)mm, t.lower, t.unit, t.a + r0 * t.ars + r0 * t.acs, t.ars, t.acs, t.b + r0 * t.brs, t.brs,
                t.bcs, t.n);
        }
        return check_cuda(cudaGetLastError(), "trsm_diag");
    }
    // split on a multiple of the diagonal block size
    int64_t m1 = ((mm / 2 + TRSM_NB - 1) / TRSM_NB) * TRSM_NB;
    if (m1 >= mm) m1 = mm - TRSM_NB;
    const int64_t m2 = mm - m1;
    int rc;
    if (t.lower) {
        if ((rc = solve(t, r0, m1))) return rc;
        if ((rc = update(t, r0 + m1, m2, r0, m1))) return rc;
        return solve(t, r0 + m1, m2);
    }
    if ((rc = solve(t, r0 + m1, m2))) return rc;
    if ((rc = update(t, r0, m1, r0 + m1, m2))) return rc;
    return solve(t, r0, m1);
}

}  // namespace

int dtrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha,
              const double* a, int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b,
              int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    if (side == GB_RIGHT) {
        brs = cs_b;
        bcs = rs_b;
        mm = n;
        nn = m;
        trans = !trans;
    }
    if (alpha == 0.0) return scal_matrix(mm, nn, 0.0, b, brs, bcs, s);
    if (alpha != 1.0) {
        int rc = scal_matrix(mm, nn, alpha, b, brs, bcs, s);
        if (rc) return rc;
    }
    TrsmCtx t;
    t.ars = trans ? cs_a : rs_a;
    t.acs = trans ? rs_a : cs_a;
    t.lower = ((uplo == GB_LOWER) != trans) ? 1 : 0;
    t.unit = (diag == GB_UNIT_DIAG) ? 1 : 0;
    t.slices = slices;
    t.a = a;
    t.b = b;
    t.brs = brs;
    t.bcs = bcs;
    t.n = nn;
    t.s = s;
    return solve(t, 0, mm);
}

}  // namespace gb
