// gb_level3x.cu -- the remaining real level-3 operations for sm_103a, built on
// the gemm kernels (native FP64 or, in the precision form, Ozaki):
//   trmm   B := alpha op(A) B  or  alpha B op(A), A triangular (in place)
//          (bli_trmm_ex, frame/3/bli_l3_oapi_ex.c:609-690; dtrmm_,
//          frame/compat/bla_trmm.c:45-121)
//   symm   C := alpha A B + beta C  or  alpha B A + beta C, A symmetric
//          (bli_symm_ex, frame/3/bli_l3_oapi_ex.c:436-520; dsymm_,
//          frame/compat/bla_symm.c)
//   gemmt  C := alpha op(A) op(B) + beta C on one triangle of C
//          (bli_gemmt_ex, frame/3/bli_l3_oapi_ex.c:151-225; dgemmt_,
//          frame/compat/extra/bla_gemmt.c), and syrk through it as BLIS
//          does (frame/3/bli_l3_oapi_ex.c:326-345: C := alpha A A^T + beta C).
//
// trmm mirrors the recursive trsm: B = [B1; B2] with A = [A11 0; A21 A22]
// (lower) becomes B2 := A22 B2; B2 += A21 B1; B1 := A11 B1, down to 64-row
// diagonal blocks multiplied in shared memory, so nearly all flops are gemm
// updates.  In the precision form (more than 256 rows) trmm is instead one
// Ozaki product on the triangle materialised with zeros, reading the old B
// from a copy; the slice GEMM skips the k blocks beyond each tile row's
// triangle, so it does little more than the triangle's products, all at the
// tensor-core rate.
// symm materialises the full symmetric A once (a copy of n^2
// elements against the n^2 m flops of the product) and calls gemm.  gemmt
// works in 1024-column blocks of C: the part of a block column strictly
// inside the triangle is one gemm written in place, the diagonal block is a
// gemm into scratch merged into the triangle (beta applied there), so the
// other triangle is never computed beyond the diagonal blocks (at most
// 1024/m of the flops) and never touched.  In the precision form gemmt is
// one Ozaki product whose slice GEMM runs only the tiles holding part of the
// triangle and whose recombination writes only the triangle.
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int DB_NB = 64;        // diagonal block
constexpr int DB_THREADS = 128;  // threads per CTA of the diagonal-block kernels

// Diagonal blocks of op(A) for trmm, packed once per call: block q becomes a
// row-major 64 x 64 array with a_ri inside the triangle (1 on the diagonal
// for a unit diagonal, and for the identity rows padding a short last block)
// and 0 elsewhere.
template <bool LOWER>
__global__ void __launch_bounds__(256) trmm_pack_diag_kernel(int64_t m, int unit, const double* __restrict__ a,
                                                             int64_t ars, int64_t acs, double* __restrict__ packed)
{
    const int64_t r0 = (int64_t)blockIdx.x * DB_NB;
    const int nb = (m - r0 < DB_NB) ? (int)(m - r0) : DB_NB;
    const double* blk = a + r0 * ars + r0 * acs;
    double* out = packed + (int64_t)blockIdx.x * DB_NB * DB_NB;
    const bool rows_fast = (ars == 1);
    for (int e = threadIdx.x; e < DB_NB * DB_NB; e += 256) {
        // read along A's contiguous direction, write row-major
        const int i = rows_fast ? e % DB_NB : e / DB_NB, l = rows_fast ? e / DB_NB : e % DB_NB;
        double v = 0.0;
        if (i == l) v = (unit || i >= nb) ? 1.0 : blk[i * ars + l * acs];
        else if (i < nb && l < nb && (LOWER ? (l < i) : (l > i))) v = blk[i * ars + l * acs];
        out[i * DB_NB + l] = v;
    }
}

// X1 := P X1 for one packed diagonal block P, in place; B(i, j) at
// b[i*brs + j*bcs], rows past nb neither read nor written.  A CTA owns
// DB_THREADS / LANES columns: P and the panel are staged in shared memory
// (coalesced along B's contiguous direction), lane g of a column computes
// rows r = q * LANES + g, y_r = sum over the triangle of P[r][l] x_l, with
// x_l read once per l for all its rows; the results replace the panel after
// a barrier.  Both loops are unrolled, so the register indices are constants
// and the groups no lane needs are dropped at compile time.  Bound by the
// FP64 pipe like the trsm kernel (the same instruction count: one FMA per
// triangle entry per column).
template <int LANES, bool LOWER>
__global__ void __launch_bounds__(DB_THREADS) trmm_diag_kernel(int nb, const double* __restrict__ pk,
                                                               double* __restrict__ b, int64_t brs, int64_t bcs,
                                                               int64_t ncols)
{
    constexpr int COLS = DB_THREADS / LANES, R = DB_NB / LANES, LL = DB_NB + 1, LX = COLS + 1;
    extern __shared__ double trmm_smem[];
    double* P = trmm_smem;             // [DB_NB][LL]
    double* X = P + DB_NB * LL;        // [DB_NB][LX]
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * COLS;
    const int cols = (ncols - j0 < COLS) ? (int)(ncols - j0) : COLS;
#pragma unroll 8
    for (int e = t; e < DB_NB * DB_NB; e += DB_THREADS) P[(e / DB_NB) * LL + e % DB_NB] = pk[e];
    const bool rows_fast = (brs == 1);
#pragma unroll 8
    for (int e = t; e < DB_NB * COLS; e += DB_THREADS) {
        const int i = rows_fast ? e % DB_NB : e / COLS, c = rows_fast ? e / DB_NB : e % COLS;
        X[i * LX + c] = (c < cols && i < nb) ? b[i * brs + (j0 + c) * bcs] : 0.0;
    }
    __syncthreads();
    const int c = t / LANES, g = t % LANES;
    double y[R];
#pragma unroll
    for (int q = 0; q < R; ++q) y[q] = 0.0;
#pragma unroll
    for (int l = 0; l < DB_NB; ++l) {
        const double xl = X[l * LX + c];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            // rows q * LANES .. q * LANES + LANES - 1; lower: rows r >= l, upper: rows r <= l
            if (LOWER ? (q * LANES + LANES - 1 >= l) : (q * LANES <= l)) {
                const int r = q * LANES + g;
                if (LOWER ? (r >= l) : (r <= l)) y[q] = fma(P[r * LL + l], xl, y[q]);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < R; ++q) X[(q * LANES + g) * LX + c] = y[q];
    __syncthreads();
#pragma unroll 8
    for (int e = t; e < DB_NB * COLS; e += DB_THREADS) {
        const int i = rows_fast ? e % DB_NB : e / COLS, cc = rows_fast ? e / DB_NB : e % COLS;
        if (cc < cols && i < nb) b[i * brs + (j0 + cc) * bcs] = X[i * LX + cc];
    }
}

constexpr size_t trmm_smem_bytes(int lanes)
{
    return sizeof(double) * (DB_NB * (DB_NB + 1) + DB_NB * (DB_THREADS / lanes + 1));
}

template <int LANES, bool LOWER>
int launch_trmm_diag(int nb, const double* pk, double* b, int64_t brs, int64_t bcs, int64_t ncols, cudaStream_t s)
{
    static bool attr = false;
    if (!attr) {
        const int rc = check_cuda(cudaFuncSetAttribute(trmm_diag_kernel<LANES, LOWER>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)trmm_smem_bytes(LANES)), "trmm smem attr");
        if (rc) return rc;
        attr = true;
    }
    const int64_t blocks = (ncols + DB_THREADS / LANES - 1) / (DB_THREADS / LANES);
    if (blocks > INT32_MAX) return set_error(GB_ERR_ARG, "dtrmm", "too many columns");
    trmm_diag_kernel<LANES, LOWER><<<(unsigned)blocks, DB_THREADS, trmm_smem_bytes(LANES), s>>>(nb, pk, b, brs, bcs,
                                                                                               ncols);
    return check_cuda(cudaGetLastError(), "trmm_diag");
}

// Full symmetric A (n x n, column-major out[i + j*n]) from the uplo triangle
// of a (element (i, j) at a[i*rs + j*cs]); the other triangle is not read.
__global__ void __launch_bounds__(256) symmetrize_kernel(int64_t n, int lower, const double* __restrict__ a,
                                                         int64_t rs, int64_t cs, double* __restrict__ out)
{
    const int64_t total = n * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / n, i = e - j * n;
        const bool stored = lower ? (i >= j) : (i <= j);
        out[e] = stored ? a[i * rs + j * cs] : a[j * rs + i * cs];
    }
}

// C := D + beta C on the uplo triangle of a w x w diagonal block (D column-
// major with leading dimension w, alpha already applied); beta = 0 writes D
// without reading C.  The other triangle of C is not touched.
__global__ void __launch_bounds__(256) triangle_merge_kernel(int64_t w, int lower, const double* __restrict__ d,
                                                             double beta, double* __restrict__ c, int64_t rs_c,
                                                             int64_t cs_c)
{
    const int64_t total = w * w;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / w, i = e - j * w;
        if (lower ? (i < j) : (i > j)) continue;
        double* cij = c + i * rs_c + j * cs_c;
        *cij = (beta == 0.0) ? d[e] : __fma_rn(beta, *cij, d[e]);
    }
}

// tri(op(A)) (m x m, op(A) (i, j) at a[i*ars + j*acs]) as a dense column-
// major matrix: the uplo triangle, ones on the diagonal when unit, zeros
// elsewhere
__global__ void __launch_bounds__(256) tri_materialize_kernel(int64_t m, int lower, int unit,
                                                              const double* __restrict__ a, int64_t ars,
                                                              int64_t acs, double* __restrict__ out)
{
    const int64_t total = m * m;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / m, i = e - j * m;
        double v = 0.0;
        if (i == j) v = unit ? 1.0 : a[i * ars + j * acs];
        else if (lower ? (i > j) : (i < j)) v = a[i * ars + j * acs];
        out[e] = v;
    }
}

// out (m x n column-major) := B (element (i, j) at b[i*rs + j*cs])
__global__ void __launch_bounds__(256) gather_matrix_kernel(int64_t m, int64_t n, const double* __restrict__ b,
                                                            int64_t rs, int64_t cs, double* __restrict__ out)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / m, i = e - j * m;
        out[e] = b[i * rs + j * cs];
    }
}

unsigned grid_for(int64_t total)
{
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t blocks = (total + 255) / 256;
    if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

int gemm_form(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t ars, int64_t acs,
              const double* b, int64_t brs, int64_t bcs, double beta, double* c, int64_t rs_c, int64_t cs_c,
              int slices, cudaStream_t s)
{
    if (slices > 0)
        return dgemm_ozaki(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, slices, s);
    return dgemm_native(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, s);
}

struct TrmmCtx {
    int lower, slices;
    const double* packed;
    const double* a;
    int64_t ars, acs;
    double* b;
    int64_t brs, bcs;
    int64_t n;
    cudaStream_t s;
};

// B[r0 : r0+rcount, :] += op(A)[r0.., c0 : c0+ccount] B[c0 : c0+ccount, :]
int trmm_update(const TrmmCtx& t, int64_t r0, int64_t rcount, int64_t c0, int64_t ccount)
{
    const double* ap = t.a + r0 * t.ars + c0 * t.acs;
    const double* xp = t.b + c0 * t.brs;
    double* bp = t.b + r0 * t.brs;
    if (t.slices > 0)
        return dgemm_ozaki(rcount, t.n, ccount, 1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp, t.brs, t.bcs,
                           t.slices, t.s);
    return dgemm_native(rcount, t.n, ccount, 1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp, t.brs, t.bcs, t.s);
}

int trmm_mult(const TrmmCtx& t, int64_t r0, int64_t mm)
{
    if (mm <= DB_NB) {
        const double* pk = t.packed + (r0 / DB_NB) * DB_NB * DB_NB;  // r0 stays a multiple of the block
        double* b1 = t.b + r0 * t.brs;
        const int nb = (int)mm;
        LaunchScope ls("trmm_diag", t.s);
        switch (diag_block_lanes(t.n)) {
        case 1:
            return t.lower ? launch_trmm_diag<1, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_trmm_diag<1, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        case 2:
            return t.lower ? launch_trmm_diag<2, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_trmm_diag<2, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        case 4:
            return t.lower ? launch_trmm_diag<4, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_trmm_diag<4, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        default:
            return t.lower ? launch_trmm_diag<8, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_trmm_diag<8, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        }
    }
    int64_t m1 = ((mm / 2 + DB_NB - 1) / DB_NB) * DB_NB;
    if (m1 >= mm) m1 = mm - DB_NB;
    const int64_t m2 = mm - m1;
    int rc;
    if (t.lower) {
        // the new B2 needs the old B1: B2 first, B1 last
        if ((rc = trmm_mult(t, r0 + m1, m2))) return rc;
        if ((rc = trmm_update(t, r0 + m1, m2, r0, m1))) return rc;
        return trmm_mult(t, r0, m1);
    }
    if ((rc = trmm_mult(t, r0, m1))) return rc;
    if ((rc = trmm_update(t, r0, m1, r0 + m1, m2))) return rc;
    return trmm_mult(t, r0 + m1, m2);
}

}  // namespace

int dtrmm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha, const double* a,
              int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    if (side == GB_RIGHT) {
        // B op(A) = (op(A)^T B^T)^T: a left-side product on B^T
        brs = cs_b;
        bcs = rs_b;
        mm = n;
        nn = m;
        trans = !trans;
    }
    if (alpha == 0.0) return scal_matrix(mm, nn, 0.0, b, brs, bcs, s);  // A is not read
    TrmmCtx t;
    t.ars = trans ? cs_a : rs_a;
    t.acs = trans ? rs_a : cs_a;
    t.lower = ((uplo == GB_LOWER) != trans) ? 1 : 0;
    if (slices > 0 && mm > 4 * DB_NB) {
        // The precision form as ONE Ozaki product on the triangle materialised
        // with zeros: twice the products of the triangle, all at the slice
        // GEMM's rate, where the recursion's FP64 diagonal multiplies and its
        // many small updates set its pace.  The old B is read from a copy.
        double* full = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(mm * mm + mm * nn), s));
        if (!full) return GB_ERR_NOMEM;
        double* old = full + mm * mm;
        {
            LaunchScope ls("trmm_materialize", s);
            tri_materialize_kernel<<<grid_for(mm * mm), 256, 0, s>>>(mm, t.lower, diag == GB_UNIT_DIAG, a, t.ars,
                                                                     t.acs, full);
            gather_matrix_kernel<<<grid_for(mm * nn), 256, 0, s>>>(mm, nn, b, brs, bcs, old);
        }
        int rc = check_cuda(cudaGetLastError(), "trmm materialize");
        OzA prep;
        if (!rc) rc = ozaki_prepare_a(mm, mm, full, 1, mm, slices, s, &prep);
        if (!rc) {
            prep.tri = t.lower ? 1 : 2;  // the slice GEMM skips the k blocks beyond each tile row's triangle
            rc = ozaki_multiply(&prep, nn, old, 1, mm, alpha, 0.0, b, brs, bcs, s);
            ozaki_release_a(&prep, s);
        }
        dev_free(full, s);
        return rc;
    }
    t.slices = slices;
    t.a = a;
    t.b = b;
    t.brs = brs;
    t.bcs = bcs;
    t.n = nn;
    t.s = s;
    const int64_t nblk = (mm + DB_NB - 1) / DB_NB;
    if (nblk > INT32_MAX) return set_error(GB_ERR_ARG, "dtrmm", "too many diagonal blocks");
    double* packed = static_cast<double*>(dev_alloc(sizeof(double) * nblk * DB_NB * DB_NB, s));
    if (!packed) return GB_ERR_NOMEM;
    {
        LaunchScope ls("trmm_pack_diag", s);
        if (t.lower)
            trmm_pack_diag_kernel<true><<<(unsigned)nblk, 256, 0, s>>>(mm, diag == GB_UNIT_DIAG, a, t.ars, t.acs,
                                                                       packed);
        else
            trmm_pack_diag_kernel<false><<<(unsigned)nblk, 256, 0, s>>>(mm, diag == GB_UNIT_DIAG, a, t.ars, t.acs,
                                                                        packed);
    }
    int rc = check_cuda(cudaGetLastError(), "trmm_pack_diag");
    t.packed = packed;
    if (!rc) rc = trmm_mult(t, 0, mm);
    // alpha as one multiply per element of the product (exact for alpha = 1 and powers of two)
    if (!rc && alpha != 1.0) rc = scal_matrix(mm, nn, alpha, b, brs, bcs, s);
    dev_free(packed, s);
    return rc;
}

// trmm3: C := beta C + alpha op(A) op(B) (left, A m x m) or beta C + alpha
// op(B) op(A) (right, A n x n), A triangular, C m x n; B is not written
// (bli_trmm3_ex, frame/3/bli_l3_oapi_ex.c:523-608; alpha == 0 scales C only,
// frame/3/bli_l3_util.c:41-65).  tri(op(A)) is materialised with zeros and
// multiplied as a gemm: in the precision form one Ozaki product whose slice
// GEMM skips the all-zero k blocks (as trmm), natively the dense DMMA gemm.
int dtrmm3_dev(int side, int uplo, int transa, int diag, int transb, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta,
               double* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    // op(B) (i, j) at b[i*brs + j*bcs]
    int64_t brs = GB_IS_TRANS(transb) ? cs_b : rs_b, bcs = GB_IS_TRANS(transb) ? rs_b : cs_b;
    int64_t crs = rs_c, ccs = cs_c, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    if (side == GB_RIGHT) {
        // C^T = beta C^T + alpha op(A)^T op(B)^T: the left form on the transposes
        const int64_t t0 = brs;
        brs = bcs;
        bcs = t0;
        crs = cs_c;
        ccs = rs_c;
        mm = n;
        nn = m;
        trans = !trans;
    }
    if (alpha == 0.0) return scal_matrix(mm, nn, beta, c, crs, ccs, s);  // A and B are not read
    const int64_t ars = trans ? cs_a : rs_a, acs = trans ? rs_a : cs_a;
    const bool lower = (uplo == GB_LOWER) != trans;
    double* full = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(mm * mm), s));
    if (!full) return GB_ERR_NOMEM;
    int rc;
    {
        LaunchScope ls("trmm_materialize", s);
        tri_materialize_kernel<<<grid_for(mm * mm), 256, 0, s>>>(mm, lower ? 1 : 0, diag == GB_UNIT_DIAG, a, ars, acs,
                                                                 full);
        rc = check_cuda(cudaGetLastError(), "trmm3 materialize");
    }
    if (!rc && slices > 0) {
        OzA prep;
        rc = ozaki_prepare_a(mm, mm, full, 1, mm, slices, s, &prep);
        if (!rc) {
            prep.tri = lower ? 1 : 2;
            rc = ozaki_multiply(&prep, nn, b, brs, bcs, alpha, beta, c, crs, ccs, s);
            ozaki_release_a(&prep, s);
        }
    } else if (!rc) {
        rc = dgemm_native(mm, nn, mm, alpha, full, 1, mm, b, brs, bcs, beta, c, crs, ccs, s);
    }
    dev_free(full, s);
    return rc;
}

int dsymm_dev(int side, int uplo, int64_t m, int64_t n, double alpha, const double* a, int64_t rs_a,
              int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c,
              int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0) return scal_matrix(m, n, beta, c, rs_c, cs_c, s);  // A and B are not read
    const int64_t na = (side == GB_LEFT) ? m : n;
    double* full = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(na * na), s));
    if (!full) return GB_ERR_NOMEM;
    {
        LaunchScope ls("symmetrize", s);
        symmetrize_kernel<<<grid_for(na * na), 256, 0, s>>>(na, uplo == GB_LOWER, a, rs_a, cs_a, full);
    }
    int rc = check_cuda(cudaGetLastError(), "symmetrize");
    if (!rc) {
        if (side == GB_LEFT)
            rc = gemm_form(m, n, m, alpha, full, 1, m, b, rs_b, cs_b, beta, c, rs_c, cs_c, slices, s);
        else
            rc = gemm_form(m, n, n, alpha, b, rs_b, cs_b, full, 1, n, beta, c, rs_c, cs_c, slices, s);
    }
    dev_free(full, s);
    return rc;
}

int dgemmt_dev(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a,
               int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c,
               int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0) return GB_SUCCESS;
    const bool lower = (uplo == GB_LOWER);
    // op(A) (i, l) at a[i*ars + l*acs]; op(B) (l, j) at b[l*brs + j*bcs]
    const int64_t ars = GB_IS_TRANS(transa) ? cs_a : rs_a, acs = GB_IS_TRANS(transa) ? rs_a : cs_a;
    const int64_t brs = GB_IS_TRANS(transb) ? cs_b : rs_b, bcs = GB_IS_TRANS(transb) ? rs_b : cs_b;
    constexpr int64_t W = 1024;  // block columns of C; a multiple of the slice GEMM's row tile
    const int64_t wmax = (m < W) ? m : W;
    double* scratch = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(wmax * wmax), s));
    if (!scratch) return GB_ERR_NOMEM;
    int rc = GB_SUCCESS;
    const bool trivial = (alpha == 0.0 || k <= 0);
    if (slices > 0 && !trivial) {
        // the precision form in one product: the slice GEMM runs only the
        // tiles that hold part of the triangle and the recombination writes
        // only the triangle (beta applied there)
        dev_free(scratch, s);
        OzA prep;
        if ((rc = ozaki_prepare_a(m, k, a, ars, acs, slices, s, &prep))) return rc;
        prep.out_tri = lower ? 1 : 2;
        rc = ozaki_multiply(&prep, m, b, brs, bcs, alpha, beta, c, rs_c, cs_c, s);
        ozaki_release_a(&prep, s);
        return rc;
    }
    // the native form (and a trivial product) in 1024-column blocks
    for (int64_t j0 = 0; j0 < m && !rc; j0 += W) {
        const int64_t w = (m - j0 < W) ? m - j0 : W;
        double* cblk = c + j0 * rs_c + j0 * cs_c;
        if (trivial) {
            // C := beta C on the triangle only: a zero product merged in
            if ((rc = check_cuda(cudaMemsetAsync(scratch, 0, sizeof(double) * (size_t)(w * w), s), "memset"))) break;
        }
        // strictly-triangle panel of this block column: rows below (lower) or above (upper)
        const int64_t pr0 = lower ? j0 + w : 0, prows = lower ? m - (j0 + w) : j0;
        if (!trivial) {
            // diagonal block into scratch (alpha applied, beta 0), merged below
            rc = dgemm_native(w, w, k, alpha, a + j0 * ars, ars, acs, b + j0 * bcs, brs, bcs, 0.0, scratch, 1, w, s);
            if (!rc && prows > 0)
                rc = dgemm_native(prows, w, k, alpha, a + pr0 * ars, ars, acs, b + j0 * bcs, brs, bcs, beta,
                                  c + pr0 * rs_c + j0 * cs_c, rs_c, cs_c, s);
        } else if (prows > 0) {
            rc = scal_matrix(prows, w, beta, c + pr0 * rs_c + j0 * cs_c, rs_c, cs_c, s);
        }
        if (rc) break;
        {
            LaunchScope ls("triangle_merge", s);
            triangle_merge_kernel<<<grid_for(w * w), 256, 0, s>>>(w, lower, scratch, beta, cblk, rs_c, cs_c);
        }
        rc = check_cuda(cudaGetLastError(), "triangle_merge");
    }
    dev_free(scratch, s);
    return rc;
}

// syr2k: the stored triangle of C := alpha op(A) op(B)^T + alpha op(B)
// op(A)^T + beta C, op(A), op(B) m x k -- as BLIS, two gemmt calls, the
// second accumulating onto the first (bli_syr2k_ex,
// frame/3/bli_l3_oapi_ex.c:267-292).
int dsyr2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a, int64_t rs_a,
               int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c,
               int64_t cs_c, int slices, cudaStream_t s)
{
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    const int na = ta ? GB_TRANSPOSE : GB_NO_TRANSPOSE, fa = ta ? GB_NO_TRANSPOSE : GB_TRANSPOSE;
    const int nb = tb ? GB_TRANSPOSE : GB_NO_TRANSPOSE, fb = tb ? GB_NO_TRANSPOSE : GB_TRANSPOSE;
    int rc = dgemmt_dev(uplo, na, fb, m, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c, slices, s);
    if (rc || alpha == 0.0 || k <= 0) return rc;
    return dgemmt_dev(uplo, nb, fa, m, k, alpha, b, rs_b, cs_b, a, rs_a, cs_a, 1.0, c, rs_c, cs_c, slices, s);
}

}  // namespace gb
