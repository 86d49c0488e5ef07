// gb_hermitian.cu -- the complex rank-k updates and the complex symmetric /
// Hermitian products for sm_103a:
//   herk   C := alpha op(A) op(A)^H + beta C, alpha and beta real, on one
//          triangle of C (bli_herk_ex, frame/3/bli_l3_oapi_ex.c:295-320;
//          zherk_ / cherk_, frame/compat/bla_herk.c)
//   her2k  C := alpha op(A) op(B)^H + conj(alpha) op(B) op(A)^H + beta C,
//          beta real (bli_her2k_ex, frame/3/bli_l3_oapi_ex.c:229-264;
//          frame/compat/bla_her2k.c)
//   hemm / symm (complex)  C := alpha A B + beta C (left) or alpha B A +
//          beta C (right), A Hermitian or symmetric with one triangle stored
//          (bli_hemm_ex / bli_symm_ex, frame/3/bli_l3_oapi_ex.c:349-520;
//          frame/compat/bla_hemm.c, bla_symm.c)
//
// BLIS computes herk as gemmt with B = A^H and her2k as two gemmt calls,
// then sets the imaginary parts of C's diagonal to zero.  On the GPU both
// are one REAL gemmt on block-real operands whose rows interleave the real
// and imaginary parts:
//     row 2i   of Xb = [ Re x_i   -Im x_i ]
//     row 2i+1 of Xb = [ Im x_i    Re x_i ]        (x_i row i of X, m x kk)
//     Yb = [ Re Y ; Im Y ]                          (Y kk x m)
// so real rows 2i and 2i+1 of Xb Yb are the real and imaginary parts of row
// i of X Y -- exactly C's interleaved storage when C is column-stored
// (rs_c == 1).  The panels below (lower) or above (upper) each diagonal
// block are then written into C in place by the real gemm with the real
// alpha and beta, and only the w x w diagonal blocks go through a scratch
// block and a triangle merge.  herk is X = op(A), Y = op(A)^H; her2k
// concatenates along k: X = [alpha op(A) | conj(alpha) op(B)],
// Y = [op(B) | op(A)]^H (alpha folded into the packing, as BLIS folds
// alpha into a packed operand).  The real gemm is the native FP64 / FP32
// kernel or, for dcomplex in the precision form, ONE Ozaki product on C's
// real view that runs only the tiles holding part of the triangle and writes
// only the triangle.
//
// hemm / symm materialise the full A from its stored triangle (the other
// triangle reflected, conjugated for Hermitian A, whose diagonal is read as
// real: ref_kernels/1m/bli_packm_cxc_diag_1er_ref.c:214-225) and call the
// complex gemm.
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int NT = 256;
constexpr int64_t W = 1024;  // block columns of C; 2W is a multiple of the slice GEMM's row tile

unsigned grid_of(int64_t total)
{
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t g = (total + NT - 1) / NT;
    if (g > (int64_t)sms * 16) g = (int64_t)sms * 16;
    return (unsigned)(g < 1 ? 1 : g);
}

// X (m x k complex, element (i, l) at x + 2*(i*xrs + l*xcs), conjugated
// when conj, times (sr + i si) when scale) into columns c0.. of the real half
// and kk + c0.. of the imaginary half of the 2m x 2kk column-major Xb.
template <typename T>
__global__ void __launch_bounds__(NT) pack_rows_interleaved_kernel(int64_t m, int64_t k, const T* __restrict__ x,
                                                                   int64_t xrs, int64_t xcs, int conj, int scale,
                                                                   T sr, T si, int64_t kk, int64_t c0,
                                                                   T* __restrict__ out)
{
    const int64_t total = m * k, ld = 2 * m;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t l = e / m, i = e - l * m;
        const T* p = x + 2 * (i * xrs + l * xcs);
        T re = p[0], im = conj ? -p[1] : p[1];
        if (scale) {
            const T r = sr * re - si * im;
            im = sr * im + si * re;
            re = r;
        }
        T* o = out + 2 * i + (c0 + l) * ld;
        o[0] = re;
        o[1] = im;
        T* q = out + 2 * i + (kk + c0 + l) * ld;
        q[0] = -im;
        q[1] = re;
    }
}

// Y = X^H (X m x k as above) into rows c0.. (real part) and kk + c0..
// (imaginary part) of the 2kk x m column-major Yb.
template <typename T>
__global__ void __launch_bounds__(NT) pack_conj_trans_kernel(int64_t m, int64_t k, const T* __restrict__ x,
                                                             int64_t xrs, int64_t xcs, int conj, int64_t kk,
                                                             int64_t c0, T* __restrict__ out)
{
    const int64_t total = m * k, ld = 2 * kk;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / k, l = e - j * k;
        const T* p = x + 2 * (j * xrs + l * xcs);
        const T im = conj ? -p[1] : p[1];
        out[c0 + l + j * ld] = p[0];
        out[kk + c0 + l + j * ld] = -im;
    }
}

// C := P + beta C on the stored triangle of the rows x cols block of C at
// (r0, c0); P is the block's real view (rows 2i and 2i+1 the real and
// imaginary parts of row i, leading dimension ldp), or zero when p is null.
// beta == 0 writes without reading C.  The imaginary parts on C's diagonal
// are set to zero when herm (herk, her2k; not the complex syrk forms).
template <typename T>
__global__ void __launch_bounds__(NT) herk_merge_kernel(int64_t rows, int64_t cols, int64_t r0, int64_t c0,
                                                        int lower, int herm, const T* __restrict__ p, int64_t ldp,
                                                        T beta, T* __restrict__ c, int64_t rs_c, int64_t cs_c)
{
    const int64_t total = rows * cols;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / rows, i = e - j * rows;
        const int64_t gi = r0 + i, gj = c0 + j;
        if (lower ? (gi < gj) : (gi > gj)) continue;
        T* cij = c + 2 * (gi * rs_c + gj * cs_c);
        T re = p ? p[2 * i + j * ldp] : T(0), im = p ? p[2 * i + 1 + j * ldp] : T(0);
        if (beta != T(0)) {
            re += beta * cij[0];
            im += beta * cij[1];
        }
        cij[0] = re;
        cij[1] = (herm && gi == gj) ? T(0) : im;
    }
}

// the full n x n matrix (column-major, leading dimension n) of the
// Hermitian (herm) or symmetric A stored in the uplo triangle, conjugated
// when conj
template <typename T>
__global__ void __launch_bounds__(NT) hermitize_kernel(int64_t n, int lower, int herm, int conj,
                                                       const T* __restrict__ a, int64_t rs, int64_t cs,
                                                       T* __restrict__ out)
{
    const int64_t total = n * n;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / n, i = e - j * n;
        const bool stored = lower ? (i >= j) : (i <= j);
        const T* p = stored ? a + 2 * (i * rs + j * cs) : a + 2 * (j * rs + i * cs);
        T im = p[1];
        if (herm && !stored) im = -im;
        if (herm && i == j) im = T(0);
        if (conj) im = -im;
        out[2 * e] = p[0];
        out[2 * e + 1] = im;
    }
}

template <typename T>
int real_gemm_cm(int64_t m, int64_t n, int64_t k, T alpha, const T* a, int64_t lda, const T* b, int64_t ldb, T beta,
                 T* c, int64_t rs_c, int64_t cs_c, cudaStream_t s);

template <>
int real_gemm_cm<double>(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t lda, const double* b,
                         int64_t ldb, double beta, double* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    return dgemm_native(m, n, k, alpha, a, 1, lda, b, 1, ldb, beta, c, rs_c, cs_c, s);
}

template <>
int real_gemm_cm<float>(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t lda, const float* b,
                        int64_t ldb, float beta, float* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    // the engine sgemm itself would take for this shape (gb_set_sgemm_mode)
    if (sgemm_use_split(m, n, k)) return sgemm_split_dev(m, n, k, alpha, a, 1, lda, b, 1, ldb, beta, c, rs_c, cs_c, s);
    return sgemm_dev(m, n, k, alpha, a, 1, lda, b, 1, ldb, beta, c, rs_c, cs_c, s);
}

template <typename T>
int launch_merge(int64_t rows, int64_t cols, int64_t r0, int64_t c0, bool lower, const T* p, int64_t ldp, T beta,
                 T* c, int64_t rs_c, int64_t cs_c, cudaStream_t s, bool herm = true)
{
    LaunchScope ls("herk_merge", s);
    herk_merge_kernel<T><<<grid_of(rows * cols), NT, 0, s>>>(rows, cols, r0, c0, lower ? 1 : 0, herm ? 1 : 0, p, ldp,
                                                             beta, c, rs_c, cs_c);
    return check_cuda(cudaGetLastError(), "herk merge");
}

// The stored triangle of C (m x m complex) := alpha Xb Yb + beta C, the
// imaginary parts of its diagonal zeroed.  Xb is 2m x 2kk (leading
// dimension 2m) and Yb 2kk x m (leading dimension 2kk), both from the pack
// kernels above.  Column blocks of width W: the diagonal block through a
// scratch block and the merge; the panel beside it straight into C when C is
// column-stored, else through the scratch panel and the merge.
// the imaginary parts of C's diagonal set to zero
// the stored triangle of the m x m complex C times (br + i bi); beta = 0
// writes zeros without reading C
template <typename T>
__global__ void __launch_bounds__(NT) tri_scale_kernel(int64_t m, int lower, T br, T bi, T* __restrict__ c,
                                                       int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * m;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / m, i = e - j * m;
        if (lower ? (i < j) : (i > j)) continue;
        T* cij = c + 2 * (i * rs_c + j * cs_c);
        if (br == T(0) && bi == T(0)) {
            cij[0] = T(0);
            cij[1] = T(0);
        } else {
            const T re = cij[0], im = cij[1];
            cij[0] = br * re - bi * im;
            cij[1] = br * im + bi * re;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(NT) zero_diag_imag_kernel(int64_t m, T* __restrict__ c, int64_t rs_c, int64_t cs_c)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < m; i += (int64_t)gridDim.x * NT)
        c[2 * (i * rs_c + i * cs_c) + 1] = T(0);
}

template <typename T>
int herk_blocks(bool lower, int64_t m, int64_t kk, T alpha, const T* xb, const T* yb, T beta, T* c, int64_t rs_c,
                int64_t cs_c, int slices, cudaStream_t s, bool herm = true)
{
    const bool direct = (rs_c == 1);
    if constexpr (sizeof(T) == 8) {
        if (slices > 0 && direct) {
            // the precision form in one product on C's real view (rows 2i, 2i + 1
            // of complex row i: out_rpc = 2), only the tiles and elements of the
            // stored triangle, then the diagonal's imaginary parts
            OzA prep;
            int rc = ozaki_prepare_a(2 * m, 2 * kk, xb, 1, 2 * m, slices, s, &prep);
            if (rc) return rc;
            prep.out_tri = lower ? 1 : 2;
            prep.out_rpc = 2;
            rc = ozaki_multiply(&prep, m, yb, 1, 2 * kk, alpha, beta, c, 1, 2 * cs_c, s);
            ozaki_release_a(&prep, s);
            if (rc || !herm) return rc;
            LaunchScope ls("herk_zero_diag", s);
            zero_diag_imag_kernel<T><<<grid_of(m), NT, 0, s>>>(m, c, rs_c, cs_c);
            return check_cuda(cudaGetLastError(), "herk zero diagonal");
        }
    }
    const int64_t wmax = (m < W) ? m : W;
    const int64_t srows = direct ? wmax : m;  // complex rows the scratch holds
    T* scratch = static_cast<T*>(dev_alloc(sizeof(T) * (size_t)(2 * srows * wmax), s));
    if (!scratch) return GB_ERR_NOMEM;
    int rc = GB_SUCCESS;
    bool oz = false;
    OzA prep;
    if constexpr (sizeof(T) == 8) {
        oz = (slices > 0);
        if (oz) rc = ozaki_prepare_a(2 * m, 2 * kk, xb, 1, 2 * m, slices, s, &prep);
    }
    for (int64_t j0 = 0; j0 < m && !rc; j0 += W) {
        const int64_t w = (m - j0 < W) ? m - j0 : W;
        const int64_t pr0 = lower ? j0 + w : 0, prows = lower ? m - (j0 + w) : j0;
        const T* yj = yb + j0 * 2 * kk;
        OzB pb;
        if constexpr (sizeof(T) == 8) {
            if (oz && (rc = ozaki_prepare_b(&prep, w, yj, 1, 2 * kk, s, &pb))) break;
        }
        // diagonal block, beta 0, merged below
        if constexpr (sizeof(T) == 8) {
            if (oz) rc = ozaki_multiply_rows(&prep, 2 * j0, 2 * w, &pb, alpha, 0.0, scratch, 1, 2 * w, s);
        }
        if (!oz) rc = real_gemm_cm<T>(2 * w, w, 2 * kk, alpha, xb + 2 * j0, 2 * m, yj, 2 * kk, T(0), scratch, 1, 2 * w, s);
        if (!rc) rc = launch_merge<T>(w, w, j0, j0, lower, scratch, 2 * w, beta, c, rs_c, cs_c, s, herm);
        if (!rc && prows > 0) {
            // panel: in place on C's real view (rows 2i, 2i+1; column stride 2 cs_c), or scratch + merge
            T* dst = direct ? c + 2 * (pr0 + j0 * cs_c) : scratch;
            const int64_t dcs = direct ? 2 * cs_c : 2 * prows;
            const T dbeta = direct ? beta : T(0);
            if constexpr (sizeof(T) == 8) {
                if (oz) rc = ozaki_multiply_rows(&prep, 2 * pr0, 2 * prows, &pb, alpha, dbeta, dst, 1, dcs, s);
            }
            if (!oz)
                rc = real_gemm_cm<T>(2 * prows, w, 2 * kk, alpha, xb + 2 * pr0, 2 * m, yj, 2 * kk, dbeta, dst, 1, dcs,
                                     s);
            if (!rc && !direct)
                rc = launch_merge<T>(prows, w, pr0, j0, lower, scratch, 2 * prows, beta, c, rs_c, cs_c, s, herm);
        }
        if constexpr (sizeof(T) == 8) {
            if (oz) ozaki_release_b(&pb, s);
        }
    }
    if constexpr (sizeof(T) == 8) {
        if (oz) ozaki_release_a(&prep, s);
    }
    dev_free(scratch, s);
    return rc;
}

template <typename T>
int launch_pack_x(int64_t m, int64_t k, const T* x, int64_t xrs, int64_t xcs, int conj, const T* scale, int64_t kk,
                  int64_t c0, T* out, cudaStream_t s)
{
    LaunchScope ls("herk_pack", s);
    pack_rows_interleaved_kernel<T><<<grid_of(m * k), NT, 0, s>>>(m, k, x, xrs, xcs, conj, scale ? 1 : 0,
                                                                  scale ? scale[0] : T(1), scale ? scale[1] : T(0),
                                                                  kk, c0, out);
    return check_cuda(cudaGetLastError(), "herk pack");
}

template <typename T>
int launch_pack_y(int64_t m, int64_t k, const T* x, int64_t xrs, int64_t xcs, int conj, int64_t kk, int64_t c0,
                  T* out, cudaStream_t s)
{
    LaunchScope ls("herk_pack", s);
    pack_conj_trans_kernel<T><<<grid_of(m * k), NT, 0, s>>>(m, k, x, xrs, xcs, conj, kk, c0, out);
    return check_cuda(cudaGetLastError(), "herk pack");
}

}  // namespace

// herk: the stored triangle of C := alpha op(A) op(A)^H + beta C, the
// imaginary parts of C's diagonal zeroed; op(A) is m x k, transa N, T, C or
// conjugate-only (the 0x10 bit of trans_t).
template <typename T>
int cherk_dev(int uplo, int transa, int64_t m, int64_t k, T alpha, const T* a, int64_t rs_a, int64_t cs_a, T beta,
              T* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0) return GB_SUCCESS;
    const bool lower = (uplo == GB_LOWER);
    if (alpha == T(0) || k <= 0) return launch_merge<T>(m, m, 0, 0, lower, nullptr, 0, beta, c, rs_c, cs_c, s);
    const bool ta = GB_IS_TRANS(transa);
    const int ca = (transa & 0x10) ? 1 : 0;
    const int64_t ars = ta ? cs_a : rs_a, acs = ta ? rs_a : cs_a;
    const size_t nx = (size_t)(4 * m * k), ny = (size_t)(2 * k * m);
    T* ws = static_cast<T*>(dev_alloc(sizeof(T) * (nx + ny) + 256, s));
    if (!ws) return GB_ERR_NOMEM;
    T* xb = ws;
    T* yb = ws + nx;
    int rc = launch_pack_x<T>(m, k, a, ars, acs, ca, nullptr, k, 0, xb, s);
    if (!rc) rc = launch_pack_y<T>(m, k, a, ars, acs, ca, k, 0, yb, s);
    if (!rc) rc = herk_blocks<T>(lower, m, k, alpha, xb, yb, beta, c, rs_c, cs_c, slices, s);
    dev_free(ws, s);
    return rc;
}

// her2k: the stored triangle of C := alpha op(A) op(B)^H + conj(alpha)
// op(B) op(A)^H + beta C (alpha complex, beta real), the imaginary parts of
// C's diagonal zeroed; op(A), op(B) m x k, each with its own trans_t.
template <typename T>
int cher2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, T beta, T* c, int64_t rs_c, int64_t cs_c,
               int slices, cudaStream_t s)
{
    if (m <= 0) return GB_SUCCESS;
    const bool lower = (uplo == GB_LOWER);
    if ((alpha[0] == T(0) && alpha[1] == T(0)) || k <= 0)
        return launch_merge<T>(m, m, 0, 0, lower, nullptr, 0, beta, c, rs_c, cs_c, s);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    const int ca = (transa & 0x10) ? 1 : 0, cb = (transb & 0x10) ? 1 : 0;
    const int64_t ars = ta ? cs_a : rs_a, acs = ta ? rs_a : cs_a;
    const int64_t brs = tb ? cs_b : rs_b, bcs = tb ? rs_b : cs_b;
    const int64_t kk = 2 * k;
    const size_t nx = (size_t)(4 * m * kk), ny = (size_t)(2 * kk * m);
    T* ws = static_cast<T*>(dev_alloc(sizeof(T) * (nx + ny) + 256, s));
    if (!ws) return GB_ERR_NOMEM;
    T* xb = ws;
    T* yb = ws + nx;
    const T conj_alpha[2] = {alpha[0], -alpha[1]};
    // X = [alpha op(A) | conj(alpha) op(B)], Y = [op(B) | op(A)]^H
    int rc = launch_pack_x<T>(m, k, a, ars, acs, ca, alpha, kk, 0, xb, s);
    if (!rc) rc = launch_pack_x<T>(m, k, b, brs, bcs, cb, conj_alpha, kk, k, xb, s);
    if (!rc) rc = launch_pack_y<T>(m, k, b, brs, bcs, cb, kk, 0, yb, s);
    if (!rc) rc = launch_pack_y<T>(m, k, a, ars, acs, ca, kk, k, yb, s);
    if (!rc) rc = herk_blocks<T>(lower, m, kk, T(1), xb, yb, beta, c, rs_c, cs_c, slices, s);
    dev_free(ws, s);
    return rc;
}

// hemm (herm = 1) / complex symm (herm = 0): C := alpha A' op(B) + beta C
// (left, A m x m) or alpha op(B) A' + beta C (right, A n x n), A stored in
// its uplo triangle, A' = A or conj(A) (conja); op(B) and C m x n.
template <typename T>
int chemm_dev(int side, int uplo, int herm, int conja, int transb, int64_t m, int64_t n, const T* alpha, const T* a,
              int64_t rs_a, int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c,
              int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    const bool left = (side == GB_LEFT);
    const int64_t na = left ? m : n;
    if ((alpha[0] == T(0) && alpha[1] == T(0)))
        return cgemm_dev<T>(GB_NO_TRANSPOSE, GB_NO_TRANSPOSE, m, n, 0, alpha, nullptr, 1, 1, nullptr, 1, 1, beta, c,
                            rs_c, cs_c, slices, s);
    T* full = static_cast<T*>(dev_alloc(sizeof(T) * (size_t)(2 * na * na), s));
    if (!full) return GB_ERR_NOMEM;
    int rc;
    {
        LaunchScope ls("hermitize", s);
        hermitize_kernel<T><<<grid_of(na * na), NT, 0, s>>>(na, uplo == GB_LOWER ? 1 : 0, herm, conja, a, rs_a, cs_a,
                                                            full);
        rc = check_cuda(cudaGetLastError(), "hermitize");
    }
    if (!rc)
        rc = left ? cgemm_dev<T>(GB_NO_TRANSPOSE, transb, m, n, m, alpha, full, 1, na, b, rs_b, cs_b, beta, c, rs_c,
                                 cs_c, slices, s)
                  : cgemm_dev<T>(transb, GB_NO_TRANSPOSE, m, n, n, alpha, b, rs_b, cs_b, full, 1, na, beta, c, rs_c,
                                 cs_c, slices, s);
    dev_free(full, s);
    return rc;
}

// complex syrk (b null) / syr2k: the stored triangle of C := alpha op(A)
// op(A)^T + beta C, or alpha op(A) op(B)^T + alpha op(B) op(A)^T + beta C,
// alpha and beta complex, no conjugate transposes (trans_t's 0x10 bit
// conjugates its operand); the diagonal keeps its imaginary parts.  A beta
// with an imaginary part scales the triangle first, and the products then
// add to it.
template <typename T>
int csyr2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c,
               int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0) return GB_SUCCESS;
    const bool lower = (uplo == GB_LOWER);
    const bool nothing = (alpha[0] == T(0) && alpha[1] == T(0)) || k <= 0;
    T rbeta = beta[0];
    if (beta[1] != T(0) || nothing) {
        LaunchScope ls("syrk_scale", s);
        tri_scale_kernel<T><<<grid_of(m * m), NT, 0, s>>>(m, lower ? 1 : 0, beta[0], beta[1], c, rs_c, cs_c);
        int rc = check_cuda(cudaGetLastError(), "syrk scale");
        if (rc || nothing) return rc;
        rbeta = T(1);
    }
    const bool two = (b != nullptr);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    const int ca = (transa & 0x10) ? 1 : 0, cb = (transb & 0x10) ? 1 : 0;
    const int64_t ars = ta ? cs_a : rs_a, acs = ta ? rs_a : cs_a;
    const int64_t brs = tb ? cs_b : rs_b, bcs = tb ? rs_b : cs_b;
    const int64_t kk = two ? 2 * k : k;
    const size_t nx = (size_t)(4 * m * kk), ny = (size_t)(2 * kk * m);
    T* ws = static_cast<T*>(dev_alloc(sizeof(T) * (nx + ny) + 256, s));
    if (!ws) return GB_ERR_NOMEM;
    T* xb = ws;
    T* yb = ws + nx;
    // X = alpha [op(A) | op(B)], Y = [op(B) | op(A)]^T: the packing of Y is a
    // conjugate transpose, so it takes the operand's conjugation flipped
    int rc = launch_pack_x<T>(m, k, a, ars, acs, ca, alpha, kk, 0, xb, s);
    if (!rc && two) rc = launch_pack_x<T>(m, k, b, brs, bcs, cb, alpha, kk, k, xb, s);
    if (!rc && two) rc = launch_pack_y<T>(m, k, b, brs, bcs, 1 - cb, kk, 0, yb, s);
    if (!rc) rc = launch_pack_y<T>(m, k, a, ars, acs, 1 - ca, kk, two ? k : 0, yb, s);
    if (!rc) rc = herk_blocks<T>(lower, m, kk, T(1), xb, yb, rbeta, c, rs_c, cs_c, slices, s, false);
    dev_free(ws, s);
    return rc;
}

template int csyr2k_dev<double>(int, int, int, int64_t, int64_t, const double*, const double*, int64_t, int64_t,
                                const double*, int64_t, int64_t, const double*, double*, int64_t, int64_t, int,
                                cudaStream_t);
template int csyr2k_dev<float>(int, int, int, int64_t, int64_t, const float*, const float*, int64_t, int64_t,
                               const float*, int64_t, int64_t, const float*, float*, int64_t, int64_t, int,
                               cudaStream_t);
template int cherk_dev<double>(int, int, int64_t, int64_t, double, const double*, int64_t, int64_t, double, double*,
                               int64_t, int64_t, int, cudaStream_t);
template int cherk_dev<float>(int, int, int64_t, int64_t, float, const float*, int64_t, int64_t, float, float*,
                              int64_t, int64_t, int, cudaStream_t);
template int cher2k_dev<double>(int, int, int, int64_t, int64_t, const double*, const double*, int64_t, int64_t,
                                const double*, int64_t, int64_t, double, double*, int64_t, int64_t, int,
                                cudaStream_t);
template int cher2k_dev<float>(int, int, int, int64_t, int64_t, const float*, const float*, int64_t, int64_t,
                               const float*, int64_t, int64_t, float, float*, int64_t, int64_t, int, cudaStream_t);
template int chemm_dev<double>(int, int, int, int, int, int64_t, int64_t, const double*, const double*, int64_t,
                               int64_t, const double*, int64_t, int64_t, const double*, double*, int64_t, int64_t,
                               int, cudaStream_t);
template int chemm_dev<float>(int, int, int, int, int, int64_t, int64_t, const float*, const float*, int64_t,
                              int64_t, const float*, int64_t, int64_t, const float*, float*, int64_t, int64_t, int,
                              cudaStream_t);

}  // namespace gb
