// gb_complex.cu -- complex gemm (zgemm / cgemm) on the real gemm kernels for
// sm_103a.  BLIS computes complex level-3 products through real kernels by
// induced methods (frame/3/bli_l3_ind.c; the 1m method, which repacks the
// operands so a real micro-kernel does the complex product,
// ref_kernels/ind/bli_gemm1m_ref.c).  The GPU form of the same idea is one
// real gemm on block-real operands:
//     [Cr]   [Ar  -Ai] [Br]
//     [Ci] = [Ai   Ar] [Bi]      (2m x 2k) (2k x n)
// so a complex product of m x n x k is a real product of 2m x n x 2k (the
// 8mnk real flops of the definition) on the native FP64 / FP32 kernels or,
// for dcomplex in the precision form, on the Ozaki kernel.  The pack kernels
// read the interleaved operands once (transpose and conjugation folded in)
// and the combine kernel applies the complex alpha and beta (beta == 0 does
// not read C).  Complex storage is interleaved (real, imaginary), strides in
// complex elements, as BLIS's scomplex / dcomplex
// (frame/include/bli_type_defs.h:191-206).
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int NT = 256;

unsigned grid_of(int64_t total)
{
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t g = (total + NT - 1) / NT;
    if (g > (int64_t)sms * 16) g = (int64_t)sms * 16;
    return (unsigned)(g < 1 ? 1 : g);
}

// op(A) (element (i, l) of the complex matrix at a + 2*(i*ars + l*acs),
// conjugated when conj) into the 2m x 2k column-major block-real matrix.
template <typename T>
__global__ void __launch_bounds__(NT) pack_a_block_kernel(int64_t m, int64_t k, const T* __restrict__ a, int64_t ars,
                                                          int64_t acs, int conj, T* __restrict__ out)
{
    const int64_t total = m * k, ld = 2 * m;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t l = e / m, i = e - l * m;
        const T* p = a + 2 * (i * ars + l * acs);
        const T re = p[0], im = conj ? -p[1] : p[1];
        out[i + l * ld] = re;
        out[m + i + l * ld] = im;
        out[i + (k + l) * ld] = -im;
        out[m + i + (k + l) * ld] = re;
    }
}

// op(B) into the 2k x n column-major [Br; Bi].
template <typename T>
__global__ void __launch_bounds__(NT) pack_b_block_kernel(int64_t k, int64_t n, const T* __restrict__ b, int64_t brs,
                                                          int64_t bcs, int conj, T* __restrict__ out)
{
    const int64_t total = k * n, ld = 2 * k;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / k, l = e - j * k;
        const T* p = b + 2 * (l * brs + j * bcs);
        out[l + j * ld] = p[0];
        out[k + l + j * ld] = conj ? -p[1] : p[1];
    }
}

// C := alpha P + beta C, P = [Pr; Pi] (2m x n column-major); beta == 0
// writes without reading C.
template <typename T>
__global__ void __launch_bounds__(NT) combine_kernel(int64_t m, int64_t n, const T* __restrict__ p, T ar, T ai, T br,
                                                     T bi, T* __restrict__ c, int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * n, ld = 2 * m;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / m, i = e - j * m;
        const T pr = p[i + j * ld], pi = p[m + i + j * ld];
        T xr = ar * pr - ai * pi, xi = ar * pi + ai * pr;
        T* cij = c + 2 * (i * rs_c + j * cs_c);
        if (br != T(0) || bi != T(0)) {
            const T cr = cij[0], ci = cij[1];
            xr += br * cr - bi * ci;
            xi += br * ci + bi * cr;
        }
        cij[0] = xr;
        cij[1] = xi;
    }
}

template <typename T>
int real_gemm(int64_t m, int64_t n, int64_t k, const T* a, const T* b, T* c, int slices, cudaStream_t s);

template <>
int real_gemm<double>(int64_t m, int64_t n, int64_t k, const double* a, const double* b, double* c, int slices,
                      cudaStream_t s)
{
    if (slices > 0) return dgemm_ozaki_blocks(m, n, k, 1.0, a, 1, m, b, 1, k, 0.0, c, 1, m, slices, s);
    return dgemm_native(m, n, k, 1.0, a, 1, m, b, 1, k, 0.0, c, 1, m, s);
}

template <>
int real_gemm<float>(int64_t m, int64_t n, int64_t k, const float* a, const float* b, float* c, int, cudaStream_t s)
{
    // the engine sgemm itself would take for this shape (gb_set_sgemm_mode)
    if (sgemm_use_split(m, n, k)) return sgemm_split_dev(m, n, k, 1.0f, a, 1, m, b, 1, k, 0.0f, c, 1, m, s);
    return sgemm_dev(m, n, k, 1.0f, a, 1, m, b, 1, k, 0.0f, c, 1, m, s);
}

template <typename T>
int scal_complex(int64_t m, int64_t n, T br, T bi, T* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    // C := beta C through the combine kernel on a zero product
    T* zero = static_cast<T*>(dev_alloc(sizeof(T) * (size_t)(2 * m * n), s));
    if (!zero) return GB_ERR_NOMEM;
    int rc = check_cuda(cudaMemsetAsync(zero, 0, sizeof(T) * (size_t)(2 * m * n), s), "memset");
    if (!rc) {
        LaunchScope ls("complex_combine", s);
        combine_kernel<T><<<grid_of(m * n), NT, 0, s>>>(m, n, zero, T(0), T(0), br, bi, c, rs_c, cs_c);
        rc = check_cuda(cudaGetLastError(), "complex combine");
    }
    dev_free(zero, s);
    return rc;
}

}  // namespace

template <typename T>
int cgemm_dev(int transa, int transb, int64_t m, int64_t n, int64_t k, const T* alpha, const T* a, int64_t rs_a,
              int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c, int64_t cs_c,
              int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if ((alpha[0] == T(0) && alpha[1] == T(0)) || k <= 0) return scal_complex(m, n, beta[0], beta[1], c, rs_c, cs_c, s);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    const int ca = (transa & 0x10) ? 1 : 0, cb = (transb & 0x10) ? 1 : 0;  // conjugation bits of trans_t
    const int64_t ars = ta ? cs_a : rs_a, acs = ta ? rs_a : cs_a;
    const int64_t brs = tb ? cs_b : rs_b, bcs = tb ? rs_b : cs_b;
    const size_t na = (size_t)(4 * m * k), nb = (size_t)(2 * k * n), np = (size_t)(2 * m * n);
    T* ws = static_cast<T*>(dev_alloc(sizeof(T) * (na + nb + np) + 256, s));
    if (!ws) return GB_ERR_NOMEM;
    T* ablk = ws;
    T* bblk = ws + na;
    T* p = bblk + nb;
    {
        LaunchScope ls("complex_pack", s);
        pack_a_block_kernel<T><<<grid_of(m * k), NT, 0, s>>>(m, k, a, ars, acs, ca, ablk);
        pack_b_block_kernel<T><<<grid_of(k * n), NT, 0, s>>>(k, n, b, brs, bcs, cb, bblk);
    }
    int rc = check_cuda(cudaGetLastError(), "complex pack");
    if (!rc) rc = real_gemm<T>(2 * m, n, 2 * k, ablk, bblk, p, slices, s);
    if (!rc) {
        LaunchScope ls("complex_combine", s);
        combine_kernel<T><<<grid_of(m * n), NT, 0, s>>>(m, n, p, alpha[0], alpha[1], beta[0], beta[1], c, rs_c, cs_c);
        rc = check_cuda(cudaGetLastError(), "complex combine");
    }
    dev_free(ws, s);
    return rc;
}

template int cgemm_dev<double>(int, int, int64_t, int64_t, int64_t, const double*, const double*, int64_t, int64_t,
                               const double*, int64_t, int64_t, const double*, double*, int64_t, int64_t, int,
                               cudaStream_t);
template int cgemm_dev<float>(int, int, int64_t, int64_t, int64_t, const float*, const float*, int64_t, int64_t,
                              const float*, int64_t, int64_t, const float*, float*, int64_t, int64_t, int,
                              cudaStream_t);

// ---------------------------------------------------------------- ztrsm
// The recursive solve of gb_trsm.cu on dcomplex data: 64-row diagonal blocks
// and complex gemm updates (block-real, native or Ozaki).  A diagonal block
// is packed once per call as in the real solver, P[r][r] = inv(a_rr) and
// P[r][i] = a_ri inv(a_ii) in the strict triangle (conjugated first for
// A^H), so the substitution works on y = D x with a unit triangle and every
// complex FMA of the triangle is four real FMAs on the FP64 pipe.
namespace {

constexpr int ZNB = 64;
constexpr int ZTHREADS = 128;

// The complex element of a real type R: double2 for ztrsm, float2 for ctrsm.
template <typename R> struct Cx;
template <> struct Cx<double> {
    using T = double2;
    __device__ __forceinline__ static T make(double x, double y) { return make_double2(x, y); }
};
template <> struct Cx<float> {
    using T = float2;
    __device__ __forceinline__ static T make(float x, float y) { return make_float2(x, y); }
};

template <typename C2>
__device__ __forceinline__ C2 cmul(C2 a, C2 b)
{
    C2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

template <typename R>
__device__ __forceinline__ typename Cx<R>::T cinv(typename Cx<R>::T a)
{
    // 1 / a with the larger component scaled out (Smith's method)
    if (fabs(a.x) >= fabs(a.y)) {
        const R r = a.y / a.x, d = a.x + a.y * r;
        return Cx<R>::make(R(1) / d, -r / d);
    }
    const R r = a.x / a.y, d = a.x * r + a.y;
    return Cx<R>::make(r / d, R(-1) / d);
}

template <typename R, bool LOWER>
__global__ void __launch_bounds__(256) ztrsm_pack_diag_kernel(int64_t m, int unit, int conj,
                                                              const typename Cx<R>::T* __restrict__ a, int64_t ars,
                                                              int64_t acs, typename Cx<R>::T* __restrict__ packed)
{
    using C2 = typename Cx<R>::T;
    __shared__ C2 Tb[ZNB][ZNB + 1];
    __shared__ C2 dinv[ZNB];
    const int64_t r0 = (int64_t)blockIdx.x * ZNB;
    const int nb = (m - r0 < ZNB) ? (int)(m - r0) : ZNB;
    const C2* blk = a + r0 * ars + r0 * acs;
    for (int e = threadIdx.x; e < ZNB * ZNB; e += 256) {
        const int i = e % ZNB, l = e / ZNB;
        const bool keep = (i < nb && l < nb) && (LOWER ? (l <= i) : (l >= i));
        C2 v = keep ? blk[i * ars + l * acs] : Cx<R>::make(R(0), R(0));
        if (conj) v.y = -v.y;
        Tb[i][l] = v;
    }
    __syncthreads();
    if (threadIdx.x < ZNB) {
        const int i = threadIdx.x;
        dinv[i] = (unit || i >= nb) ? Cx<R>::make(R(1), R(0)) : cinv<R>(Tb[i][i]);
    }
    __syncthreads();
    C2* out = packed + (int64_t)blockIdx.x * ZNB * ZNB;
    for (int e = threadIdx.x; e < ZNB * ZNB; e += 256) {
        const int r = e / ZNB, i = e % ZNB;
        C2 v = Cx<R>::make(R(0), R(0));
        if (r == i) v = dinv[r];
        else if (LOWER ? (i < r) : (i > r)) v = cmul(Tb[r][i], dinv[i]);
        out[e] = v;
    }
}

template <typename R, int LANES, bool LOWER>
__global__ void __launch_bounds__(ZTHREADS) ztrsm_diag_kernel(int nb, const typename Cx<R>::T* __restrict__ pk,
                                                              typename Cx<R>::T* __restrict__ b, int64_t brs,
                                                              int64_t bcs, int64_t ncols)
{
    using C2 = typename Cx<R>::T;
    constexpr int COLS = ZTHREADS / LANES, RR = ZNB / LANES, LL = ZNB + 1, LX = COLS + 1;
    extern __shared__ __align__(16) unsigned char ztrsm_smem[];
    C2* L = reinterpret_cast<C2*>(ztrsm_smem);  // [ZNB][LL]
    C2* X = L + ZNB * LL;                       // [ZNB][LX]
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * COLS;
    const int cols = (ncols - j0 < COLS) ? (int)(ncols - j0) : COLS;
    for (int e = t; e < ZNB * ZNB; e += ZTHREADS) L[(e / ZNB) * LL + e % ZNB] = pk[e];
    const bool rows_fast = (brs == 1);
    for (int e = t; e < ZNB * COLS; e += ZTHREADS) {
        const int i = rows_fast ? e % ZNB : e / COLS, c = rows_fast ? e / ZNB : e % COLS;
        X[i * LX + c] = (c < cols && i < nb) ? b[i * brs + (j0 + c) * bcs] : Cx<R>::make(R(0), R(0));
    }
    __syncthreads();
    const int c = t / LANES, g = t % LANES;
    const int src0 = (t % 32) - g;
    C2 x[RR];
#pragma unroll
    for (int q = 0; q < RR; ++q) x[q] = X[(q * LANES + g) * LX + c];
#pragma unroll
    for (int step = 0; step < ZNB; ++step) {
        const int i = LOWER ? step : ZNB - 1 - step;
        const int qi = i / LANES, gi = i % LANES;
        C2 v = x[qi];
        if constexpr (LANES > 1) {
            v.x = __shfl_sync(0xffffffffu, v.x, src0 + gi);
            v.y = __shfl_sync(0xffffffffu, v.y, src0 + gi);
        }
#pragma unroll
        for (int q = 0; q < RR; ++q) {
            if (LOWER ? (q * LANES + LANES - 1 > i) : (q * LANES < i)) {
                const int r = q * LANES + g;
                if (LOWER ? (r > i) : (r < i)) {
                    const C2 p = L[r * LL + i];
                    x[q].x = fma(-p.x, v.x, fma(p.y, v.y, x[q].x));
                    x[q].y = fma(-p.x, v.y, fma(-p.y, v.x, x[q].y));
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < RR; ++q) {
        const int r = q * LANES + g;
        X[r * LX + c] = cmul(x[q], L[r * LL + r]);
    }
    __syncthreads();
    for (int e = t; e < ZNB * COLS; e += ZTHREADS) {
        const int i = rows_fast ? e % ZNB : e / COLS, cc = rows_fast ? e / ZNB : e % COLS;
        if (cc < cols && i < nb) b[i * brs + (j0 + cc) * bcs] = X[i * LX + cc];
    }
}

template <typename R>
constexpr size_t ztrsm_smem_bytes(int lanes)
{
    return 2 * sizeof(R) * (ZNB * (ZNB + 1) + ZNB * (ZTHREADS / lanes + 1));
}

template <typename R, int LANES, bool LOWER>
int launch_ztrsm_diag(int nb, const typename Cx<R>::T* pk, typename Cx<R>::T* b, int64_t brs, int64_t bcs,
                      int64_t ncols, cudaStream_t s)
{
    static bool attr = false;
    if (!attr) {
        const int rc = check_cuda(cudaFuncSetAttribute(ztrsm_diag_kernel<R, LANES, LOWER>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)ztrsm_smem_bytes<R>(LANES)), "ztrsm smem attr");
        if (rc) return rc;
        attr = true;
    }
    const int64_t blocks = (ncols + ZTHREADS / LANES - 1) / (ZTHREADS / LANES);
    if (blocks > INT32_MAX) return set_error(GB_ERR_ARG, "complex trsm", "too many right-hand sides");
    ztrsm_diag_kernel<R, LANES, LOWER><<<(unsigned)blocks, ZTHREADS, ztrsm_smem_bytes<R>(LANES), s>>>(
        nb, pk, b, brs, bcs, ncols);
    return check_cuda(cudaGetLastError(), "ztrsm_diag");
}

template <typename R>
__global__ void __launch_bounds__(NT) zscal_kernel(int64_t m, int64_t n, R ar, R ai, typename Cx<R>::T* __restrict__ b,
                                                   int64_t brs, int64_t bcs)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / m, i = e - j * m;
        typename Cx<R>::T* p = b + i * brs + j * bcs;
        *p = (ar == R(0) && ai == R(0)) ? Cx<R>::make(R(0), R(0)) : cmul(Cx<R>::make(ar, ai), *p);
    }
}

template <typename R>
struct ZtrsmCtx {
    int lower, conj, slices;
    const typename Cx<R>::T* packed;
    const typename Cx<R>::T* a;
    int64_t ars, acs;
    typename Cx<R>::T* b;
    int64_t brs, bcs, n;
    cudaStream_t s;
};

template <typename R>
int ztrsm_update(const ZtrsmCtx<R>& t, int64_t r0, int64_t rcount, int64_t c0, int64_t ccount)
{
    // B[r0..] -= op(A)[r0.., c0..] X[c0..]; op(A) by the folded strides, conjugated when t.conj
    const R minus_one[2] = {R(-1), R(0)}, one[2] = {R(1), R(0)};
    return cgemm_dev<R>(t.conj ? 0x10 : 0x00, 0x00, rcount, t.n, ccount, minus_one,
                        reinterpret_cast<const R*>(t.a + r0 * t.ars + c0 * t.acs), t.ars, t.acs,
                        reinterpret_cast<const R*>(t.b + c0 * t.brs), t.brs, t.bcs, one,
                        reinterpret_cast<R*>(t.b + r0 * t.brs), t.brs, t.bcs, t.slices, t.s);
}

template <typename R>
int ztrsm_solve(const ZtrsmCtx<R>& t, int64_t r0, int64_t mm)
{
    if (mm <= ZNB) {
        const typename Cx<R>::T* pk = t.packed + (r0 / ZNB) * ZNB * ZNB;
        typename Cx<R>::T* b1 = t.b + r0 * t.brs;
        const int nb = (int)mm;
        int lanes = diag_block_lanes(t.n);
        if (lanes < 2) lanes = 2;  // 64 complex rows per lane would not fit the registers
        LaunchScope ls("ztrsm_diag", t.s);
        switch (lanes) {
        case 2:
            return t.lower ? launch_ztrsm_diag<R, 2, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_ztrsm_diag<R, 2, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        case 4:
            return t.lower ? launch_ztrsm_diag<R, 4, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_ztrsm_diag<R, 4, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        default:
            return t.lower ? launch_ztrsm_diag<R, 8, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                           : launch_ztrsm_diag<R, 8, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
        }
    }
    int64_t m1 = ((mm / 2 + ZNB - 1) / ZNB) * ZNB;
    if (m1 >= mm) m1 = mm - ZNB;
    const int64_t m2 = mm - m1;
    int rc;
    if (t.lower) {
        if ((rc = ztrsm_solve(t, r0, m1))) return rc;
        if ((rc = ztrsm_update(t, r0 + m1, m2, r0, m1))) return rc;
        return ztrsm_solve(t, r0 + m1, m2);
    }
    if ((rc = ztrsm_solve(t, r0 + m1, m2))) return rc;
    if ((rc = ztrsm_update(t, r0, m1, r0 + m1, m2))) return rc;
    return ztrsm_solve(t, r0, m1);
}

// op(A) X = alpha B (left) or X op(A) = alpha B (right) in place for complex R
// (dcomplex: R = double, scomplex: R = float); transa may be N, T or C
// (conjugate transpose: the 0x10 bit).
template <typename R>
int xtrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const R* alpha, const R* a,
              int64_t rs_a, int64_t cs_a, R* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s)
{
    using C2 = typename Cx<R>::T;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    const int conj = (transa & 0x10) ? 1 : 0;
    if (side == GB_RIGHT) {
        // X op(A) = alpha B  <=>  op(A)^T X^T = alpha B^T; the conjugation stays
        brs = cs_b;
        bcs = rs_b;
        mm = n;
        nn = m;
        trans = !trans;
    }
    C2* bz = reinterpret_cast<C2*>(b);
    if (!(alpha[0] == R(1) && alpha[1] == R(0))) {
        LaunchScope ls("zscal", s);
        zscal_kernel<R><<<grid_of(mm * nn), NT, 0, s>>>(mm, nn, alpha[0], alpha[1], bz, brs, bcs);
        int rc = check_cuda(cudaGetLastError(), "zscal");
        if (rc || (alpha[0] == R(0) && alpha[1] == R(0))) return rc;
    }
    ZtrsmCtx<R> t;
    t.ars = trans ? cs_a : rs_a;
    t.acs = trans ? rs_a : cs_a;
    t.lower = ((uplo == GB_LOWER) != trans) ? 1 : 0;
    t.conj = conj;
    t.slices = slices;
    t.a = reinterpret_cast<const C2*>(a);
    t.b = bz;
    t.brs = brs;
    t.bcs = bcs;
    t.n = nn;
    t.s = s;
    const int64_t nblk = (mm + ZNB - 1) / ZNB;
    if (nblk > INT32_MAX) return set_error(GB_ERR_ARG, "complex trsm", "too many diagonal blocks");
    C2* packed = static_cast<C2*>(dev_alloc(sizeof(C2) * nblk * ZNB * ZNB, s));
    if (!packed) return GB_ERR_NOMEM;
    {
        LaunchScope ls("ztrsm_pack_diag", s);
        if (t.lower)
            ztrsm_pack_diag_kernel<R, true><<<(unsigned)nblk, 256, 0, s>>>(mm, diag == GB_UNIT_DIAG, conj, t.a, t.ars,
                                                                           t.acs, packed);
        else
            ztrsm_pack_diag_kernel<R, false><<<(unsigned)nblk, 256, 0, s>>>(mm, diag == GB_UNIT_DIAG, conj, t.a,
                                                                            t.ars, t.acs, packed);
    }
    int rc = check_cuda(cudaGetLastError(), "ztrsm_pack_diag");
    t.packed = packed;
    if (!rc) rc = ztrsm_solve(t, 0, mm);
    dev_free(packed, s);
    return rc;
}

}  // namespace

int ztrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const double* alpha, const double* a,
              int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s)
{
    return xtrsm_dev<double>(side, uplo, transa, diag, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, slices, s);
}

// scomplex: the FP32 solve with the updates through cgemm's FP32 real product (sgemm's engine choice)
int ctrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const float* alpha, const float* a,
              int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, cudaStream_t s)
{
    return xtrsm_dev<float>(side, uplo, transa, diag, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, 0, s);
}

namespace {

// the na x na uplo triangle of A (strides in complex elements; the unit
// diagonal when unit) as a full column-major complex matrix, zeros outside it
template <typename R>
__global__ void __launch_bounds__(NT) ctri_full_kernel(int64_t na, int lower, int unit, const R* __restrict__ a,
                                                      int64_t rs, int64_t cs, R* __restrict__ out)
{
    const int64_t total = na * na;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / na, i = e - j * na;
        R re = R(0), im = R(0);
        if (i == j && unit) {
            re = R(1);
        } else if (lower ? (i >= j) : (i <= j)) {
            const R* p = a + 2 * (i * rs + j * cs);
            re = p[0];
            im = p[1];
        }
        out[2 * e] = re;
        out[2 * e + 1] = im;
    }
}

// the packed column-major m x n complex matrix into B (strides rs, cs)
template <typename R>
__global__ void __launch_bounds__(NT) cscatter_kernel(int64_t m, int64_t n, const R* __restrict__ in,
                                                     R* __restrict__ b, int64_t rs, int64_t cs)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * NT + threadIdx.x; e < total; e += (int64_t)gridDim.x * NT) {
        const int64_t j = e / m, i = e - j * m;
        R* p = b + 2 * (i * rs + j * cs);
        p[0] = in[2 * e];
        p[1] = in[2 * e + 1];
    }
}

}  // namespace

// complex trmm: B := alpha op(A) B (left, A m x m) or alpha B op(A) (right,
// A n x n), A triangular in its uplo triangle, op N, T, C or conjugate-only.
// The triangle goes into a full matrix, one complex gemm (the block-real
// product, Ozaki for double complex when slices > 0) writes a scratch, and
// the scratch is scattered back into B.
template <typename R>
int ctrmm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const R* alpha, const R* a,
              int64_t rs_a, int64_t cs_a, R* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha[0] == R(0) && alpha[1] == R(0)) {
        LaunchScope ls("ztrmm_zero", s);
        zscal_kernel<R><<<grid_of(m * n), NT, 0, s>>>(m, n, R(0), R(0), reinterpret_cast<typename Cx<R>::T*>(b),
                                                      rs_b, cs_b);
        return check_cuda(cudaGetLastError(), "ztrmm zero");
    }
    const bool left = (side == GB_LEFT);
    const int64_t na = left ? m : n;
    R* full = static_cast<R*>(dev_alloc(sizeof(R) * (size_t)(2 * na * na + 2 * m * n), s));
    if (!full) return GB_ERR_NOMEM;
    R* tmp = full + 2 * na * na;
    int rc;
    {
        LaunchScope ls("ztrmm_tri_full", s);
        ctri_full_kernel<R><<<grid_of(na * na), NT, 0, s>>>(na, uplo == GB_LOWER ? 1 : 0, diag == GB_UNIT_DIAG ? 1 : 0,
                                                             a, rs_a, cs_a, full);
        rc = check_cuda(cudaGetLastError(), "ztrmm tri full");
    }
    const R zero[2] = {R(0), R(0)};
    if (!rc)
        rc = left ? cgemm_dev<R>(transa, GB_NO_TRANSPOSE, m, n, m, alpha, full, 1, na, b, rs_b, cs_b, zero, tmp, 1, m,
                                 slices, s)
                  : cgemm_dev<R>(GB_NO_TRANSPOSE, transa, m, n, n, alpha, b, rs_b, cs_b, full, 1, na, zero, tmp, 1, m,
                                 slices, s);
    if (!rc) {
        LaunchScope ls("ztrmm_scatter", s);
        cscatter_kernel<R><<<grid_of(m * n), NT, 0, s>>>(m, n, tmp, b, rs_b, cs_b);
        rc = check_cuda(cudaGetLastError(), "ztrmm scatter");
    }
    dev_free(full, s);
    return rc;
}

namespace {

constexpr int GV_WARP_ROWS = NT / 32;  // output rows of a warp-per-row block

// Partial sums of y' = op(A) x' over the column split blockIdx.y (columns
// l0 .. l0 + chunk of op(A)): part[2 (s ly + i) + {0, 1}].  op(A)(i, l) =
// A[i ers + l ecs] (conjugated when ca), x'(l) = x[l incx] (conjugated when
// cx).  ROWS: one thread per output row, for op(A)'s rows contiguous in
// memory (ers == 1: a warp reads 32 consecutive elements of one column);
// otherwise one warp per output row with the lanes striding over l.
template <typename R, bool ROWS>
__global__ void __launch_bounds__(NT) cgemv_partial_kernel(int64_t ly, int64_t lx, int64_t chunk,
                                                          const R* __restrict__ a, int64_t ers, int64_t ecs, int ca,
                                                          const R* __restrict__ x, int64_t incx, int cx,
                                                          R* __restrict__ part)
{
    const int lane = threadIdx.x & 31;
    const int64_t i = ROWS ? (int64_t)blockIdx.x * NT + threadIdx.x
                           : (int64_t)blockIdx.x * GV_WARP_ROWS + (threadIdx.x >> 5);
    if (i >= ly) return;
    const int64_t l0 = (int64_t)blockIdx.y * chunk;
    const int64_t l1 = (l0 + chunk < lx) ? l0 + chunk : lx;
    const R sa = ca ? R(-1) : R(1), sx = cx ? R(-1) : R(1);
    R sr = R(0), si = R(0);
    for (int64_t l = l0 + (ROWS ? 0 : lane); l < l1; l += (ROWS ? 1 : 32)) {
        const R* p = a + 2 * (i * ers + l * ecs);
        const R* q = x + 2 * (l * incx);
        const R ar = p[0], ai = sa * p[1], xr = q[0], xi = sx * q[1];
        // four fused multiply-adds per element (FP64 gemv is bound by the FP64 pipe)
        sr = fma(ar, xr, sr);
        sr = fma(-ai, xi, sr);
        si = fma(ar, xi, si);
        si = fma(ai, xr, si);
    }
    if (!ROWS) {
        for (int off = 16; off > 0; off >>= 1) {
            sr += __shfl_down_sync(0xffffffffu, sr, off);
            si += __shfl_down_sync(0xffffffffu, si, off);
        }
        if (lane != 0) return;
    }
    R* o = part + 2 * ((int64_t)blockIdx.y * ly + i);
    o[0] = sr;
    o[1] = si;
}

// y(i) := alpha sum_s part(s, i) + beta y(i); beta = 0 does not read y, and
// splits = 0 (nothing to add) leaves beta y
template <typename R>
__global__ void __launch_bounds__(NT) cgemv_combine_kernel(int64_t ly, int splits, const R* __restrict__ part,
                                                          R alr, R ali, R ber, R bei, R* __restrict__ y, int64_t incy)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < ly; i += (int64_t)gridDim.x * NT) {
        R sr = R(0), si = R(0);
        for (int sp = 0; sp < splits; ++sp) {
            sr += part[2 * (sp * ly + i)];
            si += part[2 * (sp * ly + i) + 1];
        }
        R* py = y + 2 * (i * incy);
        R yr = alr * sr - ali * si, yi = alr * si + ali * sr;
        if (!(ber == R(0) && bei == R(0))) {
            const R cr = py[0], ci = py[1];
            yr += ber * cr - bei * ci;
            yi += ber * ci + bei * cr;
        }
        py[0] = yr;
        py[1] = yi;
    }
}

}  // namespace

// complex gemv: y := alpha op(A) x' + beta y, op N, T, C or conjugate-only
// (trans_t's bits 0x08, 0x10), x' = conj(x) when conjx; A m x n, strides in
// complex elements.  Bandwidth-bound: op(A)'s columns split so that the grid
// holds about four blocks per SM, partial sums in a scratch, one combine.
template <typename R>
int cgemv_dev(int transa, int conjx, int64_t m, int64_t n, const R* alpha, const R* a, int64_t rs_a, int64_t cs_a,
              const R* x, int64_t incx, const R* beta, R* y, int64_t incy, cudaStream_t s)
{
    const bool tr = GB_IS_TRANS(transa);
    const int64_t ly = tr ? n : m, lx = tr ? m : n;
    if (ly <= 0) return GB_SUCCESS;
    const bool nothing = lx <= 0 || (alpha[0] == R(0) && alpha[1] == R(0));
    const int64_t ers = tr ? cs_a : rs_a, ecs = tr ? rs_a : cs_a;
    const bool rows = (ers == 1);
    int splits = 0;
    R* part = nullptr;
    int rc = GB_SUCCESS;
    if (!nothing) {
        const int sms = sm_count() > 0 ? sm_count() : 148;
        const int64_t rb = rows ? (ly + NT - 1) / NT : (ly + GV_WARP_ROWS - 1) / GV_WARP_ROWS;
        int64_t sp = (4 * (int64_t)sms + rb - 1) / rb;
        const int64_t maxsp = (lx + 63) / 64;
        if (sp > maxsp) sp = maxsp;
        if (sp > 1024) sp = 1024;
        if (sp < 1) sp = 1;
        const int64_t chunk = (lx + sp - 1) / sp;
        splits = (int)((lx + chunk - 1) / chunk);
        part = static_cast<R*>(dev_alloc(sizeof(R) * (size_t)(2 * splits * ly), s));
        if (!part) return GB_ERR_NOMEM;
        LaunchScope ls("cgemv_partial", s);
        const dim3 grid((unsigned)rb, (unsigned)splits);
        const int ca = (transa & 0x10) ? 1 : 0;
        if (rows)
            cgemv_partial_kernel<R, true><<<grid, NT, 0, s>>>(ly, lx, chunk, a, ers, ecs, ca, x, incx, conjx, part);
        else
            cgemv_partial_kernel<R, false><<<grid, NT, 0, s>>>(ly, lx, chunk, a, ers, ecs, ca, x, incx, conjx, part);
        rc = check_cuda(cudaGetLastError(), "cgemv partial");
    }
    if (!rc) {
        LaunchScope ls("cgemv_combine", s);
        cgemv_combine_kernel<R><<<grid_of(ly), NT, 0, s>>>(ly, splits, part, alpha[0], alpha[1], beta[0], beta[1], y,
                                                          incy);
        rc = check_cuda(cudaGetLastError(), "cgemv combine");
    }
    if (part) dev_free(part, s);
    return rc;
}

template int cgemv_dev<double>(int, int, int64_t, int64_t, const double*, const double*, int64_t, int64_t,
                               const double*, int64_t, const double*, double*, int64_t, cudaStream_t);
template int cgemv_dev<float>(int, int, int64_t, int64_t, const float*, const float*, int64_t, int64_t, const float*,
                              int64_t, const float*, float*, int64_t, cudaStream_t);

template int ctrmm_dev<double>(int, int, int, int, int64_t, int64_t, const double*, const double*, int64_t, int64_t,
                               double*, int64_t, int64_t, int, cudaStream_t);
template int ctrmm_dev<float>(int, int, int, int, int64_t, int64_t, const float*, const float*, int64_t, int64_t,
                              float*, int64_t, int64_t, int, cudaStream_t);

}  // namespace gb
