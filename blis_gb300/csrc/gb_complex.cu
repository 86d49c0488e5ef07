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
    if (slices > 0) return dgemm_ozaki(m, n, k, 1.0, a, 1, m, b, 1, k, 0.0, c, 1, m, slices, s);
    return dgemm_native(m, n, k, 1.0, a, 1, m, b, 1, k, 0.0, c, 1, m, s);
}

template <>
int real_gemm<float>(int64_t m, int64_t n, int64_t k, const float* a, const float* b, float* c, int, cudaStream_t s)
{
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

}  // namespace gb
