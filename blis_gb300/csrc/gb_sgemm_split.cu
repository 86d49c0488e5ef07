// gb_sgemm_split.cu -- SGEMM on the bf16 tensor cores (the split form of sgemm).
//
// FP32 FMA SGEMM on GB300 runs on the FP32 pipe (about 80 TFLOP/s nominal at the
// boost clock); the bf16 tensor cores are twenty times wider.  This form runs
// C := alpha op(A) op(B) + beta C for FP32 operands as the digit form of the
// Ozaki product with 3 slices (6 bf16 products, exact integer accumulation):
// op(A) and op(B) are widened to FP64 (exact), multiplied by the FP64 Ozaki
// path with every row's digits holding 24 bits below 2^e (e = ilogb(row max)
// + 2), and C = RN32(alpha P + beta C) with P the FP64 product.  Its error is
// the representation error of 24-bit digits (no accumulation error at all),
// below the accumulation error of an FP32 FMA chain once k exceeds a few
// dozen; the decision between the two engines (gb_set_sgemm_mode) rests on
// measurements recorded with the library.
#include "gb_internal.h"

namespace gb {
namespace {

// dst (rows x cols, column-major, ld = rows) = (double) src(i, j) at src[i*rs + j*cs]
__global__ void f32_to_f64_kernel(int64_t rows, int64_t cols, const float* __restrict__ src, int64_t rs,
                                  int64_t cs, double* __restrict__ dst)
{
    const int64_t total = rows * cols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        // 32-bit division while the index fits (the 64-bit one costs several times more)
        const int64_t j = (total <= 0xFFFFFFFFll) ? (int64_t)((uint32_t)e / (uint32_t)rows) : e / rows;
        const int64_t i = e - j * rows;
        dst[e] = (double)src[i * rs + j * cs];
    }
}

// C(i, j) = RN32(alpha P(i, j) + beta C(i, j)); beta == 0 does not read C
__global__ void sgemm_split_epilogue_kernel(int64_t m, int64_t n, const double* __restrict__ P, double alpha,
                                            double beta, float* __restrict__ c, int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = (total <= 0xFFFFFFFFll) ? (int64_t)((uint32_t)e / (uint32_t)m) : e / m;
        const int64_t i = e - j * m;
        float* cij = c + i * rs_c + j * cs_c;
        const double t = alpha * P[e];
        *cij = (float)(beta == 0.0 ? t : fma(beta, (double)*cij, t));
    }
}

unsigned grid_for(int64_t total)
{
    const int64_t cap = (int64_t)(sm_count() > 0 ? sm_count() : 148) * 16;
    int64_t g = (total + 255) / 256;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

int sgemm_mode_setting = GB_SGEMM_AUTO;

bool sgemm_use_split(int64_t m, int64_t n, int64_t k)
{
    if (sgemm_mode_setting == GB_SGEMM_SPLIT) return true;
    if (sgemm_mode_setting == GB_SGEMM_FMA) return false;
    // automatic: the split form where its fixed costs (widening, split, recombination) are
    // small against the products
    return m >= 1024 && n >= 1024 && k >= 512;
}

int sgemm_split_dev(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                    const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                    cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0f || k <= 0) return scal_matrix_f(m, n, beta, c, rs_c, cs_c, s);
    double* ad = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(m * k), s));
    double* bd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(k * n), s));
    double* pd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(m * n), s));
    int rc = (ad && bd && pd) ? GB_SUCCESS : GB_ERR_NOMEM;
    if (!rc) {
        LaunchScope ls("sgemm_split_widen", s);
        f32_to_f64_kernel<<<grid_for(m * k), 256, 0, s>>>(m, k, a, ars, acs, ad);
        f32_to_f64_kernel<<<grid_for(k * n), 256, 0, s>>>(k, n, b, brs, bcs, bd);
        rc = check_cuda(cudaGetLastError(), "sgemm split widen");
    }
    if (!rc) {
        ModeOverride digits(GB_DGEMM_OZAKI, GB_SGEMM_SPLIT_SLICES, 0);
        rc = dgemm_ozaki(m, n, k, 1.0, ad, 1, m, bd, 1, k, 0.0, pd, 1, m, GB_SGEMM_SPLIT_SLICES, s);
    }
    if (!rc) {
        LaunchScope ls("sgemm_split_epilogue", s);
        sgemm_split_epilogue_kernel<<<grid_for(m * n), 256, 0, s>>>(m, n, pd, (double)alpha, (double)beta, c, rs_c,
                                                                    cs_c);
        rc = check_cuda(cudaGetLastError(), "sgemm split epilogue");
    }
    dev_free(ad, s);
    dev_free(bd, s);
    dev_free(pd, s);
    return rc;
}

}  // namespace gb

extern "C" int gb_set_sgemm_mode(int mode)
{
    if (mode != GB_SGEMM_FMA && mode != GB_SGEMM_SPLIT && mode != GB_SGEMM_AUTO)
        return gb::set_error(GB_ERR_ARG, "gb_set_sgemm_mode", "mode must be GB_SGEMM_FMA, _SPLIT or _AUTO");
    gb::sgemm_mode_setting = mode;
    return GB_SUCCESS;
}
