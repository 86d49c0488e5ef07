// gb_sgemm_split.cu -- SGEMM on the bf16 tensor cores (the split form of sgemm).
//
// FP32 FMA SGEMM on GB300 runs on the FP32 pipe (about 80 TFLOP/s nominal at the
// boost clock); the bf16 tensor cores are twenty times wider.  This form runs
// C := alpha op(A) op(B) + beta C for FP32 operands as the digit form of the
// Ozaki product with 3 slices (6 bf16 products, exact integer accumulation):
// the splits read op(A) and op(B) in FP32 and widen each element exactly as
// it loads, every row's digits hold 24 bits below 2^e (e = ilogb(row max) +
// 2), the slice GEMM is the FP64 path's, and the recombination writes
// C = RN32(alpha P + beta C) with P the FP64 product (sgemm_ozaki,
// gb_ozaki.cu: no FP64 copies of the operands, no separate epilogue).  Its error is
// the representation error of 24-bit digits (no accumulation error at all),
// below the accumulation error of an FP32 FMA chain once k exceeds a few
// dozen; the decision between the two engines (gb_set_sgemm_mode) rests on
// measurements recorded with the library.
#include "gb_internal.h"

namespace gb {

int sgemm_mode_setting = GB_SGEMM_AUTO;

bool sgemm_use_split(int64_t m, int64_t n, int64_t k)
{
    if (sgemm_mode_setting == GB_SGEMM_SPLIT) return true;
    if (sgemm_mode_setting == GB_SGEMM_FMA) return false;
    // automatic: the split form where its fixed costs (split, recombination) are
    // small against the products
    return m >= 1024 && n >= 1024 && k >= 512;
}

int sgemm_split_dev(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                    const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                    cudaStream_t s)
{
    return sgemm_ozaki(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, s);
}

}  // namespace gb

extern "C" int gb_set_sgemm_mode(int mode)
{
    if (mode != GB_SGEMM_FMA && mode != GB_SGEMM_SPLIT && mode != GB_SGEMM_AUTO)
        return gb::set_error(GB_ERR_ARG, "gb_set_sgemm_mode", "mode must be GB_SGEMM_FMA, _SPLIT or _AUTO");
    gb::sgemm_mode_setting = mode;
    return GB_SUCCESS;
}
