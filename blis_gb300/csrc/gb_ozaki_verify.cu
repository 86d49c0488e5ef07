// gb_ozaki_verify.cu -- error-bound verifier for the Ozaki slice count.
//
// For a proposed slice count s, the split of op(A) and op(B)^T loses at most
// 2^-(8s+1) of each row's scale 2^e (balanced digits), and the triangular
// product set drops the pairs p + q > s + 1, which sum to
// sum_p A_p R^B_{s+1-p} per product: at most s 2^(e_i+e_j-8s-2).  The
// verifier demands, on a deterministic sample of entries, that
//   2^-(8s+1) (2^e_i |B_j|_1 + |A_i|_1 2^e_j) + sqrt(k) s 2^(e_i+e_j-8s-2)
// stays below sqrt(k) u (|A||B|)_ij -- the size of a typical (random-sign,
// not worst-case) FP64 dot-product error; the dropped products are counted
// with the same random-sign sqrt(k) growth.  It reports the smallest slice
// count >= s_min that meets this.  All bulk work is one warp per sampled
// entry (five length-k reductions in FP64).
#include <math.h>

#include "gb_internal.h"

namespace gb {
namespace {

__device__ __forceinline__ uint64_t vmix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ double warp_max_d(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// One warp per sampled entry (i, j): row i of op(A), column j of op(B).
__global__ void verify_kernel(int64_t m, int64_t n, int64_t k, const double* __restrict__ a, int64_t ars,
                              int64_t acs, const double* __restrict__ b, int64_t brs, int64_t bcs, int s_min,
                              int nsample, int* __restrict__ s_req)
{
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    if (w >= nsample) return;
    const uint64_t h = vmix(0x5EED5EEDull + (uint64_t)w * 0x9E3779B97F4A7C15ull);
    const int64_t i = (int64_t)(h % (uint64_t)m), j = (int64_t)((h >> 32) % (uint64_t)n);
    double g = 0.0, ra = 0.0, rb = 0.0, ma = 0.0, mb = 0.0;
    for (int64_t l = lane; l < k; l += 32) {
        const double x = fabs(a[i * ars + l * acs]), y = fabs(b[l * brs + j * bcs]);
        g = fma(x, y, g);
        ra += x;
        rb += y;
        ma = fmax(ma, x);
        mb = fmax(mb, y);
    }
    g = warp_sum_d(g);
    ra = warp_sum_d(ra);
    rb = warp_sum_d(rb);
    ma = warp_max_d(ma);
    mb = warp_max_d(mb);
    if (lane != 0) return;
    int need = s_min;
    if (g > 0.0) {
        // row exponents of the split: 2^e > 2 * (row max)
        const double sa = ldexp(1.0, ilogb(ma) + 2), sb = ldexp(1.0, ilogb(mb) + 2);
        const double target = sqrt((double)k) * ldexp(1.0, -53) * g;
        need = 13;
        for (int s = (s_min > 2 ? s_min : 2); s <= 12; ++s) {
            // remainders: |x - sum of s digits| <= 2^-(8s+1) of the row scale
            const double rep = ldexp(1.0, -(8 * s + 1)) * (sa * rb + ra * sb);
            // dropped pairs p+q > s+1: sum_p A_p * R^B_{s+1-p}, |A_p| <= 2^(e-8p+7),
            // |R^B_t| <= (1 + 2^-7) 2^(e-8t-1) (the digits after t are at most 128 in
            // magnitude, the last remainder at most half a unit; the factor 1.01
            // covers the excess), i.e. s 2^(e_i+e_j-8s-2) per product; random
            // signs accumulate like sqrt(k), as the FP64 error it is compared with
            const double drop = sqrt((double)k) * sa * sb * ldexp(1.0, -8 * s - 2) * (double)s * 1.01;
            if (rep + drop <= target) {
                need = s;
                break;
            }
        }
    }
    atomicMax(s_req, need);
}

}  // namespace
}  // namespace gb

extern "C" int gb_ozaki_verify_slices_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                                          const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                                          gb_inc_t rs_b, gb_inc_t cs_b, int s_min, int nsample, int* s_out,
                                          void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (!s_out) return gb::set_error(GB_ERR_ARG, "gb_ozaki_verify_slices_dev", "null s_out");
    if (m <= 0 || n <= 0 || k <= 0 || nsample <= 0) {
        *s_out = s_min;
        return GB_SUCCESS;
    }
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : gb::thread_stream();
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    int* d = static_cast<int*>(gb::dev_alloc(sizeof(int), s));
    if (!d) return GB_ERR_NOMEM;
    GB_CUDA(cudaMemsetAsync(d, 0, sizeof(int), s));
    {
        gb::LaunchScope ls("ozaki_verify", s);
        gb::verify_kernel<<<(unsigned)((nsample * 32 + 255) / 256), 256, 0, s>>>(
            m, n, k, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b, tb ? rs_b : cs_b, s_min, nsample, d);
    }
    int h = 0;
    rc = gb::check_cuda(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s), "verify");
    if (!rc) rc = gb::check_cuda(cudaStreamSynchronize(s), "verify");
    gb::dev_free(d, s);
    if (rc) return rc;
    *s_out = h > s_min ? h : s_min;
    return GB_SUCCESS;
}
