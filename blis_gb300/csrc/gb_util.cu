// gb_util.cu -- device utilities around the hot path:
//
//  * gb_randm_dev: fills a matrix with seeded values from a counter-based
//    generator (SplitMix64 finaliser over seed and element index), the GPU
//    counterpart of BLIS's bli_randm (frame/util; values from
//    frame/include/bli_cast_macro_defs.h:465-525).  Uniform [lo, hi),
//    "exponent spread" (1+u) 2^e with random sign, and the testsuite's
//    narrow powers of two.  Every value is produced by integer operations and
//    exact FP64 steps, so it is identical wherever it is generated.
//  * gb_dd_gemm_entries_dev: the double-double value of selected entries of
//    alpha*op(A)*op(B) + beta*C (Dekker/Knuth error-free sums and products),
//    used to report the max componentwise error of a GEMM result.
#include "gb_internal.h"

namespace gb {
namespace {

constexpr uint64_t GOLDEN = 0x9E3779B97F4A7C15ull;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void randm_kernel(int kind, int is_float, void* out, int64_t m, int64_t n,
                             int64_t rs, int64_t cs, uint64_t seed, double p0, double p1)
{
    const uint64_t base = mix64(seed + GOLDEN);
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        // element index in column-major order of the logical m x n matrix
        const uint64_t h = mix64(base + (uint64_t)(e + 1) * GOLDEN);
        double v;
        if (kind == GB_RAND_UNIFORM) {
            const double u = (double)(h >> 11) * 0x1.0p-53;
            v = __dadd_rn(p0, __dmul_rn(__dsub_rn(p1, p0), u));
        } else if (kind == GB_RAND_EXPSPREAD) {
            const int emin = (int)p0, emax = (int)p1;
            const double mant = 1.0 + (double)(h >> 12) * 0x1.0p-52;
            const int ex = emin + (int)(((h >> 1) & 0x7FFull) % (uint64_t)(emax - emin + 1));
            v = ldexp(mant, ex);
            if (h & 1ull) v = -v;
        } else {
            const int t = (int)(h & 7ull);
            v = (t == 0) ? 0.0 : ldexp(1.0, -(t - 1));
            if ((h >> 3) & 1ull) v = -v;
        }
        const int64_t i = e % m, j = e / m;
        if (is_float) static_cast<float*>(out)[i * rs + j * cs] = __double2float_rn(v);
        else static_cast<double*>(out)[i * rs + j * cs] = v;
    }
}

struct dd {
    double hi, lo;
};

__device__ __forceinline__ dd two_sum(double a, double b)
{
    const double s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    return dd{s, __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb))};
}

__device__ __forceinline__ dd fast_two_sum(double a, double b)
{
    const double s = __dadd_rn(a, b);
    return dd{s, __dsub_rn(b, __dsub_rn(s, a))};
}

__device__ __forceinline__ dd dd_add(dd x, dd y)
{
    dd s = two_sum(x.hi, y.hi);
    const dd t = two_sum(x.lo, y.lo);
    s.lo = __dadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __dadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dd two_prod(double a, double b)
{
    const double p = __dmul_rn(a, b);
    return dd{p, __fma_rn(a, b, -p)};
}

// One warp per entry: lanes accumulate strided partial dd sums, then the
// 32 partials are combined in a fixed tree.
__global__ void dd_entries_kernel(int64_t k, double alpha, const double* __restrict__ a,
                                  int64_t ars, int64_t acs, const double* __restrict__ b,
                                  int64_t brs, int64_t bcs, double beta,
                                  const double* __restrict__ c, int64_t rs_c, int64_t cs_c,
                                  int64_t nent, const int64_t* __restrict__ ii,
                                  const int64_t* __restrict__ jj, double* hi, double* lo)
{
    const int lane = threadIdx.x & 31;
    const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (e >= nent) return;
    const int64_t i = ii[e], j = jj[e];
    dd s{0.0, 0.0};
    for (int64_t l = lane; l < k; l += 32) s = dd_add(s, two_prod(a[i * ars + l * acs], b[l * brs + j * bcs]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dd o{__shfl_xor_sync(0xffffffffu, s.hi, off), __shfl_xor_sync(0xffffffffu, s.lo, off)};
        s = dd_add(s, o);
    }
    if (lane == 0) {
        const double p = __dmul_rn(s.hi, alpha);
        double q = __fma_rn(s.hi, alpha, -p);
        q = __fma_rn(s.lo, alpha, q);
        dd r = fast_two_sum(p, q);
        if (beta != 0.0 && c) r = dd_add(r, two_prod(beta, c[i * rs_c + j * cs_c]));
        hi[e] = r.hi;
        lo[e] = r.lo;
    }
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gb_randm_dev(int kind, int is_float, void* x, gb_dim_t m, gb_dim_t n, gb_inc_t rs, gb_inc_t cs,
                 uint64_t seed, double p0, double p1, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (kind < GB_RAND_UNIFORM || kind > GB_RAND_NARROW_POW2)
        return set_error(GB_ERR_ARG, "gb_randm_dev", "unknown kind");
    if (kind == GB_RAND_EXPSPREAD && p1 < p0) return set_error(GB_ERR_ARG, "gb_randm_dev", "emax < emin");
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    int64_t blocks = (m * n + 255) / 256;
    const int64_t cap = (int64_t)(sm_count() > 0 ? sm_count() : 148) * 16;
    if (blocks > cap) blocks = cap;
    LaunchScope ls("randm", s);
    randm_kernel<<<(unsigned)blocks, 256, 0, s>>>(kind, is_float, x, m, n, rs, cs, seed, p0, p1);
    return check_cuda(cudaGetLastError(), "gb_randm_dev");
}

int gb_dd_gemm_entries_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t k, double alpha,
                           const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                           gb_inc_t rs_b, gb_inc_t cs_b, double beta, const double* c,
                           gb_inc_t rs_c, gb_inc_t cs_c, gb_dim_t nent, const int64_t* ii,
                           const int64_t* jj, double* hi, double* lo, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (nent <= 0) return GB_SUCCESS;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    const int64_t blocks = (nent * 32 + 255) / 256;
    LaunchScope ls("dd_entries", s);
    dd_entries_kernel<<<(unsigned)blocks, 256, 0, s>>>(k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b,
                                                       tb ? cs_b : rs_b, tb ? rs_b : cs_b, beta, c, rs_c,
                                                       cs_c, nent, ii, jj, hi, lo);
    return check_cuda(cudaGetLastError(), "gb_dd_gemm_entries_dev");
}

}  // extern "C"
