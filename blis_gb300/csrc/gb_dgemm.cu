// gb_dgemm.cu -- native FP64 GEMM for sm_103a (the plain form of
// bli_gemm; frame/3/bli_l3_oapi_ex.c:48-148, micro-kernel contract
// ref_kernels/3/bli_gemm_ref.c:40-130).
//
// GB300 has no tcgen05 kind for f64, and its FP64 pipe is a small fraction
// of the tensor rate, so this kernel is compute-bound by a wide margin: a
// 128x128 C tile does 262,144 FMAs per 16-deep k block but moves only 32 KB.
// The five BLIS loops collapse into a 2-D grid of C tiles (JC/IC), a k loop
// per CTA (PC) with a register-prefetched shared-memory stage (the packing
// step), and 8 warps each owning a 64x32 sub-tile (JR/IR).  Two inner
// engines are built: DMMA (mma.sync m8n8k4 f64) and plain DFMA; the host
// picks DMMA unless GB_DGEMM_ENGINE=dfma.  Operands may have any strides
// (BLIS general storage), folded with the transposes into (ars, acs) and
// (brs, bcs) by the caller.
#include <stdlib.h>
#include <string.h>

#include "gb_gemm_tiles.cuh"

namespace gb {
namespace {

using namespace tiles;

// gate != nullptr: the kernel only runs when *gate is nonzero (a device-side
// condition raised by an earlier kernel on the same stream).
__global__ void __launch_bounds__(NT) dgemm_dmma_kernel(DArgs p, const int* gate)
{
    if (gate && *gate == 0) return;
    __shared__ double As[BK * LDS];
    __shared__ double Bs[BK * LDS];
    dmma_tile(p, (int64_t)blockIdx.y * BM, (int64_t)blockIdx.x * BN, As, Bs);
}

template <typename T>
__global__ void __launch_bounds__(NT) gemm_simt_kernel(GArgs<T> p, const int* gate)
{
    if (gate && *gate == 0) return;
    __shared__ T As[BK * LDS];
    __shared__ T Bs[BK * LDS];
    simt_tile<T>(p, (int64_t)blockIdx.y * BM, (int64_t)blockIdx.x * BN, As, Bs);
}

// The gated IEEE fallbacks (Inf/NaN operands of the Ozaki and split forms):
// at most two CTAs per SM, each walking tiles (tile t: row block t / gx,
// column block t % gx), so that a launch whose flag is clear, the common
// case, retires a few hundred CTAs instead of one per tile.
__global__ void __launch_bounds__(NT) dgemm_dmma_gated_kernel(DArgs p, const int* gate, int64_t gx, int64_t tiles)
{
    if (*gate == 0) return;
    __shared__ double As[BK * LDS];
    __shared__ double Bs[BK * LDS];
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) dmma_tile(p, (t / gx) * BM, (t % gx) * BN, As, Bs);
}

template <typename T>
__global__ void __launch_bounds__(NT) gemm_simt_gated_kernel(GArgs<T> p, const int* gate, int64_t gx, int64_t tiles)
{
    if (*gate == 0) return;
    __shared__ T As[BK * LDS];
    __shared__ T Bs[BK * LDS];
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) simt_tile<T>(p, (t / gx) * BM, (t % gx) * BN, As, Bs);
}

unsigned gated_grid(int64_t tiles)
{
    const int64_t cap = 2 * (int64_t)(sm_count() > 0 ? sm_count() : 148);
    return (unsigned)(tiles < cap ? tiles : cap);
}

template <bool VEC, bool A_RC, bool B_RC>
__global__ void __launch_bounds__(NT, 2) sgemm_kernel(GArgs<float> p)  // two CTAs (16 warps) per SM
{
    __shared__ __align__(16) float As[2 * BK * LDS];
    __shared__ __align__(16) float Bs[2 * BK * LDS];
    sgemm_tile<VEC, A_RC, B_RC>(p, (int64_t)blockIdx.y * BM, (int64_t)blockIdx.x * BN, As, Bs);
}

// Whole tiles and k blocks only, 16-byte aligned operands, one unit stride
// per operand with the other stride a multiple of 4 floats.
bool sgemm_vec_ok(const GArgs<float>& p, bool* a_rc, bool* b_rc)
{
    if (p.m % BM || p.n % BN || p.k % BK) return false;
    if ((reinterpret_cast<uintptr_t>(p.a) | reinterpret_cast<uintptr_t>(p.b)) & 15) return false;
    if (p.ars == 1 && p.acs % 4 == 0) *a_rc = true;
    else if (p.acs == 1 && p.ars % 4 == 0) *a_rc = false;
    else return false;
    if (p.bcs == 1 && p.brs % 4 == 0) *b_rc = true;
    else if (p.brs == 1 && p.bcs % 4 == 0) *b_rc = false;
    else return false;
    return true;
}

template <typename T>
__global__ void scal_matrix_kernel(int64_t m, int64_t n, T beta, T* c, int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i, j;
        if (rs_c == 1 || cs_c != 1) { i = e % m; j = e / m; } else { j = e % n; i = e / n; }
        T* cij = c + i * rs_c + j * cs_c;
        *cij = (beta == T(0)) ? T(0) : beta * *cij;
    }
}

bool use_dfma()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("GB_DGEMM_ENGINE");
        v = (e && strcmp(e, "dfma") == 0) ? 1 : 0;
    }
    return v == 1;
}

}  // namespace

int scal_matrix(int64_t m, int64_t n, double beta, double* c, int64_t rs_c, int64_t cs_c,
                cudaStream_t s)
{
    if (m <= 0 || n <= 0 || beta == 1.0) return GB_SUCCESS;
    const int64_t total = m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8 * 152 * 4) blocks = 8 * 152 * 4;
    LaunchScope ls("scal_matrix", s);
    scal_matrix_kernel<double><<<blocks, 256, 0, s>>>(m, n, beta, c, rs_c, cs_c);
    return check_cuda(cudaGetLastError(), "scal_matrix");
}

int scal_matrix_f(int64_t m, int64_t n, float beta, float* c, int64_t rs_c, int64_t cs_c,
                  cudaStream_t s)
{
    if (m <= 0 || n <= 0 || beta == 1.0f) return GB_SUCCESS;
    const int64_t total = m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8 * 152 * 4) blocks = 8 * 152 * 4;
    LaunchScope ls("scal_matrix", s);
    scal_matrix_kernel<float><<<blocks, 256, 0, s>>>(m, n, beta, c, rs_c, cs_c);
    return check_cuda(cudaGetLastError(), "scal_matrix_f");
}

int dgemm_native_gated(int64_t m, int64_t n, int64_t k, double alpha,
                       const double* a, int64_t ars, int64_t acs,
                       const double* b, int64_t brs, int64_t bcs, double beta,
                       double* c, int64_t rs_c, int64_t cs_c, const int* gate, cudaStream_t s)
{
    // Early exits of frame/3/bli_l3_util.c:41-65.
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0 || k <= 0) return gate ? GB_SUCCESS : scal_matrix(m, n, beta, c, rs_c, cs_c, s);
    const int64_t gx = (n + BN - 1) / BN, gy = (m + BM - 1) / BM;
    if (gy > 65535) return set_error(GB_ERR_ARG, "gb_dgemm", "m too large for one launch");
    DArgs p{m, n, k, alpha, beta, a, ars, acs, b, brs, bcs, c, rs_c, cs_c};
    dim3 grid((unsigned)gx, (unsigned)gy);
    if (gate) {
        if (use_dfma()) {
            LaunchScope ls("dgemm_dfma_gated", s);
            gemm_simt_gated_kernel<double><<<gated_grid(gx * gy), NT, 0, s>>>(p, gate, gx, gx * gy);
        } else {
            LaunchScope ls("dgemm_dmma_gated", s);
            dgemm_dmma_gated_kernel<<<gated_grid(gx * gy), NT, 0, s>>>(p, gate, gx, gx * gy);
        }
        return check_cuda(cudaGetLastError(), "dgemm_native_gated");
    }
    if (use_dfma()) {
        LaunchScope ls("dgemm_dfma", s);
        gemm_simt_kernel<double><<<grid, NT, 0, s>>>(p, gate);
    } else {
        LaunchScope ls(gate ? "dgemm_dmma_gated" : "dgemm_dmma", s);
        dgemm_dmma_kernel<<<grid, NT, 0, s>>>(p, gate);
    }
    return check_cuda(cudaGetLastError(), "dgemm_native");
}

// FP32 C := alpha op(A) op(B) + beta C on the FP32 FMA pipe, only when *gate is
// nonzero: the IEEE fallback of the SGEMM split form for Inf/NaN operands.
int sgemm_native_gated(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                       const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                       const int* gate, cudaStream_t s)
{
    if (m <= 0 || n <= 0 || alpha == 0.0f || k <= 0) return GB_SUCCESS;  // the split form handled these
    const int64_t gx = (n + BN - 1) / BN, gy = (m + BM - 1) / BM;
    if (gy > 65535) return set_error(GB_ERR_ARG, "gb_sgemm", "m too large for one launch");
    GArgs<float> p{m, n, k, alpha, beta, a, ars, acs, b, brs, bcs, c, rs_c, cs_c};
    LaunchScope ls("sgemm_ffma_gated", s);
    gemm_simt_gated_kernel<float><<<gated_grid(gx * gy), NT, 0, s>>>(p, gate, gx, gx * gy);
    return check_cuda(cudaGetLastError(), "sgemm_native_gated");
}

int dgemm_native(int64_t m, int64_t n, int64_t k, double alpha,
                 const double* a, int64_t ars, int64_t acs,
                 const double* b, int64_t brs, int64_t bcs, double beta,
                 double* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    return dgemm_native_gated(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, nullptr, s);
}

int sgemm_dev(int64_t m, int64_t n, int64_t k, float alpha,
              const float* a, int64_t ars, int64_t acs,
              const float* b, int64_t brs, int64_t bcs, float beta,
              float* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0f || k <= 0) return scal_matrix_f(m, n, beta, c, rs_c, cs_c, s);
    const int64_t gx = (n + BN - 1) / BN, gy = (m + BM - 1) / BM;
    if (gy > 65535) return set_error(GB_ERR_ARG, "gb_sgemm", "m too large for one launch");
    GArgs<float> p{m, n, k, alpha, beta, a, ars, acs, b, brs, bcs, c, rs_c, cs_c};
    const dim3 grid((unsigned)gx, (unsigned)gy);
    bool a_rc = true, b_rc = false;
    LaunchScope ls("sgemm_ffma", s);
    if (!sgemm_vec_ok(p, &a_rc, &b_rc)) sgemm_kernel<false, true, false><<<grid, NT, 0, s>>>(p);
    else if (a_rc && !b_rc) sgemm_kernel<true, true, false><<<grid, NT, 0, s>>>(p);
    else if (a_rc && b_rc) sgemm_kernel<true, true, true><<<grid, NT, 0, s>>>(p);
    else if (!a_rc && !b_rc) sgemm_kernel<true, false, false><<<grid, NT, 0, s>>>(p);
    else sgemm_kernel<true, false, true><<<grid, NT, 0, s>>>(p);
    return check_cuda(cudaGetLastError(), "sgemm");
}

}  // namespace gb
