// gb_level1v2.cu -- bandwidth-bound level-1v / level-2 kernels for sm_103a:
// axpyv (ref_kernels/1/bli_axpyv_ref.c:37-120), dotv
// (ref_kernels/1/bli_dotv_ref.c:37-121) and gemv
// (frame/2/bli_l2_tapi.c:43-127; var1/var2 in frame/2/gemv/).
//
// None of these touch the tensor pipes.  Unit-stride operands stream with
// 16-byte (double2) loads and grid-stride loops sized to the SM count; the
// reductions are warp-shuffle trees followed by a fixed-order second pass,
// so results are bitwise reproducible run to run (no floating-point
// atomics).  Non-unit and negative strides take scalar paths with the same
// reduction order.
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int NT = 256;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---------------------------------------------------------------- axpyv
__global__ void axpyv_vec_kernel(int64_t n2, double alpha, const double2* __restrict__ x,
                                 double2* __restrict__ y)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n2; i += (int64_t)gridDim.x * NT) {
        const double2 xv = __ldcs(x + i);
        double2 yv = __ldcs(y + i);
        yv.x = fma(alpha, xv.x, yv.x);
        yv.y = fma(alpha, xv.y, yv.y);
        __stcs(y + i, yv);
    }
}

__global__ void axpyv_strided_kernel(int64_t n, double alpha, const double* __restrict__ x,
                                     int64_t incx, double* __restrict__ y, int64_t incy)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        y[i * incy] = fma(alpha, x[i * incx], y[i * incy]);
}

// ---------------------------------------------------------------- dotv
// Pass 1: block b reduces the contiguous chunk [b*chunk, min(n, (b+1)*chunk)).
__global__ void dotv_partial_kernel(int64_t n, int64_t chunk, const double* __restrict__ x,
                                    int64_t incx, const double* __restrict__ y, int64_t incy,
                                    double* __restrict__ partial)
{
    __shared__ double red[NT / 32];
    const int64_t lo = (int64_t)blockIdx.x * chunk;
    const int64_t hi = (lo + chunk < n) ? lo + chunk : n;
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0, acc3 = 0.0;
    const bool vec = (incx == 1 && incy == 1 && ((reinterpret_cast<uintptr_t>(x + lo) |
                                                  reinterpret_cast<uintptr_t>(y + lo)) & 15) == 0);
    if (vec) {
        const int64_t len2 = (hi - lo) >> 1;
        const double2* x2 = reinterpret_cast<const double2*>(x + lo);
        const double2* y2 = reinterpret_cast<const double2*>(y + lo);
        int64_t i = threadIdx.x;
        // four 16-byte loads of each vector in flight per thread
        for (; i + 3 * NT < len2; i += 4 * NT) {
            const double2 a0 = __ldcs(x2 + i), a1 = __ldcs(x2 + i + NT);
            const double2 a2 = __ldcs(x2 + i + 2 * NT), a3 = __ldcs(x2 + i + 3 * NT);
            const double2 b0 = __ldcs(y2 + i), b1 = __ldcs(y2 + i + NT);
            const double2 b2 = __ldcs(y2 + i + 2 * NT), b3 = __ldcs(y2 + i + 3 * NT);
            acc0 = fma(a0.x, b0.x, acc0); acc1 = fma(a0.y, b0.y, acc1);
            acc2 = fma(a1.x, b1.x, acc2); acc3 = fma(a1.y, b1.y, acc3);
            acc0 = fma(a2.x, b2.x, acc0); acc1 = fma(a2.y, b2.y, acc1);
            acc2 = fma(a3.x, b3.x, acc2); acc3 = fma(a3.y, b3.y, acc3);
        }
        for (; i < len2; i += NT) {
            const double2 a = __ldcs(x2 + i), b = __ldcs(y2 + i);
            acc0 = fma(a.x, b.x, acc0);
            acc1 = fma(a.y, b.y, acc1);
        }
        if (((hi - lo) & 1) && threadIdx.x == 0) acc0 = fma(x[hi - 1], y[hi - 1], acc0);
    } else {
        for (int64_t i = lo + threadIdx.x; i < hi; i += NT) acc0 = fma(x[i * incx], y[i * incy], acc0);
    }
    double v = warp_sum((acc0 + acc1) + (acc2 + acc3));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < NT / 32) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

// Pass 2: one block sums the partials in a fixed order.
__global__ void dotv_final_kernel(int nparts, const double* __restrict__ partial,
                                  double* __restrict__ rho)
{
    __shared__ double red[NT / 32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += NT) acc += partial[i];
    double v = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < NT / 32) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *rho = v;
    }
}

__global__ void set_scalar_kernel(double* p, double v) { *p = v; }

// ---------------------------------------------------------------- gemv
// Output index o, reduction index r; M(o, r) = a[o*so + r*sr].
// "dot" form (sr == 1): one warp per output, lanes stride along r.
template <bool VEC>
__global__ void gemv_dot_kernel(int64_t nout, int64_t nred, double alpha,
                                const double* __restrict__ a, int64_t so,
                                const double* __restrict__ x, int64_t incx, double beta,
                                double* __restrict__ y, int64_t incy)
{
    const int lane = threadIdx.x & 31;
    const int64_t o = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
    if (o >= nout) return;
    const double* col = a + o * so;
    double acc0 = 0.0, acc1 = 0.0;
    if (VEC) {
        const double2* c2 = reinterpret_cast<const double2*>(col);
        const double2* x2 = reinterpret_cast<const double2*>(x);
        const int64_t n2 = nred >> 1;
        int64_t i = lane;
        for (; i + 32 < n2; i += 64) {
            const double2 a0 = __ldcs(c2 + i), a1 = __ldcs(c2 + i + 32);
            const double2 x0 = __ldg(x2 + i), x1 = __ldg(x2 + i + 32);
            acc0 = fma(a0.x, x0.x, acc0); acc1 = fma(a0.y, x0.y, acc1);
            acc0 = fma(a1.x, x1.x, acc0); acc1 = fma(a1.y, x1.y, acc1);
        }
        for (; i < n2; i += 32) {
            const double2 a0 = __ldcs(c2 + i), x0 = __ldg(x2 + i);
            acc0 = fma(a0.x, x0.x, acc0); acc1 = fma(a0.y, x0.y, acc1);
        }
        if ((nred & 1) && lane == 0) acc0 = fma(col[nred - 1], x[nred - 1], acc0);
    } else {
        for (int64_t r = lane; r < nred; r += 32) acc0 = fma(col[r], x[r * incx], acc0);
    }
    const double v = warp_sum(acc0 + acc1);
    if (lane == 0) {
        double* yo = y + o * incy;
        const double yb = (beta == 0.0) ? 0.0 : beta * *yo;
        *yo = fma(alpha, v, yb);
    }
}

// "axpy" form (so == 1): threads over outputs, blockIdx.y splits r; partial
// sums land in part[split][o] and a second kernel folds them in order.
template <bool VEC>
__global__ void gemv_axpy_kernel(int64_t nout, int64_t nred, int64_t rchunk,
                                 const double* __restrict__ a, int64_t sr,
                                 const double* __restrict__ x, int64_t incx,
                                 double* __restrict__ part)
{
    const int64_t r0 = (int64_t)blockIdx.y * rchunk;
    const int64_t r1 = (r0 + rchunk < nred) ? r0 + rchunk : nred;
    if (VEC) {
        const int64_t o = ((int64_t)blockIdx.x * NT + threadIdx.x) * 2;
        if (o >= nout) return;
        double acc0 = 0.0, acc1 = 0.0;
        if (o + 1 < nout) {
            int64_t r = r0;
            for (; r + 3 < r1; r += 4) {
                const double2 a0 = __ldcs(reinterpret_cast<const double2*>(a + o + (r + 0) * sr));
                const double2 a1 = __ldcs(reinterpret_cast<const double2*>(a + o + (r + 1) * sr));
                const double2 a2 = __ldcs(reinterpret_cast<const double2*>(a + o + (r + 2) * sr));
                const double2 a3 = __ldcs(reinterpret_cast<const double2*>(a + o + (r + 3) * sr));
                const double x0 = __ldg(x + (r + 0) * incx), x1 = __ldg(x + (r + 1) * incx);
                const double x2 = __ldg(x + (r + 2) * incx), x3 = __ldg(x + (r + 3) * incx);
                acc0 = fma(a0.x, x0, acc0); acc1 = fma(a0.y, x0, acc1);
                acc0 = fma(a1.x, x1, acc0); acc1 = fma(a1.y, x1, acc1);
                acc0 = fma(a2.x, x2, acc0); acc1 = fma(a2.y, x2, acc1);
                acc0 = fma(a3.x, x3, acc0); acc1 = fma(a3.y, x3, acc1);
            }
            for (; r < r1; ++r) {
                const double2 a0 = __ldcs(reinterpret_cast<const double2*>(a + o + r * sr));
                const double x0 = __ldg(x + r * incx);
                acc0 = fma(a0.x, x0, acc0); acc1 = fma(a0.y, x0, acc1);
            }
            part[blockIdx.y * nout + o] = acc0;
            part[blockIdx.y * nout + o + 1] = acc1;
        } else {
            for (int64_t r = r0; r < r1; ++r) acc0 = fma(a[o + r * sr], x[r * incx], acc0);
            part[blockIdx.y * nout + o] = acc0;
        }
    } else {
        const int64_t o = (int64_t)blockIdx.x * NT + threadIdx.x;
        if (o >= nout) return;
        double acc = 0.0;
        for (int64_t r = r0; r < r1; ++r) acc = fma(a[o + r * sr], x[r * incx], acc);
        part[blockIdx.y * nout + o] = acc;
    }
}

__global__ void gemv_fold_kernel(int64_t nout, int nsplit, const double* __restrict__ part,
                                 double alpha, double beta, double* __restrict__ y, int64_t incy)
{
    const int64_t o = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (o >= nout) return;
    double acc = 0.0;
    for (int s = 0; s < nsplit; ++s) acc += part[(int64_t)s * nout + o];
    double* yo = y + o * incy;
    const double yb = (beta == 0.0) ? 0.0 : beta * *yo;
    *yo = fma(alpha, acc, yb);
}

// General strides: thread per output, serial reduction.
__global__ void gemv_generic_kernel(int64_t nout, int64_t nred, double alpha,
                                    const double* __restrict__ a, int64_t so, int64_t sr,
                                    const double* __restrict__ x, int64_t incx, double beta,
                                    double* __restrict__ y, int64_t incy)
{
    const int64_t o = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (o >= nout) return;
    double acc = 0.0;
    for (int64_t r = 0; r < nred; ++r) acc = fma(a[o * so + r * sr], x[r * incx], acc);
    double* yo = y + o * incy;
    const double yb = (beta == 0.0) ? 0.0 : beta * *yo;
    *yo = fma(alpha, acc, yb);
}

__global__ void scalv_kernel(int64_t n, double beta, double* y, int64_t incy)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
        double* yi = y + i * incy;
        *yi = (beta == 0.0) ? 0.0 : beta * *yi;
    }
}

inline int grid_for(int64_t work, int per_block)
{
    int64_t g = (work + per_block - 1) / per_block;
    const int64_t cap = (int64_t)(sm_count() > 0 ? sm_count() : 152) * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int daxpyv_dev(int64_t n, double alpha, const double* x, int64_t incx, double* y,
               int64_t incy, cudaStream_t s)
{
    if (n <= 0 || alpha == 0.0) return GB_SUCCESS;  // bli_axpyv_ref.c: alpha == 0 returns
    const bool vec = (incx == 1 && incy == 1 &&
                      ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0);
    if (vec) {
        const int64_t n2 = n >> 1;
        if (n2 > 0) {
            LaunchScope ls("axpyv_vec", s);
            axpyv_vec_kernel<<<grid_for(n2, NT), NT, 0, s>>>(n2, alpha,
                reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y));
        }
        if (n & 1) {
            LaunchScope ls("axpyv_tail", s);
            axpyv_strided_kernel<<<1, NT, 0, s>>>(1, alpha, x + n - 1, 1, y + n - 1, 1);
        }
    } else {
        LaunchScope ls("axpyv_strided", s);
        axpyv_strided_kernel<<<grid_for(n, NT), NT, 0, s>>>(n, alpha, x, incx, y, incy);
    }
    return check_cuda(cudaGetLastError(), "daxpyv");
}

// Number of first-pass partial sums for a dot product of length n on a GPU
// with `sms` SMs: one per 4096 elements, at most 8 per SM.
static constexpr int dotv_nparts_for(int64_t n, int sms)
{
    int64_t g = (n + 4095) / 4096;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}
// the allocation-free dotv's scratch covers every partition on GPUs of up to 256 SMs
static_assert(dotv_nparts_for(INT64_MAX / 2, 256) <= GB_DOTV_NOALLOC_MAX_PARTS,
              "allocation-free dotv scratch smaller than the largest partition");

int dotv_nparts(int64_t n) { return dotv_nparts_for(n, sm_count()); }

// Two-pass dot product with `nparts` first-pass partial sums in `scratch`
// (at least nparts doubles); the partition depends only on n and nparts.
int ddotv_dev(int64_t n, const double* x, int64_t incx, const double* y, int64_t incy,
              double* rho_dev, double* scratch, int64_t nparts, cudaStream_t s)
{
    if (n <= 0) {
        LaunchScope ls("dotv_zero", s);
        set_scalar_kernel<<<1, 1, 0, s>>>(rho_dev, 0.0);
        return check_cuda(cudaGetLastError(), "ddotv");
    }
    if (nparts < 1) return set_error(GB_ERR_ARG, "ddotv", "no scratch for the partial sums");
    int64_t chunk = (n + nparts - 1) / nparts;
    chunk = (chunk + 1) & ~int64_t(1);  // keep chunk starts 16-byte aligned
    const int nblk = (int)((n + chunk - 1) / chunk);
    {
        LaunchScope ls("dotv_partial", s);
        dotv_partial_kernel<<<nblk, NT, 0, s>>>(n, chunk, x, incx, y, incy, scratch);
    }
    {
        LaunchScope ls("dotv_final", s);
        dotv_final_kernel<<<1, NT, 0, s>>>(nblk, scratch, rho_dev);
    }
    return check_cuda(cudaGetLastError(), "ddotv");
}

int dgemv_dev(int trans, int64_t m, int64_t n, double alpha, const double* a,
              int64_t rs_a, int64_t cs_a, const double* x, int64_t incx, double beta,
              double* y, int64_t incy, cudaStream_t s)
{
    const int64_t nout = trans ? n : m, nred = trans ? m : n;
    const int64_t so = trans ? cs_a : rs_a, sr = trans ? rs_a : cs_a;
    if (nout <= 0) return GB_SUCCESS;
    if (nred <= 0 || alpha == 0.0) {
        if (beta == 1.0) return GB_SUCCESS;
        LaunchScope ls("gemv_scal", s);
        scalv_kernel<<<grid_for(nout, NT), NT, 0, s>>>(nout, beta, y, incy);
        return check_cuda(cudaGetLastError(), "dgemv");
    }
    if (sr == 1) {
        const bool vec = (incx == 1) && ((so & 1) == 0) &&
                         ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(x)) & 15) == 0;
        const int64_t blocks = (nout * 32 + NT - 1) / NT;
        LaunchScope ls("gemv_dot", s);
        if (vec)
            gemv_dot_kernel<true><<<(unsigned)blocks, NT, 0, s>>>(nout, nred, alpha, a, so, x, incx, beta, y, incy);
        else
            gemv_dot_kernel<false><<<(unsigned)blocks, NT, 0, s>>>(nout, nred, alpha, a, so, x, incx, beta, y, incy);
        return check_cuda(cudaGetLastError(), "dgemv");
    }
    if (so == 1) {
        const bool vec = ((sr & 1) == 0) && ((reinterpret_cast<uintptr_t>(a) & 15) == 0);
        const int per = vec ? 2 * NT : NT;
        const int64_t bx = (nout + per - 1) / per;
        const int64_t target = (int64_t)(sm_count() > 0 ? sm_count() : 152) * 16;
        int64_t nsplit = (target + bx - 1) / bx;
        if (nsplit > nred) nsplit = nred;
        if (nsplit > 256) nsplit = 256;
        if (nsplit < 1) nsplit = 1;
        const int64_t rchunk = (nred + nsplit - 1) / nsplit;
        nsplit = (nred + rchunk - 1) / rchunk;
        double* part = static_cast<double*>(dev_alloc(sizeof(double) * nsplit * nout, s));
        if (!part) return GB_ERR_NOMEM;
        {
            LaunchScope ls("gemv_axpy", s);
            dim3 grid((unsigned)bx, (unsigned)nsplit);
            if (vec) gemv_axpy_kernel<true><<<grid, NT, 0, s>>>(nout, nred, rchunk, a, sr, x, incx, part);
            else gemv_axpy_kernel<false><<<grid, NT, 0, s>>>(nout, nred, rchunk, a, sr, x, incx, part);
        }
        {
            LaunchScope ls("gemv_fold", s);
            gemv_fold_kernel<<<(unsigned)((nout + NT - 1) / NT), NT, 0, s>>>(nout, (int)nsplit, part,
                                                                          alpha, beta, y, incy);
        }
        dev_free(part, s);
        return check_cuda(cudaGetLastError(), "dgemv");
    }
    LaunchScope ls("gemv_generic", s);
    gemv_generic_kernel<<<(unsigned)((nout + NT - 1) / NT), NT, 0, s>>>(nout, nred, alpha, a, so, sr,
                                                                      x, incx, beta, y, incy);
    return check_cuda(cudaGetLastError(), "dgemv");
}

}  // namespace gb

// ---------------------------------------------------------------- allocation-free dotv
// gb_ddotv_noalloc_dev: the dot product for callers that cannot allocate
// device memory.  cudaMalloc/cudaFree can synchronize the whole device and
// some host applications forbid them outright (they own a fixed device
// memory budget through their own pool, or run latency-bound loops that must
// not stall).  This entry point takes its partial-sum scratch from the
// file-scope array below instead of the library's pool, and it also skips the
// library's one-time initialisation (which allocates a status word).
//
// The array lives on every GPU that loads the library until the process
// exits: GB_DOTV_NOALLOC_MAX_PARTS doubles (16 KiB).  Every call shares it and
// finds the previous call's partial sums there; each call overwrites all the
// slots it reads, so nothing needs clearing, but two calls that overlap on the
// GPU (different streams, no ordering between them) race on the array.
#include <mutex>

#define GB_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double gb_dotv_noalloc_scratch[GB_DOTV_NOALLOC_MAX_PARTS];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[GB_NOALLOC_MAX_DEVICES];  // device address of the array, per device
int g_noalloc_sms[GB_NOALLOC_MAX_DEVICES];
}  // namespace

extern "C" int gb_ddotv_noalloc_dev(gb_dim_t n, const double* x, gb_inc_t incx, const double* y,
                                    gb_inc_t incy, double* rho, void* stream)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gb::check_cuda(e, "gb_ddotv_noalloc_dev: cudaGetDevice");
    if (dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES)
        return gb::set_error(GB_ERR_UNSUPPORTED, "gb_ddotv_noalloc_dev", "device index out of range");
    double* scratch = nullptr;
    int sms = 0;
    {
        // first call on this device (with it current): look up the array's
        // device address; the host-side name is only a stand-in for it
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, gb_dotv_noalloc_scratch);
            if (e != cudaSuccess) return gb::check_cuda(e, "gb_ddotv_noalloc_dev: cudaGetSymbolAddress");
            int nsm = 0;
            e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return gb::check_cuda(e, "gb_ddotv_noalloc_dev: SM count");
            g_noalloc_sms[dev] = nsm;
            g_noalloc_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_noalloc_ptr[dev];
        sms = g_noalloc_sms[dev];
    }
    if (n > 0 && (x == nullptr || y == nullptr))
        return gb::set_error(GB_ERR_ARG, "gb_ddotv_noalloc_dev", "null vector");
    if (rho == nullptr) return gb::set_error(GB_ERR_ARG, "gb_ddotv_noalloc_dev", "null rho");
    const int nparts = gb::dotv_nparts_for(n > 0 ? n : 1, sms);
    if (nparts > GB_DOTV_NOALLOC_MAX_PARTS) {
        char buf[160];
        snprintf(buf, sizeof(buf), "needs %d partial sums; the allocation-free scratch holds %d",
                 nparts, GB_DOTV_NOALLOC_MAX_PARTS);
        return gb::set_error(GB_ERR_ARG, "gb_ddotv_noalloc_dev", buf);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    return gb::ddotv_dev(n, x, incx, y, incy, rho, scratch, nparts, s);
}
