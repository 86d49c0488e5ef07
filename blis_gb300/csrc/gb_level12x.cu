// gb_level12x.cu -- the remaining real level-1v / level-2 operations for
// sm_103a, bandwidth-bound like axpyv/dotv/gemv:
//   scalv  x := alpha x; alpha == 1 returns, alpha == 0 sets zeros without
//          reading x (ref_kernels/1/bli_scalv_ref.c:40-98)
//   copyv  y := x (ref_kernels/1/bli_copyv_ref.c)
//   amaxv  index of the first element of largest |x|, the first NaN if
//          there is one (ref_kernels/1/bli_amaxv_ref.c:44-140)
//   ger    A := A + alpha x y^T, column by column as the column-major
//          variant does: a_j += (alpha y_j) x (frame/2/ger/bli_ger_unb_var2.c)
//   trsv   x := alpha inv(op(A)) x: the trsm recursion on one right-hand
//          side with gemv updates (gb_trsm.cu)
// A stride of zero makes the reference's loops revisit one element n times;
// those cases run the same sequence in one thread, so the result is the
// reference's.
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int NT = 256;

unsigned grid_n(int64_t n)
{
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t g = (n + NT - 1) / NT;
    if (g > (int64_t)sms * 8) g = (int64_t)sms * 8;
    return (unsigned)(g < 1 ? 1 : g);
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// ---------------------------------------------------------------- scalv
__global__ void scalv_vec_kernel(int64_t n2, double alpha, double2* __restrict__ x)
{
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n2; i += (int64_t)gridDim.x * NT) {
        if (alpha == 0.0) {
            __stcs(x + i, make_double2(0.0, 0.0));
        } else {
            double2 v = __ldcs(x + i);
            v.x *= alpha;
            v.y *= alpha;
            __stcs(x + i, v);
        }
    }
}

__global__ void scalv_strided_kernel(int64_t n, double alpha, double* __restrict__ x, int64_t incx)
{
    if (incx == 0) {
        // the reference's loop scales x[0] n times
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            double v = x[0];
            for (int64_t i = 0; i < n; ++i) v = (alpha == 0.0) ? 0.0 : v * alpha;
            x[0] = v;
        }
        return;
    }
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        x[i * incx] = (alpha == 0.0) ? 0.0 : x[i * incx] * alpha;
}

// ---------------------------------------------------------------- copyv
__global__ void copyv_strided_kernel(int64_t n, const double* __restrict__ x, int64_t incx, double* __restrict__ y,
                                     int64_t incy)
{
    if (incy == 0) {
        // every element lands in y[0]: the last one stays
        if (blockIdx.x == 0 && threadIdx.x == 0) y[0] = x[(n - 1) * incx];
        return;
    }
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
        y[i * incy] = x[i * incx];
}

// ---------------------------------------------------------------- amaxv
// A candidate (|x_i|, i) beats another when it is NaN and the other is not,
// or neither is NaN and its value is larger, or both tie (equal values, or
// both NaN) and its index is smaller: the order in which the reference's
// sequential scan keeps the first NaN, else the first largest element.  The
// order is total, so the two-pass tree below gives the scan's answer.
// |x| is compared as its IEEE bit pattern (sign cleared): monotone in the
// value, NaN above the infinity pattern, +0 and -0 equal; integer compares
// keep the search off GB300's narrow FP64 pipe.
constexpr unsigned long long INF_BITS = 0x7FF0000000000000ull;

struct Cand {
    unsigned long long k;  // |x| bits; 0 with i = INT64_MAX for "none yet"
    int64_t i;
};

__device__ __forceinline__ bool beats(const Cand& a, const Cand& b)
{
    const bool an = a.k > INF_BITS, bn = b.k > INF_BITS;
    if (an != bn) return an;
    if (!an && a.k != b.k) return a.k > b.k;
    return a.i < b.i;
}

__device__ __forceinline__ Cand warp_best(Cand c)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Cand o;
        o.k = __shfl_xor_sync(0xffffffffu, c.k, off);
        o.i = __shfl_xor_sync(0xffffffffu, c.i, off);
        if (beats(o, c)) c = o;
    }
    return c;
}

__device__ __forceinline__ Cand block_best(Cand c)
{
    __shared__ unsigned long long sk[NT / 32];
    __shared__ int64_t si[NT / 32];
    c = warp_best(c);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sk[w] = c.k;
        si[w] = c.i;
    }
    __syncthreads();
    if (w == 0) {
        c.k = (lane < NT / 32) ? sk[lane] : 0ull;
        c.i = (lane < NT / 32) ? si[lane] : INT64_MAX;
        c = warp_best(c);
    }
    return c;
}

// Built from the two 32-bit halves: a 64-bit mask of the sign bit is the
// pattern of an FP64 absolute value, which would put every element on the
// FP64 pipe.
__device__ __forceinline__ unsigned long long abs_key(double v)
{
    const unsigned hi = (unsigned)__double2hiint(v) & 0x7FFFFFFFu, lo = (unsigned)__double2loint(v);
    return ((unsigned long long)hi << 32) | lo;
}

// Pass 1: block b takes the contiguous range [b*chunk, min(n, (b+1)*chunk)),
// eight loads in flight per thread.
__global__ void __launch_bounds__(NT) amaxv_partial_kernel(int64_t n, int64_t chunk, const double* __restrict__ x,
                                                           int64_t incx, unsigned long long* __restrict__ pk,
                                                           int64_t* __restrict__ pi)
{
    const int64_t lo = (int64_t)blockIdx.x * chunk;
    const int64_t hi = (lo + chunk < n) ? lo + chunk : n;
    Cand c{0ull, INT64_MAX};  // any element beats it: the reference's -1 start
    int64_t i = lo + threadIdx.x;
    for (; i + 7 * NT < hi; i += 8 * NT) {
        unsigned long long k[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) k[u] = abs_key(__ldcs(x + (i + u * NT) * incx));
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const Cand o{k[u], i + u * NT};
            if (beats(o, c)) c = o;
        }
    }
    for (; i < hi; i += NT) {
        const Cand o{abs_key(__ldcs(x + i * incx)), i};
        if (beats(o, c)) c = o;
    }
    c = block_best(c);
    if (threadIdx.x == 0) {
        pk[blockIdx.x] = c.k;
        pi[blockIdx.x] = c.i;
    }
}

// Pass 2: one block over the partial results, in fixed order.
__global__ void __launch_bounds__(NT) amaxv_final_kernel(int nparts, const unsigned long long* __restrict__ pk,
                                                         const int64_t* __restrict__ pi, int64_t* __restrict__ index)
{
    Cand c{0ull, INT64_MAX};
    for (int p = threadIdx.x; p < nparts; p += NT) {
        const Cand o{pk[p], pi[p]};
        if (beats(o, c)) c = o;
    }
    c = block_best(c);
    if (threadIdx.x == 0) *index = (c.i == INT64_MAX) ? 0 : c.i;
}

// ---------------------------------------------------------------- ger
// a(i, j) += (alpha y_j) x_i; blockIdx.y walks columns, threads walk rows
// (coalesced for column-major A), x_i kept in a register across the CTA's
// columns.
constexpr int GER_COLS = 8;

__global__ void __launch_bounds__(NT) ger_kernel(int64_t m, int64_t n, double alpha, const double* __restrict__ x,
                                                 int64_t incx, const double* __restrict__ y, int64_t incy,
                                                 double* __restrict__ a, int64_t rs_a, int64_t cs_a)
{
    for (int64_t j0 = (int64_t)blockIdx.y * GER_COLS; j0 < n; j0 += (int64_t)gridDim.y * GER_COLS) {
        const int jn = (n - j0 < GER_COLS) ? (int)(n - j0) : GER_COLS;
        double ay[GER_COLS];
#pragma unroll
        for (int q = 0; q < GER_COLS; ++q) ay[q] = (q < jn) ? alpha * y[(j0 + q) * incy] : 0.0;
        for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < m; i += (int64_t)gridDim.x * NT) {
            const double xi = x[i * incx];
#pragma unroll
            for (int q = 0; q < GER_COLS; ++q) {
                if (q < jn) {
                    double* aij = a + i * rs_a + (j0 + q) * cs_a;
                    *aij = fma(ay[q], xi, *aij);
                }
            }
        }
    }
}

// Unit-stride x and column-major A with 16-byte aligned columns: a CTA owns
// GER_COLS columns and walks all rows two at a time (double2 loads and
// stores with streaming hints), reading each pair of x once for its columns.
__global__ void __launch_bounds__(NT, 4) ger_vec_kernel(int64_t m2, int64_t n, double alpha,
                                                     const double2* __restrict__ x, const double* __restrict__ y,
                                                     int64_t incy, double* __restrict__ a, int64_t cs_a)
{
    for (int64_t j0 = (int64_t)blockIdx.x * GER_COLS; j0 < n; j0 += (int64_t)gridDim.x * GER_COLS) {
        const int jn = (n - j0 < GER_COLS) ? (int)(n - j0) : GER_COLS;
        double ay[GER_COLS];
#pragma unroll
        for (int q = 0; q < GER_COLS; ++q) ay[q] = (q < jn) ? alpha * y[(j0 + q) * incy] : 0.0;
        for (int64_t i = threadIdx.x; i < m2; i += NT) {
            const double2 xi = x[i];
#pragma unroll
            for (int q = 0; q < GER_COLS; ++q) {
                if (q < jn) {
                    double2* col = reinterpret_cast<double2*>(a + (j0 + q) * cs_a);
                    double2 v = __ldcs(col + i);
                    v.x = fma(ay[q], xi.x, v.x);
                    v.y = fma(ay[q], xi.y, v.y);
                    __stcs(col + i, v);
                }
            }
        }
    }
}

// Zero strides: the reference's loops apply every update to the one element
// in order, so one thread runs them in that order (column by column).
__global__ void ger_serial_kernel(int64_t m, int64_t n, double alpha, const double* __restrict__ x, int64_t incx,
                                  const double* __restrict__ y, int64_t incy, double* __restrict__ a, int64_t rs_a,
                                  int64_t cs_a)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int64_t j = 0; j < n; ++j) {
        const double ay = alpha * y[j * incy];
        for (int64_t i = 0; i < m; ++i) {
            double* aij = a + i * rs_a + j * cs_a;
            *aij = fma(ay, x[i * incx], *aij);
        }
    }
}

}  // namespace

int dscalv_dev(int64_t n, double alpha, double* x, int64_t incx, cudaStream_t s)
{
    if (n <= 0 || alpha == 1.0) return GB_SUCCESS;
    if (incx == 1 && aligned16(x)) {
        const int64_t n2 = n >> 1;
        if (n2 > 0) {
            LaunchScope ls("scalv_vec", s);
            scalv_vec_kernel<<<grid_n(n2), NT, 0, s>>>(n2, alpha, reinterpret_cast<double2*>(x));
        }
        if (n & 1) {
            LaunchScope ls("scalv_tail", s);
            scalv_strided_kernel<<<1, NT, 0, s>>>(1, alpha, x + n - 1, 1);
        }
    } else {
        LaunchScope ls("scalv_strided", s);
        scalv_strided_kernel<<<grid_n(n), NT, 0, s>>>(n, alpha, x, incx);
    }
    return check_cuda(cudaGetLastError(), "dscalv");
}

int dcopyv_dev(int64_t n, const double* x, int64_t incx, double* y, int64_t incy, cudaStream_t s)
{
    if (n <= 0) return GB_SUCCESS;
    if (incx == 1 && incy == 1)
        return check_cuda(cudaMemcpyAsync(y, x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s), "dcopyv");
    LaunchScope ls("copyv_strided", s);
    copyv_strided_kernel<<<grid_n(n), NT, 0, s>>>(n, x, incx, y, incy);
    return check_cuda(cudaGetLastError(), "dcopyv");
}

int damaxv_dev(int64_t n, const double* x, int64_t incx, int64_t* index_dev, cudaStream_t s)
{
    if (n <= 0) return check_cuda(cudaMemsetAsync(index_dev, 0, sizeof(int64_t), s), "damaxv");
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t parts = (n + 4095) / 4096;
    if (parts > (int64_t)sms * 8) parts = (int64_t)sms * 8;
    const int64_t chunk = (n + parts - 1) / parts;
    parts = (n + chunk - 1) / chunk;
    uint8_t* ws = static_cast<uint8_t*>(dev_alloc((size_t)parts * 16 + 64, s));
    if (!ws) return GB_ERR_NOMEM;
    unsigned long long* pk = reinterpret_cast<unsigned long long*>(ws);
    int64_t* pi = reinterpret_cast<int64_t*>(ws + (size_t)parts * 8);
    {
        LaunchScope ls("amaxv_partial", s);
        amaxv_partial_kernel<<<(unsigned)parts, NT, 0, s>>>(n, chunk, x, incx, pk, pi);
    }
    {
        LaunchScope ls("amaxv_final", s);
        amaxv_final_kernel<<<1, NT, 0, s>>>((int)parts, pk, pi, index_dev);
    }
    const int rc = check_cuda(cudaGetLastError(), "damaxv");
    dev_free(ws, s);
    return rc;
}

int dger_dev(int64_t m, int64_t n, double alpha, const double* x, int64_t incx, const double* y, int64_t incy,
             double* a, int64_t rs_a, int64_t cs_a, cudaStream_t s)
{
    if (m <= 0 || n <= 0 || alpha == 0.0) return GB_SUCCESS;
    if (incx == 0 || incy == 0 || rs_a == 0 || cs_a == 0) {
        LaunchScope ls("ger_serial", s);
        ger_serial_kernel<<<1, 32, 0, s>>>(m, n, alpha, x, incx, y, incy, a, rs_a, cs_a);
        return check_cuda(cudaGetLastError(), "dger");
    }
    // rows along threads: for a row-major A walk the transposed problem instead
    if (rs_a != 1 && cs_a == 1) return dger_dev(n, m, alpha, y, incy, x, incx, a, cs_a, rs_a, s);
    if (rs_a == 1 && incx == 1 && (m & 1) == 0 && (cs_a & 1) == 0 && aligned16(a) && aligned16(x)) {
        const int sms = sm_count() > 0 ? sm_count() : 148;
        int64_t g = (n + GER_COLS - 1) / GER_COLS;
        if (g > (int64_t)sms * 8) g = (int64_t)sms * 8;
        LaunchScope ls("ger_vec", s);
        ger_vec_kernel<<<(unsigned)g, NT, 0, s>>>(m >> 1, n, alpha, reinterpret_cast<const double2*>(x), y, incy, a,
                                                  cs_a);
        return check_cuda(cudaGetLastError(), "dger");
    }
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t gx = (m + NT - 1) / NT;
    if (gx > 64) gx = 64;
    int64_t gy = ((int64_t)sms * 8 + gx - 1) / gx;
    const int64_t cols = (n + GER_COLS - 1) / GER_COLS;
    if (gy > cols) gy = cols;
    if (gy > 65535) gy = 65535;
    LaunchScope ls("ger", s);
    ger_kernel<<<dim3((unsigned)gx, (unsigned)gy), NT, 0, s>>>(m, n, alpha, x, incx, y, incy, a, rs_a, cs_a);
    return check_cuda(cudaGetLastError(), "dger");
}

int dtrsv_dev(int uplo, int transa, int diag, int64_t m, double alpha, const double* a, int64_t rs_a, int64_t cs_a,
              double* x, int64_t incx, cudaStream_t s)
{
    // one right-hand side: B is x as an m x 1 matrix with row stride incx
    return dtrsm_dev(GB_LEFT, uplo, transa, diag, m, 1, alpha, a, rs_a, cs_a, x, incx, 1, 0, s);
}

}  // namespace gb
