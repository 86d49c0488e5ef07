// gb_trsm.cu -- triangular solve with multiple right-hand sides for sm_103a
// (bli_trsm_ex, frame/3/bli_l3_oapi_ex.c:692-801).
//
// The reference's blocked variant (frame/3/trsm/bli_trsm_blk_var1.c:37-189)
// solves a KC x KC diagonal block, then updates the rest of B with gemm;
// its macro-kernel walks MR-row panels serially (bli_trsm_ll_ker_var2.c).
// On a GPU the serial part must stay small, so the solve is recursive:
//     X1 = inv(L11) B1;  B2 -= L21 X1;  X2 = inv(L22) B2
// down to diagonal blocks of at most 64 rows, which one kernel solves by
// right-looking substitution in registers with 1 to 8 lanes per right-hand
// side (FP64, diagonal pre-inverted as with BLIS_ENABLE_TRSM_PREINVERSION,
// ref_kernels/3/bli_trsm_ref.c:110-134).
// Nearly all m^2 n flops land in the off-diagonal gemm updates, which run
// on the native FP64 kernel or, in the precision form, on the Ozaki kernel.
// Right-side solves are turned into left-side ones by swapping B's strides
// and transposing A, the reduction of frame/3/bli_l3_oapi_ex.c:753-758.
// In the precision form with at least 2048 right-hand sides the two column
// halves recurse on two streams.  A single right-hand side (trsv, or trsm
// with one column) is one launch of the flag-ordered kernel below instead
// of the recursion.
#include <stdlib.h>

#include <vector>

#include "gb_internal.h"

namespace gb {
namespace {

constexpr int TRSM_NB = 64;
constexpr int64_t TRSM_SPLIT_MIN_COLS = 1024;  // columns per half for the two-stream precision form

// Every diagonal block of op(A) in the form the solves read, packed once per
// call: block q (rows and columns 64q .. 64q + nb - 1) becomes a row-major
// 64 x 64 array P with P[r][r] = inv(a_rr) (1 for a unit diagonal and for
// the identity rows that pad a short last block), P[r][i] = a_ri inv(a_ii)
// inside the strict triangle and 0 elsewhere.  The scaling lets the solve
// work on y = D X (D = diag(a)) with a unit triangle; see trsm_diag_kernel.
// E is double, or float for strsm.
template <typename E, bool LOWER>
__global__ void __launch_bounds__(256) trsm_pack_diag_kernel(int64_t m, int unit, const E* __restrict__ a,
                                                             int64_t ars, int64_t acs, E* __restrict__ packed)
{
    __shared__ E Tb[TRSM_NB][TRSM_NB + 1];
    __shared__ E dinv[TRSM_NB];
    const int64_t r0 = (int64_t)blockIdx.x * TRSM_NB;
    const int nb = (m - r0 < TRSM_NB) ? (int)(m - r0) : TRSM_NB;
    const E* blk = a + r0 * ars + r0 * acs;
    const bool rows_fast = (ars == 1);
    for (int e = threadIdx.x; e < TRSM_NB * TRSM_NB; e += 256) {
        const int i = rows_fast ? e % TRSM_NB : e / TRSM_NB, l = rows_fast ? e / TRSM_NB : e % TRSM_NB;
        const bool keep = (i < nb && l < nb) && (LOWER ? (l <= i) : (l >= i));
        Tb[i][l] = keep ? blk[i * ars + l * acs] : E(0);
    }
    __syncthreads();
    if (threadIdx.x < TRSM_NB) {
        const int i = threadIdx.x;
        dinv[i] = (unit || i >= nb) ? E(1) : E(1) / Tb[i][i];
    }
    __syncthreads();
    E* out = packed + (int64_t)blockIdx.x * TRSM_NB * TRSM_NB;
    for (int e = threadIdx.x; e < TRSM_NB * TRSM_NB; e += 256) {
        const int r = e / TRSM_NB, i = e % TRSM_NB;
        E v = E(0);
        if (r == i) v = dinv[r];
        else if (LOWER ? (i < r) : (i > r)) v = Tb[r][i] * dinv[i];
        out[e] = v;
    }
}

// Solves op(A11) X = B1 in place for one diagonal block, from its packed form
// P; B(i, j) = b[i*brs + j*bcs], rows of B past nb are neither read nor
// written.  A CTA of TRSM_THREADS threads owns TRSM_THREADS / LANES
// right-hand sides: P and the CTA's panel of B are staged in shared memory
// (coalesced along B's contiguous direction), then each lane holds
// 64 / LANES rows of its column in registers (row r = q * LANES + g in x[q]
// of lane g) and runs right-looking substitution on y = D X with the unit
// triangle of P: y_i is final once the rows before it have been applied; the
// lane that owns row i shuffles it to the column's other lanes, which do
// y_r -= P[r][i] y_i for every later row r; at the end x_r = y_r inv(a_rr)
// (pre-inverted diagonal, as the reference's trsm kernels use).  Every FP64
// instruction of the substitution is an FMA of the triangle, so the FP64
// pipe (GB300's narrowest) does no reduction work and each row's dependent
// chain is one FMA and one shuffle.  LANES trades issue slots (the FMA of a
// group of LANES rows is one warp instruction however few of its rows are
// left) against how many warps there are to fill the SM sub-partitions.  Both
// loops are unrolled, so every register index is a constant.
constexpr int TRSM_THREADS = 128;

template <typename E, int LANES, bool LOWER>
__global__ void __launch_bounds__(TRSM_THREADS) trsm_diag_kernel(int nb, const E* __restrict__ pk,
                                                                 E* __restrict__ b, int64_t brs, int64_t bcs,
                                                                 int64_t ncols)
{
    constexpr int COLS = TRSM_THREADS / LANES, R = TRSM_NB / LANES, LL = TRSM_NB + 1, LX = COLS + 1;
    extern __shared__ __align__(16) unsigned char trsm_smem[];
    E* L = reinterpret_cast<E*>(trsm_smem);  // [TRSM_NB][LL]
    E* X = L + TRSM_NB * LL;                 // [TRSM_NB][LX]
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * COLS;
    const int cols = (ncols - j0 < COLS) ? (int)(ncols - j0) : COLS;
#pragma unroll 8
    for (int e = t; e < TRSM_NB * TRSM_NB; e += TRSM_THREADS) L[(e / TRSM_NB) * LL + e % TRSM_NB] = pk[e];
    const bool rows_fast = (brs == 1);
#pragma unroll 8
    for (int e = t; e < TRSM_NB * COLS; e += TRSM_THREADS) {
        const int i = rows_fast ? e % TRSM_NB : e / COLS, c = rows_fast ? e / TRSM_NB : e % COLS;
        X[i * LX + c] = (c < cols && i < nb) ? b[i * brs + (j0 + c) * bcs] : E(0);
    }
    __syncthreads();
    const int c = t / LANES, g = t % LANES;  // the lanes of a column share a warp
    const int src0 = (t % 32) - g;           // the column's first lane within the warp
    E x[R];
#pragma unroll
    for (int q = 0; q < R; ++q) x[q] = X[(q * LANES + g) * LX + c];
#pragma unroll
    for (int step = 0; step < TRSM_NB; ++step) {
        const int i = LOWER ? step : TRSM_NB - 1 - step;
        const int qi = i / LANES, gi = i % LANES;
        E v = x[qi];
        if constexpr (LANES > 1) v = __shfl_sync(0xffffffffu, v, src0 + gi);
#pragma unroll
        for (int q = 0; q < R; ++q) {
            // rows q * LANES .. q * LANES + LANES - 1 of this q; skip the q no lane needs
            if (LOWER ? (q * LANES + LANES - 1 > i) : (q * LANES < i)) {
                const int r = q * LANES + g;
                if (LOWER ? (r > i) : (r < i)) x[q] = fma(-L[r * LL + i], v, x[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const int r = q * LANES + g;
        X[r * LX + c] = x[q] * L[r * LL + r];
    }
    __syncthreads();
#pragma unroll 8
    for (int e = t; e < TRSM_NB * COLS; e += TRSM_THREADS) {
        const int i = rows_fast ? e % TRSM_NB : e / COLS, cc = rows_fast ? e / TRSM_NB : e % COLS;
        if (cc < cols && i < nb) b[i * brs + (j0 + cc) * bcs] = X[i * LX + cc];
    }
}

template <typename E>
constexpr size_t trsm_smem_bytes(int lanes)
{
    return sizeof(E) * (TRSM_NB * (TRSM_NB + 1) + TRSM_NB * (TRSM_THREADS / lanes + 1));
}

template <typename E, int LANES, bool LOWER>
int launch_trsm_diag(int nb, const E* pk, E* b, int64_t brs, int64_t bcs, int64_t ncols, cudaStream_t s)
{
    static bool attr = false;
    if (!attr) {
        const int rc = check_cuda(cudaFuncSetAttribute(trsm_diag_kernel<E, LANES, LOWER>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)trsm_smem_bytes<E>(LANES)), "trsm smem attr");
        if (rc) return rc;
        attr = true;
    }
    const int64_t blocks = (ncols + TRSM_THREADS / LANES - 1) / (TRSM_THREADS / LANES);
    if (blocks > INT32_MAX) return set_error(GB_ERR_ARG, "trsm", "too many right-hand sides");
    trsm_diag_kernel<E, LANES, LOWER><<<(unsigned)blocks, TRSM_THREADS, trsm_smem_bytes<E>(LANES), s>>>(
        nb, pk, b, brs, bcs, ncols);
    return check_cuda(cudaGetLastError(), "trsm_diag");
}

// Multiply-adds below which a TRSM update runs natively in the precision form
// (GB_TRSM_OZAKI_MIN_FMA; default 0: measured on GB300, even the 64 x n x 64
// updates at the bottom of the recursion are faster in the Ozaki form).
double trsm_ozaki_min_fma()
{
    static double v = -1.0;
    if (v < 0.0) {
        const char* e = getenv("GB_TRSM_OZAKI_MIN_FMA");
        v = e ? atof(e) : 0.0;
        if (v < 0.0) v = 0.0;
    }
    return v;
}

struct TrsmCtx {
    int lower, unit, slices;
    const double* packed;  // the diagonal blocks, trsm_pack_diag_kernel's layout
    const double* a;
    int64_t ars, acs;
    double* b;
    int64_t brs, bcs;
    int64_t n;
    cudaStream_t s;
    const TrsmImages* img = nullptr;  // digit images of the fused updates' A blocks
};

bool trsm_fused_enabled()
{
    // GB_TRSM_FUSED=0 turns the fused small updates off (read per call)
    const char* fz = getenv("GB_TRSM_FUSED");
    return !(fz && fz[0] == '0');
}

// ---------------------------------------------------------------- trsv
// One right-hand side in ONE launch.  CTA i (in the order of an atomic
// ticket, so every block it waits for belongs to a CTA that is already
// running or done) owns the 64-row block solved i-th: it accumulates op(A)'s
// off-diagonal blocks times each earlier block of x as soon as that block's
// flag is set, then solves its diagonal block in one warp (reciprocals of the
// diagonal, as the packed trsm blocks) and publishes its x block with a
// release flag.  Every wait is bounded: on timeout (or an abort set by
// another CTA) the CTA reports DEV_WAIT_TIMEOUT, sets the abort flag and
// returns.
constexpr int SV_NB = 64;
constexpr int SV_THREADS = 256;

struct TrsvArgs {
    int64_t m, nblk;
    const double* a;
    int64_t ars, acs;  // op(A) (i, j) at a[i*ars + j*acs]
    double* x;
    int64_t incx;
    double alpha;
    int unit;
    int* flags;   // flags[b] = 1 once block b of x is final
    int* ticket;  // next solve position
    int* abort;   // set by a CTA that gave up
    unsigned int* status;
    unsigned long long wait_ns;  // budget of each flag wait
    int64_t withhold;            // block whose flag is never published (failure-detection test), -1 none
};

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t sv_clock()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ROWMAJOR: op(A) rows contiguous (acs == 1): a warp's lanes run along the
// columns; otherwise (ars == 1 or general) the threads run along the rows.
template <bool LOWER, bool ROWMAJOR>
__global__ void __launch_bounds__(SV_THREADS) trsv_flags_kernel(const TrsvArgs p)
{
    __shared__ double T[SV_NB][SV_NB + 1];
    __shared__ double part[SV_THREADS / SV_NB][SV_NB];
    __shared__ double xs[SV_NB];
    __shared__ double dinv[SV_NB];
    __shared__ int s_pos, s_fail;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_pos = atomicAdd(p.ticket, 1);
        s_fail = 0;
    }
    __syncthreads();
    const int64_t pos = s_pos;
    if (pos >= p.nblk) return;  // the grid has exactly nblk CTAs
    const int64_t blk = LOWER ? pos : p.nblk - 1 - pos;
    const int64_t r0 = blk * SV_NB;
    const int nb = (p.m - r0 < SV_NB) ? (int)(p.m - r0) : SV_NB;
    // the diagonal block and this block's right-hand side (no other CTA writes it)
    for (int e = tid; e < SV_NB * SV_NB; e += SV_THREADS) {
        const int i = ROWMAJOR ? e / SV_NB : e % SV_NB, k = ROWMAJOR ? e % SV_NB : e / SV_NB;
        T[i][k] = (i < nb && k < nb) ? p.a[(r0 + i) * p.ars + (r0 + k) * p.acs] : 0.0;
    }
    for (int r = tid; r < SV_NB * (SV_THREADS / SV_NB); r += SV_THREADS) (&part[0][0])[r] = 0.0;
    __syncthreads();
    // off the critical path, before any wait: the reciprocal diagonal and the
    // rows of the triangle scaled by it (a unit triangle for y = D^-1 rhs)
    if (tid < SV_NB) dinv[tid] = (tid < nb && !p.unit) ? 1.0 / T[tid][tid] : 1.0;
    __syncthreads();
    if (!p.unit)
        for (int e = tid; e < SV_NB * SV_NB; e += SV_THREADS) {
            const int i = e / SV_NB, k = e % SV_NB;
            if (LOWER ? k < i : k > i) T[i][k] *= dinv[i];
        }
    double acc[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[u] = 0.0;
    const int rr = tid % SV_NB, q = tid / SV_NB;  // row-running mapping
    for (int64_t s = 0; s < pos; ++s) {
        const int64_t j = LOWER ? s : p.nblk - 1 - s;
        const int64_t c0 = j * SV_NB;
        if (tid == 0) {
            const uint64_t t0 = sv_clock();
            while (!ld_acquire(p.flags + j)) {
                if (*(volatile int*)p.abort || sv_clock() - t0 > p.wait_ns) {
                    atomicOr(p.status, DEV_WAIT_TIMEOUT);
                    atomicExch(p.abort, 1);
                    s_fail = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __syncthreads();
        if (s_fail) return;
        // columns of block j inside the matrix (the last block may be partial:
        // it is the first one an upper solve reads)
        const int ncol = (p.m - c0 < SV_NB) ? (int)(p.m - c0) : SV_NB;
        if (tid < SV_NB) xs[tid] = (tid < ncol) ? __ldcg(p.x + (c0 + tid) * p.incx) : 0.0;
        __syncthreads();
        if (ROWMAJOR) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t row = r0 + warp * 8 + u;
                if (warp * 8 + u < nb) {
                    const double* ar = p.a + row * p.ars + c0 * p.acs;
                    if (lane < ncol) acc[u] = fma(ar[lane * p.acs], xs[lane], acc[u]);
                    if (lane + 32 < ncol) acc[u] = fma(ar[(lane + 32) * p.acs], xs[lane + 32], acc[u]);
                }
            }
        } else if (rr < nb) {
            const double* ar = p.a + (r0 + rr) * p.ars + c0 * p.acs;
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int c = q + 4 * u;
                if (c < ncol) acc[u & 7] = fma(ar[c * p.acs], xs[c], acc[u & 7]);
            }
        }
    }
    if (ROWMAJOR) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            double v = acc[u];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) part[0][warp * 8 + u] = v;
        }
    } else {
        double v = 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) v += acc[u];
        part[q][rr] = v;
    }
    __syncthreads();
    if (warp == 0) {
        // rows lane and lane + 32; y = alpha b - (off-diagonal sums), then substitution
        const int ra = lane, rb = lane + 32;
        double y0 = 0.0, y1 = 0.0;
        if (ra < nb)
            y0 = dinv[ra] * (p.alpha * p.x[(r0 + ra) * p.incx] -
                             (((part[0][ra] + part[1][ra]) + part[2][ra]) + part[3][ra]));
        if (rb < nb)
            y1 = dinv[rb] * (p.alpha * p.x[(r0 + rb) * p.incx] -
                             (((part[0][rb] + part[1][rb]) + part[2][rb]) + part[3][rb]));
        // y = D^-1 rhs against the unit triangle: x_i is y_i once the rows
        // before it are applied; a half whose rows are all final is skipped
        // by the whole warp
        for (int step = 0; step < nb; ++step) {
            const int i = LOWER ? step : nb - 1 - step;
            const bool high = (i >= 32);
            const double xi = __shfl_sync(0xffffffffu, high ? y1 : y0, i & 31);
            if (LOWER ? !high : true) {
                if (ra < nb && (LOWER ? ra > i : ra < i)) y0 = fma(-T[ra][i], xi, y0);
            }
            if (LOWER ? true : high) {
                if (rb < nb && (LOWER ? rb > i : rb < i)) y1 = fma(-T[rb][i], xi, y1);
            }
        }
        if (ra < nb) p.x[(r0 + ra) * p.incx] = y0;
        if (rb < nb) p.x[(r0 + rb) * p.incx] = y1;
        __threadfence();
        __syncwarp();
        if (lane == 0 && blk != p.withhold) st_release(p.flags + blk, 1);
    }
}

int launch_trsv(bool lower, bool unit, int64_t m, double alpha, const double* a, int64_t ars, int64_t acs, double* x,
                int64_t incx, cudaStream_t s)
{
    const int64_t nblk = (m + SV_NB - 1) / SV_NB;
    if (nblk > INT32_MAX / 2) return set_error(GB_ERR_ARG, "dtrsv", "too many blocks");
    int* ws = static_cast<int*>(dev_alloc(sizeof(int) * (size_t)(nblk + 2), s));
    if (!ws) return GB_ERR_NOMEM;
    int rc = check_cuda(cudaMemsetAsync(ws, 0, sizeof(int) * (size_t)(nblk + 2), s), "trsv flags");
    if (!rc) {
        TrsvArgs p;
        p.m = m;
        p.nblk = nblk;
        p.a = a;
        p.ars = ars;
        p.acs = acs;
        p.x = x;
        p.incx = incx;
        p.alpha = alpha;
        p.unit = unit ? 1 : 0;
        p.flags = ws;
        p.ticket = ws + nblk;
        p.abort = ws + nblk + 1;
        p.status = device_status_word();
        p.wait_ns = trsv_wait_budget_ns();
        p.withhold = trsv_withheld_block();
        const bool rowmajor = (acs == 1 && ars != 1);
        LaunchScope ls("trsv_flags", s);
        if (lower)
            rowmajor ? trsv_flags_kernel<true, true><<<(unsigned)nblk, SV_THREADS, 0, s>>>(p)
                     : trsv_flags_kernel<true, false><<<(unsigned)nblk, SV_THREADS, 0, s>>>(p);
        else
            rowmajor ? trsv_flags_kernel<false, true><<<(unsigned)nblk, SV_THREADS, 0, s>>>(p)
                     : trsv_flags_kernel<false, false><<<(unsigned)nblk, SV_THREADS, 0, s>>>(p);
        rc = check_cuda(cudaGetLastError(), "trsv_flags");
    }
    dev_free(ws, s);
    return rc;
}

// Depth (k) from which a precision-form TRSM update runs in the CRT form, at the
// moduli that carry the digit form's precision (GB_TRSM_CRT_MIN_K; 0 never): its
// 16 or so products against the digit form's s(s+1)/2 pay for the wider split and
// recombination only on the deep updates at the top of the recursion.
int64_t trsm_crt_min_k()
{
    static int64_t v = -1;
    if (v < 0) {
        const char* e = getenv("GB_TRSM_CRT_MIN_K");
        v = e ? atoll(e) : 2048;
        if (v < 0) v = 0;
    }
    return v;
}

int update(const TrsmCtx& t, int64_t r0, int64_t rcount, int64_t c0, int64_t ccount)
{
    // B[r0:r0+rcount, :] -= op(A)[r0:.., c0:c0+ccount] * X[c0:c0+ccount, :]
    const double* ap = t.a + r0 * t.ars + c0 * t.acs;
    const double* xp = t.b + c0 * t.brs;
    double* bp = t.b + r0 * t.brs;
    if (t.slices > 0 && (double)rcount * (double)ccount * (double)t.n >= trsm_ozaki_min_fma()) {
        // the small updates at the bottom of the recursion: one fused launch, reading the
        // digit image of the A block built for the solve when there is one
        if (trsm_fused_enabled() && trsm_update_fused_fits(t.slices, rcount, ccount, t.n)) {
            const uint8_t* aimg = nullptr;
            const int* aexp = nullptr;
            if (t.img && t.img->slices == t.slices) {
                auto it = t.img->index.find(((uint64_t)r0 << 32) | (uint64_t)c0);
                if (it != t.img->index.end()) {
                    aimg = it->second.first;
                    aexp = it->second.second;
                }
            }
            return trsm_update_fused(t.slices, rcount, ccount, t.n, ap, t.ars, t.acs, xp, t.brs, t.bcs, bp, t.brs,
                                     t.bcs, t.s, aimg, aexp);
        }
        const int64_t kc = trsm_crt_min_k();
        const int moduli = (kc > 0 && ccount >= kc) ? ozaki_crt_moduli_for_bits(8 * t.slices - 1, ccount) : -1;
        if (moduli > 0) {
            ModeOverride crt(GB_DGEMM_OZAKI, moduli, 1);
            return dgemm_ozaki(rcount, t.n, ccount, -1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp, t.brs,
                               t.bcs, moduli, t.s);
        }
        return dgemm_ozaki(rcount, t.n, ccount, -1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp,
                           t.brs, t.bcs, t.slices, t.s);
    }
    return dgemm_native(rcount, t.n, ccount, -1.0, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0, bp,
                        t.brs, t.bcs, t.s);
}

// Whether the update of `rows` rows at depth k and the diagonal solve of those rows run as one
// fused launch (the precision form's fused updates; GB_TRSM_GEMMTRSM=0 keeps them apart).
bool gemmtrsm_applies(const TrsmCtx& t, int64_t rows, int64_t k)
{
    const char* e = getenv("GB_TRSM_GEMMTRSM");
    return !(e && e[0] == '0') && t.slices > 0 && trsm_fused_enabled() && rows <= TRSM_NB &&
           (double)rows * (double)k * (double)t.n >= trsm_ozaki_min_fma() &&
           trsm_update_fused_fits(t.slices, rows, k, t.n);
}

// B[r0:r0+rows] := solve(diagonal block at r0, B[r0:r0+rows] - op(A)[r0.., c0..c0+k] X[c0..c0+k]):
// the fused update followed, in the same launch, by the diagonal block's substitution.
int gemmtrsm(const TrsmCtx& t, int64_t r0, int64_t rows, int64_t c0, int64_t k)
{
    const double* ap = t.a + r0 * t.ars + c0 * t.acs;
    const double* xp = t.b + c0 * t.brs;
    double* bp = t.b + r0 * t.brs;
    const uint8_t* aimg = nullptr;
    const int* aexp = nullptr;
    if (t.img && t.img->slices == t.slices) {
        auto it = t.img->index.find(((uint64_t)r0 << 32) | (uint64_t)c0);
        if (it != t.img->index.end()) {
            aimg = it->second.first;
            aexp = it->second.second;
        }
    }
    // r0 is a multiple of the block size: the split in solve keeps it so
    const double* pk = t.packed + (r0 / TRSM_NB) * TRSM_NB * TRSM_NB;
    return trsm_update_fused(t.slices, rows, k, t.n, ap, t.ars, t.acs, xp, t.brs, t.bcs, bp, t.brs, t.bcs, t.s, aimg,
                             aexp, pk, t.lower);
}

int diag_solve(const TrsmCtx& t, int64_t r0, int64_t mm)
{
    // r0 is a multiple of the block size: the split in solve keeps it so
    const double* pk = t.packed + (r0 / TRSM_NB) * TRSM_NB * TRSM_NB;
    double* b1 = t.b + r0 * t.brs;
    const int nb = (int)mm;
    LaunchScope ls("trsm_diag", t.s);
    switch (diag_block_lanes(t.n)) {
    case 1:
        return t.lower ? launch_trsm_diag<double, 1, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<double, 1, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    case 2:
        return t.lower ? launch_trsm_diag<double, 2, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<double, 2, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    case 4:
        return t.lower ? launch_trsm_diag<double, 4, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<double, 4, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    default:
        return t.lower ? launch_trsm_diag<double, 8, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<double, 8, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    }
}

// The recursion over rows for nt independent column groups of B (each with
// its own stream), issued step by step in turn so that the groups' launches
// interleave on the device.
int solve(const TrsmCtx* ts, int nt, int64_t r0, int64_t mm)
{
    int rc;
    if (mm <= TRSM_NB) {
        for (int g = 0; g < nt; ++g)
            if ((rc = diag_solve(ts[g], r0, mm))) return rc;
        return GB_SUCCESS;
    }
    // split on a multiple of the diagonal block size
    int64_t m1 = ((mm / 2 + TRSM_NB - 1) / TRSM_NB) * TRSM_NB;
    if (m1 >= mm) m1 = mm - TRSM_NB;
    const int64_t m2 = mm - m1;
    if (ts[0].lower) {
        if ((rc = solve(ts, nt, r0, m1))) return rc;
        // the last diagonal block and the update before it in one fused launch
        if (m2 <= TRSM_NB && gemmtrsm_applies(ts[0], m2, m1)) {
            for (int g = 0; g < nt; ++g)
                if ((rc = gemmtrsm(ts[g], r0 + m1, m2, r0, m1))) return rc;
            return GB_SUCCESS;
        }
        for (int g = 0; g < nt; ++g)
            if ((rc = update(ts[g], r0 + m1, m2, r0, m1))) return rc;
        return solve(ts, nt, r0 + m1, m2);
    }
    if ((rc = solve(ts, nt, r0 + m1, m2))) return rc;
    if (m1 <= TRSM_NB && gemmtrsm_applies(ts[0], m1, m2)) {
        for (int g = 0; g < nt; ++g)
            if ((rc = gemmtrsm(ts[g], r0, m1, r0 + m1, m2))) return rc;
        return GB_SUCCESS;
    }
    for (int g = 0; g < nt; ++g)
        if ((rc = update(ts[g], r0, m1, r0 + m1, m2))) return rc;
    return solve(ts, nt, r0, m1);
}

// The updates of the recursion (solve's splitting rule) whose A block the fused
// kernel takes: (r0, c0, rows, k) of op(A).
void fused_update_blocks(bool lower, int64_t r0, int64_t mm, int slices, int64_t n, std::vector<TrsmImgSpec>& out)
{
    if (mm <= TRSM_NB) return;
    int64_t m1 = ((mm / 2 + TRSM_NB - 1) / TRSM_NB) * TRSM_NB;
    if (m1 >= mm) m1 = mm - TRSM_NB;
    const int64_t m2 = mm - m1;
    const TrsmImgSpec u = lower ? TrsmImgSpec{r0 + m1, r0, m2, m1} : TrsmImgSpec{r0, r0 + m1, m1, m2};
    fused_update_blocks(lower, lower ? r0 : r0 + m1, lower ? m1 : m2, slices, n, out);
    if (trsm_update_fused_fits(slices, u.rows, u.k, n)) out.push_back(u);
    fused_update_blocks(lower, lower ? r0 + m1 : r0, lower ? m2 : m1, slices, n, out);
}

}  // namespace

// Lanes per right-hand side for the diagonal kernel (GB_TRSM_DIAG_LANES =
// 1, 2, 4 or 8 fixes it).  Each warp issues one FMA per step for every group
// of LANES rows that has a row left to update, 64R - LANES R (R - 1) / 2 - R
// instructions (R = 64 / LANES rows per lane), and R multiplies: 2080, 1056,
// 544, 288 for 1, 2, 4, 8 lanes, for 32 / LANES columns; staging the packed
// block and the panel costs about as much as 96 more.  GB300's FP64 pipe
// takes tens of cycles per warp instruction on each of an SM's four
// sub-partitions, so the solve time is about one warp's cost times the warps
// that share a sub-partition (CTAs of four warps: ceil(CTAs / SMs) on the
// busiest SM), but no less than four of them: below that the dependent chain
// of each row, not the pipe, sets the time.  The constants were fitted to
// solves of 2048 to 16384 right-hand sides timed on GB300.  The fewest lanes
// win near-ties.
int diag_block_lanes(int64_t ncols)
{
    static int forced = -1;
    if (forced < 0) {
        const char* e = getenv("GB_TRSM_DIAG_LANES");
        const int v = e ? atoi(e) : 0;
        forced = (v == 1 || v == 2 || v == 4 || v == 8) ? v : 0;
    }
    if (forced) return forced;
    const int64_t sms = sm_count() > 0 ? sm_count() : 148;
    int best = 1;
    int64_t best_cost = 0;
    for (int lanes = 1; lanes <= 8; lanes *= 2) {
        const int64_t r = TRSM_NB / lanes;
        const int64_t per_warp = 64 * r - lanes * r * (r - 1) / 2 + 96;
        const int64_t ctas = (ncols + TRSM_THREADS / lanes - 1) / (TRSM_THREADS / lanes);
        const int64_t waves = (ctas + sms - 1) / sms;
        const int64_t cost = per_warp * (waves > 4 ? waves : 4);
        if (lanes == 1 || cost * 50 < best_cost * 49) {
            best = lanes;
            best_cost = cost;
        }
    }
    return best;
}

int dtrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha,
              const double* a, int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b,
              int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    // the updates take the digit form, the deep ones the CRT form at the same precision
    // (update): measured on GB300, the CRT form's residue planes cost more to split and
    // recombine than its fewer products save on shallow updates (8192 x 4096: 13.8 ms with
    // every update in 7 digit slices, 19.5 ms with every update in 16 moduli)
    if (slices > 0 && ozaki_form() == 1) slices = ozaki_digit_slices();
    ModeOverride digits(dgemm_mode(), slices, 0);
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    if (side == GB_RIGHT) {
        brs = cs_b;
        bcs = rs_b;
        mm = n;
        nn = m;
        trans = !trans;
    }
    if (alpha == 0.0) return scal_matrix(mm, nn, 0.0, b, brs, bcs, s);
    if (nn == 1) {
        // one right-hand side (trsv): the flag-ordered single launch, alpha folded in
        const int64_t ars = trans ? cs_a : rs_a, acs = trans ? rs_a : cs_a;
        return launch_trsv((uplo == GB_LOWER) != trans, diag == GB_UNIT_DIAG, mm, alpha, a, ars, acs, b, brs, s);
    }
    if (alpha != 1.0) {
        int rc = scal_matrix(mm, nn, alpha, b, brs, bcs, s);
        if (rc) return rc;
    }
    TrsmCtx t;
    t.ars = trans ? cs_a : rs_a;
    t.acs = trans ? rs_a : cs_a;
    t.lower = ((uplo == GB_LOWER) != trans) ? 1 : 0;
    t.unit = (diag == GB_UNIT_DIAG) ? 1 : 0;
    t.slices = slices;
    t.a = a;
    t.b = b;
    t.brs = brs;
    t.bcs = bcs;
    t.n = nn;
    t.s = s;
    const int64_t nblk = (mm + TRSM_NB - 1) / TRSM_NB;
    if (nblk > INT32_MAX) return set_error(GB_ERR_ARG, "dtrsm", "too many diagonal blocks");
    double* packed = static_cast<double*>(dev_alloc(sizeof(double) * nblk * TRSM_NB * TRSM_NB, s));
    if (!packed) return GB_ERR_NOMEM;
    {
        LaunchScope ls("trsm_pack_diag", s);
        if (t.lower)
            trsm_pack_diag_kernel<double, true><<<(unsigned)nblk, 256, 0, s>>>(mm, t.unit, a, t.ars, t.acs, packed);
        else
            trsm_pack_diag_kernel<double, false><<<(unsigned)nblk, 256, 0, s>>>(mm, t.unit, a, t.ars, t.acs, packed);
    }
    int rc = check_cuda(cudaGetLastError(), "trsm_pack_diag");
    t.packed = packed;
    // the fused updates' A blocks split once for the solve (both column groups read them)
    TrsmImages images;
    const char* gi = getenv("GB_TRSM_IMAGES");  // 0: each fused update splits its A block itself
    if (!rc && slices > 0 && trsm_fused_enabled() && !(gi && gi[0] == '0') && trsm_ozaki_min_fma() == 0.0) {
        std::vector<TrsmImgSpec> specs;
        fused_update_blocks(t.lower != 0, 0, mm, slices, nn, specs);
        if (!specs.empty() &&
            trsm_images_build(slices, a, t.ars, t.acs, specs.data(), (int)specs.size(), &images, s) == GB_SUCCESS)
            t.img = &images;
        else
            cudaGetLastError();  // without images each fused update splits its A block itself
    }
    // the precision form's many small launches (split, slice GEMM, recombination
    // per update) and the FP64-pipe diagonal solves of G column groups overlap
    // on G streams (the caller's and G - 1 more of this thread), forked and
    // joined by events; if an event cannot be created the solve runs on one stream
    const char* gs = getenv("GB_TRSM_STREAMS");  // column groups: 1 .. 4 (default 2)
    int groups = gs ? atoi(gs) : 2;
    groups = groups < 1 ? 1 : (groups > 4 ? 4 : groups);
    while (groups > 1 && nn < (int64_t)groups * TRSM_SPLIT_MIN_COLS) --groups;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // fork, then the joins of groups 1..
    bool multi = !rc && slices > 0 && groups > 1 && mm > 4 * TRSM_NB;
    for (int g = 0; multi && g < groups; ++g)
        multi = cudaEventCreateWithFlags(&ev[g], cudaEventDisableTiming) == cudaSuccess;
    if (multi) {
        TrsmCtx ts[4] = {t, t, t, t};
        int64_t c0 = 0;
        for (int g = 0; g < groups; ++g) {
            const int64_t c1 = (g + 1 == groups) ? nn : ((nn * (g + 1) / groups) + 7) / 8 * 8;
            ts[g].n = c1 - c0;
            ts[g].b = b + c0 * bcs;
            if (g > 0) ts[g].s = thread_aux_stream(g - 1);
            c0 = c1;
        }
        rc = check_cuda(cudaEventRecord(ev[0], s), "trsm fork");
        for (int g = 1; g < groups && !rc; ++g) rc = check_cuda(cudaStreamWaitEvent(ts[g].s, ev[0], 0), "trsm fork");
        if (!rc) rc = solve(ts, groups, 0, mm);
        // the joins are recorded whatever happened, so s never runs ahead of the other streams' work
        for (int g = 1; g < groups; ++g) {
            cudaEventRecord(ev[g], ts[g].s);
            cudaStreamWaitEvent(s, ev[g], 0);
        }
    } else if (!rc) {
        cudaGetLastError();  // a failed event creation above is not this call's error
        rc = solve(&t, 1, 0, mm);
    }
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    trsm_images_release(&images, s);
    dev_free(packed, s);
    return rc;
}

// STRSM on the GPU (the native form only): the recursion of dtrsm_dev at FP32
// with the same packed diagonal blocks and diagonal-solve kernel, the updates
// B2 -= op(A21) X1 through sgemm's own engine choice (gb_set_sgemm_mode: the
// split form on the bf16 tensor cores for large updates, the FP32 FMA kernel
// below), on the caller's stream.
namespace {

struct STrsmCtx {
    const float* packed;
    const float* a;
    int64_t ars, acs;
    float* b;
    int64_t brs, bcs, n;
    bool lower;
    cudaStream_t s;
};

int s_diag_solve(const STrsmCtx& t, int64_t r0, int64_t mm)
{
    const float* pk = t.packed + (r0 / TRSM_NB) * TRSM_NB * TRSM_NB;
    float* b1 = t.b + r0 * t.brs;
    const int nb = (int)mm;
    LaunchScope ls("trsm_diag", t.s);
    switch (diag_block_lanes(t.n)) {
    case 1:
        return t.lower ? launch_trsm_diag<float, 1, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<float, 1, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    case 2:
        return t.lower ? launch_trsm_diag<float, 2, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<float, 2, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    case 4:
        return t.lower ? launch_trsm_diag<float, 4, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<float, 4, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    default:
        return t.lower ? launch_trsm_diag<float, 8, true>(nb, pk, b1, t.brs, t.bcs, t.n, t.s)
                       : launch_trsm_diag<float, 8, false>(nb, pk, b1, t.brs, t.bcs, t.n, t.s);
    }
}

int s_update(const STrsmCtx& t, int64_t r0, int64_t rcount, int64_t c0, int64_t ccount)
{
    // B[r0:r0+rcount, :] -= op(A)[r0:.., c0:c0+ccount] * X[c0:c0+ccount, :]
    const float* ap = t.a + r0 * t.ars + c0 * t.acs;
    const float* xp = t.b + c0 * t.brs;
    float* bp = t.b + r0 * t.brs;
    if (sgemm_use_split(rcount, t.n, ccount))
        return sgemm_split_dev(rcount, t.n, ccount, -1.0f, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0f, bp, t.brs,
                               t.bcs, t.s);
    return sgemm_dev(rcount, t.n, ccount, -1.0f, ap, t.ars, t.acs, xp, t.brs, t.bcs, 1.0f, bp, t.brs, t.bcs, t.s);
}

int s_solve(const STrsmCtx& t, int64_t r0, int64_t mm)
{
    if (mm <= TRSM_NB) return s_diag_solve(t, r0, mm);
    int64_t m1 = ((mm / 2 + TRSM_NB - 1) / TRSM_NB) * TRSM_NB;
    if (m1 >= mm) m1 = mm - TRSM_NB;
    const int64_t m2 = mm - m1;
    int rc;
    if (t.lower) {
        if ((rc = s_solve(t, r0, m1)) || (rc = s_update(t, r0 + m1, m2, r0, m1))) return rc;
        return s_solve(t, r0 + m1, m2);
    }
    if ((rc = s_solve(t, r0 + m1, m2)) || (rc = s_update(t, r0, m1, r0 + m1, m2))) return rc;
    return s_solve(t, r0, m1);
}

}  // namespace

int strsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, float alpha, const float* a,
              int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    bool trans = GB_IS_TRANS(transa);
    if (side == GB_RIGHT) {  // X op(A) = B  <=>  op(A)^T X^T = B^T
        brs = cs_b;
        bcs = rs_b;
        mm = n;
        nn = m;
        trans = !trans;
    }
    if (alpha == 0.0f) return scal_matrix_f(mm, nn, 0.0f, b, brs, bcs, s);
    int rc;
    if (alpha != 1.0f && (rc = scal_matrix_f(mm, nn, alpha, b, brs, bcs, s))) return rc;
    STrsmCtx t;
    t.ars = trans ? cs_a : rs_a;
    t.acs = trans ? rs_a : cs_a;
    t.lower = (uplo == GB_LOWER) != trans;
    t.a = a;
    t.b = b;
    t.brs = brs;
    t.bcs = bcs;
    t.n = nn;
    t.s = s;
    const int64_t nblk = (mm + TRSM_NB - 1) / TRSM_NB;
    if (nblk > INT32_MAX) return set_error(GB_ERR_ARG, "strsm", "too many diagonal blocks");
    float* packed = static_cast<float*>(dev_alloc(sizeof(float) * nblk * TRSM_NB * TRSM_NB, s));
    if (!packed) return GB_ERR_NOMEM;
    {
        LaunchScope ls("trsm_pack_diag", s);
        const int unit = (diag == GB_UNIT_DIAG) ? 1 : 0;
        if (t.lower)
            trsm_pack_diag_kernel<float, true><<<(unsigned)nblk, 256, 0, s>>>(mm, unit, a, t.ars, t.acs, packed);
        else
            trsm_pack_diag_kernel<float, false><<<(unsigned)nblk, 256, 0, s>>>(mm, unit, a, t.ars, t.acs, packed);
    }
    rc = check_cuda(cudaGetLastError(), "trsm_pack_diag");
    t.packed = packed;
    if (!rc) rc = s_solve(t, 0, mm);
    dev_free(packed, s);
    return rc;
}

}  // namespace gb
