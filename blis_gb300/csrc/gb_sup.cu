// gb_sup.cu -- small / skinny GEMM (the gemmsup path) and the
// configuration-explicit GEMM entry used by the autotuner and selector.
//
// BLIS sends problems with a dimension below its sup thresholds
// (frame/base/bli_cntx.h:186-193, MT/NT/KT = 201 on haswell) to unpacked
// kernels (frame/3/bli_l3_sup.c:37-131, bli_l3_sup_var1n2m.c) because the
// packing and the large MC/NC blocking of the conventional path do not pay
// off there.  On the GPU the analogous waste is idle SMs: a 300 x 300 C has
// only 9 tiles of 128 x 128.  This engine uses 64 x 64 tiles (4 warps) and an
// optional split of K across blockIdx.z; split partial sums go to a
// workspace and a second kernel folds them in fixed order, so results are
// deterministic.  The same config space covers FP64 (DMMA m8n8k4) and FP32
// (FMA):
//   config 0      the 128 x 128 engine of gb_dgemm.cu (BF16: the tcgen05
//                 kernel of gb_ozaki.cu)
//   config 1..5   64 x 64 tiles with a K split of 1, 2, 4, 8, 16 (BF16:
//                 bf16 loads, FP32 arithmetic)
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "gb_internal.h"

namespace gb {
namespace {

// Element loads widened to the arithmetic type.
template <typename T>
__device__ __forceinline__ T sup_ld(const T* p) { return __ldg(p); }
__device__ __forceinline__ float sup_ld(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }

constexpr int SBM = 64, SBN = 64, SBK = 16, SNT = 128;
constexpr int SLDS = SBM + 8;

// T: arithmetic and C; TI: the element type of A and B (T, or bf16 for T = float).
template <typename T, typename TI = T>
struct SupArgs {
    int64_t m, n, k, kchunk;
    T alpha, beta;
    const TI* a;
    int64_t ars, acs;
    const TI* b;
    int64_t brs, bcs;
    T* c;
    int64_t rs_c, cs_c;
    T* ws;  // split partial sums [split][n][m], or nullptr when not split
};

template <typename T, typename TI>
__device__ __forceinline__ void sup_load(const SupArgs<T, TI>& p, int64_t bm, int64_t bn, int64_t k0, int64_t k1,
                                         T (&ra)[8], T (&rb)[8])
{
    const int tid = threadIdx.x;
    const bool a_rows_fast = (p.ars == 1);
    const bool b_k_fast = (p.brs == 1);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int e = tid + SNT * r;
        int i, l;
        if (a_rows_fast) { i = e % SBM; l = e / SBM; } else { i = e / SBK; l = e % SBK; }
        const int64_t gi = bm + i, gl = k0 + l;
        ra[r] = (gi < p.m && gl < k1) ? sup_ld(p.a + gi * p.ars + gl * p.acs) : T(0);
        int j;
        if (b_k_fast) { l = e % SBK; j = e / SBK; } else { j = e % SBN; l = e / SBN; }
        const int64_t gj = bn + j, gl2 = k0 + l;
        rb[r] = (gj < p.n && gl2 < k1) ? sup_ld(p.b + gl2 * p.brs + gj * p.bcs) : T(0);
    }
}

template <typename T, typename TI>
__device__ __forceinline__ void sup_store(const SupArgs<T, TI>& p, T (&ra)[8], T (&rb)[8], T* As, T* Bs)
{
    const int tid = threadIdx.x;
    const bool a_rows_fast = (p.ars == 1);
    const bool b_k_fast = (p.brs == 1);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int e = tid + SNT * r;
        int i, l;
        if (a_rows_fast) { i = e % SBM; l = e / SBM; } else { i = e / SBK; l = e % SBK; }
        As[l * SLDS + i] = ra[r];
        int j;
        if (b_k_fast) { l = e % SBK; j = e / SBK; } else { j = e % SBN; l = e / SBN; }
        Bs[l * SLDS + j] = rb[r];
    }
}

template <typename T, typename TI>
__device__ __forceinline__ void sup_out(const SupArgs<T, TI>& p, int64_t i, int64_t j, T ab, int z)
{
    if (i >= p.m || j >= p.n) return;
    if (p.ws) {
        p.ws[((int64_t)z * p.n + j) * p.m + i] = ab;
    } else {
        T* cij = p.c + i * p.rs_c + j * p.cs_c;
        const T t = p.alpha * ab;
        *cij = (p.beta == T(0)) ? t : fma(p.beta, *cij, t);
    }
}

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

// One 64 x 64 tile of C (rows bm.., columns bn..) over the z-th k chunk.
// FP64: 2 x 2 warps of 32 x 32, DMMA.  FP32: 16 x 8 threads of 4 x 8, FMA.
template <typename T, typename TI>
__device__ __forceinline__ void sup_tile(const SupArgs<T, TI>& p, int64_t bm, int64_t bn, int z, T* As, T* Bs)
{
    const int64_t k0 = (int64_t)z * p.kchunk;
    const int64_t k1 = (k0 + p.kchunk < p.k) ? k0 + p.kchunk : p.k;
    T ra[8], rb[8];
    if constexpr (sizeof(T) == 8) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int wm = warp & 1, wn = warp >> 1;
        double acc[4][4][2];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
        sup_load(p, bm, bn, k0, k1, ra, rb);
        for (int64_t kk0 = k0; kk0 < k1; kk0 += SBK) {
            __syncthreads();
            sup_store(p, ra, rb, As, Bs);
            __syncthreads();
            if (kk0 + SBK < k1) sup_load(p, bm, bn, kk0 + SBK, k1, ra, rb);
#pragma unroll
            for (int kk = 0; kk < SBK; kk += 4) {
                const int kr = kk + (lane & 3);
                double af[4], bf[4];
#pragma unroll
                for (int mi = 0; mi < 4; ++mi) af[mi] = As[kr * SLDS + wm * 32 + mi * 8 + (lane >> 2)];
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) bf[ni] = Bs[kr * SLDS + wn * 32 + ni * 8 + (lane >> 2)];
#pragma unroll
                for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                    for (int ni = 0; ni < 4; ++ni) dmma(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
            }
        }
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                const int64_t i = bm + wm * 32 + mi * 8 + (lane >> 2);
                const int64_t j = bn + wn * 32 + ni * 8 + 2 * (lane & 3);
                sup_out(p, i, j, (T)acc[mi][ni][0], z);
                sup_out(p, i, j + 1, (T)acc[mi][ni][1], z);
            }
    } else {
        const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;  // 8 x 16 threads
        T acc[4][8];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = T(0);
        sup_load(p, bm, bn, k0, k1, ra, rb);
        for (int64_t kk0 = k0; kk0 < k1; kk0 += SBK) {
            __syncthreads();
            sup_store(p, ra, rb, As, Bs);
            __syncthreads();
            if (kk0 + SBK < k1) sup_load(p, bm, bn, kk0 + SBK, k1, ra, rb);
#pragma unroll
            for (int kk = 0; kk < SBK; ++kk) {
                T av[4], bv[8];
#pragma unroll
                for (int i = 0; i < 4; ++i) av[i] = As[kk * SLDS + ty * 4 + i];
#pragma unroll
                for (int j = 0; j < 8; ++j) bv[j] = Bs[kk * SLDS + tx * 8 + j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) sup_out(p, bm + ty * 4 + i, bn + tx * 8 + j, acc[i][j], z);
    }
}

template <typename T, typename TI>
__global__ void __launch_bounds__(SNT) sup_gemm_kernel(SupArgs<T, TI> p)
{
    __shared__ T As[SBK * SLDS];
    __shared__ T Bs[SBK * SLDS];
    sup_tile(p, (int64_t)blockIdx.y * SBM, (int64_t)blockIdx.x * SBN, (int)blockIdx.z, As, Bs);
}

// c = alpha * sum_z ws[z] (+ beta c), z in increasing order.
template <typename T>
__global__ void sup_fold_kernel(int64_t m, int64_t n, int splits, const T* __restrict__ ws, T alpha, T beta,
                                T* __restrict__ c, int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % m, j = e / m;
        T acc = ws[e];
        for (int z = 1; z < splits; ++z) acc += ws[(int64_t)z * total + e];
        T* cij = c + i * rs_c + j * cs_c;
        const T t = alpha * acc;
        *cij = (beta == T(0)) ? t : fma(beta, *cij, t);
    }
}

template <typename T, typename TI = T>
int sup_gemm(int splits, int64_t m, int64_t n, int64_t k, T alpha, const TI* a, int64_t ars, int64_t acs,
             const TI* b, int64_t brs, int64_t bcs, T beta, T* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    int64_t kchunk = (k + splits - 1) / splits;
    kchunk = (kchunk + SBK - 1) / SBK * SBK;
    const int sz = (int)((k + kchunk - 1) / kchunk);  // splits actually used
    const int64_t gx = (n + SBN - 1) / SBN, gy = (m + SBM - 1) / SBM;
    if (gy > 65535 || sz > 65535) return set_error(GB_ERR_ARG, "gemm_sup", "grid too large");
    T* ws = nullptr;
    if (sz > 1) {
        ws = static_cast<T*>(dev_alloc(sizeof(T) * (size_t)sz * m * n, s));
        if (!ws) return GB_ERR_NOMEM;
    }
    SupArgs<T, TI> p{m, n, k, kchunk, alpha, beta, a, ars, acs, b, brs, bcs, c, rs_c, cs_c, ws};
    {
        LaunchScope ls(sizeof(T) == 8 ? "sup_dmma" : (sizeof(TI) == 2 ? "sup_bf16" : "sup_ffma"), s);
        sup_gemm_kernel<T, TI><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)sz), SNT, 0, s>>>(p);
    }
    int rc = check_cuda(cudaGetLastError(), "gemm_sup");
    if (!rc && sz > 1) {
        int64_t blocks = (m * n + 255) / 256;
        const int64_t cap = (int64_t)(sm_count() > 0 ? sm_count() : 148) * 8;
        if (blocks > cap) blocks = cap;
        LaunchScope ls("sup_fold", s);
        sup_fold_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(m, n, sz, ws, alpha, beta, c, rs_c, cs_c);
        rc = check_cuda(cudaGetLastError(), "sup_fold");
    }
    dev_free(ws, s);
    return rc;
}

// ---------------------------------------------------------------- grouped form
// The gemm_batch problems whose selected configuration is the 64 x 64 engine
// (configs 1..5) run in one persistent launch: a device counter hands out
// tiles (problem, k chunk z, tile row, tile column) in the order of a table
// sorted by work; problems split along k write partial sums to their own
// workspace and one grouped fold launch adds them in order of z.
template <typename T>
struct SupGroupDesc {
    SupArgs<T> p;
    int64_t tile_start;  // first tile of this problem
    int64_t fold_start;  // first fold block (split problems only)
    int32_t tiles_m, tiles_n, splits, pad;
};

template <typename T>
__global__ void __launch_bounds__(SNT) sup_grouped_kernel(const SupGroupDesc<T>* __restrict__ d, int nprob,
                                                          int64_t total_tiles, unsigned long long* counter)
{
    __shared__ T As[SBK * SLDS];
    __shared__ T Bs[SBK * SLDS];
    __shared__ long long tile_s;
    for (;;) {
        if (threadIdx.x == 0) tile_s = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long tile = tile_s;
        __syncthreads();
        if (tile >= total_tiles) break;
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (d[mid].tile_start <= tile) lo = mid;
            else hi = mid - 1;
        }
        const SupGroupDesc<T>& q = d[lo];
        const int64_t local = tile - q.tile_start;
        const int64_t per = (int64_t)q.tiles_m * q.tiles_n;
        const int z = (int)(local / per);
        const int64_t t = local - (int64_t)z * per;
        sup_tile(q.p, (t / q.tiles_n) * SBM, (t % q.tiles_n) * SBN, z, As, Bs);
    }
}

template <typename T>
__global__ void sup_grouped_fold_kernel(const SupGroupDesc<T>* __restrict__ d, const int32_t* __restrict__ fprob)
{
    const int pi = fprob[blockIdx.x];
    const SupGroupDesc<T>& q = d[pi];
    const int64_t total = q.p.m * q.p.n;
    const int64_t e = ((int64_t)blockIdx.x - q.fold_start) * 256 + threadIdx.x;
    if (e >= total) return;
    const int64_t i = e % q.p.m, j = e / q.p.m;
    T acc = q.p.ws[e];
    for (int z = 1; z < q.splits; ++z) acc += q.p.ws[(int64_t)z * total + e];
    T* cij = q.p.c + i * q.p.rs_c + j * q.p.cs_c;
    const T t = q.p.alpha * acc;
    *cij = (q.p.beta == T(0)) ? t : fma(q.p.beta, *cij, t);
}

}  // namespace

struct SupGroup {
    int dtype = 0;
    int nprob = 0;
    int64_t total_tiles = 0, fblocks = 0;
    uint8_t* arena = nullptr;  // descriptors, fold table, counter, split workspaces
    void* d_desc = nullptr;
    int32_t* d_fprob = nullptr;
    unsigned long long* d_counter = nullptr;
};

namespace {

template <typename T>
int sup_group_build(const gb_gemm_problem_t* probs, const int* configs, int64_t count, cudaStream_t s,
                    SupGroup* g)
{
    std::vector<SupGroupDesc<T>> h;
    std::vector<int64_t> work;
    size_t ws_elems = 0;
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& q = probs[i];
        const int cfg = configs[i];
        if (cfg < 1 || cfg >= GB_GEMM_NUM_CONFIGS || q.m <= 0 || q.n <= 0 || q.k <= 0 || q.alpha == 0.0)
            return set_error(GB_ERR_ARG, "gemm_batch", "problem not eligible for the 64 x 64 engine");
        const bool ta = GB_IS_TRANS(q.transa), tb = GB_IS_TRANS(q.transb);
        SupGroupDesc<T> d = {};
        const int splits = 1 << (cfg - 1);
        int64_t kchunk = (q.k + splits - 1) / splits;
        kchunk = (kchunk + SBK - 1) / SBK * SBK;
        d.splits = (int32_t)((q.k + kchunk - 1) / kchunk);
        d.p = SupArgs<T>{q.m, q.n, q.k, kchunk, (T)q.alpha, (T)q.beta, static_cast<const T*>(q.a),
                         ta ? q.lda : 1, ta ? 1 : q.lda, static_cast<const T*>(q.b), tb ? q.ldb : 1, tb ? 1 : q.ldb,
                         static_cast<T*>(q.c), 1, q.ldc, nullptr};
        d.tiles_m = (int32_t)((q.m + SBM - 1) / SBM);
        d.tiles_n = (int32_t)((q.n + SBN - 1) / SBN);
        if (d.splits > 1) {
            d.p.ws = reinterpret_cast<T*>((uintptr_t)ws_elems);  // offset until the arena exists
            ws_elems += (size_t)d.splits * q.m * q.n;
        }
        h.push_back(d);
        work.push_back(q.k / d.splits);
    }
    // longest k chunk first
    std::vector<size_t> order(h.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return work[x] > work[y]; });
    std::vector<SupGroupDesc<T>> hs;
    std::vector<int32_t> fprob;
    for (size_t i : order) hs.push_back(h[i]);
    int64_t tiles = 0, fb = 0;
    for (size_t i = 0; i < hs.size(); ++i) {
        SupGroupDesc<T>& d = hs[i];
        d.tile_start = tiles;
        tiles += (int64_t)d.splits * d.tiles_m * d.tiles_n;
        d.fold_start = fb;
        if (d.splits > 1) {
            const int64_t nb = (d.p.m * d.p.n + 255) / 256;
            fprob.insert(fprob.end(), (size_t)nb, (int32_t)i);
            fb += nb;
        }
    }
    if (fb > INT32_MAX) return set_error(GB_ERR_ARG, "gemm_batch", "fold too large for one launch");
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t b_desc = al(sizeof(SupGroupDesc<T>) * (hs.size() + 1)), b_fp = al(4 * (fprob.size() + 1));
    const size_t b_ws = al(sizeof(T) * ws_elems);
    g->arena = static_cast<uint8_t*>(dev_alloc(b_desc + b_fp + 256 + b_ws, s));
    if (!g->arena) return GB_ERR_NOMEM;
    g->d_desc = g->arena;
    g->d_fprob = reinterpret_cast<int32_t*>(g->arena + b_desc);
    g->d_counter = reinterpret_cast<unsigned long long*>(g->arena + b_desc + b_fp);
    T* ws = reinterpret_cast<T*>(g->arena + b_desc + b_fp + 256);
    for (auto& d : hs)
        if (d.splits > 1) d.p.ws = ws + (size_t)(uintptr_t)d.p.ws;
    g->nprob = (int)hs.size();
    g->total_tiles = tiles;
    g->fblocks = fb;
    int rc = GB_SUCCESS;
    if (!hs.empty())
        rc = check_cuda(cudaMemcpyAsync(g->d_desc, hs.data(), sizeof(SupGroupDesc<T>) * hs.size(),
                                        cudaMemcpyHostToDevice, s), "sup group table");
    if (!rc && !fprob.empty())
        rc = check_cuda(cudaMemcpyAsync(g->d_fprob, fprob.data(), 4 * fprob.size(), cudaMemcpyHostToDevice, s),
                        "sup group table");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "sup group table");  // host tables go out of scope
    return rc;
}

template <typename T>
int sup_group_run(SupGroup* g, cudaStream_t s)
{
    if (g->total_tiles == 0) return GB_SUCCESS;
    GB_CUDA(cudaMemsetAsync(g->d_counter, 0, sizeof(unsigned long long), s));
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t grid = (int64_t)sms * 8;  // 128-thread CTAs, several per SM
    if (grid > g->total_tiles) grid = g->total_tiles;
    {
        LaunchScope ls(sizeof(T) == 8 ? "batch_grouped_sup_dmma" : "batch_grouped_sup_ffma", s);
        sup_grouped_kernel<T><<<(unsigned)grid, SNT, 0, s>>>(static_cast<const SupGroupDesc<T>*>(g->d_desc),
                                                              g->nprob, g->total_tiles, g->d_counter);
    }
    int rc = check_cuda(cudaGetLastError(), "grouped sup");
    if (!rc && g->fblocks > 0) {
        LaunchScope ls("batch_grouped_sup_fold", s);
        sup_grouped_fold_kernel<T><<<(unsigned)g->fblocks, 256, 0, s>>>(
            static_cast<const SupGroupDesc<T>*>(g->d_desc), g->d_fprob);
        rc = check_cuda(cudaGetLastError(), "grouped sup fold");
    }
    return rc;
}

}  // namespace

int sup_group_create(int dtype, const gb_gemm_problem_t* probs, const int* configs, int64_t count, cudaStream_t s,
                     SupGroup** out)
{
    *out = nullptr;
    SupGroup* g = new SupGroup();
    g->dtype = dtype;
    const int rc = (dtype == 0) ? sup_group_build<double>(probs, configs, count, s, g)
                                : sup_group_build<float>(probs, configs, count, s, g);
    if (rc) {
        sup_group_destroy(g, s);
        return rc;
    }
    *out = g;
    return GB_SUCCESS;
}

int sup_group_launch(SupGroup* g, cudaStream_t s)
{
    if (!g) return GB_SUCCESS;
    return (g->dtype == 0) ? sup_group_run<double>(g, s) : sup_group_run<float>(g, s);
}

void sup_group_destroy(SupGroup* g, cudaStream_t s)
{
    if (!g) return;
    dev_free(g->arena, s);
    delete g;
}

int gemm_config_dev(int dtype, int config, int64_t m, int64_t n, int64_t k, double alpha,
                    const void* a, int64_t ars, int64_t acs, const void* b, int64_t brs, int64_t bcs,
                    double beta, void* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    if (config < 0 || config >= GB_GEMM_NUM_CONFIGS) return set_error(GB_ERR_ARG, "gemm_config", "unknown config");
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (dtype < 0 || dtype > 2) return set_error(GB_ERR_ARG, "gemm_config", "dtype must be 0 (FP64), 1 (FP32) or 2 (BF16)");
    if (alpha == 0.0 || k <= 0) {
        if (dtype == 0) return scal_matrix(m, n, beta, (double*)c, rs_c, cs_c, s);
        return scal_matrix_f(m, n, (float)beta, (float*)c, rs_c, cs_c, s);
    }
    if (dtype == 2) {
        // bf16 A, B; fp32 C and arithmetic: config 0 the tensor-core kernel, 1..5 the 64 x 64 engine
        if (config == 0)
            return bgemm_tc(m, n, k, (float)alpha, (const uint16_t*)a, ars, acs, (const uint16_t*)b, brs, bcs,
                            (float)beta, (float*)c, rs_c, cs_c, s);
        return sup_gemm<float, __nv_bfloat16>(1 << (config - 1), m, n, k, (float)alpha, (const __nv_bfloat16*)a,
                                              ars, acs, (const __nv_bfloat16*)b, brs, bcs, (float)beta,
                                              (float*)c, rs_c, cs_c, s);
    }
    if (config == 0) {
        if (dtype == 0)
            return dgemm_native(m, n, k, alpha, (const double*)a, ars, acs, (const double*)b, brs, bcs, beta,
                                (double*)c, rs_c, cs_c, s);
        return sgemm_dev(m, n, k, (float)alpha, (const float*)a, ars, acs, (const float*)b, brs, bcs, (float)beta,
                         (float*)c, rs_c, cs_c, s);
    }
    const int splits = 1 << (config - 1);
    if (dtype == 0)
        return sup_gemm<double>(splits, m, n, k, alpha, (const double*)a, ars, acs, (const double*)b, brs, bcs,
                                beta, (double*)c, rs_c, cs_c, s);
    return sup_gemm<float>(splits, m, n, k, (float)alpha, (const float*)a, ars, acs, (const float*)b, brs, bcs,
                           (float)beta, (float*)c, rs_c, cs_c, s);
}

}  // namespace gb

extern "C" int gb_gemm_config_dev(int dtype, int config, gb_trans_t transa, gb_trans_t transb, gb_dim_t m,
                                  gb_dim_t n, gb_dim_t k, double alpha, const void* a, gb_inc_t rs_a,
                                  gb_inc_t cs_a, const void* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta,
                                  void* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (dtype < 0 || dtype > 2) return gb::set_error(GB_ERR_ARG, "gb_gemm_config_dev", "dtype must be 0, 1 or 2");
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_gemm_config_dev", "negative dimension");
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : gb::thread_stream();
    return gb::gemm_config_dev(dtype, config, m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b,
                               tb ? cs_b : rs_b, tb ? rs_b : cs_b, beta, c, rs_c, cs_c, s);
}

extern "C" int gb_bgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, float alpha,
                            const void* a, gb_inc_t rs_a, gb_inc_t cs_a, const void* b, gb_inc_t rs_b,
                            gb_inc_t cs_b, float beta, float* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_bgemm_dev", "negative dimension");
    int cfg = (m >= 201 && n >= 201 && k >= 201) ? 0 : 1;
    if (gb::selector_auto()) {
        int sl = 0;
        if (gb::selector_choose(2, m, n, k, GB_IS_TRANS(transa), GB_IS_TRANS(transb), 0, 0.0, 0.0, &cfg, &sl))
            return gb_get_last_error(nullptr, 0);
    }
    return gb_gemm_config_dev(2, cfg, transa, transb, m, n, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c,
                              cs_c, stream);
}
