// gb_ozaki.cu -- Ozaki split-product DGEMM for sm_103a (the precision form).
//
// FP64 on GB300 runs on a narrow pipe; the bf16 tensor cores are three
// orders of magnitude wider.  This form computes C := beta*C + alpha*A*B
// from exact integer products of bf16 digit slices (Ozaki, Ogita, Oishi &
// Rump 2012; integer-slice variant of Ootomo, Ozaki & Yokota 2024):
//
//  1. oz_rowmax / oz_split: every row of op(A) and of op(B)^T is scaled by
//     2^-e (e = ilogb(row max) + 2, so |v| < 1/2) and cut into s balanced
//     base-256 digits, t = 256 v; d = rint(t); v = t - d, |d| <= 128.  Each
//     digit is exact in bf16.  Slices are stored K-major, s planes of
//     [rows_pad][K_pad] bf16, zero padded.
//  2. ozaki_slice_gemm: a persistent tcgen05 kernel computes the integer
//     level sums S_l = sum_{p+q=l} A_p B_q^T for l = 2..s+1 (triangular
//     set, s(s+1)/2 slice products).  Operand tiles arrive by TMA (128B
//     swizzle) into a 4-stage mbarrier ring; one thread issues
//     tcgen05.mma kind::f16 (M=128, N=256, K=16) into one of two fp32 TMEM
//     accumulators; every 1024 products (|sum| <= 2^24, exact in fp32) the
//     accumulator is drained by 8 epilogue warps into int32 registers, so
//     the level sums are exact.  K is cut into parts so s*Kpart*2^14 < 2^31.
//  3. oz_recombine: FP64 only here: acc = sum_l S_l 2^-8l (least
//     significant level first), AB = acc 2^(e_i+e_j), c = alpha AB + beta c.
//
// The same arithmetic, step for step, is the CPU model used by the tests,
// which therefore check this path bit for bit.
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdlib.h>

#include "gb_internal.h"
#include "gb_sm100.cuh"

namespace gb {
namespace {

using namespace sm100;

constexpr int OZ_BM = 128, OZ_BN = 256, OZ_BK = 64, OZ_STAGES = 4;
constexpr int OZ_A_BYTES = OZ_BM * OZ_BK * 2;  // 16 KB
constexpr int OZ_B_BYTES = OZ_BN * OZ_BK * 2;  // 32 KB
constexpr int OZ_STAGE_BYTES = OZ_A_BYTES + OZ_B_BYTES;
constexpr int OZ_EPI_WARPS = 8;
constexpr int OZ_PRODUCER_WARP = OZ_EPI_WARPS;
constexpr int OZ_MMA_WARP = OZ_EPI_WARPS + 1;
constexpr int OZ_THREADS = (OZ_EPI_WARPS + 2) * 32;
constexpr uint32_t OZ_TMEM_COLS = 512;  // two 128x256 fp32 accumulators
constexpr int OZ_SMEM_BYTES = OZ_STAGES * OZ_STAGE_BYTES + 1024 + 256;
constexpr int OZ_CHUNK_KB = 16;  // 16 k-blocks of 64 = 1024 products per exact fp32 chunk

struct OzGemmParams {
    int slices;
    int nparts;
    int kb_per_part;
    int kb_total;
    int tiles_m, tiles_n;
    int64_t items;
    int chunk_kb;
    int64_t mpad, npad;
    int32_t* planes;  // [(part*slices + lev-2)][npad][mpad]
    unsigned int* status;
};

struct OzItem {
    int lev, part, tm, tn, pa_lo, npairs, kb0, kbn;
};

__device__ __forceinline__ OzItem oz_decode(const OzGemmParams& p, int64_t it)
{
    OzItem w;
    const int64_t tiles = (int64_t)p.tiles_m * p.tiles_n;
    const int64_t per_lev = (int64_t)p.nparts * tiles;
    const int q = (int)(it / per_lev);
    w.lev = p.slices + 1 - q;  // heaviest (most pairs) level first
    int64_t rem = it % per_lev;
    w.part = (int)(rem / tiles);
    const int64_t t = rem % tiles;
    // grouped raster over tiles: 8 tile rows per group for L2 reuse
    const int64_t group = t / (8 * (int64_t)p.tiles_n);
    const int64_t first_m = group * 8;
    const int64_t gm = (p.tiles_m - first_m < 8) ? p.tiles_m - first_m : 8;
    const int64_t wi = t - group * 8 * (int64_t)p.tiles_n;
    w.tm = (int)(first_m + wi % gm);
    w.tn = (int)(wi / gm);
    w.pa_lo = (w.lev - p.slices > 1) ? w.lev - p.slices : 1;
    const int pa_hi = (w.lev - 1 < p.slices) ? w.lev - 1 : p.slices;
    w.npairs = pa_hi - w.pa_lo + 1;
    w.kb0 = w.part * p.kb_per_part;
    const int kb_end = (w.kb0 + p.kb_per_part < p.kb_total) ? w.kb0 + p.kb_per_part : p.kb_total;
    w.kbn = kb_end - w.kb0;
    return w;
}

__device__ __forceinline__ void oz_fail(const OzGemmParams& p, volatile int* abort_flag)
{
    atomicOr(p.status, DEV_WAIT_TIMEOUT);
    *abort_flag = 1;
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    ozaki_slice_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
                            const __grid_constant__ CUtensorMap map_b, OzGemmParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + OZ_STAGES * OZ_STAGE_BYTES);
    uint64_t* empty = full + OZ_STAGES;
    uint64_t* tfull = empty + OZ_STAGES;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int i = 0; i < OZ_STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], OZ_EPI_WARPS);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_barrier_init();
        fence_proxy_async();
    }
    if (warp == OZ_MMA_WARP) {
        tmem_alloc(tmem_slot, OZ_TMEM_COLS);
        tmem_relinquish();
    }
    if (warp == OZ_PRODUCER_WARP && lane == 0) {
        prefetch_tensormap(&map_a);
        prefetch_tensormap(&map_b);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == OZ_PRODUCER_WARP) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t issued_mask = 0, last_phase = 0;
            bool ok = true;
            for (int64_t it = blockIdx.x; it < p.items && ok; it += gridDim.x) {
                if (*abort_flag) break;
                const OzItem w = oz_decode(p, it);
                for (int pi = 0; pi < w.npairs && ok; ++pi) {
                    const int pa = w.pa_lo + pi, pb = w.lev - pa;
                    for (int kb = 0; kb < w.kbn; ++kb) {
                        if (!mbar_wait_bounded(&empty[stage], phase ^ 1u, kWaitBudgetNs)) {
                            oz_fail(p, abort_flag);
                            ok = false;
                            break;
                        }
                        uint8_t* sa = smem + stage * OZ_STAGE_BYTES;
                        uint8_t* sb = sa + OZ_A_BYTES;
                        mbar_arrive_expect_tx(&full[stage], OZ_STAGE_BYTES);
                        const int kx = (w.kb0 + kb) * OZ_BK;
                        tma_load_3d(sa, &map_a, &full[stage], kx, w.tm * OZ_BM, pa - 1);
                        tma_load_3d(sb, &map_b, &full[stage], kx, w.tn * OZ_BN, pb - 1);
                        issued_mask |= 1u << stage;
                        last_phase = (last_phase & ~(1u << stage)) | (phase << stage);
                        if (++stage == OZ_STAGES) {
                            stage = 0;
                            phase ^= 1u;
                        }
                    }
                }
            }
            if (*abort_flag) {
                // let our own copies land before the CTA's shared memory goes away
                for (int s2 = 0; s2 < OZ_STAGES; ++s2)
                    if (issued_mask & (1u << s2))
                        mbar_wait_bounded(&full[s2], (last_phase >> s2) & 1u, kWaitBudgetNs);
            }
        }
    } else if (warp == OZ_MMA_WARP) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16_f32(OZ_BM, OZ_BN);
            int stage = 0;
            uint32_t phase = 0;
            uint32_t chunk_ctr = 0;
            bool ok = true, issued_any = false;
            for (int64_t it = blockIdx.x; it < p.items && ok; it += gridDim.x) {
                if (*abort_flag) break;
                const OzItem w = oz_decode(p, it);
                const int total = w.npairs * w.kbn;
                for (int t0 = 0; t0 < total && ok; t0 += p.chunk_kb) {
                    const int nkb = (total - t0 < p.chunk_kb) ? total - t0 : p.chunk_kb;
                    const uint32_t buf = chunk_ctr & 1u, tph = (chunk_ctr >> 1) & 1u;
                    if (!mbar_wait_bounded(&tempty[buf], tph ^ 1u, kWaitBudgetNs)) {
                        oz_fail(p, abort_flag);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d_tmem = tmem_base + buf * OZ_BN;
                    for (int q = 0; q < nkb; ++q) {
                        if (!mbar_wait_bounded(&full[stage], phase, kWaitBudgetNs)) {
                            oz_fail(p, abort_flag);
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t sa = smem_addr(smem + stage * OZ_STAGE_BYTES);
                        const uint32_t sb = sa + OZ_A_BYTES;
                        const uint64_t ad = sdesc_kmajor_sw128(sa), bd = sdesc_kmajor_sw128(sb);
#pragma unroll
                        for (int j = 0; j < OZ_BK / 16; ++j)
                            mma_bf16_ss(d_tmem, ad + 2 * j, bd + 2 * j, idesc, (q | j) != 0);
                        issued_any = true;
                        mma_commit(&empty[stage]);
                        if (++stage == OZ_STAGES) {
                            stage = 0;
                            phase ^= 1u;
                        }
                    }
                    if (!ok) break;
                    mma_commit(&tfull[buf]);
                    ++chunk_ctr;
                }
            }
            if (*abort_flag && issued_any) {
                // wait for our own MMAs before TMEM is released
                mma_commit(drain);
                mbar_wait_bounded(drain, 0, kWaitBudgetNs);
            }
        }
    } else {
        // epilogue: warp w drains TMEM lanes 32*(w%4).., columns 128*(w/4)..
        const int quad = warp & 3, half = warp >> 2;
        uint32_t chunk_ctr = 0;
        bool ok = true;
        for (int64_t it = blockIdx.x; it < p.items && ok; it += gridDim.x) {
            if (__shfl_sync(0xffffffffu, *abort_flag, 0)) break;
            const OzItem w = oz_decode(p, it);
            const int total = w.npairs * w.kbn;
            const int nchunks = (total + p.chunk_kb - 1) / p.chunk_kb;
            int32_t acc[128];
#pragma unroll
            for (int i = 0; i < 128; ++i) acc[i] = 0;
            for (int c = 0; c < nchunks; ++c) {
                const uint32_t buf = chunk_ctr & 1u, tph = (chunk_ctr >> 1) & 1u;
                int got = 1;
                if (lane == 0) got = mbar_wait_bounded(&tfull[buf], tph, kWaitBudgetNs) ? 1 : 0;
                got = __shfl_sync(0xffffffffu, got, 0);
                if (!got) {
                    if (lane == 0) oz_fail(p, abort_flag);
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t taddr = tmem_base + ((uint32_t)(quad * 32) << 16) + buf * OZ_BN + half * 128;
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    uint32_t r[32];
                    tmem_ld_32x32b_x32(taddr + g * 32, r);
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 32; ++i) acc[g * 32 + i] += __float2int_rn(__uint_as_float(r[i]));
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[buf]);
                ++chunk_ctr;
            }
            if (!ok) break;
            const int64_t q = (int64_t)w.part * p.slices + (w.lev - 2);
            const int64_t i = (int64_t)w.tm * OZ_BM + quad * 32 + lane;
            const int64_t j0 = (int64_t)w.tn * OZ_BN + half * 128;
            int32_t* dst = p.planes + (q * p.npad + j0) * p.mpad + i;
#pragma unroll
            for (int c = 0; c < 128; ++c) dst[(int64_t)c * p.mpad] = acc[c];
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == OZ_MMA_WARP) tmem_dealloc(tmem_base, OZ_TMEM_COLS);
}

// ---------------------------------------------------------------- split
// Row r of the row operand R: element (r, l) at R[r*sr + l*sl].
__global__ void oz_rowmax_kernel(int64_t rows, int64_t k, const double* __restrict__ R,
                                 int64_t sr, int64_t sl, unsigned long long* __restrict__ maxbits)
{
    __shared__ unsigned long long tmax[64];
    if (threadIdx.x < 64) tmax[threadIdx.x] = 0ull;
    __syncthreads();
    const int64_t r0 = (int64_t)blockIdx.x * 64;
    const bool rows_fast = (sr == 1);
    for (int64_t lt = blockIdx.y; lt * 64 < k; lt += gridDim.y) {
        const int64_t l0 = lt * 64;
        unsigned long long local[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int e = threadIdx.x + 256 * q;
            const int rr = rows_fast ? (e & 63) : (e >> 6);
            const int ll = rows_fast ? (e >> 6) : (e & 63);
            const int64_t r = r0 + rr, l = l0 + ll;
            local[q] = (r < rows && l < k)
                           ? (unsigned long long)__double_as_longlong(fabs(__ldg(R + r * sr + l * sl)))
                           : 0ull;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int e = threadIdx.x + 256 * q;
            const int rr = rows_fast ? (e & 63) : (e >> 6);
            if (local[q]) atomicMax(&tmax[rr], local[q]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 64 && r0 + threadIdx.x < rows && tmax[threadIdx.x])
        atomicMax(maxbits + r0 + threadIdx.x, tmax[threadIdx.x]);
}

__device__ __forceinline__ int oz_row_exponent(unsigned long long bits, int* nonfinite)
{
    if (bits == 0ull) return 0;
    if (bits >= 0x7FF0000000000000ull) {
        *nonfinite = 1;
        return 0;
    }
    return ilogb(__longlong_as_double((long long)bits)) + 2;
}

// Tile of 32 rows x 64 k per block; writes s bf16 digit planes, K-major,
// zero in the padding.
__global__ void oz_split_kernel(int64_t rows, int64_t k, const double* __restrict__ R,
                                int64_t sr, int64_t sl,
                                const unsigned long long* __restrict__ maxbits, int slices,
                                int64_t rpad, int64_t kpad, __nv_bfloat16* __restrict__ out,
                                int32_t* __restrict__ exps, int* __restrict__ nonfinite)
{
    __shared__ double tile[32][65];
    const int64_t l0 = (int64_t)blockIdx.x * 64, r0 = (int64_t)blockIdx.y * 32;
    const bool rows_fast = (sr == 1);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int e = threadIdx.x + 256 * q;
        const int rr = rows_fast ? (e & 31) : (e >> 6);
        const int ll = rows_fast ? (e >> 5) : (e & 63);
        const int64_t r = r0 + rr, l = l0 + ll;
        tile[rr][ll] = (r < rows && l < k) ? __ldg(R + r * sr + l * sl) : 0.0;
    }
    __syncthreads();
    const int rr = threadIdx.x >> 3, c0 = (threadIdx.x & 7) * 8;
    const int64_t r = r0 + rr;
    int e = 0;
    if (r < rows) {
        int nf = 0;
        e = oz_row_exponent(maxbits[r], &nf);
        if (nf) *nonfinite = 1;
        if (blockIdx.x == 0 && (threadIdx.x & 7) == 0) exps[r] = e;
    }
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (r < rows) ? ldexp(tile[rr][c0 + j], -e) : 0.0;
    for (int pl = 0; pl < slices; ++pl) {
        uint32_t packed[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            const double t0 = v[j] * 256.0, t1 = v[j + 1] * 256.0;
            const double d0 = rint(t0), d1 = rint(t1);
            v[j] = t0 - d0;
            v[j + 1] = t1 - d1;
            const __nv_bfloat16 b0 = __float2bfloat16_rn((float)d0);
            const __nv_bfloat16 b1 = __float2bfloat16_rn((float)d1);
            packed[j >> 1] = (uint32_t)__bfloat16_as_ushort(b0) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
        }
        uint4* dst = reinterpret_cast<uint4*>(out + ((int64_t)pl * rpad + r) * kpad + l0 + c0);
        *dst = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

// ---------------------------------------------------------------- recombine
__global__ void oz_recombine_kernel(int64_t m, int64_t n, const int32_t* __restrict__ planes,
                                    int slices, int nparts, int64_t mpad, int64_t npad,
                                    const int32_t* __restrict__ ea, const int32_t* __restrict__ eb,
                                    double alpha, double beta, double* __restrict__ c,
                                    int64_t rs_c, int64_t cs_c)
{
    const int64_t total = m * n;
    const bool i_fast = (rs_c == 1 || cs_c != 1);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = i_fast ? e % m : e / n;
        const int64_t j = i_fast ? e / m : e % n;
        double acc = 0.0;
        for (int q = slices - 1; q >= 0; --q) {
            long long s = 0;
            for (int pt = 0; pt < nparts; ++pt)
                s += planes[(((int64_t)pt * slices + q) * npad + j) * mpad + i];
            acc += ldexp((double)s, -8 * (q + 2));
        }
        const double ab = ldexp(acc, ea[i] + eb[j]);
        double* cij = c + i * rs_c + j * cs_c;
        const double t = __dmul_rn(alpha, ab);
        *cij = (beta == 0.0) ? t : __fma_rn(beta, *cij, t);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_slice_map(CUtensorMap* map, const void* base, int64_t kpad, int64_t rpad, int slices,
                   int box_rows)
{
    auto fn = encode_fn();
    if (!fn) return set_error(GB_ERR_CUDA, "ozaki", "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rpad, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)(kpad * 2), (cuuint64_t)(rpad * kpad * 2)};
    cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                    estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GB_ERR_CUDA, "ozaki", "cuTensorMapEncodeTiled failed");
    return GB_SUCCESS;
}

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

int chunk_kb_setting()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("GB_OZAKI_CHUNK_KB");
        int c = e ? atoi(e) : OZ_CHUNK_KB;
        v = (c >= 1 && c <= OZ_CHUNK_KB) ? c : OZ_CHUNK_KB;
    }
    return v;
}

}  // namespace

// Largest K of one part: slices * Kpart * 128^2 < 2^31, in whole 1024 chunks.
int64_t ozaki_kpart_limit(int slices)
{
    int64_t lim = (int64_t)2147483647 / ((int64_t)slices * 128 * 128);
    lim = (lim / 1024) * 1024;
    return lim < 1024 ? 1024 : lim;
}

int dgemm_ozaki(int64_t m, int64_t n, int64_t k, double alpha,
                const double* a, int64_t ars, int64_t acs,
                const double* b, int64_t brs, int64_t bcs, double beta,
                double* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0 || k <= 0) return scal_matrix(m, n, beta, c, rs_c, cs_c, s);
    if (slices < 2 || slices > 16) return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "slices must be in [2, 16]");

    const int64_t kpad = round_up(k, OZ_BK), mpad = round_up(m, OZ_BM), npad = round_up(n, OZ_BN);
    const int64_t lim = ozaki_kpart_limit(slices);
    const int nparts = (int)((k + lim - 1) / lim);
    const int kb_total = (int)(kpad / OZ_BK);
    const int kb_per_part = (kb_total + nparts - 1) / nparts;
    if ((int64_t)kb_per_part * OZ_BK > lim) return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "k partition");
    if (mpad > INT32_MAX || npad > INT32_MAX || kpad > INT32_MAX)
        return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "dimension too large for TMA coordinates");

    const size_t bytes_sa = (size_t)slices * mpad * kpad * 2, bytes_sb = (size_t)slices * npad * kpad * 2;
    const size_t bytes_pl = (size_t)nparts * slices * npad * mpad * 4;
    const size_t bytes_aux = sizeof(unsigned long long) * (m + n) + sizeof(int32_t) * (m + n) + 64;
    uint8_t* ws = static_cast<uint8_t*>(dev_alloc(bytes_sa + bytes_sb + bytes_pl + bytes_aux + 1024, s));
    if (!ws) return GB_ERR_NOMEM;
    __nv_bfloat16* sa = reinterpret_cast<__nv_bfloat16*>(ws);
    __nv_bfloat16* sb = reinterpret_cast<__nv_bfloat16*>(ws + bytes_sa);
    int32_t* planes = reinterpret_cast<int32_t*>(ws + bytes_sa + bytes_sb);
    unsigned long long* maxa = reinterpret_cast<unsigned long long*>(ws + bytes_sa + bytes_sb + bytes_pl);
    unsigned long long* maxb = maxa + m;
    int32_t* ea = reinterpret_cast<int32_t*>(maxb + n);
    int32_t* eb = ea + m;
    int* nonfinite = reinterpret_cast<int*>(eb + n);

    int rc = GB_SUCCESS;
    auto bail = [&](int code) { dev_free(ws, s); return code; };
    if ((rc = check_cuda(cudaMemsetAsync(maxa, 0, sizeof(unsigned long long) * (m + n), s), "memset")))
        return bail(rc);
    if ((rc = check_cuda(cudaMemsetAsync(nonfinite, 0, sizeof(int), s), "memset"))) return bail(rc);

    const int sms = sm_count() > 0 ? sm_count() : 148;
    auto rowmax = [&](int64_t rows, const double* R, int64_t sr, int64_t sl, unsigned long long* mb) {
        const int64_t gx = (rows + 63) / 64;
        int64_t gy = (k + 63) / 64;
        const int64_t want = (int64_t)sms * 8;
        if (gx * gy > want) gy = (want + gx - 1) / gx;
        if (gy < 1) gy = 1;
        if (gy > 65535) gy = 65535;
        LaunchScope ls("oz_rowmax", s);
        oz_rowmax_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(rows, k, R, sr, sl, mb);
    };
    auto split = [&](int64_t rows, int64_t rpad, const double* R, int64_t sr, int64_t sl,
                     const unsigned long long* mb, __nv_bfloat16* out, int32_t* ex) {
        LaunchScope ls("oz_split", s);
        oz_split_kernel<<<dim3((unsigned)(kpad / 64), (unsigned)(rpad / 32)), 256, 0, s>>>(
            rows, k, R, sr, sl, mb, slices, rpad, kpad, out, ex, nonfinite);
    };
    // rows of op(A): element (i, l) = a[i*ars + l*acs]; rows of op(B)^T: (j, l) = b[l*brs + j*bcs]
    rowmax(m, a, ars, acs, maxa);
    rowmax(n, b, bcs, brs, maxb);
    split(m, mpad, a, ars, acs, maxa, sa, ea);
    split(n, npad, b, bcs, brs, maxb, sb, eb);
    if ((rc = check_cuda(cudaGetLastError(), "oz_split"))) return bail(rc);

    int nf = 0;
    if ((rc = check_cuda(cudaMemcpyAsync(&nf, nonfinite, sizeof(int), cudaMemcpyDeviceToHost, s), "nonfinite")))
        return bail(rc);
    if ((rc = check_cuda(cudaStreamSynchronize(s), "nonfinite"))) return bail(rc);
    if (nf) {
        // Inf/NaN cannot be cut into digits: IEEE semantics come from the native kernel.
        dev_free(ws, s);
        return dgemm_native(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, s);
    }

    CUtensorMap map_a, map_b;
    if ((rc = make_slice_map(&map_a, sa, kpad, mpad, slices, OZ_BM))) return bail(rc);
    if ((rc = make_slice_map(&map_b, sb, kpad, npad, slices, OZ_BN))) return bail(rc);

    static bool attr_set = false;
    if (!attr_set) {
        if ((rc = check_cuda(cudaFuncSetAttribute(ozaki_slice_gemm_kernel,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  OZ_SMEM_BYTES), "smem attr")))
            return bail(rc);
        attr_set = true;
    }
    OzGemmParams p;
    p.slices = slices;
    p.nparts = nparts;
    p.kb_per_part = kb_per_part;
    p.kb_total = kb_total;
    p.tiles_m = (int)(mpad / OZ_BM);
    p.tiles_n = (int)(npad / OZ_BN);
    p.items = (int64_t)slices * nparts * p.tiles_m * p.tiles_n;
    p.chunk_kb = chunk_kb_setting();
    p.mpad = mpad;
    p.npad = npad;
    p.planes = planes;
    p.status = device_status_word();
    const int grid = (int)((p.items < sms) ? p.items : sms);
    {
        LaunchScope ls("ozaki_slice_gemm", s);
        ozaki_slice_gemm_kernel<<<grid, OZ_THREADS, OZ_SMEM_BYTES, s>>>(map_a, map_b, p);
    }
    if ((rc = check_cuda(cudaGetLastError(), "ozaki_slice_gemm"))) return bail(rc);
    {
        const int64_t total = m * n;
        int64_t blocks = (total + 255) / 256;
        if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
        LaunchScope ls("oz_recombine", s);
        oz_recombine_kernel<<<(unsigned)blocks, 256, 0, s>>>(m, n, planes, slices, nparts, mpad, npad,
                                                            ea, eb, alpha, beta, c, rs_c, cs_c);
    }
    rc = check_cuda(cudaGetLastError(), "oz_recombine");
    dev_free(ws, s);
    return rc;
}

}  // namespace gb
