// gb_ozaki.cu -- Ozaki split-product DGEMM for sm_103a (the precision form).
//
// FP64 on GB300 runs on a narrow pipe; the bf16 tensor cores are three
// orders of magnitude wider.  This form computes C := beta*C + alpha*A*B
// from exact integer products of bf16 digit slices (Ozaki, Ogita, Oishi &
// Rump 2012; integer-slice variant of Ootomo, Ozaki & Yokota 2024), and
// keeps FP64 arithmetic out of every bulk step:
//
//  1. oz_rowmax / oz_split (integer only): every row of op(A) and of
//     op(B)^T gets e = ilogb(row max) + 2, so U = |x| 2^-e < 1/2, and is cut
//     into s balanced base-256 digits, |d| <= 128, each exact in bf16: the
//     fixed-point value U 2^(8s+2) plus a constant bias, read byte by byte
//     (oz_digits).  Slices are stored K-major: s planes of [rows_pad][K_pad]
//     bf16, zero padded.
//  2. ozaki_slice_gemm: a persistent tcgen05 kernel computes the integer
//     level sums S_l = sum_{p+q=l} A_p B_q^T, l = 2..s+1 (the triangular
//     set, s(s+1)/2 slice products).  Tiles arrive by TMA (128B swizzle)
//     into a 4-stage mbarrier ring; one thread issues tcgen05.mma kind::f16
//     (M=128, N=256, K=16) into one of two fp32 TMEM accumulators; every
//     1024 products (|sum| <= 2^24, exact in fp32) 8 epilogue warps drain
//     the accumulator into int32 registers.  Each level's K range is cut
//     into parts with npairs(l) * Kpart * 2^14 < 2^31, one int32 plane per
//     (level, part).
//  3. oz_recombine (integer + one rounding): T = sum_l S_l 2^(8(s+1-l))
//     exactly in 128-bit, AB = RNE(T 2^(e_i+e_j-8(s+1))); FP64 only for
//     c = alpha AB + beta c (skipped for alpha = 1, beta = 0).
//
// Non-finite inputs cannot be cut into digits: the split kernels raise a
// device flag, the later kernels of this form see it and return, and a
// gated native FP64 kernel computes the IEEE result instead -- no host
// round trip.  The same arithmetic is the CPU model in oracle/gb_oracle.c,
// which the tests compare against bit for bit.
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdlib.h>

#include <algorithm>
#include <type_traits>
#include <vector>

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
constexpr int OZ_MAX_SLICES = 12;
constexpr int OZ_MAX_LEVELS = 16;  // level tables: the digit form's s levels or the CRT form's moduli
constexpr int OZ_GROUP_M = 16;

struct OzLevel {
    int lev, npairs, pa_lo, nparts, kb_per_part, plane_base;
    long long item_base;
};

struct OzGemmParams {
    static constexpr bool kDynamic = false;  // items b, b + grid, ... for CTA b
    static constexpr bool kRawAcc = false;   // chunks are converted to int32 and summed
    int slices, nlevels, kb_total, tiles_m, tiles_n, chunk_kb, group_m;
    int64_t items, mpad, npad;
    int64_t m, n;     // rows and columns of C: level sums of the padding are not stored
    int32_t* planes;  // [plane][npad][mpad]
    unsigned int* status;
    const int* skip;  // non-finite flag of the split kernels
    unsigned long long* counter;  // unused here
    // op(A) triangular with zeros outside its triangle (1 lower, 2 upper; 0
    // dense): a tile row's items cover only the k blocks its rows reach.
    // Rows of tile tm start at tri_row0 + tm * tri_rows.
    int tri_mode = 0, tri_rows = 0;
    int64_t tri_row0 = 0;
    int64_t sched_p = 0;  // CTAs (pairs) that take items it, it + sched_p, ...
    // only C's stored triangle (out_tri 1 lower, 2 upper): items run over the
    // tiles_valid tiles that hold part of it, tile_cum[tm] of them in the
    // tile rows before tm, the first at column tile tile_first[tm]
    int out_tri = 0, tiles_valid = 0;
    const int* tile_cum = nullptr;
    const int* tile_first = nullptr;
    OzLevel lv[OZ_MAX_LEVELS];
    // CRT form: planes hold int16 residues of the product sums modulo plane L's modulus
    // crt_p[L] (with 1 / p and 2^16 mod p, symmetric, for the reduction); else int32 level sums
    int crt = 0;
    float crt_p[OZ_MAX_LEVELS], crt_invp[OZ_MAX_LEVELS], crt_w16[OZ_MAX_LEVELS];
};

struct OzItem {
    int lev, npairs, pa_lo, tm, tn, kb0, kbn, plane;
    int prob;  // grouped form only: index into the problem table
};

// Grouped form (gemm_batch): every problem's slices live in one arena of
// 64-deep k blocks ("boxes": 128 rows x 64 k of A = 16 KB, 256 rows x 64 k
// of B = 32 KB, contiguous, the layout a 128-byte-swizzled TMA box expects),
// so one 3-D tensor map per operand serves all problems; a box is addressed
// by its index alone.  Level sums go to per-problem planes [level][n][ld].
// A problem whose C is taller than wide can cover fewer 128 x 256 tiles as
// C^T = op(B)^T op(A)^T; `swap` marks that form.  a, b, m, n, k, the tiles,
// boxes, split units and exponents then describe the product that runs
// (its "A" is op(B)^T), while c, rs_c, cs_c, ld and the level planes keep
// C's own orientation, so the recombination reads and writes as for any
// other problem.  The digit products are the same either way: bit-identical.
struct OzBatchProb {
    const void* a;     // FP64, or FP32 in the SGEMM form of the batch (OzBatch::f32)
    int64_t ars, acs;  // rows of op(A): (i, l) at a[i*ars + l*acs]
    const void* b;
    int64_t brs, bcs;  // rows of op(B)^T: (j, l) at b[j*brs + l*bcs]
    void* c;
    int64_t rs_c, cs_c;
    double alpha, beta;
    int64_t m, n, k;
    int32_t tiles_m, tiles_n, kb, swap;
    int32_t* ea;  // row exponents of op(A), op(B)^T
    int32_t* eb;
    int64_t abox, bbox;  // first box of this problem in one slice plane
    int32_t* planes;     // [level][columns of C][ld], ld = rows of C rounded up to 4
    int64_t ld;
    int64_t units_a;     // split units (32-row blocks) of op(A); op(B)^T's follow
};

// Items of the grouped form are handed out by a device counter (zeroed
// before each launch): the producer warp of a CTA takes the next index and
// passes it to the MMA and epilogue warps through a shared-memory ring, so
// the CTAs always work on neighbouring items and share their slices in L2
// (a fixed stride lets fast and slow CTAs drift apart across problems).
struct OzBatchParams {
    static constexpr bool kDynamic = true;
    static constexpr bool kRawAcc = false;
    int slices, nlevels, chunk_kb, nprob;
    int64_t items, boxes_a, boxes_b;  // work items; boxes per slice plane
    const OzBatchProb* probs;
    const int32_t* item_prob;  // work item -> problem
    const int64_t* item_base;  // first work item of each problem
    unsigned int* status;
    const int* skip;
    unsigned long long* counter;
    OzLevel lv[OZ_MAX_LEVELS];
};

constexpr int OZ_IRING = 4;  // work-item ring depth (dynamic form)

// Work-item ring of one CTA: the producer publishes, the MMA warp and the 8
// epilogue warps (one arrival each) release.  `it` starts at -2; the next
// index is returned in it, -1 when there is none.  False: a wait timed out.
struct OzRing {
    uint64_t* full;
    uint64_t* empty;
    volatile long long* slot_val;
    int slot;
    uint32_t phase;
};

template <class P>
__device__ __forceinline__ bool oz_publish_item(const P& p, OzRing& r, int64_t& it)
{
    if constexpr (P::kDynamic) {
        if (!mbar_wait_bounded(&r.empty[r.slot], r.phase ^ 1u, kWaitBudgetNs)) return false;
        long long v = (long long)atomicAdd(p.counter, 1ull);
        if (v >= p.items) v = -1;
        r.slot_val[r.slot] = v;
        mbar_arrive(&r.full[r.slot]);
        if (++r.slot == OZ_IRING) {
            r.slot = 0;
            r.phase ^= 1u;
        }
        it = v;
    } else {
        it = (it == -2) ? (int64_t)blockIdx.x : it + gridDim.x;
        if (it >= p.items) it = -1;
    }
    return true;
}

template <class P>
__device__ __forceinline__ bool oz_receive_item(const P& p, OzRing& r, int64_t& it)
{
    if constexpr (P::kDynamic) {
        if (!mbar_wait_bounded(&r.full[r.slot], r.phase, kWaitBudgetNs)) return false;
        it = r.slot_val[r.slot];
        mbar_arrive(&r.empty[r.slot]);
        if (++r.slot == OZ_IRING) {
            r.slot = 0;
            r.phase ^= 1u;
        }
    } else {
        it = (it == -2) ? (int64_t)blockIdx.x : it + gridDim.x;
        if (it >= p.items) it = -1;
    }
    return true;
}

__device__ __forceinline__ OzItem oz_decode(const OzGemmParams& p, int64_t it)
{
    if (p.tri_mode && p.sched_p > 0) {
        // item costs vary with the tile row: the heaviest tile rows come first
        // in each level (below) and every other full round of sched_p items is
        // dealt in reverse, so the CTAs' totals even out
        const int64_t r = it / p.sched_p, c = it - r * p.sched_p;
        if ((r & 1) && (r + 1) * p.sched_p <= p.items) it = r * p.sched_p + (p.sched_p - 1 - c);
    }
    int L = 0;
    while (L + 1 < p.nlevels && it >= p.lv[L + 1].item_base) ++L;
    const OzLevel& lv = p.lv[L];
    OzItem w;
    w.lev = lv.lev;
    w.npairs = lv.npairs;
    w.pa_lo = lv.pa_lo;
    const int64_t tiles = p.out_tri ? (int64_t)p.tiles_valid : (int64_t)p.tiles_m * p.tiles_n;
    const int64_t rem = it - lv.item_base;
    const int part = (int)(rem / tiles);
    const int64_t t = rem % tiles;
    if (p.out_tri) {
        // the t-th tile holding part of C's triangle: tile rows in order
        int lo = 0, hi = p.tiles_m;  // tile_cum[lo] <= t < tile_cum[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(p.tile_cum + mid) <= t) lo = mid;
            else hi = mid;
        }
        w.tm = lo;
        w.tn = __ldg(p.tile_first + lo) + (int)(t - __ldg(p.tile_cum + lo));
    } else {
        // grouped raster over tiles, p.group_m tile rows per group (default
        // OZ_GROUP_M = 16): the tiles in flight then share a few A and B
        // panels in L2 instead of streaming whole rows of tiles
        const int64_t G = p.group_m;
        const int64_t group = t / (G * (int64_t)p.tiles_n);
        const int64_t first_m = group * G;
        const int64_t gm = (p.tiles_m - first_m < G) ? p.tiles_m - first_m : G;
        const int64_t wi = t - group * G * (int64_t)p.tiles_n;
        w.tm = (int)(first_m + wi % gm);
        w.tn = (int)(wi / gm);
    }
    if (p.tri_mode) {
        // tile rows by decreasing k extent: last row first for a lower op(A)
        const int64_t row = t / p.tiles_n;
        w.tm = (int)((p.tri_mode == 1) ? p.tiles_m - 1 - row : row);
        w.tn = (int)(t - row * p.tiles_n);
    }
    w.kb0 = part * lv.kb_per_part;
    const int kb_end = (w.kb0 + lv.kb_per_part < p.kb_total) ? w.kb0 + lv.kb_per_part : p.kb_total;
    w.kbn = kb_end - w.kb0;
    if (p.tri_mode) {
        // the blocks outside [lo, hi) hold only zero digits for these rows and
        // add nothing to the exact sums; a part with none left keeps its first
        // block (all zero here) so that its planes are still written
        const int64_t r_lo = p.tri_row0 + (int64_t)w.tm * p.tri_rows;
        int lo = w.kb0, hi = kb_end;
        if (p.tri_mode == 1) {  // lower: row i reaches columns <= i
            const int64_t need = (r_lo + p.tri_rows + OZ_BK - 1) / OZ_BK;
            if (need < hi) hi = (int)need;
        } else {  // upper: row i reaches columns >= i
            const int64_t need = r_lo / OZ_BK;
            if (need > lo) lo = (int)need;
        }
        if (hi > lo) {
            w.kb0 = lo;
            w.kbn = hi - lo;
        } else {
            w.kbn = 1;
        }
    }
    w.plane = lv.plane_base + part;
    w.prob = 0;
    return w;
}

// Grouped form: items are (problem, level, tile) with levels heaviest first
// inside a problem; one part per level (the host keeps npairs * k small
// enough).  Tiles of a problem in column-major raster.
__device__ __forceinline__ OzItem oz_decode(const OzBatchParams& p, int64_t it)
{
    const int pi = __ldg(p.item_prob + it);
    const OzBatchProb& q = p.probs[pi];
    const int64_t tiles = (int64_t)q.tiles_m * q.tiles_n;
    const int64_t rem = it - __ldg(p.item_base + pi);
    const int L = (int)(rem / tiles);
    const int64_t t = rem - (int64_t)L * tiles;
    const OzLevel& lv = p.lv[L];
    OzItem w;
    w.lev = lv.lev;
    w.npairs = lv.npairs;
    w.pa_lo = lv.pa_lo;
    w.tm = (int)(t % q.tiles_m);
    w.tn = (int)(t / q.tiles_m);
    w.kb0 = 0;
    w.kbn = q.kb;
    w.plane = L;
    w.prob = pi;
    return w;
}

// One k block of the pair (A_pa, B_pb) into a stage.
__device__ __forceinline__ void oz_load_stage(const OzGemmParams&, const CUtensorMap* ma, const CUtensorMap* mb,
                                              uint8_t* sa, uint8_t* sb, uint64_t* bar, const OzItem& w, int pa,
                                              int pb, int kb)
{
    const int kx = (w.kb0 + kb) * OZ_BK;
    tma_load_3d(sa, ma, bar, kx, w.tm * OZ_BM, pa - 1);
    tma_load_3d(sb, mb, bar, kx, w.tn * OZ_BN, pb - 1);
}

__device__ __forceinline__ void oz_load_stage(const OzBatchParams& p, const CUtensorMap* ma,
                                              const CUtensorMap* mb, uint8_t* sa, uint8_t* sb, uint64_t* bar,
                                              const OzItem& w, int pa, int pb, int kb)
{
    const OzBatchProb& q = p.probs[w.prob];
    const int64_t za = (int64_t)(pa - 1) * p.boxes_a + q.abox + (int64_t)w.tm * q.kb + kb;
    const int64_t zb = (int64_t)(pb - 1) * p.boxes_b + q.bbox + (int64_t)w.tn * q.kb + kb;
    tma_load_3d(sa, ma, bar, 0, 0, (int)za);
    tma_load_3d(sb, mb, bar, 0, 0, (int)zb);
}

// A CRT product sum v reduced to its symmetric residue modulo the plane's
// modulus p (|r| <= p/2 <= 128, stored as int16).  With v = hi 2^16 + lo,
// lo in [0, 2^16), and w = 2^16 mod p in [-p/2, p/2]: s = hi w + lo has
// |s| < 2^22 + 2^16, an integer exact in fp32 (the fma rounds nothing) with
// v's residue; rint(s / p) by one fma onto 1.5 2^23 is exact as in the split
// (s invp is within |s| 2^-24 / p < 0.27 / p of s / p, and a non-integral
// s / p is at least 1 / (2p) from a half-integer; for p = 256, invp is exact
// and a tie rounds to even, either sign being the same residue).
__device__ __forceinline__ int16_t oz_crt_reduce(int32_t v, float p, float invp, float w16)
{
    const float sv = __fmaf_rn((float)(v >> 16), w16, (float)(v & 0xFFFF));
    const float q = __fmaf_rn(sv, invp, 12582912.0f) - 12582912.0f;  // 1.5 2^23
    return (int16_t)__float2int_rn(__fmaf_rn(-q, p, sv));
}

// The product sums of one epilogue thread (row i of C, columns j0 .. j0 + 127)
// into plane w.plane: int32 level sums, or int16 residues in the CRT form.
__device__ __forceinline__ void oz_store_plane(const OzGemmParams& p, const OzItem& w, int64_t i, int64_t j0,
                                               const int32_t (&acc)[128])
{
    if (i >= p.m) return;  // level sums of padding rows and columns are not stored
    const int64_t jn = p.n - j0;  // columns of this half that exist
    const int64_t at = ((int64_t)w.plane * p.npad + j0) * p.mpad + i;
    if (p.crt) {
        int16_t* dst = reinterpret_cast<int16_t*>(p.planes) + at;
        const float pm = p.crt_p[w.plane], ip = p.crt_invp[w.plane], w16 = p.crt_w16[w.plane];
#pragma unroll
        for (int c = 0; c < 128; ++c)
            if (jn >= 128 || c < jn) dst[(int64_t)c * p.mpad] = oz_crt_reduce(acc[c], pm, ip, w16);
        return;
    }
    int32_t* dst = p.planes + at;
    if (jn >= 128) {
#pragma unroll
        for (int c = 0; c < 128; ++c) dst[(int64_t)c * p.mpad] = acc[c];
    } else {
#pragma unroll
        for (int c = 0; c < 128; ++c)
            if (c < jn) dst[(int64_t)c * p.mpad] = acc[c];
    }
}

// Level sums of one epilogue thread (row quad*32 + lane, columns half*128 ..
// +127 of the tile) into the level plane.
__device__ __forceinline__ void oz_store_sums(const OzGemmParams& p, const OzItem& w, int quad, int half,
                                              int lane, const int32_t (&acc)[128])
{
    oz_store_plane(p, w, (int64_t)w.tm * OZ_BM + quad * 32 + lane, (int64_t)w.tn * OZ_BN + half * 128, acc);
}

__device__ __forceinline__ void oz_store_sums(const OzBatchParams& p, const OzItem& w, int quad, int half,
                                              int lane, const int32_t (&acc)[128])
{
    const OzBatchProb& q = p.probs[w.prob];
    const int64_t i = (int64_t)w.tm * OZ_BM + quad * 32 + lane;
    const int64_t j0 = (int64_t)w.tn * OZ_BN + half * 128;
    if (i >= q.m) return;
    const int64_t jn = q.n - j0;  // columns of this half that exist
    if (!q.swap) {
        int32_t* dst = q.planes + ((int64_t)w.plane * q.n + j0) * q.ld + i;
#pragma unroll
        for (int c = 0; c < 128; ++c)
            if (c < jn) dst[(int64_t)c * q.ld] = acc[c];
    } else {
        // row i of the product is column i of C: the thread's 128 sums are contiguous in the
        // plane (j0 and ld are multiples of 4, so 16-byte stores)
        int32_t* dst = q.planes + ((int64_t)w.plane * q.m + i) * q.ld + j0;
        if (jn >= 128) {
#pragma unroll
            for (int c = 0; c < 128; c += 4)
                *reinterpret_cast<int4*>(dst + c) = make_int4(acc[c], acc[c + 1], acc[c + 2], acc[c + 3]);
        } else {
#pragma unroll
            for (int c = 0; c < 128; ++c)
                if (c < jn) dst[c] = acc[c];
        }
    }
}

// ---------------------------------------------------------------- BF16 GEMM
// The same kernel as a plain bf16 GEMM (no Ozaki slices): C (fp32) :=
// alpha A B + beta C with A, B in bf16.  One "slice", one level with one
// product, a single chunk over the whole k range (fp32 accumulation in TMEM
// needs no exactness here), and an epilogue that writes fp32 C instead of
// int32 level sums.  Operands arrive by TMA straight from the caller's
// K-contiguous rows (or from a packed copy); zero fill past m, n and k.
struct BgemmParams {
    static constexpr bool kDynamic = false;
    static constexpr bool kRawAcc = true;
    int tiles_m, tiles_n, kb_total, chunk_kb;
    int64_t items, m, n;
    float alpha, beta;
    float* c;
    int64_t rs_c, cs_c;
    unsigned int* status;
    const int* skip;  // null: nothing gates this form
    unsigned long long* counter;
};

__device__ __forceinline__ OzItem oz_decode(const BgemmParams& p, int64_t it)
{
    // grouped raster as in the Ozaki form: OZ_GROUP_M tile rows per group
    const int64_t group = it / (OZ_GROUP_M * (int64_t)p.tiles_n);
    const int64_t first_m = group * OZ_GROUP_M;
    const int64_t gm = (p.tiles_m - first_m < OZ_GROUP_M) ? p.tiles_m - first_m : OZ_GROUP_M;
    const int64_t wi = it - group * OZ_GROUP_M * (int64_t)p.tiles_n;
    OzItem w;
    w.lev = 2;
    w.npairs = 1;
    w.pa_lo = 1;
    w.tm = (int)(first_m + wi % gm);
    w.tn = (int)(wi / gm);
    w.kb0 = 0;
    w.kbn = p.kb_total;
    w.plane = 0;
    w.prob = 0;
    return w;
}

__device__ __forceinline__ void oz_load_stage(const BgemmParams&, const CUtensorMap* ma, const CUtensorMap* mb,
                                              uint8_t* sa, uint8_t* sb, uint64_t* bar, const OzItem& w, int,
                                              int, int kb)
{
    tma_load_3d(sa, ma, bar, kb * OZ_BK, w.tm * OZ_BM, 0);
    tma_load_3d(sb, mb, bar, kb * OZ_BK, w.tn * OZ_BN, 0);
}

__device__ __forceinline__ void oz_store_sums(const BgemmParams& p, const OzItem& w, int quad, int half, int lane,
                                              const int32_t (&acc)[128])
{
    const int64_t i = (int64_t)w.tm * OZ_BM + quad * 32 + lane;
    const int64_t j0 = (int64_t)w.tn * OZ_BN + half * 128;
    if (i >= p.m) return;
    const int64_t jn = p.n - j0;
    float* ci = p.c + i * p.rs_c + j0 * p.cs_c;
#pragma unroll
    for (int c = 0; c < 128; ++c) {
        if (c < jn) {
            float* cij = ci + (int64_t)c * p.cs_c;
            const float t = p.alpha * __int_as_float(acc[c]);
            *cij = (p.beta == 0.0f) ? t : fmaf(p.beta, *cij, t);
        }
    }
}

template <class P>
__device__ __forceinline__ void oz_fail(const P& p, volatile int* abort_flag)
{
    atomicOr(p.status, DEV_WAIT_TIMEOUT);
    *abort_flag = 1;
}

template <class P>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    ozaki_slice_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
                            const __grid_constant__ CUtensorMap map_b, const __grid_constant__ P p)
{
    if (p.skip && *p.skip) return;  // uniform across the CTA: the native kernel takes over
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + OZ_STAGES * OZ_STAGE_BYTES);
    uint64_t* empty = full + OZ_STAGES;
    uint64_t* tfull = empty + OZ_STAGES;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint64_t* ifull = drain + 1;  // work-item ring (dynamic form)
    uint64_t* iempty = ifull + OZ_IRING;
    volatile long long* iring = reinterpret_cast<volatile long long*>(iempty + OZ_IRING);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(const_cast<long long*>(iring + OZ_IRING));
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
        for (int i = 0; i < OZ_IRING; ++i) {
            mbar_init(&ifull[i], 1);
            mbar_init(&iempty[i], 1 + OZ_EPI_WARPS);  // the MMA warp and every epilogue warp
        }
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
            OzRing ring{ifull, iempty, iring, 0, 0u};
            for (int64_t it = -2; ok;) {
                if (*abort_flag) break;
                if (!oz_publish_item(p, ring, it)) {
                    oz_fail(p, abort_flag);
                    break;
                }
                if (it < 0) break;
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
                        oz_load_stage(p, &map_a, &map_b, sa, sb, &full[stage], w, pa, pb, kb);
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
            OzRing ring{ifull, iempty, iring, 0, 0u};
            for (int64_t it = -2; ok;) {
                if (*abort_flag) break;
                if (!oz_receive_item(p, ring, it)) {
                    oz_fail(p, abort_flag);
                    break;
                }
                if (it < 0) break;
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
        OzRing ring{ifull, iempty, iring, 0, 0u};
        for (int64_t it = -2; ok;) {
            if (__shfl_sync(0xffffffffu, *abort_flag, 0)) break;
            long long next = 0;
            int got = 1;
            if (lane == 0) {
                int64_t t = it;
                got = oz_receive_item(p, ring, t) ? 1 : 0;
                next = t;
            }
            got = __shfl_sync(0xffffffffu, got, 0);
            next = __shfl_sync(0xffffffffu, next, 0);
            if (!got) {
                if (lane == 0) oz_fail(p, abort_flag);
                break;
            }
            it = next;
            if (it < 0) break;
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
                    for (int i = 0; i < 32; ++i) {
                        if constexpr (P::kRawAcc) acc[g * 32 + i] = (int32_t)r[i];  // one chunk: fp32 bits
                        else acc[g * 32 + i] += __float2int_rn(__uint_as_float(r[i]));
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[buf]);
                ++chunk_ctr;
            }
            if (!ok) break;
            oz_store_sums(p, w, quad, half, lane, acc);
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == OZ_MMA_WARP) tmem_dealloc(tmem_base, OZ_TMEM_COLS);
}

// ---------------------------------------------------------------- CTA-pair form
// The same computation on clusters of two CTAs (cta_group::2): a pair owns a
// 256 x 256 tile; each CTA stages 128 rows of A and 128 rows of B per k block
// (32 KB, six stages), the even CTA issues M=256 N=256 K=16 MMAs that read
// both CTAs' shared memory and write each CTA's 128 accumulator rows into
// its own TMEM.  Per SM this halves the B bytes moved through shared memory
// (TMA writes plus MMA reads fall from ~192 to ~128 bytes per clock at full
// MMA rate).  Both CTAs' TMA loads count on the even CTA's `full` barrier;
// MMA completion is multicast to both CTAs' `empty` and `tfull` barriers; the
// odd CTA's epilogue warps release TMEM by arriving on the even CTA's
// `tempty` barrier.
constexpr int OZ2_STAGES = 6;
constexpr int OZ2_ROWS = 128;                       // rows of A and of B per CTA
constexpr int OZ2_A_BYTES = OZ2_ROWS * OZ_BK * 2;   // 16 KB
constexpr int OZ2_B_BYTES = OZ2_ROWS * OZ_BK * 2;   // 16 KB
constexpr int OZ2_STAGE_BYTES = OZ2_A_BYTES + OZ2_B_BYTES;
constexpr int OZ2_SMEM_BYTES = OZ2_STAGES * OZ2_STAGE_BYTES + 1024 + 256;

__global__ void __launch_bounds__(OZ_THREADS, 1)
    ozaki_slice_gemm_pair_kernel(const __grid_constant__ CUtensorMap map_a,
                                 const __grid_constant__ CUtensorMap map_b, const __grid_constant__ OzGemmParams p)
{
    if (*p.skip) return;  // both CTAs of a pair read the same flag
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + OZ2_STAGES * OZ2_STAGE_BYTES);
    uint64_t* empty = full + OZ2_STAGES;
    uint64_t* tfull = empty + OZ2_STAGES;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();
    const bool leader = (rank == 0);
    const int64_t pair = blockIdx.x >> 1, npair = gridDim.x >> 1;

    if (threadIdx.x == 0) {
        for (int i = 0; i < OZ2_STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 2 * OZ_EPI_WARPS);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_barrier_init();
        fence_proxy_async();
    }
    if (warp == OZ_MMA_WARP) {
        tmem_alloc_pair(tmem_slot, OZ_TMEM_COLS);
        tmem_relinquish_pair();
    }
    if (warp == OZ_PRODUCER_WARP && lane == 0) {
        prefetch_tensormap(&map_a);
        prefetch_tensormap(&map_b);
    }
    tc_fence_before();
    __syncthreads();
    cluster_sync();  // the peer's barriers exist before any cross-CTA signal
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == OZ_PRODUCER_WARP) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t issued_mask = 0, last_phase = 0;
            bool ok = true;
            for (int64_t it = pair; it < p.items && ok; it += npair) {
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
                        uint8_t* sa = smem + stage * OZ2_STAGE_BYTES;
                        uint8_t* sb = sa + OZ2_A_BYTES;
                        if (leader) mbar_arrive_expect_tx(&full[stage], 2 * OZ2_STAGE_BYTES);
                        const uint32_t bar = mapa_shared(smem_addr(&full[stage]), 0);
                        const int kx = (w.kb0 + kb) * OZ_BK;
                        tma_load_3d_pair(sa, &map_a, bar, kx, w.tm * (2 * OZ2_ROWS) + (int)rank * OZ2_ROWS, pa - 1);
                        tma_load_3d_pair(sb, &map_b, bar, kx, w.tn * OZ_BN + (int)rank * OZ2_ROWS, pb - 1);
                        issued_mask |= 1u << stage;
                        last_phase = (last_phase & ~(1u << stage)) | (phase << stage);
                        if (++stage == OZ2_STAGES) {
                            stage = 0;
                            phase ^= 1u;
                        }
                    }
                }
            }
            if (*abort_flag) {
                if (leader) {
                    for (int s2 = 0; s2 < OZ2_STAGES; ++s2)
                        if (issued_mask & (1u << s2))
                            mbar_wait_bounded(&full[s2], (last_phase >> s2) & 1u, kWaitBudgetNs);
                } else {
                    // the odd CTA's copies complete on the even CTA's barrier: give
                    // them time to land before this CTA's shared memory is released
                    const uint64_t t0 = globaltimer();
                    while (globaltimer() - t0 < 2000000ull) {
                    }
                }
            }
        }
    } else if (warp == OZ_MMA_WARP) {
        if (lane == 0 && leader) {
            constexpr uint32_t idesc = idesc_bf16_f32(2 * OZ2_ROWS, OZ_BN);
            int stage = 0;
            uint32_t phase = 0;
            uint32_t chunk_ctr = 0;
            bool ok = true, issued_any = false;
            for (int64_t it = pair; it < p.items && ok; it += npair) {
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
                        const uint32_t sa = smem_addr(smem + stage * OZ2_STAGE_BYTES);
                        const uint32_t sb = sa + OZ2_A_BYTES;
                        const uint64_t ad = sdesc_kmajor_sw128(sa), bd = sdesc_kmajor_sw128(sb);
#pragma unroll
                        for (int j = 0; j < OZ_BK / 16; ++j)
                            mma_bf16_pair(d_tmem, ad + 2 * j, bd + 2 * j, idesc, (q | j) != 0);
                        issued_any = true;
                        mma_commit_pair(&empty[stage], 0x3);
                        if (++stage == OZ2_STAGES) {
                            stage = 0;
                            phase ^= 1u;
                        }
                    }
                    if (!ok) break;
                    mma_commit_pair(&tfull[buf], 0x3);
                    ++chunk_ctr;
                }
            }
            if (*abort_flag && issued_any) {
                mma_commit_pair(drain, 0x1);
                mbar_wait_bounded(drain, 0, kWaitBudgetNs);
            }
        }
    } else {
        // epilogue: this CTA's 128 accumulator rows, as in the single-CTA form
        const int quad = warp & 3, half = warp >> 2;
        const uint32_t leader_tempty0 = mapa_shared(smem_addr(&tempty[0]), 0);
        uint32_t chunk_ctr = 0;
        bool ok = true;
        for (int64_t it = pair; it < p.items && ok; it += npair) {
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
                if (lane == 0) {
                    if (leader) mbar_arrive(&tempty[buf]);
                    else mbar_arrive_cluster(leader_tempty0 + buf * (uint32_t)sizeof(uint64_t));
                }
                ++chunk_ctr;
            }
            if (!ok) break;
            oz_store_plane(p, w, (int64_t)w.tm * (2 * OZ2_ROWS) + (int64_t)rank * OZ2_ROWS + quad * 32 + lane,
                           (int64_t)w.tn * OZ_BN + half * 128, acc);
        }
    }

    tc_fence_before();
    __syncthreads();
    cluster_sync();  // no CTA leaves while its peer may still touch its memory
    tc_fence_after();
    if (warp == OZ_MMA_WARP) tmem_dealloc_pair(tmem_base, OZ_TMEM_COLS);
}

// ---------------------------------------------------------------- split
// Row r of the row operand R: element (r, l) at R[r*sr + l*sl].  |x| as its
// IEEE bit pattern is monotone in |x|, so the row maximum is an integer max.
// Built from the two 32-bit halves: a 64-bit mask of the sign bit is the
// pattern of an FP64 absolute value, which would put every element on
// GB300's narrow FP64 pipe.
__device__ __forceinline__ unsigned long long abs_bits(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7FFFFFFFu, lo = (unsigned)__double2loint(x);
    return ((unsigned long long)hi << 32) | lo;
}

// Row-maximum keys of FP64 or FP32 elements: the IEEE bits of |x| (monotone
// in |x|), and the FP64 bits of a maximum for oz_row_exponent.  FP32 keys
// stay 32 bits; only the maximum is widened (exactly).
template <typename T>
using OzKey = std::conditional_t<sizeof(T) == 4, uint32_t, unsigned long long>;

template <typename T>
__device__ __forceinline__ OzKey<T> oz_abs_key(T x)
{
    if constexpr (sizeof(T) == 4) return __float_as_uint(x) & 0x7fffffffu;
    else return abs_bits(x);
}

template <typename T>
__device__ __forceinline__ unsigned long long oz_key_f64(unsigned long long key)
{
    if constexpr (sizeof(T) == 4) return (unsigned long long)__double_as_longlong((double)__uint_as_float((uint32_t)key));
    else return key;
}

// Rows contiguous (sr == 1, e.g. column-major op(A)): thread per row, the
// grid's y dimension splits k.
template <typename T>
__global__ void oz_rowmax_rows_kernel(int64_t rows, int64_t k, const T* __restrict__ R,
                                      int64_t sl, int64_t kchunk, unsigned long long* __restrict__ maxbits)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int64_t l0 = (int64_t)blockIdx.y * kchunk;
    const int64_t l1 = (l0 + kchunk < k) ? l0 + kchunk : k;
    // eight loads in flight per thread (one HBM round trip hides behind about 40 KB per SM)
    OzKey<T> mq[4] = {0, 0, 0, 0};
    int64_t l = l0;
    for (; l + 7 < l1; l += 8) {
        OzKey<T> b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) b[u] = oz_abs_key(__ldcs(R + r + (l + u) * sl));
#pragma unroll
        for (int u = 0; u < 8; ++u) mq[u & 3] = b[u] > mq[u & 3] ? b[u] : mq[u & 3];
    }
    for (; l < l1; ++l) {
        const OzKey<T> b0 = oz_abs_key(__ldcs(R + r + l * sl));
        mq[0] = b0 > mq[0] ? b0 : mq[0];
    }
    const OzKey<T> m01 = mq[0] > mq[1] ? mq[0] : mq[1], m23 = mq[2] > mq[3] ? mq[2] : mq[3];
    const OzKey<T> mx = m01 > m23 ? m01 : m23;
    if (mx) atomicMax(maxbits + r, oz_key_f64<T>(mx));
}

// Any other layout: warp per row, lanes stride along k.
template <typename T>
__global__ void oz_rowmax_warp_kernel(int64_t rows, int64_t k, const T* __restrict__ R,
                                      int64_t sr, int64_t sl, int64_t kchunk,
                                      unsigned long long* __restrict__ maxbits)
{
    const int lane = threadIdx.x & 31;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= rows) return;
    const int64_t l0 = (int64_t)blockIdx.y * kchunk;
    const int64_t l1 = (l0 + kchunk < k) ? l0 + kchunk : k;
    OzKey<T> mx = 0, my = 0;
    int64_t l = l0 + lane;
    for (; l + 32 * 7 < l1; l += 32 * 8) {  // eight loads in flight per lane
        OzKey<T> b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) b[u] = oz_abs_key(__ldcs(R + r * sr + (l + 32 * u) * sl));
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
            mx = b[u] > mx ? b[u] : mx;
            my = b[u + 1] > my ? b[u + 1] : my;
        }
    }
    for (; l < l1; l += 32) {
        const OzKey<T> b = oz_abs_key(__ldcs(R + r * sr + l * sl));
        mx = b > mx ? b : mx;
    }
    mx = my > mx ? my : mx;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const OzKey<T> o = __shfl_xor_sync(0xffffffffu, mx, off);
        mx = o > mx ? o : mx;
    }
    if (lane == 0 && mx) atomicMax(maxbits + r, oz_key_f64<T>(mx));
}

__device__ __forceinline__ int clz128(unsigned __int128 u)
{
    const unsigned long long hi = (unsigned long long)(u >> 64), lo = (unsigned long long)u;
    return hi ? __clzll((long long)hi) : (lo ? 64 + __clzll((long long)lo) : 128);
}

// Balanced base-256 digits of U = |x| 2^-e with the sign of x, from
// integers only.  X = U 2^F truncated (F = 8S+2 fraction bits); adding
// B = sum_p 128 2^(F-8p) + 2 makes the balanced digits the plain base-256
// digits of Y = X + B: d_1 = (Y >> (F-8)) - 128 (at most 128), d_p =
// ((Y >> (F-8p)) & 255) - 128.  The remainder lies in [-2, 2) units of
// 2^-F, i.e. |rem| <= 2^-(8S+1) 2^e, and truncating X never changes a digit
// (the rounding threshold is an integer).  x = 0 gives Y = B, all digits 0.
template <typename U>
__host__ __device__ constexpr U oz_bias(int S)
{
    U b = 2;
    for (int p = 1; p <= S; ++p) b += (U)128 << (8 * S + 2 - 8 * p);
    return b;
}

// The split is integer-bound, so each digit costs one shift, one LOP3 and
// one add on the integer pipe: with m = all ones for a negative x (else 0),
// (raw ^ m) + c is raw - 128 for x >= 0 and 128 - raw for x < 0 when c is
// -128 or +129, and adding 0x4B400000 (the fp32 1.5 * 2^23, whose unit in
// the last place is 1) to c makes that sum the fp32 bit pattern of
// 1.5 * 2^23 + d; one fp32 subtract (FMA pipe) leaves the exact float(d).
// float(d) has at most 8 significant bits for |d| <= 128, so its upper half
// is exactly the bf16 value.
constexpr uint32_t OZ_MAGIC_BITS = 0x4B400000u;  // 12582912.0f
constexpr float OZ_MAGIC = 12582912.0f;

template <int S>
__device__ __forceinline__ void oz_digit_floats(double x, int e, float (&f)[S])
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const uint32_t m = (uint32_t)((long long)bits >> 63);
    const uint32_t c = m ? OZ_MAGIC_BITS + 129u : OZ_MAGIC_BITS - 128u;
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long M = (bits & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0ull);
    const int E2 = ex ? ex - 1075 : -1074;
    constexpr int F = 8 * S + 2;
    const int sh = E2 - e + F;  // U 2^F = M 2^sh < 2^(F-1)
    if constexpr (F + 1 < 64) {
        // Y < 2^(F+1): 64 bits suffice (S <= 7)
        const unsigned long long X = (sh >= 0) ? (M << sh) : (sh > -64 ? (M >> (-sh)) : 0ull);
        const unsigned long long Y = X + oz_bias<unsigned long long>(S);
        f[0] = __uint_as_float(((uint32_t)(Y >> (F - 8)) ^ m) + c) - OZ_MAGIC;
#pragma unroll
        for (int p = 2; p <= S; ++p)
            f[p - 1] = __uint_as_float((((uint32_t)(Y >> (F - 8 * p)) & 255u) ^ m) + c) - OZ_MAGIC;
    } else {
        using u128 = unsigned __int128;
        const u128 X = (sh >= 0) ? ((u128)M << sh) : (u128)(sh > -64 ? (M >> (-sh)) : 0ull);
        const u128 Y = X + oz_bias<u128>(S);
        f[0] = __uint_as_float(((uint32_t)(unsigned long long)(Y >> (F - 8)) ^ m) + c) - OZ_MAGIC;
#pragma unroll
        for (int p = 2; p <= S; ++p)
            f[p - 1] = __uint_as_float((((uint32_t)(unsigned long long)(Y >> (F - 8 * p)) & 255u) ^ m) + c) -
                       OZ_MAGIC;
    }
}

// The same digits of an FP32 element in 32-bit integers (S <= 3: Y < 2^(8S+3)
// fits 32 bits).  X = floor(|x| 2^(F-e)) does not depend on the format x is
// held in, so the digits equal those of x widened to FP64 (subnormal inputs
// included); Inf/NaN (whose row raised the flag) give unused digits.
template <int S>
__device__ __forceinline__ void oz_digit_floats(float x, int e, float (&f)[S])
{
    static_assert(8 * S + 3 <= 32, "the 32-bit digit form holds at most 3 slices");
    const uint32_t bits = __float_as_uint(x);
    const uint32_t m = (uint32_t)((int32_t)bits >> 31);
    const uint32_t c = m ? OZ_MAGIC_BITS + 129u : OZ_MAGIC_BITS - 128u;
    const int ex = (int)((bits >> 23) & 0xFFu);
    const uint32_t M = (bits & 0x7FFFFFu) | (ex ? 0x800000u : 0u);
    const int E2 = ex ? ex - 150 : -149;
    constexpr int F = 8 * S + 2;
    const int sh = E2 - e + F;  // U 2^F = M 2^sh < 2^(F-1)
    const uint32_t X = (sh >= 0) ? (sh < 32 ? M << sh : 0u) : (sh > -32 ? M >> (-sh) : 0u);
    const uint32_t Y = X + oz_bias<uint32_t>(S);
    f[0] = __uint_as_float(((Y >> (F - 8)) ^ m) + c) - OZ_MAGIC;
#pragma unroll
    for (int p = 2; p <= S; ++p) f[p - 1] = __uint_as_float((((Y >> (F - 8 * p)) & 255u) ^ m) + c) - OZ_MAGIC;
}

// Digits of two elements, slice by slice as bf16 pairs (x0 in the low half):
// one byte permute takes the upper halves of both fp32 images.
template <int S, typename T>
__device__ __forceinline__ void oz_digits_bf16x2(T x0, T x1, int e, uint32_t (&w)[S])
{
    float f0[S], f1[S];
    oz_digit_floats<S>(x0, e, f0);
    oz_digit_floats<S>(x1, e, f1);
#pragma unroll
    for (int p = 0; p < S; ++p) w[p] = __byte_perm(__float_as_uint(f0[p]), __float_as_uint(f1[p]), 0x7632);
}

__device__ __forceinline__ int oz_row_exponent(unsigned long long bits, int* nonfinite)
{
    if (bits == 0ull) return 0;
    if (bits >= 0x7FF0000000000000ull) {
        *nonfinite = 1;
        return 0;
    }
    // ilogb of a positive finite double from its bits, integers only (the
    // tiled split calls this in every thread; a library ilogb would run on
    // the FP64 pipe): the biased exponent for normal numbers, the position
    // of the leading mantissa bit for subnormals
    const int ex = (int)(bits >> 52);
    if (ex != 0) return ex - 1023 + 2;
    return (63 - __clzll((long long)bits)) - 1074 + 2;
}

// Tile of 32 rows x 64 k per block; writes S bf16 digit planes, K-major,
// zero in the padding.
template <int S, typename T = double>
__global__ void __launch_bounds__(256) oz_split_kernel(int64_t rows, int64_t k, const T* __restrict__ R,
                                                       int64_t sr, int64_t sl,
                                                       const unsigned long long* __restrict__ maxbits,
                                                       int64_t rpad, int64_t kpad,
                                                       uint16_t* __restrict__ out, int32_t* __restrict__ exps,
                                                       int* __restrict__ nonfinite)
{
    __shared__ T tile[32][65];
    const int64_t l0 = (int64_t)blockIdx.x * 64, r0 = (int64_t)blockIdx.y * 32;
    const bool rows_fast = (sr == 1);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int e = threadIdx.x + 256 * q;
        const int rr = rows_fast ? (e & 31) : (e >> 6);
        const int ll = rows_fast ? (e >> 5) : (e & 63);
        const int64_t r = r0 + rr, l = l0 + ll;
        tile[rr][ll] = (r < rows && l < k) ? __ldcs(R + r * sr + l * sl) : T(0);
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
    uint32_t packed[S][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        uint32_t w[S];
        oz_digits_bf16x2<S>(r < rows ? tile[rr][c0 + 2 * h] : T(0), r < rows ? tile[rr][c0 + 2 * h + 1] : T(0), e, w);
#pragma unroll
        for (int p = 0; p < S; ++p) packed[p][h] = w[p];
    }
#pragma unroll
    for (int p = 0; p < S; ++p) {
        uint4* dst = reinterpret_cast<uint4*>(out + ((int64_t)p * rpad + r) * kpad + l0 + c0);
        *dst = make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
    }
}

// ---------------------------------------------------------------- recombine
// T = sum_L a_L 2^(8L), the exact weighted sum of the level sums.  Four
// levels make a group that is exact in 64 bits (|a_L| < 2^31 P for P k parts:
// |group| < 2^(55.01) P, below 2^63 for P <= 64); for 32-bit a_L each term is
// one 32 x 32 -> 64-bit multiply-add, and only one 128-bit shift and add per
// group remains (against one of each per level in a 128-bit Horner loop).
template <int S, typename A>
__device__ __forceinline__ __int128 oz_weighted_sum(const A (&a)[S])
{
    constexpr int G = (S + 3) / 4;
    long long g[G];
#pragma unroll
    for (int gi = 0; gi < G; ++gi) {
        long long v = 0;
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (4 * gi + t < S) v += (long long)a[4 * gi + t] * (1ll << (8 * t));
        g[gi] = v;
    }
    __int128 T = g[G - 1];
#pragma unroll
    for (int gi = G - 2; gi >= 0; --gi) T = (__int128)((unsigned __int128)T << 32) + g[gi];
    return T;
}

// RNE(T * 2^E) from integers only, as IEEE bits.
__device__ __forceinline__ double round_scaled(__int128 T, int E)
{
    if (T == 0) return 0.0;
    const bool neg = T < 0;
    const unsigned __int128 u = neg ? (unsigned __int128)0 - (unsigned __int128)T : (unsigned __int128)T;
    const int msb = 127 - clz128(u);
    const int lead = msb + E;
    unsigned long long bits;
    if (lead >= -1022 && lead <= 1023) {
        // normal result: take the 64 bits below the leading one, round at bit 11
        unsigned long long top;
        bool rest = false;
        if (msb >= 63) {
            top = (unsigned long long)(u >> (msb - 63));
            rest = (msb > 63) && ((u & ((((unsigned __int128)1) << (msb - 63)) - 1)) != 0);
        } else {
            top = (unsigned long long)u << (63 - msb);
        }
        unsigned long long q = top >> 11;
        const unsigned long long rb = top & 0x7FFull;
        if (rb > 0x400ull || (rb == 0x400ull && (rest || (q & 1ull)))) q += 1;
        bits = ((unsigned long long)(lead + 1022) << 52) + q;  // q in [2^52, 2^53]
        if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    } else if (lead > 1023) {
        bits = 0x7FF0000000000000ull;
    } else {
        const int lsb = (lead >= -1022) ? lead - 52 : -1074;
        const int shift = lsb - E;
        unsigned __int128 q;
        if (shift <= 0) {
            q = u << (-shift);
        } else if (shift > 128) {
            q = 0;
        } else if (shift == 128) {
            q = (u > ((unsigned __int128)1 << 127)) ? 1 : 0;
        } else {
            q = u >> shift;
            const unsigned __int128 rem = u & ((((unsigned __int128)1) << shift) - 1);
            const unsigned __int128 half = ((unsigned __int128)1) << (shift - 1);
            if (rem > half || (rem == half && (q & 1))) q += 1;
        }
        bits = ((unsigned long long)(lsb + 1074) << 52) + (unsigned long long)q;
        if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    }
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

// round_scaled for a T that fits 64 bits (the digit form at S <= 4 slices:
// one group of oz_weighted_sum): the same RNE on 64-bit integers where the
// result is a normal number, the 128-bit routine otherwise.
__device__ __forceinline__ double round_scaled64(long long T, int E)
{
    if (T == 0) return 0.0;
    const bool neg = T < 0;
    const unsigned long long u = neg ? 0ull - (unsigned long long)T : (unsigned long long)T;
    const int msb = 63 - __clzll((long long)u);
    const int lead = msb + E;
    if (lead < -1022 || lead > 1023) return round_scaled((__int128)T, E);
    const unsigned long long top = u << (63 - msb);  // every bit of u is kept: no sticky bits below
    unsigned long long q = top >> 11;
    const unsigned long long rb = top & 0x7FFull;
    if (rb > 0x400ull || (rb == 0x400ull && (q & 1ull))) q += 1;
    unsigned long long bits = ((unsigned long long)(lead + 1022) << 52) + q;  // q in [2^52, 2^53]
    if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

template <int S, typename A>
__device__ __forceinline__ long long oz_weighted_sum64(const A (&a)[S])
{
    static_assert(S <= 4, "one 64-bit group");
    long long v = 0;
#pragma unroll
    for (int t = 0; t < S; ++t) v += (long long)a[t] * (1ll << (8 * t));
    return v;
}

struct OzRecombParams {
    int slices, nlevels;
    int64_t m, n, mpad, npad;
    const int32_t* planes;
    const int32_t* ea;
    const int32_t* eb;
    double alpha, beta;
    double* c;
    float* cf = nullptr;  // FP32 C instead (SGEMM's split form): RN32(alpha P + beta C) from the FP64 P
    int64_t rs_c, cs_c;
    const int* skip;
    int out_tri = 0, out_rpc = 1;  // only C's stored triangle is read and written (as OzA::out_tri)
    OzLevel lv[OZ_MAX_LEVELS];
};

// Thread per 4 consecutive rows of one column: all S level planes are
// loaded up front as 16-byte vectors (S x 16 B in flight per thread), then
// T = sum_l S_l 2^(8(s+1-l)) is formed by Horner from the most significant
// level (l = 2, last in the table) and rounded once.
template <int S>
__global__ void __launch_bounds__(256, (S <= 7 ? 3 : 2)) oz_recombine_kernel(const __grid_constant__ OzRecombParams p)
{
    if (*p.skip) return;
    const int64_t mq = (p.m + 3) >> 2;
    const int64_t total = mq * p.n;
    const bool plain = (p.alpha == 1.0 && p.beta == 0.0);
    bool one_part = true, few_parts = true;  // the level sums fit 32 bits / the groups fit 64 bits
#pragma unroll
    for (int L = 0; L < S; ++L) {
        one_part = one_part && p.lv[L].nparts == 1;
        few_parts = few_parts && p.lv[L].nparts <= 64;
    }
    const int64_t plane_stride = p.npad * p.mpad;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        // 32-bit division while the index fits (the 64-bit one costs several times more)
        const int64_t j = (total <= 0xFFFFFFFFll) ? (int64_t)((uint32_t)e / (uint32_t)mq) : e / mq;
        const int64_t i0 = (e - j * mq) * 4;
        // rows of column j's diagonal element: lower keeps rows >= dlo, upper rows <= dhi
        const int64_t dlo = (int64_t)p.out_rpc * j, dhi = dlo + p.out_rpc - 1;
        if (p.out_tri && (p.out_tri == 1 ? i0 + 3 < dlo : i0 > dhi)) continue;
        const int64_t off = j * p.mpad + i0;  // mpad is a multiple of 128: 16-byte aligned
        int4 v[S];
#pragma unroll
        for (int L = 0; L < S; ++L)
            v[L] = __ldcs(reinterpret_cast<const int4*>(p.planes + (int64_t)p.lv[L].plane_base * plane_stride + off));
        long long acc[S][4];
#pragma unroll
        for (int L = 0; L < S; ++L) {
            acc[L][0] = v[L].x;
            acc[L][1] = v[L].y;
            acc[L][2] = v[L].z;
            acc[L][3] = v[L].w;
            for (int pt = 1; pt < p.lv[L].nparts; ++pt) {
                const int4 w = __ldcs(reinterpret_cast<const int4*>(
                    p.planes + (int64_t)(p.lv[L].plane_base + pt) * plane_stride + off));
                acc[L][0] += w.x;
                acc[L][1] += w.y;
                acc[L][2] += w.z;
                acc[L][3] += w.w;
            }
        }
        const int ebj = p.eb[j] - 8 * (S + 1);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t i = i0 + r;
            if (i >= p.m) break;
            if (p.out_tri && (p.out_tri == 1 ? i < dlo : i > dhi)) continue;
            double ab;
            bool done = false;
            if constexpr (S <= 4) {
                if (few_parts) {  // |sum| < 2^63 (oz_weighted_sum): the 64-bit rounding
                    long long a[S];
#pragma unroll
                    for (int L = 0; L < S; ++L) a[L] = acc[L][r];
                    ab = round_scaled64(oz_weighted_sum64<S>(a), p.ea[i] + ebj);
                    done = true;
                }
            }
            if (!done) {
                __int128 T = 0;
                if (one_part) {
                    int a[S];
#pragma unroll
                    for (int L = 0; L < S; ++L) a[L] = (int)acc[L][r];
                    T = oz_weighted_sum<S>(a);
                } else if (few_parts) {
                    long long a[S];
#pragma unroll
                    for (int L = 0; L < S; ++L) a[L] = acc[L][r];
                    T = oz_weighted_sum<S>(a);
                } else {
#pragma unroll
                    for (int L = S - 1; L >= 0; --L)
                        T = (__int128)((unsigned __int128)T << 8) + (__int128)acc[L][r];
                }
                ab = round_scaled(T, p.ea[i] + ebj);
            }
            if (p.cf) {
                float* cij = p.cf + i * p.rs_c + j * p.cs_c;
                if (plain) {
                    *cij = (float)ab;
                } else {
                    const double t = __dmul_rn(p.alpha, ab);
                    *cij = (float)((p.beta == 0.0) ? t : __fma_rn(p.beta, (double)*cij, t));
                }
                continue;
            }
            double* cij = p.c + i * p.rs_c + j * p.cs_c;
            if (plain) {
                *cij = ab;
            } else {
                const double t = __dmul_rn(p.alpha, ab);
                *cij = (p.beta == 0.0) ? t : __fma_rn(p.beta, *cij, t);
            }
        }
    }
}

// ---------------------------------------------------------------- grouped form
// One block's share of a split with the row maxima taken in the same
// launch: 32 rows (r0 ..) of a row operand R (element (r, l) at
// R[r*sr + l*sl]) over the whole k range.  Pass 1 takes the row maxima
// (8 threads per row) and writes the rows' exponents; pass 2 cuts nkb
// 64-wide k blocks into digits, the next block's elements loaded into
// registers while one is cut, and hands each thread's 8 bf16 digits of a
// slice to store(p, kb, rr, c0, v) (slice p, k block kb, tile row rr,
// columns c0 .. c0 + 7).  Rows past `rows` and k past `k` give zero digits.
// T is double, or float for FP32 operands (each element widened exactly on
// load; the row maxima compare the FP32 bits, and only the maximum is
// widened to the FP64 bits oz_row_exponent reads).
template <int S, typename T, typename Store>
__device__ __forceinline__ void oz_split_unit(const T* __restrict__ R, int64_t rows, int64_t sr, int64_t sl,
                                              int64_t k, int nkb, int64_t r0, int32_t* __restrict__ exps,
                                              int* __restrict__ nonfinite, Store store)
{
    __shared__ T tile[32][65];
    __shared__ unsigned long long red[8][32];
    __shared__ int rowe[32];
    const bool rows_fast = (sr == 1);
    const int t = threadIdx.x;

    // pass 1: row maxima of |x| as IEEE bits
    {
        const int rr = rows_fast ? (t & 31) : (t >> 3);
        const int l0 = rows_fast ? (t >> 5) : (t & 7);
        const int64_t r = r0 + rr;
        OzKey<T> mx = 0, my = 0;
        if (r < rows) {
            int64_t l = l0;
            for (; l + 8 * 7 < k; l += 8 * 8) {  // eight loads in flight per thread
                OzKey<T> b[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) b[u] = oz_abs_key(__ldg(R + r * sr + (l + 8 * u) * sl));
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    mx = b[u] > mx ? b[u] : mx;
                    my = b[u + 1] > my ? b[u + 1] : my;
                }
            }
            for (; l < k; l += 8) {
                const OzKey<T> b = oz_abs_key(__ldg(R + r * sr + l * sl));
                mx = b > mx ? b : mx;
            }
        }
        red[rows_fast ? (t >> 5) : (t & 7)][rr] = mx > my ? mx : my;
    }
    __syncthreads();
    if (t < 32) {
        unsigned long long mx = 0;
#pragma unroll
        for (int g = 0; g < 8; ++g) mx = red[g][t] > mx ? red[g][t] : mx;
        int e = 0;
        const int64_t r = r0 + t;
        if (r < rows) {
            int nf = 0;
            e = oz_row_exponent(oz_key_f64<T>(mx), &nf);
            if (nf) *nonfinite = 1;
            exps[r] = e;
        }
        rowe[t] = e;
    }
    __syncthreads();

    // pass 2: digits, one 32 x 64 tile at a time
    const int rr = t >> 3, c0 = (t & 7) * 8;
    const int e = rowe[rr];
    const bool live = (r0 + rr < rows);
    T nxt[8];
    auto fetch = [&](int kb) {
        const int64_t l0 = (int64_t)kb * 64;
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const int idx = t + 256 * g;
            const int tr = rows_fast ? (idx & 31) : (idx >> 6);
            const int tl = rows_fast ? (idx >> 5) : (idx & 63);
            const int64_t r = r0 + tr, l = l0 + tl;
            nxt[g] = (r < rows && l < k) ? __ldg(R + r * sr + l * sl) : T(0);
        }
    };
    fetch(0);
    for (int kb = 0; kb < nkb; ++kb) {
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const int idx = t + 256 * g;
            tile[rows_fast ? (idx & 31) : (idx >> 6)][rows_fast ? (idx >> 5) : (idx & 63)] = nxt[g];
        }
        __syncthreads();
        if (kb + 1 < nkb) fetch(kb + 1);
        uint32_t packed[S][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint32_t w[S];
            oz_digits_bf16x2<S>(live ? tile[rr][c0 + 2 * h] : T(0), live ? tile[rr][c0 + 2 * h + 1] : T(0), e, w);
#pragma unroll
            for (int p = 0; p < S; ++p) packed[p][h] = w[p];
        }
#pragma unroll
        for (int p = 0; p < S; ++p) store(p, kb, rr, c0, make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]));
        __syncthreads();
    }
}

// Split of one operand of a single product with its row maxima in the same
// launch (oz_split_unit): block u owns rows 32u .. 32u + 31 of the padded
// row range, so the padding rows up to rpad and the k padding up to kpad
// are written as zeros, in the slice planes' layout of oz_split_kernel.
template <int S, typename T = double>
__global__ void __launch_bounds__(256, 2) oz_split_rows_kernel(int64_t rows, int64_t k, const T* __restrict__ R,
                                                            int64_t sr, int64_t sl, int64_t rpad, int64_t kpad,
                                                            uint16_t* __restrict__ out, int32_t* __restrict__ exps,
                                                            int* __restrict__ nonfinite)
{
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    oz_split_unit<S>(R, rows, sr, sl, k, (int)(kpad / 64), r0, exps, nonfinite,
                     [&](int p, int kb, int rr, int c0, uint4 v) {
                         *reinterpret_cast<uint4*>(out + ((int64_t)p * rpad + r0 + rr) * kpad + kb * 64 + c0) = v;
                     });
}

// Both operands of one product in one launch (oz_split_unit): blocks
// [0, units_a) take rows of op(A), the rest rows of op(B)^T; each operand's
// padding rows up to its plane height are written as zeros.
struct OzSplitOperand {
    const double* R;
    int64_t rows, sr, sl, rpad;
    uint16_t* out;
    int32_t* exps;
};

template <int S>
__global__ void __launch_bounds__(256, 2) oz_split_two_kernel(OzSplitOperand a, OzSplitOperand b, int64_t units_a,
                                                           int64_t k, int64_t kpad, int* __restrict__ nonfinite)
{
    const bool isb = (int64_t)blockIdx.x >= units_a;
    const OzSplitOperand& o = isb ? b : a;
    const int64_t r0 = ((int64_t)blockIdx.x - (isb ? units_a : 0)) * 32;
    oz_split_unit<S>(o.R, o.rows, o.sr, o.sl, k, (int)(kpad / 64), r0, o.exps, nonfinite,
                     [&](int p, int kb, int rr, int c0, uint4 v) {
                         *reinterpret_cast<uint4*>(o.out + ((int64_t)p * o.rpad + r0 + rr) * kpad + kb * 64 + c0) = v;
                     });
}

// ---------------------------------------------------------------- grouped form
// Split for every problem of a batch in one launch.  A block owns 32 rows of
// op(A_i) or op(B_i)^T over the whole k range (oz_split_unit) and writes
// them into the problem's boxes.  Only blocks holding rows of the matrix
// run; their rows past m (n) and k past k_i up to the block width are
// written as zeros, and the remaining padding rows of a box stay as the
// plan's one-time zero fill left them.
template <int S, typename T>
__global__ void __launch_bounds__(256, (sizeof(T) == 4) ? 4 : 2) oz_split_batch_kernel(const OzBatchProb* __restrict__ probs,
                                                             const int32_t* __restrict__ unit_prob,
                                                             const int64_t* __restrict__ unit_base,
                                                             int64_t boxes_a, int64_t boxes_b,
                                                             uint16_t* __restrict__ sa, uint16_t* __restrict__ sb,
                                                             int* __restrict__ nonfinite)
{
    const int pi = unit_prob[blockIdx.x];
    const OzBatchProb& q = probs[pi];
    int64_t u = (int64_t)blockIdx.x - unit_base[pi];
    const bool isb = (u >= q.units_a);
    if (isb) u -= q.units_a;
    const int box_rows = isb ? OZ_BN : OZ_BM;
    const int box_shift = isb ? 8 : 7;  // log2 of box_rows: shifts, not a 64-bit division
    static_assert(OZ_BN == 256 && OZ_BM == 128, "box heights");
    const int64_t r0 = u * 32;
    uint16_t* out = isb ? sb : sa;
    const int64_t boxes = isb ? boxes_b : boxes_a;
    const int64_t box0 = (isb ? q.bbox : q.abox) + (r0 >> box_shift) * q.kb;
    const int64_t rb = r0 & (box_rows - 1);
    oz_split_unit<S>(static_cast<const T*>(isb ? q.b : q.a), isb ? q.n : q.m, isb ? q.brs : q.ars, isb ? q.bcs : q.acs, q.k, q.kb, r0,
                     isb ? q.eb : q.ea, nonfinite, [&](int p, int kb, int rr, int c0, uint4 v) {
                         const int64_t z = (int64_t)p * boxes + box0 + kb;
                         *reinterpret_cast<uint4*>(out + (z * box_rows + rb + rr) * 64 + c0) = v;
                     });
}

// Recombination for every problem of a batch in one launch: blocks are
// assigned to problems by a table, each thread takes 4 rows of one column.
// CT is C's type: for FP32, C = RN32(alpha P + beta C) from the FP64 product
// P, as the single-problem SGEMM split form rounds it.
template <int S, typename CT>
__global__ void __launch_bounds__(256) oz_recombine_batch_kernel(const OzBatchProb* __restrict__ probs,
                                                                 const int32_t* __restrict__ block_prob,
                                                                 const int64_t* __restrict__ block_base,
                                                                 const int* __restrict__ skip)
{
    if (*skip) return;
    const int pi = block_prob[blockIdx.x];
    const OzBatchProb& q = probs[pi];
    // C's own orientation (see OzBatchProb)
    const int64_t m = q.swap ? q.n : q.m, n = q.swap ? q.m : q.n;
    const int32_t* ea = q.swap ? q.eb : q.ea;
    const int32_t* eb = q.swap ? q.ea : q.eb;
    const int64_t mq = (m + 3) >> 2;
    const int64_t e = ((int64_t)blockIdx.x - block_base[pi]) * 256 + threadIdx.x;
    if (e >= mq * n) return;
    // 32-bit division while the index fits (the 64-bit one is a library call)
    const int64_t j = (mq * n <= 0xFFFFFFFFll) ? (int64_t)((uint32_t)e / (uint32_t)mq) : e / mq;
    const int64_t i0 = (e - j * mq) * 4;
    const int64_t plane_stride = n * q.ld;
    const int32_t* src = q.planes + j * q.ld + i0;  // ld is a multiple of 4: 16-byte aligned
    int4 v[S];
#pragma unroll
    for (int L = 0; L < S; ++L) v[L] = __ldcs(reinterpret_cast<const int4*>(src + (int64_t)L * plane_stride));
    const bool plain = (q.alpha == 1.0 && q.beta == 0.0);
    const int ebj = eb[j] - 8 * (S + 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int64_t i = i0 + r;
        if (i >= m) break;
        int a[S];
#pragma unroll
        for (int L = 0; L < S; ++L) a[L] = (r == 0) ? v[L].x : (r == 1) ? v[L].y : (r == 2) ? v[L].z : v[L].w;
        double ab;
        if constexpr (S <= 4) ab = round_scaled64(oz_weighted_sum64<S>(a), ea[i] + ebj);
        else ab = round_scaled(oz_weighted_sum<S>(a), ea[i] + ebj);
        CT* cij = static_cast<CT*>(q.c) + i * q.rs_c + j * q.cs_c;
        if (plain) {
            *cij = (CT)ab;
        } else {
            const double tt = __dmul_rn(q.alpha, ab);
            *cij = (CT)((q.beta == 0.0) ? tt : __fma_rn(q.beta, (double)*cij, tt));
        }
    }
}

// ---------------------------------------------------------------- CRT form
// The second precision form (Ozaki, Uchino & Imamura, "Ozaki scheme II", 2025,
// restated here with bf16 residues): every row of op(A) and of op(B)^T is
// scaled to integers, X = RNE(|x| 2^(t+1-e)) with the sign of x (|X| <= 2^t,
// e the row exponent of the digit form), so A'B' is an exact integer matrix
// with |C'| <= k 2^(2t).  For N pairwise coprime moduli p_l <= 257 with
// product M > 2 (17/16) k 2^(2t), the N products (A' mod p_l)(B' mod p_l)
// (symmetric residues, |r| <= 128: exact in bf16, products <= 2^14 as for
// the digits) determine C' by the Chinese remainder theorem.  N products
// replace the digit form's s(s+1)/2: at k = 16384, N = 16 gives t = 55,
// the representation error of s = 7 digits (28 products).
//
// Split: X's bytes b_q, s_l = sum_q b_q (2^(8q) mod p_l) < 2^19 (exact in
// fp32), r_l = s_l - p_l rint(s_l / p_l) (exact: |s_l / p_l - half integer|
// >= 1/514 dwarfs the fp32 error).  Recombination: the int32 products c_l
// reduced to symmetric residues, C' = sum_l r_l W_l - Q M in 128-bit
// two's-complement arithmetic (W_l the CRT weights, symmetric mod M), with
// Q = rint(sum_l r_l (W_l / M)) in fp32 (error below 2^-9 while
// |C'/M| < 0.471); then one RNE conversion of C' 2^(e_i + e_j - 2t - 2).
constexpr int OZC_MAX = 16;

struct OzCrtTab {
    int n, t;
    float p[OZC_MAX], invp[OZC_MAX], wm[OZC_MAX];
    float pw[OZC_MAX][6];  // 2^(12q) mod p_l
    float pw14[OZC_MAX][4];  // 2^(14q) mod p_l, symmetric (|.| <= p_l / 2)
    int wd[OZC_MAX][4];    // W_l = sum_q wd[l][q] 2^(32q), signed 32-bit digits
    int md[4];             // M in the same digits
};


// |x| 2^(t+1-e), rounded to the nearest integer (ties to even), from the bits.
__device__ __forceinline__ unsigned long long oz_crt_scaled(unsigned long long bits, int e, int t)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long M = (bits & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0ull);
    if (M == 0) return 0ull;
    const int E2 = ex ? ex - 1075 : -1074;
    const int sh = E2 + t + 1 - e;
    if (sh >= 0) return M << sh;  // |x| 2^(t+1-e) < 2^t
    if (sh < -54) return 0ull;    // below half a unit
    const int r = -sh;
    const unsigned long long q = M >> r, rem = M & ((1ull << r) - 1), half = 1ull << (r - 1);
    return (rem > half || (rem == half && (q & 1ull))) ? q + 1 : q;
}

// The N residues of x as floats (integers, |r| <= 128), from NL limbs of LB bits of X
// carrying x's sign: s_l = sum_q h_q (2^(LB q) mod p_l).  Four 14-bit limbs with the
// symmetric table (t <= 55: X <= 2^55 < 2^56) give |s_l| < 4 2^14 2^7 = 2^23; five or six
// 12-bit limbs with the non-negative one (t <= 59, else t <= 71) give |s_l| < 6 2^12 2^8 <
// 2^22.6.  Either is exact in fp32, and rint(s_l / p_l) by one fma onto 1.5 2^23 (unit in
// the last place 1) is exact: the fma rounds s_l invp_l, which differs from s_l / p_l by at
// most |s_l| 2^-24 / p_l < 1 / (2 p_l), while a non-integral s_l / p_l is at least
// 1 / (2 p_l) from a half-integer.  s_l - rint(s_l / p_l) p_l is then the symmetric residue
// of the signed value.
template <int N, int NL, int LB>
__device__ __forceinline__ void oz_crt_residues(double x, int e, const OzCrtTab& tab, float (&r)[N])
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned long long X = oz_crt_scaled(bits & 0x7FFFFFFFFFFFFFFFull, e, tab.t);
    // limb q of X as a float with x's sign: the limb's bits OR-ed into +-2^23, minus +-2^23
    const uint32_t sgn = (uint32_t)(bits >> 32) & 0x80000000u;
    const float off = sgn ? 8388608.0f : -8388608.0f;
    float h[NL];
#pragma unroll
    for (int q = 0; q < NL; ++q)
        h[q] = __uint_as_float(sgn | 0x4B000000u | (uint32_t)((X >> (LB * q)) & ((1u << LB) - 1u))) + off;
#pragma unroll
    for (int l = 0; l < N; ++l) {
        float sl = 0.0f;
#pragma unroll
        for (int q = 0; q < NL; ++q) sl = __fmaf_rn(h[q], LB == 14 ? tab.pw14[l][q] : tab.pw[l][q], sl);
        const float q = __fmaf_rn(sl, tab.invp[l], OZ_MAGIC) - OZ_MAGIC;
        r[l] = __fmaf_rn(-q, tab.p[l], sl);
    }
}

// Tile of 32 rows x 64 k per block (as oz_split_kernel); writes N bf16
// residue planes, K-major, zero in the padding.  Warp w converts rows 4w ..
// 4w + 3 in turn, lane c elements 2c and 2c + 1 of the row: every plane store
// of a warp is one contiguous 128-byte line.
template <int N, int NL, int LB>
__global__ void __launch_bounds__(256, 4) oz_crt_split_kernel(int64_t rows, int64_t k, const double* __restrict__ R,
                                                           int64_t sr, int64_t sl,
                                                           const unsigned long long* __restrict__ maxbits,
                                                           int64_t rpad, int64_t kpad, uint16_t* __restrict__ out,
                                                           int32_t* __restrict__ exps, int* __restrict__ nonfinite,
                                                           const __grid_constant__ OzCrtTab tab)
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
        tile[rr][ll] = (r < rows && l < k) ? __ldcs(R + r * sr + l * sl) : 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t plane_words = rpad * kpad / 2;  // one residue plane in 32-bit words
#pragma unroll 1
    for (int h = 0; h < 4; ++h) {
        const int rr = warp * 4 + h;
        const int64_t r = r0 + rr;
        int e = 0;
        if (r < rows) {
            int nf = 0;
            e = oz_row_exponent(maxbits[r], &nf);
            if (nf) *nonfinite = 1;
            if (blockIdx.x == 0 && lane == 0) exps[r] = e;
        }
        float f0[N], f1[N];
        oz_crt_residues<N, NL, LB>(r < rows ? tile[rr][2 * lane] : 0.0, e, tab, f0);
        oz_crt_residues<N, NL, LB>(r < rows ? tile[rr][2 * lane + 1] : 0.0, e, tab, f1);
        // kpad and l0 are multiples of 64: the pair's 4 bytes are aligned
        uint32_t* dst = reinterpret_cast<uint32_t*>(out + r * kpad + l0) + lane;
#pragma unroll
        for (int l = 0; l < N; ++l)
            dst[(int64_t)l * plane_words] = __byte_perm(__float_as_uint(f0[l]), __float_as_uint(f1[l]), 0x7632);
    }
}

// Thread per 4 consecutive rows of one column, as oz_recombine_kernel: the
// N product planes (one part each), CRT into 128 bits, one rounding.
template <int N>
__global__ void __launch_bounds__(256, 2) oz_crt_recombine_kernel(const __grid_constant__ OzRecombParams p,
                                                                  const __grid_constant__ OzCrtTab tab)
{
    if (*p.skip) return;
    const int64_t mq = (p.m + 3) >> 2;
    const int64_t total = mq * p.n;
    const bool plain = (p.alpha == 1.0 && p.beta == 0.0);
    const int64_t plane_stride = p.npad * p.mpad;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        // 32-bit division while the index fits (the 64-bit one costs several times more)
        const int64_t j = (total <= 0xFFFFFFFFll) ? (int64_t)((uint32_t)e / (uint32_t)mq) : e / mq;
        const int64_t i0 = (e - j * mq) * 4;
        const int64_t dlo = (int64_t)p.out_rpc * j, dhi = dlo + p.out_rpc - 1;
        if (p.out_tri && (p.out_tri == 1 ? i0 + 3 < dlo : i0 > dhi)) continue;
        const int64_t off = j * p.mpad + i0;
        // four int16 residues of consecutive rows per plane (8-byte aligned: mpad and i0 are
        // multiples of 4), sign-extended
        const int16_t* planes16 = reinterpret_cast<const int16_t*>(p.planes);
        int4 v[N];
#pragma unroll
        for (int L = 0; L < N; ++L) {
            const uint2 raw =
                __ldcs(reinterpret_cast<const uint2*>(planes16 + (int64_t)p.lv[L].plane_base * plane_stride + off));
            v[L] = make_int4((int)(int16_t)(raw.x & 0xFFFFu), (int)raw.x >> 16, (int)(int16_t)(raw.y & 0xFFFFu),
                             (int)raw.y >> 16);
        }
        const int ebj = p.eb[j] - 2 * tab.t - 2;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t i = i0 + r;
            if (i >= p.m) break;
            if (p.out_tri && (p.out_tri == 1 ? i < dlo : i > dhi)) continue;
            // sum_l r_l W_l - Q M in signed 32-bit digits: S_q = sum_l r_l wd[l][q] - Q md[q]
            // (|r_l| <= 129, |S_q| < 2^45), then one 128-bit combination
            long long S0 = 0, S1 = 0, S2 = 0, S3 = 0;
            float qf = 0.0f;
#pragma unroll
            for (int L = 0; L < N; ++L) {
                // the slice GEMM stored the symmetric residue (|rr| <= p_l / 2 <= 128)
                const int rr = (r == 0) ? v[L].x : (r == 1) ? v[L].y : (r == 2) ? v[L].z : v[L].w;
                S0 += (long long)rr * tab.wd[L][0];
                S1 += (long long)rr * tab.wd[L][1];
                S2 += (long long)rr * tab.wd[L][2];
                S3 += (long long)rr * tab.wd[L][3];
                // float(rr) from the bits of 1.5 2^23 + rr
                qf = __fmaf_rn(__int_as_float(0x4B400000 + rr) - OZ_MAGIC, tab.wm[L], qf);
            }
            const int Q = __float_as_int(qf + OZ_MAGIC) - 0x4B400000;  // rint(qf), |qf| < 2^12
            S0 -= (long long)Q * tab.md[0];
            S1 -= (long long)Q * tab.md[1];
            S2 -= (long long)Q * tab.md[2];
            S3 -= (long long)Q * tab.md[3];
            // modulo 2^128 (the true |C'| is below 2^127)
            const unsigned __int128 acc = (unsigned __int128)(__int128)S0 +
                                          ((unsigned __int128)(__int128)S1 << 32) +
                                          ((unsigned __int128)(__int128)S2 << 64) +
                                          ((unsigned __int128)(__int128)S3 << 96);
            const __int128 C = (__int128)acc;
            const double ab = round_scaled(C, p.ea[i] + ebj);
            double* cij = p.c + i * p.rs_c + j * p.cs_c;
            if (plain) {
                *cij = ab;
            } else {
                const double t = __dmul_rn(p.alpha, ab);
                *cij = (p.beta == 0.0) ? t : __fma_rn(p.beta, *cij, t);
            }
        }
    }
}

void launch_recombine(int slices, const OzRecombParams& r, unsigned blocks, cudaStream_t s)
{
    switch (slices) {
#define GB_RECOMB_CASE(S) \
    case S: oz_recombine_kernel<S><<<blocks, 256, 0, s>>>(r); break;
        GB_RECOMB_CASE(2) GB_RECOMB_CASE(3) GB_RECOMB_CASE(4) GB_RECOMB_CASE(5) GB_RECOMB_CASE(6)
        GB_RECOMB_CASE(7) GB_RECOMB_CASE(8) GB_RECOMB_CASE(9) GB_RECOMB_CASE(10) GB_RECOMB_CASE(11)
        GB_RECOMB_CASE(12)
#undef GB_RECOMB_CASE
    default: break;
    }
}

// Moduli of the CRT form, largest first: pairwise coprime (257, 251, 241, 239,
// 233, 229, 227, 223, 211, 199, 197 prime; 256 = 2^8, 255 = 3 5 17,
// 253 = 11 23, 247 = 13 19, 217 = 7 31), each at most 257 so that a
// symmetric residue has |r| <= 128.
constexpr int OZC_MODULI[OZC_MAX] = {257, 256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199, 197};

using u128 = unsigned __int128;

u128 crt_modulus(int n)
{
    u128 M = 1;
    for (int l = 0; l < n; ++l) M *= (u128)OZC_MODULI[l];
    return M;
}

int modinv_small(int a, int p)
{
    // a^-1 mod p for gcd(a, p) = 1, extended Euclid on small integers
    int t = 0, nt = 1, r = p, nr = a % p;
    while (nr != 0) {
        const int q = r / nr, tt = t - q * nt, tr = r - q * nr;
        t = nt;
        nt = tt;
        r = nr;
        nr = tr;
    }
    return t < 0 ? t + p : t;
}

// x = sum_q d[q] 2^(32q) with d[q] in [-2^31, 2^31) (|x| < 2^127)
void signed_digits32(__int128 x, int (&d)[4])
{
    for (int q = 0; q < 4; ++q) {
        const int dq = (int)(uint32_t)(u128)x;  // x mod 2^32, as a signed value
        d[q] = dq;
        x = (x - (__int128)dq) / ((__int128)1 << 32);  // exact
    }
}

void crt_table(int n, int t, OzCrtTab* tab)
{
    *tab = OzCrtTab();
    tab->n = n;
    tab->t = t;
    const u128 M = crt_modulus(n);
    for (int l = 0; l < n; ++l) {
        const int pl = OZC_MODULI[l];
        const u128 Ml = M / (u128)pl;
        const int inv = modinv_small((int)(Ml % (u128)pl), pl);
        u128 W = (Ml * (u128)inv) % M;  // W = 1 mod p_l, 0 mod the others
        __int128 Ws = (W > M / 2) ? (__int128)W - (__int128)M : (__int128)W;
        signed_digits32(Ws, tab->wd[l]);
        tab->wm[l] = (float)((double)Ws / (double)M);
        tab->p[l] = (float)pl;
        tab->invp[l] = 1.0f / (float)pl;
        int pw = 1 % pl;
        for (int q = 0; q < 6; ++q) {
            tab->pw[l][q] = (float)pw;
            pw = (pw * 4096) % pl;
        }
        pw = 1 % pl;
        for (int q = 0; q < 4; ++q) {
            tab->pw14[l][q] = (float)(2 * pw > pl ? pw - pl : pw);
            pw = (pw * 16384) % pl;
        }
    }
    signed_digits32((__int128)M, tab->md);
}

template <int N>
void launch_crt_split(int64_t rows, int64_t k, const double* R, int64_t sr, int64_t sl, const unsigned long long* mb,
                      int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out, int32_t* ex, int* nonfinite,
                      const OzCrtTab& tab, cudaStream_t s)
{
    LaunchScope ls("oz_split_crt", s);
    const dim3 grid((unsigned)(kpad / 64), (unsigned)(rcover / 32));
    if (tab.t <= 55)  // X <= 2^55: four 14-bit limbs
        oz_crt_split_kernel<N, 4, 14><<<grid, 256, 0, s>>>(rows, k, R, sr, sl, mb, rpad, kpad, out, ex, nonfinite, tab);
    else if (tab.t <= 59)  // X <= 2^59: five 12-bit limbs
        oz_crt_split_kernel<N, 5, 12><<<grid, 256, 0, s>>>(rows, k, R, sr, sl, mb, rpad, kpad, out, ex, nonfinite, tab);
    else
        oz_crt_split_kernel<N, 6, 12><<<grid, 256, 0, s>>>(rows, k, R, sr, sl, mb, rpad, kpad, out, ex, nonfinite, tab);
}

template <int N>
void launch_crt_recombine(const OzRecombParams& r, const OzCrtTab& tab, unsigned blocks, cudaStream_t s)
{
    oz_crt_recombine_kernel<N><<<blocks, 256, 0, s>>>(r, tab);
}

#define GB_CRT_CASES(X) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16)

void crt_split_dispatch(int n, int64_t rows, int64_t k, const double* R, int64_t sr, int64_t sl,
                        const unsigned long long* mb, int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out,
                        int32_t* ex, int* nonfinite, const OzCrtTab& tab, cudaStream_t s)
{
    switch (n) {
#define GB_CRT_SPLIT(N) \
    case N: launch_crt_split<N>(rows, k, R, sr, sl, mb, rpad, rcover, kpad, out, ex, nonfinite, tab, s); break;
        GB_CRT_CASES(GB_CRT_SPLIT)
#undef GB_CRT_SPLIT
    default: break;
    }
}

void crt_recombine_dispatch(int n, const OzRecombParams& r, const OzCrtTab& tab, unsigned blocks, cudaStream_t s)
{
    switch (n) {
#define GB_CRT_RECOMB(N) \
    case N: launch_crt_recombine<N>(r, tab, blocks, s); break;
        GB_CRT_CASES(GB_CRT_RECOMB)
#undef GB_CRT_RECOMB
    default: break;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* ptr = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

// Slice planes [slice][plane_rows][kpad] bf16 as a 3-D tensor map of rpad
// rows from base (rows r0 .. r0 + rpad of the planes when base is offset by
// r0 rows); plane_rows = 0 means rpad.
int make_slice_map(CUtensorMap* map, const void* base, int64_t kpad, int64_t rpad, int slices,
                   int box_rows, int64_t plane_rows = 0)
{
    auto fn = encode_fn();
    if (!fn) return set_error(GB_ERR_CUDA, "ozaki", "cuTensorMapEncodeTiled unavailable");
    if (plane_rows <= 0) plane_rows = rpad;
    cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rpad, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)(kpad * 2), (cuuint64_t)(plane_rows * kpad * 2)};
    cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                    estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GB_ERR_CUDA, "ozaki", "cuTensorMapEncodeTiled failed");
    return GB_SUCCESS;
}

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Tile rows per raster group of the slice GEMM (GB_OZAKI_GROUP_M, 1..64).
int group_m_setting()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("GB_OZAKI_GROUP_M");
        const int g = e ? atoi(e) : OZ_GROUP_M;
        v = (g >= 1 && g <= 64) ? g : OZ_GROUP_M;
    }
    return v;
}

// Whether the grouped form may run a problem as C^T (GB_OZAKI_BATCH_ORIENT,
// default 1; 0 keeps every problem as given).
int ozaki_batch_orient_setting()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("GB_OZAKI_BATCH_ORIENT");
        v = e ? (atoi(e) != 0) : 1;
    }
    return v;
}

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

// Slice-GEMM engine: 1 = one CTA per 128x256 tile, 2 = CTA pairs per
// 256x256 tile (cta_group::2).  gb_set_ozaki_ctas() or the environment
// variable GB_OZAKI_CTAS select; the pair form is the default.
static int g_ozaki_ctas = -1;

// The engine setting: 1 or 2 forced (gb_set_ozaki_ctas, GB_OZAKI_CTAS), 0 chosen per
// product (the selector's engine output, else the occupancy rule below).
int ozaki_ctas_setting()
{
    if (g_ozaki_ctas < 0) {
        const char* e = getenv("GB_OZAKI_CTAS");
        const int v = e ? atoi(e) : 0;
        g_ozaki_ctas = (v == 1 || v == 2) ? v : 0;
    }
    return g_ozaki_ctas;
}

int set_ozaki_ctas(int ctas)
{
    if (ctas != 0 && ctas != 1 && ctas != 2)
        return set_error(GB_ERR_ARG, "gb_set_ozaki_ctas", "ctas must be 0 (per product), 1 or 2");
    g_ozaki_ctas = ctas;
    return GB_SUCCESS;
}

thread_local int t_ozaki_ctas = 0;  // the engine of the product being prepared on this thread

// The engine a product's operands are prepared for: the per-product choice,
// else the forced setting, else CTA pairs.
int ozaki_engine()
{
    if (t_ozaki_ctas) return t_ozaki_ctas;
    const int v = ozaki_ctas_setting();
    return v ? v : 2;
}

// Engine for an m x n x k product when the setting leaves the choice per product:
// the selector's engine output for a shape it has decided (the host entry points
// ask it before the product; device entry points never wait for an inference), else
// CTA pairs for products of at least 2^30 FP64-equivalent flops and single CTAs
// below (on the engine-tuned training shapes single CTAs won 70% of the time,
// mostly the small ones; at 16384^3 the two are within 1%).
int ozaki_engine_choice(int64_t m, int64_t n, int64_t k)
{
    const int v = ozaki_ctas_setting();
    if (v) return v;
    const int eng = selector_auto() ? selector_cached_engine(m, n, k) : 0;
    if (eng) return eng;
    return (2.0 * (double)m * (double)n * (double)k >= 1073741824.0) ? 2 : 1;
}

struct EngineScope {
    int prev;
    explicit EngineScope(int e) : prev(t_ozaki_ctas) { t_ozaki_ctas = e; }
    ~EngineScope() { t_ozaki_ctas = prev; }
};

namespace {

// The split launchers take the slice planes' row stride (rpad) apart from
// the rows they cover (rcover, a multiple of 32): a block of rows r0.. of a
// larger operand is split by passing R, mb, out and ex offset to row r0.
template <int S, typename T>
void launch_split(int64_t rows, int64_t k, const T* R, int64_t sr, int64_t sl,
                  const unsigned long long* mb, int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out,
                  int32_t* ex, int* nonfinite, cudaStream_t s)
{
    LaunchScope ls("oz_split", s);
    oz_split_kernel<S, T><<<dim3((unsigned)(kpad / 64), (unsigned)(rcover / 32)), 256, 0, s>>>(
        rows, k, R, sr, sl, mb, rpad, kpad, out, ex, nonfinite);
}

void split_dispatch(int slices, int64_t rows, int64_t k, const double* R, int64_t sr, int64_t sl,
                    const unsigned long long* mb, int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out,
                    int32_t* ex, int* nonfinite, cudaStream_t s)
{
    switch (slices) {
#define GB_SPLIT_CASE(S) \
    case S: launch_split<S>(rows, k, R, sr, sl, mb, rpad, rcover, kpad, out, ex, nonfinite, s); break;
        GB_SPLIT_CASE(2) GB_SPLIT_CASE(3) GB_SPLIT_CASE(4) GB_SPLIT_CASE(5) GB_SPLIT_CASE(6)
        GB_SPLIT_CASE(7) GB_SPLIT_CASE(8) GB_SPLIT_CASE(9) GB_SPLIT_CASE(10) GB_SPLIT_CASE(11)
        GB_SPLIT_CASE(12)
#undef GB_SPLIT_CASE
    default: break;
    }
}

// The fused split (row maxima and digits in one launch, no maxima array)
// for k up to GB_OZAKI_FUSED_SPLIT_K (default 4096).  Beyond it the two
// passes of a block over its rows outgrow what L2 keeps between them: at
// 16384^3 on GB300 the fused form took 5.6 ms against 4.6 ms for the
// row-maximum kernel plus the tiled split, while the TRSM updates (k up to
// 4096, many small launches) ran 2-3% faster fused.
int64_t fused_split_max_k()
{
    static int64_t v = -1;
    if (v < 0) {
        const char* e = getenv("GB_OZAKI_FUSED_SPLIT_K");
        v = e ? atoll(e) : 4096;
        if (v < 0) v = 0;
    }
    return v;
}

template <int S, typename T>
void launch_split_rows(int64_t rows, int64_t k, const T* R, int64_t sr, int64_t sl, int64_t rpad,
                       int64_t rcover, int64_t kpad, uint16_t* out, int32_t* ex, int* nonfinite, cudaStream_t s)
{
    LaunchScope ls("oz_split_rows", s);
    oz_split_rows_kernel<S, T><<<(unsigned)(rcover / 32), 256, 0, s>>>(rows, k, R, sr, sl, rpad, kpad, out, ex,
                                                                        nonfinite);
}

template <typename T>
void launch_rowmax(int64_t rows, int64_t k, const T* R, int64_t sr, int64_t sl, unsigned long long* mb,
                   cudaStream_t s);

// Row maxima and digit slices of one row operand (or of rows r0.. of one,
// with R, mb, out and ex offset to row r0 and rcover rows covered): fused
// for small k, else the row-maximum kernel into mb (zeroed here) and the
// tiled split.
void split_operand(int slices, int64_t rows, int64_t k, const double* R, int64_t sr, int64_t sl,
                   unsigned long long* mb, int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out, int32_t* ex,
                   int* nonfinite, cudaStream_t s)
{
    if (k <= fused_split_max_k() && rcover / 32 <= INT32_MAX) {
        switch (slices) {
#define GB_SPLIT_CASE(S) \
    case S: launch_split_rows<S>(rows, k, R, sr, sl, rpad, rcover, kpad, out, ex, nonfinite, s); break;
            GB_SPLIT_CASE(2) GB_SPLIT_CASE(3) GB_SPLIT_CASE(4) GB_SPLIT_CASE(5) GB_SPLIT_CASE(6)
            GB_SPLIT_CASE(7) GB_SPLIT_CASE(8) GB_SPLIT_CASE(9) GB_SPLIT_CASE(10) GB_SPLIT_CASE(11)
            GB_SPLIT_CASE(12)
#undef GB_SPLIT_CASE
        default: break;
        }
        return;
    }
    cudaMemsetAsync(mb, 0, sizeof(unsigned long long) * rows, s);
    launch_rowmax(rows, k, R, sr, sl, mb, s);
    split_dispatch(slices, rows, k, R, sr, sl, mb, rpad, rcover, kpad, out, ex, nonfinite, s);
}

// split_operand for FP32 rows at the SGEMM split form's slice count: the
// same launches reading 4-byte elements (digits cut from the FP32 bits).
// The fused form gives each CTA 32 whole rows: for FP32 it pays only on
// short rows or with four CTAs per SM to run (SGEMM 4096^3: 0.28 ms fused
// against 0.14 ms for the row maxima and the tiled split).
void split_operand_f32(int64_t rows, int64_t k, const float* R, int64_t sr, int64_t sl, unsigned long long* mb,
                       int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out, int32_t* ex, int* nonfinite,
                       cudaStream_t s)
{
    constexpr int S = GB_SGEMM_SPLIT_SLICES;
    const int64_t sms = sm_count() > 0 ? sm_count() : 148;
    if (k <= fused_split_max_k() && rcover / 32 <= INT32_MAX && (k <= 256 || rcover / 32 >= 4 * sms)) {
        launch_split_rows<S>(rows, k, R, sr, sl, rpad, rcover, kpad, out, ex, nonfinite, s);
        return;
    }
    cudaMemsetAsync(mb, 0, sizeof(unsigned long long) * rows, s);
    launch_rowmax(rows, k, R, sr, sl, mb, s);
    launch_split<S>(rows, k, R, sr, sl, mb, rpad, rcover, kpad, out, ex, nonfinite, s);
}

// The CRT form's split of one row operand: row maxima, then the residues.
void crt_split_operand(int n, int t, int64_t rows, int64_t k, const double* R, int64_t sr, int64_t sl,
                       unsigned long long* mb, int64_t rpad, int64_t rcover, int64_t kpad, uint16_t* out, int32_t* ex,
                       int* nonfinite, cudaStream_t s)
{
    OzCrtTab tab;
    crt_table(n, t, &tab);
    cudaMemsetAsync(mb, 0, sizeof(unsigned long long) * rows, s);
    launch_rowmax(rows, k, R, sr, sl, mb, s);
    crt_split_dispatch(n, rows, k, R, sr, sl, mb, rpad, rcover, kpad, out, ex, nonfinite, tab, s);
}

}  // namespace

// Largest K of one part of a level with `npairs` slice products:
// npairs * Kpart * 128^2 < 2^31, Kpart a multiple of the 64-wide k block.
int64_t ozaki_kpart_limit(int npairs)
{
    int64_t lim = (int64_t)2147483647 / ((int64_t)npairs * 128 * 128);
    lim = (lim / OZ_BK) * OZ_BK;
    return lim < OZ_BK ? OZ_BK : lim;
}

// log2 of the largest |T| the recombination can meet (must stay < 126).
double ozaki_t_bound_log2(int s, int64_t k)
{
    double t = 0.0;
    for (int l = 2; l <= s + 1; ++l) {
        const int np = (l - 1 < s) ? l - 1 : s;
        t += (double)np * (double)k * 16384.0 * ldexp(1.0, 8 * (s + 1 - l));
    }
    return log2(t);
}

namespace {

template <typename T>
void launch_rowmax(int64_t rows, int64_t k, const T* R, int64_t sr, int64_t sl, unsigned long long* mb,
                   cudaStream_t s)
{
    const int sms = sm_count() > 0 ? sm_count() : 148;
    if (sr == 1) {
        const int64_t gx = (rows + 255) / 256;
        int64_t gy = ((int64_t)sms * 8 + gx - 1) / gx;
        if (gy > k) gy = k;
        if (gy > 65535) gy = 65535;
        const int64_t kchunk = (k + gy - 1) / gy;
        gy = (k + kchunk - 1) / kchunk;
        LaunchScope ls("oz_rowmax", s);
        oz_rowmax_rows_kernel<T><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(rows, k, R, sl, kchunk, mb);
    } else {
        const int64_t gx = (rows * 32 + 255) / 256;
        int64_t gy = ((int64_t)sms * 8 + gx - 1) / gx;
        if (gy > (k + 255) / 256) gy = (k + 255) / 256;
        if (gy < 1) gy = 1;
        if (gy > 65535) gy = 65535;
        const int64_t kchunk = (k + gy - 1) / gy;
        gy = (k + kchunk - 1) / kchunk;
        LaunchScope ls("oz_rowmax", s);
        oz_rowmax_warp_kernel<T><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(rows, k, R, sr, sl, kchunk, mb);
    }
}

// One-time kernel attributes of the slice GEMM engines and the number of
// CTA pairs that fit at once.
int slice_gemm_setup(int* max_pairs)
{
    static bool attr_set = false;
    static int pairs = 0;
    int rc;
    if (!attr_set) {
        const int sms = sm_count() > 0 ? sm_count() : 148;
        if ((rc = check_cuda(cudaFuncSetAttribute(ozaki_slice_gemm_kernel<OzGemmParams>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_BYTES),
                             "smem attr")))
            return rc;
        if ((rc = check_cuda(cudaFuncSetAttribute(ozaki_slice_gemm_pair_kernel,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, OZ2_SMEM_BYTES),
                             "smem attr")))
            return rc;
        cudaLaunchConfig_t qc = {};
        cudaLaunchAttribute qa[1];
        qa[0].id = cudaLaunchAttributeClusterDimension;
        qa[0].val.clusterDim.x = 2;
        qa[0].val.clusterDim.y = 1;
        qa[0].val.clusterDim.z = 1;
        qc.gridDim = dim3(2 * (unsigned)(sms / 2));
        qc.blockDim = dim3(OZ_THREADS);
        qc.dynamicSmemBytes = OZ2_SMEM_BYTES;
        qc.attrs = qa;
        qc.numAttrs = 1;
        if ((rc = check_cuda(cudaOccupancyMaxActiveClusters(&pairs, ozaki_slice_gemm_pair_kernel, &qc),
                             "cluster occupancy")))
            return rc;
        attr_set = true;
    }
    *max_pairs = pairs;
    return GB_SUCCESS;
}

}  // namespace

// Phase 1 of the Ozaki form: row maxima, exponents and digit slices of op(A)
// (element (i, l) = a[i*ars + l*acs]), kept in HBM for any number of
// multiplications.  The Inf/NaN flag lives here and is shared by them.
// ozaki_alloc_a sets up the arena; ozaki_split_a_rows splits a block of rows
// (several blocks may be split as they arrive); ozaki_prepare_a does both.
int ozaki_crt_bits(int n, int64_t k)
{
    if (n < 2 || n > OZC_MAX || k < 1) return -1;
    const u128 M = crt_modulus(n);
    const u128 lim = (M / 17) * 8 + ((M % 17) * 8) / 17;  // floor(8 M / 17): M > 2 (17/16) k 2^(2t)
    int kb = 0;
    while (kb < 63 && ((int64_t)1 << kb) < k) ++kb;  // k <= 2^kb
    for (int t = 62; t >= 1; --t) {
        if (2 * t + kb > 126) continue;
        if (((u128)k << (2 * t)) <= lim) return t;
    }
    return -1;
}

int ozaki_crt_moduli_for_bits(int bits, int64_t k)
{
    for (int n = 2; n <= OZC_MAX; ++n)
        if (ozaki_crt_bits(n, k) >= bits) return n;
    return -1;
}

int ozaki_alloc_a(int64_t m, int64_t k, const double* a, int64_t ars, int64_t acs, int slices, cudaStream_t s,
                  OzA* A)
{
    *A = OzA();
    if (ozaki_form() == 1) {
        // CRT form: `slices` moduli, one product (one int32 part) each
        if (slices < 2 || slices > OZC_MAX)
            return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "moduli must be in [2, 16]");
        A->crt_t = ozaki_crt_bits(slices, k);
        if (A->crt_t < 1)
            return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "too few moduli for this k");
        if (round_up(k, OZ_BK) > ozaki_kpart_limit(1))
            return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "k beyond the CRT form's one-part limit");
        A->crt = 1;
    } else {
        if (slices < 2 || slices > OZ_MAX_SLICES)
            return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "slices must be in [2, 12]");
        if (ozaki_t_bound_log2(slices, k) >= 126.0)
            return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "slices and k exceed the 128-bit recombination range");
    }
    A->pair_form = (ozaki_engine() == 2);
    A->row_tile = A->pair_form ? 2 * OZ2_ROWS : OZ_BM;
    A->slices = slices;
    A->m = m;
    A->k = k;
    A->kpad = round_up(k, OZ_BK);
    A->mpad = round_up(m, A->row_tile);
    if (A->mpad > INT32_MAX || A->kpad > INT32_MAX)
        return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "dimension too large for TMA coordinates");
    A->a = a;
    A->ars = ars;
    A->acs = acs;
    const size_t bytes_sa = (size_t)slices * A->mpad * A->kpad * 2;
    const size_t bytes_aux = sizeof(unsigned long long) * m + sizeof(int32_t) * m + 64;
    A->ws = static_cast<uint8_t*>(dev_alloc(bytes_sa + bytes_aux + 1024, s));
    if (!A->ws) return GB_ERR_NOMEM;
    A->sa = reinterpret_cast<uint16_t*>(A->ws);
    A->maxa = reinterpret_cast<unsigned long long*>(A->ws + bytes_sa);
    A->ea = reinterpret_cast<int32_t*>(A->maxa + m);
    A->nonfinite = reinterpret_cast<int*>(A->ea + m);
    const int rc = check_cuda(cudaMemsetAsync(A->nonfinite, 0, sizeof(int), s), "memset");
    if (rc) ozaki_release_a(A, s);
    return rc;
}

// Rows [r0, r1) of op(A); r0 a multiple of the row tile, r1 one too or m.
int ozaki_split_a_rows(const OzA* A, int64_t r0, int64_t r1, cudaStream_t s)
{
    if (r0 < 0 || r1 > A->m || r0 >= r1 || r0 % A->row_tile || (r1 != A->m && r1 % A->row_tile))
        return set_error(GB_ERR_ARG, "ozaki", "row block not aligned to the slice GEMM tile");
    const int64_t cover = (r1 == A->m ? A->mpad : r1) - r0;
    if (A->crt)
        crt_split_operand(A->slices, A->crt_t, r1 - r0, A->k, A->a + r0 * A->ars, A->ars, A->acs, A->maxa + r0,
                          A->mpad, cover, A->kpad, A->sa + r0 * A->kpad, A->ea + r0, A->nonfinite, s);
    else
        split_operand(A->slices, r1 - r0, A->k, A->a + r0 * A->ars, A->ars, A->acs, A->maxa + r0, A->mpad, cover,
                      A->kpad, A->sa + r0 * A->kpad, A->ea + r0, A->nonfinite, s);
    return check_cuda(cudaGetLastError(), "oz_split");
}

int ozaki_prepare_a(int64_t m, int64_t k, const double* a, int64_t ars, int64_t acs, int slices,
                    cudaStream_t s, OzA* A)
{
    int rc = ozaki_alloc_a(m, k, a, ars, acs, slices, s, A);
    if (rc) return rc;
    if ((rc = ozaki_split_a_rows(A, 0, m, s))) ozaki_release_a(A, s);
    return rc;
}

void ozaki_release_a(OzA* A, cudaStream_t s)
{
    dev_free(A->ws, s);
    A->ws = nullptr;
}

// Phase 2: the exponents and digit slices of an op(B) of n columns
// ((l, j) = b[l*brs + j*bcs]) for multiplications by a prepared op(A).
// Columns of op(B) are split independently, so a product done in column
// blocks gives the same bits as one call.
int ozaki_alloc_b(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, cudaStream_t s, OzB* B)
{
    *B = OzB();
    B->n = n;
    B->npad = round_up(n, OZ_BN);
    if (B->npad > INT32_MAX) return set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "dimension too large for TMA coordinates");
    B->b = b;
    B->brs = brs;
    B->bcs = bcs;
    const size_t bytes_sb = (size_t)A->slices * B->npad * A->kpad * 2;
    const size_t bytes_aux = sizeof(unsigned long long) * n + sizeof(int32_t) * n + 64;
    B->ws = static_cast<uint8_t*>(dev_alloc(bytes_sb + bytes_aux + 1024, s));
    if (!B->ws) return GB_ERR_NOMEM;
    B->sb = reinterpret_cast<uint16_t*>(B->ws);
    B->maxb = reinterpret_cast<unsigned long long*>(B->ws + bytes_sb);
    B->eb = reinterpret_cast<int32_t*>(B->maxb + n);
    return GB_SUCCESS;
}

int ozaki_prepare_b(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, cudaStream_t s, OzB* B)
{
    int rc = ozaki_alloc_b(A, n, b, brs, bcs, s, B);
    if (rc) return rc;
    // rows of op(B)^T: (j, l) = b[l*brs + j*bcs]
    if (A->crt)
        crt_split_operand(A->slices, A->crt_t, n, A->k, b, bcs, brs, B->maxb, B->npad, B->npad, A->kpad, B->sb,
                          B->eb, A->nonfinite, s);
    else
        split_operand(A->slices, n, A->k, b, bcs, brs, B->maxb, B->npad, B->npad, A->kpad, B->sb, B->eb,
                      A->nonfinite, s);
    rc = check_cuda(cudaGetLastError(), "oz_split");
    if (rc) ozaki_release_b(B, s);
    return rc;
}

void ozaki_release_b(OzB* B, cudaStream_t s)
{
    dev_free(B->ws, s);
    B->ws = nullptr;
}

// Tables of the tiles holding part of C's stored triangle (OzGemmParams::
// out_tri): kept tiles before each tile row, and each row's first column
// tile.  One thread; the host counts the same tiles for the item total.
__global__ void oz_tri_tiles_kernel(int tiles_m, int tiles_n, int64_t row_tile, int64_t m, int rpc, int out_tri,
                                    int* __restrict__ cum, int* __restrict__ first)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int total = 0;
    for (int tm = 0; tm < tiles_m; ++tm) {
        const int64_t r_lo = (int64_t)tm * row_tile;
        const int64_t r_hi = (((int64_t)(tm + 1) * row_tile < m) ? (int64_t)(tm + 1) * row_tile : m) - 1;
        int f = 0, cnt;
        if (out_tri == 1) {
            int64_t last = (r_hi / rpc) / OZ_BN;
            if (last > tiles_n - 1) last = tiles_n - 1;
            cnt = (int)last + 1;
        } else {
            const int64_t f64 = (r_lo / rpc) / OZ_BN;
            f = (int)(f64 < tiles_n ? f64 : tiles_n);
            cnt = tiles_n - f;
        }
        cum[tm] = total;
        first[tm] = f;
        total += cnt;
    }
    cum[tiles_m] = total;
}

int64_t oz_tri_tiles_count(int tiles_m, int tiles_n, int64_t row_tile, int64_t m, int rpc, int out_tri)
{
    int64_t total = 0;
    for (int tm = 0; tm < tiles_m; ++tm) {
        const int64_t r_lo = (int64_t)tm * row_tile;
        const int64_t r_hi = (((int64_t)(tm + 1) * row_tile < m) ? (int64_t)(tm + 1) * row_tile : m) - 1;
        if (out_tri == 1) {
            int64_t last = (r_hi / rpc) / OZ_BN;
            if (last > tiles_n - 1) last = tiles_n - 1;
            total += last + 1;
        } else {
            const int64_t f = (r_lo / rpc) / OZ_BN;
            total += tiles_n - (f < tiles_n ? f : tiles_n);
        }
    }
    return total;
}

// The IEEE fallback's diagonal block: C := D + beta C on the stored triangle
// of the rows x cols block at (r0, c0) (row i, column j stored when i / rpc
// >= j, lower, or <= j, upper); runs only when a split raised the flag.
__global__ void __launch_bounds__(256) oz_tri_merge_gated_kernel(int64_t rows, int64_t cols, int64_t r0, int64_t c0,
                                                                 int lower, int rpc, const double* __restrict__ d,
                                                                 double beta, double* __restrict__ c, int64_t rs_c,
                                                                 int64_t cs_c, const int* __restrict__ gate)
{
    if (!*gate) return;
    const int64_t total = rows * cols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / rows, i = e - j * rows;
        const int64_t ci = (r0 + i) / rpc, cj = c0 + j;
        if (lower ? ci < cj : ci > cj) continue;
        double* cij = c + (r0 + i) * rs_c + cj * cs_c;
        *cij = (beta == 0.0) ? d[e] : __fma_rn(beta, *cij, d[e]);
    }
}

// Phase 3: C := alpha op(A) op(B) + beta C for rows [r0, r0 + rows) of the
// prepared op(A) (r0 a multiple of the row tile) and a prepared op(B); C is
// that rows x n block; the slice GEMM, the recombination and the gated IEEE
// fallback.
namespace {

// FP32 operands and C of SGEMM's split form (multiply_rows_impl): C is written
// in FP32 by the recombination, and the IEEE fallback reads these operands.
struct OzF32 {
    const float* a;
    const float* b;
    float* c;
};

int multiply_rows_impl(const OzA* A, int64_t r0, int64_t rows, const OzB* B, double alpha, double beta, double* c,
                       int64_t rs_c, int64_t cs_c, const OzF32* f32, cudaStream_t s);

}  // namespace

int ozaki_multiply_rows(const OzA* A, int64_t r0, int64_t rows, const OzB* B, double alpha, double beta, double* c,
                        int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    return multiply_rows_impl(A, r0, rows, B, alpha, beta, c, rs_c, cs_c, nullptr, s);
}

namespace {

int multiply_rows_impl(const OzA* A, int64_t r0, int64_t rows, const OzB* B, double alpha, double beta, double* c,
                       int64_t rs_c, int64_t cs_c, const OzF32* f32, cudaStream_t s)
{
    if (r0 < 0 || rows <= 0 || r0 + rows > A->m || r0 % A->row_tile)
        return set_error(GB_ERR_ARG, "ozaki", "row block not aligned to the slice GEMM tile");
    if (f32 && (A->out_tri || A->crt))
        return set_error(GB_ERR_ARG, "ozaki", "the FP32 form writes a whole C from the digit form");
    note_ozaki_slices(A->slices);
    if (A->out_tri && (r0 != 0 || rows != A->m || A->tri || A->out_rpc < 1))
        return set_error(GB_ERR_ARG, "ozaki", "a triangle of C is written from the whole of op(A) only");
    const int64_t m = rows, n = B->n, k = A->k, kpad = A->kpad, npad = B->npad;
    const int64_t mpad = round_up(rows, A->row_tile);
    const int slices = A->slices;
    const bool pair_form = A->pair_form;
    const int kb_total = (int)(kpad / OZ_BK);

    OzGemmParams p;
    p.slices = slices;
    p.nlevels = slices;
    p.kb_total = kb_total;
    p.tiles_m = (int)(mpad / A->row_tile);
    p.tiles_n = (int)(npad / OZ_BN);
    const int64_t tiles = A->out_tri ? oz_tri_tiles_count(p.tiles_m, p.tiles_n, A->row_tile, m, A->out_rpc, A->out_tri)
                                     : (int64_t)p.tiles_m * p.tiles_n;
    int planes_total = 0;
    int64_t items = 0;
    for (int L = 0; L < slices && A->crt; ++L) {  // CRT form: modulus L + 1 is A_(L+1) B_(L+1)^T alone
        OzLevel& lv = p.lv[L];
        lv.lev = 2 * (L + 1);
        lv.pa_lo = L + 1;
        lv.npairs = 1;
        lv.nparts = 1;
        lv.kb_per_part = kb_total;
        lv.plane_base = planes_total;
        lv.item_base = items;
        planes_total += 1;
        items += tiles;
    }
    for (int L = 0; L < slices && !A->crt; ++L) {  // heaviest level (most pairs) first
        OzLevel& lv = p.lv[L];
        lv.lev = slices + 1 - L;
        lv.pa_lo = (lv.lev - slices > 1) ? lv.lev - slices : 1;
        const int pa_hi = (lv.lev - 1 < slices) ? lv.lev - 1 : slices;
        lv.npairs = pa_hi - lv.pa_lo + 1;
        const int64_t lim_kb = ozaki_kpart_limit(lv.npairs) / OZ_BK;
        lv.nparts = (int)((kb_total + lim_kb - 1) / lim_kb);
        lv.kb_per_part = (kb_total + lv.nparts - 1) / lv.nparts;
        lv.plane_base = planes_total;
        lv.item_base = items;
        planes_total += lv.nparts;
        items += (int64_t)lv.nparts * tiles;
    }
    p.items = items;
    p.chunk_kb = chunk_kb_setting();
    p.group_m = group_m_setting();
    p.mpad = mpad;
    p.npad = npad;
    p.m = m;
    p.n = n;
    p.tri_mode = A->tri;
    p.tri_rows = (int)A->row_tile;
    p.tri_row0 = r0;

    if (A->crt) {
        OzCrtTab tab;
        crt_table(slices, A->crt_t, &tab);
        p.crt = 1;
        for (int L = 0; L < slices; ++L) {
            const int pm = (int)tab.p[L];
            const int w = 65536 % pm;
            p.crt_p[L] = tab.p[L];
            p.crt_invp[L] = tab.invp[L];
            p.crt_w16[L] = (float)(2 * w > pm ? w - pm : w);
        }
    }
    // CRT planes hold int16 residues, the digit form's int32 level sums
    const size_t bytes_pl = (size_t)planes_total * npad * mpad * (A->crt ? 2 : 4);
    const size_t bytes_tab = A->out_tri ? sizeof(int) * (size_t)(2 * p.tiles_m + 1) : 0;
    int32_t* planes = static_cast<int32_t*>(dev_alloc(bytes_pl + 1024 + bytes_tab, s));
    if (!planes) return GB_ERR_NOMEM;
    if (A->out_tri) {
        int* tab = reinterpret_cast<int*>(reinterpret_cast<uint8_t*>(planes) + bytes_pl + 1024);
        p.out_tri = A->out_tri;
        p.tiles_valid = (int)tiles;
        p.tile_cum = tab;
        p.tile_first = tab + p.tiles_m + 1;
        LaunchScope ls("oz_tri_tiles", s);
        oz_tri_tiles_kernel<<<1, 1, 0, s>>>(p.tiles_m, p.tiles_n, A->row_tile, m, A->out_rpc, A->out_tri, tab,
                                            tab + p.tiles_m + 1);
    }
    p.planes = planes;
    p.status = device_status_word();
    p.skip = A->nonfinite;
    p.counter = nullptr;

    int rc = GB_SUCCESS;
    auto bail = [&](int code) { dev_free(planes, s); return code; };
    CUtensorMap map_a, map_b;
    if ((rc = make_slice_map(&map_a, A->sa + r0 * kpad, kpad, mpad, slices, OZ_BM, A->mpad))) return bail(rc);
    if ((rc = make_slice_map(&map_b, B->sb, kpad, npad, slices, pair_form ? OZ2_ROWS : OZ_BN))) return bail(rc);
    int max_pairs = 0;
    if ((rc = slice_gemm_setup(&max_pairs))) return bail(rc);
    const int sms = sm_count() > 0 ? sm_count() : 148;
    if (pair_form) {
        if (max_pairs < 1) return bail(set_error(GB_ERR_UNSUPPORTED, "ozaki", "no CTA pair fits on this GPU"));
        const int npair = (int)((p.items < max_pairs) ? p.items : max_pairs);
        p.sched_p = npair;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(2 * (unsigned)npair);
        cfg.blockDim = dim3(OZ_THREADS);
        cfg.dynamicSmemBytes = OZ2_SMEM_BYTES;
        cfg.stream = s;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        LaunchScope ls("ozaki_slice_gemm", s);
        rc = check_cuda(cudaLaunchKernelEx(&cfg, ozaki_slice_gemm_pair_kernel, map_a, map_b, p), "pair launch");
        if (rc) return bail(rc);
    } else {
        const int grid = (int)((p.items < sms) ? p.items : sms);
        p.sched_p = grid;
        LaunchScope ls("ozaki_slice_gemm", s);
        ozaki_slice_gemm_kernel<OzGemmParams><<<grid, OZ_THREADS, OZ_SMEM_BYTES, s>>>(map_a, map_b, p);
    }
    if ((rc = check_cuda(cudaGetLastError(), "ozaki_slice_gemm"))) return bail(rc);
    {
        OzRecombParams r;
        r.slices = slices;
        r.nlevels = slices;
        r.m = m;
        r.n = n;
        r.mpad = mpad;
        r.npad = npad;
        r.planes = planes;
        r.ea = A->ea + r0;
        r.eb = B->eb;
        r.alpha = alpha;
        r.beta = beta;
        r.c = c;
        r.cf = f32 ? f32->c : nullptr;
        r.rs_c = rs_c;
        r.cs_c = cs_c;
        r.skip = A->nonfinite;
        r.out_tri = A->out_tri;
        r.out_rpc = A->out_rpc;
        for (int L = 0; L < slices; ++L) r.lv[L] = p.lv[L];
        const int64_t total = ((m + 3) / 4) * n;
        int64_t blocks = (total + 255) / 256;
        if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
        LaunchScope ls("oz_recombine", s);
        if (A->crt) {
            OzCrtTab tab;
            crt_table(slices, A->crt_t, &tab);
            crt_recombine_dispatch(slices, r, tab, (unsigned)blocks, s);
        } else {
            launch_recombine(slices, r, (unsigned)blocks, s);
        }
    }
    if ((rc = check_cuda(cudaGetLastError(), "oz_recombine"))) return bail(rc);
    // IEEE path for non-finite operands: runs only when a split raised the flag
    if (f32) {
        rc = sgemm_native_gated(m, n, k, (float)alpha, f32->a + r0 * A->ars, A->ars, A->acs, f32->b, B->brs, B->bcs,
                                (float)beta, f32->c, rs_c, cs_c, A->nonfinite, s);
    } else if (!A->out_tri) {
        rc = dgemm_native_gated(m, n, k, alpha, A->a + r0 * A->ars, A->ars, A->acs, B->b, B->brs, B->bcs, beta, c,
                                rs_c, cs_c, A->nonfinite, s);
    } else {
        // only the stored triangle: per 1024-column block, the rows strictly
        // inside it in place, the diagonal block through scratch and a merge
        const int64_t rpc = A->out_rpc, W = 1024;
        const int64_t wmax = (n < W) ? n : W;
        // the diagonal-block scratch reuses the level planes, which the recombination (ordered
        // before it on s) has finished reading; a separate buffer only if they are too small
        const size_t dbytes = sizeof(double) * (size_t)(rpc * wmax * wmax);
        double* own = nullptr;
        double* d = reinterpret_cast<double*>(planes);
        if (dbytes > bytes_pl) {
            own = static_cast<double*>(dev_alloc(dbytes, s));
            if (!own) return bail(GB_ERR_NOMEM);
            d = own;
        }
        const bool lower = (A->out_tri == 1);
        for (int64_t j0 = 0; j0 < n && !rc; j0 += W) {
            const int64_t w = (n - j0 < W) ? n - j0 : W;
            const int64_t d0 = rpc * j0, dr = (rpc * (j0 + w) < m ? rpc * (j0 + w) : m) - d0;
            const int64_t pr0 = lower ? d0 + dr : 0, prows = lower ? m - (d0 + dr) : d0;
            const double* bj = B->b + j0 * B->bcs;
            if (prows > 0)
                rc = dgemm_native_gated(prows, w, k, alpha, A->a + pr0 * A->ars, A->ars, A->acs, bj, B->brs, B->bcs,
                                        beta, c + pr0 * rs_c + j0 * cs_c, rs_c, cs_c, A->nonfinite, s);
            if (!rc && dr > 0) {
                rc = dgemm_native_gated(dr, w, k, alpha, A->a + d0 * A->ars, A->ars, A->acs, bj, B->brs, B->bcs, 0.0,
                                        d, 1, dr, A->nonfinite, s);
                if (!rc) {
                    int64_t blocks = (dr * w + 255) / 256;
                    if (blocks > 4096) blocks = 4096;
                    LaunchScope ls("oz_tri_merge_gated", s);
                    oz_tri_merge_gated_kernel<<<(unsigned)blocks, 256, 0, s>>>(dr, w, d0, j0, lower ? 1 : 0, (int)rpc,
                                                                               d, beta, c, rs_c, cs_c, A->nonfinite);
                    rc = check_cuda(cudaGetLastError(), "ozaki triangle fallback");
                }
            }
        }
        if (own) dev_free(own, s);
    }
    dev_free(planes, s);
    return rc;
}

}  // namespace

// Phases 2 and 3 for all rows of op(A).
int ozaki_multiply(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, double alpha, double beta,
                   double* c, int64_t rs_c, int64_t cs_c, cudaStream_t s)
{
    OzB B;
    int rc = ozaki_prepare_b(A, n, b, brs, bcs, s, &B);
    if (rc) return rc;
    rc = ozaki_multiply_rows(A, 0, A->m, &B, alpha, beta, c, rs_c, cs_c, s);
    ozaki_release_b(&B, s);
    return rc;
}

namespace {

template <int S>
void launch_split_two(const OzA* A, const OzB* B, cudaStream_t s)
{
    OzSplitOperand oa{A->a, A->m, A->ars, A->acs, A->mpad, A->sa, A->ea};
    OzSplitOperand ob{B->b, B->n, B->bcs, B->brs, B->npad, B->sb, B->eb};  // rows of op(B)^T
    const int64_t ua = A->mpad / 32, ub = B->npad / 32;
    LaunchScope ls("oz_split_rows", s);
    oz_split_two_kernel<S><<<(unsigned)(ua + ub), 256, 0, s>>>(oa, ob, ua, A->k, A->kpad, A->nonfinite);
}

}  // namespace

int dgemm_ozaki(int64_t m, int64_t n, int64_t k, double alpha,
                const double* a, int64_t ars, int64_t acs,
                const double* b, int64_t brs, int64_t bcs, double beta,
                double* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0 || k <= 0) return scal_matrix(m, n, beta, c, rs_c, cs_c, s);
    EngineScope engine(t_ozaki_ctas ? t_ozaki_ctas : ozaki_engine_choice(m, n, k));
    OzA A;
    int rc;
    if (k > fused_split_max_k() || ozaki_form() == 1) {  // the CRT form always splits in two passes
        if ((rc = ozaki_prepare_a(m, k, a, ars, acs, slices, s, &A))) return rc;
        rc = ozaki_multiply(&A, n, b, brs, bcs, alpha, beta, c, rs_c, cs_c, s);
        ozaki_release_a(&A, s);
        return rc;
    }
    // both operands split by one launch (the fused form: small k, so one launch saves a launch
    // per product, e.g. half the split launches of a trsm)
    if ((rc = ozaki_alloc_a(m, k, a, ars, acs, slices, s, &A))) return rc;
    OzB B;
    if ((rc = ozaki_alloc_b(&A, n, b, brs, bcs, s, &B))) {
        ozaki_release_a(&A, s);
        return rc;
    }
    if ((A.mpad + B.npad) / 32 > INT32_MAX) rc = set_error(GB_ERR_ARG, "gb_dgemm_ozaki", "operands too large");
    if (!rc) {
        switch (slices) {
#define GB_SPLIT_CASE(S) \
    case S: launch_split_two<S>(&A, &B, s); break;
            GB_SPLIT_CASE(2) GB_SPLIT_CASE(3) GB_SPLIT_CASE(4) GB_SPLIT_CASE(5) GB_SPLIT_CASE(6)
            GB_SPLIT_CASE(7) GB_SPLIT_CASE(8) GB_SPLIT_CASE(9) GB_SPLIT_CASE(10) GB_SPLIT_CASE(11)
            GB_SPLIT_CASE(12)
#undef GB_SPLIT_CASE
        default: break;
        }
        rc = check_cuda(cudaGetLastError(), "oz_split");
    }
    if (!rc) rc = ozaki_multiply_rows(&A, 0, m, &B, alpha, beta, c, rs_c, cs_c, s);
    ozaki_release_b(&B, s);
    ozaki_release_a(&A, s);
    return rc;
}

namespace {

__global__ void oz_flag_or_kernel(const int* __restrict__ fa, const int* __restrict__ fb, int* __restrict__ out)
{
    *out = (*fa | *fb) ? 1 : 0;
}

}  // namespace

// out = fa | fb on s: the Inf/NaN flag of one block product of a blocked
// Ozaki product, from the flags of the row block and the column block it
// reads (each raised by that block's own split, complete before the product).
// A flag shared by all blocks could be raised by a later block's split
// between one product's recombination and its gated fallback.
int ozaki_flag_or(const int* fa, const int* fb, int* out, cudaStream_t s)
{
    LaunchScope ls("oz_flag_or", s);
    oz_flag_or_kernel<<<1, 1, 0, s>>>(fa, fb, out);
    return check_cuda(cudaGetLastError(), "ozaki flag");
}

// GB_OZAKI_DEV_BLOCKS=RxC fixes the row and column block counts of the
// blocked forms (1x1: one product); read per call (one getenv against a
// large product).  Unset or malformed: *r = *c = 0.
void ozaki_fixed_blocks(int* r, int* c)
{
    *r = *c = 0;
    const char* e = getenv("GB_OZAKI_DEV_BLOCKS");
    int rr = 0, cc = 0;
    if (e && sscanf(e, "%dx%d", &rr, &cc) == 2 && rr >= 1 && rr <= 16 && cc >= 1 && cc <= 16) {
        *r = rr;
        *c = cc;
    }
}

// The Ozaki form of dgemm_ozaki on device buffers in blocks, for the device
// entry points' large products: op(A) in row blocks and op(B) in column
// blocks, split on a stream of their own, every (row block, column block) of C
// one slice GEMM with its recombination and gated fallback, the block
// products alternating between the caller's stream and a second compute
// stream.  One block's recombination and the later blocks' splits then run
// beside another block's product instead of before and after the whole one
// (the host entry points' pipeline, without the copies).  Rows and columns
// are split independently, so with finite operands the result is
// bit-identical to dgemm_ozaki; a block whose row or column block holds an
// Inf or NaN is computed by the native kernel (ozaki_flag_or), the others
// stay in the Ozaki form.  Stream-ordered on s: nothing here waits for the device.
int dgemm_ozaki_blocks(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t ars, int64_t acs,
                       const double* b, int64_t brs, int64_t bcs, double beta, double* c, int64_t rs_c, int64_t cs_c,
                       int slices, cudaStream_t s)
{
    int fix_r = 0, fix_c = 0;
    ozaki_fixed_blocks(&fix_r, &fix_c);
    // 8 row blocks x up to 4 column blocks where they measured faster than one product on GB300
    // (ms: digit form s = 7 at 8192^3 19.9 -> 18.7 in 8 x 4, ZGEMM 4096^3's real 8192 x 4096 x
    // 8192 product 9.40 -> 9.16 in 8 x 2; CRT form, 16 moduli, 94.6 -> 87.1 at 16384^3 but
    // 12.7 -> 13.6 at 8192^3, where the blocks' smaller products lose more than the overlap
    // saves); one product otherwise
    // (every grid measured had k >= 8192; below k = 2048 the blocks' launches would outweigh
    // the overlap, so one product)
    const bool crt = (ozaki_form() == 1);
    int nch = (k < 2048) ? 1
                         : crt ? ((m >= 16384 && n >= 16384) ? 4 : 1)
                               : ((m >= 8192 && n >= 4096) ? (int)std::min<int64_t>(4, n / 2048) : 1);
    if (fix_c) nch = (int)((fix_c < n) ? fix_c : 1);
    if (m <= 0 || n <= 0 || alpha == 0.0 || k <= 0 || nch < 2 || m < 2048 || (fix_r == 1 && fix_c == 1))
        return dgemm_ozaki(m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, slices, s);
    EngineScope engine(t_ozaki_ctas ? t_ozaki_ctas : ozaki_engine_choice(m / 4, n / nch, k));
    cudaStream_t sp[2] = {s, thread_aux_stream(0)}, ss = thread_aux_stream(1);
    OzA prep;
    int rc = ozaki_alloc_a(m, k, a, ars, acs, slices, s, &prep);
    if (rc) return rc;
    // row blocks on the slice GEMM's row tile
    const int nra = fix_r ? fix_r : 8;  // m >= 8192: row blocks of at least 1024 rows
    std::vector<int64_t> rb(1, 0);
    for (int i = 1; i < nra; ++i) {
        const int64_t r = (m * i / nra + prep.row_tile - 1) / prep.row_tile * prep.row_tile;
        if (r > rb.back() && r < m) rb.push_back(r);
    }
    rb.push_back(m);
    const int na = (int)rb.size() - 1;
    // Inf/NaN flags: one per row block, per column block and per block product
    int* flags = static_cast<int*>(dev_alloc(sizeof(int) * (size_t)(na + nch + na * nch), s));
    if (!flags) {
        ozaki_release_a(&prep, s);
        return GB_ERR_NOMEM;
    }
    rc = check_cuda(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(na + nch + na * nch), s), "memset flags");
    int *fa = flags, *fb = flags + na, *fab = flags + na + nch;
    auto with_flag = [&](int* f) {
        OzA x = prep;
        x.nonfinite = f;
        return x;
    };
    // events: the fork, A blocks split, B blocks split, the second compute stream's and the
    // split stream's ends
    std::vector<cudaEvent_t> ev((size_t)(1 + na + nch + 2), nullptr);
    for (auto& e : ev)
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "ozaki blocks events");
    cudaEvent_t ev_fork = ev[0], *ev_sa = ev.data() + 1, *ev_sb = ev_sa + na, ev_aux_done = ev_sb[nch],
                ev_split_done = ev_sb[nch + 1];
    auto col0 = [&](int j) { return n * j / nch; };
    std::vector<OzB> pb((size_t)nch);
    if (!rc) {
        // the other streams start after the caller's work so far and prep's allocation
        cudaEventRecord(ev_fork, s);
        cudaStreamWaitEvent(sp[1], ev_fork, 0);
        cudaStreamWaitEvent(ss, ev_fork, 0);
        for (int i = 0; i < na && !rc; ++i) {
            const OzA ai = with_flag(fa + i);
            rc = ozaki_split_a_rows(&ai, rb[i], rb[i + 1], ss);
            cudaEventRecord(ev_sa[i], ss);
            if (i == 0) {  // op(B)'s first block right after A's first: the first product needs only these
                const int64_t nj = col0(1);
                const OzA a0 = with_flag(fb);
                if (!rc) rc = ozaki_prepare_b(&a0, nj, b, brs, bcs, ss, &pb[0]);
                cudaEventRecord(ev_sb[0], ss);
            }
        }
        for (int j = 1; j < nch && !rc; ++j) {
            const int64_t j0 = col0(j), nj = col0(j + 1) - j0;
            const OzA aj = with_flag(fb + j);
            rc = ozaki_prepare_b(&aj, nj, b + j0 * bcs, brs, bcs, ss, &pb[(size_t)j]);
            cudaEventRecord(ev_sb[j], ss);
        }
        int q = 0;
        for (int j = 0; j < nch && !rc; ++j)
            for (int i = 0; i < na && !rc; ++i) {
                const int64_t j0 = col0(j), r0 = rb[i], rows = rb[i + 1] - rb[i];
                cudaStream_t ps = sp[q];
                q ^= 1;
                cudaStreamWaitEvent(ps, ev_sa[i], 0);
                cudaStreamWaitEvent(ps, ev_sb[j], 0);
                int* f = fab + i * nch + j;
                rc = ozaki_flag_or(fa + i, fb + j, f, ps);
                const OzA aij = with_flag(f);
                if (!rc)
                    rc = ozaki_multiply_rows(&aij, r0, rows, &pb[(size_t)j], alpha, beta, c + r0 * rs_c + j0 * cs_c,
                                             rs_c, cs_c, ps);
            }
        // the join is recorded whatever happened, so s never runs ahead of the other streams
        cudaEventRecord(ev_aux_done, sp[1]);
        cudaEventRecord(ev_split_done, ss);
        cudaStreamWaitEvent(s, ev_aux_done, 0);
        cudaStreamWaitEvent(s, ev_split_done, 0);
    }
    for (auto& x : pb) ozaki_release_b(&x, s);
    ozaki_release_a(&prep, s);
    dev_free(flags, s);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return rc;
}

// SGEMM's split form on the FP32 operands themselves: the digit form at
// GB_SGEMM_SPLIT_SLICES slices splits op(A) and op(B) straight from FP32
// (each element widened exactly as it loads), the slice GEMM runs as for
// dgemm_ozaki, and the recombination writes C = RN32(alpha P + beta C) from
// the FP64 product P, the rounding of the form through FP64 copies; Inf/NaN
// operands raise the flag and an FP32 kernel gated on it computes C instead.
namespace {

// sgemm_ozaki in blocks, as dgemm_ozaki_blocks: op(A)'s row blocks and
// op(B)'s column blocks split from FP32 on a stream of their own, one slice
// GEMM with its FP32 recombination per block of C on two compute streams,
// each block gated on its own row and column blocks' Inf/NaN flags.
int sgemm_ozaki_blocks(int na_req, int nch, int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars,
                       int64_t acs, const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c,
                       int64_t cs_c, cudaStream_t s)
{
    constexpr int S = GB_SGEMM_SPLIT_SLICES;
    cudaStream_t sp[2] = {s, thread_aux_stream(0)}, ss = thread_aux_stream(1);
    OzA A;
    int rc = ozaki_alloc_a(m, k, nullptr, ars, acs, S, s, &A);
    if (rc) return rc;
    std::vector<int64_t> rb(1, 0);
    for (int i = 1; i < na_req; ++i) {
        const int64_t r = (m * i / na_req + A.row_tile - 1) / A.row_tile * A.row_tile;
        if (r > rb.back() && r < m) rb.push_back(r);
    }
    rb.push_back(m);
    const int na = (int)rb.size() - 1;
    int* flags = static_cast<int*>(dev_alloc(sizeof(int) * (size_t)(na + nch + na * nch), s));
    if (!flags) {
        ozaki_release_a(&A, s);
        return GB_ERR_NOMEM;
    }
    rc = check_cuda(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(na + nch + na * nch), s), "memset flags");
    int *fa = flags, *fb = flags + na, *fab = flags + na + nch;
    std::vector<cudaEvent_t> ev((size_t)(1 + na + nch + 2), nullptr);
    for (auto& e : ev)
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "sgemm blocks events");
    cudaEvent_t ev_fork = ev[0], *ev_sa = ev.data() + 1, *ev_sb = ev_sa + na, ev_aux_done = ev_sb[nch],
                ev_split_done = ev_sb[nch + 1];
    auto col0 = [&](int j) { return n * j / nch; };
    std::vector<OzB> pb((size_t)nch);
    if (!rc) {
        cudaEventRecord(ev_fork, s);
        cudaStreamWaitEvent(sp[1], ev_fork, 0);
        cudaStreamWaitEvent(ss, ev_fork, 0);
        auto split_b = [&](int j) {
            const int64_t j0 = col0(j), nj = col0(j + 1) - j0;
            if (!rc) rc = ozaki_alloc_b(&A, nj, nullptr, brs, bcs, ss, &pb[(size_t)j]);
            if (!rc) {  // rows of op(B)^T: (j, l) = b[l*brs + j*bcs]
                OzB& B = pb[(size_t)j];
                split_operand_f32(nj, k, b + j0 * bcs, bcs, brs, B.maxb, B.npad, B.npad, A.kpad, B.sb, B.eb, fb + j, ss);
                rc = check_cuda(cudaGetLastError(), "oz_split");
            }
            cudaEventRecord(ev_sb[j], ss);
        };
        for (int i = 0; i < na && !rc; ++i) {
            const int64_t r0 = rb[i], r1 = rb[i + 1];
            const int64_t cover = (r1 == m ? A.mpad : r1) - r0;
            split_operand_f32(r1 - r0, k, a + r0 * ars, ars, acs, A.maxa + r0, A.mpad, cover, A.kpad,
                              A.sa + r0 * A.kpad, A.ea + r0, fa + i, ss);
            rc = check_cuda(cudaGetLastError(), "oz_split");
            cudaEventRecord(ev_sa[i], ss);
            if (i == 0) split_b(0);  // the first product needs only A's and op(B)'s first blocks
        }
        for (int j = 1; j < nch && !rc; ++j) split_b(j);
        int q = 0;
        for (int j = 0; j < nch && !rc; ++j)
            for (int i = 0; i < na && !rc; ++i) {
                const int64_t j0 = col0(j), r0 = rb[i], rows = rb[i + 1] - rb[i];
                cudaStream_t ps = sp[q];
                q ^= 1;
                cudaStreamWaitEvent(ps, ev_sa[i], 0);
                cudaStreamWaitEvent(ps, ev_sb[j], 0);
                int* f = fab + i * nch + j;
                rc = ozaki_flag_or(fa + i, fb + j, f, ps);
                OzA aij = A;
                aij.nonfinite = f;
                const OzF32 f32{a, b + j0 * bcs, c + r0 * rs_c + j0 * cs_c};
                if (!rc)
                    rc = multiply_rows_impl(&aij, r0, rows, &pb[(size_t)j], (double)alpha, (double)beta, nullptr, rs_c,
                                            cs_c, &f32, ps);
            }
        cudaEventRecord(ev_aux_done, sp[1]);
        cudaEventRecord(ev_split_done, ss);
        cudaStreamWaitEvent(s, ev_aux_done, 0);
        cudaStreamWaitEvent(s, ev_split_done, 0);
    }
    for (auto& x : pb) ozaki_release_b(&x, s);
    ozaki_release_a(&A, s);
    dev_free(flags, s);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return rc;
}

}  // namespace

int sgemm_ozaki(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0f || k <= 0) return scal_matrix_f(m, n, beta, c, rs_c, cs_c, s);
    constexpr int S = GB_SGEMM_SPLIT_SLICES;
    ModeOverride digits(GB_DGEMM_OZAKI, S, 0);
    int br = 0, bc = 0;
    ozaki_fixed_blocks(&br, &bc);
    if (!br) {
        // 4 x 2 blocks from 8192: 4.29-4.35 -> 4.22 ms at 8192^3 (2 x 2, 2 x 4, 4 x 4 no better,
        // 8 x 4 worse: six products per block leave less to overlap than the FP64 forms' 16-28)
        const bool big = (m >= 8192 && n >= 8192 && k >= 2048);
        br = big ? 4 : 1;
        bc = big ? 2 : 1;
    }
    if (bc > n) bc = 1;
    if (br * bc > 1 && m >= 2048) {
        EngineScope engine(t_ozaki_ctas ? t_ozaki_ctas : ozaki_engine_choice(m / br, n / bc, k));
        return sgemm_ozaki_blocks(br, bc, m, n, k, alpha, a, ars, acs, b, brs, bcs, beta, c, rs_c, cs_c, s);
    }
    EngineScope engine(t_ozaki_ctas ? t_ozaki_ctas : ozaki_engine_choice(m, n, k));
    OzA A;
    int rc = ozaki_alloc_a(m, k, nullptr, ars, acs, S, s, &A);
    if (rc) return rc;
    OzB B;
    if ((rc = ozaki_alloc_b(&A, n, nullptr, brs, bcs, s, &B))) {
        ozaki_release_a(&A, s);
        return rc;
    }
    split_operand_f32(m, k, a, ars, acs, A.maxa, A.mpad, A.mpad, A.kpad, A.sa, A.ea, A.nonfinite, s);
    // rows of op(B)^T: (j, l) = b[l*brs + j*bcs]
    split_operand_f32(n, k, b, bcs, brs, B.maxb, B.npad, B.npad, A.kpad, B.sb, B.eb, A.nonfinite, s);
    rc = check_cuda(cudaGetLastError(), "oz_split");
    const OzF32 f32{a, b, c};
    if (!rc) rc = multiply_rows_impl(&A, 0, m, &B, (double)alpha, (double)beta, nullptr, rs_c, cs_c, &f32, s);
    ozaki_release_b(&B, s);
    ozaki_release_a(&A, s);
    return rc;
}

// ---------------------------------------------------------------- grouped form
// Every problem of a gemm_batch call through the Ozaki form in three
// launches (split, slice GEMM, recombine) plus the gated native fallback the
// caller adds.  The tables and arenas are built once and stay resident, so
// a plan can replay the launches (or a graph of them).
struct OzBatch {
    int slices = 0;
    bool f32 = false;  // FP32 operands and C (the batch's SGEMM form, GB_SGEMM_SPLIT_SLICES only)
    int nprob = 0;
    int64_t items = 0, units = 0, rblocks = 0, boxes_a = 0, boxes_b = 0;
    uint8_t* arena = nullptr;  // slices, planes, exponents, tables, flag
    OzBatchProb* d_probs = nullptr;
    int32_t* d_item_prob = nullptr;
    int64_t* d_item_base = nullptr;
    int32_t* d_unit_prob = nullptr;
    int64_t* d_unit_base = nullptr;
    int32_t* d_rblock_prob = nullptr;
    int64_t* d_rblock_base = nullptr;
    int* d_flag = nullptr;                   // Inf/NaN flag; the work-item counter 256 bytes on
    unsigned long long* d_counter = nullptr;
    uint16_t* sa = nullptr;
    uint16_t* sb = nullptr;
    CUtensorMap map_a, map_b;
    OzBatchParams gp;
};

namespace {

int make_box_map(CUtensorMap* map, const void* base, int box_rows, int64_t nboxes)
{
    auto fn = encode_fn();
    if (!fn) return set_error(GB_ERR_CUDA, "ozaki", "cuTensorMapEncodeTiled unavailable");
    if (nboxes > INT32_MAX) return set_error(GB_ERR_ARG, "ozaki batch", "too many k blocks for TMA coordinates");
    cuuint64_t dims[3] = {(cuuint64_t)OZ_BK, (cuuint64_t)box_rows, (cuuint64_t)nboxes};
    cuuint64_t strides[2] = {(cuuint64_t)(OZ_BK * 2), (cuuint64_t)box_rows * OZ_BK * 2};
    cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                    estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GB_ERR_CUDA, "ozaki batch", "cuTensorMapEncodeTiled failed");
    return GB_SUCCESS;
}

template <int S>
void launch_split_batch(const OzBatch& ob, cudaStream_t s)
{
    if constexpr (S == GB_SGEMM_SPLIT_SLICES) {
        if (ob.f32) {
            oz_split_batch_kernel<S, float><<<(unsigned)ob.units, 256, 0, s>>>(
                ob.d_probs, ob.d_unit_prob, ob.d_unit_base, ob.boxes_a, ob.boxes_b, ob.sa, ob.sb, ob.d_flag);
            return;
        }
    }
    oz_split_batch_kernel<S, double><<<(unsigned)ob.units, 256, 0, s>>>(ob.d_probs, ob.d_unit_prob, ob.d_unit_base,
                                                                         ob.boxes_a, ob.boxes_b, ob.sa, ob.sb,
                                                                         ob.d_flag);
}

template <int S>
void launch_recombine_batch(const OzBatch& ob, cudaStream_t s)
{
    if constexpr (S == GB_SGEMM_SPLIT_SLICES) {
        if (ob.f32) {
            oz_recombine_batch_kernel<S, float><<<(unsigned)ob.rblocks, 256, 0, s>>>(ob.d_probs, ob.d_rblock_prob,
                                                                                     ob.d_rblock_base, ob.d_flag);
            return;
        }
    }
    oz_recombine_batch_kernel<S, double><<<(unsigned)ob.rblocks, 256, 0, s>>>(ob.d_probs, ob.d_rblock_prob,
                                                                               ob.d_rblock_base, ob.d_flag);
}

}  // namespace

// Whether the grouped form takes a problem: one k part per level and the
// 128-bit recombination range.
bool ozaki_batch_accepts(int64_t k, int slices)
{
    const int64_t kpad = round_up(k, OZ_BK);
    return kpad <= ozaki_kpart_limit(slices) && ozaki_t_bound_log2(slices, k) < 126.0;
}

int ozaki_batch_create(const gb_gemm_problem_t* probs, int64_t count, int slices, cudaStream_t s,
                       OzBatch** out, bool f32)
{
    *out = nullptr;
    if (slices < 2 || slices > OZ_MAX_SLICES)
        return set_error(GB_ERR_ARG, "ozaki batch", "slices must be in [2, 12]");
    if (f32 && slices != GB_SGEMM_SPLIT_SLICES)
        return set_error(GB_ERR_ARG, "ozaki batch", "the FP32 form runs at the SGEMM split form's slice count");
    std::vector<OzBatchProb> h;
    h.reserve((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        if (p.m <= 0 || p.n <= 0 || p.k <= 0 || p.alpha == 0.0 || !ozaki_batch_accepts(p.k, slices))
            return set_error(GB_ERR_ARG, "ozaki batch", "problem not eligible for the grouped form");
        const bool ta = GB_IS_TRANS(p.transa), tb = GB_IS_TRANS(p.transb);
        OzBatchProb q = {};
        const void* pa = p.a;
        const int64_t ars = ta ? p.lda : 1, acs = ta ? 1 : p.lda;
        const void* pb = p.b;
        const int64_t brs = tb ? 1 : p.ldb, bcs = tb ? p.ldb : 1;  // rows of op(B)^T are columns of op(B)
        // tiles covered as C and as C^T; the transposed form when it needs fewer
        const int64_t cover = ((p.m + OZ_BM - 1) / OZ_BM) * ((p.n + OZ_BN - 1) / OZ_BN);
        const int64_t cover_t = ((p.n + OZ_BM - 1) / OZ_BM) * ((p.m + OZ_BN - 1) / OZ_BN);
        q.swap = (cover_t < cover && ozaki_batch_orient_setting()) ? 1 : 0;
        q.a = q.swap ? pb : pa;
        q.ars = q.swap ? brs : ars;
        q.acs = q.swap ? bcs : acs;
        q.b = q.swap ? pa : pb;
        q.brs = q.swap ? ars : brs;
        q.bcs = q.swap ? acs : bcs;
        q.c = p.c;
        q.rs_c = 1;
        q.cs_c = p.ldc;
        q.alpha = p.alpha;
        q.beta = p.beta;
        q.m = q.swap ? p.n : p.m;
        q.n = q.swap ? p.m : p.n;
        q.k = p.k;
        q.kb = (int32_t)((p.k + OZ_BK - 1) / OZ_BK);
        q.tiles_m = (int32_t)((q.m + OZ_BM - 1) / OZ_BM);
        q.tiles_n = (int32_t)((q.n + OZ_BN - 1) / OZ_BN);
        q.units_a = (q.m + 31) / 32;  // 32-row blocks holding rows of op(A); the padding is zeroed once
        q.ld = round_up(p.m, 4);      // rows of C
        h.push_back(q);
    }
    // longest k first: the last items handed out are the cheapest
    std::stable_sort(h.begin(), h.end(), [](const OzBatchProb& x, const OzBatchProb& y) { return x.k > y.k; });

    OzBatch* ob = new OzBatch();
    ob->slices = slices;
    ob->f32 = f32;
    ob->nprob = (int)h.size();
    OzBatchParams& gp = ob->gp;
    gp.slices = slices;
    gp.nlevels = slices;
    gp.chunk_kb = chunk_kb_setting();
    gp.nprob = ob->nprob;
    for (int L = 0; L < slices; ++L) {  // same level table as the single-problem form, one part each
        OzLevel& lv = gp.lv[L];
        lv.lev = slices + 1 - L;
        lv.pa_lo = (lv.lev - slices > 1) ? lv.lev - slices : 1;
        const int pa_hi = (lv.lev - 1 < slices) ? lv.lev - 1 : slices;
        lv.npairs = pa_hi - lv.pa_lo + 1;
        lv.nparts = 1;
        lv.kb_per_part = 0;
        lv.plane_base = L;
        lv.item_base = 0;
    }
    // tables: boxes, level planes, exponents, work items, split units, recombine blocks
    std::vector<int32_t> item_prob, unit_prob, rblock_prob;
    std::vector<int64_t> item_base, unit_base, rblock_base;
    int64_t planes_elems = 0, exps = 0;
    for (int i = 0; i < ob->nprob; ++i) {
        OzBatchProb& q = h[(size_t)i];
        q.abox = ob->boxes_a;
        q.bbox = ob->boxes_b;
        ob->boxes_a += (int64_t)q.tiles_m * q.kb;
        ob->boxes_b += (int64_t)q.tiles_n * q.kb;
        planes_elems += (int64_t)slices * (q.swap ? q.m : q.n) * q.ld;
        exps += q.m + q.n;
        const int64_t it = (int64_t)slices * q.tiles_m * q.tiles_n;
        item_base.push_back(ob->items);
        item_prob.insert(item_prob.end(), (size_t)it, i);
        ob->items += it;
        const int64_t un = q.units_a + (q.n + 31) / 32;
        unit_base.push_back(ob->units);
        unit_prob.insert(unit_prob.end(), (size_t)un, i);
        ob->units += un;
        const int64_t mc = q.swap ? q.n : q.m, nc = q.swap ? q.m : q.n;  // C's rows and columns
        const int64_t rb = (((mc + 3) / 4) * nc + 255) / 256;
        rblock_base.push_back(ob->rblocks);
        rblock_prob.insert(rblock_prob.end(), (size_t)rb, i);
        ob->rblocks += rb;
    }
    if (ob->units > INT32_MAX || ob->rblocks > INT32_MAX) {
        delete ob;
        return set_error(GB_ERR_ARG, "ozaki batch", "batch too large for one launch");
    }
    auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
    const size_t b_sa = al((size_t)slices * ob->boxes_a * OZ_BM * OZ_BK * 2);
    const size_t b_sb = al((size_t)slices * ob->boxes_b * OZ_BN * OZ_BK * 2);
    const size_t b_pl = al((size_t)planes_elems * 4);
    const size_t b_ex = al((size_t)exps * 4);
    const size_t b_pr = al(sizeof(OzBatchProb) * h.size());
    const size_t b_it = al(4 * item_prob.size()), b_ib = al(8 * item_base.size());
    const size_t b_up = al(4 * unit_prob.size()), b_ub = al(8 * unit_base.size());
    const size_t b_rp = al(4 * rblock_prob.size()), b_rb = al(8 * rblock_base.size());
    const size_t total = b_sa + b_sb + b_pl + b_ex + b_pr + b_it + b_ib + b_up + b_ub + b_rp + b_rb + 1024;
    ob->arena = static_cast<uint8_t*>(dev_alloc(total, s));
    if (!ob->arena) {
        delete ob;
        return GB_ERR_NOMEM;
    }
    uint8_t* cur = ob->arena;
    auto take = [&](size_t b) { uint8_t* r = cur; cur += b; return r; };
    ob->sa = reinterpret_cast<uint16_t*>(take(b_sa));
    ob->sb = reinterpret_cast<uint16_t*>(take(b_sb));
    int32_t* planes = reinterpret_cast<int32_t*>(take(b_pl));
    int32_t* ex = reinterpret_cast<int32_t*>(take(b_ex));
    ob->d_probs = reinterpret_cast<OzBatchProb*>(take(b_pr));
    ob->d_item_prob = reinterpret_cast<int32_t*>(take(b_it));
    ob->d_item_base = reinterpret_cast<int64_t*>(take(b_ib));
    ob->d_unit_prob = reinterpret_cast<int32_t*>(take(b_up));
    ob->d_unit_base = reinterpret_cast<int64_t*>(take(b_ub));
    ob->d_rblock_prob = reinterpret_cast<int32_t*>(take(b_rp));
    ob->d_rblock_base = reinterpret_cast<int64_t*>(take(b_rb));
    ob->d_flag = reinterpret_cast<int*>(take(1024));
    ob->d_counter = reinterpret_cast<unsigned long long*>(reinterpret_cast<uint8_t*>(ob->d_flag) + 256);
    int64_t pl_off = 0, ex_off = 0;
    for (auto& q : h) {
        q.planes = planes + pl_off;
        pl_off += (int64_t)slices * (q.swap ? q.m : q.n) * q.ld;
        q.ea = ex + ex_off;
        q.eb = q.ea + q.m;
        ex_off += q.m + q.n;
    }
    // rows past m (n) up to the tile height are never written by the split: zero them once here
    int rc = check_cuda(cudaMemsetAsync(ob->sa, 0, b_sa + b_sb, s), "memset slices");
    auto up = [&](void* d, const void* src, size_t b) {
        if (!rc && b) rc = check_cuda(cudaMemcpyAsync(d, src, b, cudaMemcpyHostToDevice, s), "batch tables");
    };
    up(ob->d_probs, h.data(), sizeof(OzBatchProb) * h.size());
    up(ob->d_item_prob, item_prob.data(), 4 * item_prob.size());
    up(ob->d_item_base, item_base.data(), 8 * item_base.size());
    up(ob->d_unit_prob, unit_prob.data(), 4 * unit_prob.size());
    up(ob->d_unit_base, unit_base.data(), 8 * unit_base.size());
    up(ob->d_rblock_prob, rblock_prob.data(), 4 * rblock_prob.size());
    up(ob->d_rblock_base, rblock_base.data(), 8 * rblock_base.size());
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "batch tables");  // host vectors go out of scope
    if (!rc && ob->nprob > 0) rc = make_box_map(&ob->map_a, ob->sa, OZ_BM, (int64_t)slices * ob->boxes_a);
    if (!rc && ob->nprob > 0) rc = make_box_map(&ob->map_b, ob->sb, OZ_BN, (int64_t)slices * ob->boxes_b);
    if (!rc && ob->nprob > 0) {
        static bool attr = false;
        if (!attr) {
            rc = check_cuda(cudaFuncSetAttribute(ozaki_slice_gemm_kernel<OzBatchParams>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_BYTES),
                            "smem attr");
            attr = (rc == GB_SUCCESS);
        }
    }
    if (rc) {
        dev_free(ob->arena, s);
        delete ob;
        return rc;
    }
    gp.items = ob->items;
    gp.boxes_a = ob->boxes_a;
    gp.boxes_b = ob->boxes_b;
    gp.probs = ob->d_probs;
    gp.item_prob = ob->d_item_prob;
    gp.item_base = ob->d_item_base;
    gp.status = device_status_word();
    gp.skip = ob->d_flag;
    gp.counter = ob->d_counter;
    *out = ob;
    return GB_SUCCESS;
}

const int* ozaki_batch_flag(const OzBatch* ob) { return ob ? ob->d_flag : nullptr; }

int ozaki_batch_launch(OzBatch* ob, cudaStream_t s)
{
    if (!ob || ob->nprob == 0) return GB_SUCCESS;
    int rc;
    // the flag and the work-item counter (256 bytes further) in one memset
    if ((rc = check_cuda(cudaMemsetAsync(ob->d_flag, 0, 256 + sizeof(unsigned long long), s), "memset")))
        return rc;
    {
        LaunchScope ls("oz_split_batch", s);
        switch (ob->slices) {
#define GB_SPLITB_CASE(S) \
    case S: launch_split_batch<S>(*ob, s); break;
            GB_SPLITB_CASE(2) GB_SPLITB_CASE(3) GB_SPLITB_CASE(4) GB_SPLITB_CASE(5) GB_SPLITB_CASE(6)
            GB_SPLITB_CASE(7) GB_SPLITB_CASE(8) GB_SPLITB_CASE(9) GB_SPLITB_CASE(10) GB_SPLITB_CASE(11)
            GB_SPLITB_CASE(12)
#undef GB_SPLITB_CASE
        default: break;
        }
    }
    if ((rc = check_cuda(cudaGetLastError(), "oz_split_batch"))) return rc;
    {
        const int sms = sm_count() > 0 ? sm_count() : 148;
        const int grid = (int)((ob->items < sms) ? ob->items : sms);
        LaunchScope ls("ozaki_slice_gemm_batch", s);
        ozaki_slice_gemm_kernel<OzBatchParams><<<grid, OZ_THREADS, OZ_SMEM_BYTES, s>>>(ob->map_a, ob->map_b, ob->gp);
    }
    if ((rc = check_cuda(cudaGetLastError(), "ozaki_slice_gemm batch"))) return rc;
    {
        LaunchScope ls("oz_recombine_batch", s);
        switch (ob->slices) {
#define GB_RECB_CASE(S) \
    case S: launch_recombine_batch<S>(*ob, s); break;
            GB_RECB_CASE(2) GB_RECB_CASE(3) GB_RECB_CASE(4) GB_RECB_CASE(5) GB_RECB_CASE(6)
            GB_RECB_CASE(7) GB_RECB_CASE(8) GB_RECB_CASE(9) GB_RECB_CASE(10) GB_RECB_CASE(11)
            GB_RECB_CASE(12)
#undef GB_RECB_CASE
        default: break;
        }
    }
    return check_cuda(cudaGetLastError(), "oz_recombine_batch");
}

void ozaki_batch_destroy(OzBatch* ob, cudaStream_t s)
{
    if (!ob) return;
    dev_free(ob->arena, s);
    delete ob;
}

// ---------------------------------------------------------------- BF16 GEMM host side
namespace {

// K-major copy of a bf16 operand: out[r*kst + l] = X(r, l) = x[r*rs + l*ls],
// 32 x 32 tiles through shared memory (coalesced on both sides).
__global__ void bf16_pack_kernel(int64_t rows, int64_t k, const uint16_t* __restrict__ x, int64_t rs, int64_t ls,
                                 uint16_t* __restrict__ out, int64_t kst)
{
    __shared__ uint16_t t[32][33];
    const int64_t r0 = (int64_t)blockIdx.y * 32, l0 = (int64_t)blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    const bool rows_fast = (rs == 1);
    for (int q = ty; q < 32; q += 8) {
        const int64_t r = r0 + (rows_fast ? tx : q), l = l0 + (rows_fast ? q : tx);
        const uint16_t v = (r < rows && l < k) ? x[r * rs + l * ls] : (uint16_t)0;
        if (rows_fast) t[tx][q] = v;
        else t[q][tx] = v;
    }
    __syncthreads();
    for (int q = ty; q < 32; q += 8) {
        const int64_t r = r0 + q, l = l0 + tx;
        if (r < rows && l < kst) out[r * kst + l] = (l < k) ? t[q][tx] : (uint16_t)0;
    }
}

// Rows x k bf16 with row stride `rst` elements (k contiguous), boxes of
// 64 k x box_rows rows, zero fill outside.
int make_kmajor_map(CUtensorMap* map, const void* base, int64_t k, int64_t rows, int64_t rst, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) return set_error(GB_ERR_CUDA, "bgemm", "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, 1};
    cuuint64_t strides[2] = {(cuuint64_t)(rst * 2), (cuuint64_t)(rst * 2 * rows)};
    cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GB_ERR_CUDA, "bgemm", "cuTensorMapEncodeTiled failed");
    return GB_SUCCESS;
}

// The operand as TMA-loadable K-major rows: the caller's memory when k is
// contiguous (ls == 1) with a 16-byte row stride and base, else a packed copy.
int bf16_kmajor(const uint16_t* x, int64_t rows, int64_t k, int64_t rs, int64_t ls, cudaStream_t s,
                const uint16_t** out, int64_t* rst, uint16_t** owned)
{
    *owned = nullptr;
    if (ls == 1 && rs % 8 == 0 && rs >= k && (reinterpret_cast<uintptr_t>(x) & 15) == 0) {
        *out = x;
        *rst = rs;
        return GB_SUCCESS;
    }
    const int64_t kst = round_up(k, 8);
    uint16_t* buf = static_cast<uint16_t*>(dev_alloc(sizeof(uint16_t) * (size_t)(rows * kst), s));
    if (!buf) return GB_ERR_NOMEM;
    const int64_t gy = (rows + 31) / 32, gx = (kst + 31) / 32;
    if (gy > 65535) {
        dev_free(buf, s);
        return set_error(GB_ERR_ARG, "bgemm", "too many rows for the pack grid");
    }
    {
        LaunchScope ls2("bf16_pack", s);
        bf16_pack_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(rows, k, x, rs, ls, buf, kst);
    }
    int rc = check_cuda(cudaGetLastError(), "bf16_pack");
    if (rc) {
        dev_free(buf, s);
        return rc;
    }
    *out = buf;
    *rst = kst;
    *owned = buf;
    return GB_SUCCESS;
}

}  // namespace

// C (fp32) := alpha op(A) op(B) + beta C with bf16 A, B on the tensor cores
// (tcgen05.mma kind::f16, bf16 in, fp32 accumulate).  op(A)(i, l) =
// a[i*ars + l*acs], op(B)(l, j) = b[l*brs + j*bcs].
int bgemm_tc(int64_t m, int64_t n, int64_t k, float alpha, const uint16_t* a, int64_t ars, int64_t acs,
             const uint16_t* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
             cudaStream_t s)
{
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (alpha == 0.0f || k <= 0) return scal_matrix_f(m, n, beta, c, rs_c, cs_c, s);
    if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX)
        return set_error(GB_ERR_ARG, "bgemm", "dimension too large for TMA coordinates");
    const uint16_t *ak, *bk;
    int64_t ast, bst;
    uint16_t *own_a = nullptr, *own_b = nullptr;
    int rc = bf16_kmajor(a, m, k, ars, acs, s, &ak, &ast, &own_a);
    if (!rc) rc = bf16_kmajor(b, n, k, bcs, brs, s, &bk, &bst, &own_b);  // rows of op(B)^T
    CUtensorMap map_a, map_b;
    if (!rc) rc = make_kmajor_map(&map_a, ak, k, m, ast, OZ_BM);
    if (!rc) rc = make_kmajor_map(&map_b, bk, k, n, bst, OZ_BN);
    if (!rc) {
        static bool attr = false;
        if (!attr) {
            rc = check_cuda(cudaFuncSetAttribute(ozaki_slice_gemm_kernel<BgemmParams>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_BYTES),
                            "smem attr");
            attr = (rc == GB_SUCCESS);
        }
    }
    if (!rc) {
        BgemmParams p;
        p.tiles_m = (int)((m + OZ_BM - 1) / OZ_BM);
        p.tiles_n = (int)((n + OZ_BN - 1) / OZ_BN);
        p.kb_total = (int)((k + OZ_BK - 1) / OZ_BK);
        p.chunk_kb = p.kb_total;  // one chunk: fp32 accumulation over the whole k range
        p.items = (int64_t)p.tiles_m * p.tiles_n;
        p.m = m;
        p.n = n;
        p.alpha = alpha;
        p.beta = beta;
        p.c = c;
        p.rs_c = rs_c;
        p.cs_c = cs_c;
        p.status = device_status_word();
        p.skip = nullptr;
        p.counter = nullptr;
        const int sms = sm_count() > 0 ? sm_count() : 148;
        const int grid = (int)((p.items < sms) ? p.items : sms);
        LaunchScope ls("bgemm_tcgen05", s);
        ozaki_slice_gemm_kernel<BgemmParams><<<grid, OZ_THREADS, OZ_SMEM_BYTES, s>>>(map_a, map_b, p);
        rc = check_cuda(cudaGetLastError(), "bgemm");
    }
    dev_free(own_a, s);
    dev_free(own_b, s);
    return rc;
}

namespace {

// ---------------------------------------------------------------- fused TRSM update
// B := B - A X for one of the small updates at the bottom of the TRSM
// recursion (R <= 128 rows, depth K <= 128, any n columns), the digit form
// at S <= 7 slices in one launch instead of four (split, slice GEMM,
// recombination, gated IEEE fallback).  CTA j owns columns [32j, 32j + 32)
// of X and B.  It takes the row exponents of A and the column exponents of
// its X columns as the split kernels do, writes the digits of each 64-deep
// k chunk of both operands into shared memory in the 128-byte-swizzled
// K-major layout that TMA gives the slice GEMM, and issues the S(S+1)/2
// digit products of the chunk as M=128 N=32 K=16 tcgen05 MMAs (one thread)
// into S level accumulators in TMEM.  fp32 holds the level sums exactly:
// |sum| <= K P 128^2 <= 2^24 for K <= 128 and P <= 8 products per level.
// The epilogue reads the level sums back and recombines each entry as
// oz_recombine_kernel does (exact weighted sum, one rounding, B - AB rounded
// once), so the update is bit-identical to the four-launch form.  A tile
// with an Inf or NaN in A or in its X columns takes FP64 FMAs instead.
constexpr int TU_THREADS = 256;
constexpr int TU_N = 32;                      // columns of X and B per CTA
constexpr int TU_ROWS = 128;                  // MMA rows (zero beyond R)
constexpr int TU_KC = 64;                     // k of one chunk
constexpr int TU_MAXS = 8;                    // slices (TMEM: 8 levels x 32 columns)
constexpr int TU_A_PLANE = TU_ROWS * 128;     // one digit plane of a chunk of A: 16 KB
constexpr int TU_B_PLANE = TU_N * 128;        // one of X^T: 4 KB
constexpr int TU_SMEM_BYTES = TU_MAXS * (TU_A_PLANE + TU_B_PLANE) + 1024 + 64;
constexpr uint32_t TU_TMEM_COLS = 256;

struct TuArgs {
    int R, K;
    int64_t n;
    const double* a;  // A(i, l) = a[i*ars + l*acs]
    int64_t ars, acs;
    const double* x;  // X(l, j) = x[l*xrs + j*xcs]
    int64_t xrs, xcs;
    double* b;  // B(i, j) = b[i*brs + j*bcs]
    int64_t brs, bcs;
    unsigned int* status;
    // A's digits prepared once per solve by trsm_image_kernel (null: the CTA splits A itself):
    // chunk c, slice q at aimg + (c S + q) 16 KB; row exponents aexp[0..127], aexp[128] = 1 if
    // the block holds an Inf or NaN
    const uint8_t* aimg;
    const int* aexp;
    // gemmtrsm shape: after the update, the R <= 64 rows solve their diagonal block in place
    // from its packed form (64 x 64 row-major, inverted diagonal, the trsm solves' layout);
    // null: update only
    const double* pk;
    int diag_lower;
};

// In-place substitution of one packed 64 x 64 diagonal block for 32 columns,
// 8 lanes per column, 8 rows per lane: the arithmetic of trsm_diag_kernel<8>
// (same FMAs in the same order), on Ls = P [64][65] and Xs = X [64][33] in
// shared memory.
template <bool LOWER>
__device__ __forceinline__ void tu_diag_solve(const double* Ls, double* Xs, int tid)
{
    const int c = tid >> 3, g = tid & 7;
    const int src0 = (tid & 31) - g;
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = Xs[(q * 8 + g) * 33 + c];
#pragma unroll
    for (int step = 0; step < 64; ++step) {
        const int i = LOWER ? step : 63 - step;
        const int qi = i >> 3, gi = i & 7;
        const double v = __shfl_sync(0xffffffffu, x[qi], src0 + gi);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (LOWER ? (q * 8 + 7 > i) : (q * 8 < i)) {
                const int r = q * 8 + g;
                if (LOWER ? (r > i) : (r < i)) x[q] = fma(-Ls[r * 65 + i], v, x[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int r = q * 8 + g;
        Xs[r * 33 + c] = x[q] * Ls[r * 65 + r];
    }
}

// A block of op(A) whose digit image trsm_image_kernel writes.
struct TuImgBlock {
    int64_t r0, c0;  // first row and column in op(A)
    int R, K;
    int64_t img_off, exp_off;  // bytes into the image arena, ints into the exponent arena
};

// byte offset of element (row, k) of a 128-byte-swizzled K-major plane of bf16 (k < 64)
__device__ __forceinline__ uint32_t tu_swz(int row, int k)
{
    return (uint32_t)(row * 128 + ((((k >> 3) ^ (row & 7))) << 4) + (k & 7) * 2);
}

// RNE(T 2^E) for T = sum_t a[t] 2^(8t), |a[t]| <= 2^24 (the fused kernel's level
// sums), equal to round_scaled(oz_weighted_sum(a), E).  T = hi 2^(8P) + lo with
// P = max(S - 4, 0): each part spans at most four levels, so |hi|, |lo| < 2^48.01
// are exact doubles; for E in [-1000, 900] hi 2^(E+8P) is exact, and one fma adds
// lo 2^E to it exactly before its single rounding (gradual underflow included).
// Outside that range the integer path rounds.
template <int S>
__device__ __forceinline__ double tu_round_levels(const int (&a)[S], int E)
{
    if (E < -1000 || E > 900) return round_scaled(oz_weighted_sum<S>(a), E);
    constexpr int P = S > 4 ? S - 4 : 0;
    long long hi = 0, lo = 0;
#pragma unroll
    for (int t = S - 1; t >= P; --t) hi = hi * 256 + a[t];
#pragma unroll
    for (int t = P - 1; t >= 0; --t) lo = lo * 256 + a[t];
    const double sh = __longlong_as_double((long long)(E + 8 * P + 1023) << 52);  // 2^(E+8P), normal
    const double sl = __longlong_as_double((long long)(E + 1023) << 52);          // 2^E, normal
    return __fma_rn((double)lo, sl, (double)hi * sh);
}

template <int S>
__global__ void __launch_bounds__(TU_THREADS, 1) trsm_update_fused_kernel(const TuArgs p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sa = smem;                          // S planes of 16 KB
    uint8_t* sb = smem + TU_MAXS * TU_A_PLANE;   // S planes of 4 KB
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + TU_MAXS * (TU_A_PLANE + TU_B_PLANE));
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    __shared__ int er[TU_ROWS], ec[TU_N];
    __shared__ int s_nf, s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t c0 = (int64_t)blockIdx.x * TU_N;
    const int ncols = (p.n - c0 < TU_N) ? (int)(p.n - c0) : TU_N;
    const int R = p.R, K = p.K;
    if (tid == 0) {
        mbar_init(bar, 1);      // MMA completion of a chunk
        mbar_init(bar + 1, 1);  // A's image planes of a chunk
        fence_barrier_init();
        s_nf = 0;
        s_fail = 0;
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, TU_TMEM_COLS);
        tmem_relinquish();
    }
    __syncthreads();
    // exponents: thread per row of A (or the image's); warp w for columns 4w .. 4w + 3 of X
    if (p.aimg) {
        if (tid < TU_ROWS) er[tid] = p.aexp[tid];
        if (tid == 0 && p.aexp[TU_ROWS]) s_nf = 1;
    } else if (tid < TU_ROWS) {
        unsigned long long mx = 0;
        if (tid < R)
            for (int l = 0; l < K; ++l) {
                const unsigned long long v = abs_bits(p.a[(int64_t)tid * p.ars + (int64_t)l * p.acs]);
                mx = v > mx ? v : mx;
            }
        int nf = 0;
        er[tid] = oz_row_exponent(mx, &nf);
        if (nf) s_nf = 1;
    }
    {
        // all 16 loads of a lane (4 columns x k = lane + 32 i, K <= 128) in flight at once
        double xv[4][2 * TU_KC / 32];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            const int c = warp * 4 + cc;
#pragma unroll
            for (int i = 0; i < 2 * TU_KC / 32; ++i) {
                const int l = lane + 32 * i;
                xv[cc][i] = (c < ncols && l < K) ? p.x[(int64_t)l * p.xrs + (c0 + c) * p.xcs] : 0.0;
            }
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            unsigned long long mx = 0;
#pragma unroll
            for (int i = 0; i < 2 * TU_KC / 32; ++i) {
                const unsigned long long v = abs_bits(xv[cc][i]);
                mx = v > mx ? v : mx;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
                mx = v > mx ? v : mx;
            }
            if (lane == 0) {
                int nf = 0;
                ec[warp * 4 + cc] = oz_row_exponent(mx, &nf);
                if (nf) s_nf = 1;
            }
        }
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (s_nf) {
        // IEEE path for this tile: B - A X by FP64 FMAs
        for (int e = tid; e < R * ncols; e += TU_THREADS) {
            const int i = e % R, j = e / R;
            double t = 0.0;
            for (int l = 0; l < K; ++l)
                t = fma(p.a[(int64_t)i * p.ars + (int64_t)l * p.acs], p.x[(int64_t)l * p.xrs + (c0 + j) * p.xcs], t);
            double* bij = p.b + (int64_t)i * p.brs + (c0 + j) * p.bcs;
            *bij = *bij - t;
        }
    } else {
        uint32_t phase = 0;
        for (int k0 = 0; k0 < K; k0 += TU_KC) {
            if (p.aimg) {
                // the chunk's S digit planes of A, prepared once per solve, by bulk copy
                if (tid == 0) {
                    mbar_arrive_expect_tx(bar + 1, (uint32_t)(S * TU_A_PLANE));
                    const uint8_t* src = p.aimg + (int64_t)(k0 / TU_KC) * S * TU_A_PLANE;
#pragma unroll
                    for (int q = 0; q < S; ++q) bulk_load(sa + q * TU_A_PLANE, src + q * TU_A_PLANE, TU_A_PLANE, bar + 1);
                }
            } else
            // digits of A (rows beyond R and k beyond K are zero), two k per 32-bit word;
            // consecutive threads take consecutive rows (column-major A reads coalesce)
            for (int e = tid; e < TU_ROWS * (TU_KC / 2); e += TU_THREADS) {
                const int row = e & (TU_ROWS - 1), kp = e >> 7;
                const int l = k0 + 2 * kp;
                const double* ar = p.a + (int64_t)row * p.ars;
                const double v0 = (row < R && l < K) ? ar[(int64_t)l * p.acs] : 0.0;
                const double v1 = (row < R && l + 1 < K) ? ar[(int64_t)(l + 1) * p.acs] : 0.0;
                uint32_t w[S];
                oz_digits_bf16x2<S>(v0, v1, er[row], w);
                const uint32_t off = tu_swz(row, 2 * kp);
#pragma unroll
                for (int q = 0; q < S; ++q) *reinterpret_cast<uint32_t*>(sa + q * TU_A_PLANE + off) = w[q];
            }
            // digits of X^T (columns beyond n are zero); lanes run along k, the loads of all
            // of a thread's items first
            {
                constexpr int IT = TU_N * (TU_KC / 2) / TU_THREADS;
                double xv[IT][2];
#pragma unroll
                for (int it = 0; it < IT; ++it) {
                    const int e = tid + it * TU_THREADS, kp = e & 31, c = e >> 5;
                    const int l = k0 + 2 * kp;
                    const double* xc = p.x + (c0 + c) * p.xcs;
                    xv[it][0] = (c < ncols && l < K) ? xc[(int64_t)l * p.xrs] : 0.0;
                    xv[it][1] = (c < ncols && l + 1 < K) ? xc[(int64_t)(l + 1) * p.xrs] : 0.0;
                }
#pragma unroll
                for (int it = 0; it < IT; ++it) {
                    const int e = tid + it * TU_THREADS, kp = e & 31, c = e >> 5;
                    uint32_t w[S];
                    oz_digits_bf16x2<S>(xv[it][0], xv[it][1], ec[c], w);
                    const uint32_t off = tu_swz(c, 2 * kp);
#pragma unroll
                    for (int q = 0; q < S; ++q) *reinterpret_cast<uint32_t*>(sb + q * TU_B_PLANE + off) = w[q];
                }
            }
            fence_proxy_async();  // the digits, written by threads, become visible to the MMAs
            if (p.aimg && tid == 0 && !mbar_wait_bounded(bar + 1, phase, kWaitBudgetNs)) {
                atomicOr(p.status, DEV_WAIT_TIMEOUT);
                s_fail = 1;
            }
            __syncthreads();
            if (s_fail) break;  // no MMA was issued for this chunk
            if (tid == 0) {
                tc_fence_after();
                constexpr uint32_t idesc = idesc_bf16_f32(TU_ROWS, TU_N);
                for (int L = 2; L <= S + 1; ++L) {
                    const uint32_t d_tmem = tmem + (uint32_t)((L - 2) * TU_N);
                    bool first = (k0 == 0);
                    const int pa_lo = (L - S > 1) ? L - S : 1, pa_hi = (L - 1 < S) ? L - 1 : S;
                    for (int pa = pa_lo; pa <= pa_hi; ++pa) {
                        const uint64_t ad = sdesc_kmajor_sw128(smem_addr(sa + (pa - 1) * TU_A_PLANE));
                        const uint64_t bd = sdesc_kmajor_sw128(smem_addr(sb + (L - pa - 1) * TU_B_PLANE));
#pragma unroll
                        for (int j = 0; j < TU_KC / 16; ++j)
                            mma_bf16_ss(d_tmem, ad + 2 * j, bd + 2 * j, idesc, (first && j == 0) ? 0u : 1u);
                        first = false;
                    }
                }
                mma_commit(bar);
            }
            __syncwarp();
            int ok = 1;
            if (lane == 0) ok = mbar_wait_bounded(bar, phase, kWaitBudgetNs) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok && lane == 0) {
                atomicOr(p.status, DEV_WAIT_TIMEOUT);
                s_fail = 1;
            }
            phase ^= 1u;
            __syncthreads();  // the next chunk overwrites the digits only after the MMAs read them
            tc_fence_after();
            if (s_fail) break;
        }
        if (!s_fail) {
            // warp w reads TMEM lanes 32 (w % 4) .. (rows) and columns 16 (w / 4) .. + 15
            const int qd = warp & 3, half = warp >> 2;
            const int row = qd * 32 + lane;
#pragma unroll 1
            for (int g = 0; g < 2; ++g) {
                const int cb = half * 16 + g * 8;
                uint32_t r8[S][8];
#pragma unroll
                for (int li = 0; li < S; ++li)
                    tmem_ld_32x32b_x8(tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(li * TU_N + cb), r8[li]);
                tmem_ld_wait();
                if (row < R) {
                    // the 8 entries of B first (loads in flight together), then the updates
                    double* brow = p.b + (int64_t)row * p.brs + (c0 + cb) * p.bcs;
                    double bv[8];
#pragma unroll
                    for (int c = 0; c < 8; ++c) bv[c] = (cb + c < ncols) ? brow[(int64_t)c * p.bcs] : 0.0;
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        int a[S];  // a[t] is level S + 1 - t, weight 2^(8t)
#pragma unroll
                        for (int li = 0; li < S; ++li) a[S - 1 - li] = __float2int_rn(__uint_as_float(r8[li][c]));
                        bv[c] = __fma_rn(1.0, bv[c], -tu_round_levels<S>(a, er[row] + ec[cb + c] - 8 * (S + 1)));
                    }
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        if (cb + c < ncols) brow[(int64_t)c * p.bcs] = bv[c];
                }
            }
        }
    }
    if (p.pk && !s_fail) {
        // the diagonal block of the updated rows (the reference's gemmtrsm shape): the digit
        // planes' shared memory is free once the MMAs have completed
        __syncthreads();  // the updated rows of B are in global memory
        double* Ls = reinterpret_cast<double*>(sa);  // [64][65]
        double* Xs = reinterpret_cast<double*>(sb);  // [64][33]
        for (int e = tid; e < 64 * 64; e += TU_THREADS) Ls[(e >> 6) * 65 + (e & 63)] = p.pk[e];
        for (int e = tid; e < 64 * TU_N; e += TU_THREADS) {
            const int i = e & 63, c = e >> 6;  // B column-major: consecutive threads, consecutive rows
            Xs[i * 33 + c] = (c < ncols && i < R) ? p.b[(int64_t)i * p.brs + (c0 + c) * p.bcs] : 0.0;
        }
        __syncthreads();
        if (p.diag_lower) tu_diag_solve<true>(Ls, Xs, tid);
        else tu_diag_solve<false>(Ls, Xs, tid);
        __syncthreads();
        for (int e = tid; e < 64 * TU_N; e += TU_THREADS) {
            const int i = e & 63, c = e >> 6;
            if (c < ncols && i < R) p.b[(int64_t)i * p.brs + (c0 + c) * p.bcs] = Xs[i * 33 + c];
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, TU_TMEM_COLS);
}

// The digit images of the A blocks of a solve's small updates, once per solve:
// CTA b writes block b's row exponents (the split kernels' rule over the
// block's columns), its Inf/NaN flag and, per 64-deep k chunk, S planes of
// 128 rows in the fused kernel's shared-memory layout (zero beyond R and K).
// Thread items are (row, 8 consecutive k): one 16-byte store per plane.
template <int S>
__global__ void __launch_bounds__(TU_THREADS) trsm_image_kernel(const double* __restrict__ a, int64_t ars,
                                                                int64_t acs, const TuImgBlock* __restrict__ blocks,
                                                                uint8_t* __restrict__ img, int* __restrict__ exps)
{
    const TuImgBlock blk = blocks[blockIdx.x];
    const double* ab = a + blk.r0 * ars + blk.c0 * acs;
    __shared__ unsigned long long part[2][TU_ROWS];
    __shared__ int er[TU_ROWS];
    __shared__ int s_nf;
    const int tid = threadIdx.x;
    if (tid == 0) s_nf = 0;
    {
        const int row = tid & (TU_ROWS - 1), h = tid >> 7;
        unsigned long long mx = 0;
        if (row < blk.R)
            for (int l = h; l < blk.K; l += 2) {
                const unsigned long long v = abs_bits(ab[(int64_t)row * ars + (int64_t)l * acs]);
                mx = v > mx ? v : mx;
            }
        part[h][row] = mx;
    }
    __syncthreads();
    if (tid < TU_ROWS) {
        const unsigned long long m0 = part[0][tid], m1 = part[1][tid];
        int nf = 0;
        er[tid] = oz_row_exponent(m0 > m1 ? m0 : m1, &nf);
        if (nf) s_nf = 1;
        exps[blk.exp_off + tid] = er[tid];
    }
    __syncthreads();
    if (tid == 0) exps[blk.exp_off + TU_ROWS] = s_nf;
    const int nch = (blk.K + TU_KC - 1) / TU_KC;
    for (int e = tid; e < nch * TU_ROWS * (TU_KC / 8); e += TU_THREADS) {
        const int row = e & (TU_ROWS - 1), k8 = (e >> 7) % (TU_KC / 8), c = (e >> 7) / (TU_KC / 8);
        const int l0 = c * TU_KC + k8 * 8;
        uint32_t w[S][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int l = l0 + 2 * h;
            const double* ar = ab + (int64_t)row * ars;
            const double v0 = (row < blk.R && l < blk.K) ? ar[(int64_t)l * acs] : 0.0;
            const double v1 = (row < blk.R && l + 1 < blk.K) ? ar[(int64_t)(l + 1) * acs] : 0.0;
            uint32_t ww[S];
            oz_digits_bf16x2<S>(v0, v1, er[row], ww);
#pragma unroll
            for (int q = 0; q < S; ++q) w[q][h] = ww[q];
        }
        uint8_t* base = img + blk.img_off + (int64_t)c * S * TU_A_PLANE + tu_swz(row, k8 * 8);
#pragma unroll
        for (int q = 0; q < S; ++q)
            *reinterpret_cast<uint4*>(base + q * TU_A_PLANE) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
    }
}

template <int S>
int launch_trsm_image(const double* a, int64_t ars, int64_t acs, const TuImgBlock* blocks, int nblocks, uint8_t* img,
                      int* exps, cudaStream_t s)
{
    LaunchScope ls("trsm_image", s);
    trsm_image_kernel<S><<<(unsigned)nblocks, TU_THREADS, 0, s>>>(a, ars, acs, blocks, img, exps);
    return check_cuda(cudaGetLastError(), "trsm_image");
}

template <int S>
int launch_trsm_update_fused(const TuArgs& a, cudaStream_t s)
{
    static bool attr = false;
    if (!attr) {
        const int rc = check_cuda(cudaFuncSetAttribute(trsm_update_fused_kernel<S>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, TU_SMEM_BYTES),
                                  "trsm update smem attr");
        if (rc) return rc;
        attr = true;
    }
    const int64_t grid = (a.n + TU_N - 1) / TU_N;
    LaunchScope ls("trsm_update_fused", s);
    trsm_update_fused_kernel<S><<<(unsigned)grid, TU_THREADS, TU_SMEM_BYTES, s>>>(a);
    return check_cuda(cudaGetLastError(), "trsm_update_fused");
}

}  // namespace

bool trsm_update_fused_fits(int slices, int64_t rows, int64_t k, int64_t n)
{
    return slices >= 2 && slices <= TU_MAXS && rows >= 1 && rows <= TU_ROWS && k >= 1 && k <= 2 * TU_KC && n >= 1 &&
           (n + TU_N - 1) / TU_N <= INT32_MAX;
}

// Digit images of the A blocks (rows R <= 128, depth K <= 128) that fused updates of
// one solve will read: arena layout by the host, one launch for all blocks.
int trsm_images_build(int slices, const double* a, int64_t ars, int64_t acs, const TrsmImgSpec* specs, int nspecs,
                      TrsmImages* out, cudaStream_t s)
{
    *out = TrsmImages();
    if (nspecs <= 0) return GB_SUCCESS;
    if (slices < 2 || slices > TU_MAXS) return set_error(GB_ERR_ARG, "trsm_images_build", "slices outside 2..8");
    std::vector<TuImgBlock> blocks((size_t)nspecs);
    int64_t img_bytes = 0, exp_ints = 0;
    for (int i = 0; i < nspecs; ++i) {
        const TrsmImgSpec& q = specs[i];
        if (q.rows < 1 || q.rows > TU_ROWS || q.k < 1 || q.k > 2 * TU_KC)
            return set_error(GB_ERR_ARG, "trsm_images_build", "block outside the fused kernel's shape");
        TuImgBlock& b = blocks[(size_t)i];
        b.r0 = q.r0;
        b.c0 = q.c0;
        b.R = (int)q.rows;
        b.K = (int)q.k;
        b.img_off = img_bytes;
        b.exp_off = exp_ints;
        img_bytes += (int64_t)((q.k + TU_KC - 1) / TU_KC) * slices * TU_A_PLANE;
        exp_ints += TU_ROWS + 4;  // exponents, flag, padding to 16 bytes
    }
    const size_t bytes_tab = sizeof(TuImgBlock) * (size_t)nspecs;
    const size_t total = (size_t)img_bytes + sizeof(int) * (size_t)exp_ints + bytes_tab + 256;
    uint8_t* arena = static_cast<uint8_t*>(dev_alloc(total, s));
    if (!arena) return GB_ERR_NOMEM;
    int* exps = reinterpret_cast<int*>(arena + img_bytes);
    TuImgBlock* d_blocks = reinterpret_cast<TuImgBlock*>(arena + img_bytes + sizeof(int) * (size_t)exp_ints);
    int rc = check_cuda(cudaMemcpyAsync(d_blocks, blocks.data(), bytes_tab, cudaMemcpyHostToDevice, s), "trsm images");
    if (!rc) {
        switch (slices) {
        case 2: rc = launch_trsm_image<2>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        case 3: rc = launch_trsm_image<3>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        case 4: rc = launch_trsm_image<4>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        case 5: rc = launch_trsm_image<5>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        case 6: rc = launch_trsm_image<6>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        case 7: rc = launch_trsm_image<7>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        default: rc = launch_trsm_image<8>(a, ars, acs, d_blocks, nspecs, arena, exps, s); break;
        }
    }
    // the host table is only read by the copy above, which the stream orders before any use
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "trsm images");
    if (rc) {
        dev_free(arena, s);
        return rc;
    }
    out->arena = arena;
    out->slices = slices;
    for (int i = 0; i < nspecs; ++i) {
        const TuImgBlock& b = blocks[(size_t)i];
        out->index[((uint64_t)b.r0 << 32) | (uint64_t)b.c0] =
            std::make_pair(static_cast<const uint8_t*>(arena + b.img_off), static_cast<const int*>(exps + b.exp_off));
    }
    return GB_SUCCESS;
}

void trsm_images_release(TrsmImages* im, cudaStream_t s)
{
    dev_free(im->arena, s);
    im->arena = nullptr;
    im->index.clear();
}

int trsm_update_fused(int slices, int64_t rows, int64_t k, int64_t n, const double* a, int64_t ars, int64_t acs,
                      const double* x, int64_t xrs, int64_t xcs, double* b, int64_t brs, int64_t bcs, cudaStream_t s,
                      const uint8_t* aimg, const int* aexp, const double* packed_diag, int diag_lower)
{
    if (!trsm_update_fused_fits(slices, rows, k, n) || (packed_diag && rows > 64))
        return set_error(GB_ERR_ARG, "trsm_update_fused", "update outside the fused kernel's shape");
    TuArgs t;
    t.R = (int)rows;
    t.K = (int)k;
    t.n = n;
    t.a = a;
    t.ars = ars;
    t.acs = acs;
    t.x = x;
    t.xrs = xrs;
    t.xcs = xcs;
    t.b = b;
    t.brs = brs;
    t.bcs = bcs;
    t.status = device_status_word();
    t.aimg = aimg;
    t.aexp = aexp;
    t.pk = packed_diag;
    t.diag_lower = diag_lower;
    note_ozaki_slices(slices);
    switch (slices) {
    case 2: return launch_trsm_update_fused<2>(t, s);
    case 3: return launch_trsm_update_fused<3>(t, s);
    case 4: return launch_trsm_update_fused<4>(t, s);
    case 5: return launch_trsm_update_fused<5>(t, s);
    case 6: return launch_trsm_update_fused<6>(t, s);
    case 7: return launch_trsm_update_fused<7>(t, s);
    default: return launch_trsm_update_fused<8>(t, s);
    }
}

}  // namespace gb

extern "C" int gb_set_ozaki_ctas(int ctas) { return gb::set_ozaki_ctas(ctas); }
