// gb_gemm_tiles.cuh -- the per-tile GEMM engines shared by the single-problem
// kernels (gb_dgemm.cu) and the grouped batch kernel (gb_batch.cu).
//
// A CTA of 256 threads computes one 128x128 tile of C := beta*C +
// alpha*op(A)*op(B) for operands with arbitrary element strides
// (op(A)(i, l) = a[i*ars + l*acs], B(l, j) = b[l*brs + j*bcs]): a
// register-prefetched 16-deep shared-memory stage feeds either DMMA
// (mma.sync m8n8k4 f64) or plain FMA.  The epilogue is the micro-kernel
// contract of ref_kernels/3/bli_gemm_ref.c:40-130: beta == 0 overwrites C
// (NaN in C ignored), otherwise c = beta*c + alpha*ab.
#pragma once

#include "gb_internal.h"

namespace gb {
namespace tiles {

constexpr int BM = 128, BN = 128, BK = 16, NT = 256;
constexpr int LDS = BM + 8;  // padded smem row (doubles); 136*2 banks = 16 mod 32

template <typename T>
struct GArgs {
    int64_t m, n, k;
    T alpha, beta;
    const T* a;
    int64_t ars, acs;
    const T* b;
    int64_t brs, bcs;
    T* c;
    int64_t rs_c, cs_c;
};
using DArgs = GArgs<double>;

__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

// Loads the A tile (rows bm.., cols k0..) and B tile (rows k0.., cols bn..)
// into registers; 8 elements each per thread, zero outside the matrix.
template <typename T>
__device__ __forceinline__ void load_tiles(const GArgs<T>& p, int64_t bm, int64_t bn, int64_t k0,
                                           T (&ra)[8], T (&rb)[8])
{
    const int tid = threadIdx.x;
    const bool a_rows_fast = (p.ars == 1);
    const bool b_k_fast = (p.brs == 1);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int e = tid + NT * r;
        int i, l;
        if (a_rows_fast) { i = e % BM; l = e / BM; } else { i = e / BK; l = e % BK; }
        const int64_t gi = bm + i, gl = k0 + l;
        ra[r] = (gi < p.m && gl < p.k) ? __ldg(p.a + gi * p.ars + gl * p.acs) : T(0);
        int j;
        if (b_k_fast) { l = e % BK; j = e / BK; } else { j = e % BN; l = e / BN; }
        const int64_t gj = bn + j;
        const int64_t gl2 = k0 + l;
        rb[r] = (gj < p.n && gl2 < p.k) ? __ldg(p.b + gl2 * p.brs + gj * p.bcs) : T(0);
    }
}

template <typename T>
__device__ __forceinline__ void store_tiles(const GArgs<T>& p, T (&ra)[8], T (&rb)[8], T* As, T* Bs)
{
    const int tid = threadIdx.x;
    const bool a_rows_fast = (p.ars == 1);
    const bool b_k_fast = (p.brs == 1);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int e = tid + NT * r;
        int i, l;
        if (a_rows_fast) { i = e % BM; l = e / BM; } else { i = e / BK; l = e % BK; }
        As[l * LDS + i] = ra[r];
        int j;
        if (b_k_fast) { l = e % BK; j = e / BK; } else { j = e % BN; l = e / BN; }
        Bs[l * LDS + j] = rb[r];
    }
}

template <typename T>
__device__ __forceinline__ void write_c(const GArgs<T>& p, int64_t i, int64_t j, T ab)
{
    if (i < p.m && j < p.n) {
        T* cij = p.c + i * p.rs_c + j * p.cs_c;
        const T t = p.alpha * ab;
        *cij = (p.beta == T(0)) ? t : fma(p.beta, *cij, t);
    }
}

// One BM x BN tile of C with the DMMA engine; As/Bs are BK*LDS doubles of
// shared memory.
__device__ __forceinline__ void dmma_tile(const DArgs& p, int64_t bm, int64_t bn, double* As, double* Bs)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = warp & 1, wn = warp >> 1;  // 2 x 4 warps, 64x32 each
    double acc[8][4][2];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    double ra[8], rb[8];
    load_tiles(p, bm, bn, 0, ra, rb);
    for (int64_t k0 = 0; k0 < p.k; k0 += BK) {
        __syncthreads();
        store_tiles(p, ra, rb, As, Bs);
        __syncthreads();
        if (k0 + BK < p.k) load_tiles(p, bm, bn, k0 + BK, ra, rb);
#pragma unroll
        for (int kk = 0; kk < BK; kk += 4) {
            const int kr = kk + (lane & 3);
            double af[8], bf[4];
#pragma unroll
            for (int mi = 0; mi < 8; ++mi) af[mi] = As[kr * LDS + wm * 64 + mi * 8 + (lane >> 2)];
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) bf[ni] = Bs[kr * LDS + wn * 32 + ni * 8 + (lane >> 2)];
#pragma unroll
            for (int mi = 0; mi < 8; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) dmma_8x8x4(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
        }
    }
#pragma unroll
    for (int mi = 0; mi < 8; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            const int64_t i = bm + wm * 64 + mi * 8 + (lane >> 2);
            const int64_t j = bn + wn * 32 + ni * 8 + 2 * (lane & 3);
            write_c(p, i, j, acc[mi][ni][0]);
            write_c(p, i, j + 1, acc[mi][ni][1]);
        }
}

// One tile with the SIMT engine (DFMA for double, FFMA for float): 16x16
// threads, 8x8 each.
template <typename T>
__device__ __forceinline__ void simt_tile(const GArgs<T>& p, int64_t bm, int64_t bn, T* As, T* Bs)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 8x8 each
    T acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = T(0);
    T ra[8], rb[8];
    load_tiles(p, bm, bn, 0, ra, rb);
    for (int64_t k0 = 0; k0 < p.k; k0 += BK) {
        __syncthreads();
        store_tiles(p, ra, rb, As, Bs);
        __syncthreads();
        if (k0 + BK < p.k) load_tiles(p, bm, bn, k0 + BK, ra, rb);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T av[8], bv[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = As[kk * LDS + ty * 8 + i];
#pragma unroll
            for (int j = 0; j < 8; ++j) bv[j] = Bs[kk * LDS + tx * 8 + j];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) write_c(p, bm + ty * 8 + i, bn + tx * 8 + j, acc[i][j]);
}

// Aligned operand tiles for the FP32 engine: a 128 x 16 (rows x k) tile of
// X(r, l) = x[r*rs + l*ls] as two 16-byte loads per thread, when either the
// rows are contiguous (rs == 1, ls a multiple of 4: vectors along r) or k
// is (ls == 1, rs a multiple of 4: vectors along l); the tile must lie
// inside the matrix.  S[l*LDS + r] is the shared-memory image.
template <bool R_CONTIG>
__device__ __forceinline__ void load_vec_tile(const float* __restrict__ x, int64_t rs, int64_t ls, int64_t r0,
                                              int64_t l0, float4 (&v)[2])
{
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int r, l;
        if (R_CONTIG) { r = (t & 31) * 4; l = (t >> 5) + 8 * q; }
        else { l = (t & 3) * 4; r = (t >> 2) + 64 * q; }
        v[q] = __ldg(reinterpret_cast<const float4*>(x + (r0 + r) * rs + (l0 + l) * ls));
    }
}

// Group swizzle of a transposed tile: in row l the 4-float groups are
// permuted by XOR with vec_swz(l), so the four rows a warp stores at once
// (l = 0, 4, 8, 12 apart) land in different banks; readers of row l XOR the
// group index the same way (a permutation: 16-byte fragments stay whole and
// conflict-free).
__device__ __forceinline__ int vec_swz(int l) { return ((l >> 2) & 3) << 1; }

template <bool R_CONTIG>
__device__ __forceinline__ void store_vec_tile(const float4 (&v)[2], float* S)
{
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        if (R_CONTIG) {
            *reinterpret_cast<float4*>(S + ((t >> 5) + 8 * q) * LDS + (t & 31) * 4) = v[q];
        } else {
            const int l = (t & 3) * 4, r = (t >> 2) + 64 * q;
            const float e[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
            for (int u = 0; u < 4; ++u)
                S[(l + u) * LDS + (((r >> 2) ^ vec_swz(l + u)) << 2) + (r & 3)] = e[u];
        }
    }
}

// FP32 tile engine: two shared-memory stages (one barrier per 16-deep k
// block, the next block's global loads overlap the FMAs), and each thread's
// 8x8 block split into 4-row/4-column halves 64 apart so its fragments are
// two 16-byte loads per operand per k step: B's are conflict-free across the
// warp, A's are broadcasts.  As/Bs hold 2*BK*LDS floats each.  VEC: every
// tile and k block lies inside the matrices and both operands meet the
// conditions of load_vec_tile; A_RC: op(A)(i, l) contiguous in i (ars == 1),
// otherwise in l; B_RC: op(B)(l, j) contiguous in j (bcs == 1), otherwise
// in l.
template <bool VEC = false, bool A_RC = true, bool B_RC = false>
__device__ __forceinline__ void sgemm_tile(const GArgs<float>& p, int64_t bm, int64_t bn, float* As, float* Bs)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    float ra[8], rb[8];
    float4 va[2], vb[2];
    // B's tile as rows j (= n index) x k: X(j, l) = b[j*bcs + l*brs]
    auto fetch = [&](int64_t k0) {
        if constexpr (VEC) {
            load_vec_tile<A_RC>(p.a, p.ars, p.acs, bm, k0, va);
            load_vec_tile<B_RC>(p.b, p.bcs, p.brs, bn, k0, vb);
        } else {
            load_tiles(p, bm, bn, k0, ra, rb);
        }
    };
    auto stash = [&](float* A, float* B) {
        if constexpr (VEC) {
            store_vec_tile<A_RC>(va, A);
            store_vec_tile<B_RC>(vb, B);
        } else {
            store_tiles(p, ra, rb, A, B);
        }
    };
    fetch(0);
    stash(As, Bs);
    __syncthreads();
    int cur = 0;
    for (int64_t k0 = 0; k0 < p.k; k0 += BK) {
        const bool more = (k0 + BK < p.k);
        if (more) fetch(k0 + BK);
        const float* A = As + cur * (BK * LDS);
        const float* B = Bs + cur * (BK * LDS);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            // transposed tiles of the aligned path carry the group swizzle
            const int sa = (VEC && !A_RC) ? vec_swz(kk) : 0, sb = (VEC && !B_RC) ? vec_swz(kk) : 0;
            const float4 a0 = *reinterpret_cast<const float4*>(A + kk * LDS + ((ty ^ sa) << 2));
            const float4 a1 = *reinterpret_cast<const float4*>(A + kk * LDS + 64 + ((ty ^ sa) << 2));
            const float4 b0 = *reinterpret_cast<const float4*>(B + kk * LDS + ((tx ^ sb) << 2));
            const float4 b1 = *reinterpret_cast<const float4*>(B + kk * LDS + 64 + ((tx ^ sb) << 2));
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (more) {
            // the other stage was last read before the previous barrier
            stash(As + (cur ^ 1) * (BK * LDS), Bs + (cur ^ 1) * (BK * LDS));
            __syncthreads();
            cur ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int64_t gi = bm + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t gj = bn + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            write_c(p, gi, gj, acc[i][j]);
        }
    }
}


}  // namespace tiles
}  // namespace gb
