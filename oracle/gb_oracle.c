/*
 * gb_oracle.c -- CPU restatement of the BLIS dense hot path.  TEST
 * INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference leg of bench.py, always as the checker or the
 * timed CPU baseline, never as part of the product.
 *
 * Compiled with -ffp-contract=off: every fused multiply-add below is an
 * explicit fma(), so the results are bit-identical on x86-64 and aarch64.
 *
 * Reference behaviour restated here (paths relative to the BLIS 1.0 tree):
 *   gemm  early exits          frame/3/bli_l3_util.c:41-65
 *         five-loop algorithm  frame/3/gemm/bli_gemm_blk_var{1,2,3}.c,
 *                              bli_gemm_ker_var2.c:216-276 (JR/IR loops);
 *                              beta applied at the first KC block only
 *                              (bli_gemm_blk_var3.c:108-110)
 *         micro-kernel math    ref_kernels/3/bli_gemm_ref.c:40-130
 *                              (ab = sum_k a*b; ab *= alpha;
 *                               beta == 0 ? c = ab : c = ab + beta*c)
 *   trsm  left/right reduction frame/3/bli_l3_oapi_ex.c:753-758
 *         blocked solve + gemm frame/3/trsm/bli_trsm_blk_var1.c:37-189
 *         pre-inverted diagonal ref_kernels/3/bli_trsm_ref.c:40-125
 *   trmm, symm, gemmt (syrk)    frame/3/bli_l3_oapi_ex.c:609-690, 436-520,
 *                              151-225 (326-345): the operation's definition on
 *                              dense temporaries (tri(op(A)), the symmetric A,
 *                              the full product) through the gemm below, so the
 *                              rounding of each entry is the gemm micro-kernel's
 *   gemv  var2 (axpyf), var1 (dotxf) frame/2/gemv/bli_gemv_unf_var2.c:37-129,
 *                              bli_gemv_unf_var1.c:37-102; beta == 0 is setv
 *   axpyv ref_kernels/1/bli_axpyv_ref.c:37-120 (alpha == 0 returns)
 *   scalv ref_kernels/1/bli_scalv_ref.c:40-98 (alpha == 1 returns, 0 sets)
 *   copyv ref_kernels/1/bli_copyv_ref.c
 *   amaxv ref_kernels/1/bli_amaxv_ref.c:44-140 (first NaN, else first max)
 *   ger   column-wise axpys a_j += (alpha y_j) x, frame/2/ger/bli_ger_unb_var2.c
 *   trsv  orc_dtrsm on one column (frame/2/trsv: the same substitution)
 *   zgemm the complex definition, op() with the conjugation bit of trans_t
 *         (0x10; 'C' = 0x18), accumulation over l in order, then
 *         beta == 0 ? c = alpha ab : c = alpha ab + beta c (complex)
 *   herk, her2k  frame/3/bli_l3_oapi_ex.c:295-320, 229-264: the uplo triangle
 *         of the product(s) with op(.)^H, accumulated over l in order, the
 *         imaginary parts of C's diagonal set to zero
 *   hemm, complex symm  :349-520 on the materialised A, then zgemm
 *   syr2k :267-292, two gemmt calls (the second with beta = 1)
 *   trmm3 :523-608, the dense tri(A) through the gemm (B not written)
 *   dotv  ref_kernels/1/bli_dotv_ref.c:37-121 (n == 0 gives rho = 0)
 * Not in the reference: the double-double evaluator (error oracle) and the
 * Ozaki split-product model (Ozaki, Ogita, Oishi & Rump 2012; integer-slice
 * variant of Ootomo, Ozaki & Yokota 2024), restated from the papers.
 */
#include "gb_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* RNG: SplitMix64 finaliser applied to seed and element index.        */
/* ------------------------------------------------------------------ */
#define GOLDEN 0x9E3779B97F4A7C15ull

uint64_t orc_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t orc_hash(uint64_t seed, uint64_t idx)
{
    return orc_mix64(orc_mix64(seed + GOLDEN) + (idx + 1) * GOLDEN);
}

static inline double u01(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }

void orc_fill_uniform(double* x, int64_t n, uint64_t seed, double lo, double hi)
{
    const double w = hi - lo;
    for (int64_t i = 0; i < n; ++i) x[i] = lo + w * u01(orc_hash(seed, (uint64_t)i));
}

void orc_fill_uniform_f(float* x, int64_t n, uint64_t seed, double lo, double hi)
{
    const double w = hi - lo;
    for (int64_t i = 0; i < n; ++i) x[i] = (float)(lo + w * u01(orc_hash(seed, (uint64_t)i)));
}

/* (1 + u) * 2^e with random sign; e uniform integer in [emin, emax]. */
void orc_fill_expspread(double* x, int64_t n, uint64_t seed, int emin, int emax)
{
    const uint64_t span = (uint64_t)(emax - emin + 1);
    for (int64_t i = 0; i < n; ++i) {
        uint64_t h = orc_hash(seed, (uint64_t)i);
        double mant = 1.0 + (double)(h >> 12) * 0x1.0p-52;
        int e = emin + (int)(((h >> 1) & 0x7FFull) % span);
        double v = ldexp(mant, e);
        x[i] = (h & 1ull) ? -v : v;
    }
}

/* {0, +-2^0 .. +-2^-6}, the testsuite's "narrow power of two" values
   (frame/include/bli_cast_macro_defs.h:477-525). */
void orc_fill_narrow_pow2(double* x, int64_t n, uint64_t seed)
{
    for (int64_t i = 0; i < n; ++i) {
        uint64_t h = orc_hash(seed, (uint64_t)i);
        int t = (int)(h & 7ull);
        double v = (t == 0) ? 0.0 : ldexp(1.0, -(t - 1));
        x[i] = ((h >> 3) & 1ull) ? -v : v;
    }
}

/* ------------------------------------------------------------------ */
/* Tiny pthread parallel-for.                                          */
/* ------------------------------------------------------------------ */
typedef void (*orc_task_fn)(void* arg, int tid, int nt);
typedef struct { orc_task_fn fn; void* arg; int tid; int nt; } orc_task_t;

static void* orc_task_tramp(void* p)
{
    orc_task_t* t = (orc_task_t*)p;
    t->fn(t->arg, t->tid, t->nt);
    return NULL;
}

static void orc_parallel(orc_task_fn fn, void* arg, int nt)
{
    if (nt <= 1) { fn(arg, 0, 1); return; }
    pthread_t th[256];
    orc_task_t ts[256];
    if (nt > 256) nt = 256;
    for (int t = 0; t < nt; ++t) {
        ts[t].fn = fn; ts[t].arg = arg; ts[t].tid = t; ts[t].nt = nt;
        if (t > 0) pthread_create(&th[t], NULL, orc_task_tramp, &ts[t]);
    }
    fn(arg, 0, nt);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* Five-loop GEMM (JC -> PC -> pack B -> IC -> pack A -> JR/IR -> ukr). */
/* Instantiated for double and float by a macro.                        */
/* ------------------------------------------------------------------ */
#define ORC_TRANS(t) (((t) & ORC_TRANSPOSE) != 0)

#define GEN_GEMM(T, CH, FMA, MR, NR, MC, KC, NC)                                         \
static void CH##_ukr(int64_t kc, const T* restrict ap, const T* restrict bp,             \
                     T* restrict ab)                                                      \
{                                                                                        \
    T acc[NR][MR];                                                                       \
    for (int j = 0; j < NR; ++j) for (int i = 0; i < MR; ++i) acc[j][i] = (T)0;          \
    for (int64_t l = 0; l < kc; ++l) {                                                   \
        const T* a = ap + l * MR; const T* b = bp + l * NR;                              \
        for (int j = 0; j < NR; ++j) {                                                   \
            const T bj = b[j];                                                           \
            for (int i = 0; i < MR; ++i) acc[j][i] = FMA(a[i], bj, acc[j][i]);           \
        }                                                                                \
    }                                                                                    \
    for (int j = 0; j < NR; ++j) for (int i = 0; i < MR; ++i) ab[j * MR + i] = acc[j][i];\
}                                                                                        \
                                                                                         \
/* C[0:m,0:n] := beta*C + alpha*A*B where A(i,l) = a[i*ars+l*acs], B(l,j)=b[l*brs+j*bcs] */\
static void CH##_gemm_serial(int64_t m, int64_t n, int64_t k, T alpha,                   \
                             const T* a, int64_t ars, int64_t acs,                        \
                             const T* b, int64_t brs, int64_t bcs, T beta,                \
                             T* c, int64_t rs_c, int64_t cs_c)                            \
{                                                                                        \
    T* apack = (T*)malloc(sizeof(T) * (size_t)(MC + MR) * KC);                           \
    T* bpack = (T*)malloc(sizeof(T) * (size_t)KC * (NC + NR));                           \
    T ab[MR * NR];                                                                       \
    for (int64_t jc = 0; jc < n; jc += NC) {                                             \
        const int64_t nc = (n - jc < NC) ? n - jc : NC;                                  \
        for (int64_t pc = 0; pc < k; pc += KC) {                                         \
            const int64_t kc = (k - pc < KC) ? k - pc : KC;                              \
            const T beta_use = (pc == 0) ? beta : (T)1;                                  \
            for (int64_t jp = 0; jp < nc; jp += NR)                                      \
                for (int64_t l = 0; l < kc; ++l)                                         \
                    for (int j = 0; j < NR; ++j) {                                       \
                        int64_t jj = jc + jp + j;                                        \
                        bpack[(jp / NR) * KC * NR + l * NR + j] = (jp + j < nc)          \
                            ? b[(pc + l) * brs + jj * bcs] : (T)0;                       \
                    }                                                                    \
            for (int64_t ic = 0; ic < m; ic += MC) {                                     \
                const int64_t mc = (m - ic < MC) ? m - ic : MC;                          \
                for (int64_t ip = 0; ip < mc; ip += MR)                                  \
                    for (int64_t l = 0; l < kc; ++l)                                     \
                        for (int i = 0; i < MR; ++i) {                                   \
                            int64_t ii = ic + ip + i;                                    \
                            apack[(ip / MR) * KC * MR + l * MR + i] = (ip + i < mc)      \
                                ? a[ii * ars + (pc + l) * acs] : (T)0;                   \
                        }                                                                \
                for (int64_t jr = 0; jr < nc; jr += NR) {                                \
                    const int64_t nr = (nc - jr < NR) ? nc - jr : NR;                    \
                    for (int64_t ir = 0; ir < mc; ir += MR) {                            \
                        const int64_t mr = (mc - ir < MR) ? mc - ir : MR;                \
                        CH##_ukr(kc, apack + (ir / MR) * KC * MR,                        \
                                 bpack + (jr / NR) * KC * NR, ab);                       \
                        for (int64_t j = 0; j < nr; ++j)                                 \
                            for (int64_t i = 0; i < mr; ++i) {                           \
                                T* cij = c + (ic + ir + i) * rs_c + (jc + jr + j) * cs_c;\
                                T t = alpha * ab[j * MR + i];                            \
                                *cij = (beta_use == (T)0) ? t : FMA(beta_use, *cij, t);  \
                            }                                                            \
                    }                                                                    \
                }                                                                        \
            }                                                                            \
        }                                                                                \
    }                                                                                    \
    free(apack); free(bpack);                                                            \
}                                                                                        \
                                                                                         \
typedef struct { int64_t m, n, k; T alpha, beta; const T* a; int64_t ars, acs;           \
                 const T* b; int64_t brs, bcs; T* c; int64_t rs_c, cs_c; int tm, tn; }   \
    CH##_gemm_args;                                                                      \
                                                                                         \
static void CH##_gemm_task(void* p, int tid, int nt)                                     \
{                                                                                        \
    CH##_gemm_args* g = (CH##_gemm_args*)p; (void)nt;                                    \
    int ti = tid % g->tm, tj = tid / g->tm;                                              \
    int64_t r0 = g->m * ti / g->tm, r1 = g->m * (ti + 1) / g->tm;                        \
    int64_t c0 = g->n * tj / g->tn, c1 = g->n * (tj + 1) / g->tn;                        \
    /* keep row splits on MR boundaries so the partition does not change results */    \
    r0 = (r0 / MR) * MR; r1 = (ti + 1 == g->tm) ? g->m : (r1 / MR) * MR;                 \
    if (r1 <= r0 || c1 <= c0) return;                                                    \
    CH##_gemm_serial(r1 - r0, c1 - c0, g->k, g->alpha, g->a + r0 * g->ars, g->ars,       \
                     g->acs, g->b + c0 * g->bcs, g->brs, g->bcs, g->beta,                \
                     g->c + r0 * g->rs_c + c0 * g->cs_c, g->rs_c, g->cs_c);              \
}                                                                                        \
                                                                                         \
static void CH##_scalm(int64_t m, int64_t n, T beta, T* c, int64_t rs_c, int64_t cs_c)  \
{                                                                                        \
    for (int64_t j = 0; j < n; ++j)                                                      \
        for (int64_t i = 0; i < m; ++i) {                                                \
            T* cij = c + i * rs_c + j * cs_c;                                            \
            *cij = (beta == (T)0) ? (T)0 : beta * *cij;                                  \
        }                                                                                \
}                                                                                        \
                                                                                         \
void orc_##CH##gemm(int transa, int transb, int64_t m, int64_t n, int64_t k,            \
                    T alpha, const T* a, int64_t rs_a, int64_t cs_a,                     \
                    const T* b, int64_t rs_b, int64_t cs_b,                              \
                    T beta, T* c, int64_t rs_c, int64_t cs_c, int nthreads)              \
{                                                                                        \
    if (m <= 0 || n <= 0) return;                                                        \
    if (alpha == (T)0 || k <= 0) { CH##_scalm(m, n, beta, c, rs_c, cs_c); return; }      \
    CH##_gemm_args g;                                                                    \
    g.m = m; g.n = n; g.k = k; g.alpha = alpha; g.beta = beta;                           \
    g.a = a; g.ars = ORC_TRANS(transa) ? cs_a : rs_a; g.acs = ORC_TRANS(transa) ? rs_a : cs_a; \
    g.b = b; g.brs = ORC_TRANS(transb) ? cs_b : rs_b; g.bcs = ORC_TRANS(transb) ? rs_b : cs_b; \
    g.c = c; g.rs_c = rs_c; g.cs_c = cs_c;                                               \
    int nt = nthreads < 1 ? 1 : nthreads;                                                \
    /* 2-D thread grid: tm x tn, rows get the larger share when m >= n */               \
    int best_tm = 1; double best = 1e300;                                                \
    for (int tm = 1; tm <= nt; ++tm) {                                                   \
        if (nt % tm) continue;                                                           \
        int tn = nt / tm;                                                                \
        double cost = (double)m / tm * k + (double)n / tn * k; /* packing traffic */     \
        if ((m + tm - 1) / tm < MR && tm > 1) continue;                                  \
        if (cost < best) { best = cost; best_tm = tm; }                                  \
    }                                                                                    \
    g.tm = best_tm; g.tn = nt / best_tm;                                                 \
    orc_parallel(CH##_gemm_task, &g, nt);                                                \
}

GEN_GEMM(double, d, fma, 8, 6, 128, 256, 3072)
GEN_GEMM(float, s, fmaf, 16, 6, 128, 256, 3072)

/* ------------------------------------------------------------------ */
/* TRSM: left solves only; the right side is handled by transposing    */
/* B and A (frame/3/bli_l3_oapi_ex.c:753-758).                         */
/* ------------------------------------------------------------------ */
#define TRSM_NB 128

void orc_dtrsm(int side, int uplo, int transa, int diag, int64_t m, int64_t n,
               double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               double* b, int64_t rs_b, int64_t cs_b, int nthreads)
{
    if (m <= 0 || n <= 0) return;
    int64_t brs = rs_b, bcs = cs_b, mm = m, nn = n;
    int trans = ORC_TRANS(transa);
    if (side == ORC_RIGHT) {
        /* B*inv(op(A)) = (inv(op(A))^T * B^T)^T */
        brs = cs_b; bcs = rs_b; mm = n; nn = m; trans = !trans;
    }
    /* effective op(A)(i,l) = a[i*ars + l*acs] */
    const int64_t ars = trans ? cs_a : rs_a, acs = trans ? rs_a : cs_a;
    const int lower = ((uplo == ORC_LOWER) != (trans != 0));
    const int unit = (diag == ORC_UNIT_DIAG);

    if (alpha == 0.0) {
        for (int64_t j = 0; j < nn; ++j) for (int64_t i = 0; i < mm; ++i) b[i * brs + j * bcs] = 0.0;
        return;
    }
    if (alpha != 1.0)
        for (int64_t j = 0; j < nn; ++j) for (int64_t i = 0; i < mm; ++i) b[i * brs + j * bcs] *= alpha;

    for (int64_t blk = 0; blk < mm; blk += TRSM_NB) {
        const int64_t nb = (mm - blk < TRSM_NB) ? mm - blk : TRSM_NB;
        /* block rows [i0, i0+nb) processed in forward (lower) or backward (upper) order */
        const int64_t i0 = lower ? blk : mm - blk - nb;
        for (int64_t j = 0; j < nn; ++j) {
            double* bj = b + j * bcs;
            if (lower) {
                for (int64_t i = i0; i < i0 + nb; ++i) {
                    double t = bj[i * brs];
                    for (int64_t l = i0; l < i; ++l) t = fma(-a[i * ars + l * acs], bj[l * brs], t);
                    bj[i * brs] = unit ? t : t * (1.0 / a[i * ars + i * acs]);
                }
            } else {
                for (int64_t i = i0 + nb - 1; i >= i0; --i) {
                    double t = bj[i * brs];
                    for (int64_t l = i + 1; l < i0 + nb; ++l) t = fma(-a[i * ars + l * acs], bj[l * brs], t);
                    bj[i * brs] = unit ? t : t * (1.0 / a[i * ars + i * acs]);
                }
            }
        }
        /* update the rows not yet solved: B2 -= A21 * X1 */
        if (lower && i0 + nb < mm) {
            const int64_t r0 = i0 + nb, rcount = mm - r0;
            orc_dgemm(ORC_NO_TRANSPOSE, ORC_NO_TRANSPOSE, rcount, nn, nb, -1.0,
                      a + r0 * ars + i0 * acs, ars, acs, b + i0 * brs, brs, bcs,
                      1.0, b + r0 * brs, brs, bcs, nthreads);
        } else if (!lower && i0 > 0) {
            orc_dgemm(ORC_NO_TRANSPOSE, ORC_NO_TRANSPOSE, i0, nn, nb, -1.0,
                      a + i0 * acs, ars, acs, b + i0 * brs, brs, bcs,
                      1.0, b, brs, bcs, nthreads);
        }
    }
}

/* ------------------------------------------------------------------ */
/* trmm, symm, gemmt: definitions on dense temporaries through orc_dgemm */
/* ------------------------------------------------------------------ */
/* B := alpha tri(op(A)) B (left) or alpha B tri(op(A)) (right), in place. */
void orc_dtrmm(int side, int uplo, int transa, int diag, int64_t m, int64_t n,
               double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               double* b, int64_t rs_b, int64_t cs_b, int nthreads)
{
    if (m <= 0 || n <= 0) return;
    const int64_t na = (side == ORC_LEFT) ? m : n;
    double* t = (double*)calloc((size_t)(na * na), sizeof(double));  /* tri(A), column-major */
    double* b0 = (double*)malloc(sizeof(double) * (size_t)(m * n));  /* copy of B, column-major */
    for (int64_t j = 0; j < na; ++j)
        for (int64_t i = 0; i < na; ++i) {
            const int in = (uplo == ORC_LOWER) ? (i >= j) : (i <= j);
            if (i == j) t[i + j * na] = (diag == ORC_UNIT_DIAG) ? 1.0 : a[i * rs_a + j * cs_a];
            else if (in) t[i + j * na] = a[i * rs_a + j * cs_a];
        }
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) b0[i + j * m] = b[i * rs_b + j * cs_b];
    if (side == ORC_LEFT)
        orc_dgemm(transa, ORC_NO_TRANSPOSE, m, n, m, alpha, t, 1, na, b0, 1, m, 0.0, b, rs_b, cs_b, nthreads);
    else
        orc_dgemm(ORC_NO_TRANSPOSE, transa, m, n, n, alpha, b0, 1, m, t, 1, na, 0.0, b, rs_b, cs_b, nthreads);
    free(t);
    free(b0);
}

/* C := alpha A B + beta C (left) or alpha B A + beta C (right), A symmetric
   with only its uplo triangle read. */
void orc_dsymm(int side, int uplo, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
               int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads)
{
    if (m <= 0 || n <= 0) return;
    const int64_t na = (side == ORC_LEFT) ? m : n;
    double* f = (double*)malloc(sizeof(double) * (size_t)(na * na));
    for (int64_t j = 0; j < na; ++j)
        for (int64_t i = 0; i < na; ++i) {
            const int in = (uplo == ORC_LOWER) ? (i >= j) : (i <= j);
            f[i + j * na] = in ? a[i * rs_a + j * cs_a] : a[j * rs_a + i * cs_a];
        }
    if (side == ORC_LEFT)
        orc_dgemm(ORC_NO_TRANSPOSE, ORC_NO_TRANSPOSE, m, n, m, alpha, f, 1, na, b, rs_b, cs_b, beta, c, rs_c,
                  cs_c, nthreads);
    else
        orc_dgemm(ORC_NO_TRANSPOSE, ORC_NO_TRANSPOSE, m, n, n, alpha, b, rs_b, cs_b, f, 1, na, beta, c, rs_c,
                  cs_c, nthreads);
    free(f);
}

/* The uplo triangle of the m x m C := alpha op(A) op(B) + beta C; the other
   triangle is left as it is.  Each entry is the gemm micro-kernel's
   (ab *= alpha; beta == 0 ? c = ab : c = fma(beta, c, ab)). */
void orc_dgemmt(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads)
{
    if (m <= 0) return;
    double* p = (double*)malloc(sizeof(double) * (size_t)(m * m));
    for (int64_t j = 0; j < m; ++j)
        for (int64_t i = 0; i < m; ++i) p[i + j * m] = c[i * rs_c + j * cs_c];
    orc_dgemm(transa, transb, m, m, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, p, 1, m, nthreads);
    for (int64_t j = 0; j < m; ++j)
        for (int64_t i = 0; i < m; ++i)
            if ((uplo == ORC_LOWER) ? (i >= j) : (i <= j)) c[i * rs_c + j * cs_c] = p[i + j * m];
    free(p);
}

/* ------------------------------------------------------------------ */
/* Level-2 / level-1v                                                  */
/* ------------------------------------------------------------------ */
void orc_dgemv(int transa, int conjx, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a,
               const double* x, int64_t incx, double beta, double* y, int64_t incy)
{
    (void)conjx;
    const int trans = ORC_TRANS(transa);
    const int64_t my = trans ? n : m, nx = trans ? m : n;
    if (my <= 0) return;
    /* y := beta*y, with beta == 0 overwriting (setv) */
    for (int64_t i = 0; i < my; ++i) y[i * incy] = (beta == 0.0) ? 0.0 : beta * y[i * incy];
    if (nx <= 0 || alpha == 0.0) return;
    if (!trans) {
        /* var2: y += (alpha*x_j) * a_j, column by column */
        for (int64_t j = 0; j < n; ++j) {
            const double chi = alpha * x[j * incx];
            for (int64_t i = 0; i < m; ++i) y[i * incy] = fma(chi, a[i * rs_a + j * cs_a], y[i * incy]);
        }
    } else {
        /* var1: y_i += alpha * (a_i^T x) */
        for (int64_t i = 0; i < n; ++i) {
            double rho = 0.0;
            for (int64_t l = 0; l < m; ++l) rho = fma(a[l * rs_a + i * cs_a], x[l * incx], rho);
            y[i * incy] = fma(alpha, rho, y[i * incy]);
        }
    }
}

void orc_daxpyv(int conjx, int64_t n, double alpha, const double* x, int64_t incx,
                double* y, int64_t incy)
{
    (void)conjx;
    if (n <= 0 || alpha == 0.0) return;
    for (int64_t i = 0; i < n; ++i) y[i * incy] = fma(alpha, x[i * incx], y[i * incy]);
}

/* Interleaved complex operands, strides in complex elements. */
void orc_zgemm(int transa, int transb, int64_t m, int64_t n, int64_t k, const double* alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b,
               const double* beta, double* c, int64_t rs_c, int64_t cs_c)
{
    const int ta = ORC_TRANS(transa), tb = ORC_TRANS(transb);
    const double sa = (transa & 0x10) ? -1.0 : 1.0, sb = (transb & 0x10) ? -1.0 : 1.0;
    const int64_t ars = ta ? cs_a : rs_a, acs = ta ? rs_a : cs_a;
    const int64_t brs = tb ? cs_b : rs_b, bcs = tb ? rs_b : cs_b;
    const int zero_beta = (beta[0] == 0.0 && beta[1] == 0.0);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            double sr = 0.0, si = 0.0;
            for (int64_t l = 0; l < k; ++l) {
                const double* pa = a + 2 * (i * ars + l * acs);
                const double* pb = b + 2 * (l * brs + j * bcs);
                const double xr = pa[0], xi = sa * pa[1], yr = pb[0], yi = sb * pb[1];
                sr = fma(xr, yr, fma(-xi, yi, sr));
                si = fma(xr, yi, fma(xi, yr, si));
            }
            double* pc = c + 2 * (i * rs_c + j * cs_c);
            double cr = alpha[0] * sr - alpha[1] * si, ci = alpha[0] * si + alpha[1] * sr;
            if (!zero_beta) {
                cr += beta[0] * pc[0] - beta[1] * pc[1];
                ci += beta[0] * pc[1] + beta[1] * pc[0];
            }
            pc[0] = cr;
            pc[1] = ci;
        }
}

void orc_dscalv(int64_t n, double alpha, double* x, int64_t incx)
{
    if (n <= 0 || alpha == 1.0) return;
    for (int64_t i = 0; i < n; ++i) x[i * incx] = (alpha == 0.0) ? 0.0 : alpha * x[i * incx];
}

void orc_dcopyv(int64_t n, const double* x, int64_t incx, double* y, int64_t incy)
{
    for (int64_t i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}

void orc_damaxv(int64_t n, const double* x, int64_t incx, int64_t* index)
{
    int64_t best = 0;
    double vmax = -1.0;
    for (int64_t i = 0; i < n; ++i) {
        const double v = fabs(x[i * incx]);
        if (vmax < v || (isnan(v) && !isnan(vmax))) {
            vmax = v;
            best = i;
        }
    }
    *index = best;
}

void orc_dger(int64_t m, int64_t n, double alpha, const double* x, int64_t incx, const double* y,
              int64_t incy, double* a, int64_t rs_a, int64_t cs_a)
{
    if (m <= 0 || n <= 0 || alpha == 0.0) return;
    for (int64_t j = 0; j < n; ++j) {
        const double ay = alpha * y[j * incy];
        for (int64_t i = 0; i < m; ++i) a[i * rs_a + j * cs_a] = fma(ay, x[i * incx], a[i * rs_a + j * cs_a]);
    }
}

void orc_dtrsv(int uplo, int transa, int diag, int64_t m, double alpha, const double* a, int64_t rs_a,
               int64_t cs_a, double* x, int64_t incx)
{
    orc_dtrsm(ORC_LEFT, uplo, transa, diag, m, 1, alpha, a, rs_a, cs_a, x, incx, 1, 1);
}

void orc_ddotv(int conjx, int conjy, int64_t n, const double* x, int64_t incx,
               const double* y, int64_t incy, double* rho)
{
    (void)conjx; (void)conjy;
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = fma(x[i * incx], y[i * incy], s);
    *rho = s;
}

/* ------------------------------------------------------------------ */
/* Double-double evaluation (Dekker/Knuth error-free transformations). */
/* ------------------------------------------------------------------ */
typedef struct { double hi, lo; } dd_t;

static inline dd_t two_sum(double a, double b)
{
    double s = a + b, bb = s - a;
    dd_t r = { s, (a - (s - bb)) + (b - bb) };
    return r;
}

static inline dd_t fast_two_sum(double a, double b)
{
    double s = a + b;
    dd_t r = { s, b - (s - a) };
    return r;
}

static inline dd_t dd_add(dd_t x, dd_t y)
{
    dd_t s = two_sum(x.hi, y.hi);
    dd_t t = two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}

static inline dd_t dd_mul_d(dd_t x, double b)
{
    double p = x.hi * b;
    double e = fma(x.hi, b, -p);
    e = fma(x.lo, b, e);
    return fast_two_sum(p, e);
}

static inline dd_t two_prod(double a, double b)
{
    double p = a * b;
    dd_t r = { p, fma(a, b, -p) };
    return r;
}

typedef struct {
    int64_t k; double alpha, beta; const double* a; int64_t ars, acs;
    const double* b; int64_t brs, bcs; const double* c; int64_t rs_c, cs_c;
    int64_t nent; const int64_t* ii; const int64_t* jj; double* hi; double* lo;
} dd_args;

static void dd_task(void* p, int tid, int nt)
{
    dd_args* g = (dd_args*)p;
    for (int64_t e = tid; e < g->nent; e += nt) {
        const int64_t i = g->ii[e], j = g->jj[e];
        dd_t s = { 0.0, 0.0 };
        for (int64_t l = 0; l < g->k; ++l)
            s = dd_add(s, two_prod(g->a[i * g->ars + l * g->acs], g->b[l * g->brs + j * g->bcs]));
        dd_t r = dd_mul_d(s, g->alpha);
        if (g->beta != 0.0) r = dd_add(r, two_prod(g->beta, g->c[i * g->rs_c + j * g->cs_c]));
        g->hi[e] = r.hi; g->lo[e] = r.lo;
    }
}

void orc_dd_gemm_entries(int transa, int transb, int64_t m, int64_t n, int64_t k,
                         double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                         const double* b, int64_t rs_b, int64_t cs_b,
                         double beta, const double* c, int64_t rs_c, int64_t cs_c,
                         int64_t nent, const int64_t* ii, const int64_t* jj,
                         double* hi, double* lo, int nthreads)
{
    (void)m; (void)n;
    dd_args g;
    g.k = k; g.alpha = alpha; g.beta = beta; g.a = a;
    g.ars = ORC_TRANS(transa) ? cs_a : rs_a; g.acs = ORC_TRANS(transa) ? rs_a : cs_a;
    g.b = b; g.brs = ORC_TRANS(transb) ? cs_b : rs_b; g.bcs = ORC_TRANS(transb) ? rs_b : cs_b;
    g.c = c; g.rs_c = rs_c; g.cs_c = cs_c; g.nent = nent; g.ii = ii; g.jj = jj; g.hi = hi; g.lo = lo;
    orc_parallel(dd_task, &g, nthreads < 1 ? 1 : nthreads);
}

void orc_dd_dotv(int64_t n, const double* x, int64_t incx, const double* y,
                 int64_t incy, double* hi, double* lo)
{
    dd_t s = { 0.0, 0.0 };
    for (int64_t i = 0; i < n; ++i) s = dd_add(s, two_prod(x[i * incx], y[i * incy]));
    *hi = s.hi; *lo = s.lo;
}

/* ------------------------------------------------------------------ */
/* Ozaki split-product model (exact integer specification).            */
/*                                                                     */
/* Each row r of the row operand (op(A), or op(B)^T) gets the exponent  */
/* e_r = ilogb(max_k |r_k|) + 2, so U = |x| 2^-e_r < 1/2 for every      */
/* element x of the row, and x = sign(x) 2^e_r sum_p d_p 2^-8p + rem    */
/* with balanced base-256 digits of U read off the fixed-point value    */
/* U 2^(8s+2) plus a constant bias (oz_digits below): |d_p| <= 128,     */
/* every digit is exact in bf16, |rem| <= 2^-(8s+1) 2^e_r.  The digits  */
/* come from integers only, never from floating point.                  */
/*                                                                     */
/* Level sums S_l = sum_{p+q=l} D^A_p (D^B_q)^T, l = 2..s+1 (the        */
/* triangular set, s(s+1)/2 products), are exact integers.  The GPU     */
/* accumulates 1024 products at a time in fp32 (|sum| <= 2^24, exact)   */
/* and level sums in int32, cutting K into parts so that                */
/* npairs(l) * Kpart * 2^14 < 2^31.                                     */
/*                                                                     */
/* Recombination is one rounding of an exact value:                     */
/*     T  = sum_l S_l 2^(8(s+1-l))          (exact, signed 128-bit)     */
/*     AB = RNE(T * 2^(e_i + e_j - 8(s+1)))                             */
/*     c  = beta == 0 ? alpha*AB : fma(beta, c, alpha*AB)               */
/* (alpha == 1, beta == 0 gives c = AB, the correctly rounded value of  */
/* the truncated split product).                                        */
/* ------------------------------------------------------------------ */
typedef __int128 i128;
typedef unsigned __int128 u128;

int64_t orc_ozaki_kpart_limit(int npairs)
{
    /* int32 level sums: npairs * Kpart * 128^2 < 2^31, Kpart a multiple of 64 */
    int64_t lim = (int64_t)2147483647 / ((int64_t)npairs * 128 * 128);
    lim = (lim / 64) * 64;
    return lim < 64 ? 64 : lim;
}

/* Largest |T| the recombination can meet, as a power-of-two exponent. */
static double oz_t_bound_log2(int s, int64_t k)
{
    double t = 0.0;
    for (int l = 2; l <= s + 1; ++l) {
        const int np = (l - 1 < s) ? l - 1 : s;
        t += (double)np * (double)k * 16384.0 * ldexp(1.0, 8 * (s + 1 - l));
    }
    return log2(t);
}

static int clz128(u128 u)
{
    const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
    if (hi) return __builtin_clzll(hi);
    if (lo) return 64 + __builtin_clzll(lo);
    return 128;
}

/* RNE(T * 2^E) as a double, from integers only. */
static double oz_round_scaled(i128 T, int E)
{
    if (T == 0) return 0.0;
    const int neg = T < 0;
    const u128 u = neg ? (u128)0 - (u128)T : (u128)T;
    const int msb = 127 - clz128(u);
    const int lead = msb + E;
    uint64_t bits;
    if (lead > 1023) {
        bits = 0x7FF0000000000000ull;
    } else {
        const int lsb = (lead >= -1022) ? lead - 52 : -1074;  /* exponent of the last kept bit */
        const int shift = lsb - E;
        u128 q;
        if (shift <= 0) {
            q = u << (-shift);
        } else if (shift > 128) {
            q = 0;
        } else if (shift == 128) {
            q = (u > ((u128)1 << 127)) ? 1 : 0;
        } else {
            q = u >> shift;
            const u128 rem = u & ((((u128)1) << shift) - 1);
            const u128 half = ((u128)1) << (shift - 1);
            if (rem > half || (rem == half && (q & 1))) q += 1;
        }
        bits = ((uint64_t)(lsb + 1074) << 52) + (uint64_t)q;
        if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    }
    if (neg) bits |= 0x8000000000000000ull;
    double r;
    memcpy(&r, &bits, sizeof r);
    return r;
}

/* Balanced base-256 digits of |x| 2^-e, with the sign of x.  X is       */
/* U 2^F truncated to an integer (F = 8s+2 fraction bits); adding        */
/* B = sum_p 128 2^(F-8p) + 2 turns the balanced digits into the plain   */
/* base-256 digits of Y = X + B: d_1 = floor(Y / 2^(F-8)) - 128 (up to   */
/* 128), d_p = (floor(Y / 2^(F-8p)) mod 256) - 128 for p >= 2.  The      */
/* remainder X_exact - sum_p d_p 2^(F-8p) lies in [-2, 2), i.e.          */
/* |rem| <= 2^-(8s+1) 2^e; the truncated bits of X never change a digit  */
/* (the rounding threshold 2 is an integer).                             */
static void oz_digits(double x, int e, int s, int16_t* d, int64_t stride)
{
    uint64_t bits;
    memcpy(&bits, &x, sizeof bits);
    const int neg = (int)(bits >> 63);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const uint64_t frac = bits & ((1ull << 52) - 1);
    if (ex == 0 && frac == 0) {
        for (int p = 0; p < s; ++p) d[p * stride] = 0;
        return;
    }
    const uint64_t M = ex ? (frac | (1ull << 52)) : frac;
    const int E2 = ex ? ex - 1075 : -1074;  /* |x| = M 2^E2 */
    const int F = 8 * s + 2;                /* fraction bits kept */
    const int sh = E2 - e + F;              /* U 2^F = M 2^sh */
    u128 X;
    if (sh >= 0) X = (u128)M << sh;
    else if (sh > -64) X = (u128)(M >> (-sh));
    else X = 0;
    u128 B = 2;
    for (int p = 1; p <= s; ++p) B += (u128)128 << (F - 8 * p);
    const u128 Y = X + B;
    for (int p = 1; p <= s; ++p) {
        const u128 q = Y >> (F - 8 * p);
        const int dg = (int)(p == 1 ? (uint64_t)q : (uint64_t)(q & 255)) - 128;
        d[(p - 1) * stride] = (int16_t)(neg ? -dg : dg);
    }
}

void orc_ozaki_split(int64_t rows, int64_t k, const double* r, int64_t rs, int64_t cs,
                     int slices, int32_t* exps, int16_t* digits)
{
    for (int64_t i = 0; i < rows; ++i) {
        double mx = 0.0;
        for (int64_t l = 0; l < k; ++l) { double v = fabs(r[i * rs + l * cs]); if (v > mx) mx = v; }
        const int e = (mx == 0.0) ? 0 : ilogb(mx) + 2;
        exps[i] = e;
        for (int64_t l = 0; l < k; ++l)
            oz_digits(r[i * rs + l * cs], e, slices, digits + i * k + l, rows * k);
    }
}

typedef struct {
    int64_t m, n, k; int s; const int16_t* da; const int16_t* db;
    const int32_t* ea; const int32_t* eb; double alpha, beta;
    double* c; int64_t rs_c, cs_c;
} oz_args;

static void oz_task(void* p, int tid, int nt)
{
    oz_args* g = (oz_args*)p;
    const int s = g->s;
    int64_t lev[64];
    for (int64_t i = tid; i < g->m; i += nt) {
        for (int64_t j = 0; j < g->n; ++j) {
            for (int l = 0; l <= s + 1; ++l) lev[l] = 0;
            for (int pa = 1; pa <= s; ++pa)
                for (int pb = 1; pa + pb <= s + 1; ++pb) {
                    const int16_t* ra = g->da + ((int64_t)(pa - 1) * g->m + i) * g->k;
                    const int16_t* rb = g->db + ((int64_t)(pb - 1) * g->n + j) * g->k;
                    int64_t acc = 0;
                    for (int64_t l = 0; l < g->k; ++l) acc += (int64_t)ra[l] * (int64_t)rb[l];
                    lev[pa + pb] += acc;
                }
            i128 T = 0;
            for (int l = 2; l <= s + 1; ++l) T += (i128)lev[l] * ((i128)1 << (8 * (s + 1 - l)));
            const double ab = oz_round_scaled(T, g->ea[i] + g->eb[j] - 8 * (s + 1));
            double* cij = g->c + i * g->rs_c + j * g->cs_c;
            if (g->alpha == 1.0 && g->beta == 0.0) { *cij = ab; continue; }
            const double t = g->alpha * ab;
            *cij = (g->beta == 0.0) ? t : fma(g->beta, *cij, t);
        }
    }
}

/* ---------------------------------------------------------------------- */
/* The CRT form of the Ozaki products, as a model of exact integers.       */
/* Each row of op(A) and of op(B)^T is scaled to integers                  */
/* X = RNE(|x| 2^(t+1-e)) with the sign of x (e = ilogb(row max) + 2, as   */
/* the digit form), C' = sum_l A'(i,l) B'(l,j) exactly, and the result is  */
/* RNE(C' 2^(e_i + e_j - 2t - 2)), then alpha and beta as in the digit     */
/* form.  t is the largest integer with k 2^(2t) <= floor(8 M / 17) for    */
/* the product M of the first n moduli (and 2t + ceil(log2 k) <= 126):     */
/* the device computes C' from n residue products by the Chinese           */
/* remainder theorem, which is exact under that bound, so the model needs  */
/* no moduli beyond choosing t.                                            */
static const int orc_crt_moduli[16] = {257, 256, 255, 253, 251, 247, 241, 239,
                                       233, 229, 227, 223, 217, 211, 199, 197};

int orc_ozaki_crt_bits(int n, int64_t k)
{
    if (n < 2 || n > 16 || k < 1) return -1;
    u128 M = 1;
    for (int l = 0; l < n; ++l) M *= (u128)orc_crt_moduli[l];
    const u128 lim = (M / 17) * 8 + ((M % 17) * 8) / 17;
    int kb = 0;
    while (kb < 63 && ((int64_t)1 << kb) < k) ++kb;
    for (int t = 62; t >= 1; --t) {
        if (2 * t + kb > 126) continue;
        if (((u128)k << (2 * t)) <= lim) return t;
    }
    return -1;
}

static int64_t crt_scaled(double x, int e, int t)
{
    uint64_t bits;
    memcpy(&bits, &x, sizeof bits);
    const int neg = (int)(bits >> 63);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const uint64_t M = (bits & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0ull);
    if (M == 0) return 0;
    const int E2 = ex ? ex - 1075 : -1074;
    const int sh = E2 + t + 1 - e;
    uint64_t X;
    if (sh >= 0) {
        X = M << sh;
    } else if (sh < -54) {
        X = 0;
    } else {
        const int r = -sh;
        const uint64_t q = M >> r, rem = M & ((1ull << r) - 1), half = 1ull << (r - 1);
        X = (rem > half || (rem == half && (q & 1ull))) ? q + 1 : q;
    }
    return neg ? -(int64_t)X : (int64_t)X;
}

static void crt_scale_rows(int64_t rows, int64_t k, const double* r, int64_t rs, int64_t cs, int t,
                           int32_t* exps, int64_t* X)
{
    for (int64_t i = 0; i < rows; ++i) {
        double mx = 0.0;
        for (int64_t l = 0; l < k; ++l) { double v = fabs(r[i * rs + l * cs]); if (v > mx) mx = v; }
        const int e = (mx == 0.0) ? 0 : ilogb(mx) + 2;
        exps[i] = e;
        for (int64_t l = 0; l < k; ++l) X[i * k + l] = crt_scaled(r[i * rs + l * cs], e, t);
    }
}

typedef struct {
    int64_t m, n, k; int t; const int64_t* xa; const int64_t* xb;
    const int32_t* ea; const int32_t* eb; double alpha, beta;
    double* c; int64_t rs_c, cs_c;
} crt_args;

static void crt_task(void* p, int tid, int nt)
{
    crt_args* g = (crt_args*)p;
    for (int64_t i = tid; i < g->m; i += nt) {
        for (int64_t j = 0; j < g->n; ++j) {
            const int64_t* ra = g->xa + i * g->k;
            const int64_t* rb = g->xb + j * g->k;
            i128 T = 0;
            for (int64_t l = 0; l < g->k; ++l) T += (i128)ra[l] * (i128)rb[l];
            const double ab = oz_round_scaled(T, g->ea[i] + g->eb[j] - 2 * g->t - 2);
            double* cij = g->c + i * g->rs_c + j * g->cs_c;
            if (g->alpha == 1.0 && g->beta == 0.0) { *cij = ab; continue; }
            const double tt = g->alpha * ab;
            *cij = (g->beta == 0.0) ? tt : fma(g->beta, *cij, tt);
        }
    }
}

int orc_ozaki_crt_dgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
                        double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                        const double* b, int64_t rs_b, int64_t cs_b,
                        double beta, double* c, int64_t rs_c, int64_t cs_c,
                        int moduli, int nthreads)
{
    if (m <= 0 || n <= 0) return 0;
    if (alpha == 0.0 || k <= 0) { d_scalm(m, n, beta, c, rs_c, cs_c); return 0; }
    const int t = orc_ozaki_crt_bits(moduli, k);
    if (t < 1) return -1;
    const int64_t ars = ORC_TRANS(transa) ? cs_a : rs_a, acs = ORC_TRANS(transa) ? rs_a : cs_a;
    const int64_t brs = ORC_TRANS(transb) ? cs_b : rs_b, bcs = ORC_TRANS(transb) ? rs_b : cs_b;
    for (int64_t i = 0; i < m; ++i) for (int64_t l = 0; l < k; ++l)
        if (!isfinite(a[i * ars + l * acs])) goto native;
    for (int64_t l = 0; l < k; ++l) for (int64_t j = 0; j < n; ++j)
        if (!isfinite(b[l * brs + j * bcs])) goto native;
    {
        int64_t* xa = (int64_t*)malloc(sizeof(int64_t) * (size_t)m * k);
        int64_t* xb = (int64_t*)malloc(sizeof(int64_t) * (size_t)n * k);
        int32_t* ea = (int32_t*)malloc(sizeof(int32_t) * m);
        int32_t* eb = (int32_t*)malloc(sizeof(int32_t) * n);
        crt_scale_rows(m, k, a, ars, acs, t, ea, xa);
        crt_scale_rows(n, k, b, bcs, brs, t, eb, xb);
        crt_args g = { m, n, k, t, xa, xb, ea, eb, alpha, beta, c, rs_c, cs_c };
        orc_parallel(crt_task, &g, nthreads < 1 ? 1 : nthreads);
        free(xa); free(xb); free(ea); free(eb);
        return 0;
    }
native:
    orc_dgemm(transa, transb, m, n, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c, nthreads);
    return 1;
}

int orc_ozaki_dgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
                    double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                    const double* b, int64_t rs_b, int64_t cs_b,
                    double beta, double* c, int64_t rs_c, int64_t cs_c,
                    int slices, int nthreads)
{
    if (m <= 0 || n <= 0) return 0;
    if (alpha == 0.0 || k <= 0) { d_scalm(m, n, beta, c, rs_c, cs_c); return 0; }
    if (slices < 2 || slices > 12 || oz_t_bound_log2(slices, k) >= 126.0) return -1;
    const int64_t ars = ORC_TRANS(transa) ? cs_a : rs_a, acs = ORC_TRANS(transa) ? rs_a : cs_a;
    const int64_t brs = ORC_TRANS(transb) ? cs_b : rs_b, bcs = ORC_TRANS(transb) ? rs_b : cs_b;
    /* non-finite operands cannot be sliced: the native FP64 path is used */
    for (int64_t i = 0; i < m; ++i) for (int64_t l = 0; l < k; ++l)
        if (!isfinite(a[i * ars + l * acs])) goto native;
    for (int64_t l = 0; l < k; ++l) for (int64_t j = 0; j < n; ++j)
        if (!isfinite(b[l * brs + j * bcs])) goto native;
    {
        int16_t* da = (int16_t*)malloc(sizeof(int16_t) * (size_t)slices * m * k);
        int16_t* db = (int16_t*)malloc(sizeof(int16_t) * (size_t)slices * n * k);
        int32_t* ea = (int32_t*)malloc(sizeof(int32_t) * m);
        int32_t* eb = (int32_t*)malloc(sizeof(int32_t) * n);
        orc_ozaki_split(m, k, a, ars, acs, slices, ea, da);
        /* rows of op(B)^T are the columns of op(B): element (j, l) = B(l, j) */
        orc_ozaki_split(n, k, b, bcs, brs, slices, eb, db);
        oz_args g = { m, n, k, slices, da, db, ea, eb, alpha, beta, c, rs_c, cs_c };
        orc_parallel(oz_task, &g, nthreads < 1 ? 1 : nthreads);
        free(da); free(db); free(ea); free(eb);
        return 0;
    }
native:
    orc_dgemm(transa, transb, m, n, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c, nthreads);
    return 1;
}

/* ------------------------------------------------------------------ */
/* herk / her2k / hemm / complex symm / syr2k                          */
/* ------------------------------------------------------------------ */
/* element (i, l) of op(X) with the conjugation bit of trans_t applied */
static void z_op(const double* x, int64_t rs, int64_t cs, int trans, int64_t i, int64_t l,
                 double* re, double* im)
{
    const int64_t r = ORC_TRANS(trans) ? l : i, c = ORC_TRANS(trans) ? i : l;
    const double* p = x + 2 * (r * rs + c * cs);
    *re = p[0];
    *im = (trans & 0x10) ? -p[1] : p[1];
}

/* sum_l op(X)(i, l) conj(op(Y)(j, l)), accumulated over l in order */
static void z_dot_conj(const double* x, int64_t xrs, int64_t xcs, int tx, const double* y,
                       int64_t yrs, int64_t ycs, int ty, int64_t i, int64_t j, int64_t k,
                       double* sr, double* si)
{
    double ar = 0.0, ai = 0.0;
    for (int64_t l = 0; l < k; ++l) {
        double xr, xi, yr, yi;
        z_op(x, xrs, xcs, tx, i, l, &xr, &xi);
        z_op(y, yrs, ycs, ty, j, l, &yr, &yi);
        yi = -yi;
        ar = fma(xr, yr, fma(-xi, yi, ar));
        ai = fma(xr, yi, fma(xi, yr, ai));
    }
    *sr = ar;
    *si = ai;
}

/* herk (frame/3/bli_l3_oapi_ex.c:295-320): gemmt with B = op(A)^H on the
   uplo triangle, c = alpha s + beta c (beta == 0 does not read c), then the
   imaginary parts of C's diagonal set to zero (bli_setid). */
void orc_zherk(int uplo, int transa, int64_t m, int64_t k, double alpha, const double* a,
               int64_t rs_a, int64_t cs_a, double beta, double* c, int64_t rs_c, int64_t cs_c)
{
    for (int64_t j = 0; j < m; ++j)
        for (int64_t i = 0; i < m; ++i) {
            if ((uplo == ORC_LOWER) ? (i < j) : (i > j)) continue;
            double sr = 0.0, si = 0.0;
            if (alpha != 0.0) z_dot_conj(a, rs_a, cs_a, transa, a, rs_a, cs_a, transa, i, j, k, &sr, &si);
            double* pc = c + 2 * (i * rs_c + j * cs_c);
            double cr = alpha * sr, ci = alpha * si;
            if (beta != 0.0) {
                cr += beta * pc[0];
                ci += beta * pc[1];
            }
            pc[0] = cr;
            pc[1] = (i == j) ? 0.0 : ci;
        }
}

/* her2k (frame/3/bli_l3_oapi_ex.c:229-264): alpha op(A) op(B)^H +
   conj(alpha) op(B) op(A)^H + beta c on the uplo triangle, the imaginary
   parts of C's diagonal set to zero. */
void orc_zher2k(int uplo, int transa, int transb, int64_t m, int64_t k, const double* alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c)
{
    const int nz = !(alpha[0] == 0.0 && alpha[1] == 0.0);
    for (int64_t j = 0; j < m; ++j)
        for (int64_t i = 0; i < m; ++i) {
            if ((uplo == ORC_LOWER) ? (i < j) : (i > j)) continue;
            double s1r = 0.0, s1i = 0.0, s2r = 0.0, s2i = 0.0;
            if (nz) {
                z_dot_conj(a, rs_a, cs_a, transa, b, rs_b, cs_b, transb, i, j, k, &s1r, &s1i);
                z_dot_conj(b, rs_b, cs_b, transb, a, rs_a, cs_a, transa, i, j, k, &s2r, &s2i);
            }
            double* pc = c + 2 * (i * rs_c + j * cs_c);
            double cr = (alpha[0] * s1r - alpha[1] * s1i) + (alpha[0] * s2r + alpha[1] * s2i);
            double ci = (alpha[0] * s1i + alpha[1] * s1r) + (alpha[0] * s2i - alpha[1] * s2r);
            if (beta != 0.0) {
                cr += beta * pc[0];
                ci += beta * pc[1];
            }
            pc[0] = cr;
            pc[1] = (i == j) ? 0.0 : ci;
        }
}

/* hemm (herm = 1) / complex symm (herm = 0) (frame/3/bli_l3_oapi_ex.c:349-520):
   the full A from its uplo triangle -- the other triangle reflected,
   conjugated for Hermitian A, the Hermitian diagonal read as real
   (ref_kernels/1m/bli_packm_cxc_diag_1er_ref.c:214-225) -- conjugated when
   conja, then the complex gemm with op(B) (transb). */
void orc_zhemm(int side, int uplo, int herm, int conja, int transb, int64_t m, int64_t n,
               const double* alpha, const double* a, int64_t rs_a, int64_t cs_a, const double* b,
               int64_t rs_b, int64_t cs_b, const double* beta, double* c, int64_t rs_c, int64_t cs_c)
{
    if (m <= 0 || n <= 0) return;
    const int64_t na = (side == ORC_LEFT) ? m : n;
    double* f = (double*)malloc(sizeof(double) * (size_t)(2 * na * na));
    for (int64_t j = 0; j < na; ++j)
        for (int64_t i = 0; i < na; ++i) {
            const int stored = (uplo == ORC_LOWER) ? (i >= j) : (i <= j);
            const double* p = stored ? a + 2 * (i * rs_a + j * cs_a) : a + 2 * (j * rs_a + i * cs_a);
            double im = p[1];
            if (herm && !stored) im = -im;
            if (herm && i == j) im = 0.0;
            if (conja) im = -im;
            f[2 * (i + j * na)] = p[0];
            f[2 * (i + j * na) + 1] = im;
        }
    if (side == ORC_LEFT)
        orc_zgemm(ORC_NO_TRANSPOSE, transb, m, n, m, alpha, f, 1, na, b, rs_b, cs_b, beta, c, rs_c, cs_c);
    else
        orc_zgemm(transb, ORC_NO_TRANSPOSE, m, n, n, alpha, b, rs_b, cs_b, f, 1, na, beta, c, rs_c, cs_c);
    free(f);
}

/* syr2k (frame/3/bli_l3_oapi_ex.c:267-292): two gemmt calls, the second
   with beta = 1. */
void orc_dsyr2k(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads)
{
    const int ta = ORC_TRANS(transa), tb = ORC_TRANS(transb);
    orc_dgemmt(uplo, ta ? ORC_TRANSPOSE : ORC_NO_TRANSPOSE, tb ? ORC_NO_TRANSPOSE : ORC_TRANSPOSE, m, k,
               alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c, nthreads);
    orc_dgemmt(uplo, tb ? ORC_TRANSPOSE : ORC_NO_TRANSPOSE, ta ? ORC_NO_TRANSPOSE : ORC_TRANSPOSE, m, k,
               alpha, b, rs_b, cs_b, a, rs_a, cs_a, 1.0, c, rs_c, cs_c, nthreads);
}

/* trmm3 (frame/3/bli_l3_oapi_ex.c:523-608): C := beta C + alpha op(A) op(B)
   (left) or beta C + alpha op(B) op(A) (right) on the dense tri(A) through
   the gemm below; alpha == 0 scales C only (frame/3/bli_l3_util.c:41-65). */
void orc_dtrmm3(int side, int uplo, int transa, int diag, int transb, int64_t m, int64_t n,
                double alpha, const double* a, int64_t rs_a, int64_t cs_a, const double* b,
                int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c,
                int nthreads)
{
    if (m <= 0 || n <= 0) return;
    const int64_t na = (side == ORC_LEFT) ? m : n;
    if (alpha == 0.0) {
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < m; ++i)
                c[i * rs_c + j * cs_c] = (beta == 0.0) ? 0.0 : beta * c[i * rs_c + j * cs_c];
        return;
    }
    double* t = (double*)calloc((size_t)(na * na), sizeof(double));
    for (int64_t j = 0; j < na; ++j)
        for (int64_t i = 0; i < na; ++i) {
            const int in = (uplo == ORC_LOWER) ? (i >= j) : (i <= j);
            if (i == j) t[i + j * na] = (diag == ORC_UNIT_DIAG) ? 1.0 : a[i * rs_a + j * cs_a];
            else if (in) t[i + j * na] = a[i * rs_a + j * cs_a];
        }
    if (side == ORC_LEFT)
        orc_dgemm(transa, transb, m, n, m, alpha, t, 1, na, b, rs_b, cs_b, beta, c, rs_c, cs_c, nthreads);
    else
        orc_dgemm(transb, transa, m, n, n, alpha, b, rs_b, cs_b, t, 1, na, beta, c, rs_c, cs_c, nthreads);
    free(t);
}
