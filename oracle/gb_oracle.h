/*
 * gb_oracle.h -- CPU restatement of the BLIS dense hot path, used ONLY as
 * test infrastructure: the parity checker of the pytest suite, the smoke
 * check, and the timed CPU baseline of bench.py.  Nothing in the product
 * library (blis_gb300/csrc) links or calls this code.
 *
 * Enum values follow BLIS's bit encodings (frame/include/bli_type_defs.h:
 * trans_t :395-401, conj_t :403-407, uplo_t :409-415, side_t :417-421,
 * diag_t :423-427) so that the same integers drive the oracle and the
 * product's typed API.
 *
 * Parity pins (what the oracle is checked against before it is trusted):
 *   - the DDOT/DAXPY golden vectors of the netlib BLAS test driver shipped
 *     with the reference (blastest/src/dblat1.c:424-431, check2_ :590-660),
 *     extracted as text into tests/golden/dblat1_check2.json;
 *   - "narrow power of two" inputs (frame/include/bli_cast_macro_defs.h:
 *     477-525), on which every product and partial sum is exact, so any
 *     correct gemm/gemv/dotv must agree bit for bit;
 *   - the DMMCH test-ratio criterion of blastest/src/dblat3.c:4109-4290 on
 *     the DBEG-generated matrices (dblat3.c:4458-4505) for the N, ALPHA and
 *     BETA values of blastest/input/dblat3.in;
 *   - the testsuite residual of testsuite/src/test_gemm.c:303-414 and
 *     test_trsm.c:292-389 against a double-double evaluation.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BLIS enum encodings (values only; frame/include/bli_type_defs.h). */
enum { ORC_NO_TRANSPOSE = 0x00, ORC_TRANSPOSE = 0x08,
       ORC_CONJ_NO_TRANSPOSE = 0x10, ORC_CONJ_TRANSPOSE = 0x18 };
enum { ORC_NO_CONJUGATE = 0x00, ORC_CONJUGATE = 0x10 };
enum { ORC_LOWER = 0xC0, ORC_UPPER = 0x60 };
enum { ORC_LEFT = 0, ORC_RIGHT = 1 };
enum { ORC_NONUNIT_DIAG = 0x000, ORC_UNIT_DIAG = 0x100 };

/* ---- counter-based RNG (SplitMix64 finaliser over seed and index) ---- */
uint64_t orc_mix64(uint64_t x);
uint64_t orc_hash(uint64_t seed, uint64_t idx);
void orc_fill_uniform(double* x, int64_t n, uint64_t seed, double lo, double hi);
void orc_fill_uniform_f(float* x, int64_t n, uint64_t seed, double lo, double hi);
void orc_fill_expspread(double* x, int64_t n, uint64_t seed, int emin, int emax);
void orc_fill_narrow_pow2(double* x, int64_t n, uint64_t seed);

/* ---- level-3 ---- */
void orc_dgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
               double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               const double* b, int64_t rs_b, int64_t cs_b,
               double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads);
void orc_sgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
               float alpha, const float* a, int64_t rs_a, int64_t cs_a,
               const float* b, int64_t rs_b, int64_t cs_b,
               float beta, float* c, int64_t rs_c, int64_t cs_c, int nthreads);
void orc_dtrsm(int side, int uplo, int transa, int diag, int64_t m, int64_t n,
               double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               double* b, int64_t rs_b, int64_t cs_b, int nthreads);
void orc_dtrmm(int side, int uplo, int transa, int diag, int64_t m, int64_t n,
               double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               double* b, int64_t rs_b, int64_t cs_b, int nthreads);
void orc_dsymm(int side, int uplo, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
               int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads);
void orc_dgemmt(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads);

/* ---- level-2 / level-1v ---- */
void orc_dgemv(int transa, int conjx, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a,
               const double* x, int64_t incx, double beta, double* y, int64_t incy);
void orc_daxpyv(int conjx, int64_t n, double alpha, const double* x, int64_t incx,
                double* y, int64_t incy);
void orc_zgemm(int transa, int transb, int64_t m, int64_t n, int64_t k, const double* alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b,
               const double* beta, double* c, int64_t rs_c, int64_t cs_c);
void orc_zherk(int uplo, int transa, int64_t m, int64_t k, double alpha, const double* a,
               int64_t rs_a, int64_t cs_a, double beta, double* c, int64_t rs_c, int64_t cs_c);
void orc_zher2k(int uplo, int transa, int transb, int64_t m, int64_t k, const double* alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c);
void orc_zhemm(int side, int uplo, int herm, int conja, int transb, int64_t m, int64_t n,
               const double* alpha, const double* a, int64_t rs_a, int64_t cs_a, const double* b,
               int64_t rs_b, int64_t cs_b, const double* beta, double* c, int64_t rs_c, int64_t cs_c);
void orc_dtrmm3(int side, int uplo, int transa, int diag, int transb, int64_t m, int64_t n,
                double alpha, const double* a, int64_t rs_a, int64_t cs_a, const double* b,
                int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c,
                int nthreads);
void orc_dsyr2k(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha,
                const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b,
                int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c, int nthreads);
void orc_dscalv(int64_t n, double alpha, double* x, int64_t incx);
void orc_dcopyv(int64_t n, const double* x, int64_t incx, double* y, int64_t incy);
void orc_damaxv(int64_t n, const double* x, int64_t incx, int64_t* index);
void orc_dger(int64_t m, int64_t n, double alpha, const double* x, int64_t incx, const double* y,
              int64_t incy, double* a, int64_t rs_a, int64_t cs_a);
void orc_dtrsv(int uplo, int transa, int diag, int64_t m, double alpha, const double* a, int64_t rs_a,
               int64_t cs_a, double* x, int64_t incx);
void orc_ddotv(int conjx, int conjy, int64_t n, const double* x, int64_t incx,
               const double* y, int64_t incy, double* rho);

/* ---- double-double evaluation (error oracle; no reference counterpart) ---- */
void orc_dd_gemm_entries(int transa, int transb, int64_t m, int64_t n, int64_t k,
                         double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                         const double* b, int64_t rs_b, int64_t cs_b,
                         double beta, const double* c, int64_t rs_c, int64_t cs_c,
                         int64_t nent, const int64_t* ii, const int64_t* jj,
                         double* hi, double* lo, int nthreads);
void orc_dd_dotv(int64_t n, const double* x, int64_t incx, const double* y,
                 int64_t incy, double* hi, double* lo);

/* ---- Ozaki split-product model (bit-exact model of the GPU form) ---- */
int64_t orc_ozaki_kpart_limit(int npairs);
void orc_ozaki_split(int64_t rows, int64_t k, const double* r, int64_t rs, int64_t cs,
                     int slices, int32_t* exps, int16_t* digits);
/* the CRT form (integer bits t for n moduli and depth k; the model) */
int orc_ozaki_crt_bits(int n, int64_t k);
int orc_ozaki_crt_dgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
                        double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                        const double* b, int64_t rs_b, int64_t cs_b,
                        double beta, double* c, int64_t rs_c, int64_t cs_c,
                        int moduli, int nthreads);
int orc_ozaki_dgemm(int transa, int transb, int64_t m, int64_t n, int64_t k,
                    double alpha, const double* a, int64_t rs_a, int64_t cs_a,
                    const double* b, int64_t rs_b, int64_t cs_b,
                    double beta, double* c, int64_t rs_c, int64_t cs_c,
                    int slices, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
