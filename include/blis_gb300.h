/*
 * blis_gb300.h -- C ABI of libblis_gb300.so, the GB300 (sm_103a) implementation
 * of BLIS's dense hot path.
 *
 * Three groups of entry points:
 *
 *  1. Drop-ins with the exact signatures of the BLIS 1.0 entry points they
 *     replace (BLAS compat layer, CBLAS, typed BLIS API).  They take HOST
 *     pointers owned by the caller, move the operands through HBM, and
 *     return with the result in place, like the CPU library.  Argument errors
 *     go through xerbla_ exactly as frame/compat/check/bla_*_check.h does.
 *  2. The "gb_" addon (device pointers, explicit CUDA stream) used by callers
 *     that keep operands resident in HBM; the drop-ins are built on it.
 *  3. Controls and introspection (precision mode, status, counters).
 *
 * Citations are to the BLIS 1.0 source tree (file:line).
 * Integer widths follow BLIS: dim_t/inc_t are int64_t
 * (frame/include/bli_type_defs.h:112-115); the BLAS integer is 32-bit
 * (BLIS_BLAS_INT_TYPE_SIZE 32 default).  trans_t/conj_t/uplo_t/side_t/diag_t
 * carry BLIS's bit encodings (frame/include/bli_type_defs.h:395-427).
 */
#ifndef BLIS_GB300_H
#define BLIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t gb_dim_t;  /* dim_t */
typedef int64_t gb_inc_t;  /* inc_t */
typedef int32_t gb_f77_int;  /* f77_int (32-bit BLAS integer) */
typedef char gb_f77_char;  /* f77_char */
typedef int gb_trans_t;    /* trans_t: 0x00 N, 0x08 T, 0x10 conj-N, 0x18 conj-T */
typedef int gb_conj_t;     /* conj_t:  0x00, 0x10 */
typedef int gb_uplo_t;     /* uplo_t:  0xC0 lower, 0x60 upper */
typedef int gb_side_t;     /* side_t:  0 left, 1 right */
typedef int gb_diag_t;     /* diag_t:  0x000 non-unit, 0x100 unit */

#define GB_NO_TRANSPOSE 0x00
#define GB_TRANSPOSE 0x08
#define GB_CONJ_NO_TRANSPOSE 0x10
#define GB_CONJ_TRANSPOSE 0x18
#define GB_NO_CONJUGATE 0x00
#define GB_CONJUGATE 0x10
/* scomplex / dcomplex, frame/include/bli_type_defs.h:191-206: interleaved
   (real, imag); complex strides and leading dimensions count complex
   elements */
typedef struct { float real, imag; } gb_scomplex;
typedef struct { double real, imag; } gb_dcomplex;

#define GB_LOWER 0xC0
#define GB_UPPER 0x60
#define GB_LEFT 0
#define GB_RIGHT 1
#define GB_NONUNIT_DIAG 0x000
#define GB_UNIT_DIAG 0x100

/* Status codes of the gb_ addon (0 = success). */
#define GB_SUCCESS 0
#define GB_ERR_ARG (-1)
#define GB_ERR_CUDA (-2)
#define GB_ERR_DEVICE (-3)   /* a kernel reported a bounded-wait timeout or bad index */
#define GB_ERR_NOMEM (-4)
#define GB_ERR_UNSUPPORTED (-5)

/* Code compiled against BLIS's own blis.h (a gemm sandbox, the glue library
   that registers kernels in BLIS's context) defines GB300_ADDON_ONLY before
   including this header: the BLAS, CBLAS and typed bli_ declarations of
   groups 1a-1c would clash with blis.h's, and that code calls the gb_ names
   below, which cannot resolve back into libblis. */
#ifndef GB300_ADDON_ONLY

/* ===================================================================== */
/* 1a. Fortran-77 BLAS compat layer                                        */
/* ===================================================================== */

/* replaces dgemm_/sgemm_, frame/compat/bla_gemm.c:122-262 (m==1 / n==1 go
   to gemv as in :180-218; checks frame/compat/check/bla_gemm_check.h:37-86) */
void dgemm_(const gb_f77_char* transa, const gb_f77_char* transb,
            const gb_f77_int* m, const gb_f77_int* n, const gb_f77_int* k,
            const double* alpha, const double* a, const gb_f77_int* lda,
            const double* b, const gb_f77_int* ldb,
            const double* beta, double* c, const gb_f77_int* ldc);
void sgemm_(const gb_f77_char* transa, const gb_f77_char* transb,
            const gb_f77_int* m, const gb_f77_int* n, const gb_f77_int* k,
            const float* alpha, const float* a, const gb_f77_int* lda,
            const float* b, const gb_f77_int* ldb,
            const float* beta, float* c, const gb_f77_int* ldc);

/* replaces dtrsm_, frame/compat/bla_trsm.c:121-219 (checks
   frame/compat/check/bla_trmm_check.h:37-86) */
void dtrsm_(const gb_f77_char* side, const gb_f77_char* uploa,
            const gb_f77_char* transa, const gb_f77_char* diaga,
            const gb_f77_int* m, const gb_f77_int* n, const double* alpha,
            const double* a, const gb_f77_int* lda, double* b, const gb_f77_int* ldb);
/* replaces strsm_ (the same macro instance of frame/compat/bla_trsm.c:121-219) */
void strsm_(const gb_f77_char* side, const gb_f77_char* uploa,
            const gb_f77_char* transa, const gb_f77_char* diaga,
            const gb_f77_int* m, const gb_f77_int* n, const float* alpha,
            const float* a, const gb_f77_int* lda, float* b, const gb_f77_int* ldb);

/* replaces dtrmm_, frame/compat/bla_trmm.c:45-121 (checks
   frame/compat/check/bla_trmm_check.h:37-86): B := alpha op(A) B or alpha B op(A) */
void dtrmm_(const gb_f77_char* side, const gb_f77_char* uploa,
            const gb_f77_char* transa, const gb_f77_char* diaga,
            const gb_f77_int* m, const gb_f77_int* n, const double* alpha,
            const double* a, const gb_f77_int* lda, double* b, const gb_f77_int* ldb);

/* replaces dsymm_, frame/compat/bla_symm.c:45-119 (checks
   frame/compat/check/bla_hemm_check.h:37-81): C := alpha A B + beta C or
   alpha B A + beta C, A symmetric, only the uploa triangle of A read */
void dsymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m,
            const gb_f77_int* n, const double* alpha, const double* a, const gb_f77_int* lda,
            const double* b, const gb_f77_int* ldb, const double* beta, double* c,
            const gb_f77_int* ldc);

/* replaces dsyrk_, frame/compat/bla_syrk.c:45-121 (checks
   frame/compat/check/bla_syrk_check.h:37-84): C := alpha op(A) op(A)^T + beta C on
   the uploc triangle, through gemmt as bli_syrk_ex does
   (frame/3/bli_l3_oapi_ex.c:326-345) */
void dsyrk_(const gb_f77_char* uploc, const gb_f77_char* transa, const gb_f77_int* m,
            const gb_f77_int* k, const double* alpha, const double* a, const gb_f77_int* lda,
            const double* beta, double* c, const gb_f77_int* ldc);

/* replaces dgemmt_, frame/compat/extra/bla_gemmt.c:45-121 (checks
   frame/compat/check/bla_gemmt_check.h:37-92): C := alpha op(A) op(B) + beta C on
   the uploc triangle of the m x m C; the other triangle is not touched */
void dgemmt_(const gb_f77_char* uploc, const gb_f77_char* transa, const gb_f77_char* transb,
             const gb_f77_int* m, const gb_f77_int* k, const double* alpha, const double* a,
             const gb_f77_int* lda, const double* b, const gb_f77_int* ldb, const double* beta,
             double* c, const gb_f77_int* ldc);

/* replace zgemm_ / cgemm_ (frame/compat/bla_gemm.c:122-262 for the complex
   types; checks frame/compat/check/bla_gemm_check.h: 'C' is the conjugate
   transpose): one real gemm on the block-real form [Ar -Ai; Ai Ar] [Br; Bi],
   the GPU counterpart of BLIS's induced methods (frame/3/bli_l3_ind.c,
   ref_kernels/ind/bli_gemm1m_ref.c).  m == 1 or n == 1 is computed as a gemm
   (the reference sends it to gemv, frame/compat/bla_gemm.c:180-218) */
void zgemm_(const gb_f77_char* transa, const gb_f77_char* transb,
            const gb_f77_int* m, const gb_f77_int* n, const gb_f77_int* k,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda,
            const gb_dcomplex* b, const gb_f77_int* ldb, const gb_dcomplex* beta,
            gb_dcomplex* c, const gb_f77_int* ldc);
void cgemm_(const gb_f77_char* transa, const gb_f77_char* transb,
            const gb_f77_int* m, const gb_f77_int* n, const gb_f77_int* k,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda,
            const gb_scomplex* b, const gb_f77_int* ldb, const gb_scomplex* beta,
            gb_scomplex* c, const gb_f77_int* ldc);

/* replaces ztrsm_, frame/compat/bla_trsm.c:121-219 for dcomplex (checks
   frame/compat/check/bla_trmm_check.h:37-86; 'C' solves with A^H): the
   recursive solve with complex diagonal-block kernels and complex gemm
   updates */
void ztrsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, gb_dcomplex* b,
            const gb_f77_int* ldb);
/* replaces ctrsm_ (the scomplex instance of frame/compat/bla_trsm.c:121-219) */
void ctrsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, gb_scomplex* b,
            const gb_f77_int* ldb);

/* replace zherk_ / cherk_ (frame/compat/bla_herk.c:45-130, checks
   frame/compat/check/bla_herk_check.h:37-77; trans N or C; the BLAS early
   return when nothing is added and beta == 1), zher2k_ / cher2k_
   (frame/compat/bla_her2k.c:45-136, checks bla_her2k_check.h:37-79), zhemm_
   / chemm_ (frame/compat/bla_hemm.c:45-120), zsymm_ / csymm_
   (frame/compat/bla_symm.c:45-120; checks bla_hemm_check.h:37-79) and
   dsyr2k_ (frame/compat/bla_syr2k.c:45-128, checks bla_syr2k_check.h:37-84):
   herk and her2k as one real gemmt on interleaved block-real operands, the
   imaginary parts of C's diagonal zeroed (frame/3/bli_l3_oapi_ex.c:229-320);
   hemm / symm as the complex gemm on the materialised A; syr2k as two
   gemmt calls (frame/3/bli_l3_oapi_ex.c:267-292) */
void zherk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const double* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const double* beta,
            gb_dcomplex* c, const gb_f77_int* ldc);
void cherk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const float* alpha, const gb_scomplex* a, const gb_f77_int* lda, const float* beta,
            gb_scomplex* c, const gb_f77_int* ldc);
void zher2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
             const gb_f77_int* ldb, const double* beta, gb_dcomplex* c, const gb_f77_int* ldc);
void cher2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
             const gb_f77_int* ldb, const float* beta, gb_scomplex* c, const gb_f77_int* ldc);
/* replace zgemv_ / cgemv_ (frame/compat/bla_gemv.c:45-143, checks
   frame/compat/check/bla_gemv_check.h:37-75; negative increments address
   the vectors from their far end) */
void zgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const gb_dcomplex* alpha,
            const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* x, const gb_f77_int* incx,
            const gb_dcomplex* beta, gb_dcomplex* y, const gb_f77_int* incy);
void cgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const gb_scomplex* alpha,
            const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* x, const gb_f77_int* incx,
            const gb_scomplex* beta, gb_scomplex* y, const gb_f77_int* incy);
/* replace ztrmm_ / ctrmm_ (frame/compat/bla_trmm.c:45-121, checks
   frame/compat/check/bla_trmm_check.h:37-86) */
void ztrmm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_dcomplex* alpha,
            const gb_dcomplex* a, const gb_f77_int* lda, gb_dcomplex* b, const gb_f77_int* ldb);
void ctrmm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_scomplex* alpha,
            const gb_scomplex* a, const gb_f77_int* lda, gb_scomplex* b, const gb_f77_int* ldb);
/* replace zsyrk_ / csyrk_ (frame/compat/bla_syrk.c:45-121) and zsyr2k_ /
   csyr2k_ (frame/compat/bla_syr2k.c:45-128); checks
   frame/compat/check/bla_syrk_check.h:37-84 and bla_syr2k_check.h:37-84
   (complex: trans N or T, 'C' is info 2); the BLAS early return when nothing
   is added and beta == 1 */
void zsyrk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* beta,
            gb_dcomplex* c, const gb_f77_int* ldc);
void csyrk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* beta,
            gb_scomplex* c, const gb_f77_int* ldc);
void zsyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
             const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc);
void csyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
             const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc);
void zhemm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
            const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc);
void chemm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
            const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc);
void zsymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
            const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc);
void csymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
            const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc);
void dsyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const double* alpha, const double* a, const gb_f77_int* lda, const double* b, const gb_f77_int* ldb,
             const double* beta, double* c, const gb_f77_int* ldc);

/* replace dscal_ (frame/compat/bla_scal.c:44-85; alpha == 0 sets zeros
   without reading x, ref_kernels/1/bli_scalv_ref.c:54-75), dcopy_
   (frame/compat/bla_copy.c:44-81), idamax_ (frame/compat/bla_amax.c:44-91:
   1-based, 0 for n < 1 or incx <= 0; the first NaN, else the first largest
   |x_i|, ref_kernels/1/bli_amaxv_ref.c:97-106), dger_ (frame/compat/bla_ger.c:
   44-106, checks frame/compat/check/bla_ger_check.h:37-68) and dtrsv_
   (frame/compat/bla_trsv.c:44-113, checks bla_trmv_check.h:37-77) */
void dscal_(const gb_f77_int* n, const double* alpha, double* x, const gb_f77_int* incx);
void dcopy_(const gb_f77_int* n, const double* x, const gb_f77_int* incx, double* y,
            const gb_f77_int* incy);
gb_f77_int idamax_(const gb_f77_int* n, const double* x, const gb_f77_int* incx);
void dger_(const gb_f77_int* m, const gb_f77_int* n, const double* alpha, const double* x,
           const gb_f77_int* incx, const double* y, const gb_f77_int* incy, double* a,
           const gb_f77_int* lda);
void dtrsv_(const gb_f77_char* uploa, const gb_f77_char* transa, const gb_f77_char* diaga,
            const gb_f77_int* m, const double* a, const gb_f77_int* lda, double* x,
            const gb_f77_int* incx);

/* replaces dgemv_, frame/compat/bla_gemv.c:45-143 (checks
   frame/compat/check/bla_gemv_check.h:37-75; n_x == 0 returns untouched, :95-106) */
void dgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n,
            const double* alpha, const double* a, const gb_f77_int* lda,
            const double* x, const gb_f77_int* incx, const double* beta,
            double* y, const gb_f77_int* incy);

/* replaces daxpy_, frame/compat/bla_axpy.c:45-86 (negative increments:
   frame/include/bli_blas_macro_defs.h:50-75) */
void daxpy_(const gb_f77_int* n, const double* alpha, const double* x,
            const gb_f77_int* incx, double* y, const gb_f77_int* incy);

/* replaces ddot_, frame/compat/bla_dot.c:45-93 */
double ddot_(const gb_f77_int* n, const double* x, const gb_f77_int* incx,
             const double* y, const gb_f77_int* incy);

/* replaces dgemm_batch_/sgemm_batch_, frame/compat/extra/bla_gemm_batch.c:135-249
   (the reference loops over the problems serially, :227; here every group
   member of every group runs in one grouped launch) */
void dgemm_batch_(const gb_f77_char* transa_array, const gb_f77_char* transb_array,
                  const gb_f77_int* m_array, const gb_f77_int* n_array,
                  const gb_f77_int* k_array, const double* alpha_array,
                  const double** a_array, const gb_f77_int* lda_array,
                  const double** b_array, const gb_f77_int* ldb_array,
                  const double* beta_array, double** c_array,
                  const gb_f77_int* ldc_array, const gb_f77_int* group_count,
                  const gb_f77_int* group_size);
void sgemm_batch_(const gb_f77_char* transa_array, const gb_f77_char* transb_array,
                  const gb_f77_int* m_array, const gb_f77_int* n_array,
                  const gb_f77_int* k_array, const float* alpha_array,
                  const float** a_array, const gb_f77_int* lda_array,
                  const float** b_array, const gb_f77_int* ldb_array,
                  const float* beta_array, float** c_array,
                  const gb_f77_int* ldc_array, const gb_f77_int* group_count,
                  const gb_f77_int* group_size);

/* replaces xerbla_, frame/compat/f2c/bla_xerbla.c:45-88 (prints, returns) */
int xerbla_(const gb_f77_char* srname, const gb_f77_int* info, long srname_len);

/* ===================================================================== */
/* 1b. CBLAS (frame/compat/cblas/src)                                     */
/* ===================================================================== */
enum GB_CBLAS_ORDER { GbCblasRowMajor = 101, GbCblasColMajor = 102 };
enum GB_CBLAS_TRANSPOSE { GbCblasNoTrans = 111, GbCblasTrans = 112, GbCblasConjTrans = 113 };
enum GB_CBLAS_UPLO { GbCblasUpper = 121, GbCblasLower = 122 };
enum GB_CBLAS_DIAG { GbCblasNonUnit = 131, GbCblasUnit = 132 };
enum GB_CBLAS_SIDE { GbCblasLeft = 141, GbCblasRight = 142 };

/* replaces cblas_dgemm, frame/compat/cblas/src/cblas_dgemm.c:14-110 */
void cblas_dgemm(int order, int transa, int transb, gb_f77_int m, gb_f77_int n,
                 gb_f77_int k, double alpha, const double* a, gb_f77_int lda,
                 const double* b, gb_f77_int ldb, double beta, double* c, gb_f77_int ldc);
/* replaces cblas_sgemm, frame/compat/cblas/src/cblas_sgemm.c:14-110 */
void cblas_sgemm(int order, int transa, int transb, gb_f77_int m, gb_f77_int n,
                 gb_f77_int k, float alpha, const float* a, gb_f77_int lda,
                 const float* b, gb_f77_int ldb, float beta, float* c, gb_f77_int ldc);
/* replaces cblas_dtrsm, frame/compat/cblas/src/cblas_dtrsm.c:12-140 */
void cblas_dtrsm(int order, int side, int uplo, int transa, int diag, gb_f77_int m,
                 gb_f77_int n, double alpha, const double* a, gb_f77_int lda,
                 double* b, gb_f77_int ldb);
/* replaces cblas_dgemv, frame/compat/cblas/src/cblas_dgemv.c:11-80 */
void cblas_dgemv(int order, int transa, gb_f77_int m, gb_f77_int n, double alpha,
                 const double* a, gb_f77_int lda, const double* x, gb_f77_int incx,
                 double beta, double* y, gb_f77_int incy);
/* replaces cblas_daxpy / cblas_ddot, frame/compat/cblas/src/cblas_daxpy.c, cblas_ddot.c */
void cblas_daxpy(gb_f77_int n, double alpha, const double* x, gb_f77_int incx, double* y,
                 gb_f77_int incy);
double cblas_ddot(gb_f77_int n, const double* x, gb_f77_int incx, const double* y,
                  gb_f77_int incy);
/* replaces cblas_dgemm_batch, frame/compat/cblas/src/extra/cblas_dgemm_batch.c:14-168 */
void cblas_dgemm_batch(int order, const int* transa_array, const int* transb_array,
                       const gb_f77_int* m_array, const gb_f77_int* n_array,
                       const gb_f77_int* k_array, const double* alpha_array,
                       const double** a_array, const gb_f77_int* lda_array,
                       const double** b_array, const gb_f77_int* ldb_array,
                       const double* beta_array, double** c_array,
                       const gb_f77_int* ldc_array, gb_f77_int group_count,
                       const gb_f77_int* group_size);

/* ===================================================================== */
/* 1c. Typed BLIS API (host pointers, general strides)                     */
/* ===================================================================== */

/* replaces bli_dgemm / bli_sgemm, frame/3/bli_l3_tapi.c (basic) and
   bli_?gemm_ex, frame/3/bli_l3_tapi_ex.c:42-99 (cntx/rntm accepted and ignored) */
void bli_dgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta,
               double* c, gb_inc_t rs_c, gb_inc_t cs_c);
void bli_dgemm_ex(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                  const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta,
                  double* c, gb_inc_t rs_c, gb_inc_t cs_c, const void* cntx, const void* rntm);
void bli_sgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const float* b, gb_inc_t rs_b, gb_inc_t cs_b, const float* beta,
               float* c, gb_inc_t rs_c, gb_inc_t cs_c);

/* replace bli_zgemm / bli_cgemm (frame/3/bli_l3_tapi_ex.c:45-99 for the
   complex types; trans_t carries the conjugation bit 0x10) */
void bli_zgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta,
               gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);
void bli_cgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta,
               gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);

/* replaces bli_ztrsm (frame/3/bli_l3_tapi_ex.c:536-586 for dcomplex) */
void bli_ztrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               gb_dim_t n, const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a,
               gb_inc_t cs_a, gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b);
/* replaces bli_ctrsm (the same, for scomplex) */
void bli_ctrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               gb_dim_t n, const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a,
               gb_inc_t cs_a, gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b);

/* replace bli_zherk / bli_cherk, bli_zher2k / bli_cher2k, bli_zhemm /
   bli_chemm, bli_zsymm / bli_csymm and bli_dsyr2k (frame/3/bli_l3_tapi_ex.c;
   prototypes frame/3/bli_l3_tapi_ex.h:62-168): herk takes real alpha and
   beta, her2k a real beta; hemm / symm take conja (conjugates A) and transb */
/* replace bli_zgemv / bli_cgemv (frame/2/bli_l2_tapi.c:43-127): trans_t may
   carry the conjugation bit 0x10, conjx conjugates x */
void bli_zgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const gb_dcomplex* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* x, gb_inc_t incx,
               const gb_dcomplex* beta, gb_dcomplex* y, gb_inc_t incy);
void bli_cgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const gb_scomplex* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* x, gb_inc_t incx,
               const gb_scomplex* beta, gb_scomplex* y, gb_inc_t incy);
/* replace bli_ztrmm / bli_ctrmm (frame/3/bli_l3_tapi_ex.c; trans_t may carry
   the conjugation bit 0x10) */
void bli_ztrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b);
void bli_ctrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b);
/* replace bli_zsyrk / bli_csyrk and bli_zsyr2k / bli_csyr2k (the same
   files): complex alpha and beta, C's stored triangle only */
void bli_zsyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const gb_dcomplex* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* beta, gb_dcomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_csyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const gb_scomplex* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* beta, gb_scomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_zsyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);
void bli_csyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);
void bli_zherk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const double* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* beta, gb_dcomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_cherk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const float* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const float* beta, gb_scomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_zher2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, gb_dcomplex* c,
                gb_inc_t rs_c, gb_inc_t cs_c);
void bli_cher2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const float* beta, gb_scomplex* c,
                gb_inc_t rs_c, gb_inc_t cs_c);
void bli_zhemm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_chemm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_zsymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_csymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
/* replaces bli_dtrmm3 (frame/3/bli_l3_tapi_ex.c; prototype frame/3/bli_l3_tapi_ex.h:170-192; object
   form frame/3/bli_l3_oapi_ex.c:523-608): C := beta C + alpha op(A) op(B) (left) or
   beta C + alpha op(B) op(A) (right), A triangular, B not written */
void bli_dtrmm3(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_trans_t transb,
                gb_dim_t m, gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c,
                gb_inc_t cs_c);
void bli_dsyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c);

/* replace bli_dscalv (frame/1/bli_l1v_tapi.c:314-345), bli_dcopyv (:46-77),
   bli_damaxv (:84-112), bli_dger (frame/2/bli_l2_tapi.c:129-175) and
   bli_dtrsv (:441-509); conjugation is the identity for real data */
void bli_dscalv(gb_conj_t conjalpha, gb_dim_t n, const double* alpha, double* x, gb_inc_t incx);
void bli_dcopyv(gb_conj_t conjx, gb_dim_t n, const double* x, gb_inc_t incx, double* y,
                gb_inc_t incy);
void bli_damaxv(gb_dim_t n, const double* x, gb_inc_t incx, gb_dim_t* index);
void bli_dger(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t m, gb_dim_t n, const double* alpha,
              const double* x, gb_inc_t incx, const double* y, gb_inc_t incy, double* a,
              gb_inc_t rs_a, gb_inc_t cs_a);
void bli_dtrsv(gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* x,
               gb_inc_t incx);

/* replace bli_dtrmm (frame/3/bli_l3_tapi_ex.c:536-585), bli_dsymm
   (:104-164; conja is the identity for real data, transb applies to B),
   bli_dsyrk (:290-339) and bli_dgemmt (:408-463) */
void bli_dtrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
               double* b, gb_inc_t rs_b, gb_inc_t cs_b);
void bli_dsymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m,
               gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_dsyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const double* alpha,
               const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* beta, double* c,
               gb_inc_t rs_c, gb_inc_t cs_c);
void bli_dgemmt(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c,
                gb_inc_t cs_c);

/* replaces bli_dtrsm / bli_dtrsm_ex, frame/3/bli_l3_tapi_ex.c:533-586 */
void bli_dtrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
               gb_dim_t m, gb_dim_t n, const double* alpha, const double* a,
               gb_inc_t rs_a, gb_inc_t cs_a, double* b, gb_inc_t rs_b, gb_inc_t cs_b);
/* replaces bli_strsm (frame/3/bli_l3_tapi_ex.c:533-586, float instance) */
void bli_strsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
               gb_dim_t m, gb_dim_t n, const float* alpha, const float* a,
               gb_inc_t rs_a, gb_inc_t cs_a, float* b, gb_inc_t rs_b, gb_inc_t cs_b);
void bli_dtrsm_ex(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
                  gb_dim_t m, gb_dim_t n, const double* alpha, const double* a,
                  gb_inc_t rs_a, gb_inc_t cs_a, double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                  const void* cntx, const void* rntm);

/* replaces bli_dgemv / bli_dgemv_ex, frame/2/bli_l2_tapi.c:43-127 */
void bli_dgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
               const double* x, gb_inc_t incx, const double* beta, double* y, gb_inc_t incy);
void bli_dgemv_ex(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n,
                  const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  const double* x, gb_inc_t incx, const double* beta, double* y,
                  gb_inc_t incy, const void* cntx, const void* rntm);

/* replaces bli_daxpyv / bli_daxpyv_ex, frame/1/bli_l1v_tapi.c:155-191 */
void bli_daxpyv(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x,
                gb_inc_t incx, double* y, gb_inc_t incy);
void bli_daxpyv_ex(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x,
                   gb_inc_t incx, double* y, gb_inc_t incy, const void* cntx,
                   const void* rntm);

/* replaces bli_ddotv / bli_ddotv_ex, frame/1/bli_l1v_tapi.c:195-232 */
void bli_ddotv(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x,
               gb_inc_t incx, const double* y, gb_inc_t incy, double* rho);
void bli_ddotv_ex(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x,
                  gb_inc_t incx, const double* y, gb_inc_t incy, double* rho,
                  const void* cntx, const void* rntm);

#endif /* GB300_ADDON_ONLY */

/* Host-pointer entry points under the addon prefix, with the typed-API
   argument lists above.  A BLIS build that keeps its own bli_?gemm symbols
   (for instance a sandbox bli_gemm_ex that forwards to this library) calls
   these instead, which cannot resolve back into libblis. */
void gb_dgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
              const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta,
              double* c, gb_inc_t rs_c, gb_inc_t cs_c);
void gb_sgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a,
              const float* b, gb_inc_t rs_b, gb_inc_t cs_b, const float* beta,
              float* c, gb_inc_t rs_c, gb_inc_t cs_c);
/* The Ozaki form for one call, whatever gb_set_dgemm_mode says (slices 0:
   the selector's proposal checked by the verifier); the sandbox maps a
   comp_prec request on the obj_t to it. */
void gb_dgemm_ozaki(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                    const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                    const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c,
                    gb_inc_t rs_c, gb_inc_t cs_c, int slices);
/* Complex host aliases for the sandbox (same as bli_zgemm / bli_cgemm). */
void gb_zgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
              const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta,
              gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);
void gb_cgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
              const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta,
              gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c);
void gb_dtrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
              gb_dim_t m, gb_dim_t n, const double* alpha, const double* a,
              gb_inc_t rs_a, gb_inc_t cs_a, double* b, gb_inc_t rs_b, gb_inc_t cs_b);
void gb_strsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
              gb_dim_t m, gb_dim_t n, const float* alpha, const float* a,
              gb_inc_t rs_a, gb_inc_t cs_a, float* b, gb_inc_t rs_b, gb_inc_t cs_b);
/* same as bli_ztrsm (frame/3/bli_l3_tapi_ex.c:533-586, complex instance) */
void gb_ztrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
              gb_dim_t m, gb_dim_t n, const gb_dcomplex* alpha, const gb_dcomplex* a,
              gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b);
void gb_ctrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
              gb_dim_t m, gb_dim_t n, const gb_scomplex* alpha, const gb_scomplex* a,
              gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b);
void gb_dgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n,
              const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
              const double* x, gb_inc_t incx, const double* beta, double* y, gb_inc_t incy);
void gb_daxpyv(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x,
               gb_inc_t incx, double* y, gb_inc_t incy);
void gb_ddotv(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x,
              gb_inc_t incx, const double* y, gb_inc_t incy, double* rho);

/* ===================================================================== */
/* 2. gb_ addon: device pointers, explicit stream (NULL = the calling      */
/*    thread's library stream).  Return GB_SUCCESS or a negative code.     */
/*    Device operands use the same (rs, cs) element-stride convention as   */
/*    the typed BLIS API.  Calls are asynchronous on the given stream.     */
/* ===================================================================== */

/* Native FP64 GEMM on the FP64 pipe: C := beta*C + alpha*op(A)*op(B).
   Counterpart of bli_gemm_ex, frame/3/bli_l3_oapi_ex.c:48-148. */
int gb_dgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const double* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta,
                 double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);

/* Ozaki split-product DGEMM: FP64 operands cut into `slices` bf16 digit
   slices, products on the tcgen05 tensor cores, exact integer level sums,
   FP64 recombination.  Always the digit form, whatever form
   gb_set_dgemm_mode chose for the host entry points (the CRT form is
   gb_dgemm_ozaki_crt_dev).  From m >= 8192, n >= 4096 and k >= 2048 (CRT
   form: m, n >= 16384) the product runs in 8 x 2..4 blocks of C on `stream` and two more of
   the calling thread's streams, forked from and joined to it (GB_OZAKI_DEV_BLOCKS fixes
   the grid): the same bits on finite operands; a block whose rows of op(A) or
   columns of op(B) hold an Inf or NaN is computed by the native kernel, the
   others stay in the Ozaki form.  No reference counterpart (precision form). */
int gb_dgemm_ozaki_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
                       gb_dim_t k, double alpha, const double* a, gb_inc_t rs_a,
                       gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                       double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, int slices,
                       void* stream);
/* The CRT form of the Ozaki product (no reference counterpart): `moduli` bf16
   residue products (2..16) instead of the digit form's s(s+1)/2; the operands
   are scaled to t-bit integers, t = the largest with k 2^(2t) <= 8 M / 17 for
   the product M of the moduli (t = 55 for 16 moduli at k = 16384), and the
   result is the single rounding of their exact integer product.  k must be at
   most 131072.  Large products run in blocks as for gb_dgemm_ozaki_dev. */
int gb_dgemm_ozaki_crt_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                           double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                           gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c,
                           gb_inc_t cs_c, int moduli, void* stream);

int gb_sgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 float alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const float* b, gb_inc_t rs_b, gb_inc_t cs_b, float beta,
                 float* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);

/* Counterpart of bli_trsm_ex, frame/3/bli_l3_oapi_ex.c:692-801. */
int gb_dtrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
                 gb_dim_t m, gb_dim_t n, double alpha, const double* a, gb_inc_t rs_a,
                 gb_inc_t cs_a, double* b, gb_inc_t rs_b, gb_inc_t cs_b, void* stream);
/* The float instance (native form: FP32 diagonal solves of 64-row blocks,
   updates through sgemm's engine choice, gb_set_sgemm_mode). */
int gb_strsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga,
                 gb_dim_t m, gb_dim_t n, float alpha, const float* a, gb_inc_t rs_a,
                 gb_inc_t cs_a, float* b, gb_inc_t rs_b, gb_inc_t cs_b, void* stream);

/* Device-pointer complex gemm (zgemm: native FP64 or the Ozaki form by
   gb_set_dgemm_mode with a fixed slice count; cgemm: FP32). */
int gb_zgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta,
                 gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_cgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, gb_scomplex beta,
                 gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);

int gb_ztrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                 gb_dim_t n, gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, void* stream);
/* The scomplex instance: FP32 diagonal solves, updates through cgemm's FP32 real product. */
int gb_ctrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                 gb_dim_t n, gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 gb_scomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, void* stream);

/* Device-pointer forms of zherk, zher2k, zhemm, zsymm, dtrmm3 and dsyr2k
   (asynchronous on the stream). */
/* complex gemv on device pointers: op(A)'s columns split over the grid,
   partial sums in a scratch, one combine with alpha and beta */
int gb_zgemv_dev(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, gb_dcomplex alpha,
                 const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* x, gb_inc_t incx,
                 gb_dcomplex beta, gb_dcomplex* y, gb_inc_t incy, void* stream);
int gb_cgemv_dev(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, gb_scomplex alpha,
                 const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* x, gb_inc_t incx,
                 gb_scomplex beta, gb_scomplex* y, gb_inc_t incy, void* stream);
/* complex trmm on device pointers: the triangle as a full matrix, one complex
   gemm into a scratch, scattered back into B */
int gb_ztrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream);
int gb_ctrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream);
/* complex syrk / syr2k on device pointers: the products on herk's block-real
   form (Ozaki for double complex when the library's level-3 mode selects it) */
int gb_zsyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, gb_dcomplex alpha,
                 const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex beta, gb_dcomplex* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_csyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, gb_scomplex alpha,
                 const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex beta, gb_scomplex* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_zsyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                  gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                  gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                  void* stream);
int gb_csyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                  gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
                  gb_inc_t rs_b, gb_inc_t cs_b, gb_scomplex beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                  void* stream);
int gb_zherk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, double alpha,
                 const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, double beta, gb_dcomplex* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_zher2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                  gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta, gb_dcomplex* c,
                  gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_zhemm_dev(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m,
                 gb_dim_t n, gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_zsymm_dev(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m,
                 gb_dim_t n, gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a,
                 const gb_dcomplex* b, gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_dtrmm3_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_trans_t transb,
                  gb_dim_t m, gb_dim_t n, double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  const double* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c,
                  gb_inc_t cs_c, void* stream);
int gb_dsyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                  double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                  gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c,
                  void* stream);

/* Device-pointer forms of scalv, copyv, amaxv (the 0-based index written to
   device memory), ger and trsv (asynchronous on the stream). */
int gb_dscalv_dev(gb_dim_t n, double alpha, double* x, gb_inc_t incx, void* stream);
int gb_dcopyv_dev(gb_dim_t n, const double* x, gb_inc_t incx, double* y, gb_inc_t incy,
                  void* stream);
int gb_damaxv_dev(gb_dim_t n, const double* x, gb_inc_t incx, gb_dim_t* index_dev, void* stream);
int gb_dger_dev(gb_dim_t m, gb_dim_t n, double alpha, const double* x, gb_inc_t incx,
                const double* y, gb_inc_t incy, double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                void* stream);
int gb_dtrsv_dev(gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, double alpha,
                 const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* x, gb_inc_t incx,
                 void* stream);

/* Device-pointer forms of trmm, symm, gemmt and syrk (asynchronous on the
   stream; native FP64 or the Ozaki form by gb_set_dgemm_mode, with a fixed
   slice count). */
int gb_dtrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                 gb_dim_t n, double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream);
int gb_dsymm_dev(gb_side_t side, gb_uplo_t uploa, gb_dim_t m, gb_dim_t n, double alpha,
                 const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);
int gb_dgemmt_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                  double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                  gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c,
                  void* stream);
int gb_dsyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, double alpha,
                 const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double beta, double* c, gb_inc_t rs_c,
                 gb_inc_t cs_c, void* stream);

/* Allocation-free dot product (no counterpart in the reference).  For callers
   that cannot call cudaMalloc/cudaFree -- those calls can synchronize the
   whole device, and some host applications own a fixed device-memory budget
   or run latency-bound loops where allocation is not allowed.  Same result as
   gb_ddotv_dev (same partition and reduction order), but the partial-sum
   scratch is a file-scope device array of GB_DOTV_NOALLOC_MAX_PARTS doubles
   (16 KiB), resident on every GPU that loads the library until exit, and the
   library's one-time initialisation (which allocates) is not used.  The first
   call on a device, with that device current, looks up the array's device
   address; make that first call before any stream capture.  Calls share the
   array: calls that overlap on the GPU (unordered streams) race.  A problem
   that would need more partial sums than the array holds is rejected with
   GB_ERR_ARG.  x, y, rho are device pointers; stream NULL is the legacy
   default stream. */
#define GB_DOTV_NOALLOC_MAX_PARTS 2048
int gb_ddotv_noalloc_dev(gb_dim_t n, const double* x, gb_inc_t incx, const double* y,
                         gb_inc_t incy, double* rho, void* stream);

/* Counterparts of the axpyv / dotv / gemv kernels (frame/1/bli_l1v_ker_params.h:61-83,
   frame/2/bli_l2_tapi.c:43-127).  gb_ddotv_dev writes rho to DEVICE memory. */
int gb_daxpyv_dev(gb_dim_t n, double alpha, const double* x, gb_inc_t incx, double* y,
                  gb_inc_t incy, void* stream);
int gb_ddotv_dev(gb_dim_t n, const double* x, gb_inc_t incx, const double* y,
                 gb_inc_t incy, double* rho, void* stream);
int gb_dgemv_dev(gb_trans_t transa, gb_dim_t m, gb_dim_t n, double alpha, const double* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, const double* x, gb_inc_t incx,
                 double beta, double* y, gb_inc_t incy, void* stream);

/* GEMM with an explicit kernel configuration (the autotuner's and the
   selector's vocabulary); dtype 0 = FP64, 1 = FP32, 2 = BF16 (A and B bf16,
   C and arithmetic FP32), alpha/beta passed as double.  Config 0: 128x128
   tiles (BF16: the tcgen05 kernel, 128x256 tiles); configs 1..5: the
   small/skinny (gemmsup) engine with 64x64 tiles and K split into 1, 2, 4,
   8, 16 parts (split partials folded in a fixed order).  Counterpart of the
   gemmsup decision of frame/3/bli_l3_sup.c:37-131 (thresholds
   frame/base/bli_cntx.h:186-193). */
#define GB_GEMM_NUM_CONFIGS 6
int gb_gemm_config_dev(int dtype, int config, gb_trans_t transa, gb_trans_t transb, gb_dim_t m,
                       gb_dim_t n, gb_dim_t k, double alpha, const void* a, gb_inc_t rs_a,
                       gb_inc_t cs_a, const void* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta,
                       void* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);

/* BF16 GEMM, C := alpha op(A) op(B) + beta C with A, B bf16 (bit patterns,
   BLIS-style strides) and C fp32.  BLIS 1.0 has no bf16 datatype; this entry
   completes the selector's dtype set.  The configuration comes from the
   selector when gb_set_gemm_autoselect(1) and a model are loaded, else from
   the small-problem threshold rule (tensor cores when every dimension is at
   least 201). */
int gb_bgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, float alpha,
                 const void* a, gb_inc_t rs_a, gb_inc_t cs_a, const void* b, gb_inc_t rs_b, gb_inc_t cs_b,
                 float beta, float* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream);

/* One problem of a grouped GEMM on device operands (column-major, BLAS
   leading dimensions): C := beta*C + alpha*op(A)*op(B). */
typedef struct {
    gb_trans_t transa, transb;
    gb_dim_t m, n, k;
    double alpha, beta;
    const void* a;
    gb_inc_t lda;
    const void* b;
    gb_inc_t ldb;
    void* c;
    gb_inc_t ldc;
} gb_gemm_problem_t;

#define GB_BATCH_GROUPED 0  /* one persistent launch, device tile scheduler */
#define GB_BATCH_LOOP 1     /* one launch per problem (comparison baseline) */

#define GB_BATCH_FP64 0        /* native FP64 (DMMA) */
#define GB_BATCH_FP32 1        /* FP32 */
#define GB_BATCH_FP64_OZAKI 2  /* FP64 through the Ozaki form, slice count of gb_set_dgemm_mode
                                  (8 when that is 0 = automatic) */

/* Counterpart of dgemm_batch_/sgemm_batch_ (frame/compat/extra/bla_gemm_batch.c:
   135-249) on device operands; dtype is one of GB_BATCH_FP64/FP32/FP64_OZAKI.
   GB_BATCH_FP64_OZAKI runs all problems in three grouped launches (split,
   slice GEMM, recombine); a problem with an Inf/NaN operand sends the batch
   to the native grouped launch, and problems whose k exceeds one exact
   integer part are run one by one through the Ozaki form.  Its results are
   bit-identical to gb_dgemm_ozaki_dev on each problem with the same slices.
   With GB_BATCH_LOOP each problem gets its own launches. */
int gb_gemm_batch_dev(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, int mode,
                      void* stream);

/* Resident plan for repeated grouped launches: the descriptor tables (and for
   GB_BATCH_FP64_OZAKI the slice and level-sum arenas) stay in HBM and
   gb_batch_plan_run(use_graph=1) replays the launches as one captured CUDA
   graph. */
int gb_batch_plan_create(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, void** plan);
int gb_batch_plan_run(void* plan, int use_graph, void* stream);
int gb_batch_plan_destroy(void* plan);

/* Configuration policy of a native (FP64 / FP32) plan: 0 = every problem on
   the 128x128 engine; 1 = the 64x64 engine for the problems the selector
   assigns to configs 1..5, without split-K; 2 = the selected configuration
   including split-K (those problems run in a second grouped launch and a
   grouped fold, in the same graph); 3 (FP32 only) = SGEMM's split form for
   the whole batch: the grouped Ozaki form at 3 slices on the bf16 tensor
   cores, its split reading op(A) and op(B) in FP32 (each element widened
   exactly), its recombination rounding alpha P + beta C to FP32 once.
   gb_batch_plan_create autotunes it: each candidate runs on the batch's
   shapes with scratch outputs and the fastest is kept.  Candidates: 0; 1 and
   2 when a selector model is loaded and auto-selection is on; 3 for FP32
   unless gb_set_sgemm_mode(GB_SGEMM_FMA).  One-shot gb_gemm_batch_dev /
   dgemm_batch_ calls use policy 0.  gb_batch_plan_create_ex fixes the policy
   (-1 = autotune). */
int gb_batch_plan_create_ex(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, int policy, void** plan);
int gb_batch_plan_policy(const void* plan);

/* Seeded matrix fill on the device, the counterpart of bli_randm (frame/util,
   value generators frame/include/bli_cast_macro_defs.h:465-525) with a
   counter-based generator: element (i, j) of the logical m x n matrix takes
   index i + j*m, so values do not depend on the storage strides.
   GB_RAND_UNIFORM: uniform [p0, p1); GB_RAND_EXPSPREAD: (1+u) 2^e, e uniform
   integer in [p0, p1], random sign; GB_RAND_NARROW_POW2: {0, +-2^0..+-2^-6}. */
#define GB_RAND_UNIFORM 0
#define GB_RAND_EXPSPREAD 1
#define GB_RAND_NARROW_POW2 2
int gb_randm_dev(int kind, int is_float, void* x, gb_dim_t m, gb_dim_t n, gb_inc_t rs,
                 gb_inc_t cs, uint64_t seed, double p0, double p1, void* stream);

/* Double-double value (hi + lo) of entries (ii[e], jj[e]) of
   alpha*op(A)*op(B) + beta*C, for reporting the max componentwise error of a
   GEMM result.  All pointers are device pointers.  No reference counterpart. */
int gb_dd_gemm_entries_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t k, double alpha,
                           const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                           gb_inc_t rs_b, gb_inc_t cs_b, double beta, const double* c,
                           gb_inc_t rs_c, gb_inc_t cs_c, gb_dim_t nent, const int64_t* ii,
                           const int64_t* jj, double* hi, double* lo, void* stream);

/* ===================================================================== */
/* 2b. Learned configuration selector (no reference counterpart: BLIS picks */
/*     kernels from static per-architecture tables,                        */
/*     config/<arch>/bli_cntx_init_<arch>.c)                                */
/* ===================================================================== */

/* MLP 16 -> 64 -> 64 -> 64 -> 8, GELU, FP32.  Parameters are one vector of
   GB_MLP_NPARAMS floats: W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64]
   W4[8][64] b4[8].  Inputs x[batch][16], outputs / targets / mask [batch][8];
   all pointers are device pointers. */
#define GB_MLP_IN 16
#define GB_MLP_HIDDEN 64
#define GB_MLP_OUT 8
#define GB_MLP_NPARAMS 9928
int gb_mlp_forward_dev(const float* params, const float* x, gb_dim_t batch, float* out, void* stream);
/* grad := d/dparams of sum_b sum_o mask*(out - y)^2 / norm, loss := that sum;
   deterministic (fixed-order fold of per-block partials). */
int gb_mlp_loss_grad_dev(const float* params, const float* x, const float* y, const float* mask,
                         gb_dim_t batch, float norm, float* grad, float* loss, void* stream);
/* One Adam step (step counts from 1) with decoupled weight decay added to the gradient. */
int gb_mlp_adam_dev(float* params, const float* grad, float* m, float* v, gb_dim_t n, float lr,
                    float beta1, float beta2, float eps, float weight_decay, int step, void* stream);

/* Error-bound verifier for the Ozaki slice count: the smallest s >= s_min
   such that, on a deterministic sample of `nsample` entries (i, j),
     2^-(8s+1) (2^e_i |B_j|_1 + |A_i|_1 2^e_j) + sqrt(k) s 2^(e_i+e_j-8s-2)
       <= sqrt(k) u (|A||B|)_ij,          u = 2^-53,
   i.e. the split's representation error plus the dropped slice products
   (random-sign growth) stays at the level of a typical FP64 dot-product
   error.  *s_out receives s (at most 12; a
   sample that needs more reports 13).  Device operands, host s_out. */
int gb_ozaki_verify_slices_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
                               gb_dim_t k, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                               const double* b, gb_inc_t rs_b, gb_inc_t cs_b, int s_min,
                               int nsample, int* s_out, void* stream);

/* The selector inside the library.  gb_selector_load takes GB_MLP_NPARAMS
   host floats; gb_selector_load_file reads the binary model written by
   blis_gb300/selector.py (magic "GBSELMLP", version 1, parameter count,
   CRC-32 of the parameters, parameters).  With gb_set_gemm_autoselect(1)
   and a model loaded, the host GEMM entry points (dgemm_, sgemm_,
   bli_?gemm, gb_?gemm) run the configuration of least predicted time; the
   Ozaki mode with slices = 0 takes the model's slice proposal, raised by
   gb_ozaki_verify_slices_dev where it fails.  Without a model the BLIS sup
   threshold rule is used.  gb_selector_choose exposes the decision. */
int gb_selector_load(const float* params, int nparams);
int gb_selector_load_file(const char* path);
int gb_selector_unload(void);
int gb_set_gemm_autoselect(int on);
int gb_selector_choose(int dtype, gb_dim_t m, gb_dim_t n, gb_dim_t k, int transa, int transb, int pad,
                       double spread_a, double spread_b, int* config, int* slices);

/* ===================================================================== */
/* 3. Controls and introspection                                           */
/* ===================================================================== */

/* Selects the device used by this library (default: the current device). */
int gb_init(int device);

/* Routes dgemm_ / cblas_dgemm / bli_dgemm through the native FP64 kernel
   (GB_DGEMM_NATIVE) or the Ozaki split form with the given slice count
   (2..12), or with slices = 0 the count chosen per call by the selector and
   the error-bound verifier (the native kernel when no count reaches it). */
#define GB_DGEMM_NATIVE 0
#define GB_DGEMM_OZAKI 1
/* The CRT form of the Ozaki products (no reference counterpart): `slices` is
   the number of moduli N (2..16, or 0 for the count whose precision matches
   the digit count the selector and verifier choose); N bf16 residue products
   replace the digit form's s(s+1)/2 (N = 16 at k = 16384 carries the 55-bit
   operands of s = 7 digits).  The grouped batch keeps the digit form at the
   slice count of equal precision. */
#define GB_DGEMM_OZAKI_CRT 2
int gb_set_dgemm_mode(int mode, int slices);

/* SGEMM engine (no reference counterpart): GB_SGEMM_FMA the FP32 FMA kernel;
   GB_SGEMM_SPLIT the split form on the bf16 tensor cores (op(A), op(B)
   split from FP32, each element widened exactly, and multiplied as the Ozaki
   digit form with 3 slices, six bf16 products with exact integer
   accumulation, then C = RN32(alpha P + beta C) from the FP64 product P); GB_SGEMM_AUTO (default) the split form
   when m, n >= 1024 and k >= 512, the FMA kernel otherwise.  Host and device
   sgemm entry points follow it; from m, n >= 8192 the split form runs in 4 x 2
   blocks of C on three streams, as gb_dgemm_ozaki_dev's blocked form. */
#define GB_SGEMM_FMA 0
#define GB_SGEMM_SPLIT 1
#define GB_SGEMM_AUTO 2
int gb_set_sgemm_mode(int mode);

/* Engine of the Ozaki slice products: 1 = one CTA per 128x256 tile,
   2 = pairs of CTAs on two SMs per 256x256 tile (cta_group::2, a cluster of
   two), 0 = chosen per product (default): the learned selector's engine
   output for shapes a host entry point has asked it about, else CTA pairs
   for products of at least 2^30 flops and single CTAs below.  The
   GB_OZAKI_CTAS environment variable (1 or 2) forces one engine. */
int gb_set_ozaki_ctas(int ctas);

/* Last error of the calling thread (GB_SUCCESS if none), with its message. */
int gb_get_last_error(char* msg, size_t len);
void gb_clear_last_error(void);

/* Number of kernels this library has launched since load. */
int64_t gb_launch_count(void);

/* Slice count of the calling thread's most recent Ozaki split product (so a
   caller that let the library choose, slices = 0, can learn the count); 0 if
   the last double-precision gemm in the Ozaki form ran on the native FP64
   kernel instead (no slice count reached the error bound), -1 before any.
   No reference counterpart. */
int gb_last_ozaki_slices(void);

/* Per-kernel device time (CUDA events on the launching stream), enabled by
   gb_set_kernel_timing(1).  gb_kernel_time_ms() synchronises the recorded
   events and returns the summed time and launch count of kernels whose name
   starts with `prefix`, then forgets them. */
int gb_set_kernel_timing(int enable);
double gb_kernel_time_ms(const char* prefix, int64_t* launches);

/* The recorded launches as a timeline, in the order they were issued: name,
   start and end in milliseconds from the first record's start (CUDA events on
   each launch's stream, so launches on different streams show their overlap;
   the host pipeline of dgemm_ also records its copies, as "copy_*").  Writes
   at most max_entries, returns how many it wrote, and forgets every record.
   No reference counterpart (the profiling aid of a box without nsys). */
typedef struct {
    char name[40];
    double start_ms, end_ms;
} gb_trace_entry_t;
int64_t gb_kernel_trace(gb_trace_entry_t* out, int64_t max_entries);

/* Blocks until the calling thread's library stream is idle. */
int gb_synchronize(void);

/* Failure-detection test hook (no reference counterpart).  The one-launch
   dtrsv (trsv_flags_kernel) hands each 64-row block of x from CTA to CTA
   through flags with bounded waits.  With withhold_block >= 0 the CTA that
   solves that block does not publish its flag, so the CTAs after it wait
   until the budget runs out (wait_budget_ns, 0 = the default 2 s, else
   0.1 ms .. 10 s), report DEV_WAIT_TIMEOUT in the device status word, stop
   every other CTA through the grid's abort word and return; the call then
   fails with GB_ERR_DEVICE and the context stays usable.  Nothing faults,
   traps or waits without a bound.  (-1, 0) restores normal operation.
   Process-wide; for tests only. */
int gb_test_trsv_wait_fault(int64_t withhold_block, int64_t wait_budget_ns);

#ifdef __cplusplus
}
#endif
#endif /* BLIS_GB300_H */
