/*
 * bli_gemm_ex.c -- the gb300 gemm sandbox: BLIS's object-API gemm on the GB300.
 *
 * Built into libblis with the sandbox enabled (BLIS_ENABLE_SANDBOX), this
 * definition replaces the framework's bli_gemm_ex, which BLIS then compiles
 * as bli_gemm_def_ex (frame/3/bli_l3_oapi_ex.c:43-58).  Every gemm entry of
 * BLIS arrives here with obj_t operands: bli_gemm (frame/3/bli_l3_oapi.c),
 * the typed bli_?gemm[_ex] (frame/3/bli_l3_tapi_ex.c:83-93), dgemm_
 * (frame/compat/bla_gemm.c), cblas_dgemm and dgemm_batch_
 * (frame/compat/extra/bla_gemm_batch.c:227).
 *
 * Semantics kept from the framework version (frame/3/bli_l3_oapi_ex.c:48-148):
 * bli_init_once, bli_gemm_check when error checking is on, and
 * bli_l3_return_early_if_trivial (zero dimensions, alpha == 0 scales C by
 * beta).  Then the operands are unpacked -- dimensions after transposition,
 * the conj/trans bits, the element at each object's offset, row and column
 * strides (any sign, general stride included), alpha and beta cast to C's
 * datatype, and the internal scalars attached to A and B folded into alpha,
 * as bli_gemm_cntl_init does -- and handed to libblis_gb300.so's host entry
 * points (gb_dgemm, gb_sgemm, gb_zgemm, gb_cgemm), which move the operands
 * through HBM and return with C updated in place.
 *
 * Computation precision (docs/MixedDatatypes.md:62-80): double-precision
 * operands whose C carries a single-precision computation request
 * (bli_obj_set_comp_prec(BLIS_SINGLE_PREC, &c)) run in the Ozaki split form
 * (gb_dgemm_ozaki: bf16 slices on the tensor cores, slice count from the
 * library's selector checked by its error-bound verifier, FP64-level error),
 * whatever the library-wide mode says.
 *
 * Operands of mixed datatypes (mixed domain or storage precision) are not on
 * the GPU path: they are forwarded to BLIS's own implementation
 * (bli_gemm_def_ex) and counted as such (bls_gb300_gemm_calls), never passed
 * off as GPU work.
 *
 * Sandbox rules (docs/Sandboxes.md:115-121): the only bli_ symbol defined
 * here is bli_gemm_ex; the rest uses the bls_ prefix.
 */
#include "blis.h"

#define GB300_ADDON_ONLY
#include "blis_gb300.h"

static long bls_gb300_gpu_calls = 0;
static long bls_gb300_cpu_forwarded = 0;

void bls_gb300_gemm_calls(long* gpu_calls, long* cpu_forwarded)
{
	if ( gpu_calls )     *gpu_calls     = __atomic_load_n( &bls_gb300_gpu_calls, __ATOMIC_RELAXED );
	if ( cpu_forwarded ) *cpu_forwarded = __atomic_load_n( &bls_gb300_cpu_forwarded, __ATOMIC_RELAXED );
}

// Alpha in C's datatype, times the internal scalars attached to A and B.
static void bls_gb300_effective_alpha( num_t dt, const obj_t* alpha, const obj_t* a, const obj_t* b, obj_t* alpha_eff )
{
	obj_t scalar_a, scalar_b;
	bli_obj_scalar_init_detached_copy_of( dt, BLIS_NO_CONJUGATE, alpha, alpha_eff );
	bli_obj_scalar_detach( a, &scalar_a );
	bli_obj_scalar_detach( b, &scalar_b );
	bli_mulsc( &scalar_a, alpha_eff );
	bli_mulsc( &scalar_b, alpha_eff );
}

void bli_gemm_ex
     (
       const obj_t*  alpha,
       const obj_t*  a,
       const obj_t*  b,
       const obj_t*  beta,
       const obj_t*  c,
       const cntx_t* cntx,
       const rntm_t* rntm
     )
{
	bli_init_once();

	if ( bli_error_checking_is_enabled() )
		bli_gemm_check( alpha, a, b, beta, c, cntx );

	if ( bli_l3_return_early_if_trivial( alpha, a, b, beta, c ) == BLIS_SUCCESS )
		return;

	const num_t dt = bli_obj_dt( c );

	if ( bli_obj_dt( a ) != dt || bli_obj_dt( b ) != dt ||
	     !( dt == BLIS_FLOAT || dt == BLIS_DOUBLE || dt == BLIS_SCOMPLEX || dt == BLIS_DCOMPLEX ) )
	{
		__atomic_add_fetch( &bls_gb300_cpu_forwarded, 1, __ATOMIC_RELAXED );
		bli_gemm_def_ex( alpha, a, b, beta, c, cntx, rntm );
		return;
	}

	const trans_t transa = bli_obj_conjtrans_status( a );
	const trans_t transb = bli_obj_conjtrans_status( b );
	const dim_t   m      = bli_obj_length( c );
	const dim_t   n      = bli_obj_width( c );
	const dim_t   k      = bli_obj_width_after_trans( a );

	obj_t alpha_eff, beta_cast;
	bls_gb300_effective_alpha( dt, alpha, a, b, &alpha_eff );
	bli_obj_scalar_init_detached_copy_of( dt, BLIS_NO_CONJUGATE, beta, &beta_cast );
	const void* al = bli_obj_buffer( &alpha_eff );
	const void* be = bli_obj_buffer( &beta_cast );

	const void* pa = bli_obj_buffer_at_off( a );
	const void* pb = bli_obj_buffer_at_off( b );
	void*       pc = bli_obj_buffer_at_off( c );
	const inc_t rsa = bli_obj_row_stride( a ), csa = bli_obj_col_stride( a );
	const inc_t rsb = bli_obj_row_stride( b ), csb = bli_obj_col_stride( b );
	const inc_t rsc = bli_obj_row_stride( c ), csc = bli_obj_col_stride( c );

	__atomic_add_fetch( &bls_gb300_gpu_calls, 1, __ATOMIC_RELAXED );

	switch ( dt )
	{
	case BLIS_DOUBLE:
		if ( bli_obj_comp_prec( c ) == BLIS_SINGLE_PREC )
			gb_dgemm_ozaki( transa, transb, m, n, k, al, pa, rsa, csa, pb, rsb, csb,
			                be, pc, rsc, csc, 0 );
		else
			gb_dgemm( transa, transb, m, n, k, al, pa, rsa, csa, pb, rsb, csb,
			          be, pc, rsc, csc );
		break;
	case BLIS_FLOAT:
		gb_sgemm( transa, transb, m, n, k, al, pa, rsa, csa, pb, rsb, csb,
		          be, pc, rsc, csc );
		break;
	case BLIS_DCOMPLEX:
		gb_zgemm( transa, transb, m, n, k, al, pa, rsa, csa, pb, rsb, csb,
		          be, pc, rsc, csc );
		break;
	default: /* BLIS_SCOMPLEX */
		gb_cgemm( transa, transb, m, n, k, al, pa, rsa, csa, pb, rsb, csb,
		          be, pc, rsc, csc );
		break;
	}
}
