/*
 * gb300_blis.c -- glue library that puts BLIS's trsm, gemv, axpyv and dotv on
 * the GB300.  Built against BLIS's own headers into libgb300_blis.so; an
 * application links it ahead of libblis (-lgb300_blis -lblis), and with a
 * libblis built with the gb300 gemm sandbox (integration/sandbox/gb300) every
 * operation of BLIS's dense hot path runs through BLIS's own host code into
 * libblis_gb300.so:
 *
 *   gemm   sandbox bli_gemm_ex (no symbol here)
 *   trsm   bli_trsm_ex, interposed: BLIS has no seam for it
 *          (frame/3/bli_l3_oapi_ex.c:692 is unconditional), and bli_trsm,
 *          the typed bli_?trsm[_ex] (frame/3/bli_l3_tapi_ex.c:533-586) and
 *          dtrsm_ (frame/compat/bla_trsm.c:202) all reach it
 *   gemv   bli_dgemv_ex, interposed: the typed entry that dgemv_ and the
 *          object API bli_gemv_ex both reach (frame/2/bli_l2_tapi.c:43-127);
 *          the context's axpyf/dotxf slots are not used because the unfused
 *          variants call them once per 8 columns (bli_gemv_unf_var2.c:104-125)
 *   axpyv  the context's BLIS_AXPYV_KER slot for BLIS_DOUBLE, and
 *   dotv   BLIS_DOTV_KER, overwritten at load time through bli_cntx_set_ukrs
 *          (the pattern of config/haswell/bli_cntx_init_haswell.c:47-135;
 *          docs/PluginHowTo.md): the typed level-1v API calls the context
 *          kernel once per vector (frame/1/bli_l1v_tapi.c:155-232)
 *
 * Datatypes the GPU library does not cover (gemv other than double) keep
 * BLIS's own code: trsm (all four datatypes on the GPU) is
 * forwarded to the next bli_trsm_ex in the link order (libblis's), gemv is
 * simply not interposed for them.  Forwarded calls are counted, and with
 * GB300_BLIS_REPORT set the library prints the counts of GPU and forwarded
 * calls and the number of GPU kernels launched when the process exits.
 *
 * Argument errors keep BLIS's behaviour: when error checking is on and an
 * operand is not conformal, the call is handed to BLIS's own bli_trsm_ex,
 * whose bli_trsm_check reports it (and aborts, as BLIS does).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#include "blis.h"

#define GB300_ADDON_ONLY
#include "blis_gb300.h"

static long n_trsm_gpu, n_trsm_cpu, n_gemv_gpu, n_axpyv_gpu, n_dotv_gpu;

#define COUNT( v ) __atomic_add_fetch( &( v ), 1, __ATOMIC_RELAXED )

// ------------------------------------------------------------------ level-1v kernels
// axpyv_ker_ft / dotv_ker_ft (frame/1/bli_l1v_ker_params.h:61-83, frame/1/bli_l1v_ker_ft.h):
// the kernel owns the n == 0 and alpha == 0 cases, as the reference kernels do
// (ref_kernels/1/bli_axpyv_ref.c, bli_dotv_ref.c); conjugation is a no-op for real data.

static void gb300_daxpyv_ker( axpyv_params, BLIS_CNTX_PARAM )
{
	( void )conjx; ( void )cntx;
	COUNT( n_axpyv_gpu );
	gb_daxpyv( BLIS_NO_CONJUGATE, n, ( const double* )alpha, ( const double* )x, incx,
	           ( double* )y, incy );
}

static void gb300_ddotv_ker( dotv_params, BLIS_CNTX_PARAM )
{
	( void )conjx; ( void )conjy; ( void )cntx;
	COUNT( n_dotv_gpu );
	gb_ddotv( BLIS_NO_CONJUGATE, BLIS_NO_CONJUGATE, n, ( const double* )x, incx,
	          ( const double* )y, incy, ( double* )rho );
}

// Overwrites the double-precision axpyv and dotv slots of BLIS's global context.
void gb300_blis_register( void )
{
	bli_init();
	cntx_t* cntx = ( cntx_t* )bli_gks_query_cntx();
	bli_cntx_set_ukrs
	(
	  cntx,
	  BLIS_AXPYV_KER, BLIS_DOUBLE, ( void_fp )gb300_daxpyv_ker,
	  BLIS_DOTV_KER,  BLIS_DOUBLE, ( void_fp )gb300_ddotv_ker,
	  BLIS_VA_END
	);
}

// ------------------------------------------------------------------ trsm
typedef void ( *trsm_ex_ft )( side_t, const obj_t*, const obj_t*, const obj_t*, const cntx_t*, const rntm_t* );

static void blis_trsm_ex( side_t side, const obj_t* alpha, const obj_t* a, const obj_t* b,
                          const cntx_t* cntx, const rntm_t* rntm )
{
	static trsm_ex_ft next = NULL;
	if ( next == NULL ) next = ( trsm_ex_ft )dlsym( RTLD_NEXT, "bli_trsm_ex" );
	if ( next == NULL )
	{
		fprintf( stderr, "gb300_blis: BLIS's bli_trsm_ex not found after this library\n" );
		abort();
	}
	COUNT( n_trsm_cpu );
	next( side, alpha, a, b, cntx, rntm );
}

void bli_trsm_ex( side_t side, const obj_t* alpha, const obj_t* a, const obj_t* b,
                  const cntx_t* cntx, const rntm_t* rntm )
{
	bli_init();

	const num_t dt = bli_obj_dt( b );
	const dim_t m = bli_obj_length( b ), n = bli_obj_width( b );
	const dim_t na = bli_is_left( side ) ? m : n;

	// On the GPU: A and B of one datatype the library covers, A square and conformal,
	// A's diagonal through its first element, B without a transposition bit.  Anything
	// else (including the operands that bli_trsm_check rejects) goes to BLIS.
	const bool gpu_dt = ( dt == BLIS_DOUBLE || dt == BLIS_FLOAT || dt == BLIS_DCOMPLEX || dt == BLIS_SCOMPLEX ) &&
	                    bli_obj_dt( a ) == dt;
	if ( !gpu_dt ||
	     bli_obj_length( a ) != bli_obj_width( a ) || bli_obj_length( a ) != na ||
	     bli_obj_diag_offset( a ) != 0 || bli_obj_has_trans( b ) || bli_obj_has_conj( b ) ||
	     !( bli_obj_is_lower( a ) || bli_obj_is_upper( a ) ) )
	{
		blis_trsm_ex( side, alpha, a, b, cntx, rntm );
		return;
	}

	// zero dimensions, alpha == 0 (B := 0): frame/3/bli_l3_oapi_ex.c:710-711
	if ( bli_l3_return_early_if_trivial( alpha, a, b, &BLIS_ZERO, b ) == BLIS_SUCCESS )
		return;

	obj_t alpha_cast;
	bli_obj_scalar_init_detached_copy_of( dt, BLIS_NO_CONJUGATE, alpha, &alpha_cast );

	const side_t  sd = side;
	const uplo_t  uplo = bli_obj_uplo( a );
	const trans_t ta = bli_obj_conjtrans_status( a );
	const diag_t  diag = bli_obj_diag( a );
	const void*   pa = bli_obj_buffer_at_off( a );
	void*         pb = bli_obj_buffer_at_off( b );
	const inc_t   rsa = bli_obj_row_stride( a ), csa = bli_obj_col_stride( a );
	const inc_t   rsb = bli_obj_row_stride( b ), csb = bli_obj_col_stride( b );

	COUNT( n_trsm_gpu );
	if ( dt == BLIS_DOUBLE )
		gb_dtrsm( sd == BLIS_LEFT ? GB_LEFT : GB_RIGHT, uplo, ta, diag, m, n,
		          ( const double* )bli_obj_buffer( &alpha_cast ), ( const double* )pa, rsa, csa,
		          ( double* )pb, rsb, csb );
	else if ( dt == BLIS_FLOAT )
		gb_strsm( sd == BLIS_LEFT ? GB_LEFT : GB_RIGHT, uplo, ta, diag, m, n,
		          ( const float* )bli_obj_buffer( &alpha_cast ), ( const float* )pa, rsa, csa,
		          ( float* )pb, rsb, csb );
	else if ( dt == BLIS_DCOMPLEX )
		gb_ztrsm( sd == BLIS_LEFT ? GB_LEFT : GB_RIGHT, uplo, ta, diag, m, n,
		          ( const gb_dcomplex* )bli_obj_buffer( &alpha_cast ), ( const gb_dcomplex* )pa, rsa, csa,
		          ( gb_dcomplex* )pb, rsb, csb );
	else
		gb_ctrsm( sd == BLIS_LEFT ? GB_LEFT : GB_RIGHT, uplo, ta, diag, m, n,
		          ( const gb_scomplex* )bli_obj_buffer( &alpha_cast ), ( const gb_scomplex* )pa, rsa, csa,
		          ( gb_scomplex* )pb, rsb, csb );
}

// ------------------------------------------------------------------ gemv
void bli_dgemv_ex( trans_t transa, conj_t conjx, dim_t m, dim_t n, const double* alpha,
                   const double* a, inc_t rs_a, inc_t cs_a, const double* x, inc_t incx,
                   const double* beta, double* y, inc_t incy, const cntx_t* cntx, const rntm_t* rntm )
{
	( void )cntx; ( void )rntm;
	COUNT( n_gemv_gpu );
	gb_dgemv( transa, conjx, m, n, alpha, a, rs_a, cs_a, x, incx, beta, y, incy );
}

// ------------------------------------------------------------------ report
typedef void ( *gemm_calls_ft )( long*, long* );

// Counts of calls per path, for applications and tests that want to see which path ran.
void gb300_blis_counts( long* counts /* [8] */ )
{
	long gemm_gpu = -1, gemm_cpu = -1;
	gemm_calls_ft f = ( gemm_calls_ft )dlsym( RTLD_DEFAULT, "bls_gb300_gemm_calls" );
	if ( f ) f( &gemm_gpu, &gemm_cpu );
	counts[ 0 ] = gemm_gpu;
	counts[ 1 ] = gemm_cpu;
	counts[ 2 ] = __atomic_load_n( &n_trsm_gpu, __ATOMIC_RELAXED );
	counts[ 3 ] = __atomic_load_n( &n_trsm_cpu, __ATOMIC_RELAXED );
	counts[ 4 ] = __atomic_load_n( &n_gemv_gpu, __ATOMIC_RELAXED );
	counts[ 5 ] = __atomic_load_n( &n_axpyv_gpu, __ATOMIC_RELAXED );
	counts[ 6 ] = __atomic_load_n( &n_dotv_gpu, __ATOMIC_RELAXED );
	counts[ 7 ] = ( long )gb_launch_count();
}

static void gb300_blis_report( void )
{
	long c[ 8 ];
	gb300_blis_counts( c );
	fprintf( stderr,
	         "gb300_blis: gemm_gpu=%ld gemm_cpu_forwarded=%ld trsm_gpu=%ld trsm_cpu_forwarded=%ld "
	         "gemv_gpu=%ld axpyv_gpu=%ld dotv_gpu=%ld kernel_launches=%ld\n",
	         c[ 0 ], c[ 1 ], c[ 2 ], c[ 3 ], c[ 4 ], c[ 5 ], c[ 6 ], c[ 7 ] );
}

__attribute__(( constructor )) static void gb300_blis_load( void )
{
	gb300_blis_register();
	if ( getenv( "GB300_BLIS_REPORT" ) ) atexit( gb300_blis_report );
}
