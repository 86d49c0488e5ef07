/*
 * bli_sandbox.h -- header every BLIS gemm sandbox provides (blis.h includes it
 * when BLIS is built with the sandbox enabled, frame/include/bli_sbox.h:42-44).
 *
 * The gb300 sandbox replaces bli_gemm_ex() with a version that runs the
 * product on the GB300 through libblis_gb300.so.  The one extra symbol it
 * exports, bls_gb300_gemm_calls(), reports how many gemm calls took the GPU
 * path and how many were forwarded to BLIS's own CPU implementation
 * (mixed-datatype operands), so an application or a test can see which path
 * ran.
 */
#ifndef BLIS_SANDBOX_H
#define BLIS_SANDBOX_H

BLIS_EXPORT_BLIS void bls_gb300_gemm_calls(long* gpu_calls, long* cpu_forwarded);

#endif
