/*
 * obj_gemm_comp_prec.c -- one BLIS object-API gemm on double operands with a
 * single-precision computation request, the case the gb300 sandbox's
 * bli_gemm_ex sends to the Ozaki split form (docs/MixedDatatypes.md:62-80:
 * the computation precision is a property of C, bli_obj_set_comp_prec).
 *
 * usage: obj_gemm_comp_prec.x IN OUT
 *   IN : int64 m, n, k; double alpha, beta; A (m x k), B (k x n), C (m x n),
 *        all column-major
 *   OUT: int32 slice count the library used (gb_last_ozaki_slices), then C
 * Exit status 0 on success.
 */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>

#include "blis.h"

#define GB300_ADDON_ONLY
#include "blis_gb300.h"

static int read_all(FILE* f, void* p, size_t bytes)
{
	return fread(p, 1, bytes, f) == bytes;
}

int main(int argc, char** argv)
{
	if (argc != 3) { fprintf(stderr, "usage: %s IN OUT\n", argv[0]); return 2; }
	FILE* f = fopen(argv[1], "rb");
	if (!f) { perror(argv[1]); return 2; }
	int64_t dims[3];
	double ab[2];
	if (!read_all(f, dims, sizeof dims) || !read_all(f, ab, sizeof ab)) return 2;
	const int64_t m = dims[0], n = dims[1], k = dims[2];
	double* a = malloc(sizeof(double) * m * k);
	double* b = malloc(sizeof(double) * k * n);
	double* c = malloc(sizeof(double) * m * n);
	if (!a || !b || !c) return 2;
	if (!read_all(f, a, sizeof(double) * m * k) || !read_all(f, b, sizeof(double) * k * n) ||
	    !read_all(f, c, sizeof(double) * m * n)) return 2;
	fclose(f);

	bli_init();
	obj_t ao, bo, co, alpha, beta;
	bli_obj_create_with_attached_buffer(BLIS_DOUBLE, m, k, a, 1, m, &ao);
	bli_obj_create_with_attached_buffer(BLIS_DOUBLE, k, n, b, 1, k, &bo);
	bli_obj_create_with_attached_buffer(BLIS_DOUBLE, m, n, c, 1, m, &co);
	bli_obj_create_1x1_with_attached_buffer(BLIS_DOUBLE, &ab[0], &alpha);
	bli_obj_create_1x1_with_attached_buffer(BLIS_DOUBLE, &ab[1], &beta);

	bli_obj_set_comp_prec(BLIS_SINGLE_PREC, &co);
	bli_gemm(&alpha, &ao, &bo, &beta, &co);

	const int32_t slices = gb_last_ozaki_slices();
	FILE* g = fopen(argv[2], "wb");
	if (!g) { perror(argv[2]); return 2; }
	fwrite(&slices, sizeof slices, 1, g);
	fwrite(c, sizeof(double), m * n, g);
	fclose(g);
	free(a); free(b); free(c);
	return 0;
}
