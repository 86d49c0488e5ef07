// gb_internal.h -- private declarations shared by the CUDA translation units
// of libblis_gb300.so.  Nothing here is part of the exported C ABI (that is
// include/blis_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <unordered_map>
#include <utility>

#include "../../include/blis_gb300.h"

// BLIS bit encodings (frame/include/bli_type_defs.h:395-427).
#define GB_TRANS_BIT 0x08
#define GB_CONJ_BIT 0x10
#define GB_IS_TRANS(t) (((t) & GB_TRANS_BIT) != 0)

namespace gb {

// ---------------------------------------------------------------- status
// Records a failure in the calling thread's status word and prints it once.
int set_error(int code, const char* where, const char* what);
int check_cuda(cudaError_t e, const char* where);
#define GB_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) return ::gb::check_cuda(_e, #call);             \
    } while (0)

// ---------------------------------------------------------------- context
// One CUDA stream per calling host thread (created lazily on the library's
// device); device memory comes from a stream-ordered pool that keeps freed
// blocks cached.
cudaStream_t thread_stream();
cudaStream_t thread_copy_stream(int i);  // i = 0, 1: copy streams of the calling thread
cudaStream_t thread_aux_stream(int i = 0);  // i = 0, 1, 2: more compute streams of the calling thread
int ensure_init();
int sm_count();

// Stream-ordered device allocations (cudaMallocAsync on the pool).
void* dev_alloc(size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);

// Device-side status word shared by all kernels of the library: a kernel
// that gives up on a bounded wait, or finds an impossible index, ORs a flag
// into it and returns instead of trapping.
unsigned int* device_status_word();
int read_and_clear_device_status(cudaStream_t s, const char* where);

enum : unsigned int {
    DEV_WAIT_TIMEOUT = 1u,
    DEV_BAD_INDEX = 2u,
    DEV_INT_OVERFLOW = 4u,
    DEV_NONFINITE = 8u,
};

// Wrap every kernel launch: counts it and, when per-kernel timing is on,
// brackets it with CUDA events recorded on the launching stream.  A copy
// wrapped for the timeline passes is_kernel = false (recorded, not counted).
class LaunchScope {
  public:
    LaunchScope(const char* name, cudaStream_t s, bool is_kernel = true);
    ~LaunchScope();

  private:
    const char* name_;
    cudaStream_t s_;
    bool timed_;
    cudaEvent_t start_, stop_;
};

// Bounded-wait budget for spin loops in device code (nanoseconds of
// %globaltimer); a wait that exceeds it reports DEV_WAIT_TIMEOUT.
constexpr unsigned long long kWaitBudgetNs = 2000000000ull;
// Failure-detection test hook (gb_test_trsv_wait_fault): the budget of the
// one-launch trsv's flag waits, and a block whose flag it withholds (-1 none).
unsigned long long trsv_wait_budget_ns();
int64_t trsv_withheld_block();

// ---------------------------------------------------------------- kernels
// All take device pointers and BLIS-style element strides (rs, cs).  op(A)
// element (i, l) lives at a[i*ars + l*acs] after the caller folded the
// transpose into the strides.
int dgemm_native(int64_t m, int64_t n, int64_t k, double alpha,
                 const double* a, int64_t ars, int64_t acs,
                 const double* b, int64_t brs, int64_t bcs, double beta,
                 double* c, int64_t rs_c, int64_t cs_c, cudaStream_t s);
int sgemm_native_gated(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                       const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                       const int* gate, cudaStream_t s);
int dgemm_native_gated(int64_t m, int64_t n, int64_t k, double alpha,
                       const double* a, int64_t ars, int64_t acs,
                       const double* b, int64_t brs, int64_t bcs, double beta,
                       double* c, int64_t rs_c, int64_t cs_c, const int* gate, cudaStream_t s);
double ozaki_t_bound_log2(int s, int64_t k);
bool selector_auto();
// Ozaki engine for an m x n x k product from the selector's engine output
// (2 CTA pairs, 1 single CTAs), or *engine = 0 when the model has none.
int selector_ozaki_engine(int64_t m, int64_t n, int64_t k, int* engine);
int selector_cached_engine(int64_t m, int64_t n, int64_t k);
int selector_cached_config(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad);
int selector_choose_ex(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad, double sa, double sb,
                       int* config, int* slices, int* engine);
int selector_heuristic(int64_t m, int64_t n, int64_t k);
int selector_choose(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad, double sa, double sb,
                    int* config, int* slices);
double host_exponent_spread(const double* x, int64_t rows, int64_t cols, int64_t rs, int64_t cs);
int gemm_config_dev(int dtype, int config, int64_t m, int64_t n, int64_t k, double alpha,
                    const void* a, int64_t ars, int64_t acs, const void* b, int64_t brs, int64_t bcs,
                    double beta, void* c, int64_t rs_c, int64_t cs_c, cudaStream_t s);
int sgemm_dev(int64_t m, int64_t n, int64_t k, float alpha,
              const float* a, int64_t ars, int64_t acs,
              const float* b, int64_t brs, int64_t bcs, float beta,
              float* c, int64_t rs_c, int64_t cs_c, cudaStream_t s);
int dgemm_ozaki(int64_t m, int64_t n, int64_t k, double alpha,
                const double* a, int64_t ars, int64_t acs,
                const double* b, int64_t brs, int64_t bcs, double beta,
                double* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s);
int dtrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha,
              const double* a, int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b,
              int64_t cs_b, int slices, cudaStream_t s);
int strsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, float alpha, const float* a,
              int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, cudaStream_t s);  // gb_trsm.cu
int64_t ozaki_kpart_limit(int slices);
// Lanes per right-hand side (1, 2, 4, 8) for the 64-row diagonal-block
// kernels of trsm and trmm, from the FP64-instruction cost model (gb_trsm.cu).
int diag_block_lanes(int64_t ncols);
// Complex gemm (T = double: dcomplex, float: scomplex; interleaved storage,
// alpha/beta as {real, imag}); one real gemm on the block-real form
// (gb_complex.cu).
template <typename T>
int cgemm_dev(int transa, int transb, int64_t m, int64_t n, int64_t k, const T* alpha, const T* a, int64_t rs_a,
              int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c, int64_t cs_c,
              int slices, cudaStream_t s);
int ztrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const double* alpha, const double* a,
              int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s);
int ctrsm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const float* alpha, const float* a,
              int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, cudaStream_t s);  // gb_complex.cu
int dscalv_dev(int64_t n, double alpha, double* x, int64_t incx, cudaStream_t s);
int dcopyv_dev(int64_t n, const double* x, int64_t incx, double* y, int64_t incy, cudaStream_t s);
int damaxv_dev(int64_t n, const double* x, int64_t incx, int64_t* index_dev, cudaStream_t s);
int dger_dev(int64_t m, int64_t n, double alpha, const double* x, int64_t incx, const double* y, int64_t incy,
             double* a, int64_t rs_a, int64_t cs_a, cudaStream_t s);
int dtrsv_dev(int uplo, int transa, int diag, int64_t m, double alpha, const double* a, int64_t rs_a, int64_t cs_a,
              double* x, int64_t incx, cudaStream_t s);
int dtrmm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha,
              const double* a, int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, int slices,
              cudaStream_t s);
int dsymm_dev(int side, int uplo, int64_t m, int64_t n, double alpha, const double* a, int64_t rs_a,
              int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c,
              int64_t cs_c, int slices, cudaStream_t s);
int dgemmt_dev(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a,
               int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c,
               int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s);
int dtrmm3_dev(int side, int uplo, int transa, int diag, int transb, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta,
               double* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s);
int dsyr2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a, int64_t rs_a, int64_t cs_a,
               const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c,
               int slices, cudaStream_t s);
template <typename T>
int cherk_dev(int uplo, int transa, int64_t m, int64_t k, T alpha, const T* a, int64_t rs_a, int64_t cs_a, T beta,
              T* c, int64_t rs_c, int64_t cs_c, int slices, cudaStream_t s);
template <typename R>
int cgemv_dev(int transa, int conjx, int64_t m, int64_t n, const R* alpha, const R* a, int64_t rs_a, int64_t cs_a,
              const R* x, int64_t incx, const R* beta, R* y, int64_t incy, cudaStream_t s);
template <typename R>
int ctrmm_dev(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const R* alpha, const R* a,
              int64_t rs_a, int64_t cs_a, R* b, int64_t rs_b, int64_t cs_b, int slices, cudaStream_t s);
template <typename T>
int csyr2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c,
               int64_t cs_c, int slices, cudaStream_t s);
template <typename T>
int cher2k_dev(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, T beta, T* c, int64_t rs_c, int64_t cs_c,
               int slices, cudaStream_t s);
template <typename T>
int chemm_dev(int side, int uplo, int herm, int conja, int transb, int64_t m, int64_t n, const T* alpha, const T* a,
              int64_t rs_a, int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c,
              int64_t cs_c, int slices, cudaStream_t s);
// The Ozaki form in two phases (gb_ozaki.cu): op(A) split once, then any
// number of products with column blocks of op(B) (bit-identical to one call).
struct OzA {
    int slices = 0;             // digit slices, or the CRT form's moduli count
    int crt = 0;                // 1: the CRT form (residues mod `slices` moduli, crt_t-bit integers)
    int crt_t = 0;
    bool pair_form = false;
    int64_t row_tile = 0;       // rows of one slice GEMM output tile (256 for CTA pairs, 128 else)
    int tri = 0;                // op(A) zero outside its lower (1) / upper (2) triangle: zero k blocks skipped
    int out_tri = 0;            // write only C's lower (1) / upper (2) triangle: row i, column j stored when
    int out_rpc = 1;            //   i / out_rpc >= j (<= j); out_rpc = 2 for a complex C's real view
    int64_t m = 0, k = 0, mpad = 0, kpad = 0;
    const double* a = nullptr;  // op(A) (i, l) = a[i*ars + l*acs], kept for the IEEE fallback
    int64_t ars = 0, acs = 0;
    uint8_t* ws = nullptr;      // slices, row maxima, exponents, Inf/NaN flag
    uint16_t* sa = nullptr;
    unsigned long long* maxa = nullptr;
    int32_t* ea = nullptr;
    int* nonfinite = nullptr;
};
struct OzB {
    int64_t n = 0, npad = 0;
    const double* b = nullptr;  // op(B) (l, j) = b[l*brs + j*bcs], kept for the IEEE fallback
    int64_t brs = 0, bcs = 0;
    uint8_t* ws = nullptr;      // slices, column maxima, exponents
    uint16_t* sb = nullptr;
    unsigned long long* maxb = nullptr;
    int32_t* eb = nullptr;
};
int ozaki_alloc_a(int64_t m, int64_t k, const double* a, int64_t ars, int64_t acs, int slices, cudaStream_t s,
                  OzA* A);
int ozaki_split_a_rows(const OzA* A, int64_t r0, int64_t r1, cudaStream_t s);
int ozaki_prepare_a(int64_t m, int64_t k, const double* a, int64_t ars, int64_t acs, int slices,
                    cudaStream_t s, OzA* A);
int ozaki_alloc_b(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, cudaStream_t s, OzB* B);
int ozaki_prepare_b(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, cudaStream_t s, OzB* B);
void ozaki_release_b(OzB* B, cudaStream_t s);
int ozaki_multiply_rows(const OzA* A, int64_t r0, int64_t rows, const OzB* B, double alpha, double beta, double* c,
                        int64_t rs_c, int64_t cs_c, cudaStream_t s);
int ozaki_multiply(const OzA* A, int64_t n, const double* b, int64_t brs, int64_t bcs, double alpha,
                   double beta, double* c, int64_t rs_c, int64_t cs_c, cudaStream_t s);
void ozaki_release_a(OzA* A, cudaStream_t s);
// bf16 GEMM on the tensor cores (gb_ozaki.cu): C fp32, A and B as bf16 bit
// patterns with element strides.
int bgemm_tc(int64_t m, int64_t n, int64_t k, float alpha, const uint16_t* a, int64_t ars, int64_t acs,
             const uint16_t* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
             cudaStream_t s);
// Grouped Ozaki form for gemm_batch (gb_ozaki.cu): every accepted problem
// (m, n, k > 0, alpha != 0, ozaki_batch_accepts) in three launches.  The
// flag is raised when an operand holds Inf/NaN; the launches then do
// nothing and a native grouped launch gated on the flag must follow.
// f32: FP32 operands and C (SGEMM's split form at GB_SGEMM_SPLIT_SLICES),
// each element widened exactly as it is split, C rounded once.
struct OzBatch;
bool ozaki_batch_accepts(int64_t k, int slices);
int ozaki_batch_create(const gb_gemm_problem_t* probs, int64_t count, int slices, cudaStream_t s,
                       OzBatch** out, bool f32 = false);
int ozaki_batch_launch(OzBatch* ob, cudaStream_t s);
const int* ozaki_batch_flag(const OzBatch* ob);
void ozaki_batch_destroy(OzBatch* ob, cudaStream_t s);
// gemm_batch problems whose selected configuration is the 64 x 64 engine
// (configs 1..5; m, n, k > 0, alpha != 0), grouped in one launch plus one
// fold launch for the problems split along k (gb_sup.cu).
struct SupGroup;
int sup_group_create(int dtype, const gb_gemm_problem_t* probs, const int* configs, int64_t count, cudaStream_t s,
                     SupGroup** out);
int sup_group_launch(SupGroup* g, cudaStream_t s);
void sup_group_destroy(SupGroup* g, cudaStream_t s);
int dotv_nparts(int64_t n);
int scal_matrix(int64_t m, int64_t n, double beta, double* c, int64_t rs_c, int64_t cs_c,
                cudaStream_t s);
int scal_matrix_f(int64_t m, int64_t n, float beta, float* c, int64_t rs_c, int64_t cs_c,
                  cudaStream_t s);
int daxpyv_dev(int64_t n, double alpha, const double* x, int64_t incx, double* y,
               int64_t incy, cudaStream_t s);
int ddotv_dev(int64_t n, const double* x, int64_t incx, const double* y, int64_t incy,
              double* rho_dev, double* scratch, int64_t scratch_len, cudaStream_t s);
int dgemv_dev(int trans, int64_t m, int64_t n, double alpha, const double* a,
              int64_t rs_a, int64_t cs_a, const double* x, int64_t incx, double beta,
              double* y, int64_t incy, cudaStream_t s);

// Default precision mode for dgemm entry points (GB_DGEMM_NATIVE or
// GB_DGEMM_OZAKI) and slice count, set by gb_set_dgemm_mode().
int dgemm_mode();
int ozaki_slices();
// Scoped per-thread dgemm mode (restored on destruction).
// Form of the Ozaki products (0: digit slices, 1: CRT residues), process-wide
// (gb_set_dgemm_mode) with a per-thread override.
int ozaki_form();
// CRT form: integer bits t of the scaled operands for n moduli and depth k
// (the largest t with k 2^(2t) <= 8 M / 17), or -1; the smallest n whose t
// reaches `bits`, or -1; the digit count of equal precision (grouped batch).
int ozaki_crt_bits(int n, int64_t k);
int ozaki_crt_moduli_for_bits(int bits, int64_t k);
// B := B - A X in the digit form at `slices` slices, one launch (R <= 128 rows,
// k <= 128): bit-identical to dgemm_ozaki(rows, n, k, -1, A, X, 1, B) with
// the same slices.
// aimg/aexp: A's digit image from trsm_images_build (null: the kernel splits A).
// packed_diag: the packed 64 x 64 diagonal block of the updated rows (rows <= 64), which the
// kernel then solves in place (lower or upper substitution), as trsm_diag_kernel would.
bool trsm_update_fused_fits(int slices, int64_t rows, int64_t k, int64_t n);
int trsm_update_fused(int slices, int64_t rows, int64_t k, int64_t n, const double* a, int64_t ars, int64_t acs,
                      const double* x, int64_t xrs, int64_t xcs, double* b, int64_t brs, int64_t bcs, cudaStream_t s,
                      const uint8_t* aimg = nullptr, const int* aexp = nullptr, const double* packed_diag = nullptr,
                      int diag_lower = 0);
// Digit images of the A blocks of a solve's fused updates, built by one launch:
// block (r0, c0) of op(A) (rows x k) -> (image, exponents).
struct TrsmImgSpec {
    int64_t r0, c0, rows, k;
};
struct TrsmImages {
    uint8_t* arena = nullptr;
    int slices = 0;
    std::unordered_map<uint64_t, std::pair<const uint8_t*, const int*>> index;
};
int trsm_images_build(int slices, const double* a, int64_t ars, int64_t acs, const TrsmImgSpec* specs, int nspecs,
                      TrsmImages* out, cudaStream_t s);
void trsm_images_release(TrsmImages* im, cudaStream_t s);
int ozaki_digit_slices();
// SGEMM split form (gb_sgemm_split.cu): the digit form with this many slices on
// FP64-widened operands; whether a shape takes it (gb_set_sgemm_mode).
constexpr int GB_SGEMM_SPLIT_SLICES = 3;
extern int sgemm_mode_setting;  // GB_SGEMM_FMA, _SPLIT or _AUTO (gb_set_sgemm_mode)
bool sgemm_use_split(int64_t m, int64_t n, int64_t k);
int ozaki_flag_or(const int* fa, const int* fb, int* out, cudaStream_t s);  // out = *fa | *fb, on s
int dgemm_ozaki_blocks(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t ars, int64_t acs,
                       const double* b, int64_t brs, int64_t bcs, double beta, double* c, int64_t rs_c, int64_t cs_c,
                       int slices, cudaStream_t s);  // gb_ozaki.cu: dgemm_ozaki in blocks on three streams
int sgemm_ozaki(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                cudaStream_t s);  // gb_ozaki.cu
int sgemm_split_dev(int64_t m, int64_t n, int64_t k, float alpha, const float* a, int64_t ars, int64_t acs,
                    const float* b, int64_t brs, int64_t bcs, float beta, float* c, int64_t rs_c, int64_t cs_c,
                    cudaStream_t s);
// Records the slice count of an Ozaki product on the calling thread
// (gb_last_ozaki_slices); 0 when a gemm's product ran on the native kernel.
void note_ozaki_slices(int slices);
class ModeOverride {
public:
    ModeOverride(int mode, int slices, int form = -1);
    ~ModeOverride();

private:
    int mode_, slices_, form_;
};

}  // namespace gb
