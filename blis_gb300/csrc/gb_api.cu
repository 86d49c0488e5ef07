// gb_api.cu -- the exported C ABI: BLAS compat layer, CBLAS, typed BLIS API
// and the gb_ device-pointer addon.
//
// Host-pointer entry points follow the reference's argument handling line
// for line in behaviour (checks and xerbla numbering from
// frame/compat/check/bla_*_check.h, negative-increment conversion from
// frame/include/bli_blas_macro_defs.h:50-75, the m==1/n==1 gemv redirect of
// frame/compat/bla_gemm.c:180-218, the gemv n_x==0 quirk of
// frame/compat/bla_gemv.c:88-106), then stage operands into HBM with
// stream-ordered allocations, run the device kernels and copy results back
// before returning, as a synchronous BLAS call must.
#include <ctype.h>
#include <string.h>

#include <vector>

#include "gb_internal.h"

namespace gb {
namespace {

// ---------------------------------------------------------------- staging
struct Staged {
    char* alloc = nullptr;
    char* origin = nullptr;
    int64_t rs = 0, cs = 0;
    int layout = 0;  // 0 packed column-major, 1 packed row-major, 2 span
};

int pick_layout(int64_t rows, int64_t cols, int64_t rs, int64_t cs)
{
    if (rs == 1 && (cols == 1 || cs >= rows)) return 0;
    if (cs == 1 && (rows == 1 || rs >= cols)) return 1;
    return 2;
}

void span_of(int64_t rows, int64_t cols, int64_t rs, int64_t cs, int64_t* lo, int64_t* hi)
{
    const int64_t o[4] = {0, (rows - 1) * rs, (cols - 1) * cs, (rows - 1) * rs + (cols - 1) * cs};
    *lo = o[0];
    *hi = o[0];
    for (int i = 1; i < 4; ++i) {
        if (o[i] < *lo) *lo = o[i];
        if (o[i] > *hi) *hi = o[i];
    }
}

// Copies a host (or any UVA) matrix into a fresh device buffer.  Packed
// layouts drop the leading-dimension padding; general strides copy the
// whole span and keep the strides.  `need_data` false skips the copy for
// packed outputs that are fully overwritten (beta == 0).
int stage_in(const void* host, int64_t rows, int64_t cols, int64_t rs, int64_t cs, size_t esz,
             bool need_data, Staged* st, cudaStream_t s)
{
    *st = Staged();
    if (rows <= 0 || cols <= 0) return GB_SUCCESS;
    st->layout = pick_layout(rows, cols, rs, cs);
    if (st->layout == 0) {
        st->alloc = static_cast<char*>(dev_alloc((size_t)rows * cols * esz, s));
        if (!st->alloc) return GB_ERR_NOMEM;
        st->origin = st->alloc;
        st->rs = 1;
        st->cs = rows;
        const size_t sp = (size_t)((cols == 1) ? rows : cs) * esz;
        if (need_data)
            GB_CUDA(cudaMemcpy2DAsync(st->alloc, rows * esz, host, sp, rows * esz, cols,
                                      cudaMemcpyDefault, s));
    } else if (st->layout == 1) {
        st->alloc = static_cast<char*>(dev_alloc((size_t)rows * cols * esz, s));
        if (!st->alloc) return GB_ERR_NOMEM;
        st->origin = st->alloc;
        st->rs = cols;
        st->cs = 1;
        const size_t sp = (size_t)((rows == 1) ? cols : rs) * esz;
        if (need_data)
            GB_CUDA(cudaMemcpy2DAsync(st->alloc, cols * esz, host, sp, cols * esz, rows,
                                      cudaMemcpyDefault, s));
    } else {
        int64_t lo, hi;
        span_of(rows, cols, rs, cs, &lo, &hi);
        const size_t count = (size_t)(hi - lo + 1);
        st->alloc = static_cast<char*>(dev_alloc(count * esz, s));
        if (!st->alloc) return GB_ERR_NOMEM;
        st->origin = st->alloc - lo * (int64_t)esz;
        st->rs = rs;
        st->cs = cs;
        // always copied: the write-back below covers the whole span
        GB_CUDA(cudaMemcpyAsync(st->alloc, static_cast<const char*>(host) + lo * (int64_t)esz,
                                count * esz, cudaMemcpyDefault, s));
    }
    return GB_SUCCESS;
}

int stage_out(void* host, int64_t rows, int64_t cols, int64_t rs, int64_t cs, size_t esz,
              const Staged& st, cudaStream_t s)
{
    if (rows <= 0 || cols <= 0 || !st.alloc) return GB_SUCCESS;
    if (st.layout == 0) {
        const size_t dp = (size_t)((cols == 1) ? rows : cs) * esz;
        GB_CUDA(cudaMemcpy2DAsync(host, dp, st.alloc, rows * esz, rows * esz, cols, cudaMemcpyDefault, s));
    } else if (st.layout == 1) {
        const size_t dp = (size_t)((rows == 1) ? cols : rs) * esz;
        GB_CUDA(cudaMemcpy2DAsync(host, dp, st.alloc, cols * esz, cols * esz, rows, cudaMemcpyDefault, s));
    } else {
        int64_t lo, hi;
        span_of(rows, cols, rs, cs, &lo, &hi);
        GB_CUDA(cudaMemcpyAsync(static_cast<char*>(host) + lo * (int64_t)esz, st.alloc,
                                (size_t)(hi - lo + 1) * esz, cudaMemcpyDefault, s));
    }
    return GB_SUCCESS;
}

struct Bufs {
    cudaStream_t s;
    Staged b[4];
    int n = 0;
    explicit Bufs(cudaStream_t st) : s(st) {}
    Staged& next() { return b[n++]; }
    ~Bufs()
    {
        for (int i = 0; i < n; ++i) dev_free(b[i].alloc, s);
    }
};

int finish(cudaStream_t s, const char* where)
{
    GB_CUDA(cudaStreamSynchronize(s));
    return read_and_clear_device_status(s, where);
}

// ---------------------------------------------------------------- host ops
// The Ozaki form on host buffers, pipelined: op(A) goes to HBM and is split
// once while op(B) (column-major) streams in column blocks on one copy stream
// and finished blocks of C (column-major) stream back on another, so the
// host<->device transfers of B and C overlap the slice GEMMs.  Column blocks
// of op(B) are split independently: the result is bit-identical to one call.
int ozaki_host_pipelined(int transa, int64_t m, int64_t n, int64_t k, double alpha, const double* a,
                         int64_t rs_a, int64_t cs_a, const double* b, int64_t ldb, double beta, double* c,
                         int64_t ldc, int slices, int nch, const char* where)
{
    cudaStream_t s = thread_stream(), cin = thread_copy_stream(0), cout = thread_copy_stream(1);
    const bool ta = GB_IS_TRANS(transa);
    int rc;
    Bufs bufs(s);
    Staged& A = bufs.next();
    if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, sizeof(double), true, &A, s))) return rc;
    OzA prep;
    double* bd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(k * n), s));
    double* cd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(m * n), s));
    cudaEvent_t ev[2 * 8 + 3];
    const int nev = 2 * nch + 3;
    for (int i = 0; i < nev; ++i) cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
    cudaEvent_t *ev_in = ev, *ev_out = ev + nch, ev_alloc = ev[2 * nch], ev_in_done = ev[2 * nch + 1],
                ev_out_done = ev[2 * nch + 2];
    rc = (bd && cd) ? GB_SUCCESS : GB_ERR_NOMEM;
    if (!rc) {
        // The copy streams may touch bd/cd only after their stream-ordered allocation, and
        // op(B)'s blocks go up only after A (both ordered by ev_alloc): sharing the link with
        // them would delay A, which every slice product needs.  A's split below then overlaps
        // the first block's transfer.
        cudaEventRecord(ev_alloc, s);
        cudaStreamWaitEvent(cin, ev_alloc, 0);
        cudaStreamWaitEvent(cout, ev_alloc, 0);
        for (int j = 0; j < nch && !rc; ++j) {
            const int64_t j0 = n * j / nch, nj = n * (j + 1) / nch - j0;
            rc = check_cuda(cudaMemcpy2DAsync(bd + j0 * k, k * sizeof(double), b + j0 * ldb, ldb * sizeof(double),
                                              k * sizeof(double), nj, cudaMemcpyDefault, cin), "B block");
            if (!rc && beta != 0.0)
                rc = check_cuda(cudaMemcpy2DAsync(cd + j0 * m, m * sizeof(double), c + j0 * ldc, ldc * sizeof(double),
                                                  m * sizeof(double), nj, cudaMemcpyDefault, cin), "C block");
            cudaEventRecord(ev_in[j], cin);
        }
        if (!rc)
            rc = ozaki_prepare_a(m, k, reinterpret_cast<const double*>(A.origin), ta ? A.cs : A.rs,
                                 ta ? A.rs : A.cs, slices, s, &prep);
        for (int j = 0; j < nch && !rc; ++j) {
            const int64_t j0 = n * j / nch, nj = n * (j + 1) / nch - j0;
            cudaStreamWaitEvent(s, ev_in[j], 0);
            rc = ozaki_multiply(&prep, nj, bd + j0 * k, 1, k, alpha, beta, cd + j0 * m, 1, m, s);
            cudaEventRecord(ev_out[j], s);
            cudaStreamWaitEvent(cout, ev_out[j], 0);
            if (!rc)
                rc = check_cuda(cudaMemcpy2DAsync(c + j0 * ldc, ldc * sizeof(double), cd + j0 * m, m * sizeof(double),
                                                  m * sizeof(double), nj, cudaMemcpyDefault, cout), "C back");
        }
        // frees below are ordered after every copy on either copy stream
        cudaEventRecord(ev_in_done, cin);
        cudaEventRecord(ev_out_done, cout);
        cudaStreamWaitEvent(s, ev_in_done, 0);
        cudaStreamWaitEvent(s, ev_out_done, 0);
    }
    ozaki_release_a(&prep, s);
    dev_free(bd, s);
    dev_free(cd, s);
    const int rc2 = finish(s, where);
    for (int i = 0; i < nev; ++i) cudaEventDestroy(ev[i]);
    return rc ? rc : rc2;
}

// The same with op(A) in row blocks too, for a column-major stored A
// (rs_a == 1): row block 0 of A and column block 0 of op(B) go up first, the
// first slice GEMM starts after them, and the other blocks of A arrive (and
// are split) while it runs; every (row block, column block) of C is one
// slice GEMM and goes back as soon as it is recombined.  Only about a
// quarter of A and of one op(B) block, and one C block, are not overlapped
// with compute.  The block products alternate between the thread's stream
// and a second compute stream, so one block's last wave of tiles shares the
// SMs with the next block's first (a 4096 x 4096 block is 256 tiles of
// 256 x 256, 3.4 waves of 76 CTA pairs); the splits run on a third stream as
// the blocks land, and each product waits only for the splits it reads.
// Rows and columns are split independently: with finite operands the result
// is bit-identical to one call.  Each block product is gated on the Inf/NaN
// flags of its own row and column blocks (ozaki_flag_or): a flag shared by
// all blocks could be raised by a later block's split between one product's
// recombination and its gated fallback, applying beta twice.
int ozaki_host_pipelined_2d(int transa, int64_t m, int64_t n, int64_t k, double alpha, const double* a,
                            int64_t lda, const double* b, int64_t ldb, double beta, double* c, int64_t ldc,
                            int slices, int nch, const char* where)
{
    cudaStream_t s = thread_stream(), cin = thread_copy_stream(0), cout = thread_copy_stream(1);
    cudaStream_t sp[2] = {s, thread_aux_stream(0)}, ss = thread_aux_stream(1);
    const bool ta = GB_IS_TRANS(transa);
    // op(A) on the device: m x k column-major (ars 1, acs m), or for op(A) = A^T the stored k x m
    // column-major A (ars k, acs 1)
    double* ad = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(m * k), s));
    double* bd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(k * n), s));
    double* cd = static_cast<double*>(dev_alloc(sizeof(double) * (size_t)(m * n), s));
    int rc = (ad && bd && cd) ? GB_SUCCESS : GB_ERR_NOMEM;
    OzA prep;
    if (!rc) rc = ozaki_alloc_a(m, k, ad, ta ? k : 1, ta ? 1 : m, slices, s, &prep);
    // row blocks on the slice GEMM's row tile: 8 where the device entry points' blocked form
    // measured faster with them (digit form from 8192 rows, CRT form from 16384)
    const int64_t big = (ozaki_form() == 1) ? 16384 : 8192;
    const int nra = (m >= big && n >= big) ? 8 : ((m >= 8 * prep.row_tile) ? 4 : ((m >= 2 * prep.row_tile) ? 2 : 1));
    std::vector<int64_t> rb(1, 0);
    for (int i = 1; i < nra && !rc; ++i) {
        const int64_t r = (m * i / nra + prep.row_tile - 1) / prep.row_tile * prep.row_tile;
        if (r > rb.back() && r < m) rb.push_back(r);
    }
    rb.push_back(m);
    const int na = (int)rb.size() - 1;
    // Inf/NaN flags: one per row block, per column block and per block product
    int* flags = rc ? nullptr : static_cast<int*>(dev_alloc(sizeof(int) * (size_t)(na + nch + na * nch), s));
    if (!rc && !flags) rc = GB_ERR_NOMEM;
    if (!rc) rc = check_cuda(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(na + nch + na * nch), s), "flags");
    int *fa = flags, *fb = flags + na, *fab = flags + na + nch;
    auto with_flag = [&](int* f) {
        OzA x = prep;
        x.nonfinite = f;
        return x;
    };
    // events: A blocks in, B blocks in, A blocks split, B blocks split, C blocks done, then
    // the allocation, the two copy streams' ends, the second compute stream's end and the
    // split stream's end
    std::vector<cudaEvent_t> ev((size_t)(2 * na + 2 * nch + na * nch + 5));
    for (auto& e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaEvent_t* ev_a = ev.data();
    cudaEvent_t* ev_b = ev_a + na;
    cudaEvent_t* ev_sa = ev_b + nch;
    cudaEvent_t* ev_sb = ev_sa + na;
    cudaEvent_t* ev_c = ev_sb + nch;
    cudaEvent_t ev_alloc = ev_c[na * nch], ev_in_done = ev_c[na * nch + 1], ev_out_done = ev_c[na * nch + 2],
                ev_aux_done = ev_c[na * nch + 3], ev_split_done = ev_c[na * nch + 4];
    auto col0 = [&](int j) { return n * j / nch; };
    std::vector<OzB> pb((size_t)nch);
    if (!rc) {
        // copies start after the stream-ordered allocations; A's block 0 and op(B)'s block 0 first
        cudaEventRecord(ev_alloc, s);
        cudaStreamWaitEvent(cin, ev_alloc, 0);
        cudaStreamWaitEvent(cout, ev_alloc, 0);
        cudaStreamWaitEvent(sp[1], ev_alloc, 0);
        cudaStreamWaitEvent(ss, ev_alloc, 0);
        auto copy_a = [&](int i) {
            const int64_t r0 = rb[i], rows = rb[i + 1] - rb[i];
            LaunchScope ls("copy_h2d_a", cin, false);
            if (!rc)
                rc = ta ? check_cuda(cudaMemcpy2DAsync(ad + r0 * k, k * sizeof(double), a + r0 * lda,
                                                       lda * sizeof(double), k * sizeof(double), rows,
                                                       cudaMemcpyDefault, cin), "A block")
                        : check_cuda(cudaMemcpy2DAsync(ad + r0, m * sizeof(double), a + r0, lda * sizeof(double),
                                                       rows * sizeof(double), k, cudaMemcpyDefault, cin), "A block");
            cudaEventRecord(ev_a[i], cin);
        };
        auto copy_b = [&](int j) {
            const int64_t j0 = col0(j), nj = col0(j + 1) - j0;
            LaunchScope ls("copy_h2d_b", cin, false);
            if (!rc)
                rc = check_cuda(cudaMemcpy2DAsync(bd + j0 * k, k * sizeof(double), b + j0 * ldb, ldb * sizeof(double),
                                                  k * sizeof(double), nj, cudaMemcpyDefault, cin), "B block");
            if (!rc && beta != 0.0)
                rc = check_cuda(cudaMemcpy2DAsync(cd + j0 * m, m * sizeof(double), c + j0 * ldc, ldc * sizeof(double),
                                                  m * sizeof(double), nj, cudaMemcpyDefault, cin), "C block");
            cudaEventRecord(ev_b[j], cin);
        };
        copy_a(0);
        copy_b(0);
        for (int i = 1; i < na; ++i) copy_a(i);
        for (int j = 1; j < nch; ++j) copy_b(j);
        // splits on their own stream, in arrival order: A0, B0, the other A blocks, the other B blocks
        auto split_a = [&](int i) {
            cudaStreamWaitEvent(ss, ev_a[i], 0);
            const OzA ai = with_flag(fa + i);
            if (!rc) rc = ozaki_split_a_rows(&ai, rb[i], rb[i + 1], ss);
            cudaEventRecord(ev_sa[i], ss);
        };
        auto split_b = [&](int j) {
            const int64_t j0 = col0(j), nj = col0(j + 1) - j0;
            cudaStreamWaitEvent(ss, ev_b[j], 0);
            const OzA aj = with_flag(fb + j);
            if (!rc) rc = ozaki_prepare_b(&aj, nj, bd + j0 * k, 1, k, ss, &pb[(size_t)j]);
            cudaEventRecord(ev_sb[j], ss);
        };
        int q = 0;  // product stream of the next block
        auto product = [&](int i, int j) {
            const int64_t j0 = col0(j), nj = col0(j + 1) - j0, r0 = rb[i], rows = rb[i + 1] - rb[i];
            cudaStream_t ps = sp[q];
            q ^= 1;
            cudaStreamWaitEvent(ps, ev_sa[i], 0);
            cudaStreamWaitEvent(ps, ev_sb[j], 0);
            int* f = fab + i * nch + j;
            if (!rc) rc = ozaki_flag_or(fa + i, fb + j, f, ps);
            const OzA aij = with_flag(f);
            if (!rc) rc = ozaki_multiply_rows(&aij, r0, rows, &pb[(size_t)j], alpha, beta, cd + j0 * m + r0, 1, m, ps);
            cudaEventRecord(ev_c[i * nch + j], ps);
            cudaStreamWaitEvent(cout, ev_c[i * nch + j], 0);
            LaunchScope ls("copy_d2h_c", cout, false);
            if (!rc)
                rc = check_cuda(cudaMemcpy2DAsync(c + j0 * ldc + r0, ldc * sizeof(double), cd + j0 * m + r0,
                                                  m * sizeof(double), rows * sizeof(double), nj, cudaMemcpyDefault,
                                                  cout), "C back");
        };
        split_a(0);
        split_b(0);
        for (int i = 1; i < na; ++i) split_a(i);
        for (int j = 1; j < nch; ++j) split_b(j);
        for (int j = 0; j < nch; ++j)
            for (int i = 0; i < na; ++i) product(i, j);
        // frees below are ordered after every copy and every product on either compute stream
        cudaEventRecord(ev_in_done, cin);
        cudaEventRecord(ev_out_done, cout);
        cudaEventRecord(ev_aux_done, sp[1]);
        cudaEventRecord(ev_split_done, ss);
        cudaStreamWaitEvent(s, ev_in_done, 0);
        cudaStreamWaitEvent(s, ev_out_done, 0);
        cudaStreamWaitEvent(s, ev_aux_done, 0);
        cudaStreamWaitEvent(s, ev_split_done, 0);
    }
    for (auto& x : pb) ozaki_release_b(&x, s);
    ozaki_release_a(&prep, s);
    dev_free(flags, s);
    dev_free(ad, s);
    dev_free(bd, s);
    dev_free(cd, s);
    const int rc2 = finish(s, where);
    for (auto& e : ev) cudaEventDestroy(e);
    return rc ? rc : rc2;
}

template <typename T>
int gemm_host(int transa, int transb, int64_t m, int64_t n, int64_t k, T alpha, const T* a,
              int64_t rs_a, int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, T beta, T* c,
              int64_t rs_c, int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    if (sizeof(T) == 8 && dgemm_mode() == GB_DGEMM_OZAKI && ozaki_slices() >= 2 && alpha != T(0) && k > 0 &&
        !GB_IS_TRANS(transb) && rs_b == 1 && cs_b >= k && rs_c == 1 && cs_c >= m && n >= 2048 &&
        m * k >= (int64_t(1) << 22)) {
        // large products with a fixed slice count, column-major op(B) and C: the transfers
        // of op(B) and C overlap the compute
        const int nch = (n >= 8192) ? 4 : 2;
        if (rs_a == 1 && cs_a >= (GB_IS_TRANS(transa) ? k : m))
            return ozaki_host_pipelined_2d(transa, m, n, k, (double)alpha, (const double*)a, cs_a,
                                           (const double*)b, cs_b, (double)beta, (double*)c, cs_c, ozaki_slices(),
                                           nch, where);
        return ozaki_host_pipelined(transa, m, n, k, (double)alpha, (const double*)a, rs_a, cs_a, (const double*)b,
                                    cs_b, (double)beta, (double*)c, cs_c, ozaki_slices(), nch, where);
    }
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = sizeof(T);
    const bool trivial = (alpha == T(0) || k <= 0);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, n, rs_c, cs_c, esz, beta != T(0), &C, s))) return rc;
    T* cd = reinterpret_cast<T*>(C.origin);
    if (trivial) {
        if (sizeof(T) == 8) rc = scal_matrix(m, n, (double)beta, (double*)cd, C.rs, C.cs, s);
        else rc = scal_matrix_f(m, n, (float)beta, (float*)cd, C.rs, C.cs, s);
    } else {
        const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
        Staged& A = bufs.next();
        Staged& B = bufs.next();
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, esz, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? n : k, tb ? k : n, rs_b, cs_b, esz, true, &B, s))) return rc;
        const int64_t ars = ta ? A.cs : A.rs, acs = ta ? A.rs : A.cs;
        const int64_t brs = tb ? B.cs : B.rs, bcs = tb ? B.rs : B.cs;
        // leading-dimension padding of the caller's operand, a selector feature
        const int64_t pad = (rs_a == 1) ? cs_a - (ta ? k : m) : ((cs_a == 1) ? rs_a - (ta ? m : k) : 0);
        if (sizeof(T) == 8 && dgemm_mode() == GB_DGEMM_OZAKI) {
            const double* ad = reinterpret_cast<const double*>(A.origin);
            const double* bd = reinterpret_cast<const double*>(B.origin);
            int slices = ozaki_slices();
            if (selector_auto()) {
                // the selector's Ozaki engine for this shape, decided now (a host call waits anyway)
                int eng = 0;
                if ((rc = selector_ozaki_engine(m, n, k, &eng))) return rc;
            }
            bool native = false;
            if (slices == 0) {
                // auto: the selector's proposal, checked by the error-bound verifier
                int cfg = 0, prop = 8;
                const double sa = host_exponent_spread((const double*)a, ta ? k : m, ta ? m : k, rs_a, cs_a);
                const double sb = host_exponent_spread((const double*)b, tb ? n : k, tb ? k : n, rs_b, cs_b);
                if ((rc = selector_choose(0, m, n, k, ta, tb, (int)pad, sa, sb, &cfg, &prop))) return rc;
                int checked = prop;
                if ((rc = gb_ozaki_verify_slices_dev(transa, transb, m, n, k, ad, A.rs, A.cs, bd, B.rs, B.cs, prop,
                                                     256, &checked, s)))
                    return rc;
                slices = checked;
                native = checked > 12;  // no slice count reaches the bound: IEEE path
                if (!native && ozaki_form() == 1) {
                    // the CRT form at the precision of the verified digit count (8s - 1 bits)
                    slices = ozaki_crt_moduli_for_bits(8 * checked - 1, k);
                    native = slices < 0;
                }
            }
            if (native) {
                note_ozaki_slices(0);
                rc = dgemm_native(m, n, k, (double)alpha, ad, ars, acs, bd, brs, bcs, (double)beta, (double*)cd,
                                  C.rs, C.cs, s);
            }
            else
                rc = dgemm_ozaki(m, n, k, (double)alpha, ad, ars, acs, bd, brs, bcs, (double)beta, (double*)cd,
                                 C.rs, C.cs, slices, s);
        } else {
            if (sizeof(T) == 4 && sgemm_use_split(m, n, k)) {
                rc = sgemm_split_dev(m, n, k, (float)alpha, (const float*)A.origin, ars, acs,
                                     (const float*)B.origin, brs, bcs, (float)beta, (float*)cd, C.rs, C.cs, s);
                if (rc) return rc;
                if ((rc = stage_out(c, m, n, rs_c, cs_c, esz, C, s))) return rc;
                return finish(s, where);
            }
            // the learned selector when it is on (by default: the committed model), else the
            // occupancy rule
            int cfg = selector_heuristic(m, n, k), unused = 0;
            if (selector_auto() && (rc = selector_choose(sizeof(T) == 8 ? 0 : 1, m, n, k, ta, tb, (int)pad, 0.0,
                                                         0.0, &cfg, &unused)))
                return rc;
            rc = gemm_config_dev(sizeof(T) == 8 ? 0 : 1, cfg, m, n, k, (double)alpha, A.origin, ars, acs, B.origin,
                                 brs, bcs, (double)beta, cd, C.rs, C.cs, s);
        }
    }
    if (rc) return rc;
    if ((rc = stage_out(c, m, n, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

int gemv_host(int transa, int64_t m, int64_t n, double alpha, const double* a, int64_t rs_a,
              int64_t cs_a, const double* x, int64_t incx, double beta, double* y, int64_t incy,
              const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    const bool tr = GB_IS_TRANS(transa);
    const int64_t my = tr ? n : m, nx = tr ? m : n;
    if (my <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& Y = bufs.next();
    if ((rc = stage_in(y, my, 1, incy, my, 8, beta != 0.0, &Y, s))) return rc;
    const double* ad = nullptr;
    const double* xd = nullptr;
    int64_t ars = rs_a, acs = cs_a, xinc = incx;
    if (nx > 0 && alpha != 0.0) {
        Staged& A = bufs.next();
        Staged& X = bufs.next();
        if ((rc = stage_in(a, m, n, rs_a, cs_a, 8, true, &A, s))) return rc;
        if ((rc = stage_in(x, nx, 1, incx, nx, 8, true, &X, s))) return rc;
        ad = reinterpret_cast<const double*>(A.origin);
        xd = reinterpret_cast<const double*>(X.origin);
        ars = A.rs;
        acs = A.cs;
        xinc = X.rs;
    }
    if ((rc = dgemv_dev(tr ? 1 : 0, m, n, alpha, ad, ars, acs, xd, xinc, beta,
                        reinterpret_cast<double*>(Y.origin), Y.rs, s)))
        return rc;
    if ((rc = stage_out(y, my, 1, incy, my, 8, Y, s))) return rc;
    return finish(s, where);
}

int axpyv_host(int64_t n, double alpha, const double* x, int64_t incx, double* y, int64_t incy)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n <= 0 || alpha == 0.0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    Staged& Y = bufs.next();
    if ((rc = stage_in(x, n, 1, incx, n, 8, true, &X, s))) return rc;
    if ((rc = stage_in(y, n, 1, incy, n, 8, true, &Y, s))) return rc;
    if ((rc = daxpyv_dev(n, alpha, reinterpret_cast<const double*>(X.origin), X.rs,
                         reinterpret_cast<double*>(Y.origin), Y.rs, s)))
        return rc;
    if ((rc = stage_out(y, n, 1, incy, n, 8, Y, s))) return rc;
    return finish(s, "axpyv");
}

int dotv_host(int64_t n, const double* x, int64_t incx, const double* y, int64_t incy, double* rho)
{
    int rc = ensure_init();
    if (rc) return rc;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    Staged& Y = bufs.next();
    if (n > 0) {
        if ((rc = stage_in(x, n, 1, incx, n, 8, true, &X, s))) return rc;
        if ((rc = stage_in(y, n, 1, incy, n, 8, true, &Y, s))) return rc;
    }
    const int nparts = dotv_nparts(n > 0 ? n : 1);
    double* scratch = static_cast<double*>(dev_alloc(sizeof(double) * (nparts + 1), s));
    if (!scratch) return GB_ERR_NOMEM;
    rc = ddotv_dev(n, reinterpret_cast<const double*>(X.origin), X.rs,
                   reinterpret_cast<const double*>(Y.origin), Y.rs, scratch + nparts, scratch, nparts, s);
    if (!rc) rc = check_cuda(cudaMemcpyAsync(rho, scratch + nparts, sizeof(double), cudaMemcpyDeviceToHost, s), "dotv");
    dev_free(scratch, s);
    if (rc) return rc;
    return finish(s, "dotv");
}

int trsm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha,
              const double* a, int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, 8, alpha != 0.0, &B, s))) return rc;
    Staged& A = bufs.next();
    if (alpha != 0.0 && (rc = stage_in(a, na, na, rs_a, cs_a, 8, true, &A, s))) return rc;
    const int slices = (dgemm_mode() == GB_DGEMM_OZAKI) ? ozaki_slices() : 0;
    if ((rc = dtrsm_dev(side, uplo, transa, diag, m, n, alpha,
                        reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                        reinterpret_cast<double*>(B.origin), B.rs, B.cs, slices, s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, 8, B, s))) return rc;
    return finish(s, "trsm");
}

// strsm on host buffers: the operands staged into HBM, strsm_dev (native FP32 recursion)
int strsm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, float alpha, const float* a,
               int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, 4, alpha != 0.0f, &B, s))) return rc;
    Staged& A = bufs.next();
    if (alpha != 0.0f && (rc = stage_in(a, na, na, rs_a, cs_a, 4, true, &A, s))) return rc;
    if ((rc = strsm_dev(side, uplo, transa, diag, m, n, alpha, reinterpret_cast<const float*>(A.origin), A.rs,
                        A.cs, reinterpret_cast<float*>(B.origin), B.rs, B.cs, s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, 4, B, s))) return rc;
    return finish(s, where);
}

int level3_slices() { return (dgemm_mode() == GB_DGEMM_OZAKI) ? ozaki_slices() : 0; }

int trmm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha, const double* a,
              int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, 8, alpha != 0.0, &B, s))) return rc;
    Staged& A = bufs.next();
    if (alpha != 0.0 && (rc = stage_in(a, na, na, rs_a, cs_a, 8, true, &A, s))) return rc;
    if ((rc = dtrmm_dev(side, uplo, transa, diag, m, n, alpha, reinterpret_cast<const double*>(A.origin), A.rs,
                        A.cs, reinterpret_cast<double*>(B.origin), B.rs, B.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, 8, B, s))) return rc;
    return finish(s, where);
}

int symm_host(int side, int uplo, int64_t m, int64_t n, double alpha, const double* a, int64_t rs_a, int64_t cs_a,
              const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c, int64_t cs_c,
              const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, n, rs_c, cs_c, 8, beta != 0.0, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (alpha != 0.0) {
        if ((rc = stage_in(a, na, na, rs_a, cs_a, 8, true, &A, s))) return rc;
        if ((rc = stage_in(b, m, n, rs_b, cs_b, 8, true, &B, s))) return rc;
    }
    if ((rc = dsymm_dev(side, uplo, m, n, alpha, reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                        reinterpret_cast<const double*>(B.origin), B.rs, B.cs, beta,
                        reinterpret_cast<double*>(C.origin), C.rs, C.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(c, m, n, rs_c, cs_c, 8, C, s))) return rc;
    return finish(s, where);
}

// C (m x m, one triangle) := alpha op(A) op(B) + beta C; syrk passes B = A with transb = !transa
int gemmt_host(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a, int64_t rs_a,
               int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c,
               int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    // the whole of C goes up and comes back: the untouched triangle round-trips unchanged
    if ((rc = stage_in(c, m, m, rs_c, cs_c, 8, true, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    const bool need = (alpha != 0.0 && k > 0);
    if (need) {
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, 8, true, &A, s))) return rc;
        if (b == a && rs_b == rs_a && cs_b == cs_a) B = Staged{};  // syrk: the same staged copy
        else if ((rc = stage_in(b, tb ? m : k, tb ? k : m, rs_b, cs_b, 8, true, &B, s))) return rc;
    }
    const Staged& Bs = (need && b == a && rs_b == rs_a && cs_b == cs_a) ? A : B;
    if ((rc = dgemmt_dev(uplo, transa, transb, m, k, alpha, reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                         reinterpret_cast<const double*>(Bs.origin), Bs.rs, Bs.cs, beta,
                         reinterpret_cast<double*>(C.origin), C.rs, C.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(c, m, m, rs_c, cs_c, 8, C, s))) return rc;
    return finish(s, where);
}

int scalv_host(int64_t n, double alpha, double* x, int64_t incx, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n <= 0 || alpha == 1.0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    if ((rc = stage_in(x, n, 1, incx, n, 8, alpha != 0.0 || incx == 0, &X, s))) return rc;
    if ((rc = dscalv_dev(n, alpha, reinterpret_cast<double*>(X.origin), X.rs, s))) return rc;
    if ((rc = stage_out(x, n, 1, incx, n, 8, X, s))) return rc;
    return finish(s, where);
}

int copyv_host(int64_t n, const double* x, int64_t incx, double* y, int64_t incy, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    Staged& Y = bufs.next();
    if ((rc = stage_in(x, n, 1, incx, n, 8, true, &X, s))) return rc;
    if ((rc = stage_in(y, n, 1, incy, n, 8, false, &Y, s))) return rc;
    if ((rc = dcopyv_dev(n, reinterpret_cast<const double*>(X.origin), X.rs, reinterpret_cast<double*>(Y.origin),
                         Y.rs, s)))
        return rc;
    if ((rc = stage_out(y, n, 1, incy, n, 8, Y, s))) return rc;
    return finish(s, where);
}

int amaxv_host(int64_t n, const double* x, int64_t incx, int64_t* index, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    *index = 0;
    if (n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    if ((rc = stage_in(x, n, 1, incx, n, 8, true, &X, s))) return rc;
    int64_t* d = static_cast<int64_t*>(dev_alloc(sizeof(int64_t), s));
    if (!d) return GB_ERR_NOMEM;
    rc = damaxv_dev(n, reinterpret_cast<const double*>(X.origin), X.rs, d, s);
    if (!rc) rc = check_cuda(cudaMemcpyAsync(index, d, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "amaxv");
    dev_free(d, s);
    if (rc) return rc;
    return finish(s, where);
}

int ger_host(int64_t m, int64_t n, double alpha, const double* x, int64_t incx, const double* y, int64_t incy,
             double* a, int64_t rs_a, int64_t cs_a, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0 || alpha == 0.0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& A = bufs.next();
    Staged& X = bufs.next();
    Staged& Y = bufs.next();
    if ((rc = stage_in(a, m, n, rs_a, cs_a, 8, true, &A, s))) return rc;
    if ((rc = stage_in(x, m, 1, incx, m, 8, true, &X, s))) return rc;
    if ((rc = stage_in(y, n, 1, incy, n, 8, true, &Y, s))) return rc;
    if ((rc = dger_dev(m, n, alpha, reinterpret_cast<const double*>(X.origin), X.rs,
                       reinterpret_cast<const double*>(Y.origin), Y.rs, reinterpret_cast<double*>(A.origin), A.rs,
                       A.cs, s)))
        return rc;
    if ((rc = stage_out(a, m, n, rs_a, cs_a, 8, A, s))) return rc;
    return finish(s, where);
}

int trsv_host(int uplo, int transa, int diag, int64_t m, double alpha, const double* a, int64_t rs_a, int64_t cs_a,
              double* x, int64_t incx, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    Staged& X = bufs.next();
    if ((rc = stage_in(x, m, 1, incx, m, 8, true, &X, s))) return rc;
    Staged& A = bufs.next();
    if (alpha != 0.0 && (rc = stage_in(a, m, m, rs_a, cs_a, 8, true, &A, s))) return rc;
    if ((rc = dtrsv_dev(uplo, transa, diag, m, alpha, reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                        reinterpret_cast<double*>(X.origin), X.rs, s)))
        return rc;
    if ((rc = stage_out(x, m, 1, incx, m, 8, X, s))) return rc;
    return finish(s, where);
}

template <typename T>
int cgemm_host(int transa, int transb, int64_t m, int64_t n, int64_t k, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c, int64_t cs_c,
               const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, n, rs_c, cs_c, esz, beta[0] != T(0) || beta[1] != T(0), &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if ((alpha[0] != T(0) || alpha[1] != T(0)) && k > 0) {
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, esz, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? n : k, tb ? k : n, rs_b, cs_b, esz, true, &B, s))) return rc;
    }
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = cgemm_dev<T>(transa, transb, m, n, k, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs,
                           reinterpret_cast<const T*>(B.origin), B.rs, B.cs, beta, reinterpret_cast<T*>(C.origin),
                           C.rs, C.cs, slices, s)))
        return rc;
    if ((rc = stage_out(c, m, n, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

int ztrsm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const double* alpha, const double* a,
               int64_t rs_a, int64_t cs_a, double* b, int64_t rs_b, int64_t cs_b, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    const bool nz = !(alpha[0] == 0.0 && alpha[1] == 0.0);
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, 16, nz, &B, s))) return rc;
    Staged& A = bufs.next();
    if (nz && (rc = stage_in(a, na, na, rs_a, cs_a, 16, true, &A, s))) return rc;
    if ((rc = ztrsm_dev(side, uplo, transa, diag, m, n, alpha, reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                        reinterpret_cast<double*>(B.origin), B.rs, B.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, 16, B, s))) return rc;
    return finish(s, where);
}

int ctrsm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const float* alpha, const float* a,
               int64_t rs_a, int64_t cs_a, float* b, int64_t rs_b, int64_t cs_b, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    const bool nz = !(alpha[0] == 0.0f && alpha[1] == 0.0f);
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, 8, nz, &B, s))) return rc;
    Staged& A = bufs.next();
    if (nz && (rc = stage_in(a, na, na, rs_a, cs_a, 8, true, &A, s))) return rc;
    if ((rc = ctrsm_dev(side, uplo, transa, diag, m, n, alpha, reinterpret_cast<const float*>(A.origin), A.rs, A.cs,
                        reinterpret_cast<float*>(B.origin), B.rs, B.cs, s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, 8, B, s))) return rc;
    return finish(s, where);
}

// herk / her2k: the whole of C goes up and comes back, so the untouched
// triangle round-trips unchanged
template <typename T>
int cherk_host(int uplo, int transa, int64_t m, int64_t k, T alpha, const T* a, int64_t rs_a, int64_t cs_a, T beta,
               T* c, int64_t rs_c, int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const bool ta = GB_IS_TRANS(transa);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, m, rs_c, cs_c, esz, true, &C, s))) return rc;
    Staged& A = bufs.next();
    if (alpha != T(0) && k > 0 && (rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, esz, true, &A, s))) return rc;
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = cherk_dev<T>(uplo, transa, m, k, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs, beta,
                           reinterpret_cast<T*>(C.origin), C.rs, C.cs, slices, s)))
        return rc;
    if ((rc = stage_out(c, m, m, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

template <typename T>
int cher2k_host(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
                int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, T beta, T* c, int64_t rs_c, int64_t cs_c,
                const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, m, rs_c, cs_c, esz, true, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (!(alpha[0] == T(0) && alpha[1] == T(0)) && k > 0) {
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, esz, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? k : m, tb ? m : k, rs_b, cs_b, esz, true, &B, s))) return rc;
    }
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = cher2k_dev<T>(uplo, transa, transb, m, k, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs,
                            reinterpret_cast<const T*>(B.origin), B.rs, B.cs, beta, reinterpret_cast<T*>(C.origin),
                            C.rs, C.cs, slices, s)))
        return rc;
    if ((rc = stage_out(c, m, m, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

// complex gemv: y up (read unless beta == 0) and back, A and x up when
// something is added
template <typename T>
int cgemv_host(int transa, int conjx, int64_t m, int64_t n, const T* alpha, const T* a, int64_t rs_a, int64_t cs_a,
               const T* x, int64_t incx, const T* beta, T* y, int64_t incy, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    const bool tr = GB_IS_TRANS(transa);
    const int64_t my = tr ? n : m, nx = tr ? m : n;
    if (my <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    Staged& Y = bufs.next();
    if ((rc = stage_in(y, my, 1, incy, my, esz, !(beta[0] == T(0) && beta[1] == T(0)), &Y, s))) return rc;
    const T* ad = nullptr;
    const T* xd = nullptr;
    int64_t ars = rs_a, acs = cs_a, xinc = incx;
    if (nx > 0 && !(alpha[0] == T(0) && alpha[1] == T(0))) {
        Staged& A = bufs.next();
        Staged& X = bufs.next();
        if ((rc = stage_in(a, m, n, rs_a, cs_a, esz, true, &A, s))) return rc;
        if ((rc = stage_in(x, nx, 1, incx, nx, esz, true, &X, s))) return rc;
        ad = reinterpret_cast<const T*>(A.origin);
        xd = reinterpret_cast<const T*>(X.origin);
        ars = A.rs;
        acs = A.cs;
        xinc = X.rs;
    }
    if ((rc = cgemv_dev<T>(transa, conjx, m, n, alpha, ad, ars, acs, xd, xinc, beta, reinterpret_cast<T*>(Y.origin),
                           Y.rs, s)))
        return rc;
    if ((rc = stage_out(y, my, 1, incy, my, esz, Y, s))) return rc;
    return finish(s, where);
}

// complex trmm: B up (read unless alpha == 0) and back, A up
template <typename T>
int ctrmm_host(int side, int uplo, int transa, int diag, int64_t m, int64_t n, const T* alpha, const T* a,
               int64_t rs_a, int64_t cs_a, T* b, int64_t rs_b, int64_t cs_b, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const int64_t na = (side == GB_LEFT) ? m : n;
    const bool nz = !(alpha[0] == T(0) && alpha[1] == T(0));
    Staged& B = bufs.next();
    if ((rc = stage_in(b, m, n, rs_b, cs_b, esz, nz, &B, s))) return rc;
    Staged& A = bufs.next();
    if (nz && (rc = stage_in(a, na, na, rs_a, cs_a, esz, true, &A, s))) return rc;
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = ctrmm_dev<T>(side, uplo, transa, diag, m, n, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs,
                           reinterpret_cast<T*>(B.origin), B.rs, B.cs, slices, s)))
        return rc;
    if ((rc = stage_out(b, m, n, rs_b, cs_b, esz, B, s))) return rc;
    return finish(s, where);
}

// complex syrk (b null) / syr2k, the same staging as herk / her2k
template <typename T>
int csyr2k_host(int uplo, int transa, int transb, int64_t m, int64_t k, const T* alpha, const T* a, int64_t rs_a,
                int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c,
                int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, m, rs_c, cs_c, esz, true, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (!(alpha[0] == T(0) && alpha[1] == T(0)) && k > 0) {
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, esz, true, &A, s))) return rc;
        if (b && (rc = stage_in(b, tb ? k : m, tb ? m : k, rs_b, cs_b, esz, true, &B, s))) return rc;
    }
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = csyr2k_dev<T>(uplo, transa, transb, m, k, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs,
                            b ? reinterpret_cast<const T*>(B.origin) : nullptr, B.rs, B.cs, beta,
                            reinterpret_cast<T*>(C.origin), C.rs, C.cs, slices, s)))
        return rc;
    if ((rc = stage_out(c, m, m, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

template <typename T>
int chemm_host(int side, int uplo, int herm, int conja, int transb, int64_t m, int64_t n, const T* alpha, const T* a, int64_t rs_a,
               int64_t cs_a, const T* b, int64_t rs_b, int64_t cs_b, const T* beta, T* c, int64_t rs_c, int64_t cs_c,
               const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const size_t esz = 2 * sizeof(T);
    const int64_t na = (side == GB_LEFT) ? m : n;
    const bool tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, n, rs_c, cs_c, esz, beta[0] != T(0) || beta[1] != T(0), &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (!(alpha[0] == T(0) && alpha[1] == T(0))) {
        if ((rc = stage_in(a, na, na, rs_a, cs_a, esz, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? n : m, tb ? m : n, rs_b, cs_b, esz, true, &B, s))) return rc;
    }
    const int slices = (sizeof(T) == 8) ? level3_slices() : 0;
    if ((rc = chemm_dev<T>(side, uplo, herm, conja, transb, m, n, alpha, reinterpret_cast<const T*>(A.origin), A.rs, A.cs,
                           reinterpret_cast<const T*>(B.origin), B.rs, B.cs, beta, reinterpret_cast<T*>(C.origin),
                           C.rs, C.cs, slices, s)))
        return rc;
    if ((rc = stage_out(c, m, n, rs_c, cs_c, esz, C, s))) return rc;
    return finish(s, where);
}

int trmm3_host(int side, int uplo, int transa, int diag, int transb, int64_t m, int64_t n, double alpha,
               const double* a, int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta,
               double* c, int64_t rs_c, int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0 || n <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const int64_t na = (side == GB_LEFT) ? m : n;
    const bool tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, n, rs_c, cs_c, 8, beta != 0.0, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (alpha != 0.0) {
        if ((rc = stage_in(a, na, na, rs_a, cs_a, 8, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? n : m, tb ? m : n, rs_b, cs_b, 8, true, &B, s))) return rc;
    }
    if ((rc = dtrmm3_dev(side, uplo, transa, diag, transb, m, n, alpha, reinterpret_cast<const double*>(A.origin), A.rs,
                         A.cs, reinterpret_cast<const double*>(B.origin), B.rs, B.cs, beta,
                         reinterpret_cast<double*>(C.origin), C.rs, C.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(c, m, n, rs_c, cs_c, 8, C, s))) return rc;
    return finish(s, where);
}

int syr2k_host(int uplo, int transa, int transb, int64_t m, int64_t k, double alpha, const double* a, int64_t rs_a,
               int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, double beta, double* c, int64_t rs_c,
               int64_t cs_c, const char* where)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (m <= 0) return GB_SUCCESS;
    cudaStream_t s = thread_stream();
    Bufs bufs(s);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    Staged& C = bufs.next();
    if ((rc = stage_in(c, m, m, rs_c, cs_c, 8, true, &C, s))) return rc;
    Staged& A = bufs.next();
    Staged& B = bufs.next();
    if (alpha != 0.0 && k > 0) {
        if ((rc = stage_in(a, ta ? k : m, ta ? m : k, rs_a, cs_a, 8, true, &A, s))) return rc;
        if ((rc = stage_in(b, tb ? k : m, tb ? m : k, rs_b, cs_b, 8, true, &B, s))) return rc;
    }
    if ((rc = dsyr2k_dev(uplo, transa, transb, m, k, alpha, reinterpret_cast<const double*>(A.origin), A.rs, A.cs,
                         reinterpret_cast<const double*>(B.origin), B.rs, B.cs, beta,
                         reinterpret_cast<double*>(C.origin), C.rs, C.cs, level3_slices(), s)))
        return rc;
    if ((rc = stage_out(c, m, m, rs_c, cs_c, 8, C, s))) return rc;
    return finish(s, where);
}

// ---------------------------------------------------------------- BLAS helpers
bool lsame(char a, char b) { return toupper((unsigned char)a) == toupper((unsigned char)b); }

void call_xerbla(const char* name, int info)
{
    gb_f77_int i = info;
    xerbla_(name, &i, 6);
}

int map_trans(char t) { return lsame(t, 'N') ? GB_NO_TRANSPOSE : (lsame(t, 'T') ? GB_TRANSPOSE : GB_CONJ_TRANSPOSE); }

// frame/compat/check/bla_gemm_check.h:37-86
int gemm_check(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc)
{
    const bool nota = lsame(ta, 'N'), notb = lsame(tb, 'N');
    const bool conja = lsame(ta, 'C'), conjb = lsame(tb, 'C');
    const bool tta = lsame(ta, 'T'), ttb = lsame(tb, 'T');
    const int nrowa = nota ? m : k, nrowb = notb ? k : n;
    if (!nota && !conja && !tta) return 1;
    if (!notb && !conjb && !ttb) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (k < 0) return 5;
    if (lda < (nrowa > 1 ? nrowa : 1)) return 8;
    if (ldb < (nrowb > 1 ? nrowb : 1)) return 10;
    if (ldc < (m > 1 ? m : 1)) return 13;
    return 0;
}

// frame/include/bli_blas_macro_defs.h:50-75: BLAS passes element 0 of the
// traversal; BLIS wants the pointer to element 0 with a signed stride.
template <typename T>
const T* blas_vec(const T* x, int64_t n, int64_t inc)
{
    return (inc < 0) ? x + (n - 1) * (-inc) : x;
}

template <typename T>
void gemm_blas(const char* name, const char* transa, const char* transb, const gb_f77_int* m,
               const gb_f77_int* n, const gb_f77_int* k, const T* alpha, const T* a,
               const gb_f77_int* lda, const T* b, const gb_f77_int* ldb, const T* beta, T* c,
               const gb_f77_int* ldc)
{
    const int info = gemm_check(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);
    if (info) {
        call_xerbla(name, info);
        return;
    }
    const int ta = map_trans(*transa), tb = map_trans(*transb);
    const int64_t m0 = *m, n0 = *n, k0 = *k;
    const int64_t rs_a = 1, cs_a = *lda, rs_b = 1, cs_b = *ldb, rs_c = 1, cs_c = *ldc;
    if (sizeof(T) == 8) {
        // m == 1 or n == 1 become gemv (frame/compat/bla_gemm.c:180-218)
        if (n0 == 1) {
            const int64_t m0t = GB_IS_TRANS(ta) ? k0 : m0, k0t = GB_IS_TRANS(ta) ? m0 : k0;
            gemv_host(ta, m0t, k0t, (double)*alpha, (const double*)a, rs_a, cs_a, (const double*)b,
                      GB_IS_TRANS(tb) ? cs_b : rs_b, (double)*beta, (double*)c, rs_c, name);
            return;
        }
        if (m0 == 1) {
            const int64_t n0t = GB_IS_TRANS(tb) ? k0 : n0, k0t = GB_IS_TRANS(tb) ? n0 : k0;
            gemv_host(tb, n0t, k0t, (double)*alpha, (const double*)b, cs_b, rs_b, (const double*)a,
                      GB_IS_TRANS(ta) ? rs_a : cs_a, (double)*beta, (double*)c, cs_c, name);
            return;
        }
    }
    gemm_host<T>(ta, tb, m0, n0, k0, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c, name);
}

// herk / her2k checks (frame/compat/check/bla_herk_check.h:37-77,
// bla_her2k_check.h:37-79): trans N or C only
int herk_check(gb_f77_char uploc, gb_f77_char trans, gb_f77_int m, gb_f77_int k, gb_f77_int lda,
                      gb_f77_int ldb, gb_f77_int ldc, bool two)
{
    const bool lower = lsame(uploc, 'L'), upper = lsame(uploc, 'U');
    const bool nota = lsame(trans, 'N'), conja = lsame(trans, 'C');
    const int nrowa = nota ? m : k;
    if (!lower && !upper) return 1;
    if (!nota && !conja) return 2;
    if (m < 0) return 3;
    if (k < 0) return 4;
    if (lda < (nrowa > 1 ? nrowa : 1)) return 7;
    if (two && ldb < (nrowa > 1 ? nrowa : 1)) return 9;
    if (ldc < (m > 1 ? m : 1)) return two ? 12 : 10;
    return 0;
}

template <typename T, typename C>
void herk_blas(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
                      const T* alpha, const C* a, const gb_f77_int* lda, const T* beta, C* c, const gb_f77_int* ldc,
                      const char* name)
{
    // frame/compat/bla_herk.c:45-130
    const int info = herk_check(*uploc, *trans, *m, *k, *lda, 0, *ldc, false);
    if (info) {
        call_xerbla(sizeof(T) == 8 ? "ZHERK " : "CHERK ", info);
        return;
    }
    // the BLAS early return: nothing to add and C not scaled (the diagonal is left as it is)
    if (*m == 0 || ((*alpha == T(0) || *k == 0) && *beta == T(1))) return;
    cherk_host<T>(lsame(*uploc, 'L') ? GB_LOWER : GB_UPPER, map_trans(*trans), *m, *k, *alpha, &a->real, 1, *lda,
                  *beta, &c->real, 1, *ldc, name);
}

template <typename T, typename C>
void her2k_blas(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
                       const C* alpha, const C* a, const gb_f77_int* lda, const C* b, const gb_f77_int* ldb,
                       const T* beta, C* c, const gb_f77_int* ldc, const char* name)
{
    // frame/compat/bla_her2k.c:45-136
    const int info = herk_check(*uploc, *trans, *m, *k, *lda, *ldb, *ldc, true);
    if (info) {
        call_xerbla(sizeof(T) == 8 ? "ZHER2K" : "CHER2K", info);
        return;
    }
    if (*m == 0 || (((alpha->real == T(0) && alpha->imag == T(0)) || *k == 0) && *beta == T(1))) return;
    const int t = map_trans(*trans);
    cher2k_host<T>(lsame(*uploc, 'L') ? GB_LOWER : GB_UPPER, t, t, *m, *k, &alpha->real, &a->real, 1, *lda,
                   &b->real, 1, *ldb, *beta, &c->real, 1, *ldc, name);
}

// complex gemv (frame/compat/bla_gemv.c:45-143, checks
// frame/compat/check/bla_gemv_check.h:37-75)
template <typename T, typename C>
void cgemv_blas(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const C* alpha, const C* a,
                const gb_f77_int* lda, const C* x, const gb_f77_int* incx, const C* beta, C* y,
                const gb_f77_int* incy, const char* xname, const char* name)
{
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    int info = 0;
    if (!nota && !ta && !conja) info = 1;
    else if (*m < 0) info = 2;
    else if (*n < 0) info = 3;
    else if (*lda < (*m > 1 ? *m : 1)) info = 6;
    else if (*incx == 0) info = 8;
    else if (*incy == 0) info = 11;
    if (info) {
        call_xerbla(xname, info);
        return;
    }
    const int t = map_trans(*transa);
    const int64_t m0 = *m, n0 = *n;
    const int64_t m_y = GB_IS_TRANS(t) ? n0 : m0, n_x = GB_IS_TRANS(t) ? m0 : n0;
    if (m_y > 0 && n_x == 0) return;  // netlib quirk kept by frame/compat/bla_gemv.c:88-106
    cgemv_host<T>(t, 0, m0, n0, &alpha->real, &a->real, 1, *lda, &blas_vec<C>(x, n_x, *incx)->real, *incx,
                  &beta->real, const_cast<T*>(&blas_vec<C>(y, m_y, *incy)->real), *incy, name);
}

// complex trmm (frame/compat/bla_trmm.c:45-121, checks
// frame/compat/check/bla_trmm_check.h:37-86)
template <typename T, typename C>
void ctrmm_blas(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
                const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const C* alpha, const C* a,
                const gb_f77_int* lda, C* b, const gb_f77_int* ldb, const char* xname, const char* name)
{
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla(xname, info);
        return;
    }
    ctrmm_host<T>(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
                  unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, &alpha->real, &a->real, 1, *lda, &b->real, 1, *ldb,
                  name);
}

// complex syrk / syr2k (frame/compat/bla_syrk.c:45-121, bla_syr2k.c:45-128;
// checks frame/compat/check/bla_syrk_check.h:37-84, bla_syr2k_check.h:37-84):
// trans N or T only in the complex domain
template <typename T, typename C>
void csyr2k_blas(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
                 const C* alpha, const C* a, const gb_f77_int* lda, const C* b, const gb_f77_int* ldb,
                 const C* beta, C* c, const gb_f77_int* ldc, const char* xname, const char* name)
{
    const bool two = (b != nullptr);
    const bool lower = lsame(*uploc, 'L'), upper = lsame(*uploc, 'U');
    const bool nota = lsame(*trans, 'N'), ta = lsame(*trans, 'T');
    const int nrowa = nota ? *m : *k;
    int info = 0;
    if (!lower && !upper) info = 1;
    else if (!nota && !ta) info = 2;
    else if (*m < 0) info = 3;
    else if (*k < 0) info = 4;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 7;
    else if (two && *ldb < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldc < (*m > 1 ? *m : 1)) info = two ? 12 : 10;
    if (info) {
        call_xerbla(xname, info);
        return;
    }
    if (*m == 0 || (((alpha->real == T(0) && alpha->imag == T(0)) || *k == 0) && beta->real == T(1) &&
                    beta->imag == T(0)))
        return;
    const int t = nota ? GB_NO_TRANSPOSE : GB_TRANSPOSE;
    csyr2k_host<T>(lower ? GB_LOWER : GB_UPPER, t, t, *m, *k, &alpha->real, &a->real, 1, *lda,
                   two ? &b->real : nullptr, 1, two ? *ldb : 1, &beta->real, &c->real, 1, *ldc, name);
}

template <typename T, typename C>
void hemm_blas(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
                      const C* alpha, const C* a, const gb_f77_int* lda, const C* b, const gb_f77_int* ldb,
                      const C* beta, C* c, const gb_f77_int* ldc, int herm, const char* xname, const char* name)
{
    // frame/compat/bla_hemm.c:45-120 / bla_symm.c:45-120, checks frame/compat/check/bla_hemm_check.h:37-79
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (*m < 0) info = 3;
    else if (*n < 0) info = 4;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 7;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 9;
    else if (*ldc < (*m > 1 ? *m : 1)) info = 12;
    if (info) {
        call_xerbla(xname, info);
        return;
    }
    chemm_host<T>(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, herm, 0, GB_NO_TRANSPOSE, *m, *n,
                  &alpha->real, &a->real, 1, *lda, &b->real, 1, *ldb, &beta->real, &c->real, 1, *ldc, name);
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

// ==================================================================== BLAS
int xerbla_(const gb_f77_char* srname, const gb_f77_int* info, long srname_len)
{
    char buf[16] = {0};
    const long n = (srname_len > 0 && srname_len < 15) ? srname_len : 6;
    for (long i = 0; i < n && srname[i]; ++i) buf[i] = srname[i];
    printf("** On entry to %6s, parameter number %2i had an illegal value\n", buf, (int)*info);
    fflush(stdout);
    gb::set_error(GB_ERR_ARG, buf, "illegal BLAS argument");
    return 0;
}

void dgemm_(const gb_f77_char* transa, const gb_f77_char* transb, const gb_f77_int* m,
            const gb_f77_int* n, const gb_f77_int* k, const double* alpha, const double* a,
            const gb_f77_int* lda, const double* b, const gb_f77_int* ldb, const double* beta,
            double* c, const gb_f77_int* ldc)
{
    gemm_blas<double>("DGEMM ", transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void sgemm_(const gb_f77_char* transa, const gb_f77_char* transb, const gb_f77_int* m,
            const gb_f77_int* n, const gb_f77_int* k, const float* alpha, const float* a,
            const gb_f77_int* lda, const float* b, const gb_f77_int* ldb, const float* beta,
            float* c, const gb_f77_int* ldc)
{
    gemm_blas<float>("SGEMM ", transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void dtrsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const double* alpha,
            const double* a, const gb_f77_int* lda, double* b, const gb_f77_int* ldb)
{
    // frame/compat/check/bla_trmm_check.h:37-86
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla("DTRSM ", info);
        return;
    }
    trsm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
              unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, *alpha, a, 1, *lda, b, 1, *ldb);
}

void strsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const float* alpha,
            const float* a, const gb_f77_int* lda, float* b, const gb_f77_int* ldb)
{
    // the argument checks of dtrsm_ (frame/compat/check/bla_trmm_check.h:37-86)
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla("STRSM ", info);
        return;
    }
    strsm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
               unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, *alpha, a, 1, *lda, b, 1, *ldb, "strsm_");
}

void zgemm_(const gb_f77_char* transa, const gb_f77_char* transb, const gb_f77_int* m, const gb_f77_int* n,
            const gb_f77_int* k, const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda,
            const gb_dcomplex* b, const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c,
            const gb_f77_int* ldc)
{
    // frame/compat/bla_gemm.c:122-262 for dcomplex; checks frame/compat/check/bla_gemm_check.h
    const int info = gemm_check(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);
    if (info) {
        call_xerbla("ZGEMM ", info);
        return;
    }
    cgemm_host<double>(map_trans(*transa), map_trans(*transb), *m, *n, *k, &alpha->real, &a->real, 1, *lda,
                       &b->real, 1, *ldb, &beta->real, &c->real, 1, *ldc, "ZGEMM");
}

void cgemm_(const gb_f77_char* transa, const gb_f77_char* transb, const gb_f77_int* m, const gb_f77_int* n,
            const gb_f77_int* k, const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda,
            const gb_scomplex* b, const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c,
            const gb_f77_int* ldc)
{
    const int info = gemm_check(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);
    if (info) {
        call_xerbla("CGEMM ", info);
        return;
    }
    cgemm_host<float>(map_trans(*transa), map_trans(*transb), *m, *n, *k, &alpha->real, &a->real, 1, *lda,
                      &b->real, 1, *ldb, &beta->real, &c->real, 1, *ldc, "CGEMM");
}

void ztrsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_dcomplex* alpha,
            const gb_dcomplex* a, const gb_f77_int* lda, gb_dcomplex* b, const gb_f77_int* ldb)
{
    // frame/compat/bla_trsm.c:121-219 for dcomplex, checks frame/compat/check/bla_trmm_check.h:37-86
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla("ZTRSM ", info);
        return;
    }
    ztrsm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
               unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, &alpha->real, &a->real, 1, *lda, &b->real, 1, *ldb,
               "ZTRSM");
}

void ctrsm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_scomplex* alpha,
            const gb_scomplex* a, const gb_f77_int* lda, gb_scomplex* b, const gb_f77_int* ldb)
{
    // the argument checks of ztrsm_ (frame/compat/check/bla_trmm_check.h:37-86)
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla("CTRSM ", info);
        return;
    }
    ctrsm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
               unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, &alpha->real, &a->real, 1, *lda, &b->real, 1, *ldb,
               "CTRSM");
}

void zherk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const double* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const double* beta, gb_dcomplex* c,
            const gb_f77_int* ldc)
{
    herk_blas<double, gb_dcomplex>(uploc, trans, m, k, alpha, a, lda, beta, c, ldc, "ZHERK");
}

void cherk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const float* alpha, const gb_scomplex* a, const gb_f77_int* lda, const float* beta, gb_scomplex* c,
            const gb_f77_int* ldc)
{
    herk_blas<float, gb_scomplex>(uploc, trans, m, k, alpha, a, lda, beta, c, ldc, "CHERK");
}

void zher2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
             const gb_f77_int* ldb, const double* beta, gb_dcomplex* c, const gb_f77_int* ldc)
{
    her2k_blas<double, gb_dcomplex>(uploc, trans, m, k, alpha, a, lda, b, ldb, beta, c, ldc, "ZHER2K");
}

void zgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const gb_dcomplex* alpha,
            const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* x, const gb_f77_int* incx,
            const gb_dcomplex* beta, gb_dcomplex* y, const gb_f77_int* incy)
{
    cgemv_blas<double, gb_dcomplex>(transa, m, n, alpha, a, lda, x, incx, beta, y, incy, "ZGEMV ", "ZGEMV");
}

void cgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const gb_scomplex* alpha,
            const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* x, const gb_f77_int* incx,
            const gb_scomplex* beta, gb_scomplex* y, const gb_f77_int* incy)
{
    cgemv_blas<float, gb_scomplex>(transa, m, n, alpha, a, lda, x, incx, beta, y, incy, "CGEMV ", "CGEMV");
}

void ztrmm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_dcomplex* alpha,
            const gb_dcomplex* a, const gb_f77_int* lda, gb_dcomplex* b, const gb_f77_int* ldb)
{
    ctrmm_blas<double, gb_dcomplex>(side, uploa, transa, diaga, m, n, alpha, a, lda, b, ldb, "ZTRMM ", "ZTRMM");
}

void ctrmm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const gb_scomplex* alpha,
            const gb_scomplex* a, const gb_f77_int* lda, gb_scomplex* b, const gb_f77_int* ldb)
{
    ctrmm_blas<float, gb_scomplex>(side, uploa, transa, diaga, m, n, alpha, a, lda, b, ldb, "CTRMM ", "CTRMM");
}

void zsyrk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* beta,
            gb_dcomplex* c, const gb_f77_int* ldc)
{
    csyr2k_blas<double, gb_dcomplex>(uploc, trans, m, k, alpha, a, lda, nullptr, nullptr, beta, c, ldc, "ZSYRK ",
                                     "ZSYRK");
}

void csyrk_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* beta,
            gb_scomplex* c, const gb_f77_int* ldc)
{
    csyr2k_blas<float, gb_scomplex>(uploc, trans, m, k, alpha, a, lda, nullptr, nullptr, beta, c, ldc, "CSYRK ",
                                    "CSYRK");
}

void zsyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
             const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc)
{
    csyr2k_blas<double, gb_dcomplex>(uploc, trans, m, k, alpha, a, lda, b, ldb, beta, c, ldc, "ZSYR2K", "ZSYR2K");
}

void csyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
             const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc)
{
    csyr2k_blas<float, gb_scomplex>(uploc, trans, m, k, alpha, a, lda, b, ldb, beta, c, ldc, "CSYR2K", "CSYR2K");
}

void cher2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
             const gb_f77_int* ldb, const float* beta, gb_scomplex* c, const gb_f77_int* ldc)
{
    her2k_blas<float, gb_scomplex>(uploc, trans, m, k, alpha, a, lda, b, ldb, beta, c, ldc, "CHER2K");
}

void zhemm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
            const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc)
{
    hemm_blas<double, gb_dcomplex>(side, uploa, m, n, alpha, a, lda, b, ldb, beta, c, ldc, 1, "ZHEMM ", "ZHEMM");
}

void chemm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
            const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc)
{
    hemm_blas<float, gb_scomplex>(side, uploa, m, n, alpha, a, lda, b, ldb, beta, c, ldc, 1, "CHEMM ", "CHEMM");
}

void zsymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_dcomplex* alpha, const gb_dcomplex* a, const gb_f77_int* lda, const gb_dcomplex* b,
            const gb_f77_int* ldb, const gb_dcomplex* beta, gb_dcomplex* c, const gb_f77_int* ldc)
{
    hemm_blas<double, gb_dcomplex>(side, uploa, m, n, alpha, a, lda, b, ldb, beta, c, ldc, 0, "ZSYMM ", "ZSYMM");
}

void csymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const gb_scomplex* alpha, const gb_scomplex* a, const gb_f77_int* lda, const gb_scomplex* b,
            const gb_f77_int* ldb, const gb_scomplex* beta, gb_scomplex* c, const gb_f77_int* ldc)
{
    hemm_blas<float, gb_scomplex>(side, uploa, m, n, alpha, a, lda, b, ldb, beta, c, ldc, 0, "CSYMM ", "CSYMM");
}

void dsyr2k_(const gb_f77_char* uploc, const gb_f77_char* trans, const gb_f77_int* m, const gb_f77_int* k,
             const double* alpha, const double* a, const gb_f77_int* lda, const double* b, const gb_f77_int* ldb,
             const double* beta, double* c, const gb_f77_int* ldc)
{
    // frame/compat/bla_syr2k.c:45-128, checks frame/compat/check/bla_syr2k_check.h:37-84 (real: 'C' is 'T')
    const bool lower = lsame(*uploc, 'L'), upper = lsame(*uploc, 'U');
    const bool nota = lsame(*trans, 'N'), ta = lsame(*trans, 'T') || lsame(*trans, 'C');
    const int nrowa = nota ? *m : *k;
    int info = 0;
    if (!lower && !upper) info = 1;
    else if (!nota && !ta) info = 2;
    else if (*m < 0) info = 3;
    else if (*k < 0) info = 4;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 7;
    else if (*ldb < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldc < (*m > 1 ? *m : 1)) info = 12;
    if (info) {
        call_xerbla("DSYR2K", info);
        return;
    }
    const int t = nota ? GB_NO_TRANSPOSE : GB_TRANSPOSE;
    syr2k_host(lower ? GB_LOWER : GB_UPPER, t, t, *m, *k, *alpha, a, 1, *lda, b, 1, *ldb, *beta, c, 1, *ldc,
               "DSYR2K");
}

void dtrmm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_char* transa,
            const gb_f77_char* diaga, const gb_f77_int* m, const gb_f77_int* n, const double* alpha,
            const double* a, const gb_f77_int* lda, double* b, const gb_f77_int* ldb)
{
    // frame/compat/bla_trmm.c:45-121, checks frame/compat/check/bla_trmm_check.h:37-86
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (!nota && !ta && !conja) info = 3;
    else if (!unita && !nonua) info = 4;
    else if (*m < 0) info = 5;
    else if (*n < 0) info = 6;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 9;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 11;
    if (info) {
        call_xerbla("DTRMM ", info);
        return;
    }
    trmm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, map_trans(*transa),
              unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, *n, *alpha, a, 1, *lda, b, 1, *ldb, "DTRMM");
}

void dsymm_(const gb_f77_char* side, const gb_f77_char* uploa, const gb_f77_int* m, const gb_f77_int* n,
            const double* alpha, const double* a, const gb_f77_int* lda, const double* b, const gb_f77_int* ldb,
            const double* beta, double* c, const gb_f77_int* ldc)
{
    // frame/compat/bla_symm.c:45-119, checks frame/compat/check/bla_hemm_check.h:37-79
    const bool left = lsame(*side, 'L'), right = lsame(*side, 'R');
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const int nrowa = left ? *m : *n;
    int info = 0;
    if (!left && !right) info = 1;
    else if (!lower && !upper) info = 2;
    else if (*m < 0) info = 3;
    else if (*n < 0) info = 4;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 7;
    else if (*ldb < (*m > 1 ? *m : 1)) info = 9;
    else if (*ldc < (*m > 1 ? *m : 1)) info = 12;
    if (info) {
        call_xerbla("DSYMM ", info);
        return;
    }
    symm_host(left ? GB_LEFT : GB_RIGHT, lower ? GB_LOWER : GB_UPPER, *m, *n, *alpha, a, 1, *lda, b, 1, *ldb,
              *beta, c, 1, *ldc, "DSYMM");
}

void dsyrk_(const gb_f77_char* uploc, const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* k,
            const double* alpha, const double* a, const gb_f77_int* lda, const double* beta, double* c,
            const gb_f77_int* ldc)
{
    // frame/compat/bla_syrk.c:45-121, checks frame/compat/check/bla_syrk_check.h:37-84 (real: 'C' is 'T')
    const bool lower = lsame(*uploc, 'L'), upper = lsame(*uploc, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T') || lsame(*transa, 'C');
    const int nrowa = nota ? *m : *k;
    int info = 0;
    if (!lower && !upper) info = 1;
    else if (!nota && !ta) info = 2;
    else if (*m < 0) info = 3;
    else if (*k < 0) info = 4;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 7;
    else if (*ldc < (*m > 1 ? *m : 1)) info = 10;
    if (info) {
        call_xerbla("DSYRK ", info);
        return;
    }
    // C := alpha op(A) op(A)^T + beta C (frame/3/bli_l3_oapi_ex.c:326-345)
    const int t = nota ? GB_NO_TRANSPOSE : GB_TRANSPOSE;
    gemmt_host(lower ? GB_LOWER : GB_UPPER, t, nota ? GB_TRANSPOSE : GB_NO_TRANSPOSE, *m, *k, *alpha, a, 1, *lda,
               a, 1, *lda, *beta, c, 1, *ldc, "DSYRK");
}

void dgemmt_(const gb_f77_char* uploc, const gb_f77_char* transa, const gb_f77_char* transb, const gb_f77_int* m,
             const gb_f77_int* k, const double* alpha, const double* a, const gb_f77_int* lda, const double* b,
             const gb_f77_int* ldb, const double* beta, double* c, const gb_f77_int* ldc)
{
    // frame/compat/extra/bla_gemmt.c:45-121, checks frame/compat/check/bla_gemmt_check.h:37-92
    const bool lower = lsame(*uploc, 'L'), upper = lsame(*uploc, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool notb = lsame(*transb, 'N'), tb = lsame(*transb, 'T'), conjb = lsame(*transb, 'C');
    const int nrowa = nota ? *m : *k, nrowb = notb ? *k : *m;
    int info = 0;
    if (!lower && !upper) info = 1;
    else if (!nota && !conja && !ta) info = 2;
    else if (!notb && !conjb && !tb) info = 3;
    else if (*m < 0) info = 4;
    else if (*k < 0) info = 5;
    else if (*lda < (nrowa > 1 ? nrowa : 1)) info = 8;
    else if (*ldb < (nrowb > 1 ? nrowb : 1)) info = 10;
    else if (*ldc < (*m > 1 ? *m : 1)) info = 13;
    if (info) {
        call_xerbla("DGEMMT", info);
        return;
    }
    gemmt_host(lower ? GB_LOWER : GB_UPPER, map_trans(*transa), map_trans(*transb), *m, *k, *alpha, a, 1, *lda, b,
               1, *ldb, *beta, c, 1, *ldc, "DGEMMT");
}

void dgemv_(const gb_f77_char* transa, const gb_f77_int* m, const gb_f77_int* n, const double* alpha,
            const double* a, const gb_f77_int* lda, const double* x, const gb_f77_int* incx,
            const double* beta, double* y, const gb_f77_int* incy)
{
    // frame/compat/check/bla_gemv_check.h:37-75
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    int info = 0;
    if (!nota && !ta && !conja) info = 1;
    else if (*m < 0) info = 2;
    else if (*n < 0) info = 3;
    else if (*lda < (*m > 1 ? *m : 1)) info = 6;
    else if (*incx == 0) info = 8;
    else if (*incy == 0) info = 11;
    if (info) {
        call_xerbla("DGEMV ", info);
        return;
    }
    const int t = map_trans(*transa);
    const int64_t m0 = *m, n0 = *n;
    const int64_t m_y = GB_IS_TRANS(t) ? n0 : m0, n_x = GB_IS_TRANS(t) ? m0 : n0;
    if (m_y > 0 && n_x == 0) return;  // netlib quirk kept by frame/compat/bla_gemv.c:88-106
    gemv_host(t, m0, n0, *alpha, a, 1, *lda, blas_vec(x, n_x, *incx), *incx, *beta,
              const_cast<double*>(blas_vec<double>(y, m_y, *incy)), *incy, "DGEMV ");
}

void dscal_(const gb_f77_int* n, const double* alpha, double* x, const gb_f77_int* incx)
{
    // frame/compat/bla_scal.c:44-85: no argument checks; negative increments by pointer
    const int64_t n0 = (*n > 0) ? *n : 0;
    scalv_host(n0, *alpha, const_cast<double*>(blas_vec<double>(x, n0, *incx)), *incx, "DSCAL");
}

void dcopy_(const gb_f77_int* n, const double* x, const gb_f77_int* incx, double* y, const gb_f77_int* incy)
{
    // frame/compat/bla_copy.c:44-81
    const int64_t n0 = (*n > 0) ? *n : 0;
    copyv_host(n0, blas_vec(x, n0, *incx), *incx, const_cast<double*>(blas_vec<double>(y, n0, *incy)), *incy,
               "DCOPY");
}

gb_f77_int idamax_(const gb_f77_int* n, const double* x, const gb_f77_int* incx)
{
    // frame/compat/bla_amax.c:44-91: empty vector or non-positive increment -> 0, else 1-based
    if (*n < 1 || *incx <= 0) return 0;
    int64_t idx = 0;
    if (amaxv_host(*n, x, *incx, &idx, "IDAMAX")) return 0;
    return (gb_f77_int)(idx + 1);
}

void dger_(const gb_f77_int* m, const gb_f77_int* n, const double* alpha, const double* x, const gb_f77_int* incx,
           const double* y, const gb_f77_int* incy, double* a, const gb_f77_int* lda)
{
    // frame/compat/bla_ger.c:44-106, checks frame/compat/check/bla_ger_check.h:37-68
    int info = 0;
    if (*m < 0) info = 1;
    else if (*n < 0) info = 2;
    else if (*incx == 0) info = 5;
    else if (*incy == 0) info = 7;
    else if (*lda < (*m > 1 ? *m : 1)) info = 9;
    if (info) {
        call_xerbla("DGER  ", info);
        return;
    }
    ger_host(*m, *n, *alpha, blas_vec(x, *m, *incx), *incx, blas_vec(y, *n, *incy), *incy, a, 1, *lda, "DGER");
}

void dtrsv_(const gb_f77_char* uploa, const gb_f77_char* transa, const gb_f77_char* diaga, const gb_f77_int* m,
            const double* a, const gb_f77_int* lda, double* x, const gb_f77_int* incx)
{
    // frame/compat/bla_trsv.c:44-113, checks frame/compat/check/bla_trmv_check.h:37-77
    const bool lower = lsame(*uploa, 'L'), upper = lsame(*uploa, 'U');
    const bool nota = lsame(*transa, 'N'), ta = lsame(*transa, 'T'), conja = lsame(*transa, 'C');
    const bool unita = lsame(*diaga, 'U'), nonua = lsame(*diaga, 'N');
    int info = 0;
    if (!lower && !upper) info = 1;
    else if (!nota && !ta && !conja) info = 2;
    else if (!unita && !nonua) info = 3;
    else if (*m < 0) info = 4;
    else if (*lda < (*m > 1 ? *m : 1)) info = 6;
    else if (*incx == 0) info = 8;
    if (info) {
        call_xerbla("DTRSV ", info);
        return;
    }
    trsv_host(lower ? GB_LOWER : GB_UPPER, map_trans(*transa), unita ? GB_UNIT_DIAG : GB_NONUNIT_DIAG, *m, 1.0, a,
              1, *lda, const_cast<double*>(blas_vec<double>(x, *m, *incx)), *incx, "DTRSV");
}

void daxpy_(const gb_f77_int* n, const double* alpha, const double* x, const gb_f77_int* incx,
            double* y, const gb_f77_int* incy)
{
    const int64_t n0 = (*n > 0) ? *n : 0;
    axpyv_host(n0, *alpha, blas_vec(x, n0, *incx), *incx,
               const_cast<double*>(blas_vec<double>(y, n0, *incy)), *incy);
}

double ddot_(const gb_f77_int* n, const double* x, const gb_f77_int* incx, const double* y,
             const gb_f77_int* incy)
{
    const int64_t n0 = (*n > 0) ? *n : 0;
    double rho = 0.0;
    dotv_host(n0, blas_vec(x, n0, *incx), *incx, blas_vec(y, n0, *incy), *incy, &rho);
    return rho;
}

// ==================================================================== CBLAS
static char cblas_trans_char(int t)
{
    return t == GbCblasNoTrans ? 'N' : (t == GbCblasTrans ? 'T' : (t == GbCblasConjTrans ? 'C' : '?'));
}

void cblas_dgemm(int order, int transa, int transb, gb_f77_int m, gb_f77_int n, gb_f77_int k,
                 double alpha, const double* a, gb_f77_int lda, const double* b, gb_f77_int ldb,
                 double beta, double* c, gb_f77_int ldc)
{
    char ta = cblas_trans_char(transa), tb = cblas_trans_char(transb);
    if (order == GbCblasColMajor) {
        dgemm_(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
    } else if (order == GbCblasRowMajor) {
        // row-major C = A B is column-major C^T = B^T A^T (cblas_dgemm.c:73-103)
        dgemm_(&tb, &ta, &n, &m, &k, &alpha, b, &ldb, a, &lda, &beta, c, &ldc);
    } else {
        call_xerbla("cblas_dgemm", 1);
    }
}

void cblas_sgemm(int order, int transa, int transb, gb_f77_int m, gb_f77_int n, gb_f77_int k,
                 float alpha, const float* a, gb_f77_int lda, const float* b, gb_f77_int ldb,
                 float beta, float* c, gb_f77_int ldc)
{
    char ta = cblas_trans_char(transa), tb = cblas_trans_char(transb);
    if (order == GbCblasColMajor) sgemm_(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
    else if (order == GbCblasRowMajor) sgemm_(&tb, &ta, &n, &m, &k, &alpha, b, &ldb, a, &lda, &beta, c, &ldc);
    else call_xerbla("cblas_sgemm", 1);
}

void cblas_dtrsm(int order, int side, int uplo, int transa, int diag, gb_f77_int m, gb_f77_int n,
                 double alpha, const double* a, gb_f77_int lda, double* b, gb_f77_int ldb)
{
    char sd = side == GbCblasLeft ? 'L' : (side == GbCblasRight ? 'R' : '?');
    char ul = uplo == GbCblasUpper ? 'U' : (uplo == GbCblasLower ? 'L' : '?');
    char ta = cblas_trans_char(transa);
    char dg = diag == GbCblasUnit ? 'U' : (diag == GbCblasNonUnit ? 'N' : '?');
    if (order == GbCblasColMajor) {
        dtrsm_(&sd, &ul, &ta, &dg, &m, &n, &alpha, a, &lda, b, &ldb);
    } else if (order == GbCblasRowMajor) {
        // row-major: swap side and uplo, swap m and n (cblas_dtrsm.c)
        char sd2 = (sd == 'L') ? 'R' : (sd == 'R' ? 'L' : '?');
        char ul2 = (ul == 'U') ? 'L' : (ul == 'L' ? 'U' : '?');
        dtrsm_(&sd2, &ul2, &ta, &dg, &n, &m, &alpha, a, &lda, b, &ldb);
    } else {
        call_xerbla("cblas_dtrsm", 1);
    }
}

void cblas_dgemv(int order, int transa, gb_f77_int m, gb_f77_int n, double alpha, const double* a,
                 gb_f77_int lda, const double* x, gb_f77_int incx, double beta, double* y,
                 gb_f77_int incy)
{
    char ta = cblas_trans_char(transa);
    if (order == GbCblasColMajor) {
        dgemv_(&ta, &m, &n, &alpha, a, &lda, x, &incx, &beta, y, &incy);
    } else if (order == GbCblasRowMajor) {
        char t2 = (ta == 'N') ? 'T' : 'N';
        dgemv_(&t2, &n, &m, &alpha, a, &lda, x, &incx, &beta, y, &incy);
    } else {
        call_xerbla("cblas_dgemv", 1);
    }
}

void cblas_daxpy(gb_f77_int n, double alpha, const double* x, gb_f77_int incx, double* y, gb_f77_int incy)
{
    daxpy_(&n, &alpha, x, &incx, y, &incy);
}

double cblas_ddot(gb_f77_int n, const double* x, gb_f77_int incx, const double* y, gb_f77_int incy)
{
    return ddot_(&n, x, &incx, y, &incy);
}

// ==================================================================== typed BLIS API
void bli_dgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c,
               gb_inc_t cs_c)
{
    gemm_host<double>(transa, transb, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c,
                      cs_c, "bli_dgemm");
}

void bli_dgemm_ex(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                  const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  const double* b, gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c,
                  gb_inc_t rs_c, gb_inc_t cs_c, const void* cntx, const void* rntm)
{
    (void)cntx;
    (void)rntm;
    bli_dgemm(transa, transb, m, n, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c);
}

void bli_sgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
               const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a, const float* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const float* beta, float* c, gb_inc_t rs_c,
               gb_inc_t cs_c)
{
    gemm_host<float>(transa, transb, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c,
                     cs_c, "bli_sgemm");
}

void bli_dtrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
               double* b, gb_inc_t rs_b, gb_inc_t cs_b)
{
    trsm_host(side, uploa, transa, diaga, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b);
}

void bli_strsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
               gb_dim_t n, const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a,
               float* b, gb_inc_t rs_b, gb_inc_t cs_b)
{
    strsm_host(side, uploa, transa, diaga, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, "bli_strsm");
}

void bli_dtrsm_ex(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                  gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
                  double* b, gb_inc_t rs_b, gb_inc_t cs_b, const void* cntx, const void* rntm)
{
    (void)cntx;
    (void)rntm;
    bli_dtrsm(side, uploa, transa, diaga, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b);
}

void bli_zgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, const gb_dcomplex* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b, gb_inc_t rs_b,
               gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cgemm_host<double>(transa, transb, m, n, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                       &beta->real, &c->real, rs_c, cs_c, "bli_zgemm");
}

void bli_cgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, const gb_scomplex* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b, gb_inc_t rs_b,
               gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cgemm_host<float>(transa, transb, m, n, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                      &beta->real, &c->real, rs_c, cs_c, "bli_cgemm");
}

void bli_ztrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b)
{
    ztrsm_host(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
               "bli_ztrsm");
}

void bli_ctrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b)
{
    ctrsm_host(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
               "bli_ctrsm");
}

// frame/3/bli_l3_tapi_ex.c herk / her2k / hemm / symm / syr2k (prototypes
// frame/3/bli_l3_tapi_ex.h:62-168)
void bli_zgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const gb_dcomplex* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* x, gb_inc_t incx,
               const gb_dcomplex* beta, gb_dcomplex* y, gb_inc_t incy)
{
    cgemv_host<double>(transa, conjx == GB_CONJUGATE, m, n, &alpha->real, &a->real, rs_a, cs_a, &x->real, incx,
                       &beta->real, &y->real, incy, "bli_zgemv");
}

void bli_cgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const gb_scomplex* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* x, gb_inc_t incx,
               const gb_scomplex* beta, gb_scomplex* y, gb_inc_t incy)
{
    cgemv_host<float>(transa, conjx == GB_CONJUGATE, m, n, &alpha->real, &a->real, rs_a, cs_a, &x->real, incx,
                      &beta->real, &y->real, incy, "bli_cgemv");
}

void bli_ztrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b)
{
    ctrmm_host<double>(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                       "bli_ztrmm");
}

void bli_ctrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b)
{
    ctrmm_host<float>(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                      "bli_ctrmm");
}

void bli_zsyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const gb_dcomplex* alpha,
               const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* beta, gb_dcomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c)
{
    csyr2k_host<double>(uploc, transa, transa, m, k, &alpha->real, &a->real, rs_a, cs_a, nullptr, 1, 1, &beta->real,
                        &c->real, rs_c, cs_c, "bli_zsyrk");
}

void bli_csyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const gb_scomplex* alpha,
               const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* beta, gb_scomplex* c,
               gb_inc_t rs_c, gb_inc_t cs_c)
{
    csyr2k_host<float>(uploc, transa, transa, m, k, &alpha->real, &a->real, rs_a, cs_a, nullptr, 1, 1, &beta->real,
                       &c->real, rs_c, cs_c, "bli_csyrk");
}

void bli_zsyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    csyr2k_host<double>(uploc, transa, transb, m, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                        &beta->real, &c->real, rs_c, cs_c, "bli_zsyr2k");
}

void bli_csyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    csyr2k_host<float>(uploc, transa, transb, m, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                       &beta->real, &c->real, rs_c, cs_c, "bli_csyr2k");
}

void bli_zherk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const double* alpha, const gb_dcomplex* a,
               gb_inc_t rs_a, gb_inc_t cs_a, const double* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cherk_host<double>(uploc, transa, m, k, *alpha, &a->real, rs_a, cs_a, *beta, &c->real, rs_c, cs_c, "bli_zherk");
}

void bli_cherk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const float* alpha, const gb_scomplex* a,
               gb_inc_t rs_a, gb_inc_t cs_a, const float* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cherk_host<float>(uploc, transa, m, k, *alpha, &a->real, rs_a, cs_a, *beta, &c->real, rs_c, cs_c, "bli_cherk");
}

void bli_zher2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cher2k_host<double>(uploc, transa, transb, m, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b, *beta,
                        &c->real, rs_c, cs_c, "bli_zher2k");
}

void bli_cher2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k,
                const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const float* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cher2k_host<float>(uploc, transa, transb, m, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b, *beta,
                       &c->real, rs_c, cs_c, "bli_cher2k");
}

void bli_zhemm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    chemm_host<double>(side, uploa, 1, conja == GB_CONJUGATE, transb, m, n, &alpha->real, &a->real, rs_a, cs_a,
                       &b->real, rs_b, cs_b, &beta->real, &c->real, rs_c, cs_c, "bli_zhemm");
}

void bli_chemm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    chemm_host<float>(side, uploa, 1, conja == GB_CONJUGATE, transb, m, n, &alpha->real, &a->real, rs_a, cs_a,
                      &b->real, rs_b, cs_b, &beta->real, &c->real, rs_c, cs_c, "bli_chemm");
}

void bli_zsymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    chemm_host<double>(side, uploa, 0, conja == GB_CONJUGATE, transb, m, n, &alpha->real, &a->real, rs_a, cs_a,
                       &b->real, rs_b, cs_b, &beta->real, &c->real, rs_c, cs_c, "bli_zsymm");
}

void bli_csymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b,
               gb_inc_t rs_b, gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    chemm_host<float>(side, uploa, 0, conja == GB_CONJUGATE, transb, m, n, &alpha->real, &a->real, rs_a, cs_a,
                      &b->real, rs_b, cs_b, &beta->real, &c->real, rs_c, cs_c, "bli_csymm");
}

void bli_dtrmm3(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_trans_t transb, gb_dim_t m,
                gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    trmm3_host(side, uploa, transa, diaga, transb, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c,
               "bli_dtrmm3");
}

void bli_dsyr2k(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, const double* alpha,
                const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    syr2k_host(uploc, transa, transb, m, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c, "bli_dsyr2k");
}

void bli_dscalv(gb_conj_t conjalpha, gb_dim_t n, const double* alpha, double* x, gb_inc_t incx)
{
    (void)conjalpha;  // real
    scalv_host(n, *alpha, x, incx, "bli_dscalv");
}

void bli_dcopyv(gb_conj_t conjx, gb_dim_t n, const double* x, gb_inc_t incx, double* y, gb_inc_t incy)
{
    (void)conjx;
    copyv_host(n, x, incx, y, incy, "bli_dcopyv");
}

void bli_damaxv(gb_dim_t n, const double* x, gb_inc_t incx, gb_dim_t* index)
{
    int64_t idx = 0;
    amaxv_host(n, x, incx, &idx, "bli_damaxv");
    *index = idx;
}

void bli_dger(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t m, gb_dim_t n, const double* alpha, const double* x,
              gb_inc_t incx, const double* y, gb_inc_t incy, double* a, gb_inc_t rs_a, gb_inc_t cs_a)
{
    (void)conjx;
    (void)conjy;
    ger_host(m, n, *alpha, x, incx, y, incy, a, rs_a, cs_a, "bli_dger");
}

void bli_dtrsv(gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, const double* alpha, const double* a,
               gb_inc_t rs_a, gb_inc_t cs_a, double* x, gb_inc_t incx)
{
    trsv_host(uploa, transa, diaga, m, *alpha, a, rs_a, cs_a, x, incx, "bli_dtrsv");
}

void bli_dtrmm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* b, gb_inc_t rs_b,
               gb_inc_t cs_b)
{
    trmm_host(side, uploa, transa, diaga, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, "bli_dtrmm");
}

void bli_dsymm(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
               const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b,
               gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    (void)conja;  // real: conjugation is the identity
    // op(B) by its strides: B^T (element (i, j) at b[j*rs_b + i*cs_b])
    const bool tb = GB_IS_TRANS(transb);
    symm_host(side, uploa, m, n, *alpha, a, rs_a, cs_a, b, tb ? cs_b : rs_b, tb ? rs_b : cs_b, *beta, c, rs_c,
              cs_c, "bli_dsymm");
}

void bli_dsyrk(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, const double* alpha, const double* a,
               gb_inc_t rs_a, gb_inc_t cs_a, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    const bool ta = GB_IS_TRANS(transa);
    gemmt_host(uploc, ta ? GB_TRANSPOSE : GB_NO_TRANSPOSE, ta ? GB_NO_TRANSPOSE : GB_TRANSPOSE, m, k, *alpha, a,
               rs_a, cs_a, a, rs_a, cs_a, *beta, c, rs_c, cs_c, "bli_dsyrk");
}

void bli_dgemmt(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, const double* alpha,
                const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    gemmt_host(uploc, transa, transb, m, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c,
               "bli_dgemmt");
}

void bli_dgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const double* alpha,
               const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* x, gb_inc_t incx,
               const double* beta, double* y, gb_inc_t incy)
{
    (void)conjx;
    gemv_host(transa, m, n, *alpha, a, rs_a, cs_a, x, incx, *beta, y, incy, "bli_dgemv");
}

void bli_dgemv_ex(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const double* alpha,
                  const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* x, gb_inc_t incx,
                  const double* beta, double* y, gb_inc_t incy, const void* cntx, const void* rntm)
{
    (void)cntx;
    (void)rntm;
    bli_dgemv(transa, conjx, m, n, alpha, a, rs_a, cs_a, x, incx, beta, y, incy);
}

void bli_daxpyv(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x, gb_inc_t incx,
                double* y, gb_inc_t incy)
{
    (void)conjx;
    axpyv_host(n, *alpha, x, incx, y, incy);
}

void bli_daxpyv_ex(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x, gb_inc_t incx,
                   double* y, gb_inc_t incy, const void* cntx, const void* rntm)
{
    (void)cntx;
    (void)rntm;
    bli_daxpyv(conjx, n, alpha, x, incx, y, incy);
}

void bli_ddotv(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x, gb_inc_t incx,
               const double* y, gb_inc_t incy, double* rho)
{
    (void)conjx;
    (void)conjy;
    dotv_host(n, x, incx, y, incy, rho);
}

void bli_ddotv_ex(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x, gb_inc_t incx,
                  const double* y, gb_inc_t incy, double* rho, const void* cntx, const void* rntm)
{
    (void)cntx;
    (void)rntm;
    bli_ddotv(conjx, conjy, n, x, incx, y, incy, rho);
}

// ==================================================================== gb_ host aliases
void gb_dgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
              gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    gemm_host<double>(transa, transb, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c,
                      cs_c, "gb_dgemm");
}

void gb_dgemm_ozaki(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                    const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                    gb_inc_t rs_b, gb_inc_t cs_b, const double* beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c,
                    int slices)
{
    gb::ModeOverride form(GB_DGEMM_OZAKI, slices < 0 ? 0 : slices);
    gemm_host<double>(transa, transb, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c,
                      "gb_dgemm_ozaki");
}

void gb_zgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, const gb_dcomplex* alpha,
              const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b, gb_inc_t rs_b,
              gb_inc_t cs_b, const gb_dcomplex* beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cgemm_host<double>(transa, transb, m, n, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                       &beta->real, &c->real, rs_c, cs_c, "gb_zgemm");
}

void gb_cgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, const gb_scomplex* alpha,
              const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b, gb_inc_t rs_b,
              gb_inc_t cs_b, const gb_scomplex* beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    cgemm_host<float>(transa, transb, m, n, k, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                      &beta->real, &c->real, rs_c, cs_c, "gb_cgemm");
}

void gb_sgemm(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
              const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a, const float* b,
              gb_inc_t rs_b, gb_inc_t cs_b, const float* beta, float* c, gb_inc_t rs_c, gb_inc_t cs_c)
{
    gemm_host<float>(transa, transb, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c,
                     cs_c, "gb_sgemm");
}

void gb_dtrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
              gb_dim_t n, const double* alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a,
              double* b, gb_inc_t rs_b, gb_inc_t cs_b)
{
    trsm_host(side, uploa, transa, diaga, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b);
}

void gb_strsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
              gb_dim_t n, const float* alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a,
              float* b, gb_inc_t rs_b, gb_inc_t cs_b)
{
    strsm_host(side, uploa, transa, diaga, m, n, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, "gb_strsm");
}

void gb_ztrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
              const gb_dcomplex* alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
              gb_inc_t rs_b, gb_inc_t cs_b)
{
    ztrsm_host(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
               "gb_ztrsm");
}

void gb_ctrsm(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
              const gb_scomplex* alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
              gb_inc_t rs_b, gb_inc_t cs_b)
{
    ctrsm_host(side, uploa, transa, diaga, m, n, &alpha->real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
               "gb_ctrsm");
}

void gb_dgemv(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, const double* alpha,
              const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* x, gb_inc_t incx,
              const double* beta, double* y, gb_inc_t incy)
{
    (void)conjx;
    gemv_host(transa, m, n, *alpha, a, rs_a, cs_a, x, incx, *beta, y, incy, "gb_dgemv");
}

void gb_daxpyv(gb_conj_t conjx, gb_dim_t n, const double* alpha, const double* x, gb_inc_t incx,
               double* y, gb_inc_t incy)
{
    (void)conjx;
    axpyv_host(n, *alpha, x, incx, y, incy);
}

void gb_ddotv(gb_conj_t conjx, gb_conj_t conjy, gb_dim_t n, const double* x, gb_inc_t incx,
              const double* y, gb_inc_t incy, double* rho)
{
    (void)conjx;
    (void)conjy;
    dotv_host(n, x, incx, y, incy, rho);
}

// ==================================================================== gb_ addon
static cudaStream_t pick_stream(void* stream)
{
    return stream ? static_cast<cudaStream_t>(stream) : gb::thread_stream();
}

int gb_dgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c,
                 gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_dgemm_dev", "negative dimension");
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    // a configuration the selector already decided for this shape, else the occupancy rule (a
    // device entry point never waits for an inference)
    int cfg = gb::selector_auto() ? gb::selector_cached_config(0, m, n, k, ta, tb, 0) : -1;
    if (cfg < 0) cfg = gb::selector_heuristic(m, n, k);
    return gb::gemm_config_dev(0, cfg, m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b,
                               tb ? rs_b : cs_b, beta, c, rs_c, cs_c, pick_stream(stream));
}

int gb_dgemm_ozaki_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                       double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                       gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c,
                       gb_inc_t cs_c, int slices, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_dgemm_ozaki_dev", "negative dimension");
    // the digit form at `slices` slices whatever form gb_set_dgemm_mode chose for the host entry
    // points (the CRT form has its own entry point)
    gb::ModeOverride form(GB_DGEMM_OZAKI, slices, 0);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    return gb::dgemm_ozaki_blocks(m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b,
                                  tb ? rs_b : cs_b, beta, c, rs_c, cs_c, slices, pick_stream(stream));
}

int gb_dgemm_ozaki_crt_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                           double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                           gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c,
                           gb_inc_t cs_c, int moduli, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_dgemm_ozaki_crt_dev", "negative dimension");
    if (moduli < 2 || moduli > 16) return gb::set_error(GB_ERR_ARG, "gb_dgemm_ozaki_crt_dev", "moduli must be in [2, 16]");
    gb::ModeOverride form(GB_DGEMM_OZAKI, moduli, 1);
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    return gb::dgemm_ozaki_blocks(m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b,
                                  tb ? rs_b : cs_b, beta, c, rs_c, cs_c, moduli, pick_stream(stream));
}

int gb_sgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k,
                 float alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a, const float* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, float beta, float* c, gb_inc_t rs_c, gb_inc_t cs_c,
                 void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_sgemm_dev", "negative dimension");
    const bool ta = GB_IS_TRANS(transa), tb = GB_IS_TRANS(transb);
    if (gb::sgemm_use_split(m, n, k))
        return gb::sgemm_split_dev(m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b,
                                   tb ? rs_b : cs_b, beta, c, rs_c, cs_c, pick_stream(stream));
    int cfg = gb::selector_auto() ? gb::selector_cached_config(1, m, n, k, ta, tb, 0) : -1;
    if (cfg < 0) cfg = gb::selector_heuristic(m, n, k);
    return gb::gemm_config_dev(1, cfg, m, n, k, alpha, a, ta ? cs_a : rs_a, ta ? rs_a : cs_a, b, tb ? cs_b : rs_b,
                               tb ? rs_b : cs_b, beta, c, rs_c, cs_c, pick_stream(stream));
}

int gb_dtrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                 gb_dim_t n, double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_dtrsm_dev", "negative dimension");
    const int slices = (gb::dgemm_mode() == GB_DGEMM_OZAKI) ? gb::ozaki_slices() : 0;
    return gb::dtrsm_dev(side, uploa, transa, diaga, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, slices,
                         pick_stream(stream));
}

int gb_strsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m,
                 gb_dim_t n, float alpha, const float* a, gb_inc_t rs_a, gb_inc_t cs_a, float* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_strsm_dev", "negative dimension");
    return gb::strsm_dev(side, uploa, transa, diaga, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, pick_stream(stream));
}

int gb_zgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, gb_dcomplex alpha,
                 const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_zgemm_dev", "negative dimension");
    return gb::cgemm_dev<double>(transa, transb, m, n, k, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                                 &beta.real, &c->real, rs_c, cs_c, gb::level3_slices(), pick_stream(stream));
}

int gb_cgemm_dev(gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t n, gb_dim_t k, gb_scomplex alpha,
                 const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, gb_scomplex beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_cgemm_dev", "negative dimension");
    return gb::cgemm_dev<float>(transa, transb, m, n, k, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                                &beta.real, &c->real, rs_c, cs_c, 0, pick_stream(stream));
}

int gb_ztrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_ztrsm_dev", "negative dimension");
    return gb::ztrsm_dev(side, uploa, transa, diaga, m, n, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                         gb::level3_slices(), pick_stream(stream));
}

int gb_ctrsm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_ctrsm_dev", "negative dimension");
    return gb::ctrsm_dev(side, uploa, transa, diaga, m, n, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                         pick_stream(stream));
}

int gb_zgemv_dev(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, gb_dcomplex alpha, const gb_dcomplex* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* x, gb_inc_t incx, gb_dcomplex beta, gb_dcomplex* y,
                 gb_inc_t incy, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_zgemv_dev", "negative dimension");
    return gb::cgemv_dev<double>(transa, conjx == GB_CONJUGATE, m, n, &alpha.real, &a->real, rs_a, cs_a, &x->real,
                                 incx, &beta.real, &y->real, incy, pick_stream(stream));
}

int gb_cgemv_dev(gb_trans_t transa, gb_conj_t conjx, gb_dim_t m, gb_dim_t n, gb_scomplex alpha, const gb_scomplex* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* x, gb_inc_t incx, gb_scomplex beta, gb_scomplex* y,
                 gb_inc_t incy, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_cgemv_dev", "negative dimension");
    return gb::cgemv_dev<float>(transa, conjx == GB_CONJUGATE, m, n, &alpha.real, &a->real, rs_a, cs_a, &x->real,
                                incx, &beta.real, &y->real, incy, pick_stream(stream));
}

int gb_ztrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_ztrmm_dev", "negative dimension");
    return gb::ctrmm_dev<double>(side, uploa, transa, diaga, m, n, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b,
                                 cs_b, gb::level3_slices(), pick_stream(stream));
}

int gb_ctrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 gb_scomplex alpha, const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_ctrmm_dev", "negative dimension");
    return gb::ctrmm_dev<float>(side, uploa, transa, diaga, m, n, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b,
                                cs_b, 0, pick_stream(stream));
}

int gb_zsyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, gb_dcomplex alpha, const gb_dcomplex* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                 void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_zsyrk_dev", "negative dimension");
    return gb::csyr2k_dev<double>(uploc, transa, transa, m, k, &alpha.real, &a->real, rs_a, cs_a, nullptr, 1, 1,
                                  &beta.real, &c->real, rs_c, cs_c, gb::level3_slices(), pick_stream(stream));
}

int gb_csyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, gb_scomplex alpha, const gb_scomplex* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, gb_scomplex beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                 void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_csyrk_dev", "negative dimension");
    return gb::csyr2k_dev<float>(uploc, transa, transa, m, k, &alpha.real, &a->real, rs_a, cs_a, nullptr, 1, 1,
                                 &beta.real, &c->real, rs_c, cs_c, 0, pick_stream(stream));
}

int gb_zsyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, gb_dcomplex alpha,
                  const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b, gb_inc_t rs_b,
                  gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_zsyr2k_dev", "negative dimension");
    return gb::csyr2k_dev<double>(uploc, transa, transb, m, k, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b,
                                  cs_b, &beta.real, &c->real, rs_c, cs_c, gb::level3_slices(), pick_stream(stream));
}

int gb_csyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, gb_scomplex alpha,
                  const gb_scomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_scomplex* b, gb_inc_t rs_b,
                  gb_inc_t cs_b, gb_scomplex beta, gb_scomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_csyr2k_dev", "negative dimension");
    return gb::csyr2k_dev<float>(uploc, transa, transb, m, k, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                                 &beta.real, &c->real, rs_c, cs_c, 0, pick_stream(stream));
}

int gb_zherk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, double alpha, const gb_dcomplex* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, double beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_zherk_dev", "negative dimension");
    return gb::cherk_dev<double>(uploc, transa, m, k, alpha, &a->real, rs_a, cs_a, beta, &c->real, rs_c, cs_c,
                                 gb::level3_slices(), pick_stream(stream));
}

int gb_zher2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, gb_dcomplex alpha,
                  const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b, gb_inc_t rs_b,
                  gb_inc_t cs_b, double beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_zher2k_dev", "negative dimension");
    return gb::cher2k_dev<double>(uploc, transa, transb, m, k, &alpha.real, &a->real, rs_a, cs_a, &b->real, rs_b, cs_b,
                                  beta, &c->real, rs_c, cs_c, gb::level3_slices(), pick_stream(stream));
}

int gb_zhemm_dev(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                 void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_zhemm_dev", "negative dimension");
    return gb::chemm_dev<double>(side, uploa, 1, conja == GB_CONJUGATE, transb, m, n, &alpha.real, &a->real, rs_a,
                                 cs_a, &b->real, rs_b, cs_b, &beta.real, &c->real, rs_c, cs_c, gb::level3_slices(),
                                 pick_stream(stream));
}

int gb_zsymm_dev(gb_side_t side, gb_uplo_t uploa, gb_conj_t conja, gb_trans_t transb, gb_dim_t m, gb_dim_t n,
                 gb_dcomplex alpha, const gb_dcomplex* a, gb_inc_t rs_a, gb_inc_t cs_a, const gb_dcomplex* b,
                 gb_inc_t rs_b, gb_inc_t cs_b, gb_dcomplex beta, gb_dcomplex* c, gb_inc_t rs_c, gb_inc_t cs_c,
                 void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_zsymm_dev", "negative dimension");
    return gb::chemm_dev<double>(side, uploa, 0, conja == GB_CONJUGATE, transb, m, n, &alpha.real, &a->real, rs_a,
                                 cs_a, &b->real, rs_b, cs_b, &beta.real, &c->real, rs_c, cs_c, gb::level3_slices(),
                                 pick_stream(stream));
}

int gb_dtrmm3_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_trans_t transb, gb_dim_t m,
                  gb_dim_t n, double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b,
                  gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_dtrmm3_dev", "negative dimension");
    return gb::dtrmm3_dev(side, uploa, transa, diaga, transb, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c,
                          cs_c, gb::level3_slices(), pick_stream(stream));
}

int gb_dsyr2k_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, double alpha,
                  const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                  double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_dsyr2k_dev", "negative dimension");
    return gb::dsyr2k_dev(uploc, transa, transb, m, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c,
                          gb::level3_slices(), pick_stream(stream));
}

int gb_dscalv_dev(gb_dim_t n, double alpha, double* x, gb_inc_t incx, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    return gb::dscalv_dev(n, alpha, x, incx, pick_stream(stream));
}

int gb_dcopyv_dev(gb_dim_t n, const double* x, gb_inc_t incx, double* y, gb_inc_t incy, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    return gb::dcopyv_dev(n, x, incx, y, incy, pick_stream(stream));
}

int gb_damaxv_dev(gb_dim_t n, const double* x, gb_inc_t incx, gb_dim_t* index_dev, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    return gb::damaxv_dev(n, x, incx, index_dev, pick_stream(stream));
}

int gb_dger_dev(gb_dim_t m, gb_dim_t n, double alpha, const double* x, gb_inc_t incx, const double* y, gb_inc_t incy,
                double* a, gb_inc_t rs_a, gb_inc_t cs_a, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_dger_dev", "negative dimension");
    return gb::dger_dev(m, n, alpha, x, incx, y, incy, a, rs_a, cs_a, pick_stream(stream));
}

int gb_dtrsv_dev(gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, double alpha, const double* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, double* x, gb_inc_t incx, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0) return gb::set_error(GB_ERR_ARG, "gb_dtrsv_dev", "negative dimension");
    return gb::dtrsv_dev(uploa, transa, diaga, m, alpha, a, rs_a, cs_a, x, incx, pick_stream(stream));
}

int gb_dtrmm_dev(gb_side_t side, gb_uplo_t uploa, gb_trans_t transa, gb_diag_t diaga, gb_dim_t m, gb_dim_t n,
                 double alpha, const double* a, gb_inc_t rs_a, gb_inc_t cs_a, double* b, gb_inc_t rs_b,
                 gb_inc_t cs_b, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_dtrmm_dev", "negative dimension");
    return gb::dtrmm_dev(side, uploa, transa, diaga, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, gb::level3_slices(),
                         pick_stream(stream));
}

int gb_dsymm_dev(gb_side_t side, gb_uplo_t uploa, gb_dim_t m, gb_dim_t n, double alpha, const double* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b, double beta, double* c,
                 gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || n < 0) return gb::set_error(GB_ERR_ARG, "gb_dsymm_dev", "negative dimension");
    return gb::dsymm_dev(side, uploa, m, n, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c,
                         gb::level3_slices(), pick_stream(stream));
}

int gb_dgemmt_dev(gb_uplo_t uploc, gb_trans_t transa, gb_trans_t transb, gb_dim_t m, gb_dim_t k, double alpha,
                  const double* a, gb_inc_t rs_a, gb_inc_t cs_a, const double* b, gb_inc_t rs_b, gb_inc_t cs_b,
                  double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    if (m < 0 || k < 0) return gb::set_error(GB_ERR_ARG, "gb_dgemmt_dev", "negative dimension");
    return gb::dgemmt_dev(uploc, transa, transb, m, k, alpha, a, rs_a, cs_a, b, rs_b, cs_b, beta, c, rs_c, cs_c,
                          gb::level3_slices(), pick_stream(stream));
}

int gb_dsyrk_dev(gb_uplo_t uploc, gb_trans_t transa, gb_dim_t m, gb_dim_t k, double alpha, const double* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, double beta, double* c, gb_inc_t rs_c, gb_inc_t cs_c, void* stream)
{
    const bool ta = GB_IS_TRANS(transa);
    return gb_dgemmt_dev(uploc, ta ? GB_TRANSPOSE : GB_NO_TRANSPOSE, ta ? GB_NO_TRANSPOSE : GB_TRANSPOSE, m, k,
                         alpha, a, rs_a, cs_a, a, rs_a, cs_a, beta, c, rs_c, cs_c, stream);
}

int gb_daxpyv_dev(gb_dim_t n, double alpha, const double* x, gb_inc_t incx, double* y, gb_inc_t incy,
                  void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    return gb::daxpyv_dev(n, alpha, x, incx, y, incy, pick_stream(stream));
}

int gb_ddotv_dev(gb_dim_t n, const double* x, gb_inc_t incx, const double* y, gb_inc_t incy,
                 double* rho, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    cudaStream_t s = pick_stream(stream);
    const int nparts = gb::dotv_nparts(n > 0 ? n : 1);
    double* scratch = static_cast<double*>(gb::dev_alloc(sizeof(double) * nparts, s));
    if (!scratch) return GB_ERR_NOMEM;
    rc = gb::ddotv_dev(n, x, incx, y, incy, rho, scratch, nparts, s);
    gb::dev_free(scratch, s);
    return rc;
}

int gb_dgemv_dev(gb_trans_t transa, gb_dim_t m, gb_dim_t n, double alpha, const double* a,
                 gb_inc_t rs_a, gb_inc_t cs_a, const double* x, gb_inc_t incx, double beta, double* y,
                 gb_inc_t incy, void* stream)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    return gb::dgemv_dev(GB_IS_TRANS(transa) ? 1 : 0, m, n, alpha, a, rs_a, cs_a, x, incx, beta, y, incy,
                         pick_stream(stream));
}

}  // extern "C"
