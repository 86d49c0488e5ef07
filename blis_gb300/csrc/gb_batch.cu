// gb_batch.cu -- grouped GEMM: every problem of a gemm_batch call in one
// persistent launch (the batching form).
//
// The reference's dgemm_batch_ (frame/compat/extra/bla_gemm_batch.c:
// 135-249) checks every group, then calls bli_gemm_ex once per problem,
// serially (:227), each call with its own thread fan-out.  Here the host
// builds a descriptor table (one row per problem, sorted by k so the
// longest tiles are handed out first), prefix-sums the 128x128 tile counts,
// and launches one persistent grid; each CTA pulls the next tile index from
// a device-side atomic counter, finds its problem by binary search over the
// prefix sums, and runs the shared tile engine (DMMA for FP64, FFMA for
// FP32).  A tile is owned by one CTA for its whole k range, so results are
// deterministic.  A plan object keeps the table resident and replays the
// counter reset + launch as a captured CUDA graph.
#include <algorithm>
#include <vector>

#include "gb_gemm_tiles.cuh"

namespace gb {
namespace {

using namespace tiles;

struct BatchDesc {
    int64_t m, n, k;
    double alpha, beta;
    const void* a;
    int64_t ars, acs;
    const void* b;
    int64_t brs, bcs;
    void* c;
    int64_t rs_c, cs_c;
    int64_t tile_start;
    int64_t tiles_n;
};

template <typename T, bool DMMA>
__global__ void __launch_bounds__(NT) grouped_gemm_kernel(const BatchDesc* __restrict__ d, int nprob,
                                                          int64_t total_tiles,
                                                          unsigned long long* counter, const int* gate)
{
    if (gate && *gate == 0) return;  // fallback launch of the Ozaki form: only on Inf/NaN operands
    __shared__ T As[BK * LDS];
    __shared__ T Bs[BK * LDS];
    __shared__ long long tile_s;
    for (;;) {
        if (threadIdx.x == 0) tile_s = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long tile = tile_s;
        __syncthreads();
        if (tile >= total_tiles) break;
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (d[mid].tile_start <= tile) lo = mid;
            else hi = mid - 1;
        }
        const BatchDesc& q = d[lo];
        const int64_t local = tile - q.tile_start;
        const int64_t bm = (local / q.tiles_n) * BM, bn = (local % q.tiles_n) * BN;
        GArgs<T> p{q.m, q.n, q.k, (T)q.alpha, (T)q.beta, static_cast<const T*>(q.a), q.ars, q.acs,
                   static_cast<const T*>(q.b), q.brs, q.bcs, static_cast<T*>(q.c), q.rs_c, q.cs_c};
        if constexpr (DMMA) dmma_tile(p, bm, bn, As, Bs);
        else simt_tile<T>(p, bm, bn, As, Bs);
    }
}

}  // namespace

// A resident batch: descriptor table in HBM, tile counter, optional graph.
// The Ozaki form (GB_BATCH_FP64_OZAKI, and FP32 policy 3) adds the grouped
// Ozaki tables and arenas; this plan's own table then holds the same problems
// for the native launch gated on the Ozaki form's Inf/NaN flag, `rest` the problems with
// k == 0 or alpha == 0 (C := beta C) and `singles` those with a k too long
// for the grouped form.
struct BatchPlan {
    int dtype;  // GB_BATCH_FP64, GB_BATCH_FP32, GB_BATCH_FP64_OZAKI
    int nprob;
    int64_t total_tiles;
    BatchDesc* d_desc;
    unsigned long long* d_counter;
    std::vector<BatchDesc> host;
    cudaGraphExec_t graph;
    cudaStream_t graph_stream;
    OzBatch* oz = nullptr;
    SupGroup* sup = nullptr;  // problems the selector sends to the 64 x 64 engine
    int policy = 0;           // configuration policy the plan's autotuning kept (native plans)
    const int* gate = nullptr;
    BatchPlan* rest = nullptr;
    std::vector<gb_gemm_problem_t> singles;
    int slices = 0;
};

static int launch_plan(BatchPlan* pl, cudaStream_t s)
{
    int rc;
    if (pl->oz && (rc = ozaki_batch_launch(pl->oz, s))) return rc;
    if (pl->rest && (rc = launch_plan(pl->rest, s))) return rc;
    for (const gb_gemm_problem_t& p : pl->singles) {
        const bool ta = GB_IS_TRANS(p.transa), tb = GB_IS_TRANS(p.transb);
        if (pl->dtype == GB_BATCH_FP32) {  // policy 3: k past the grouped form's range
            rc = sgemm_split_dev(p.m, p.n, p.k, (float)p.alpha, (const float*)p.a, ta ? p.lda : 1, ta ? 1 : p.lda,
                                 (const float*)p.b, tb ? p.ldb : 1, tb ? 1 : p.ldb, (float)p.beta, (float*)p.c, 1,
                                 p.ldc, s);
            if (rc) return rc;
            continue;
        }
        rc = dgemm_ozaki(p.m, p.n, p.k, p.alpha, (const double*)p.a, ta ? p.lda : 1, ta ? 1 : p.lda,
                         (const double*)p.b, tb ? p.ldb : 1, tb ? 1 : p.ldb, p.beta, (double*)p.c, 1, p.ldc,
                         pl->slices, s);
        if (rc) return rc;
    }
    if (pl->sup && (rc = sup_group_launch(pl->sup, s))) return rc;
    if (pl->total_tiles == 0) return GB_SUCCESS;
    GB_CUDA(cudaMemsetAsync(pl->d_counter, 0, sizeof(unsigned long long), s));
    const int sms = sm_count() > 0 ? sm_count() : 148;
    int64_t grid = (int64_t)sms * 2;  // 2 resident CTAs of 256 threads per SM (DMMA: 240 regs)
    if (grid > pl->total_tiles) grid = pl->total_tiles;
    LaunchScope ls(pl->dtype == 1 ? (pl->gate ? "batch_grouped_ffma_gated" : "batch_grouped_ffma")
                                  : (pl->gate ? "batch_grouped_dmma_gated" : "batch_grouped_dmma"), s);
    if (pl->dtype != 1)
        grouped_gemm_kernel<double, true><<<(unsigned)grid, NT, 0, s>>>(pl->d_desc, pl->nprob,
                                                                       pl->total_tiles, pl->d_counter, pl->gate);
    else
        grouped_gemm_kernel<float, false><<<(unsigned)grid, NT, 0, s>>>(pl->d_desc, pl->nprob,
                                                                       pl->total_tiles, pl->d_counter, pl->gate);
    return check_cuda(cudaGetLastError(), "grouped_gemm");
}

void batch_plan_destroy(BatchPlan* pl);
int batch_plan_run(BatchPlan* pl, cudaStream_t s, bool use_graph);
static int batch_plan_build(const gb_gemm_problem_t* probs, int64_t count, int dtype, BatchPlan** out);

// Policy 3, FP32 only: SGEMM's split form for the whole batch, the grouped
// Ozaki form on the FP32 operands themselves at GB_SGEMM_SPLIT_SLICES
// (every element widened exactly as it is split, C = RN32(alpha P + beta C)
// in the recombination), bit-identical per problem to the single-problem
// split form.  Problems with k = 0 or alpha = 0 (C := beta C) take the FP32
// grouped launch; a k past the grouped form's range runs alone through the
// single-problem split form; Inf/NaN in any operand raises the grouped
// form's flag, and the FP32 grouped launch gated on it recomputes every
// grouped problem.
static int batch_plan_split(const gb_gemm_problem_t* probs, int64_t count, BatchPlan** out)
{
    *out = nullptr;
    const int slices = GB_SGEMM_SPLIT_SLICES;
    std::vector<gb_gemm_problem_t> grouped, rest, singles;
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        if (p.m < 0 || p.n < 0 || p.k < 0) return set_error(GB_ERR_ARG, "gb_batch", "negative dimension");
        if (p.m == 0 || p.n == 0) continue;
        if (p.k == 0 || p.alpha == 0.0) rest.push_back(p);
        else if (ozaki_batch_accepts(p.k, slices)) grouped.push_back(p);
        else singles.push_back(p);
    }
    BatchPlan* pl = nullptr;
    int rc = batch_plan_build(grouped.data(), (int64_t)grouped.size(), GB_BATCH_FP32, &pl);
    if (rc) return rc;
    pl->slices = slices;
    pl->singles = singles;
    cudaStream_t s = thread_stream();
    if ((rc = ozaki_batch_create(grouped.data(), (int64_t)grouped.size(), slices, s, &pl->oz, true)) ||
        (!rest.empty() && (rc = batch_plan_build(rest.data(), (int64_t)rest.size(), GB_BATCH_FP32, &pl->rest)))) {
        batch_plan_destroy(pl);
        return rc;
    }
    pl->gate = ozaki_batch_flag(pl->oz);
    pl->policy = 3;
    *out = pl;
    return GB_SUCCESS;
}

// Native FP64/FP32 batch with one configuration policy: 0 = every problem
// on the 128 x 128 engine; 1 = the 64 x 64 engine for the problems whose
// selected configuration is 1..5, without split-K (a batch already has
// parallelism); 2 = the selected configuration including its split-K.
int batch_plan_policy(const gb_gemm_problem_t* probs, int64_t count, int dtype, int policy, BatchPlan** out)
{
    if (policy == 3) {
        if (dtype != GB_BATCH_FP32) return set_error(GB_ERR_ARG, "gb_batch", "policy 3 (split form) is FP32 only");
        return batch_plan_split(probs, count, out);
    }
    std::vector<gb_gemm_problem_t> big, small;
    std::vector<int> cfgs;
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        if (p.m < 0 || p.n < 0 || p.k < 0) return set_error(GB_ERR_ARG, "gb_batch", "negative dimension");
        int cfg = 0, sl = 0;
        if (policy > 0 && p.m > 0 && p.n > 0 && p.k > 0 && p.alpha != 0.0 &&
            selector_choose(dtype, p.m, p.n, p.k, GB_IS_TRANS(p.transa), GB_IS_TRANS(p.transb), 0, 0.0, 0.0, &cfg,
                            &sl) != GB_SUCCESS)
            cfg = 0;
        if (policy == 1 && cfg > 1) cfg = 1;
        if (cfg >= 1 && cfg < GB_GEMM_NUM_CONFIGS) {
            small.push_back(p);
            cfgs.push_back(cfg);
        } else {
            big.push_back(p);
        }
    }
    BatchPlan* pl = nullptr;
    int rc = batch_plan_build(big.data(), (int64_t)big.size(), dtype, &pl);
    if (rc) return rc;
    if (!small.empty() &&
        (rc = sup_group_create(dtype, small.data(), cfgs.data(), (int64_t)small.size(), thread_stream(), &pl->sup))) {
        batch_plan_destroy(pl);
        return rc;
    }
    *out = pl;
    return GB_SUCCESS;
}

// Native FP64/FP32 plan, autotuned when it is created: each candidate policy
// runs twice on the batch's own shapes with scratch outputs (the caller's C
// is not touched), timed with CUDA events, and the fastest is kept.  The
// candidates: policy 0 always; 1 and 2 with a selector model loaded
// (gb_selector_load_file + gb_set_gemm_autoselect); 3 for FP32 unless
// gb_set_sgemm_mode pinned SGEMM to the FP32 pipe.
static int batch_plan_selected(const gb_gemm_problem_t* probs, int64_t count, int dtype, BatchPlan** out)
{
    std::vector<int> cands{0};
    if (selector_auto()) cands.insert(cands.end(), {1, 2});
    if (dtype == GB_BATCH_FP32 && sgemm_mode_setting != GB_SGEMM_FMA) cands.push_back(3);
    if (cands.size() == 1) return batch_plan_policy(probs, count, dtype, 0, out);
    cudaStream_t s = thread_stream();
    const size_t esz = dtype == GB_BATCH_FP32 ? 4 : 8;
    std::vector<gb_gemm_problem_t> tune(probs, probs + count);
    size_t elems = 0;
    for (const auto& p : tune) elems += (p.m > 0 && p.n > 0) ? (size_t)(p.m * p.n) : 0;
    char* scratch = static_cast<char*>(dev_alloc(esz * (elems + 1), s));
    if (!scratch) return GB_ERR_NOMEM;
    size_t off = 0;
    for (auto& p : tune) {
        if (p.m <= 0 || p.n <= 0) continue;
        p.c = scratch + off * esz;
        p.ldc = p.m;
        off += (size_t)(p.m * p.n);
    }
    int rc = check_cuda(cudaMemsetAsync(scratch, 0, esz * (elems + 1), s), "batch tuning");
    int best = 0;
    float best_ms = 0.0f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (size_t ci = 0; ci < cands.size() && !rc; ++ci) {
        const int policy = cands[ci];
        BatchPlan* t = nullptr;
        if ((rc = batch_plan_policy(tune.data(), count, dtype, policy, &t))) break;
        rc = batch_plan_run(t, s, false);  // warm-up
        cudaEventRecord(e0, s);
        if (!rc) rc = batch_plan_run(t, s, false);
        cudaEventRecord(e1, s);
        if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "batch tuning");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (!rc && (policy == 0 || ms < best_ms)) {
            best = policy;
            best_ms = ms;
        }
        batch_plan_destroy(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dev_free(scratch, s);
    if (rc) return rc;
    rc = batch_plan_policy(probs, count, dtype, best, out);
    if (!rc) (*out)->policy = best;
    return rc;
}

// `tune`: resident plans autotune their configuration policy (see above);
// one-shot grouped calls take the 128 x 128 engine for every problem.
int batch_plan_create(const gb_gemm_problem_t* probs, int64_t count, int dtype, BatchPlan** out, bool tune)
{
    *out = nullptr;
    if (dtype != GB_BATCH_FP64_OZAKI)
        return tune ? batch_plan_selected(probs, count, dtype, out) : batch_plan_policy(probs, count, dtype, 0, out);
    // the grouped batch runs the digit form (at the CRT form's precision when that form is set)
    int slices = ozaki_digit_slices();
    if (slices < 2) slices = 8;  // automatic: the verifier is per problem; the batch uses 8
    std::vector<gb_gemm_problem_t> grouped, rest, singles;
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        if (p.m < 0 || p.n < 0 || p.k < 0) return set_error(GB_ERR_ARG, "gb_batch", "negative dimension");
        if (p.m == 0 || p.n == 0) continue;
        if (p.k == 0 || p.alpha == 0.0) rest.push_back(p);
        else if (ozaki_batch_accepts(p.k, slices)) grouped.push_back(p);
        else singles.push_back(p);
    }
    BatchPlan* pl = nullptr;
    int rc = batch_plan_build(grouped.data(), (int64_t)grouped.size(), GB_BATCH_FP64, &pl);
    if (rc) return rc;
    pl->dtype = GB_BATCH_FP64_OZAKI;
    pl->slices = slices;
    pl->singles = singles;
    cudaStream_t s = thread_stream();
    if ((rc = ozaki_batch_create(grouped.data(), (int64_t)grouped.size(), slices, s, &pl->oz)) ||
        (!rest.empty() && (rc = batch_plan_build(rest.data(), (int64_t)rest.size(), GB_BATCH_FP64, &pl->rest)))) {
        batch_plan_destroy(pl);
        return rc;
    }
    pl->gate = ozaki_batch_flag(pl->oz);
    *out = pl;
    return GB_SUCCESS;
}

static int batch_plan_build(const gb_gemm_problem_t* probs, int64_t count, int dtype, BatchPlan** out)
{
    *out = nullptr;
    BatchPlan* pl = new BatchPlan();
    pl->dtype = dtype;
    pl->graph = nullptr;
    pl->graph_stream = nullptr;
    pl->host.reserve((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        if (p.m < 0 || p.n < 0 || p.k < 0) {
            delete pl;
            return set_error(GB_ERR_ARG, "gb_batch", "negative dimension");
        }
        if (p.m == 0 || p.n == 0) continue;
        const bool ta = GB_IS_TRANS(p.transa), tb = GB_IS_TRANS(p.transb);
        BatchDesc d;
        d.m = p.m;
        d.n = p.n;
        d.k = (p.alpha == 0.0) ? 0 : p.k;  // alpha == 0: C := beta*C (frame/3/bli_l3_util.c:56-62)
        d.alpha = p.alpha;
        d.beta = p.beta;
        d.a = p.a;
        d.ars = ta ? p.lda : 1;
        d.acs = ta ? 1 : p.lda;
        d.b = p.b;
        d.brs = tb ? p.ldb : 1;
        d.bcs = tb ? 1 : p.ldb;
        d.c = p.c;
        d.rs_c = 1;
        d.cs_c = p.ldc;
        d.tiles_n = (p.n + BN - 1) / BN;
        d.tile_start = 0;
        pl->host.push_back(d);
    }
    // longest k first: the last tiles handed out are the cheapest
    std::stable_sort(pl->host.begin(), pl->host.end(),
                     [](const BatchDesc& x, const BatchDesc& y) { return x.k > y.k; });
    int64_t t = 0;
    for (auto& d : pl->host) {
        d.tile_start = t;
        t += ((d.m + BM - 1) / BM) * d.tiles_n;
    }
    pl->total_tiles = t;
    pl->nprob = (int)pl->host.size();
    cudaStream_t s = thread_stream();
    pl->d_desc = static_cast<BatchDesc*>(dev_alloc(sizeof(BatchDesc) * (pl->host.size() + 1), s));
    pl->d_counter = static_cast<unsigned long long*>(dev_alloc(sizeof(unsigned long long), s));
    if (!pl->d_desc || !pl->d_counter) {
        delete pl;
        return GB_ERR_NOMEM;
    }
    if (!pl->host.empty())
        GB_CUDA(cudaMemcpyAsync(pl->d_desc, pl->host.data(), sizeof(BatchDesc) * pl->host.size(),
                                cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaStreamSynchronize(s));
    *out = pl;
    return GB_SUCCESS;
}

int batch_plan_run(BatchPlan* pl, cudaStream_t s, bool use_graph)
{
    // problems run one by one through the Ozaki form allocate workspace per call: no graph
    if (!use_graph || !pl->singles.empty()) return launch_plan(pl, s);
    if (!pl->graph) {
        cudaStream_t cap;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g;
        GB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int rc = launch_plan(pl, cap);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        if (rc) {
            cudaStreamDestroy(cap);
            return rc;
        }
        GB_CUDA(e);
        GB_CUDA(cudaGraphInstantiate(&pl->graph, g, 0));
        cudaGraphDestroy(g);
        pl->graph_stream = cap;
    }
    LaunchScope ls("batch_graph", s);
    return check_cuda(cudaGraphLaunch(pl->graph, s), "cudaGraphLaunch");
}

void batch_plan_destroy(BatchPlan* pl)
{
    if (!pl) return;
    cudaStream_t s = thread_stream();
    cudaStreamSynchronize(s);
    if (pl->graph) cudaGraphExecDestroy(pl->graph);
    if (pl->graph_stream) cudaStreamDestroy(pl->graph_stream);
    dev_free(pl->d_desc, s);
    dev_free(pl->d_counter, s);
    ozaki_batch_destroy(pl->oz, s);
    sup_group_destroy(pl->sup, s);
    cudaStreamSynchronize(s);
    batch_plan_destroy(pl->rest);
    delete pl;
}

// The per-problem launch loop the grouped form is compared against.
int batch_loop(const gb_gemm_problem_t* probs, int64_t count, int dtype, cudaStream_t s)
{
    for (int64_t i = 0; i < count; ++i) {
        const gb_gemm_problem_t& p = probs[i];
        const bool ta = GB_IS_TRANS(p.transa), tb = GB_IS_TRANS(p.transb);
        int rc;
        if (dtype == GB_BATCH_FP64_OZAKI) {
            int slices = ozaki_digit_slices();
            if (slices < 2) slices = 8;
            ModeOverride digits(GB_DGEMM_OZAKI, slices, 0);
            rc = dgemm_ozaki(p.m, p.n, p.k, p.alpha, (const double*)p.a, ta ? p.lda : 1, ta ? 1 : p.lda,
                             (const double*)p.b, tb ? p.ldb : 1, tb ? 1 : p.ldb, p.beta, (double*)p.c, 1, p.ldc,
                             slices, s);
        } else if (dtype == GB_BATCH_FP64)
            rc = dgemm_native(p.m, p.n, p.k, p.alpha, (const double*)p.a, ta ? p.lda : 1, ta ? 1 : p.lda,
                              (const double*)p.b, tb ? p.ldb : 1, tb ? 1 : p.ldb, p.beta, (double*)p.c, 1,
                              p.ldc, s);
        else
            rc = sgemm_dev(p.m, p.n, p.k, (float)p.alpha, (const float*)p.a, ta ? p.lda : 1, ta ? 1 : p.lda,
                           (const float*)p.b, tb ? p.ldb : 1, tb ? 1 : p.ldb, (float)p.beta, (float*)p.c, 1,
                           p.ldc, s);
        if (rc) return rc;
    }
    return GB_SUCCESS;
}

}  // namespace gb

using namespace gb;

namespace {

bool lsame_c(char a, char b) { return (a | 0x20) == (b | 0x20); }

int gemm_check_group(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc)
{
    const bool nota = lsame_c(ta, 'N'), notb = lsame_c(tb, 'N');
    const bool oka = nota || lsame_c(ta, 'T') || lsame_c(ta, 'C');
    const bool okb = notb || lsame_c(tb, 'T') || lsame_c(tb, 'C');
    const int nrowa = nota ? m : k, nrowb = notb ? k : n;
    if (!oka) return 1;
    if (!okb) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (k < 0) return 5;
    if (lda < (nrowa > 1 ? nrowa : 1)) return 8;
    if (ldb < (nrowb > 1 ? nrowb : 1)) return 10;
    if (ldc < (m > 1 ? m : 1)) return 13;
    return 0;
}

// Host-pointer grouped GEMM: every operand is copied into one device arena
// (packed column-major), the grouped kernel runs once, C's come back.
template <typename T>
void batch_blas(const char* name, const char* transa_array, const char* transb_array,
                const gb_f77_int* m_array, const gb_f77_int* n_array, const gb_f77_int* k_array,
                const T* alpha_array, const T** a_array, const gb_f77_int* lda_array,
                const T** b_array, const gb_f77_int* ldb_array, const T* beta_array, T** c_array,
                const gb_f77_int* ldc_array, const gb_f77_int* group_count, const gb_f77_int* group_size)
{
    for (int g = 0; g < *group_count; ++g) {
        const int info = gemm_check_group(transa_array[g], transb_array[g], m_array[g], n_array[g],
                                          k_array[g], lda_array[g], ldb_array[g], ldc_array[g]);
        if (info) {
            gb_f77_int i = info;
            xerbla_(name, &i, 6);
            return;
        }
    }
    if (ensure_init()) return;
    cudaStream_t s = thread_stream();
    struct Host {
        const T* a; const T* b; T* c;
        int64_t m, n, k, lda, ldb, ldc, ra, ca, rb, cb;
        bool ta, tb;
        T alpha, beta;
        size_t off_a, off_b, off_c;
    };
    std::vector<Host> hs;
    size_t total = 0;
    int64_t idx = 0;
    for (int g = 0; g < *group_count; ++g) {
        for (int j = 0; j < group_size[g]; ++j, ++idx) {
            Host h;
            h.ta = !lsame_c(transa_array[g], 'N');
            h.tb = !lsame_c(transb_array[g], 'N');
            h.m = m_array[g] > 0 ? m_array[g] : 0;
            h.n = n_array[g] > 0 ? n_array[g] : 0;
            h.k = k_array[g] > 0 ? k_array[g] : 0;
            h.lda = lda_array[g];
            h.ldb = ldb_array[g];
            h.ldc = ldc_array[g];
            h.alpha = alpha_array[g];
            h.beta = beta_array[g];
            h.a = a_array[idx];
            h.b = b_array[idx];
            h.c = c_array[idx];
            h.ra = h.ta ? h.k : h.m;
            h.ca = h.ta ? h.m : h.k;
            h.rb = h.tb ? h.n : h.k;
            h.cb = h.tb ? h.k : h.n;
            auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
            h.off_a = total; total += al(sizeof(T) * h.ra * h.ca);
            h.off_b = total; total += al(sizeof(T) * h.rb * h.cb);
            h.off_c = total; total += al(sizeof(T) * h.m * h.n);
            hs.push_back(h);
        }
    }
    char* arena = static_cast<char*>(dev_alloc(total ? total : 256, s));
    if (!arena) return;
    std::vector<gb_gemm_problem_t> probs;
    probs.reserve(hs.size());
    for (auto& h : hs) {
        if (h.m == 0 || h.n == 0) continue;
        const bool work = (h.k > 0 && h.alpha != T(0));
        if (work && h.ra * h.ca > 0)
            cudaMemcpy2DAsync(arena + h.off_a, h.ra * sizeof(T), h.a, h.lda * sizeof(T), h.ra * sizeof(T),
                              h.ca, cudaMemcpyDefault, s);
        if (work && h.rb * h.cb > 0)
            cudaMemcpy2DAsync(arena + h.off_b, h.rb * sizeof(T), h.b, h.ldb * sizeof(T), h.rb * sizeof(T),
                              h.cb, cudaMemcpyDefault, s);
        if (h.beta != T(0))
            cudaMemcpy2DAsync(arena + h.off_c, h.m * sizeof(T), h.c, h.ldc * sizeof(T), h.m * sizeof(T), h.n,
                              cudaMemcpyDefault, s);
        gb_gemm_problem_t p;
        p.transa = h.ta ? GB_TRANSPOSE : GB_NO_TRANSPOSE;
        p.transb = h.tb ? GB_TRANSPOSE : GB_NO_TRANSPOSE;
        p.m = h.m;
        p.n = h.n;
        p.k = work ? h.k : 0;
        p.alpha = (double)h.alpha;
        p.beta = (double)h.beta;
        p.a = arena + h.off_a;
        p.lda = h.ra > 0 ? h.ra : 1;
        p.b = arena + h.off_b;
        p.ldb = h.rb > 0 ? h.rb : 1;
        p.c = arena + h.off_c;
        p.ldc = h.m;
        probs.push_back(p);
    }
    BatchPlan* pl = nullptr;
    // dgemm_batch_ follows the precision mode of dgemm_ (gb_set_dgemm_mode)
    const int dtype = sizeof(T) == 4 ? GB_BATCH_FP32
                                     : (dgemm_mode() == GB_DGEMM_OZAKI ? GB_BATCH_FP64_OZAKI : GB_BATCH_FP64);
    int rc = batch_plan_create(probs.data(), (int64_t)probs.size(), dtype, &pl, false);
    if (!rc) rc = batch_plan_run(pl, s, false);
    if (!rc) {
        for (auto& h : hs) {
            if (h.m == 0 || h.n == 0) continue;
            cudaMemcpy2DAsync(h.c, h.ldc * sizeof(T), arena + h.off_c, h.m * sizeof(T), h.m * sizeof(T), h.n,
                              cudaMemcpyDefault, s);
        }
        cudaStreamSynchronize(s);
        read_and_clear_device_status(s, name);
    }
    batch_plan_destroy(pl);
    dev_free(arena, s);
    cudaStreamSynchronize(s);
}

char cblas_tc(int t) { return t == GbCblasNoTrans ? 'N' : (t == GbCblasTrans ? 'T' : (t == GbCblasConjTrans ? 'C' : '?')); }

}  // namespace

extern "C" {

void dgemm_batch_(const gb_f77_char* transa_array, const gb_f77_char* transb_array,
                  const gb_f77_int* m_array, const gb_f77_int* n_array, const gb_f77_int* k_array,
                  const double* alpha_array, const double** a_array, const gb_f77_int* lda_array,
                  const double** b_array, const gb_f77_int* ldb_array, const double* beta_array,
                  double** c_array, const gb_f77_int* ldc_array, const gb_f77_int* group_count,
                  const gb_f77_int* group_size)
{
    batch_blas<double>("DGEMM ", transa_array, transb_array, m_array, n_array, k_array, alpha_array, a_array,
                       lda_array, b_array, ldb_array, beta_array, c_array, ldc_array, group_count, group_size);
}

void sgemm_batch_(const gb_f77_char* transa_array, const gb_f77_char* transb_array,
                  const gb_f77_int* m_array, const gb_f77_int* n_array, const gb_f77_int* k_array,
                  const float* alpha_array, const float** a_array, const gb_f77_int* lda_array,
                  const float** b_array, const gb_f77_int* ldb_array, const float* beta_array,
                  float** c_array, const gb_f77_int* ldc_array, const gb_f77_int* group_count,
                  const gb_f77_int* group_size)
{
    batch_blas<float>("SGEMM ", transa_array, transb_array, m_array, n_array, k_array, alpha_array, a_array,
                      lda_array, b_array, ldb_array, beta_array, c_array, ldc_array, group_count, group_size);
}

void cblas_dgemm_batch(int order, const int* transa_array, const int* transb_array,
                       const gb_f77_int* m_array, const gb_f77_int* n_array, const gb_f77_int* k_array,
                       const double* alpha_array, const double** a_array, const gb_f77_int* lda_array,
                       const double** b_array, const gb_f77_int* ldb_array, const double* beta_array,
                       double** c_array, const gb_f77_int* ldc_array, gb_f77_int group_count,
                       const gb_f77_int* group_size)
{
    std::vector<char> ta(group_count > 0 ? group_count : 1), tb(group_count > 0 ? group_count : 1);
    for (int g = 0; g < group_count; ++g) {
        ta[g] = cblas_tc(transa_array[g]);
        tb[g] = cblas_tc(transb_array[g]);
    }
    if (order == GbCblasColMajor) {
        dgemm_batch_(ta.data(), tb.data(), m_array, n_array, k_array, alpha_array, a_array, lda_array, b_array,
                     ldb_array, beta_array, c_array, ldc_array, &group_count, group_size);
    } else if (order == GbCblasRowMajor) {
        // row-major: C^T = op(B)^T op(A)^T (cblas_dgemm_batch.c:99,154)
        dgemm_batch_(tb.data(), ta.data(), n_array, m_array, k_array, alpha_array, b_array, ldb_array, a_array,
                     lda_array, beta_array, c_array, ldc_array, &group_count, group_size);
    } else {
        gb_f77_int info = 1;
        xerbla_("cblas_dgemm_batch", &info, 17);
    }
}

int gb_gemm_batch_dev(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, int mode, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    if (dtype != GB_BATCH_FP64 && dtype != GB_BATCH_FP32 && dtype != GB_BATCH_FP64_OZAKI)
        return set_error(GB_ERR_ARG, "gb_gemm_batch_dev", "dtype must be GB_BATCH_FP64, FP32 or FP64_OZAKI");
    if (mode == GB_BATCH_LOOP) return batch_loop(probs, count, dtype, s);
    BatchPlan* pl = nullptr;
    if ((rc = batch_plan_create(probs, count, dtype, &pl, false))) return rc;
    rc = batch_plan_run(pl, s, false);
    cudaStreamSynchronize(s);
    batch_plan_destroy(pl);
    return rc;
}

int gb_batch_plan_create(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, void** plan)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (dtype != GB_BATCH_FP64 && dtype != GB_BATCH_FP32 && dtype != GB_BATCH_FP64_OZAKI)
        return set_error(GB_ERR_ARG, "gb_batch_plan_create", "dtype must be GB_BATCH_FP64, FP32 or FP64_OZAKI");
    BatchPlan* pl = nullptr;
    rc = batch_plan_create(probs, count, dtype, &pl, true);
    *plan = pl;
    return rc;
}

int gb_batch_plan_run(void* plan, int use_graph, void* stream)
{
    if (!plan) return set_error(GB_ERR_ARG, "gb_batch_plan_run", "null plan");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    return batch_plan_run(static_cast<BatchPlan*>(plan), s, use_graph != 0);
}

int gb_batch_plan_destroy(void* plan)
{
    batch_plan_destroy(static_cast<BatchPlan*>(plan));
    return GB_SUCCESS;
}

}  // extern "C"

extern "C" int gb_batch_plan_create_ex(const gb_gemm_problem_t* probs, gb_dim_t count, int dtype, int policy,
                                       void** plan)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    *plan = nullptr;
    if (dtype != GB_BATCH_FP64 && dtype != GB_BATCH_FP32)
        return gb::set_error(GB_ERR_ARG, "gb_batch_plan_create_ex", "dtype must be GB_BATCH_FP64 or FP32");
    if (policy < -1 || policy > 3 || (policy == 3 && dtype != GB_BATCH_FP32))
        return gb::set_error(GB_ERR_ARG, "gb_batch_plan_create_ex", "policy in -1..2, or 3 for FP32");
    if ((policy == 1 || policy == 2) && !gb::selector_auto())
        return gb::set_error(GB_ERR_ARG, "gb_batch_plan_create_ex", "policies 1 and 2 need a loaded selector");
    gb::BatchPlan* pl = nullptr;
    rc = (policy < 0) ? gb::batch_plan_create(probs, count, dtype, &pl, true)
                      : gb::batch_plan_policy(probs, count, dtype, policy, &pl);
    if (!rc && policy >= 0) pl->policy = policy;
    *plan = pl;
    return rc;
}

extern "C" int gb_batch_plan_policy(const void* plan)
{
    if (!plan) return gb::set_error(GB_ERR_ARG, "gb_batch_plan_policy", "null plan");
    return static_cast<const gb::BatchPlan*>(plan)->policy;
}
