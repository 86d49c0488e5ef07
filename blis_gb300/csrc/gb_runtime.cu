// gb_runtime.cu -- context, streams, stream-ordered memory pool, status
// reporting, launch accounting and per-kernel event timing for
// libblis_gb300.so.
//
// BLIS itself keeps per-call runtime state in rntm_t and reports framework
// errors through bli_check_error_code()/bli_abort() (frame/base/bli_error.c:
// 126-139).  A GPU library cannot abort the host process on a device-side
// problem, so device failures become a per-thread status (gb_get_last_error)
// plus a printed message, and the entry point returns.
#include <atomic>
#include <mutex>
#include <string>
#include <vector>
#include <string.h>

#include "gb_internal.h"

namespace gb {

namespace {
std::mutex g_init_mu;
int g_device = -1;
bool g_inited = false;
int g_sms = 0;
unsigned int* g_status = nullptr;  // device word, one per library instance
std::atomic<int64_t> g_launches{0};
std::atomic<unsigned long long> g_trsv_wait_ns{kWaitBudgetNs};
std::atomic<int64_t> g_trsv_withhold{-1};
std::atomic<int> g_timing{0};
int g_dgemm_mode = GB_DGEMM_NATIVE;
int g_ozaki_slices = 8;
int g_ozaki_form = 0;

thread_local int t_err = GB_SUCCESS;
thread_local char t_msg[512] = {0};
thread_local cudaStream_t t_stream = nullptr;
thread_local int t_stream_dev = -1;

struct TimedLaunch {
    std::string name;
    cudaEvent_t start, stop;
};
std::mutex g_timing_mu;
std::vector<TimedLaunch> g_timed;
}  // namespace

int set_error(int code, const char* where, const char* what)
{
    t_err = code;
    snprintf(t_msg, sizeof(t_msg), "%s: %s", where ? where : "?", what ? what : "?");
    fprintf(stderr, "libblis_gb300: %s\n", t_msg);
    return code;
}

int check_cuda(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return GB_SUCCESS;
    return set_error(e == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA, where,
                     cudaGetErrorString(e));
}

int ensure_init()
{
    if (g_inited) {
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != g_device) GB_CUDA(cudaSetDevice(g_device));
        return GB_SUCCESS;
    }
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (!g_inited) {
        if (g_device < 0) GB_CUDA(cudaGetDevice(&g_device));
        GB_CUDA(cudaSetDevice(g_device));
        cudaDeviceProp prop;
        GB_CUDA(cudaGetDeviceProperties(&prop, g_device));
        if (prop.major != 10 || prop.minor != 3) {
            char buf[160];
            snprintf(buf, sizeof(buf), "device %d is %s (sm_%d%d); this library is built for sm_103a only",
                     g_device, prop.name, prop.major, prop.minor);
            return set_error(GB_ERR_UNSUPPORTED, "gb_init", buf);
        }
        g_sms = prop.multiProcessorCount;
        // Keep freed device blocks cached in the default pool.
        cudaMemPool_t pool;
        GB_CUDA(cudaDeviceGetDefaultMemPool(&pool, g_device));
        uint64_t thresh = UINT64_MAX;
        GB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh));
        GB_CUDA(cudaMalloc(&g_status, sizeof(unsigned int)));
        GB_CUDA(cudaMemset(g_status, 0, sizeof(unsigned int)));
        g_inited = true;
    } else {
        GB_CUDA(cudaSetDevice(g_device));
    }
    return GB_SUCCESS;
}

int sm_count() { return g_sms; }

cudaStream_t thread_stream()
{
    if (t_stream == nullptr || t_stream_dev != g_device) {
        cudaStreamCreateWithFlags(&t_stream, cudaStreamNonBlocking);
        t_stream_dev = g_device;
    }
    return t_stream;
}

// Two more non-blocking streams per calling thread for host<->device copies
// that overlap the compute stream (the pipelined host entry points).
thread_local cudaStream_t t_copy[2] = {nullptr, nullptr};
thread_local int t_copy_dev = -1;

cudaStream_t thread_copy_stream(int i)
{
    if (t_copy_dev != g_device) {
        t_copy[0] = t_copy[1] = nullptr;
        t_copy_dev = g_device;
    }
    if (t_copy[i & 1] == nullptr) cudaStreamCreateWithFlags(&t_copy[i & 1], cudaStreamNonBlocking);
    return t_copy[i & 1];
}

// Three more compute streams per calling thread (work that forks from the
// thread's stream and joins it again within one call).
thread_local cudaStream_t t_aux[3] = {nullptr, nullptr, nullptr};
thread_local int t_aux_dev = -1;

cudaStream_t thread_aux_stream(int i)
{
    if (t_aux_dev != g_device) {
        t_aux[0] = t_aux[1] = t_aux[2] = nullptr;
        t_aux_dev = g_device;
    }
    i = (i < 0 || i > 2) ? 0 : i;
    if (t_aux[i] == nullptr) cudaStreamCreateWithFlags(&t_aux[i], cudaStreamNonBlocking);
    return t_aux[i];
}

void* dev_alloc(size_t bytes, cudaStream_t s)
{
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(&p, bytes, s);
    if (e != cudaSuccess) {
        check_cuda(e, "cudaMallocAsync");
        return nullptr;
    }
    return p;
}

void dev_free(void* p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

unsigned int* device_status_word() { return g_status; }

int read_and_clear_device_status(cudaStream_t s, const char* where)
{
    unsigned int h = 0;
    GB_CUDA(cudaMemcpyAsync(&h, g_status, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (h == 0) return GB_SUCCESS;
    GB_CUDA(cudaMemsetAsync(g_status, 0, sizeof(unsigned int), s));
    char buf[160];
    snprintf(buf, sizeof(buf), "device status 0x%x (%s%s%s%s)", h,
             (h & DEV_WAIT_TIMEOUT) ? "bounded wait timed out " : "",
             (h & DEV_BAD_INDEX) ? "index out of range " : "",
             (h & DEV_INT_OVERFLOW) ? "integer accumulator bound exceeded " : "",
             (h & DEV_NONFINITE) ? "non-finite operand " : "");
    return set_error(GB_ERR_DEVICE, where, buf);
}

// A per-call form (gb_dgemm_ozaki) overrides the process-wide mode on the
// calling thread for the duration of the call.
thread_local int t_mode = -1, t_slices = -1, t_form = -1;

int dgemm_mode() { return t_mode >= 0 ? t_mode : g_dgemm_mode; }
int ozaki_slices() { return t_slices >= 0 ? t_slices : g_ozaki_slices; }
int ozaki_form() { return t_form >= 0 ? t_form : g_ozaki_form; }

int ozaki_digit_slices()
{
    const int sl = ozaki_slices();
    if (ozaki_form() != 1 || sl < 2) return sl;
    const int t = ozaki_crt_bits(sl, 16384);
    int d = (t + 1) / 8;
    return d < 2 ? 2 : (d > 12 ? 12 : d);
}

ModeOverride::ModeOverride(int mode, int slices, int form) : mode_(t_mode), slices_(t_slices), form_(t_form)
{
    t_mode = mode;
    t_slices = slices;
    if (form >= 0) t_form = form;
}

ModeOverride::~ModeOverride()
{
    t_mode = mode_;
    t_slices = slices_;
    t_form = form_;
}

unsigned long long trsv_wait_budget_ns() { return g_trsv_wait_ns.load(std::memory_order_relaxed); }
int64_t trsv_withheld_block() { return g_trsv_withhold.load(std::memory_order_relaxed); }

// Slice count of the calling thread's most recent Ozaki product (0 = the last
// double-precision product of a gemm call ran on the native FP64 kernel).
thread_local int t_last_slices = -1;
void note_ozaki_slices(int slices) { t_last_slices = slices; }

// ---------------------------------------------------------------- launches
LaunchScope::LaunchScope(const char* name, cudaStream_t s, bool is_kernel) : name_(name), s_(s), timed_(false)
{
    if (is_kernel) g_launches.fetch_add(1, std::memory_order_relaxed);
    if (g_timing.load(std::memory_order_relaxed)) {
        timed_ = true;
        cudaEventCreate(&start_);
        cudaEventCreate(&stop_);
        cudaEventRecord(start_, s_);
    }
}

LaunchScope::~LaunchScope()
{
    if (!timed_) return;
    cudaEventRecord(stop_, s_);
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timed.push_back(TimedLaunch{name_, start_, stop_});
}

}  // namespace gb

// ==================================================================== C ABI
extern "C" {

int gb_init(int device)
{
    {
        std::lock_guard<std::mutex> lk(gb::g_init_mu);
        if (!gb::g_inited) gb::g_device = device;
    }
    return gb::ensure_init();
}

int gb_set_dgemm_mode(int mode, int slices)
{
    if (mode != GB_DGEMM_NATIVE && mode != GB_DGEMM_OZAKI && mode != GB_DGEMM_OZAKI_CRT)
        return gb::set_error(GB_ERR_ARG, "gb_set_dgemm_mode",
                             "mode must be GB_DGEMM_NATIVE, GB_DGEMM_OZAKI or GB_DGEMM_OZAKI_CRT");
    if (mode == GB_DGEMM_OZAKI && slices != 0 && (slices < 2 || slices > 12))
        return gb::set_error(GB_ERR_ARG, "gb_set_dgemm_mode", "slices must be 0 (automatic) or in [2, 12]");
    if (mode == GB_DGEMM_OZAKI_CRT && slices != 0 && (slices < 2 || slices > 16))
        return gb::set_error(GB_ERR_ARG, "gb_set_dgemm_mode", "moduli must be 0 (automatic) or in [2, 16]");
    gb::g_dgemm_mode = (mode == GB_DGEMM_NATIVE) ? GB_DGEMM_NATIVE : GB_DGEMM_OZAKI;
    if (mode != GB_DGEMM_NATIVE) {
        gb::g_ozaki_slices = slices;
        gb::g_ozaki_form = (mode == GB_DGEMM_OZAKI_CRT) ? 1 : 0;
    }
    return GB_SUCCESS;
}

int gb_get_last_error(char* msg, size_t len)
{
    if (msg && len) {
        strncpy(msg, gb::t_msg, len - 1);
        msg[len - 1] = 0;
    }
    return gb::t_err;
}

void gb_clear_last_error(void)
{
    gb::t_err = GB_SUCCESS;
    gb::t_msg[0] = 0;
}

int64_t gb_launch_count(void) { return gb::g_launches.load(); }

int gb_last_ozaki_slices(void) { return gb::t_last_slices; }

int gb_test_trsv_wait_fault(int64_t withhold_block, int64_t wait_budget_ns)
{
    if (wait_budget_ns < 0 || (wait_budget_ns > 0 && wait_budget_ns < 100000) || wait_budget_ns > 10000000000ll)
        return gb::set_error(GB_ERR_ARG, "gb_test_trsv_wait_fault", "budget outside [0.1 ms, 10 s]");
    gb::g_trsv_withhold.store(withhold_block < 0 ? -1 : withhold_block);
    gb::g_trsv_wait_ns.store(wait_budget_ns == 0 ? gb::kWaitBudgetNs : (unsigned long long)wait_budget_ns);
    return GB_SUCCESS;
}

int gb_set_kernel_timing(int enable)
{
    gb::g_timing.store(enable ? 1 : 0);
    return GB_SUCCESS;
}

double gb_kernel_time_ms(const char* prefix, int64_t* launches)
{
    std::lock_guard<std::mutex> lk(gb::g_timing_mu);
    double total = 0.0;
    int64_t cnt = 0;
    size_t plen = prefix ? strlen(prefix) : 0;
    std::vector<gb::TimedLaunch> keep;
    for (auto& t : gb::g_timed) {
        if (plen == 0 || t.name.compare(0, plen, prefix) == 0) {
            cudaEventSynchronize(t.stop);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t.start, t.stop);
            total += ms;
            ++cnt;
            cudaEventDestroy(t.start);
            cudaEventDestroy(t.stop);
        } else {
            keep.push_back(t);
        }
    }
    gb::g_timed.swap(keep);
    if (launches) *launches = cnt;
    return total;
}

int64_t gb_kernel_trace(gb_trace_entry_t* out, int64_t max_entries)
{
    std::lock_guard<std::mutex> lk(gb::g_timing_mu);
    const int64_t n = (int64_t)gb::g_timed.size();
    if (n == 0) return 0;
    cudaEvent_t origin = gb::g_timed[0].start;
    for (auto& t : gb::g_timed) cudaEventSynchronize(t.stop);
    int64_t w = 0;
    for (auto& t : gb::g_timed) {
        if (out && w < max_entries) {
            float t0 = 0.f, t1 = 0.f;
            cudaEventElapsedTime(&t0, origin, t.start);
            cudaEventElapsedTime(&t1, origin, t.stop);
            gb_trace_entry_t& e = out[w];
            strncpy(e.name, t.name.c_str(), sizeof(e.name) - 1);
            e.name[sizeof(e.name) - 1] = 0;
            e.start_ms = t0;
            e.end_ms = t1;
            ++w;
        }
    }
    for (auto& t : gb::g_timed) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    gb::g_timed.clear();
    return w;
}

int gb_synchronize(void)
{
    int rc = gb::ensure_init();
    if (rc) return rc;
    GB_CUDA(cudaStreamSynchronize(gb::thread_stream()));
    return gb::read_and_clear_device_status(gb::thread_stream(), "gb_synchronize");
}

}  // extern "C"
