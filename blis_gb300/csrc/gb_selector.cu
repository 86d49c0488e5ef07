// gb_selector.cu -- the learned configuration selector inside the library.
//
// A trained MLP (gb_mlp.cu) is loaded from a checked binary blob; for a GEMM
// shape it predicts the log-time of every configuration of
// gb_gemm_config_dev and the Ozaki slice count.  Host entry points use it
// when auto-selection is on: the configuration of least predicted time,
// and in the Ozaki "auto" mode the proposed slice count, checked by the
// error-bound verifier and raised if it fails.  Inference runs on the GPU
// (one sample per new shape; results are cached per shape).
//
// By default the host entry points use the model committed next to the
// library (tuning/selector_mlp.bin, loaded on first use unless the caller
// loaded, unloaded or switched the selector off first, or GB_SELECTOR=rule).
// Without a model, an occupancy rule stands in for BLIS's small-problem
// thresholds (frame/base/bli_cntx.h:186-193): 128x128 tiles when they fill
// the SMs, else the 64x64 engine with the least split of K that gives two
// waves of CTAs (on the 13,334 FP64/FP32 autotuned shapes: mean regret 0.71 /
// 0.20 against 3.19 / 2.21 for the threshold rule).
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "gb_internal.h"

namespace gb {
namespace {

constexpr double kWorkCap = 34359738368.0;  // 2^35 flops: above the trained range use config 0
std::mutex g_mu;
float* g_params = nullptr;  // device copy of the MLP parameters
float* g_io = nullptr;      // device scratch: 16 features + 8 outputs
bool g_loaded = false;
bool g_engine_output = false;  // the loaded model was trained with the Ozaki engine output (file version 2)
bool g_auto = false;
bool g_user_configured = false;  // the caller loaded, unloaded or switched the selector itself
std::once_flag g_default_once;
std::unordered_map<uint64_t, uint64_t> g_cache;

uint32_t crc32_bytes(const unsigned char* p, size_t n)
{
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) {
        c ^= p[i];
        for (int b = 0; b < 8; ++b) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return c ^ 0xFFFFFFFFu;
}

// Same feature map as blis_gb300/selector.py:features().
void features(float* f, int64_t m, int64_t n, int64_t k, int dtype, int ta, int tb, int pad, double sa, double sb)
{
    for (int i = 0; i < GB_MLP_IN; ++i) f[i] = 0.0f;
    f[0] = (float)(log2((double)m + 1) / 15.0);
    f[1] = (float)(log2((double)n + 1) / 15.0);
    f[2] = (float)(log2((double)k + 1) / 15.0);
    f[3 + (dtype == 0 ? 0 : (dtype == 1 ? 1 : 2))] = 1.0f;
    f[6] = (float)ta;
    f[7] = (float)tb;
    f[8 + (pad >= 64 ? 2 : (pad >= 8 ? 1 : 0))] = 1.0f;
    f[11] = (float)(sa / 40.0);
    f[12] = (float)(sb / 40.0);
    f[13] = (float)(log2((double)m * (double)n + 1) / 30.0);
    f[14] = (float)(log2((double)m * (double)n * (double)k + 1) / 45.0);
    f[15] = (m < n ? m : n) <= 64 ? 1.0f : 0.0f;
}

uint64_t key_of(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad, int qa, int qb)
{
    uint64_t h = 1469598103934665603ull;
    const uint64_t v[9] = {(uint64_t)dtype, (uint64_t)m, (uint64_t)n, (uint64_t)k, (uint64_t)ta,
                           (uint64_t)tb, (uint64_t)pad, (uint64_t)qa, (uint64_t)qb};
    for (uint64_t x : v) {
        h ^= x + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
        h *= 1099511628211ull;
    }
    return h;
}

}  // namespace

namespace {
// Reads a model file (magic, version, parameter count, CRC-32 of the parameters).
// Version 1: configuration times and slice count; version 2 adds the Ozaki engine output.
bool read_model_file(const char* path, float* p, int* version)
{
    FILE* f = path ? fopen(path, "rb") : nullptr;
    if (!f) return false;
    char magic[8];
    uint32_t hdr[3];
    const bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "GBSELMLP", 8) == 0 &&
                    fread(hdr, sizeof(uint32_t), 3, f) == 3 && (hdr[0] == 1 || hdr[0] == 2) &&
                    hdr[1] == GB_MLP_NPARAMS &&
                    fread(p, sizeof(float), GB_MLP_NPARAMS, f) == GB_MLP_NPARAMS &&
                    crc32_bytes(reinterpret_cast<const unsigned char*>(p), sizeof(float) * GB_MLP_NPARAMS) == hdr[2];
    fclose(f);
    if (ok && version) *version = (int)hdr[0];
    return ok;
}

// Copies the parameters to the device.  A load the caller asked for (user) takes
// charge of the selector; the default load switches auto-selection on unless the
// caller already decided.
int load_params(const float* params, bool user, bool engine_output)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!user && g_user_configured) return GB_SUCCESS;
    g_engine_output = engine_output;
    if (!g_params) {
        GB_CUDA(cudaMalloc(&g_params, sizeof(float) * GB_MLP_NPARAMS));
        GB_CUDA(cudaMalloc(&g_io, sizeof(float) * (GB_MLP_IN + GB_MLP_OUT)));
    }
    GB_CUDA(cudaMemcpy(g_params, params, sizeof(float) * GB_MLP_NPARAMS, cudaMemcpyHostToDevice));
    g_cache.clear();
    g_loaded = true;
    if (user) g_user_configured = true;
    else g_auto = true;
    return GB_SUCCESS;
}
}  // namespace

// The occupancy rule: config 0 (128x128 tiles) when its tiles cover the SMs,
// else the 64x64 engine (configs 1..5 = K split 1, 2, 4, 8, 16) with the least
// split that reaches two waves of CTAs or would leave fewer than 128 values of
// k per part.
int selector_heuristic(int64_t m, int64_t n, int64_t k)
{
    const int64_t sms = sm_count();
    const int64_t t128 = ((m + 127) / 128) * ((n + 127) / 128);
    if (t128 >= sms) return 0;
    const int64_t t64 = ((m + 63) / 64) * ((n + 63) / 64);
    for (int c = 1; c < GB_GEMM_NUM_CONFIGS; ++c) {
        const int64_t split = int64_t(1) << (c - 1);
        if (t64 * split >= 2 * sms || k / (2 * split) < 128) return c;
    }
    return GB_GEMM_NUM_CONFIGS - 1;
}

namespace {
// tuning/selector_mlp.bin beside this library, when the caller has not taken charge
void load_default_model()
{
    const char* env = getenv("GB_SELECTOR");
    if (env && (strcmp(env, "rule") == 0 || strcmp(env, "off") == 0)) return;
    Dl_info info;
    if (!dladdr(reinterpret_cast<void*>(&load_default_model), &info) || !info.dli_fname) return;
    std::string path(info.dli_fname);
    const size_t slash = path.rfind('/');
    path = (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/tuning/selector_mlp.bin";
    if (access(path.c_str(), R_OK) != 0) return;
    std::vector<float> p(GB_MLP_NPARAMS);
    int version = 0;
    if (!read_model_file(path.c_str(), p.data(), &version)) return;
    if (ensure_init() != GB_SUCCESS || load_params(p.data(), false, version >= 2) != GB_SUCCESS)
        gb_clear_last_error();
}
}  // namespace

bool selector_auto()
{
    std::call_once(g_default_once, load_default_model);
    return g_auto && g_loaded;
}

// Config (0..GB_GEMM_NUM_CONFIGS-1) and proposed Ozaki slice count for a shape.
int selector_choose(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad, double sa, double sb,
                    int* config, int* slices)
{
    return selector_choose_ex(dtype, m, n, k, ta, tb, pad, sa, sb, config, slices, nullptr);
}

// Config, proposed slice count and (engine != nullptr) Ozaki engine for a shape.
int selector_choose_ex(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad, double sa, double sb,
                       int* config, int* slices, int* engine)
{
    *config = selector_heuristic(m, n, k);
    *slices = 8;
    if (engine) *engine = 0;
    if (!g_loaded) return GB_SUCCESS;
    if (2.0 * (double)m * (double)n * (double)k > kWorkCap) {
        *config = 0;
        if (engine) *engine = 2;  // above the trained range: the pairs' large tiles
        return GB_SUCCESS;
    }
    const uint64_t key = key_of(dtype, m, n, k, ta, tb, pad, (int)lround(sa), (int)lround(sb));
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
        *config = (int)(it->second & 0xFF);
        *slices = (int)((it->second >> 8) & 0xFF);
        if (engine) *engine = (int)((it->second >> 16) & 0xFF);
        return GB_SUCCESS;
    }
    float host[GB_MLP_IN + GB_MLP_OUT];
    features(host, m, n, k, dtype, ta, tb, pad, sa, sb);
    cudaStream_t s = thread_stream();
    GB_CUDA(cudaMemcpyAsync(g_io, host, sizeof(float) * GB_MLP_IN, cudaMemcpyHostToDevice, s));
    int rc = gb_mlp_forward_dev(g_params, g_io, 1, g_io + GB_MLP_IN, s);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(host + GB_MLP_IN, g_io + GB_MLP_IN, sizeof(float) * GB_MLP_OUT, cudaMemcpyDeviceToHost,
                            s));
    GB_CUDA(cudaStreamSynchronize(s));
    const float* out = host + GB_MLP_IN;
    int best = 0;
    for (int c = 1; c < GB_GEMM_NUM_CONFIGS; ++c)
        if (out[c] < out[best]) best = c;
    int sl = (int)ceil(out[GB_GEMM_NUM_CONFIGS] * 12.0 - 0.25);
    sl = sl < 2 ? 2 : (sl > 12 ? 12 : sl);
    // engine output: log2(t_one_cta / t_pair) / 10 for the Ozaki form, positive when the
    // CTA pairs are faster (models trained before it carry a zero output: pairs)
    const int eng = (out[GB_MLP_OUT - 1] >= 0.0f) ? 2 : 1;
    *config = best;
    *slices = sl;
    if (engine) *engine = eng;
    g_cache[key] = (uint64_t)best | ((uint64_t)sl << 8) | ((uint64_t)eng << 16);
    return GB_SUCCESS;
}

int selector_ozaki_engine(int64_t m, int64_t n, int64_t k, int* engine)
{
    *engine = 0;
    if (!g_loaded || !g_engine_output) return GB_SUCCESS;
    int cfg = 0, sl = 0;
    return selector_choose_ex(0, m, n, k, 0, 0, 0, 0.0, 0.0, &cfg, &sl, engine);
}

// The configuration of an already decided shape (no inference, no synchronization), or -1.
int selector_cached_config(int dtype, int64_t m, int64_t n, int64_t k, int ta, int tb, int pad)
{
    if (!g_loaded) return -1;
    if (2.0 * (double)m * (double)n * (double)k > kWorkCap) return 0;
    const uint64_t key = key_of(dtype, m, n, k, ta, tb, pad, 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    return (it == g_cache.end()) ? -1 : (int)(it->second & 0xFF);
}

// The engine of an already decided shape (no inference, no synchronization), or 0.
int selector_cached_engine(int64_t m, int64_t n, int64_t k)
{
    if (!g_loaded || !g_engine_output) return 0;
    if (2.0 * (double)m * (double)n * (double)k > kWorkCap) return 2;
    const uint64_t key = key_of(0, m, n, k, 0, 0, 0, 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    return (it == g_cache.end()) ? 0 : (int)((it->second >> 16) & 0xFF);
}

// Binary exponent half-range over a strided sample of a host matrix, the
// statistic the selector was trained on.
double host_exponent_spread(const double* x, int64_t rows, int64_t cols, int64_t rs, int64_t cs)
{
    if (rows <= 0 || cols <= 0) return 0.0;
    const int64_t total = rows * cols;
    const int64_t step = total > 4096 ? total / 4096 : 1;
    int lo = 100000, hi = -100000;
    for (int64_t e = 0; e < total; e += step) {
        const double v = x[(e % rows) * rs + (e / rows) * cs];
        if (v == 0.0 || !isfinite(v)) continue;
        int ex;
        frexp(v, &ex);
        lo = ex < lo ? ex : lo;
        hi = ex > hi ? ex : hi;
    }
    return hi >= lo ? 0.5 * (hi - lo) : 0.0;
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_selector_load(const float* params, int nparams)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (!params || nparams != GB_MLP_NPARAMS)
        return set_error(GB_ERR_ARG, "gb_selector_load", "expected GB_MLP_NPARAMS parameters");
    return load_params(params, true, false);
}

int gb_selector_load_file(const char* path)
{
    std::vector<float> p(GB_MLP_NPARAMS);
    int version = 0;
    if (!read_model_file(path, p.data(), &version))
        return set_error(GB_ERR_ARG, "gb_selector_load_file", "cannot open the model file, or bad magic, version, "
                                                              "size or checksum");
    int rc = ensure_init();
    if (rc) return rc;
    return load_params(p.data(), true, version >= 2);
}

int gb_selector_unload(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_user_configured = true;
    g_loaded = false;
    g_cache.clear();
    return GB_SUCCESS;
}

int gb_set_gemm_autoselect(int on)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_user_configured = true;
    g_auto = on != 0;
    return GB_SUCCESS;
}

int gb_selector_choose(int dtype, gb_dim_t m, gb_dim_t n, gb_dim_t k, int transa, int transb, int pad,
                       double spread_a, double spread_b, int* config, int* slices)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (!config || !slices) return set_error(GB_ERR_ARG, "gb_selector_choose", "null output");
    return selector_choose(dtype, m, n, k, transa ? 1 : 0, transb ? 1 : 0, pad, spread_a, spread_b, config, slices);
}

}  // extern "C"
