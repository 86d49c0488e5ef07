// gb_mlp.cu -- the learned configuration selector's network: a 16-64-64-64-8
// MLP with GELU activations in FP32, with hand-written forward, backward and
// Adam kernels (no reference counterpart; BLIS picks kernels from static
// per-architecture tables, config/<arch>/bli_cntx_init_<arch>.c).
//
// Parameters are one contiguous FP32 vector:
//   W1[64][16] b1[64]  W2[64][64] b2[64]  W3[64][64] b3[64]  W4[8][64] b4[8]
// Inputs are 16 shape/dtype/layout/exponent features, outputs 8 targets
// (predicted log-times of the GEMM configs and the Ozaki slice count).  The
// loss is a masked mean squared error.  Each block owns a fixed slice of the
// batch and accumulates its gradient in shared memory (every thread owns
// one column of each weight matrix, so there are no atomics); a second
// kernel folds the per-block partials in block order.  Gradients are
// therefore bitwise reproducible.
#include <math.h>

#include "gb_internal.h"

namespace gb {
namespace {

constexpr int NIN = GB_MLP_IN, NH = GB_MLP_HIDDEN, NOUT = GB_MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN;
constexpr int OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NH;
constexpr int OFF_W4 = OFF_B3 + NH, OFF_B4 = OFF_W4 + NOUT * NH;
constexpr int NPARAM = OFF_B4 + NOUT;
static_assert(NPARAM == GB_MLP_NPARAMS, "parameter count");
constexpr int MLP_THREADS = 64;  // one thread per hidden unit

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z)
{
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = expf(-0.5f * z * z) * 0.39894228040143268f;
    return cdf + z * pdf;
}

// Weights are staged transposed in shared memory (wt[in][out]) so that the
// threads of a layer (one per output unit) read consecutive addresses.
struct MlpSmem {
    float w1t[NIN][NH], w2t[NH][NH], w3t[NH][NH], w4t[NH][NOUT];
    float b1[NH], b2[NH], b3[NH], b4[NOUT];
    float x[NIN], z1[NH], a1[NH], z2[NH], a2[NH], z3[NH], a3[NH], out[NOUT], g4[NOUT];
    float g3[NH], g2[NH], g1[NH];
};

__device__ void stage_weights(const float* __restrict__ p, MlpSmem& s)
{
    for (int e = threadIdx.x; e < NH * NIN; e += blockDim.x) s.w1t[e % NIN][e / NIN] = p[OFF_W1 + e];
    for (int e = threadIdx.x; e < NH * NH; e += blockDim.x) {
        s.w2t[e % NH][e / NH] = p[OFF_W2 + e];
        s.w3t[e % NH][e / NH] = p[OFF_W3 + e];
    }
    for (int e = threadIdx.x; e < NOUT * NH; e += blockDim.x) s.w4t[e % NH][e / NH] = p[OFF_W4 + e];
    for (int e = threadIdx.x; e < NH; e += blockDim.x) {
        s.b1[e] = p[OFF_B1 + e];
        s.b2[e] = p[OFF_B2 + e];
        s.b3[e] = p[OFF_B3 + e];
    }
    if (threadIdx.x < NOUT) s.b4[threadIdx.x] = p[OFF_B4 + threadIdx.x];
}

__device__ void forward_one(const float* __restrict__ x, MlpSmem& s)
{
    const int j = threadIdx.x;
    if (j < NIN) s.x[j] = x[j];
    __syncthreads();
    float z = s.b1[j];
#pragma unroll
    for (int i = 0; i < NIN; ++i) z = fmaf(s.w1t[i][j], s.x[i], z);
    s.z1[j] = z;
    s.a1[j] = gelu(z);
    __syncthreads();
    z = s.b2[j];
#pragma unroll 8
    for (int i = 0; i < NH; ++i) z = fmaf(s.w2t[i][j], s.a1[i], z);
    s.z2[j] = z;
    s.a2[j] = gelu(z);
    __syncthreads();
    z = s.b3[j];
#pragma unroll 8
    for (int i = 0; i < NH; ++i) z = fmaf(s.w3t[i][j], s.a2[i], z);
    s.z3[j] = z;
    s.a3[j] = gelu(z);
    __syncthreads();
    if (j < NOUT) {
        float o = s.b4[j];
#pragma unroll 8
        for (int i = 0; i < NH; ++i) o = fmaf(s.w4t[i][j], s.a3[i], o);
        s.out[j] = o;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(MLP_THREADS) mlp_forward_kernel(const float* __restrict__ params,
                                                                  const float* __restrict__ x, int64_t batch,
                                                                  float* __restrict__ out)
{
    extern __shared__ float smem_f[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(smem_f);
    stage_weights(params, s);
    __syncthreads();
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        forward_one(x + b * NIN, s);
        if (threadIdx.x < NOUT) out[b * NOUT + threadIdx.x] = s.out[threadIdx.x];
        __syncthreads();
    }
}

// Per-block gradient of sum_b sum_o mask*(out-y)^2 / norm over samples
// b = blockIdx.x, blockIdx.x + gridDim.x, ...; also the block's loss sum.
__global__ void __launch_bounds__(MLP_THREADS) mlp_grad_kernel(const float* __restrict__ params,
                                                               const float* __restrict__ x,
                                                               const float* __restrict__ y,
                                                               const float* __restrict__ mask, int64_t batch,
                                                               float inv_norm, float* __restrict__ partial,
                                                               float* __restrict__ loss_partial)
{
    extern __shared__ float smem_f[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(smem_f);
    float* g = smem_f + sizeof(MlpSmem) / sizeof(float);  // NPARAM gradient accumulators
    stage_weights(params, s);
    for (int e = threadIdx.x; e < NPARAM; e += blockDim.x) g[e] = 0.0f;
    __syncthreads();
    const int t = threadIdx.x;
    float loss = 0.0f;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        forward_one(x + b * NIN, s);
        if (t < NOUT) {
            const float mk = mask[b * NOUT + t];
            const float d = s.out[t] - y[b * NOUT + t];
            s.g4[t] = 2.0f * mk * d * inv_norm;
            if (t == 0) {
                float l = 0.0f;
                for (int o = 0; o < NOUT; ++o) {
                    const float dd = s.out[o] - y[b * NOUT + o];
                    l += mask[b * NOUT + o] * dd * dd;
                }
                loss += l * inv_norm;
            }
        }
        __syncthreads();
        // output layer: thread t owns column t of W4 (input unit t)
#pragma unroll
        for (int o = 0; o < NOUT; ++o) g[OFF_W4 + o * NH + t] += s.g4[o] * s.a3[t];
        if (t < NOUT) g[OFF_B4 + t] += s.g4[t];
        {
            float acc = 0.0f;
#pragma unroll
            for (int o = 0; o < NOUT; ++o) acc = fmaf(s.w4t[t][o], s.g4[o], acc);
            s.g3[t] = acc * gelu_grad(s.z3[t]);
        }
        __syncthreads();
        for (int j = 0; j < NH; ++j) g[OFF_W3 + j * NH + t] += s.g3[j] * s.a2[t];
        g[OFF_B3 + t] += s.g3[t];
        {
            float acc = 0.0f;
            for (int j = 0; j < NH; ++j) acc = fmaf(s.w3t[t][j], s.g3[j], acc);
            s.g2[t] = acc * gelu_grad(s.z2[t]);
        }
        __syncthreads();
        for (int j = 0; j < NH; ++j) g[OFF_W2 + j * NH + t] += s.g2[j] * s.a1[t];
        g[OFF_B2 + t] += s.g2[t];
        {
            float acc = 0.0f;
            for (int j = 0; j < NH; ++j) acc = fmaf(s.w2t[t][j], s.g2[j], acc);
            s.g1[t] = acc * gelu_grad(s.z1[t]);
        }
        __syncthreads();
        if (t < NIN)
            for (int j = 0; j < NH; ++j) g[OFF_W1 + j * NIN + t] += s.g1[j] * s.x[t];
        g[OFF_B1 + t] += s.g1[t];
        __syncthreads();
    }
    for (int e = threadIdx.x; e < NPARAM; e += blockDim.x) partial[(int64_t)blockIdx.x * NPARAM + e] = g[e];
    if (threadIdx.x == 0) loss_partial[blockIdx.x] = loss;
}

__global__ void mlp_fold_kernel(const float* __restrict__ partial, int nblk, float* __restrict__ grad,
                                const float* __restrict__ loss_partial, float* __restrict__ loss)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < NPARAM) {
        float acc = 0.0f;
        for (int b = 0; b < nblk; ++b) acc += partial[(int64_t)b * NPARAM + e];
        grad[e] = acc;
    }
    if (e == 0 && loss) {
        float l = 0.0f;
        for (int b = 0; b < nblk; ++b) l += loss_partial[b];
        *loss = l;
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                            float bc1, float bc2, float wd)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float ge = g[e] + wd * p[e];
        const float me = b1 * m[e] + (1.0f - b1) * ge;
        const float ve = b2 * v[e] + (1.0f - b2) * ge * ge;
        m[e] = me;
        v[e] = ve;
        p[e] -= lr * (me / bc1) / (sqrtf(ve / bc2) + eps);
    }
}

constexpr size_t kFwdSmem = sizeof(MlpSmem);
constexpr size_t kGradSmem = sizeof(MlpSmem) + sizeof(float) * NPARAM;
constexpr int kGradBlocks = 128;

bool mlp_attrs()
{
    static int done = 0;
    if (!done) {
        if (cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem) !=
                cudaSuccess)
            return false;
        done = 1;
    }
    return true;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gb_mlp_forward_dev(const float* params, const float* x, gb_dim_t batch, float* out, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (batch <= 0) return GB_SUCCESS;
    if (!mlp_attrs()) return set_error(GB_ERR_CUDA, "gb_mlp_forward_dev", "shared-memory attribute");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    int64_t blocks = batch < 4096 ? batch : 4096;
    LaunchScope ls("mlp_forward", s);
    mlp_forward_kernel<<<(unsigned)blocks, MLP_THREADS, kFwdSmem, s>>>(params, x, batch, out);
    return check_cuda(cudaGetLastError(), "gb_mlp_forward_dev");
}

int gb_mlp_loss_grad_dev(const float* params, const float* x, const float* y, const float* mask, gb_dim_t batch,
                         float norm, float* grad, float* loss, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (batch <= 0 || norm <= 0.0f) return set_error(GB_ERR_ARG, "gb_mlp_loss_grad_dev", "empty batch");
    if (!mlp_attrs()) return set_error(GB_ERR_CUDA, "gb_mlp_loss_grad_dev", "shared-memory attribute");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    const int nblk = (int)(batch < kGradBlocks ? batch : kGradBlocks);
    float* partial = static_cast<float*>(dev_alloc(sizeof(float) * ((size_t)nblk * NPARAM + nblk), s));
    if (!partial) return GB_ERR_NOMEM;
    {
        LaunchScope ls("mlp_grad", s);
        mlp_grad_kernel<<<nblk, MLP_THREADS, kGradSmem, s>>>(params, x, y, mask, batch, 1.0f / norm, partial,
                                                             partial + (size_t)nblk * NPARAM);
    }
    {
        LaunchScope ls("mlp_fold", s);
        mlp_fold_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(partial, nblk, grad, partial + (size_t)nblk * NPARAM,
                                                            loss);
    }
    rc = check_cuda(cudaGetLastError(), "gb_mlp_loss_grad_dev");
    dev_free(partial, s);
    return rc;
}

int gb_mlp_adam_dev(float* params, const float* grad, float* m, float* v, gb_dim_t n, float lr, float beta1,
                    float beta2, float eps, float weight_decay, int step, void* stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (step < 1) return set_error(GB_ERR_ARG, "gb_mlp_adam_dev", "step counts from 1");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : thread_stream();
    const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    LaunchScope ls("mlp_adam", s);
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(params, grad, m, v, n, lr, beta1, beta2, eps, bc1, bc2,
                                                            weight_decay);
    return check_cuda(cudaGetLastError(), "gb_mlp_adam_dev");
}

}  // extern "C"
