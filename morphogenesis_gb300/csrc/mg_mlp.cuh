// mg_mlp.cuh - the learned reaction surrogate: MLP 48 -> 128 -> 128 -> 16 with GELU.
//
// Inputs per particle: 16 concentrations (after diffusion and decay), 16 neighbour-mean
// concentrations (over the diffusion neighbours), both divided by the particle's largest
// concentration, and 16 gene bits as 0/1.  Output: the gene reaction's concentration increment
// over the same scale.  BF16 weights and activations, FP32 accumulation.  Training keeps FP32 master weights for Adam; inference uses weights with the
// input and output normalisation folded into the first and last layer.
#pragma once
#include <cstdint>
#include <cuda.h>  // CUtensorMap (types only; the encoder is looked up through the runtime)
#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace mg {

constexpr int MLP_IN = 48, MLP_H = 128, MLP_OUT = 16;
// FP32 parameter vector layout (normalised network): W1[128][48] b1[128] W2[128][128] b2[128]
// W3[16][128] b3[16]
constexpr int P_W1 = 0;
constexpr int P_B1 = P_W1 + MLP_H * MLP_IN;
constexpr int P_W2 = P_B1 + MLP_H;
constexpr int P_B2 = P_W2 + MLP_H * MLP_H;
constexpr int P_W3 = P_B2 + MLP_H;
constexpr int P_B3 = P_W3 + MLP_OUT * MLP_H;
constexpr int P_COUNT = P_B3 + MLP_OUT;  // 24848

// Inference weights (normalisation folded), device resident: bf16 matrices in the
// tcgen05 K-major core-matrix layout, fp32 biases.
struct InferWeights {
    __nv_bfloat16* w1;  // [128 x 48]  canonical layout
    __nv_bfloat16* w2;  // [128 x 128]
    __nv_bfloat16* w3;  // [16 x 128]
    float* b1;          // [128]
    float* b2;          // [128]
    float* b3;          // [16]
};

// Offset (in elements) of (row, k) inside a rows x K tile stored as 8x8 core matrices, K-major,
// no swizzle: core matrix (row/8, k/8) at ((row/8)*(K/8) + k/8)*64 elements, rows of 8 elements.
__host__ __device__ __forceinline__ uint32_t core_offset(uint32_t row, uint32_t k, uint32_t K) {
    return (((row >> 3) * (K >> 3) + (k >> 3)) << 6) + ((row & 7u) << 3) + (k & 7u);
}

// GELU in its tanh form (Hendrycks & Gimpel): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))),
// with the hardware tanh approximation (relative error below 2^-10, under the bf16 rounding
// the activations get anyway).
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float GELU_K0 = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float GELU_K1 = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    // 0.5 x (1 + tanh(x (k0 + k0 k1 x^2))) as four fused operations around the tanh
    const float u = x * __fmaf_rn(GELU_K0 * GELU_K1, x * x, GELU_K0);
    const float hx = 0.5f * x;
    return __fmaf_rn(hx, tanh_hw(u), hx);
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float u = x * __fmaf_rn(GELU_K0 * GELU_K1, x * x, GELU_K0);
    const float t = tanh_hw(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_K0 * (1.0f + 3.0f * GELU_K1 * x * x);
}

// ---- inference (tcgen05) --------------------------------------------------------------
// Error bits raised by the inference kernel.
enum : uint32_t { MLP_ERR_MBAR_TIMEOUT = 1u << 8 };

// Normalisation vector: mu_x[48] isd_x[48] mu_y[16] isd_y[16]
constexpr int NORM_COUNT = 2 * MLP_IN + 2 * MLP_OUT;

// One network: FP32 master parameters, gradients and Adam moments (device), BF16 copy for the
// training GEMMs, normalisation, folded inference weights and a training workspace.
struct Mlp {
    float* params;
    float* grads;
    float* adam_m;
    float* adam_v;
    __nv_bfloat16* wb;
    float* norm;
    uint32_t* err;  // MLP_ERR_* bits of the training GEMMs (bounded completion waits)
    InferWeights inf;
    void* inf_mem;
    void* ws;
    uint32_t ws_batch;
    int adam_t;
    cudaStream_t st;
};

inline uint64_t mix_seed(uint64_t seed, int step) {
    return seed * 0x9E3779B97F4A7C15ull + (uint64_t)step * 0xD1B54A32D192ED03ull + 1;
}

cudaError_t mlp_init_attributes();
cudaError_t mlp_alloc(Mlp* m, uint64_t seed, cudaStream_t st);
void mlp_free(Mlp* m);
// failure-detection self-test: the completion wait of an inference CTA whose MMAs are withheld
cudaError_t mlp_selftest_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st);
// failure-detection self-test: the completion wait of a training-GEMM CTA whose MMAs are withheld
cudaError_t mlp_selftest_gemm_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st);
cudaError_t mlp_set_params(Mlp* m, const float* host);
cudaError_t mlp_get_params(Mlp* m, float* host);
cudaError_t mlp_set_norm(Mlp* m, const float* host);
cudaError_t mlp_get_norm(Mlp* m, float* host);
cudaError_t mlp_refresh_inference(Mlp* m);
cudaError_t mlp_fit_norm(Mlp* m, const float* dx, const float* dy, uint64_t rows);
cudaError_t mlp_train(Mlp* m, const float* dx, const float* dy, uint64_t rows, uint32_t steps,
                      uint32_t batch, float lr, uint64_t seed, float* loss_host);
cudaError_t mlp_grad(Mlp* m, const float* dx, const float* dy, uint32_t n, float* grads_host,
                     double* loss);
// Tensor map of a [rows][48] bf16 feature matrix for the inference kernel's TMA loads: boxes
// of 8 features x 128 rows (one 2 KB plane of core matrices each), rows past `rows` read as 0.
cudaError_t make_feat_map(const __nv_bfloat16* feat, uint32_t rows, CUtensorMap* map);
void launch_mlp_infer(const Mlp* m, const CUtensorMap& feat_map, const float* feat_scale,
                      const float* conc_in,
                      const float* conc_plain, float* conc_out, uint32_t* genes,
                      const uint32_t* nactive, uint32_t n_override, const uint32_t* step,
                      uint32_t period, uint32_t stride, float threshold, uint32_t* stats,
                      uint32_t* err, int num_sms, cudaStream_t st);

}  // namespace mg
