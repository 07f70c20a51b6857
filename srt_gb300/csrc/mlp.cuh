// mlp.cuh — the radiance-cache network: 96 -> 64 -> 64 -> 64 -> 64 -> 64 -> 16
// (five hidden ReLU layers of width 64, RGB output through exp), BF16
// weights and activations, FP32 accumulation on the tensor cores
// (tcgen05.mma for inference, mma.sync m16n8k16 for training), no biases
// (a constant-1 input feature plays the first layer's bias).
//
// Inputs of one query (16 floats, four float4): position (3), roughness,
// shading normal (3), -, outgoing direction (3), -, albedo (3), -.  The
// position is normalised to the scene box and encoded with 12 octaves of
// sin/cos per axis (72 features); with the normal, direction, roughness,
// albedo and the constant it fills 83 of the 96 input columns.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"

namespace srt {

constexpr int kMlpIn = 96;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 16;    // 3 used
constexpr int kMlpLayers = 6;  // 5 hidden + output
constexpr int kMlpFreqs = 12;

// parameter offsets (row-major W_l[out][in]) in the packed parameter vector
__host__ __device__ constexpr int mlp_in(int l) { return l == 0 ? kMlpIn : kMlpHidden; }
__host__ __device__ constexpr int mlp_out(int l) { return l == kMlpLayers - 1 ? kMlpOut : kMlpHidden; }
__host__ __device__ constexpr int mlp_offset(int l)
{
    return l == 0 ? 0 : kMlpIn * kMlpHidden + (l - 1) * kMlpHidden * kMlpHidden;
}
constexpr int kMlpParams = kMlpIn * kMlpHidden + 4 * kMlpHidden * kMlpHidden + kMlpHidden * kMlpOut;  // 23552

// per-row activation storage for training: inputs of every layer (bf16)
constexpr int kActCols = kMlpIn + 5 * kMlpHidden;        // 416
constexpr int kGradCols = 5 * kMlpHidden + kMlpOut;       // 336: dZ of every layer
__host__ __device__ constexpr int act_col(int l) { return l == 0 ? 0 : kMlpIn + (l - 1) * kMlpHidden; }
__host__ __device__ constexpr int grad_col(int l) { return l * kMlpHidden; }

// Scene box used to normalise positions.
struct MlpBox {
    float3 lo;
    float3 inv_extent;
};

// Device view of the network for the tracer.
struct MlpView {
    const __nv_bfloat16* w;  // kMlpParams bf16
    MlpBox box;
};

}  // namespace srt

// Network state: FP32 master weights, BF16 copy, Adam moments, gradient.
struct srt_mlp {
    srt::DeviceBuffer params;  // fp32 master | adam m | adam v | grad | loss | bf16 copy | bf16 packed
    float* wf = nullptr;
    __nv_bfloat16* wb = nullptr;
    __nv_bfloat16* wpack = nullptr;  // bf16 weights in the tensor cores' canonical layout (umma.cuh)
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    float* loss = nullptr;
    srt::DeviceBuffer scratch;  // per-row layer inputs and gradients for training
    srt::DeviceBuffer partial;  // per-chunk weight gradients, summed in a fixed order
    int64_t scratch_rows = 0;
    srt::MlpBox box{};
    int64_t step = 0;
    float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
};

namespace srt {
// refreshes the packed weights from the FP32 master weights
srt_status mlp_pack(srt_mlp* p, cudaStream_t st);
srt_status mlp_infer_launch(const srt_mlp* p, const float4* rec, int64_t n, float4* out, cudaStream_t st);
srt_status mlp_train_launch(srt_mlp* p, const float4* rec, const float4* target, int64_t n, float lr, bool update,
                            cudaStream_t st);
}  // namespace srt
