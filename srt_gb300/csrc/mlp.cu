// mlp.cu — fused BF16 tensor-core kernels of the radiance-cache network
// (see mlp.cuh): inference (tcgen05.mma with TMEM accumulators, the fused
// kernel of umma_mlp.cuh: standalone and the tracer's cache queries),
// forward+backward-data for training, weight gradients (mma.sync), Adam.
// The reference's learned part (tiny-cuda-nn HashGrid + CutlassMLP,
// src/passes/npr/neural_radiosity.cu:6-52) is an un-vendored library; the
// network here is a plain fully fused MLP.
//
// Fragment layout (mma.sync m16n8k16, bf16 inputs, f32 accumulators), lane
// = 4*g + t: A regs {0,1,2,3} hold (row g, cols 2t..2t+1), (row g+8, same),
// (row g, cols 2t+8..), (row g+8, cols 2t+8..); B regs hold (k = 2t..2t+1,
// n = g) and (k = 2t+8.., n = g); C holds (row g, cols 2t..2t+1), (row g+8,
// same).  The C fragments of n-tiles 2k and 2k+1 are exactly the A
// fragment of k-tile k, so activations stay in registers between layers.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "mlp.cuh"
#include "umma_mlp.cuh"
#include "wavefront.cuh"

namespace srt {

namespace {

constexpr int kMlpThreads = 128;  // 4 warps, 16 rows per warp per tile

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// shared-memory layouts: W_l[out][in + 8] and W_l^T[in][out + 8] (padding
// makes the fragment loads bank-conflict free)
__host__ __device__ constexpr int w_stride(int l) { return mlp_in(l) + 8; }
__host__ __device__ constexpr int wt_stride(int l) { return mlp_out(l) + 8; }
__host__ __device__ constexpr int w_smem_off(int l)
{
    int o = 0;
    for (int k = 0; k < l; ++k) o += mlp_out(k) * w_stride(k);
    return o;
}
constexpr int kWSmem = w_smem_off(kMlpLayers);  // bf16 elements
__host__ __device__ constexpr int wt_smem_off(int l)
{
    int o = 0;
    for (int k = 1; k < l; ++k) o += mlp_in(k) * wt_stride(k);
    return o;
}
constexpr int kWtSmem = wt_smem_off(kMlpLayers);

__device__ void load_weights(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* ws, __nv_bfloat16* wts)
{
    for (int l = 0; l < kMlpLayers; ++l) {
        const int in = mlp_in(l), out = mlp_out(l);
        const __nv_bfloat16* src = w + mlp_offset(l);
        for (int i = threadIdx.x; i < in * out; i += blockDim.x) {
            int o = i / in, k = i % in;
            __nv_bfloat16 v = src[i];
            ws[w_smem_off(l) + o * w_stride(l) + k] = v;
            if (wts && l >= 1) wts[wt_smem_off(l) + k * wt_stride(l) + o] = v;
        }
    }
    __syncthreads();
}

// C[NT] += A[KT] x B where B fragments come from a [n][k] bf16 matrix with
// row stride `stride` (W for the forward pass, W^T for the backward pass).
template <int KT, int NT>
__device__ __forceinline__ void gemm_tile(const uint32_t (&a)[KT][4], const __nv_bfloat16* m, int stride,
                                          float (&c)[NT][4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __nv_bfloat16* p = m + (nt * 8 + g) * stride + kt * 16 + 2 * t;
            uint32_t b0 = *reinterpret_cast<const uint32_t*>(p);
            uint32_t b1 = *reinterpret_cast<const uint32_t*>(p + 8);
            mma16816(c[nt], a[kt], b0, b1);
        }
    }
}

// ReLU'd C fragments of a 64-wide layer -> A fragments of the next layer,
// plus the ReLU derivative mask (bit 4*nt + e).
__device__ __forceinline__ void relu_to_a(const float (&c)[8][4], uint32_t (&a)[4][4], uint32_t& mask)
{
    mask = 0;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) mask |= (c[nt][e] > 0.0f ? 1u : 0u) << (4 * nt + e);
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        a[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        a[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        a[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
}

// dA (C fragments) * ReLU mask -> dZ as A fragments
template <int NT>
__device__ __forceinline__ void mask_to_a(const float (&c)[NT][4], uint32_t mask, uint32_t (&a)[NT / 2][4])
{
    float v[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) v[nt][e] = ((mask >> (4 * nt + e)) & 1u) ? c[nt][e] : 0.0f;
#pragma unroll
    for (int kt = 0; kt < NT / 2; ++kt) {
        a[kt][0] = pack_bf16(v[2 * kt][0], v[2 * kt][1]);
        a[kt][1] = pack_bf16(v[2 * kt][2], v[2 * kt][3]);
        a[kt][2] = pack_bf16(v[2 * kt + 1][0], v[2 * kt + 1][1]);
        a[kt][3] = pack_bf16(v[2 * kt + 1][2], v[2 * kt + 1][3]);
    }
}

// two input features starting at the even column `col` of one query record
__device__ __forceinline__ float2 feature_pair(const float4 (&r)[4], const MlpBox& box, int col)
{
    if (col < 72) {
        int a = col / 24, j = (col % 24) >> 1;
        float p = a == 0 ? (r[0].x - box.lo.x) * box.inv_extent.x
                : a == 1 ? (r[0].y - box.lo.y) * box.inv_extent.y
                         : (r[0].z - box.lo.z) * box.inv_extent.z;
        float s, c;
        sincospif(ldexpf(p, j), &s, &c);
        return make_float2(s, c);
    }
    switch (col) {
    case 72: return make_float2(r[1].x, r[1].y);
    case 74: return make_float2(r[1].z, r[2].x);
    case 76: return make_float2(r[2].y, r[2].z);
    case 78: return make_float2(r[0].w, r[3].x);
    case 80: return make_float2(r[3].y, r[3].z);
    case 82: return make_float2(1.0f, 0.0f);
    default: return make_float2(0.0f, 0.0f);
    }
}

// input A fragments (6 k-tiles) for rows g and g+8 of a 16-row tile
__device__ __forceinline__ void input_fragments(const float4 (&r0)[4], const float4 (&r1)[4], bool v0, bool v1,
                                                const MlpBox& box, uint32_t (&a)[6][4])
{
    const int t = threadIdx.x & 3;
#pragma unroll
    for (int kt = 0; kt < 6; ++kt) {
#pragma unroll
        for (int reg = 0; reg < 4; ++reg) {
            int col = kt * 16 + 2 * t + ((reg & 2) ? 8 : 0);
            bool hi = reg & 1;
            float2 f = (hi ? v1 : v0) ? feature_pair(hi ? r1 : r0, box, col) : make_float2(0.f, 0.f);
            a[kt][reg] = pack_bf16(f.x, f.y);
        }
    }
}

__device__ __forceinline__ void load_record(const float4* __restrict__ rec, int64_t row, bool valid, float4 (&r)[4])
{
#pragma unroll
    for (int k = 0; k < 4; ++k) r[k] = valid ? __ldg(rec + 4 * row + k) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// forward through the five hidden layers; returns the output-layer C
// fragments (2 n-tiles) and, if requested, stores layer inputs and masks
template <bool kStore>
__device__ __forceinline__ void forward_tile(const __nv_bfloat16* ws, const uint32_t (&a0)[6][4], float (&z)[2][4],
                                             uint32_t (&masks)[5], uint32_t (*a_out)[4][4])
{
    float c[8][4];
    uint32_t a[4][4];
    gemm_tile<6, 8>(a0, ws + w_smem_off(0), w_stride(0), c);
    relu_to_a(c, a, masks[0]);
    if (kStore) {
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int e = 0; e < 4; ++e) a_out[0][kt][e] = a[kt][e];
    }
#pragma unroll
    for (int l = 1; l < 5; ++l) {
        gemm_tile<4, 8>(a, ws + w_smem_off(l), w_stride(l), c);
        relu_to_a(c, a, masks[l]);
        if (kStore) {
#pragma unroll
            for (int kt = 0; kt < 4; ++kt)
#pragma unroll
                for (int e = 0; e < 4; ++e) a_out[l][kt][e] = a[kt][e];
        }
    }
    gemm_tile<4, 2>(a, ws + w_smem_off(5), w_stride(5), z);
}

__device__ __forceinline__ float safe_exp(float z) { return __expf(fminf(z, 15.0f)); }

// Forward + relative-L2 loss + backward-data for one 16-row tile per warp.
// Stores the input of every layer (act) and dL/dz of every layer (dz) as
// bf16 rows for the weight-gradient kernel.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_train(const __nv_bfloat16* __restrict__ w, MlpBox box,
                                                           const float4* __restrict__ rec,
                                                           const float4* __restrict__ target, int64_t n,
                                                           __nv_bfloat16* __restrict__ act,
                                                           __nv_bfloat16* __restrict__ dz, float* loss_sum)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* ws = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* wts = ws + kWSmem;
    load_weights(w, ws, wts);
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warp = threadIdx.x >> 5;
    const int64_t tiles = (n + 15) / 16;
    const float inv_count = 1.0f / (3.0f * (float)n);
    float loss = 0.0f;
    for (int64_t tile = (int64_t)blockIdx.x * 4 + warp; tile < tiles; tile += (int64_t)gridDim.x * 4) {
        int64_t r0 = tile * 16 + g, r1 = r0 + 8;
        bool v0 = r0 < n, v1 = r1 < n;
        float4 q0[4], q1[4];
        load_record(rec, r0, v0, q0);
        load_record(rec, r1, v1, q1);
        uint32_t a0[6][4];
        input_fragments(q0, q1, v0, v1, box, a0);
        uint32_t ah[5][4][4];
        float z[2][4];
        uint32_t masks[5];
        forward_tile<true>(ws, a0, z, masks, ah);
        // store layer inputs: A0 (96 cols) and A1..A5 (64 cols)
        auto store_a = [&](int col0, int kt, const uint32_t (&f)[4]) {
            int c = col0 + kt * 16 + 2 * t;
            if (v0) {
                *reinterpret_cast<uint32_t*>(act + r0 * kActCols + c) = f[0];
                *reinterpret_cast<uint32_t*>(act + r0 * kActCols + c + 8) = f[2];
            }
            if (v1) {
                *reinterpret_cast<uint32_t*>(act + r1 * kActCols + c) = f[1];
                *reinterpret_cast<uint32_t*>(act + r1 * kActCols + c + 8) = f[3];
            }
        };
#pragma unroll
        for (int kt = 0; kt < 6; ++kt) store_a(act_col(0), kt, a0[kt]);
#pragma unroll
        for (int l = 0; l < 5; ++l)
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) store_a(act_col(l + 1), kt, ah[l][kt]);
        // relative L2 loss on the exp output (channels 0..2): d/dz of
        // (p - y)^2 / (sg(p)^2 + 0.01) with p = exp(z)
        float dzo[2][4];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int col = nt * 8 + 2 * t + (e & 1);
                bool row_hi = e >= 2;
                bool valid = (row_hi ? v1 : v0) && col < 3;
                float d = 0.0f;
                if (valid) {
                    float4 y4 = __ldg(target + (row_hi ? r1 : r0));
                    float y = col == 0 ? y4.x : (col == 1 ? y4.y : y4.z);
                    float p = safe_exp(z[nt][e]);
                    float den = p * p + 0.01f;
                    loss += (p - y) * (p - y) / den;
                    d = 2.0f * (p - y) / den * p * inv_count;
                }
                dzo[nt][e] = d;
            }
        uint32_t adz[1][4];
        adz[0][0] = pack_bf16(dzo[0][0], dzo[0][1]);
        adz[0][1] = pack_bf16(dzo[0][2], dzo[0][3]);
        adz[0][2] = pack_bf16(dzo[1][0], dzo[1][1]);
        adz[0][3] = pack_bf16(dzo[1][2], dzo[1][3]);
        auto store_dz = [&](int col0, int kt, const uint32_t (&f)[4]) {
            int c = col0 + kt * 16 + 2 * t;
            if (v0) {
                *reinterpret_cast<uint32_t*>(dz + r0 * kGradCols + c) = f[0];
                *reinterpret_cast<uint32_t*>(dz + r0 * kGradCols + c + 8) = f[2];
            }
            if (v1) {
                *reinterpret_cast<uint32_t*>(dz + r1 * kGradCols + c) = f[1];
                *reinterpret_cast<uint32_t*>(dz + r1 * kGradCols + c + 8) = f[3];
            }
        };
        store_dz(grad_col(5), 0, adz[0]);
        // backward data: dA_5 = dZ_5 W_5, dZ_4 = dA_5 * mask_4, ...
        float c[8][4];
        gemm_tile<1, 8>(adz, wts + wt_smem_off(5), wt_stride(5), c);
        uint32_t a[4][4];
#pragma unroll
        for (int l = 4; l >= 0; --l) {
            mask_to_a<8>(c, masks[l], a);
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) store_dz(grad_col(l), kt, a[kt]);
            if (l > 0) gemm_tile<4, 8>(a, wts + wt_smem_off(l), wt_stride(l), c);
        }
    }
    // loss: warp reduce, one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0 && loss_sum) atomicAdd(loss_sum, loss * inv_count);
}

// dW_l = dZ_l^T A_l over a chunk of rows: M = out, N = in, K = rows.
// The chunk's rows of dZ_l and A_l are staged in shared memory; each warp
// owns a set of 16x8 output tiles and writes its FP32 sums to the chunk's
// slice of the partial-gradient buffer (summed by k_dw_reduce).
constexpr int kDwRows = 32;         // rows staged per step (two k16 steps)
constexpr int kMaxDwChunks = 256;  // row chunks of one weight-gradient pass

__global__ void __launch_bounds__(kMlpThreads) k_mlp_dw(const __nv_bfloat16* __restrict__ act,
                                                        const __nv_bfloat16* __restrict__ dz, int64_t n,
                                                        int64_t rows_per_block, float* __restrict__ partial)
{
    const int l = blockIdx.y;
    const int in = mlp_in(l), out = mlp_out(l);
    __shared__ __align__(16) __nv_bfloat16 sdz[kDwRows][kMlpHidden + 8];
    __shared__ __align__(16) __nv_bfloat16 sa[kDwRows][kMlpIn + 8];
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warp = threadIdx.x >> 5;
    const int mtiles = out / 16, ntiles = in / 8;
    const int tiles = mtiles * ntiles;  // <= 48
    float acc[12][4];
#pragma unroll
    for (int i = 0; i < 12; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
    const int64_t row_begin = (int64_t)blockIdx.x * rows_per_block;
    const int64_t row_end = min(n, row_begin + rows_per_block);
    for (int64_t r = row_begin; r < row_end; r += kDwRows) {
        __syncthreads();
        for (int i = threadIdx.x; i < kDwRows * out; i += blockDim.x) {
            int rr = i / out, cc = i % out;
            int64_t row = r + rr;
            sdz[rr][cc] = row < row_end ? dz[row * kGradCols + grad_col(l) + cc] : __float2bfloat16(0.0f);
        }
        for (int i = threadIdx.x; i < kDwRows * in; i += blockDim.x) {
            int rr = i / in, cc = i % in;
            int64_t row = r + rr;
            sa[rr][cc] = row < row_end ? act[row * kActCols + act_col(l) + cc] : __float2bfloat16(0.0f);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kDwRows / 16; ++ks) {
            const int k0 = ks * 16;
#pragma unroll
            for (int i = 0; i < 12; ++i) {
                int tile = warp + 4 * i;
                if (tile >= tiles) break;
                int mt = tile / ntiles, nt = tile % ntiles;
                // A = dZ^T (M = out rows, K = data rows): element (m, k) = sdz[k][m]
                auto ldA = [&](int m, int k) {
                    uint16_t lo = reinterpret_cast<const uint16_t&>(sdz[k0 + k][mt * 16 + m]);
                    uint16_t hi = reinterpret_cast<const uint16_t&>(sdz[k0 + k + 1][mt * 16 + m]);
                    return (uint32_t)lo | ((uint32_t)hi << 16);
                };
                uint32_t a[4] = {ldA(g, 2 * t), ldA(g + 8, 2 * t), ldA(g, 2 * t + 8), ldA(g + 8, 2 * t + 8)};
                // B = A_l (K = data rows, N = in): element (k, n) = sa[k][n]
                auto ldB = [&](int k, int nn) {
                    uint16_t lo = reinterpret_cast<const uint16_t&>(sa[k0 + k][nt * 8 + nn]);
                    uint16_t hi = reinterpret_cast<const uint16_t&>(sa[k0 + k + 1][nt * 8 + nn]);
                    return (uint32_t)lo | ((uint32_t)hi << 16);
                };
                mma16816(acc[i], a, ldB(2 * t, g), ldB(2 * t + 8, g));
            }
        }
    }
    // this chunk's partial gradient; k_dw_reduce sums the chunks in a fixed
    // order, so training is deterministic (no floating-point atomics)
    float* gl = partial + (size_t)blockIdx.x * kMlpParams + mlp_offset(l);
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        int tile = warp + 4 * i;
        if (tile >= tiles) break;
        int mt = tile / ntiles, nt = tile % ntiles;
        int m0 = mt * 16 + g, n0 = nt * 8 + 2 * t;
        *reinterpret_cast<float2*>(gl + m0 * in + n0) = make_float2(acc[i][0], acc[i][1]);
        *reinterpret_cast<float2*>(gl + (m0 + 8) * in + n0) = make_float2(acc[i][2], acc[i][3]);
    }
}

// grad += sum of the chunks' partial gradients, chunk 0 first
__global__ void k_dw_reduce(const float* __restrict__ partial, int chunks, float* __restrict__ grad)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kMlpParams; p += gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int c = 0; c < chunks; ++c) s += __ldg(partial + (size_t)c * kMlpParams + p);
        grad[p] += s;
    }
}

// Element i of the parameter vector (W_l[out][in], layer after layer) in the
// packed canonical layout of the tensor-core kernels.
__device__ __forceinline__ int packed_index(int i)
{
    int l = 0;
    while (l + 1 < kMlpLayers && i >= mlp_offset(l + 1)) ++l;
    const int j = i - mlp_offset(l), in = mlp_in(l);
    return mlp_offset(l) + (int)(canon_off(j / in, j % in, in) / 2);
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the bf16
// copy and its packed canonical copy, and clears the gradient.
__global__ void k_adam(float* __restrict__ wf, __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wpack,
                       float* __restrict__ m, float* __restrict__ v, float* __restrict__ grad, int n, float lr,
                       float b1, float b2, float eps, float c1, float c2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = grad[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = wf[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    wf[i] = wi;
    wb[i] = __float2bfloat16(wi);
    wpack[packed_index(i)] = __float2bfloat16_rn(wi);
    grad[i] = 0.0f;
}

__global__ void k_to_bf16(const float* __restrict__ wf, __nv_bfloat16* __restrict__ wb, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16(wf[i]);
}

size_t train_smem() { return (size_t)(kWSmem + kWtSmem) * 2; }

// The 96 input features of one query record (feature_pair) as row r of a
// 128-row A tile in the canonical layout (K = 96): twelve 16-byte stores.
__device__ __forceinline__ void write_features(const float4 (&q)[4], bool valid, const MlpBox& box, uint8_t* a, int r)
{
#pragma unroll
    for (int j = 0; j < kMlpIn / 8; ++j) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 f = valid ? feature_pair(q, box, 8 * j + 2 * e) : make_float2(0.0f, 0.0f);
            w[e] = pack2_bf16(f.x, f.y);
        }
        *reinterpret_cast<uint4*>(a + canon_off(r, 8 * j, kMlpIn)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

}  // namespace

// The network's shape as a fused tensor-core task (umma_mlp.cuh): all six
// layers' packed weights (46 KB) resident in shared memory, the input tile
// built by the threads from the query records, ReLU after the hidden layers.
struct MlpTaskShape {
    static constexpr int kLayers = kMlpLayers;
    static constexpr bool kResident = true;
    static constexpr bool kInputBulk = false;
    __host__ __device__ static constexpr int in(int l) { return mlp_in(l); }
    __host__ __device__ static constexpr int out(int l) { return mlp_out(l); }
    __host__ __device__ static constexpr bool relu(int l) { return l + 1 < kMlpLayers; }
    __host__ __device__ static constexpr uint32_t w_off(int l) { return (uint32_t)mlp_offset(l) * 2u; }
    __device__ const void* input_tile(int64_t) const { return nullptr; }
};

// srt_mlp_infer: records in, RGB radiance (exp of the first three outputs) out.
struct MlpInferTask : MlpTaskShape {
    const float4* rec;
    float4* y;
    int64_t n;
    MlpBox box;
    const __nv_bfloat16* w;
    __device__ int64_t rows() const { return n; }
    __device__ const uint8_t* weights() const { return reinterpret_cast<const uint8_t*>(w); }
    __device__ void make_input(int64_t row, bool valid, uint8_t* a, int r) const
    {
        float4 q[4];
        load_record(rec, row, valid, q);
        write_features(q, valid, box, a, r);
    }
    __device__ void store(int64_t row, const float (&o)[kMlpOut]) const
    {
        y[row] = make_float4(safe_exp(o[0]), safe_exp(o[1]), safe_exp(o[2]), 0.0f);
    }
};

// The tracer's radiance-cache queries of job blockIdx.y: the network's
// output times the path throughput is added to the pixel's in-flight
// radiance (one path per pixel in flight, so a plain read-modify-write).
struct CacheQueryTask : MlpTaskShape {
    const JobRec* jobs;
    __device__ const JobRec& job() const { return jobs[blockIdx.y]; }
    __device__ int64_t rows() const
    {
        const JobRec& J = job();
        if (!J.cache.wpack) return 0;  // a plain job
        return min((int64_t)J.cache.q_count[0], (int64_t)J.npix);
    }
    __device__ const uint8_t* weights() const { return reinterpret_cast<const uint8_t*>(job().cache.wpack); }
    __device__ void make_input(int64_t row, bool valid, uint8_t* a, int r) const
    {
        const CacheRec& C = job().cache;
        float4 q[4];
        load_record(C.q_rec, row, valid, q);
        write_features(q, valid, C.box, a, r);
    }
    __device__ void store(int64_t row, const float (&o)[kMlpOut]) const
    {
        const JobRec& J = job();
        const float4 b = J.cache.q_beta[row];
        float4* lp = J.lpath + __float_as_int(b.w);
        const float4 l = *lp;
        *lp = make_float4(l.x + b.x * safe_exp(o[0]), l.y + b.y * safe_exp(o[1]), l.z + b.z * safe_exp(o[2]), l.w);
    }
};

}  // namespace srt

using namespace srt;

namespace {

srt_status ensure_scratch(srt_mlp* p, int64_t n)
{
    if (!p->partial.get())
        SRT_TRY(p->partial.alloc((size_t)kMaxDwChunks * kMlpParams * 4, "mlp gradient partials"));
    if (n <= p->scratch_rows) return SRT_OK;
    int64_t rows = std::max<int64_t>(n, 1 << 16);
    SRT_TRY(p->scratch.alloc((size_t)rows * (kActCols + kGradCols) * 2, "mlp training scratch"));
    p->scratch_rows = rows;
    return SRT_OK;
}

srt_status configure_smem()
{
    static bool done = false;
    if (done) return SRT_OK;
    SRT_CUDA_TRY(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    done = true;
    return SRT_OK;
}

int grid_rows(int64_t n)
{
    int64_t tiles = (n + 15) / 16;
    int64_t blocks = (tiles + 3) / 4;
    return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)device_sm_count() * 4));
}

}  // namespace

namespace srt {

srt_status mlp_pack(srt_mlp* p, cudaStream_t st)
{
    for (int l = 0; l < kMlpLayers; ++l)
        SRT_TRY(umma_pack_layer(p->wf + mlp_offset(l), mlp_in(l), mlp_out(l), p->wpack + mlp_offset(l), st));
    return SRT_OK;
}

// the fused tensor-core inference (the tracer's cache path uses the same kernel)
srt_status mlp_infer_launch(const srt_mlp* p, const float4* rec, int64_t n, float4* out, cudaStream_t st)
{
    if (n <= 0) return SRT_OK;
    MlpInferTask t{};
    t.rec = rec;
    t.y = out;
    t.n = n;
    t.box = p->box;
    t.w = p->wpack;
    return umma_mlp_launch(t, n, 1, st);
}

srt_status mlp_train_launch(srt_mlp* p, const float4* rec, const float4* target, int64_t n, float lr, bool update,
                            cudaStream_t st)
{
    SRT_TRY(configure_smem());
    if (n <= 0) return SRT_OK;
    SRT_TRY(ensure_scratch(p, n));
    __nv_bfloat16* act = p->scratch.as<__nv_bfloat16>();
    __nv_bfloat16* dz = act + (size_t)p->scratch_rows * kActCols;
    SRT_CUDA_TRY(cudaMemsetAsync(p->loss, 0, 4, st));
    k_mlp_train<<<grid_rows(n), kMlpThreads, train_smem(), st>>>(p->wb, p->box, rec, target, n, act, dz, p->loss);
    // at most kMaxDwChunks chunks of a multiple of kDwRows rows
    int64_t chunk = std::max<int64_t>(kDwRows, ((n + kMaxDwChunks - 1) / kMaxDwChunks + kDwRows - 1) / kDwRows * kDwRows);
    const int chunks = (int)((n + chunk - 1) / chunk);
    dim3 grid((unsigned)chunks, kMlpLayers);
    k_mlp_dw<<<grid, kMlpThreads, 0, st>>>(act, dz, n, chunk, p->partial.as<float>());
    k_dw_reduce<<<(kMlpParams + 255) / 256, 256, 0, st>>>(p->partial.as<float>(), chunks, p->grad);
    if (update) {
        p->step += 1;
        float c1 = 1.0f - std::pow(p->b1, (float)p->step), c2 = 1.0f - std::pow(p->b2, (float)p->step);
        k_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(p->wf, p->wb, p->wpack, p->m, p->v, p->grad, kMlpParams, lr,
                                                         p->b1, p->b2, p->eps, c1, c2);
    }
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

MlpView mlp_view(const srt_mlp* p) { return MlpView{p->wb, p->box}; }

void launch_cache_queries(const JobRec* jobs, int max_jobs, cudaStream_t st)
{
    // the query count is read on the device: launch the resident CTAs
    CacheQueryTask t{};
    t.jobs = jobs;
    umma_mlp_launch(t, (int64_t)1 << 40, (unsigned)max_jobs, st);
}

srt_status mlp_prepare_kernels()
{
    SRT_TRY(umma_prepare());
    SRT_TRY(configure_smem());
    // kernel attributes of both fused tasks, outside any stream capture
    SRT_TRY(umma_mlp_launch(MlpInferTask{}, 0, 1, 0));
    SRT_TRY(umma_mlp_launch(CacheQueryTask{}, 0, 1, 0));
    return SRT_OK;
}

}  // namespace srt

extern "C" srt_status srt_mlp_create(uint64_t seed, srt_mlp** out)
{
    clear_error();
    if (!out) return set_error(SRT_ERR_ARG, "NULL argument");
    *out = nullptr;
    srt_mlp* p = new (std::nothrow) srt_mlp();
    if (!p) return set_error(SRT_ERR_OOM, "host allocation failed");
    size_t bytes = (size_t)kMlpParams * (4 + 2 + 4 + 4 + 4) + 64 + 256 + (size_t)kMlpParams * 2;
    srt_status st = mlp_prepare_kernels();
    if (st == SRT_OK) st = p->params.alloc(bytes, "mlp parameters");
    if (st != SRT_OK) {
        delete p;
        return st;
    }
    char* b = p->params.as<char>();
    p->wf = reinterpret_cast<float*>(b);
    p->m = p->wf + kMlpParams;
    p->v = p->m + kMlpParams;
    p->grad = p->v + kMlpParams;
    p->loss = p->grad + kMlpParams;
    p->wb = reinterpret_cast<__nv_bfloat16*>(p->loss + 16);
    // 256-byte aligned: the kernels bulk-copy it into shared memory
    p->wpack = reinterpret_cast<__nv_bfloat16*>((reinterpret_cast<uintptr_t>(p->wb + kMlpParams) + 255) & ~(uintptr_t)255);
    // He-uniform initialisation from a seeded 64-bit LCG; padded rows/columns are zero
    std::vector<float> w(kMlpParams, 0.0f);
    uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return (float)((s >> 40) & 0xffffff) / 16777216.0f;
    };
    for (int l = 0; l < kMlpLayers; ++l) {
        int in = mlp_in(l), outn = mlp_out(l);
        int fan_in = l == 0 ? 83 : in;
        float lim = std::sqrt(6.0f / (float)fan_in) * (l == kMlpLayers - 1 ? 0.1f : 1.0f);
        for (int o = 0; o < outn; ++o)
            for (int k = 0; k < in; ++k) {
                bool live = (l == 0 ? k < 83 : true) && (l == kMlpLayers - 1 ? o < 3 : true);
                w[mlp_offset(l) + o * in + k] = live ? (2.0f * uni() - 1.0f) * lim : 0.0f;
            }
    }
    cudaError_t e = cudaMemcpy(p->wf, w.data(), w.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(p->m, 0, (size_t)kMlpParams * 4 * 3 + 64);
    if (e == cudaSuccess) {
        k_to_bf16<<<(kMlpParams + 255) / 256, 256>>>(p->wf, p->wb, kMlpParams);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && mlp_pack(p, 0) != SRT_OK) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        delete p;
        return cuda_error(e, "mlp init");
    }
    p->box.lo = make_float3(0.f, 0.f, 0.f);
    p->box.inv_extent = make_float3(1.f, 1.f, 1.f);
    *out = p;
    return SRT_OK;
}

extern "C" srt_status srt_mlp_set_box(srt_mlp* p, const float* lo, const float* hi)
{
    clear_error();
    if (!p || !lo || !hi) return set_error(SRT_ERR_ARG, "NULL argument");
    p->box.lo = make_float3(lo[0], lo[1], lo[2]);
    p->box.inv_extent = make_float3(1.0f / std::max(hi[0] - lo[0], 1e-6f), 1.0f / std::max(hi[1] - lo[1], 1e-6f),
                                    1.0f / std::max(hi[2] - lo[2], 1e-6f));
    return SRT_OK;
}

extern "C" srt_status srt_mlp_get_params(const srt_mlp* p, float* host)
{
    clear_error();
    if (!p || !host) return set_error(SRT_ERR_ARG, "NULL argument");
    SRT_CUDA_TRY(cudaMemcpy(host, p->wf, (size_t)kMlpParams * 4, cudaMemcpyDeviceToHost));
    return SRT_OK;
}

extern "C" srt_status srt_mlp_set_params(srt_mlp* p, const float* host)
{
    clear_error();
    if (!p || !host) return set_error(SRT_ERR_ARG, "NULL argument");
    SRT_CUDA_TRY(cudaMemcpy(p->wf, host, (size_t)kMlpParams * 4, cudaMemcpyHostToDevice));
    k_to_bf16<<<(kMlpParams + 255) / 256, 256>>>(p->wf, p->wb, kMlpParams);
    SRT_CUDA_TRY(cudaGetLastError());
    SRT_TRY(mlp_pack(p, 0));
    SRT_CUDA_TRY(cudaDeviceSynchronize());
    p->step = 0;
    SRT_CUDA_TRY(cudaMemset(p->m, 0, (size_t)kMlpParams * 4 * 3));
    return SRT_OK;
}

extern "C" srt_status srt_mlp_infer(const srt_mlp* p, const float* rec, int64_t n, float* out, void* stream)
{
    clear_error();
    if (!p || n < 0 || (n > 0 && (!rec || !out))) return set_error(SRT_ERR_ARG, "bad arguments");
    if ((reinterpret_cast<uintptr_t>(rec) | reinterpret_cast<uintptr_t>(out)) % 16)
        return set_error(SRT_ERR_ARG, "records and outputs must be 16-byte aligned");
    return mlp_infer_launch(p, reinterpret_cast<const float4*>(rec), n, reinterpret_cast<float4*>(out),
                            as_stream(stream));
}

extern "C" srt_status srt_mlp_train_step(srt_mlp* p, const float* rec, const float* target, int64_t n, float lr,
                                         float* loss, void* stream)
{
    clear_error();
    if (!p || n <= 0 || !rec || !target || !(lr >= 0.0f)) return set_error(SRT_ERR_ARG, "bad arguments");
    if ((reinterpret_cast<uintptr_t>(rec) | reinterpret_cast<uintptr_t>(target)) % 16)
        return set_error(SRT_ERR_ARG, "records and targets must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    SRT_TRY(mlp_train_launch(p, reinterpret_cast<const float4*>(rec), reinterpret_cast<const float4*>(target), n, lr,
                             true, st));
    if (loss) {
        SRT_CUDA_TRY(cudaMemcpyAsync(loss, p->loss, 4, cudaMemcpyDeviceToHost, st));
        SRT_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return SRT_OK;
}

extern "C" srt_status srt_mlp_gradient(srt_mlp* p, const float* rec, const float* target, int64_t n, float* host_grad,
                                       float* loss, void* stream)
{
    clear_error();
    if (!p || n <= 0 || !rec || !target || !host_grad) return set_error(SRT_ERR_ARG, "bad arguments");
    cudaStream_t st = as_stream(stream);
    SRT_CUDA_TRY(cudaMemsetAsync(p->grad, 0, (size_t)kMlpParams * 4, st));
    SRT_TRY(mlp_train_launch(p, reinterpret_cast<const float4*>(rec), reinterpret_cast<const float4*>(target), n,
                             0.0f, false, st));
    SRT_CUDA_TRY(cudaMemcpyAsync(host_grad, p->grad, (size_t)kMlpParams * 4, cudaMemcpyDeviceToHost, st));
    if (loss) SRT_CUDA_TRY(cudaMemcpyAsync(loss, p->loss, 4, cudaMemcpyDeviceToHost, st));
    SRT_CUDA_TRY(cudaStreamSynchronize(st));
    SRT_CUDA_TRY(cudaMemsetAsync(p->grad, 0, (size_t)kMlpParams * 4, st));
    return SRT_OK;
}

extern "C" void srt_mlp_destroy(srt_mlp* p) { delete p; }
