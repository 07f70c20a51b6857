// umma_mlp.cu — host side of the fused tensor-core MLP kernels: weight
// packing into the canonical shared-memory layout, kernel set-up and the
// timeout flag their bounded waits report through.
#include <mutex>

#include "umma_mlp.cuh"

namespace srt {

namespace {

// set to 1 by a fused-MLP CTA whose mbarrier wait ran out of time
__device__ int g_umma_timeout;

__global__ void k_pack_canonical(const float* __restrict__ src, int in, int out, __nv_bfloat16* __restrict__ dst)
{
    const int64_t n = (int64_t)in * out;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int r = (int)(i / in), k = (int)(i % in);
        dst[canon_off(r, k, in) / 2] = __float2bfloat16_rn(src[i]);
    }
}

__global__ void k_pack_chunked(const float* __restrict__ src, int in, int out, __nv_bfloat16* __restrict__ dst)
{
    const int64_t n = (int64_t)in * out;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int r = (int)(i / in), k = (int)(i % in);
        const size_t chunk = (size_t)(k / kChunkK) * out * kChunkK;  // elements before the chunk
        dst[chunk + canon_off(r, k % kChunkK, kChunkK) / 2] = __float2bfloat16_rn(src[i]);
    }
}

// One thread initialises an mbarrier that expects one arrival and waits for
// a phase that nothing completes: the bounded wait of the fused kernels
// runs out after limit_ns and the CTA reports it as they do.
__global__ void k_wait_timeout_selftest(uint64_t limit_ns, int* err)
{
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    mbar_fence_init();
    if (!mbar_wait(&bar, 0u, limit_ns)) atomicExch(err, 1);
}

std::mutex g_mu;
int* g_err[128] = {};

}  // namespace

srt_status umma_pack_layer(const float* src, int in, int out, __nv_bfloat16* dst, cudaStream_t st)
{
    if (in % 16 || out % 16 || in <= 0 || out <= 0) return set_error(SRT_ERR_ARG, "layer shape not a multiple of 16");
    const int64_t n = (int64_t)in * out;
    k_pack_canonical<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(src, in, out, dst);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

srt_status umma_pack_layer_chunked(const float* src, int in, int out, __nv_bfloat16* dst, cudaStream_t st)
{
    if (in % kChunkK || out % 16 || in <= 0 || out <= 0)
        return set_error(SRT_ERR_ARG, "layer shape not a multiple of the chunk");
    const int64_t n = (int64_t)in * out;
    k_pack_chunked<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(src, in, out, dst);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

srt_status umma_prepare()
{
    int dev = 0;
    SRT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return set_error(SRT_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_err[dev]) {
        void* p = nullptr;
        SRT_CUDA_TRY(cudaGetSymbolAddress(&p, g_umma_timeout));
        SRT_CUDA_TRY(cudaMemset(p, 0, sizeof(int)));
        g_err[dev] = static_cast<int*>(p);
    }
    return SRT_OK;
}

int* umma_error_word()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return nullptr;
    std::lock_guard<std::mutex> lock(g_mu);
    return g_err[dev];
}

srt_status umma_take_error()
{
    int* p = umma_error_word();
    if (!p) return SRT_OK;
    int v = 0;
    SRT_CUDA_TRY(cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost));
    if (!v) return SRT_OK;
    SRT_CUDA_TRY(cudaMemset(p, 0, sizeof(int)));
    return set_error(SRT_ERR_TIMEOUT, "a tensor-core MLP kernel gave up waiting for its copies or MMAs");
}

}  // namespace srt

using namespace srt;

extern "C" srt_status srt_selftest_wait_timeout(int64_t limit_ns)
{
    clear_error();
    if (limit_ns < 1000 || limit_ns > 1000000000) return set_error(SRT_ERR_ARG, "limit_ns out of [1e3, 1e9]");
    SRT_TRY(umma_prepare());
    SRT_TRY(umma_take_error());  // a timeout of an earlier kernel is not this call's
    k_wait_timeout_selftest<<<1, 32>>>((uint64_t)limit_ns, umma_error_word());
    SRT_CUDA_TRY(cudaGetLastError());
    SRT_CUDA_TRY(cudaDeviceSynchronize());
    return umma_take_error();
}
