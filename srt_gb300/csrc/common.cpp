// common.cpp — error state, device buffers, device queries.
#include "common.h"

#include <mutex>
#include <vector>

namespace srt {

namespace {
thread_local std::string g_last_error;
}

srt_status set_error(srt_status st, const std::string& msg)
{
    g_last_error = msg;
    return st;
}

void clear_error() { g_last_error.clear(); }

srt_status cuda_error(cudaError_t e, const char* what)
{
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the sticky-free allocation error
        return set_error(SRT_ERR_OOM, msg);
    }
    return set_error(SRT_ERR_CUDA, msg);
}

srt_status DeviceBuffer::alloc(size_t bytes, const char* what)
{
    reset();
    if (bytes == 0) return SRT_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return cuda_error(e, what);
    ptr_ = p;
    bytes_ = bytes;
    return SRT_OK;
}

srt_status DeviceBuffer::upload(const void* host, size_t bytes, const char* what)
{
    SRT_TRY(alloc(bytes, what));
    if (bytes == 0) return SRT_OK;
    cudaError_t e = cudaMemcpy(ptr_, host, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, what);
    return SRT_OK;
}

void DeviceBuffer::reset()
{
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
}

int device_sm_count()
{
    static std::mutex mu;
    static std::vector<int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        cache[dev] = n;
    }
    return cache[dev];
}

}  // namespace srt

extern "C" const char* srt_last_error(void) { return srt::g_last_error.c_str(); }
extern "C" const char* srt_version(void) { return "srt-gb300 0.1 (sm_103a)"; }
