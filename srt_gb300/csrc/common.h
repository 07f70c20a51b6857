// common.h — host-side helpers shared by the library's translation units:
// error reporting (status + thread-local message, never exit/trap) and an
// owning device allocation.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

#include "../../include/srt.h"

namespace srt {

// Records `msg` as this thread's last error and returns `st`.
srt_status set_error(srt_status st, const std::string& msg);
void clear_error();

// Maps a failing CUDA call to SRT_ERR_CUDA / SRT_ERR_OOM with context.
srt_status cuda_error(cudaError_t e, const char* what);

#define SRT_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t srt_e_ = (expr);                         \
        if (srt_e_ != cudaSuccess) return ::srt::cuda_error(srt_e_, #expr); \
    } while (0)

#define SRT_TRY(expr)                          \
    do {                                       \
        srt_status srt_s_ = (expr);            \
        if (srt_s_ != SRT_OK) return srt_s_;   \
    } while (0)

// Owning device buffer (cudaMalloc / cudaFree).
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    ~DeviceBuffer() { reset(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_)
    {
        o.ptr_ = nullptr;
        o.bytes_ = 0;
    }

    srt_status alloc(size_t bytes, const char* what);
    srt_status upload(const void* host, size_t bytes, const char* what);
    void reset();
    void* get() const { return ptr_; }
    template <class T>
    T* as() const
    {
        return reinterpret_cast<T*>(ptr_);
    }
    size_t bytes() const { return bytes_; }

private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int device_sm_count();

}  // namespace srt
