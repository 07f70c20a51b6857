// film.cu — film passes: Accumulate, ToneMapping and the Measure metric.
//
// All three are HBM-bound elementwise passes over float4[n]; each thread
// moves whole 16-byte pixels.  The Measure metric drops the largest
// `discard` percent of the per-pixel errors; instead of sorting (thrust::sort
// in the reference, measure.cu:46-49) it finds the exact cut value with a
// three-pass radix select over the error bits (11 + 11 + 10 bits) and sums
// everything below it.
#include <cuda.h>  // CUcontext / CUresult types only (the driver call is looked up at run time)

#include <mutex>

#include "common.h"
#include "vmath.h"

using namespace srt;

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t n)
{
    int64_t blocks = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)device_sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

// Accumulate::render (accumulate.cu:10-29)
__global__ void __launch_bounds__(kThreads) k_accumulate(float4* __restrict__ film, float4* __restrict__ acc,
                                                         int64_t n, float w)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 a = acc[i], p = film[i];
        float k = 1.0f - w;
        float4 r = make_float4(a.x * k + p.x * w, a.y * k + p.y * w, a.z * k + p.z * w, a.w * k + p.w * w);
        acc[i] = r;
        film[i] = r;
    }
}

// ToneMapping::render (tonemapping.cu:5-70)
__global__ void __launch_bounds__(kThreads) k_tonemap(float4* __restrict__ film, int64_t n, int type, float ex,
                                                      int use_gamma)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 px = film[i];
        float3 c = f3(px) * ex;
        if (type == SRT_TONE_CLAMP) {
            c = make_float3(clampf(c.x, 0.f, 1.f), clampf(c.y, 0.f, 1.f), clampf(c.z, 0.f, 1.f));
        } else if (type == SRT_TONE_REINHARD) {
            float l = luminance(c);
            c = c / (1.0f + l);
        } else if (type == SRT_TONE_UNCHARTED2) {
            const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f, W = 11.2f;
            float3 num = c * (A * c + f3(C * B)) + f3(D * E);
            float3 den = c * (A * c + f3(B)) + f3(D * F);
            c = num / den - f3(E / F);
            float white = ((W * (A * W + C * B) + D * E) / (W * (A * W + B) + D * F)) - E / F;
            c = c / white;
        } else if (type == SRT_TONE_ACES) {
            c = c * 0.6f;
            const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
            c = (c * (a * c + f3(b))) / (c * (cc * c + f3(d)) + f3(e));
            c = make_float3(clampf(c.x, 0.f, 1.f), clampf(c.y, 0.f, 1.f), clampf(c.z, 0.f, 1.f));
        }
        if (use_gamma) {
            const float g = 1.0f / 2.2f;
            c = make_float3(powf(c.x, g), powf(c.y, g), powf(c.z, g));
        }
        film[i] = make_float4(c.x, c.y, c.z, 1.0f);
    }
}

// Metrics::cal_pixel (metrics.h:16-51)
__device__ __forceinline__ float pixel_error(float4 xa, float4 ra, int type)
{
    const float eps = 1e-6f;
    float3 x = f3(xa), r = f3(ra);
    if (type == SRT_METRIC_MSE) {
        float3 d = x - r;
        return dot(d, d) / 3.0f;
    }
    if (type == SRT_METRIC_MAPE) {
        float3 t = make_float3(fabsf(x.x - r.x), fabsf(x.y - r.y), fabsf(x.z - r.z)) / (r + f3(eps));
        return dot(t, f3(1.0f)) / 3.0f;
    }
    if (type == SRT_METRIC_SMAPE) {
        float3 t = 2.0f * make_float3(fabsf(x.x - r.x), fabsf(x.y - r.y), fabsf(x.z - r.z)) / (x + r + f3(eps));
        return dot(t, f3(1.0f)) / 3.0f;
    }
    float3 t = (x - r) / (r + f3(eps));
    return dot(t, t) / 3.0f;
}

// Measure's display options (measure.cu:29-39): the film shows the
// reference, or each pixel's error as grey.
__global__ void __launch_bounds__(kThreads) k_measure_view(float4* __restrict__ film, const float4* __restrict__ r,
                                                           int64_t n, int type, int option)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 ref = __ldg(r + i);
        if (option == SRT_MEASURE_REFERENCE) {
            film[i] = make_float4(ref.x, ref.y, ref.z, 1.0f);
        } else {
            const float e = pixel_error(film[i], ref, type);
            film[i] = make_float4(e, e, e, 1.0f);
        }
    }
}

// Radix-select scratch (after the per-pixel error array).
struct SelectState {
    uint32_t prefix;       // bits of the cut value fixed so far
    uint32_t prefix_mask;  // which bits are fixed
    long long remaining;   // rank still to find inside the prefix bucket
    long long count_below; // elements strictly below the prefix bucket
    double sum_below;
    long long keep;
    float result;
    int pad;
};
constexpr int kBins = 2048;

struct MetricScratch {
    unsigned long long counts[kBins];
    double sums[kBins];
    SelectState s;
};

size_t scratch_bytes(int64_t n) { return ((size_t)n * 4 + 255) / 256 * 256 + sizeof(MetricScratch); }

// Order-preserving key of a float error: non-negative floats compare like
// their bit patterns; negatives (not produced by the metrics) sort first.
__device__ __forceinline__ uint32_t fkey(float e)
{
    uint32_t b = __float_as_uint(e);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void __launch_bounds__(kThreads) k_metric_errors(const float4* __restrict__ x, const float4* __restrict__ r,
                                                            int64_t n, int type, float* __restrict__ err)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        err[i] = pixel_error(__ldg(x + i), __ldg(r + i), type);
}

// Histogram of the digit at `shift` (width `bits`) over elements whose key
// matches the current prefix; per-block shared histograms, merged globally.
__global__ void __launch_bounds__(kThreads) k_metric_hist(const float* __restrict__ err, int64_t n,
                                                          MetricScratch* sc, int shift, int bits)
{
    __shared__ unsigned int cnt[kBins];
    __shared__ double sum[kBins];
    const int nb = 1 << bits;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        cnt[b] = 0;
        sum[b] = 0.0;
    }
    __syncthreads();
    const uint32_t prefix = sc->s.prefix, pmask = sc->s.prefix_mask;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float e = err[i];
        uint32_t k = fkey(e);
        if ((k & pmask) != prefix) continue;
        uint32_t d = (k >> shift) & (uint32_t)(nb - 1);
        atomicAdd(&cnt[d], 1u);
        atomicAdd(&sum[d], (double)e);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        if (cnt[b]) {
            atomicAdd(&sc->counts[b], (unsigned long long)cnt[b]);
            atomicAdd(&sc->sums[b], sum[b]);
        }
    }
}

// One thread: picks the digit holding rank `remaining`, folds the lower
// buckets into count/sum below, clears the histogram for the next pass.
__global__ void k_metric_select(MetricScratch* sc, int shift, int bits, int last)
{
    SelectState& s = sc->s;
    const int nb = 1 << bits;
    long long acc = 0;
    double accs = 0.0;
    int pick = nb - 1;
    for (int b = 0; b < nb; ++b) {
        long long c = (long long)sc->counts[b];
        if (acc + c >= s.remaining) {
            pick = b;
            break;
        }
        acc += c;
        accs += sc->sums[b];
    }
    s.count_below += acc;
    s.sum_below += accs;
    s.remaining -= acc;
    s.prefix |= (uint32_t)pick << shift;
    s.prefix_mask |= (uint32_t)(nb - 1) << shift;
    for (int b = 0; b < nb; ++b) {
        sc->counts[b] = 0;
        sc->sums[b] = 0.0;
    }
    if (last) {
        uint32_t k = s.prefix;
        uint32_t bitsv = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
        float cut = __uint_as_float(bitsv);
        double total = s.sum_below + (double)(s.keep - s.count_below) * (double)cut;
        s.result = (float)(total / (double)s.keep);
    }
}

__global__ void k_metric_init(MetricScratch* sc, long long keep)
{
    for (int b = threadIdx.x; b < kBins; b += blockDim.x) {
        sc->counts[b] = 0;
        sc->sums[b] = 0.0;
    }
    if (threadIdx.x == 0) {
        SelectState& s = sc->s;
        s.prefix = 0;
        s.prefix_mask = 0;
        s.remaining = keep;
        s.count_below = 0;
        s.sum_below = 0.0;
        s.keep = keep;
        s.result = 0.0f;
    }
}

}  // namespace

extern "C" srt_status srt_film_accumulate(float* film, float* acc, int64_t n, int32_t frame_count, void* stream)
{
    clear_error();
    if (n < 0 || frame_count < 0) return set_error(SRT_ERR_ARG, "bad arguments");
    if (n == 0) return SRT_OK;
    if (!film || !acc) return set_error(SRT_ERR_ARG, "NULL film");
    if ((reinterpret_cast<uintptr_t>(film) | reinterpret_cast<uintptr_t>(acc)) % 16)
        return set_error(SRT_ERR_ARG, "film buffers must be 16-byte aligned");
    float w = 1.0f / (float)(frame_count + 1);
    k_accumulate<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(reinterpret_cast<float4*>(film),
                                                                  reinterpret_cast<float4*>(acc), n, w);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

extern "C" srt_status srt_film_tonemap(float* film, int64_t n, int32_t type, float exposure, int32_t use_gamma,
                                       void* stream)
{
    clear_error();
    if (n < 0 || type < SRT_TONE_NONE || type > SRT_TONE_ACES) return set_error(SRT_ERR_ARG, "bad arguments");
    if (n == 0) return SRT_OK;
    if (!film) return set_error(SRT_ERR_ARG, "NULL film");
    if (reinterpret_cast<uintptr_t>(film) % 16) return set_error(SRT_ERR_ARG, "film must be 16-byte aligned");
    float ex = powf(2.0f, exposure);
    k_tonemap<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(reinterpret_cast<float4*>(film), n, type, ex,
                                                               use_gamma ? 1 : 0);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

extern "C" size_t srt_film_metric_scratch_bytes(int64_t n) { return n < 0 ? 0 : scratch_bytes(n); }

extern "C" srt_status srt_film_measure_view(float* film, const float* ref, int64_t n, int32_t type, int32_t option,
                                            void* stream)
{
    clear_error();
    if (n < 0 || type < SRT_METRIC_MSE || type > SRT_METRIC_RELMSE || option < SRT_MEASURE_NONE ||
        option > SRT_MEASURE_ERROR)
        return set_error(SRT_ERR_ARG, "bad arguments");
    if (n == 0 || option == SRT_MEASURE_NONE) return SRT_OK;
    if (!film || !ref) return set_error(SRT_ERR_ARG, "NULL buffer");
    if ((reinterpret_cast<uintptr_t>(film) | reinterpret_cast<uintptr_t>(ref)) % 16)
        return set_error(SRT_ERR_ARG, "film buffers must be 16-byte aligned");
    k_measure_view<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(reinterpret_cast<float4*>(film),
                                                                    reinterpret_cast<const float4*>(ref), n, type,
                                                                    option);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

namespace {

// The Measure metric's launch sequence (measure.cu:35-49 with a radix select
// in place of the sort) over a per-pixel error buffer `err` and select state
// `sc`; returns the metric in *out once the stream has reached it.
srt_status run_metric(const float* x, const float* ref, int64_t n, int32_t type, long long keep, float* err,
                      MetricScratch* sc, cudaStream_t st, float* out)
{
    const int g = grid_for(n);
    k_metric_init<<<1, 256, 0, st>>>(sc, keep);  // clears the histograms and the select state
    k_metric_errors<<<g, kThreads, 0, st>>>(reinterpret_cast<const float4*>(x), reinterpret_cast<const float4*>(ref),
                                            n, type, err);
    const int shifts[3] = {21, 10, 0}, widths[3] = {11, 11, 10};
    for (int p = 0; p < 3; ++p) {
        k_metric_hist<<<g, kThreads, 0, st>>>(err, n, sc, shifts[p], widths[p]);
        k_metric_select<<<1, 1, 0, st>>>(sc, shifts[p], widths[p], p == 2 ? 1 : 0);
    }
    SRT_CUDA_TRY(cudaGetLastError());
    float res = 0.0f;
    SRT_CUDA_TRY(cudaMemcpyAsync(&res, &sc->s.result, sizeof(float), cudaMemcpyDeviceToHost, st));
    SRT_CUDA_TRY(cudaStreamSynchronize(st));
    *out = res;
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_film_metric(const float* x, const float* ref, int64_t n, int32_t type, float discard,
                                      void* scratch, float* out, void* stream)
{
    clear_error();
    if (!out) return set_error(SRT_ERR_ARG, "out is NULL");
    if (n < 0 || type < SRT_METRIC_MSE || type > SRT_METRIC_RELMSE || !(discard >= 0.0f && discard <= 100.0f))
        return set_error(SRT_ERR_ARG, "bad arguments");
    // final_num = (int)(num * (1 - discard / 100)) (measure.cu:47)
    long long keep = (long long)((float)n * (1.0f - discard / 100.0f));
    if (keep <= 0) {
        *out = NAN;  // the reference divides an empty sum by zero
        return SRT_OK;
    }
    if (!x || !ref || !scratch) return set_error(SRT_ERR_ARG, "NULL buffer");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(ref)) % 16 ||
        reinterpret_cast<uintptr_t>(scratch) % 256)
        return set_error(SRT_ERR_ARG, "films must be 16-byte aligned and scratch 256-byte aligned");
    float* err = reinterpret_cast<float*>(scratch);
    MetricScratch* sc = reinterpret_cast<MetricScratch*>(reinterpret_cast<char*>(scratch) +
                                                         ((size_t)n * 4 + 255) / 256 * 256);
    return run_metric(x, ref, n, type, keep, err, sc, as_stream(stream), out);
}

// ---------------------------------------------------------------------------
// Allocation-free Measure metric.  Some callers cannot allocate device
// memory when they measure a film: a render-serving loop that reserved its
// whole HBM budget up front, or a caller that must not let cudaMalloc /
// cudaFree synchronise the device while other jobs' frames are in flight.
// This variant keeps its scratch (the per-pixel errors and the radix-select
// state) in a fixed array in device memory instead of the caller's buffer.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kStaticMetricPixels = (int64_t)1 << 21;  // 2,097,152 pixels (1920x1080 fits)
constexpr size_t kStaticMetricErrBytes = ((size_t)kStaticMetricPixels * 4 + 255) / 256 * 256;

// Every GPU that loads the library holds this array (about 8 MB) until the
// process exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_metric_scratch[kStaticMetricErrBytes + sizeof(MetricScratch)];

// The calling thread's current CUDA context (the driver's cuCtxGetCurrent,
// found through the runtime so the library needs no link to the driver
// library), or null where it cannot be asked.
CUcontext current_context()
{
    typedef CUresult (*GetCurrent)(CUcontext*);
    static GetCurrent fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<GetCurrent>(f);
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// Device address of g_metric_scratch on the current device.  The array's
// host-side name is only a stand-in, never a device address, so the address
// is looked up with cudaGetSymbolAddress: once per device and context (a
// context made anew, e.g. after cudaDeviceReset, places the array anew and
// is looked up again; where the context cannot be told, every call looks
// it up).
srt_status static_metric_scratch(void** out)
{
    struct Entry {
        CUcontext ctx;
        void* ptr;
    };
    static std::mutex mu;
    static Entry cache[128] = {};
    int dev = 0;
    SRT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return set_error(SRT_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    const CUcontext ctx = current_context();
    if (!cache[dev].ptr || !ctx || ctx != cache[dev].ctx) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_metric_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_metric_scratch)");
        cache[dev].ptr = p;
        cache[dev].ctx = current_context();  // the lookup made the context current if it was not
    }
    *out = cache[dev].ptr;
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_film_metric_noalloc(const float* x, const float* ref, int64_t n, int32_t type,
                                              float discard, float* out, void* stream)
{
    clear_error();
    if (!out) return set_error(SRT_ERR_ARG, "out is NULL");
    if (n < 0 || type < SRT_METRIC_MSE || type > SRT_METRIC_RELMSE || !(discard >= 0.0f && discard <= 100.0f))
        return set_error(SRT_ERR_ARG, "bad arguments");
    if (n > kStaticMetricPixels)
        return set_error(SRT_ERR_ARG, "srt_film_metric_noalloc: n = " + std::to_string(n) +
                                          " exceeds its fixed scratch of 2097152 pixels; use srt_film_metric");
    long long keep = (long long)((float)n * (1.0f - discard / 100.0f));
    if (keep <= 0) {
        *out = NAN;
        return SRT_OK;
    }
    if (!x || !ref) return set_error(SRT_ERR_ARG, "NULL buffer");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(ref)) % 16)
        return set_error(SRT_ERR_ARG, "films must be 16-byte aligned");
    void* base = nullptr;
    SRT_TRY(static_metric_scratch(&base));
    float* err = reinterpret_cast<float*>(base);
    MetricScratch* sc = reinterpret_cast<MetricScratch*>(reinterpret_cast<char*>(base) + kStaticMetricErrBytes);
    return run_metric(x, ref, n, type, keep, err, sc, as_stream(stream), out);
}
