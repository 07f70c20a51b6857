// ORACLE (test infrastructure only; never linked into the product).
//
// Host build of the CUDA toolkit's header-only curand device API, so the
// CPU oracle draws exactly the per-pixel XORWOW streams the reference uses:
// RandomGenerator(seed, 0) -> curand_init(seed, 0, 0, &state) and
// random_float() -> 1 - curand_uniform(&state)
// (src/device_include/math/random.h:14-31).  This translation unit is
// compiled with `__device__` defined empty; it calls the toolkit functions
// and restates nothing of them.
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <string.h>

extern "C" {

// Opaque 64-byte state for callers that do not include curand headers.
int oracle_curand_state_bytes(void) { return (int)sizeof(curandState); }

void oracle_curand_init(unsigned long long seed, void* state)
{
    curand_init(seed, 0ULL, 0ULL, reinterpret_cast<curandState*>(state));
}

float oracle_curand_uniform01(void* state)
{
    return 1.0f - curand_uniform(reinterpret_cast<curandState*>(state));
}

// Tape of the first `ndraws` draws of pixel streams [0, npix) for frame seed
// `seed`: the stream of pixel idx is seeded with (int)(seed + idx) widened
// to unsigned long long, as `params.seed + idx` is in path_tracer.cu:56.
void oracle_curand_tape(int seed, long long npix, int ndraws, float* out)
{
    for (long long p = 0; p < npix; ++p) {
        curandState s;
        int si = (int)((unsigned)seed + (unsigned)p);
        curand_init((unsigned long long)(long long)si, 0ULL, 0ULL, &s);
        for (int k = 0; k < ndraws; ++k) out[p * ndraws + k] = 1.0f - curand_uniform(&s);
    }
}

}  // extern "C"
