// Force-included before the reference's device headers when they are built
// for the host (oracle/ref/Makefile).  Without the float overloads, host
// `max(float, float)` resolves to an integer overload, the Disney roughness
// terms become 0 and every Disney value comes out NaN.  Textures do not
// exist in the synthetic scenes, so tex2D returns a zero value.
#pragma once
#include <cmath>
#include <cuda_runtime.h>

inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
template <class T>
inline T tex2D(cudaTextureObject_t, float, float)
{
    return T{};
}
