// cache.cuh — radiance-cache state of a job that trains the network on its
// own paths (the PathTracer's cached render keeps its own; the serving loop
// uses these for jobs that train online).
#pragma once

#include "common.h"
#include "mlp.cuh"
#include "wavefront.cuh"

namespace srt {

// Device bytes of a cached job's query and training buffers: npix pixels,
// n_train training pixels (up to kTrainVertices recorded vertices each).
size_t cache_job_bytes(int64_t npix, int64_t n_train);
// Places those buffers at `base` (cache_job_bytes of device memory, zeroed
// query counters) and points the job's cache record at them.
void cache_job_carve(char* base, int64_t npix, int64_t n_train, CacheRec& C);
// Gathers the training vertices the job's paths recorded (complete once every
// training pixel has finished its first sample) and takes `steps` Adam steps
// on `mlp` over them, stream-ordered on `st`; *vertices = the batch size.
srt_status cache_job_train(char* base, int64_t npix, int64_t n_train, srt_mlp* mlp, int steps, float lr,
                           cudaStream_t st, int64_t* vertices);

}  // namespace srt
