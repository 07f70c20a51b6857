// ORACLE input synthesis (test infrastructure).  The benchmark's procedural
// scenes (the Cornell box and the 5.2M-triangle icosphere scene) built into
// the oracle library from the same generator source the CUDA library
// compiles, so that a process timing the oracle (the benchmark's CPU arm)
// generates identical inputs without loading the CUDA library.  Compiled
// with hidden visibility: only the oracle_* entry point below is exported.
#include "../srt_gb300/csrc/procedural.cpp"

#include "srt_oracle.h"

namespace srt {
// the generator's error reporting: statuses are returned, messages dropped
srt_status set_error(srt_status st, const std::string&) { return st; }
void clear_error() {}
}  // namespace srt

// An oracle scene of the procedural scene `name` ("cornell" | "spheres")
// with the camera's aspect set to `aspect`; null on a bad argument.
extern "C" __attribute__((visibility("default"))) oracle_scene* oracle_scene_create_procedural(
    const char* name, uint64_t seed, int32_t n_spheres, int32_t subdiv, float aspect)
{
    srt_procedural* p = nullptr;
    if (srt_procedural_create(name, seed, n_spheres, subdiv, &p) != SRT_OK || !p) return nullptr;
    srt_scene_desc d{};
    oracle_scene* s = nullptr;
    if (srt_procedural_desc(p, &d) == SRT_OK) {
        d.camera.aspect = aspect;
        s = oracle_scene_create(&d);
    }
    srt_procedural_destroy(p);
    return s;
}
