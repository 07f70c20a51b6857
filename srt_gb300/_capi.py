"""ctypes mirror of include/srt.h (struct layouts and entry points).

The library is loaded from the package directory; a missing library is an
error (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsrt_gb300.so")

SRT_OK = 0
STATUS_NAMES = {
    0: "SRT_OK", 1: "SRT_ERR_ARG", 2: "SRT_ERR_OOM", 3: "SRT_ERR_CUDA", 4: "SRT_ERR_TIMEOUT",
    5: "SRT_ERR_BUDGET", 6: "SRT_ERR_STACK", 7: "SRT_ERR_NOT_FOUND", 8: "SRT_ERR_PARSE",
    9: "SRT_ERR_UNSUPPORTED",
}

BXDF_DIFFUSE, BXDF_DIFFUSE_TRANSMISSION, BXDF_DIELECTRIC, BXDF_DISNEY = 0, 1, 2, 3
CAMERA_PERSPECTIVE, CAMERA_ORTHOGRAPHIC = 0, 1
CAMERA_MIRROR_X = 0x100  # flag OR'd into CameraDesc.type (left-handed pbrt camera frame)
RNG_CURAND, RNG_HASH = 0, 1
PT_FIXED_CDF_REMAP = 1
PT_NEE_FIRST_VERTEX_ONLY = 2
LAUNCH_GRAPH, LAUNCH_DIRECT = 0, 1
PT_TAIL_DEFAULT = 65536
TONE_NONE, TONE_CLAMP, TONE_REINHARD, TONE_UNCHARTED2, TONE_ACES = 0, 1, 2, 3, 4
METRIC_MSE, METRIC_MAPE, METRIC_SMAPE, METRIC_RELMSE = 0, 1, 2, 3
MEASURE_NONE, MEASURE_REFERENCE, MEASURE_ERROR = 0, 1, 2

f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)


class Bxdf(C.Structure):
    _fields_ = [("type", C.c_int32)] + [(n, C.c_float) for n in (
        "ior", "metallic", "subsurface", "roughness", "specular", "specularTint", "anisotropic",
        "sheen", "sheenTint", "clearcoat", "clearcoatGloss", "specTrans")]


class Material(C.Structure):
    _fields_ = [("bxdf", Bxdf), ("base_color", C.c_float * 3), ("emission_color", C.c_float * 3),
                ("intensity", C.c_float)]


class Mesh(C.Structure):
    _fields_ = [("vertices", f32p), ("indices", u32p), ("normals", f32p), ("num_vertices", C.c_int32),
                ("num_faces", C.c_int32), ("material_id", C.c_int32), ("pad", C.c_int32),
                ("texcoords", f32p), ("tangents", f32p)]


TEXTURE_RGBA8, TEXTURE_RGBA32F = 0, 1


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("format", C.c_int32), ("pad", C.c_int32),
                ("pixels", C.c_void_p)]


class Instance(C.Structure):
    _fields_ = [("mesh_id", C.c_int32), ("transform", C.c_float * 12)]


class CameraDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", C.c_float * 3), ("target", C.c_float * 3),
                ("up", C.c_float * 3), ("fov", C.c_float), ("aspect", C.c_float),
                ("aperture", C.c_float), ("focal", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(Mesh)), ("num_meshes", C.c_int32),
                ("instances", C.POINTER(Instance)), ("num_instances", C.c_int32),
                ("materials", C.POINTER(Material)), ("num_materials", C.c_int32),
                ("camera", CameraDesc), ("env_color", C.c_float * 3),
                ("textures", C.POINTER(Texture)), ("num_textures", C.c_int32), ("env_map", C.c_int32),
                ("material_textures", C.POINTER(C.c_int32))]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_int64), ("num_nodes", C.c_int64), ("num_lights", C.c_int64),
                ("device_bytes", C.c_int64), ("bvh_depth", C.c_int32), ("build_ms", C.c_float),
                ("light_weight_sum", C.c_float)]


class PtParams(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "samples_per_pixel", "max_depth", "rr_depth", "use_nee", "use_mis", "seed", "rng_mode", "flags")]


class PtStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("closest_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("iterations", C.c_int64), ("stack_overflows", C.c_int64), ("render_ms", C.c_float),
                ("kernel_launches", C.c_int64), ("kernel_ms", C.c_float * 5), ("closest_nodes", C.c_int64),
                ("closest_tris", C.c_int64), ("shadow_nodes", C.c_int64), ("shadow_tris", C.c_int64),
                ("tail_paths", C.c_int64), ("tail_ms", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_paths", C.c_int64), ("max_jobs", C.c_int32),
                ("iterations_per_step", C.c_int32)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("params", PtParams),
                ("film", C.c_void_p), ("cache", C.c_void_p), ("cache_train", C.c_int32), ("pad", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("frames_done", C.c_int32), ("submit_s", C.c_double),
                ("admit_s", C.c_double), ("first_frame_s", C.c_double), ("done_s", C.c_double),
                ("device_bytes", C.c_int64)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3
MLP_PARAMS = 23552


class CacheParams(C.Structure):
    _fields_ = [("train_paths", C.c_int32), ("train_steps", C.c_int32), ("learning_rate", C.c_float),
                ("region_threshold", C.c_float), ("region_res", C.c_int32), ("train", C.c_int32)]


class NrStats(C.Structure):
    _fields_ = [("rows", C.c_int64), ("encode_ms", C.c_float), ("network_ms", C.c_float)]


class CacheStats(C.Structure):
    _fields_ = [("queries", C.c_int64), ("fallback_queries", C.c_int64), ("train_vertices", C.c_int64),
                ("loss", C.c_float), ("disabled_cells", C.c_int32), ("trace_ms", C.c_float),
                ("train_ms", C.c_float)]


class BxdfBatch(C.Structure):
    _fields_ = [("n", C.c_int64), ("type", C.c_int32), ("normal", C.c_void_p), ("wo", C.c_void_p),
                ("color", C.c_void_p), ("params", C.c_void_p), ("rnd", C.c_void_p), ("wi", C.c_void_p),
                ("f", C.c_void_p), ("pdf", C.c_void_p), ("delta", C.c_void_p)]


# (name, restype, argtypes)
_PROTOS = [
    ("srt_last_error", C.c_char_p, []),
    ("srt_version", C.c_char_p, []),
    ("srt_scene_create", C.c_int, [C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    ("srt_scene_set_camera", C.c_int, [C.c_void_p, C.POINTER(CameraDesc)]),
    ("srt_scene_get_info", C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    ("srt_scene_prim_to_instance", C.c_int, [C.c_void_p, C.c_int64, i32p, i32p]),
    ("srt_scene_destroy", None, [C.c_void_p]),
    ("srt_trace_closest", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("srt_trace_shadow", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("srt_scene_texture_lookup", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("srt_pt_create", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    ("srt_pt_render", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(PtParams), C.c_void_p]),
    ("srt_lt_render", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(PtParams), C.POINTER(PtStats), C.c_void_p]),
    ("srt_nr_num_params", C.c_int64, []),
    ("srt_nr_create", C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    ("srt_nr_get_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("srt_nr_set_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("srt_nr_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("srt_nr_load", C.c_int, [C.c_void_p, C.c_char_p]),
    ("srt_nr_infer", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("srt_nr_set_profiling", C.c_int, [C.c_void_p, C.c_int32]),
    ("srt_nr_get_stats", C.c_int, [C.c_void_p, C.c_void_p]),
    ("srt_selftest_wait_timeout", C.c_int, [C.c_int64]),
    ("srt_nr_destroy", None, [C.c_void_p]),
    ("srt_nr_trace", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_void_p]),
    ("srt_nr_render", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                C.c_void_p, C.c_void_p]),
    ("srt_pt_get_stats", C.c_int, [C.c_void_p, C.POINTER(PtStats)]),
    ("srt_pt_set_profiling", C.c_int, [C.c_void_p, C.c_int32]),
    ("srt_pt_set_launch_mode", C.c_int, [C.c_void_p, C.c_int32]),
    ("srt_pt_set_tail", C.c_int, [C.c_void_p, C.c_int64]),
    ("srt_pt_get_iteration_counts", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    ("srt_pt_get_pixel_samples", C.c_int, [C.c_void_p, C.c_void_p]),
    ("srt_pt_destroy", None, [C.c_void_p]),
    ("srt_rng_tape", C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]),
    ("srt_bxdf_sample", C.c_int, [C.POINTER(BxdfBatch), C.c_void_p]),
    ("srt_bxdf_eval", C.c_int, [C.POINTER(BxdfBatch), C.c_void_p]),
    ("srt_bxdf_generate", C.c_int, [C.c_int64, C.POINTER(BxdfBatch), C.c_void_p]),
    ("srt_film_accumulate", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]),
    ("srt_film_tonemap", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_float, C.c_int32, C.c_void_p]),
    ("srt_film_metric_scratch_bytes", C.c_size_t, [C.c_int64]),
    ("srt_film_measure_view", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p]),
    ("srt_film_metric", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_float, C.c_void_p,
                                  f32p, C.c_void_p]),
    ("srt_mlp_create", C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    ("srt_mlp_set_box", C.c_int, [C.c_void_p, f32p, f32p]),
    ("srt_mlp_get_params", C.c_int, [C.c_void_p, f32p]),
    ("srt_mlp_set_params", C.c_int, [C.c_void_p, f32p]),
    ("srt_mlp_infer", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("srt_mlp_train_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, f32p, C.c_void_p]),
    ("srt_mlp_gradient", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, f32p, f32p, C.c_void_p]),
    ("srt_mlp_destroy", None, [C.c_void_p]),
    ("srt_pt_render_cached", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(PtParams), C.c_void_p,
                                       C.POINTER(CacheParams), C.POINTER(CacheStats), C.c_void_p]),
    ("srt_server_create", C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    ("srt_server_submit", C.c_int, [C.c_void_p, C.POINTER(JobDesc), C.POINTER(C.c_int64)]),
    ("srt_server_step", C.c_int, [C.c_void_p, i32p, i32p]),
    ("srt_server_drain", C.c_int, [C.c_void_p, C.c_double]),
    ("srt_server_job_info", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(JobInfo)]),
    ("srt_server_frame_times", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_int32, i32p]),
    ("srt_server_film", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    ("srt_server_release", C.c_int, [C.c_void_p, C.c_int64]),
    ("srt_server_now", C.c_double, [C.c_void_p]),
    ("srt_server_destroy", None, [C.c_void_p]),
    ("srt_film_metric_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_float, f32p,
                                          C.c_void_p]),
    ("srt_procedural_create", C.c_int, [C.c_char_p, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    ("srt_procedural_desc", C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    ("srt_procedural_destroy", None, [C.c_void_p]),
    ("srt_import_scene", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("srt_procedural_resolution", C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("srt_renderer_create", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("srt_renderer_run", C.c_int, [C.c_void_p, C.c_int32]),
    ("srt_renderer_size", C.c_int, [C.c_void_p, i32p, i32p]),
    ("srt_renderer_read_film", C.c_int, [C.c_void_p, f32p]),
    ("srt_renderer_save_pfm", C.c_int, [C.c_void_p, C.c_char_p]),
    ("srt_renderer_create_ex", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_void_p]),
    ("srt_renderer_create_file", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_void_p]),
    ("srt_renderer_output", C.c_char_p, [C.c_void_p]),
    ("srt_renderer_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("srt_image_write", C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32]),
    ("srt_image_read", C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p, C.c_int32]),
    ("srt_image_read_rgba8", C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p, C.c_int32]),
    ("srt_renderer_destroy", None, [C.c_void_p]),
    ("srt_registered_passes", C.c_char_p, []),
]

_lib = None


class SrtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: the CUDA library must be built "
                              "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, res, args in _PROTOS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def declared_symbols():
    return [p[0] for p in _PROTOS]


def check(status: int):
    if status != SRT_OK:
        raise SrtError(status, lib().srt_last_error().decode())
