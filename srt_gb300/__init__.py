"""srt_gb300 — GB300-native wavefront path tracer behind the C ABI of include/srt.h.

Python is a thin harness over the C ABI (ctypes): host scene arrays,
device buffers from torch, and the calls a user of the library makes.
Every compute call goes to the CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import json as _json
import os

import numpy as np

from . import _capi
from ._capi import (BXDF_DIELECTRIC, BXDF_DIFFUSE, BXDF_DIFFUSE_TRANSMISSION, BXDF_DISNEY, CAMERA_ORTHOGRAPHIC,
                    CAMERA_PERSPECTIVE, LAUNCH_DIRECT, LAUNCH_GRAPH, METRIC_MAPE, METRIC_MSE, METRIC_RELMSE,
                    METRIC_SMAPE, PT_FIXED_CDF_REMAP, PT_TAIL_DEFAULT, RNG_CURAND, RNG_HASH, TONE_ACES, TONE_CLAMP,
                    TONE_NONE, TONE_REINHARD, TONE_UNCHARTED2, SrtError, check, lib)

__all__ = [
    "SceneArrays", "Scene", "PathTracer", "procedural", "import_scene", "lib", "check", "SrtError", "bxdf_sample", "bxdf_eval",
    "bxdf_generate", "film_accumulate", "film_tonemap", "film_metric", "film_measure_view", "rng_tape", "Renderer", "image_write",
    "image_read", "image_read_rgba8",
]

DISNEY_PARAM_NAMES = ("ior", "metallic", "subsurface", "roughness", "specular", "specularTint", "anisotropic",
                      "sheen", "sheenTint", "clearcoat", "clearcoatGloss", "specTrans")


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class SceneArrays:
    """Host description of a scene (object-space meshes + instances) that
    builds the srt_scene_desc struct; it keeps the arrays alive."""

    def __init__(self):
        self.meshes = []      # dicts: vertices (V,3) f32, indices (F,3) u32, normals, texcoords (V,2),
        #                       tangents (V,3) (each optional / None), material
        self.instances = []   # (mesh_id, 3x4 transform)
        self.materials = []   # _capi.Material
        self.camera = _capi.CameraDesc()
        self.env = (0.0, 0.0, 0.0)
        self.resolution = (0, 0)  # film size an imported file asks for
        self.textures = []    # (H, W, 4) uint8 (sRGB) or float32 (linear) arrays, row 0 = v 0
        self.material_textures = None  # per material (color, normal) texture index or -1; None: untextured
        self.env_map = None   # texture index of a "uvmap" environment

    def desc(self):
        n = len(self.meshes)
        self._mesh_arr = (_capi.Mesh * max(1, n))()
        self._keep = []
        for i, m in enumerate(self.meshes):
            v = np.ascontiguousarray(m["vertices"], dtype=np.float32).reshape(-1, 3)
            f = np.ascontiguousarray(m["indices"], dtype=np.uint32).reshape(-1, 3)
            nr = None if m.get("normals") is None else np.ascontiguousarray(m["normals"], np.float32).reshape(-1, 3)
            tc = None if m.get("texcoords") is None else np.ascontiguousarray(m["texcoords"], np.float32).reshape(-1, 2)
            tg = None if m.get("tangents") is None else np.ascontiguousarray(m["tangents"], np.float32).reshape(-1, 3)
            self._keep += [v, f, nr, tc, tg]
            d = self._mesh_arr[i]
            d.vertices = v.ctypes.data_as(_capi.f32p)
            d.indices = f.ctypes.data_as(_capi.u32p)
            d.normals = nr.ctypes.data_as(_capi.f32p) if nr is not None else None
            d.texcoords = tc.ctypes.data_as(_capi.f32p) if tc is not None else None
            d.tangents = tg.ctypes.data_as(_capi.f32p) if tg is not None else None
            d.num_vertices, d.num_faces, d.material_id = len(v), len(f), int(m["material"])
        self._inst_arr = (_capi.Instance * max(1, len(self.instances)))()
        for i, (mid, xf) in enumerate(self.instances):
            self._inst_arr[i].mesh_id = mid
            for k, x in enumerate(np.asarray(xf, np.float32).reshape(12)):
                self._inst_arr[i].transform[k] = float(x)
        self._mat_arr = (_capi.Material * max(1, len(self.materials)))(*self.materials)
        d = _capi.SceneDesc()
        d.meshes, d.num_meshes = self._mesh_arr, n
        d.instances, d.num_instances = self._inst_arr, len(self.instances)
        d.materials, d.num_materials = self._mat_arr, len(self.materials)
        d.camera = self.camera
        for k in range(3):
            d.env_color[k] = float(self.env[k])
        if self.textures:
            self._tex_arr = (_capi.Texture * len(self.textures))()
            for i, t in enumerate(self.textures):
                a = np.ascontiguousarray(t)
                assert a.ndim == 3 and a.shape[2] == 4 and a.dtype in (np.uint8, np.float32)
                self._keep.append(a)
                tt = self._tex_arr[i]
                tt.height, tt.width = a.shape[0], a.shape[1]
                tt.format = _capi.TEXTURE_RGBA8 if a.dtype == np.uint8 else _capi.TEXTURE_RGBA32F
                tt.pixels = a.ctypes.data_as(C.c_void_p)
            d.textures, d.num_textures = self._tex_arr, len(self.textures)
        d.env_map = 0 if self.env_map is None else int(self.env_map) + 1
        if self.material_textures is not None:
            mt = np.ascontiguousarray(np.asarray(self.material_textures, np.int32).reshape(-1, 2))
            self._keep.append(mt)
            d.material_textures = mt.ctypes.data_as(C.POINTER(C.c_int32))
        self._desc = d
        return d

    @property
    def num_triangles(self):
        return sum(len(self.meshes[m]["indices"]) for m, _ in self.instances)

    def set_aspect(self, aspect):
        self.camera.aspect = float(aspect)


def _arrays_of(h) -> SceneArrays:
    """Copy of the host scene behind an srt_procedural handle."""
    L = lib()
    d = _capi.SceneDesc()
    check(L.srt_procedural_desc(h, C.byref(d)))
    s = SceneArrays()
    for i in range(d.num_meshes):
        m = d.meshes[i]
        v = np.ctypeslib.as_array(m.vertices, shape=(m.num_vertices * 3,)).reshape(-1, 3).copy()
        f = np.ctypeslib.as_array(m.indices, shape=(m.num_faces * 3,)).reshape(-1, 3).copy()
        n = tc = tg = None
        if m.normals and m.num_vertices:
            n = np.ctypeslib.as_array(m.normals, shape=(m.num_vertices * 3,)).reshape(-1, 3).copy()
        if m.texcoords and m.num_vertices:
            tc = np.ctypeslib.as_array(m.texcoords, shape=(m.num_vertices * 2,)).reshape(-1, 2).copy()
        if m.tangents and m.num_vertices:
            tg = np.ctypeslib.as_array(m.tangents, shape=(m.num_vertices * 3,)).reshape(-1, 3).copy()
        s.meshes.append({"vertices": v, "indices": f, "normals": n, "texcoords": tc, "tangents": tg,
                         "material": m.material_id})
    for i in range(d.num_instances):
        s.instances.append((d.instances[i].mesh_id, np.array(d.instances[i].transform[:], np.float32)))
    for i in range(d.num_materials):
        mm = _capi.Material()
        C.memmove(C.byref(mm), C.byref(d.materials[i]), C.sizeof(_capi.Material))
        s.materials.append(mm)
    C.memmove(C.byref(s.camera), C.byref(d.camera), C.sizeof(_capi.CameraDesc))
    s.env = tuple(d.env_color[:])
    for i in range(d.num_textures):
        t = d.textures[i]
        dt, nb = (np.uint8, 1) if t.format == _capi.TEXTURE_RGBA8 else (np.float32, 4)
        buf = (C.c_uint8 * (t.width * t.height * 4 * nb)).from_address(t.pixels)
        s.textures.append(np.frombuffer(buf, dt).reshape(t.height, t.width, 4).copy())
    s.env_map = d.env_map - 1 if d.env_map > 0 else None
    if d.material_textures:
        s.material_textures = [(d.material_textures[2 * i], d.material_textures[2 * i + 1])
                               for i in range(d.num_materials)]
    w, hh = C.c_int32(), C.c_int32()
    check(L.srt_procedural_resolution(h, C.byref(w), C.byref(hh)))
    s.resolution = (w.value, hh.value)
    return s


def image_write(path, rgba, width, height, flip=True):
    """srt_image_write of float4[w*h] host pixels (film order)."""
    px = np.ascontiguousarray(rgba, np.float32).reshape(-1)
    assert px.size == 4 * width * height
    check(lib().srt_image_write(os.fsencode(str(path)), width, height, _ptr(px), 1 if flip else 0))


def _flip_code(flip):
    return {False: 0, True: 1, "xy": 1, "y": 2, None: 0}[flip]


def image_read(path, flip=True):
    """srt_image_read: (float4[w*h] array, width, height) of an exr / hdr / pfm.
    flip: True / "xy" (load_from_file(p, true, true)), "y", or False."""
    L = lib()
    w, h = C.c_int32(), C.c_int32()
    check(L.srt_image_read(os.fsencode(str(path)), C.byref(w), C.byref(h), None, _flip_code(flip)))
    out = np.empty((w.value * h.value, 4), np.float32)
    check(L.srt_image_read(os.fsencode(str(path)), C.byref(w), C.byref(h), _ptr(out), _flip_code(flip)))
    return out, w.value, h.value


def image_read_rgba8(path, flip=False):
    """srt_image_read_rgba8: (uint8 RGBA [w*h, 4], width, height) of a png / bmp."""
    L = lib()
    w, h = C.c_int32(), C.c_int32()
    check(L.srt_image_read_rgba8(os.fsencode(str(path)), C.byref(w), C.byref(h), None, _flip_code(flip)))
    out = np.empty((w.value * h.value, 4), np.uint8)
    check(L.srt_image_read_rgba8(os.fsencode(str(path)), C.byref(w), C.byref(h), _ptr(out), _flip_code(flip)))
    return out, w.value, h.value


def procedural(name: str, seed: int = 1, n_spheres: int = 64, subdiv: int = 6) -> SceneArrays:
    """Host copy of a generated scene ("cornell" or "spheres")."""
    L = lib()
    h = C.c_void_p()
    check(L.srt_procedural_create(name.encode(), seed, n_spheres, subdiv, C.byref(h)))
    try:
        return _arrays_of(h)
    finally:
        L.srt_procedural_destroy(h)


def import_scene(path: str) -> SceneArrays:
    """Host copy of a scene file (.pbrt, .obj + .mtl, .ply) read by
    srt_import_scene; `resolution` holds the pbrt Film size or (0, 0)."""
    L = lib()
    h = C.c_void_p()
    check(L.srt_import_scene(os.fsencode(path), C.byref(h)))
    try:
        return _arrays_of(h)
    finally:
        L.srt_procedural_destroy(h)


class Scene:
    """A resident device scene (srt_scene_create)."""

    def __init__(self, arrays: SceneArrays):
        self.arrays = arrays
        self.handle = C.c_void_p()
        check(lib().srt_scene_create(C.byref(arrays.desc()), C.byref(self.handle)))

    def info(self):
        i = _capi.SceneInfo()
        check(lib().srt_scene_get_info(self.handle, C.byref(i)))
        return {k: getattr(i, k) for k, _ in _capi.SceneInfo._fields_}

    def set_camera(self, cam: _capi.CameraDesc):
        check(lib().srt_scene_set_camera(self.handle, C.byref(cam)))

    def prim_to_instance(self, prim: int):
        a, b = C.c_int32(), C.c_int32()
        check(lib().srt_scene_prim_to_instance(self.handle, prim, C.byref(a), C.byref(b)))
        return a.value, b.value

    def trace_closest(self, rays, hits, stream=0):
        """rays: device float32 [n, 8]; hits: device float32 [n, 4]."""
        check(lib().srt_trace_closest(self.handle, C.c_void_p(rays.data_ptr()), rays.shape[0],
                                      C.c_void_p(hits.data_ptr()), C.c_void_p(stream)))

    def trace_shadow(self, rays, visible, stream=0):
        check(lib().srt_trace_shadow(self.handle, C.c_void_p(rays.data_ptr()), rays.shape[0],
                                     C.c_void_p(visible.data_ptr()), C.c_void_p(stream)))

    def close(self):
        if self.handle:
            lib().srt_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pt_params(spp=1, max_depth=16, rr_depth=4, use_nee=True, use_mis=True, seed=0, rng_mode=RNG_CURAND, flags=0):
    p = _capi.PtParams()
    p.samples_per_pixel, p.max_depth, p.rr_depth = spp, max_depth, rr_depth
    p.use_nee, p.use_mis, p.seed, p.rng_mode, p.flags = int(use_nee), int(use_mis), seed, rng_mode, flags
    return p


class PathTracer:
    """The PathTracer pass on a resident scene (srt_pt_*)."""

    def __init__(self, scene: Scene, width: int, height: int):
        self.scene, self.width, self.height = scene, width, height
        self.handle = C.c_void_p()
        check(lib().srt_pt_create(scene.handle, width, height, C.byref(self.handle)))

    def render(self, film, params, stream=0):
        """film: device float32 [h*w, 4]."""
        check(lib().srt_pt_render(self.handle, C.c_void_p(film.data_ptr()), C.byref(params), C.c_void_p(stream)))

    def stats(self):
        s = _capi.PtStats()
        check(lib().srt_pt_get_stats(self.handle, C.byref(s)))
        out = {k: getattr(s, k) for k, _ in _capi.PtStats._fields_}
        out["kernel_ms"] = list(s.kernel_ms)
        return out

    def set_profiling(self, mode):
        """0 off; 1 (or True) timestamps + traversal work counters; 2 timestamps only."""
        check(lib().srt_pt_set_profiling(self.handle, int(mode)))

    def set_launch_mode(self, mode):
        """LAUNCH_GRAPH (one graph launch per frame) or LAUNCH_DIRECT (the
        same kernels launched one by one)."""
        check(lib().srt_pt_set_launch_mode(self.handle, int(mode)))

    def set_tail(self, max_paths):
        """Paths in flight at or below which one kernel finishes the frame's
        remaining samples (0: the wavefront iterations run to the end)."""
        check(lib().srt_pt_set_tail(self.handle, int(max_paths)))

    def iteration_counts(self, max_iterations=4096):
        """int32 [iterations, 5]: closest rays, hits, misses, shadow rays,
        samples ended, per wavefront iteration of the last render."""
        out = np.zeros((max_iterations, 5), np.int32)
        n = C.c_int32()
        check(lib().srt_pt_get_iteration_counts(self.handle, _ptr(out), max_iterations, C.byref(n)))
        return out[: min(n.value, max_iterations)].copy()

    def pixel_samples(self):
        """int32 [w*h]: finished samples per pixel of the last render."""
        out = np.zeros(self.width * self.height, np.int32)
        check(lib().srt_pt_get_pixel_samples(self.handle, _ptr(out)))
        return out

    def close(self):
        if self.handle:
            lib().srt_pt_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _batch(n, type_, normal, wo, color, params, rnd, wi, f, pdf, delta):
    b = _capi.BxdfBatch()
    b.n, b.type = n, type_
    for name, t in (("normal", normal), ("wo", wo), ("color", color), ("params", params), ("rnd", rnd),
                    ("wi", wi), ("f", f), ("pdf", pdf), ("delta", delta)):
        setattr(b, name, None if t is None else t.data_ptr())
    return b


def bxdf_sample(type_, normal, wo, color, params, rnd, wi, f, pdf, delta, stream=0):
    b = _batch(normal.shape[0], type_, normal, wo, color, params, rnd, wi, f, pdf, delta)
    check(lib().srt_bxdf_sample(C.byref(b), C.c_void_p(stream)))


def bxdf_eval(type_, normal, wo, color, params, rnd, wi, f, pdf, stream=0):
    b = _batch(normal.shape[0], type_, normal, wo, color, params, rnd, wi, f, pdf, None)
    check(lib().srt_bxdf_eval(C.byref(b), C.c_void_p(stream)))


def bxdf_generate(first, normal, wo, color, params, rnd, wi, f, pdf, stream=0):
    b = _batch(normal.shape[0], BXDF_DISNEY, normal, wo, color, params, rnd, wi, f, pdf, None)
    check(lib().srt_bxdf_generate(first, C.byref(b), C.c_void_p(stream)))


def film_accumulate(film, acc, frame_count, stream=0):
    check(lib().srt_film_accumulate(C.c_void_p(film.data_ptr()), C.c_void_p(acc.data_ptr()), film.shape[0],
                                    frame_count, C.c_void_p(stream)))


def film_tonemap(film, type_, exposure=0.0, use_gamma=True, stream=0):
    check(lib().srt_film_tonemap(C.c_void_p(film.data_ptr()), film.shape[0], type_, exposure, int(use_gamma),
                                 C.c_void_p(stream)))


def film_metric(x, ref, type_, discard=0.1, scratch=None, stream=0):
    import torch
    n = x.shape[0]
    if scratch is None:
        nbytes = lib().srt_film_metric_scratch_bytes(n)
        scratch = torch.empty(nbytes // 4 + 64, dtype=torch.float32, device=x.device)
    out = C.c_float()
    check(lib().srt_film_metric(C.c_void_p(x.data_ptr()), C.c_void_p(ref.data_ptr()), n, type_, discard,
                                C.c_void_p(scratch.data_ptr()), C.byref(out), C.c_void_p(stream)))
    return out.value


def film_measure_view(film, ref, type_, option, stream=0):
    """Measure's display option on device float4 tensors (in place on film)."""
    check(lib().srt_film_measure_view(C.c_void_p(film.data_ptr()), C.c_void_p(ref.data_ptr()), film.shape[0], type_,
                                      option, C.c_void_p(stream)))


def rng_tape(seed, npix, ndraws, out, stream=0):
    check(lib().srt_rng_tape(seed, npix, ndraws, C.c_void_p(out.data_ptr()), C.c_void_p(stream)))


class Renderer:
    """JSON-configured renderer (render / passes / scene) over the C ABI."""

    def __init__(self, config=None, *, path=None):
        """config: JSON text or dict (scene files resolve against the working
        directory); path: a config file (scene files resolve against its
        directory, srt_renderer_create_file)."""
        self.handle = C.c_void_p()
        if path is not None:
            check(lib().srt_renderer_create_file(os.fsencode(path), None, None, None, C.byref(self.handle)))
        else:
            text = config if isinstance(config, str) else _json.dumps(config)
            check(lib().srt_renderer_create(text.encode(), C.byref(self.handle)))
        w, h = C.c_int32(), C.c_int32()
        check(lib().srt_renderer_size(self.handle, C.byref(w), C.byref(h)))
        self.width, self.height = w.value, h.value

    def run(self, frames=1):
        check(lib().srt_renderer_run(self.handle, frames))

    def film(self):
        out = np.empty((self.height * self.width, 4), np.float32)
        check(lib().srt_renderer_read_film(self.handle, out.ctypes.data_as(_capi.f32p)))
        return out

    def save_pfm(self, path):
        check(lib().srt_renderer_save_pfm(self.handle, str(path).encode()))

    def save(self, path):
        """The film through srt_image_write with the reference's flip
        (png, bmp, hdr, pfm, exr by extension)."""
        check(lib().srt_renderer_save(self.handle, str(path).encode()))

    def close(self):
        if self.handle:
            lib().srt_renderer_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Render serving loop (srt_server_*): jobs share one wavefront engine."""

    def __init__(self, hbm_budget_bytes=150 << 30, max_paths=1 << 23, max_jobs=64, iterations_per_step=8):
        cfg = _capi.ServerConfig(hbm_budget_bytes, max_paths, max_jobs, iterations_per_step)
        self.handle = C.c_void_p()
        check(lib().srt_server_create(C.byref(cfg), C.byref(self.handle)))

    def submit(self, scene: Scene, width, height, params, film=None, cache=None, cache_train=False):
        """cache: an srt_mlp handle (radiance cache of the scene) or None;
        cache_train: the network trains online on this job's own paths."""
        d = _capi.JobDesc(scene.handle, width, height, params, None if film is None else film.data_ptr(),
                          cache, int(bool(cache_train)), 0)
        jid = C.c_int64()
        check(lib().srt_server_submit(self.handle, C.byref(d), C.byref(jid)))
        return jid.value

    def step(self):
        r, q = C.c_int32(), C.c_int32()
        check(lib().srt_server_step(self.handle, C.byref(r), C.byref(q)))
        return r.value, q.value

    def drain(self, timeout_s=600.0):
        check(lib().srt_server_drain(self.handle, timeout_s))

    def info(self, jid):
        i = _capi.JobInfo()
        check(lib().srt_server_job_info(self.handle, jid, C.byref(i)))
        return {k: getattr(i, k) for k, _ in _capi.JobInfo._fields_}

    def frame_times(self, jid, max_frames=4096):
        buf = (C.c_double * max_frames)()
        n = C.c_int32()
        check(lib().srt_server_frame_times(self.handle, jid, buf, max_frames, C.byref(n)))
        return list(buf[: min(n.value, max_frames)])

    def film_ptr(self, jid):
        p = C.c_void_p()
        check(lib().srt_server_film(self.handle, jid, C.byref(p)))
        return p.value

    def release(self, jid):
        check(lib().srt_server_release(self.handle, jid))

    def now(self):
        return lib().srt_server_now(self.handle)

    def close(self):
        if self.handle:
            lib().srt_server_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
