"""ORACLE — ctypes wrapper of the CPU restatement (oracle/liboracle.so) and of
the reference-header build (oracle/_ref/libsrtref.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference arm, as the results the CUDA path is
compared against or as the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsrtref.so")

_vp = C.c_void_p
_i64 = C.c_int64


def _np(a):
    return a.ctypes.data_as(_vp)


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        protos = {
            "oracle_pcg_uniforms": (None, [C.c_uint64, C.c_uint64, C.c_int, _vp]),
            "oracle_bxdf_generate": (None, [_i64, _i64, _vp, _vp, _vp, _vp, _vp]),
            "oracle_bxdf_sample": (None, [C.c_int, C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
            "oracle_bxdf_sample_mt": (None, [C.c_int, C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                             C.c_int]),
            "oracle_bxdf_eval_pdf": (None, [C.c_int, C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
            "oracle_scene_create": (_vp, [_vp]),
            "oracle_scene_destroy": (None, [_vp]),
            "oracle_scene_num_triangles": (_i64, [_vp]),
            "oracle_scene_light_weight_sum": (C.c_float, [_vp]),
            "oracle_scene_build_bvh": (None, [_vp]),
            "oracle_trace_closest": (None, [_vp, _vp, _i64, _vp, _vp, C.c_int, C.c_int]),
            "oracle_trace_shadow": (None, [_vp, _vp, _i64, _vp, C.c_int, C.c_int]),
            "oracle_camera_rays": (None, [_vp, _i64, _vp, _vp]),
            "oracle_light_sample": (None, [_vp, _i64, _vp, C.c_int, _vp]),
            "oracle_hitinfo": (None, [_vp, _i64, _vp, _vp, _vp]),
            "oracle_texture_lookup": (None, [_vp, C.c_int, _i64, _vp, _vp]),
            "oracle_light_trace": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp, _vp]),
            "oracle_nr_trace": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
            "oracle_nr_infer": (None, [_vp, _i64, _vp, _vp, C.c_int]),
            "oracle_render": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int,
                                        C.c_int, _vp, _vp, _vp, _vp]),
            "oracle_render_events": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp,
                                               C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_int]),
            "oracle_render_pixels": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _i64, _vp, C.c_int, C.c_int, _vp, _vp,
                                               _vp, _vp]),
            "oracle_scene_create_procedural": (_vp, [C.c_char_p, C.c_uint64, C.c_int32, C.c_int32, C.c_float]),
            "oracle_accumulate": (None, [_vp, _vp, _i64, C.c_int]),
            "oracle_tonemap": (None, [_vp, _i64, C.c_int, C.c_float, C.c_int]),
            "oracle_metric": (C.c_double, [_vp, _vp, _i64, C.c_int, C.c_float, _vp]),
            "oracle_hash_uniform": (C.c_float, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
            "oracle_curand_tape": (None, [C.c_int, C.c_longlong, C.c_int, _vp]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    """The reference's own headers built for the host (only where built)."""
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        protos = {
            "ref_bxdf_sample": (None, [C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
            "ref_bxdf_eval_pdf": (None, [C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
            "ref_camera_rays": (None, [_vp, _i64, _vp, _vp]),
            "ref_pbrt_camera_rays": (None, [_vp, C.c_float, C.c_float, _i64, _vp, _vp]),
            "ref_scene_create": (_vp, [_vp]),
            "ref_scene_destroy": (None, [_vp]),
            "ref_light_sample": (None, [_vp, _i64, _vp, _vp]),
            "ref_hitinfo": (None, [_vp, _i64, _vp, _vp, _vp]),
            "ref_render": (None, [_vp] + [C.c_int] * 12 + [_vp]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _ref = L
    return _ref


# ---------------------------------------------------------------------------
# convenience wrappers
# ---------------------------------------------------------------------------

def bxdf_inputs(first, n):
    """Disney batch inputs from the PCG32 streams (host FP32)."""
    normal = np.empty((n, 3), np.float32)
    wo = np.empty((n, 3), np.float32)
    color = np.empty((n, 3), np.float32)
    params = np.empty((n, 12), np.float32)
    rnd4 = np.empty((n, 4), np.float32)
    lib().oracle_bxdf_generate(first, n, _np(normal), _np(wo), _np(color), _np(params), _np(rnd4))
    return normal, wo, color, params, rnd4


def bxdf_sample(precision, type_, normal, wo, color, params, rnd2, threads=1):
    n = len(normal)
    wi = np.zeros((n, 3), np.float64)
    f = np.zeros((n, 3), np.float64)
    pdf = np.zeros(n, np.float64)
    delta = np.zeros(n, np.int32)
    rnd2 = np.ascontiguousarray(rnd2, np.float32)
    lib().oracle_bxdf_sample_mt(precision, type_, n, _np(normal), _np(wo), _np(color), _np(params), _np(rnd2),
                                _np(wi), _np(f), _np(pdf), _np(delta), int(threads))
    return wi, f, pdf, delta


def bxdf_eval_pdf(precision, type_, normal, wo, color, params, wi):
    n = len(normal)
    f = np.zeros((n, 3), np.float64)
    pdf = np.zeros(n, np.float64)
    wi = np.ascontiguousarray(wi, np.float64)
    lib().oracle_bxdf_eval_pdf(precision, type_, n, _np(normal), _np(wo), _np(color), _np(params), _np(wi),
                               _np(f), _np(pdf))
    return f, pdf


class PtParams(C.Structure):
    """srt_pt_params of include/srt.h (the PathTracer JSON keys + frame seed)."""
    _fields_ = [("samples_per_pixel", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("use_nee", C.c_int32), ("use_mis", C.c_int32), ("seed", C.c_int32), ("rng_mode", C.c_int32),
                ("flags", C.c_int32)]


def pt_params(spp=1, max_depth=16, rr_depth=4, use_nee=True, use_mis=True, seed=0, rng_mode=0, flags=0):
    return PtParams(spp, max_depth, rr_depth, int(use_nee), int(use_mis), seed, rng_mode, flags)


class OracleScene:
    def __init__(self, desc, bvh=False, handle=None):
        self.h = handle if handle else lib().oracle_scene_create(C.cast(C.pointer(desc), _vp))
        if not self.h:
            raise ValueError("oracle_scene_create failed")
        self.has_bvh = False
        if bvh:
            self.build_bvh()

    @classmethod
    def procedural(cls, name, seed=1, n_spheres=64, subdiv=6, aspect=1.0, bvh=False):
        """The benchmark's procedural scene built inside the oracle library
        (same generator source as the CUDA library's srt_procedural_create)."""
        h = lib().oracle_scene_create_procedural(name.encode(), seed, n_spheres, subdiv, aspect)
        if not h:
            raise ValueError(f"oracle_scene_create_procedural({name}) failed")
        return cls(None, bvh=bvh, handle=h)

    def build_bvh(self):
        lib().oracle_scene_build_bvh(self.h)
        self.has_bvh = True

    @property
    def num_triangles(self):
        return lib().oracle_scene_num_triangles(self.h)

    def trace_closest(self, rays, threads=8):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        hits = np.zeros((n, 4), np.float32)
        edge = np.zeros(n, np.float32)
        lib().oracle_trace_closest(self.h, _np(rays), n, _np(hits), _np(edge), int(self.has_bvh), threads)
        return hits, edge

    def trace_shadow(self, rays, threads=8):
        rays = np.ascontiguousarray(rays, np.float32)
        vis = np.zeros(len(rays), np.int32)
        lib().oracle_trace_shadow(self.h, _np(rays), len(rays), _np(vis), int(self.has_bvh), threads)
        return vis

    def light_sample(self, u2, fixed=False):
        u2 = np.ascontiguousarray(u2, np.float32)
        out = np.zeros((len(u2), 10), np.float32)
        lib().oracle_light_sample(self.h, len(u2), _np(u2), int(fixed), _np(out))
        return out

    def hitinfo(self, prim, uv):
        prim = np.ascontiguousarray(prim, np.int32)
        uv = np.ascontiguousarray(uv, np.float32)
        out = np.zeros((len(prim), 15), np.float32)
        lib().oracle_hitinfo(self.h, len(prim), _np(prim), _np(uv), _np(out))
        return out

    def texture_lookup(self, texture, uv):
        uv = np.ascontiguousarray(uv, np.float32)
        out = np.zeros((len(uv), 4), np.float32)
        lib().oracle_texture_lookup(self.h, int(texture), len(uv), _np(uv), _np(out))
        return out

    def light_trace(self, w, h, params, threads=8):
        film = np.zeros((w * h, 3), np.float64)
        cnt = np.zeros(2, np.int64)
        rc = lib().oracle_light_trace(self.h, w, h, C.cast(C.pointer(params), _vp), int(self.has_bvh), threads,
                                      _np(film), _np(cnt))
        if rc != 0:
            raise ValueError(f"oracle_light_trace failed ({rc})")
        return film, cnt

    def nr_trace(self, w, h, type_, seed):
        n = w * h
        mask = np.zeros(n, np.uint8)
        base = np.zeros((n, 3), np.float32)
        weight = np.zeros((n, 3), np.float32)
        inputs = np.zeros((n, 12), np.float32)
        rc = lib().oracle_nr_trace(self.h, w, h, int(type_), int(seed), int(self.has_bvh), _np(mask), _np(base),
                                   _np(weight), _np(inputs))
        if rc != 0:
            raise ValueError(f"oracle_nr_trace failed ({rc})")
        return mask, base, weight, inputs

    def render(self, w, h, params, crop=None, threads=8):
        x0, y0, cw, ch = crop if crop else (0, 0, w, h)
        film = np.zeros((ch * cw, 4), np.float32)
        s1 = np.zeros((ch * cw, 3), np.float64)
        s2 = np.zeros((ch * cw, 3), np.float64)
        cnt = np.zeros(4, np.int64)
        rc = lib().oracle_render(self.h, w, h, x0, y0, cw, ch, C.cast(C.pointer(params), _vp), int(self.has_bvh),
                                 threads, _np(film), _np(s1), _np(s2), _np(cnt))
        if rc != 0:
            raise ValueError(f"oracle_render failed ({rc})")
        return film, s1, s2, cnt

    def render_pixels(self, w, h, params, pixels, threads=8):
        """The listed pixels (index iy*w + ix) of a w x h frame."""
        pixels = np.ascontiguousarray(pixels, np.int32)
        n = len(pixels)
        film = np.zeros((n, 4), np.float32)
        s1 = np.zeros((n, 3), np.float64)
        s2 = np.zeros((n, 3), np.float64)
        cnt = np.zeros(4, np.int64)
        rc = lib().oracle_render_pixels(self.h, w, h, _np(pixels), n, C.cast(C.pointer(params), _vp),
                                        int(self.has_bvh), threads, _np(film), _np(s1), _np(s2), _np(cnt))
        if rc != 0:
            raise ValueError(f"oracle_render_pixels failed ({rc})")
        return film, s1, s2, cnt

    def render_timeline(self, w, h, params, threads=8):
        """The whole frame plus its wavefront timeline: int64 [iterations, 5]
        = closest rays, hits, misses, shadow rays, samples ended, where
        iteration k holds segment k of every pixel's sample sequence (one
        path per pixel in flight, the next sample started in the iteration
        the previous one ends)."""
        n = w * h
        ev_max = max(1, params.samples_per_pixel * params.max_depth)
        film = np.zeros((n, 4), np.float32)
        s1 = np.zeros((n, 3), np.float64)
        s2 = np.zeros((n, 3), np.float64)
        cnt = np.zeros(4, np.int64)
        ev = np.zeros((n, ev_max), np.uint8)
        rc = lib().oracle_render_events(self.h, w, h, 0, 0, w, h, C.cast(C.pointer(params), _vp),
                                        int(self.has_bvh), threads, _np(film), _np(s1), _np(s2), _np(cnt), _np(ev),
                                        ev_max)
        if rc != 0:
            raise ValueError(f"oracle_render_events failed ({rc})")
        traced = (ev & 1).astype(bool)
        last = int(np.nonzero(traced.any(0))[0].max()) + 1 if traced.any() else 0
        tl = np.zeros((last, 5), np.int64)
        for k0 in range(0, last, 64):
            blk = ev[:, k0:min(last, k0 + 64)]
            tl[k0:k0 + blk.shape[1], 0] = (blk & 1).astype(bool).sum(0)
            tl[k0:k0 + blk.shape[1], 1] = (blk & 2).astype(bool).sum(0)
            tl[k0:k0 + blk.shape[1], 3] = (blk & 4).astype(bool).sum(0)
            tl[k0:k0 + blk.shape[1], 4] = (blk & 8).astype(bool).sum(0)
        tl[:, 2] = tl[:, 0] - tl[:, 1]
        return film, s1, s2, cnt, tl

    def __del__(self):
        try:
            if self.h:
                lib().oracle_scene_destroy(self.h)
        except Exception:
            pass


def nr_infer(params, inputs, threads=8):
    params = np.ascontiguousarray(params, np.float32)
    inputs = np.ascontiguousarray(inputs, np.float32)
    out = np.zeros((len(inputs), 3), np.float32)
    lib().oracle_nr_infer(_np(params), len(inputs), _np(inputs), _np(out), threads)
    return out


def camera_rays(cam, xy):
    xy = np.ascontiguousarray(xy, np.float32)
    rays = np.zeros((len(xy), 8), np.float32)
    lib().oracle_camera_rays(C.cast(C.pointer(cam), _vp), len(xy), _np(xy), _np(rays))
    return rays


def curand_tape(seed, npix, ndraws):
    out = np.zeros((npix, ndraws), np.float32)
    lib().oracle_curand_tape(seed, npix, ndraws, _np(out))
    return out


def accumulate(film, acc, frame_count):
    film = np.ascontiguousarray(film, np.float32).copy()
    acc = np.ascontiguousarray(acc, np.float32).copy()
    lib().oracle_accumulate(_np(film), _np(acc), len(film), frame_count)
    return film, acc


def tonemap(film, type_, exposure=0.0, use_gamma=True):
    film = np.ascontiguousarray(film, np.float32).copy()
    lib().oracle_tonemap(_np(film), len(film), type_, exposure, int(use_gamma))
    return film


def metric(x, ref_img, type_, discard=0.1):
    x = np.ascontiguousarray(x, np.float32)
    ref_img = np.ascontiguousarray(ref_img, np.float32)
    err = np.zeros(len(x), np.float32)
    v = lib().oracle_metric(_np(x), _np(ref_img), len(x), type_, discard, _np(err))
    return v, err
