"""Writes the golden vectors that pin the CPU oracle to the reference.

Run in a container that has the reference tree (it builds
oracle/_ref/libsrtref.so from the reference's own device headers):

    python tests/golden/make_golden.py

Outputs (committed): tests/golden/bxdf.npz, camera.npz, pbrt_camera.npz,
image.npz with img_*.exr / img_stb.hdr (files written by the reference's
vendored tinyexr / stb_image_write), scene.npz (the
Cornell scene arrays plus light samples, hit attributes and a small
render, all produced by the reference's classes compiled for the host).
The Cornell scene arrays come from the library's procedural generator.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from srt_gb300 import _capi  # noqa: E402
from srt_gb300.build import build_reference  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _np(a):
    return a.ctypes.data_as(C.c_void_p)


def ref_sample(type_, normal, wo, color, params, rnd2):
    R = O.ref()
    n = len(normal)
    wi = np.zeros((n, 3), np.float32)
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    delta = np.zeros(n, np.int32)
    R.ref_bxdf_sample(type_, n, _np(normal), _np(wo), _np(color), _np(params), _np(np.ascontiguousarray(rnd2)),
                      _np(wi), _np(f), _np(pdf), _np(delta))
    return wi, f, pdf, delta


def ref_eval(type_, normal, wo, color, params, wi):
    R = O.ref()
    n = len(normal)
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    R.ref_bxdf_eval_pdf(type_, n, _np(normal), _np(wo), _np(color), _np(params), _np(np.ascontiguousarray(wi)),
                        _np(f), _np(pdf))
    return f, pdf


def bxdf_sets(n=4096):
    normal, wo, color, params, rnd4 = O.bxdf_inputs(0, n)
    rng = np.random.default_rng(7)
    sets = {}
    sets["disney"] = (_capi.BXDF_DISNEY, params)
    p2 = params.copy()
    p2[:, 11] = rng.random(n, dtype=np.float32)          # specTrans: refraction lobe
    sets["disney_trans"] = (_capi.BXDF_DISNEY, p2)
    sets["diffuse"] = (_capi.BXDF_DIFFUSE, params)
    sets["diffuse_transmission"] = (_capi.BXDF_DIFFUSE_TRANSMISSION, params)
    sets["dielectric"] = (_capi.BXDF_DIELECTRIC, params)
    out = {"normal": normal, "wo": wo, "color": color, "rnd4": rnd4}
    # independent directions for eval/pdf (both hemispheres)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out["wi_rand"] = d
    for name, (t, p) in sets.items():
        p = np.ascontiguousarray(p, np.float32)
        wi, f, pdf, delta = ref_sample(t, normal, wo, color, p, rnd4[:, :2].copy())
        fe, pe = ref_eval(t, normal, wo, color, p, d)
        out[f"{name}_type"] = np.int32(t)
        out[f"{name}_params"] = p
        out[f"{name}_wi"], out[f"{name}_f"], out[f"{name}_pdf"], out[f"{name}_delta"] = wi, f, pdf, delta
        out[f"{name}_eval_f"], out[f"{name}_eval_pdf"] = fe, pe
    np.savez_compressed(os.path.join(OUT, "bxdf.npz"), **out)


def camera_set():
    out = {}
    rng = np.random.default_rng(11)
    xy = rng.random((512, 2), dtype=np.float32)
    for name, typ, aspect, fov in (("persp", 0, 1.0, 40.0), ("persp_wide", 0, 16 / 9, 60.0), ("ortho", 1, 1.5, 40.0)):
        cam = _capi.CameraDesc()
        cam.type = typ
        cam.position[:] = [0.3, 0.2, 3.5]
        cam.target[:] = [0.0, -0.1, 0.0]
        cam.up[:] = [0.0, 1.0, 0.0]
        cam.fov, cam.aspect, cam.focal = fov, aspect, 1.0
        rays = np.zeros((512, 8), np.float32)
        O.ref().ref_camera_rays(C.cast(C.pointer(cam), C.c_void_p), 512, _np(xy), _np(rays))
        out[f"{name}_cam"] = np.array([typ, fov, aspect, 0.3, 0.2, 3.5, 0.0, -0.1, 0.0], np.float32)
        out[f"{name}_rays"] = rays
    out["xy"] = xy
    np.savez_compressed(os.path.join(OUT, "camera.npz"), **out)


def pbrt_lookat(eye, look, up, mirror=False):
    """The 16 numbers of a pbrt `Transform` statement for a camera made by
    pbrt's LookAt (camera-from-world; pbrt lists a matrix column by column),
    after an optional `Scale -1 1 1`."""
    eye, look, up = (np.asarray(a, np.float64) for a in (eye, look, up))
    d = look - eye
    d /= np.linalg.norm(d)
    right = np.cross(up / np.linalg.norm(up), d)
    right /= np.linalg.norm(right)
    new_up = np.cross(d, right)
    world_from_camera = np.eye(4)
    world_from_camera[:3, 0], world_from_camera[:3, 1], world_from_camera[:3, 2] = right, new_up, d
    world_from_camera[:3, 3] = eye
    m = np.linalg.inv(world_from_camera)
    if mirror:
        m = np.diag([-1.0, 1.0, 1.0, 1.0]) @ m
    return m.T.reshape(16).astype(np.float32)


PBRT_CAMERAS = (
    ("front", ([0.3, 1.2, 4.0], [0.0, 0.5, 0.0], [0.0, 1.0, 0.0]), False, 40.0, 4 / 3),
    ("above", ([-2.0, 3.0, -1.0], [0.5, 0.0, 0.2], [0.0, 1.0, 0.0]), False, 55.0, 16 / 9),
    ("tilted", ([1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [0.1, 0.9, 0.2]), False, 30.0, 1.0),
    ("mirrored", ([0.5, 1.5, -3.0], [0.0, 1.0, 0.0], [0.0, 1.0, 0.0]), True, 45.0, 1.5),
)


def pbrt_camera_set():
    """Rays of the reference's pbrt camera (PBRTParser::parse_options)."""
    out = {}
    rng = np.random.default_rng(12)
    xy = rng.random((256, 2), dtype=np.float32)
    for name, look, mirror, fov, aspect in PBRT_CAMERAS:
        m16 = pbrt_lookat(*look, mirror=mirror)
        rays = np.zeros((256, 8), np.float32)
        O.ref().ref_pbrt_camera_rays(_np(m16), fov, aspect, 256, _np(xy), _np(rays))
        out[f"{name}_m16"] = m16
        out[f"{name}_fov_aspect"] = np.array([fov, aspect], np.float32)
        out[f"{name}_rays"] = rays
    out["xy"] = xy
    np.savez_compressed(os.path.join(OUT, "pbrt_camera.npz"), **out)


def _img_lib():
    return C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libsrtimg.so"))


def golden_image_pixels():
    """37 x 29 RGBA: smooth ramps (compressible), values above 1 and below 0,
    and a block of random values."""
    h, w = 29, 37
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    px = np.stack([xx / w * 3.0 - 0.5, yy / h, np.round(xx / 8) / 4, np.ones_like(xx)], -1)
    rng = np.random.default_rng(21)
    px[20:26, 3:15] = rng.random((6, 12, 4), dtype=np.float32) * 100.0 - 20.0
    return px.reshape(-1, 4).astype(np.float32), w, h


def half_probe_values():
    """Float32 inputs whose half encodings pin the writer's rounding:
    random bit patterns, the midpoints between neighbouring halves (ties),
    overflow, subnormal and special values."""
    rng = np.random.default_rng(22)
    rand = rng.integers(0, 2**32, size=4096, dtype=np.uint64).astype(np.uint32).view(np.float32)
    hv = np.arange(0, 0x7c00, dtype=np.uint16).view(np.float16).astype(np.float64)
    mids = ((hv[:-1] + hv[1:]) / 2)[::15].astype(np.float32)
    special = np.array([0.0, -0.0, 1.0, 65504.0, 65519.0, 65520.0, 1e5, 2.0**-24, 2.0**-25, 1.5 * 2.0**-25,
                        2.0**-26, 1e-40, np.inf, -np.inf, np.nan, -np.nan], np.float32)
    return np.concatenate([special, mids, -mids, rand]).astype(np.float32)


def image_set():
    """Files written by the reference's image code (tinyexr as save_exr calls
    it, stb_image_write as save_hdr does) and what its load_from_file reads
    back from them."""
    L = _img_lib()
    px, w, h = golden_image_pixels()
    out = {"src": px, "size": np.array([w, h], np.int32)}
    for name, comp in (("none", 0), ("rle", 1), ("zips", 2), ("zip", 3), ("piz", 4)):
        path = os.path.join(OUT, f"img_{name}.exr")
        assert L.ref_save_exr(path.encode(), w, h, _np(px), comp) == 0
        if name != "piz":
            out[f"{name}_decoded"] = _ref_load(L, path)
    path = os.path.join(OUT, "img_stb.hdr")
    assert L.ref_save_stb(path.encode(), 0, w, h, _np(np.abs(px))) == 0
    out["stb_hdr_decoded"] = _ref_load(L, path)
    # half encodings: one-row image, channel B holds the probes
    v = half_probe_values()
    probe = np.zeros((len(v), 4), np.float32)
    probe[:, 2] = v
    tmp = os.path.join(OUT, "_probe.exr")
    assert L.ref_save_exr(tmp.encode(), len(v), 1, _np(probe), 0) == 0
    data = open(tmp, "rb").read()
    os.remove(tmp)
    out["half_in"] = v
    out["half_out"] = np.frombuffer(data[-2 * 4 * len(v):], np.uint16)[:len(v)].copy()  # B is the first channel
    np.savez_compressed(os.path.join(OUT, "image.npz"), **out)


def png_bytes(samples, w, h, ctype, depth, interlace=0, palette=None, trns=None):
    """A PNG written here from the specification (all five filter types in
    turn, optional Adam7) for the decoder fixtures; samples[y][x][c]."""
    import zlib
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]

    def pack_row(row):
        if depth >= 8:
            nb = depth // 8
            return b"".join(int(v).to_bytes(nb, "big") for px in row for v in px[:ch])
        bits, out, acc, n = depth, bytearray(), 0, 0
        for px in row:
            acc = (acc << bits) | int(px[0])
            n += bits
            if n == 8:
                out.append(acc)
                acc, n = 0, 0
        if n:
            out.append(acc << (8 - n))
        return bytes(out)

    bpp = max(1, ch * depth // 8)

    def filt(rows):
        out, prev, k = bytearray(), None, 0
        for r in rows:
            r = bytearray(r)
            p = prev if prev is not None else bytearray(len(r))
            ft = k % 5
            k += 1
            f = bytearray(len(r))
            for i in range(len(r)):
                a = r[i - bpp] if i >= bpp else 0
                b = p[i]
                c = p[i - bpp] if i >= bpp else 0
                if ft == 0:
                    pred = 0
                elif ft == 1:
                    pred = a
                elif ft == 2:
                    pred = b
                elif ft == 3:
                    pred = (a + b) >> 1
                else:
                    pp = a + b - c
                    pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                f[i] = (r[i] - pred) & 0xff
            out += bytes([ft]) + f
            prev = r
        return out

    raw = bytearray()
    if interlace:
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            rows = [pack_row([samples[y][x] for x in range(x0, w, dx)]) for y in range(y0, h, dy)]
            if rows and rows[0]:
                raw += filt(rows)
    else:
        raw += filt([pack_row(samples[y]) for y in range(h)])

    def chunk(t, d):
        return len(d).to_bytes(4, "big") + t + d + (zlib.crc32(t + d) & 0xffffffff).to_bytes(4, "big")
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", w.to_bytes(4, "big") + h.to_bytes(4, "big") +
                                       bytes([depth, ctype, 0, 0, interlace]))
    if palette is not None:
        out += chunk(b"PLTE", bytes(palette))
    if trns is not None:
        out += chunk(b"tRNS", bytes(trns))
    return out + chunk(b"IDAT", zlib.compress(bytes(raw), 6)) + chunk(b"IEND", b"")


PNG_CASES = (
    # name, colour type, bit depth, interlace
    ("g1", 0, 1, 0), ("g2", 0, 2, 0), ("g4", 0, 4, 1), ("g8", 0, 8, 0), ("g16", 0, 16, 1),
    ("rgb8", 2, 8, 0), ("rgb16", 2, 16, 0), ("rgb8i", 2, 8, 1), ("p1", 3, 1, 0), ("p4", 3, 4, 1), ("p8", 3, 8, 0),
    ("ga8", 4, 8, 0), ("ga16", 4, 16, 1), ("rgba8", 6, 8, 0), ("rgba16", 6, 16, 0), ("rgba8i", 6, 8, 1),
    ("g8t", 0, 8, 0), ("rgb8t", 2, 8, 0),
)


def png_set():
    """PNG decoder fixtures and what the reference's stbi_load(.., 4) makes of them."""
    L = _img_lib()
    rng = np.random.default_rng(23)
    out = {}
    for name, ctype, depth, inter in PNG_CASES:
        w, h = 13, 11
        ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
        top = (1 << depth) - 1 if ctype != 3 else min(15, (1 << depth) - 1)
        smp = rng.integers(0, top + 1, size=(h, w, ch))
        smp[2:5, 3:9] = smp[2, 3]  # a flat patch: long runs and zero filter residues
        palette = trns = None
        if ctype == 3:
            palette = rng.integers(0, 256, size=3 * (top + 1)).tolist()
            trns = rng.integers(0, 256, size=max(1, (top + 1) // 2)).tolist()
        if name.endswith("t"):
            key = smp[2, 3]
            trns = [b for v in key[:ch] for b in int(v).to_bytes(2, "big")]
        path = os.path.join(OUT, f"png_{name}.png")
        with open(path, "wb") as f:
            f.write(png_bytes(smp.tolist(), w, h, ctype, depth, inter, palette, trns))
        ww, hh = C.c_int(), C.c_int()
        a = np.zeros((w * h, 4), np.uint8)
        assert L.ref_load_u8_image(path.encode(), C.byref(ww), C.byref(hh), a.ctypes.data_as(C.c_void_p)) == 0
        out[name] = a
    np.savez_compressed(os.path.join(OUT, "png.npz"), **out)


def jpg_set():
    """JPEG fixtures written by the reference's stb_image_write and what its
    stbi_load(.., 4) decodes from them: quality 100 (4:4:4, what save_ldr
    writes), 75 (4:2:0), grey at 90."""
    L = _img_lib()
    h, w = 29, 37
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.stack([xx * 6 % 256, yy * 8 % 256, (xx + yy) * 3 % 256, np.full_like(xx, 255)], -1).astype(np.uint8)
    img[5:12, 5:20] = np.random.default_rng(24).integers(0, 256, size=(7, 15, 4))
    img[..., 3] = 255
    out = {"src": img}
    for name, comp, q in (("q100", 4, 100), ("q75", 3, 75), ("grey90", 1, 90)):
        px = np.ascontiguousarray(img[..., :comp])
        path = os.path.join(OUT, f"jpg_{name}.jpg")
        assert L.ref_save_jpg(path.encode(), w, h, comp, px.ctypes.data_as(C.c_void_p), q) == 0
        ww, hh = C.c_int(), C.c_int()
        a = np.zeros((w * h, 4), np.uint8)
        assert L.ref_load_u8_image(path.encode(), C.byref(ww), C.byref(hh), a.ctypes.data_as(C.c_void_p)) == 0
        out[name] = a
    np.savez_compressed(os.path.join(OUT, "jpg.npz"), **out)


def _ref_load(L, path):
    w, h = C.c_int(), C.c_int()
    assert L.ref_load_float_image(path.encode(), C.byref(w), C.byref(h), None) == 0
    a = np.zeros((w.value * h.value, 4), np.float32)
    assert L.ref_load_float_image(path.encode(), C.byref(w), C.byref(h), _np(a)) == 0
    return a


def scene_arrays_to_npz(s):
    out = {}
    out["num_meshes"] = np.int32(len(s.meshes))
    for i, m in enumerate(s.meshes):
        out[f"mesh{i}_v"] = m["vertices"].astype(np.float32)
        out[f"mesh{i}_f"] = m["indices"].astype(np.uint32)
        out[f"mesh{i}_mat"] = np.int32(m["material"])
    out["inst_mesh"] = np.array([i for i, _ in s.instances], np.int32)
    out["inst_xf"] = np.array([x for _, x in s.instances], np.float32)
    out["materials"] = np.frombuffer(b"".join(bytes(m) for m in s.materials), np.uint8)
    out["camera"] = np.frombuffer(bytes(s.camera), np.uint8)
    out["env"] = np.array(s.env, np.float32)
    return out


def scene_set():
    import srt_gb300 as S
    s = S.procedural("cornell")
    desc = s.desc()
    R = O.ref()
    h = R.ref_scene_create(C.cast(C.pointer(desc), C.c_void_p))
    out = scene_arrays_to_npz(s)
    rng = np.random.default_rng(5)
    u2 = rng.random((2048, 2), dtype=np.float32)
    ls = np.zeros((2048, 10), np.float32)
    R.ref_light_sample(h, 2048, _np(u2), _np(ls))
    out["light_u2"], out["light_ref"] = u2, ls
    ntri = sum(len(m["indices"]) for m in s.meshes)
    prim = rng.integers(0, ntri, 1024).astype(np.int32)
    uv = rng.random((1024, 2), dtype=np.float32)
    uv = np.where(uv.sum(1, keepdims=True) > 1, 1 - uv, uv).astype(np.float32)
    hi = np.zeros((1024, 15), np.float32)
    R.ref_hitinfo(h, 1024, _np(prim), _np(np.ascontiguousarray(uv)), _np(hi))
    out["hit_prim"], out["hit_uv"], out["hit_ref"] = prim, uv, hi
    # small renders through the reference's classes (curand streams, brute force hits)
    for tag, (w, hh, spp, md, rr, nee, mis, seed) in {
        "r0": (16, 16, 8, 8, 3, 1, 1, 1234),
        "r1": (12, 10, 4, 6, 2, 1, 0, 99),
        "r2": (10, 12, 4, 5, 3, 0, 0, 2024),
    }.items():
        film = np.zeros((w * hh, 4), np.float32)
        s.camera.aspect = w / hh
        desc = s.desc()
        R.ref_scene_destroy(h)
        h = R.ref_scene_create(C.cast(C.pointer(desc), C.c_void_p))
        R.ref_render(h, w, hh, 0, 0, w, hh, spp, md, rr, nee, mis, seed, _np(film))
        out[f"{tag}_cfg"] = np.array([w, hh, spp, md, rr, nee, mis, seed], np.int32)
        out[f"{tag}_film"] = film
    R.ref_scene_destroy(h)
    np.savez_compressed(os.path.join(OUT, "scene.npz"), **out)


if __name__ == "__main__":
    if build_reference() is None:
        sys.exit("the reference tree is needed to write golden vectors")
    O.build()
    bxdf_sets()
    camera_set()
    pbrt_camera_set()
    image_set()
    png_set()
    jpg_set()
    scene_set()
    print("golden vectors written to", OUT)
