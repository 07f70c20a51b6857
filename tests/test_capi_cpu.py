"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/srt.h declares, validates arguments before any
CUDA call, parses configurations, and generates the synthetic scenes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import srt_gb300 as S
from srt_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(srt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = S.lib()
    names = _declared("srt.h")
    assert len(names) > 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes mirror binds exactly the header's entry points
    assert set(_capi.declared_symbols()) <= set(names)


def test_version_and_passes():
    assert b"sm_103a" in S.lib().srt_version()
    assert set(S.lib().srt_registered_passes().decode().split(";")) >= {
        "PathTracer", "Wavefront", "Accumulate", "ToneMapping", "Measure"}


def test_scene_validation_errors():
    s = S.procedural("cornell")
    s.meshes[0]["indices"] = s.meshes[0]["indices"].copy()
    s.meshes[0]["indices"][0, 0] = 10_000
    with pytest.raises(S.SrtError) as e:
        S.Scene(s)
    assert e.value.status == 1 and "out of range" in str(e.value)
    s = S.procedural("cornell")
    s.instances.append((99, np.eye(3, 4, dtype=np.float32)))
    with pytest.raises(S.SrtError):
        S.Scene(s)
    s = S.procedural("cornell")
    s.materials[0].bxdf.type = 9
    with pytest.raises(S.SrtError):
        S.Scene(s)
    s = S.procedural("cornell")
    s.camera.type = 2  # thin lens is not built
    with pytest.raises(S.SrtError) as e:
        S.Scene(s)
    assert e.value.status == 9


def test_config_parse_errors_and_unknown_names():
    L = S.lib()
    h = C.c_void_p()
    assert L.srt_renderer_create(b"{ not json", C.byref(h)) == 8
    assert b"offset" in L.srt_last_error()
    cfg = b'{"render": {"resolution": [4, 4]}, "passes": [], "scene": {"model": "no_such_dir/cornell_box.obj"}}'
    assert L.srt_renderer_create(cfg, C.byref(h)) == 1  # a scene file that cannot be opened
    cfg = b'{"render": {"resolution": [4, 4]}, "passes": [], "scene": {"model": "cornell_box.gltf"}}'
    assert L.srt_renderer_create(cfg, C.byref(h)) == 9
    cfg = b'{"render": {"type": "interactive"}, "passes": [], "scene": {"model": "procedural:cornell"}}'
    assert L.srt_renderer_create(cfg, C.byref(h)) == 9
    # comments are allowed, as the reference's parser allows them
    cfg = b'// c\n{"render": {"resolution": [4, 4]}, /* x */ "passes": [], "scene": {"model": "procedural:nosuch"}}'
    assert L.srt_renderer_create(cfg, C.byref(h)) == 7


def test_procedural_scenes():
    c = S.procedural("cornell")
    assert c.num_triangles == 36
    lights = [m for m in c.materials if m.intensity > 0]
    assert len(lights) == 1
    le = np.array(lights[0].emission_color[:]) * lights[0].intensity
    np.testing.assert_allclose(le, [17, 12, 4], rtol=1e-6)
    s = S.procedural("spheres", seed=1, n_spheres=2, subdiv=6)
    assert s.num_triangles == 2 * 81920 + 2 + 4 * 2
    v = s.meshes[0]["vertices"]
    assert len(v) == 40962
    s2 = S.procedural("spheres", seed=1, n_spheres=2, subdiv=6)
    np.testing.assert_array_equal(s2.meshes[0]["vertices"], v)
    s3 = S.procedural("spheres", seed=2, n_spheres=2, subdiv=6)
    assert not np.array_equal(s3.meshes[0]["vertices"], v)
    with pytest.raises(S.SrtError):
        S.procedural("spheres", n_spheres=-1)
    with pytest.raises(S.SrtError):
        S.procedural("teapot")


def test_batch_argument_checks_without_gpu():
    L = S.lib()
    b = _capi.BxdfBatch()
    b.n, b.type = 10, 7
    assert L.srt_bxdf_sample(C.byref(b), None) == 1
    b.type = 3
    assert L.srt_bxdf_sample(C.byref(b), None) == 1  # NULL arrays
    assert L.srt_film_tonemap(None, 10, 99, 0.0, 1, None) == 1
    out = C.c_float()
    # keep == 0 returns NaN like the reference's 0/0
    assert L.srt_film_metric(None, None, 1, 0, 0.1, None, C.byref(out), None) == 0 and np.isnan(out.value)
    assert L.srt_film_metric_scratch_bytes(1000) >= 4000
    # path-tracer handle calls validate their arguments before any CUDA call
    assert L.srt_pt_set_launch_mode(None, S.LAUNCH_DIRECT) == 1
    assert L.srt_pt_set_tail(None, 0) == 1
    n = C.c_int32()
    assert L.srt_pt_get_iteration_counts(None, None, 0, C.byref(n)) == 1
    assert L.srt_pt_get_pixel_samples(None, None) == 1


def _film(w, h):
    rng = np.random.default_rng(3)
    f = rng.uniform(-0.2, 1.3, (h * w, 4)).astype(np.float32)
    f[0, :3] = (2.0, 0.5, 0.25)
    f[5, :3] = (1e-3, 4e-3, 0.0)
    return f


def _write(path, w, h, film, flip):
    return S.lib().srt_image_write(str(path).encode(), w, h, film.ctypes.data_as(C.c_void_p), flip)


def _flipped(film, w, h):
    """The reference's save order: film mirrored in x and y (Image::flip(true, true))."""
    return film.reshape(h, w, 4)[::-1, ::-1]


def _u8(x):
    return (np.clip(np.nan_to_num(x, nan=0.0), 0.0, 1.0) * np.float32(255.0)).astype(np.uint8)


def test_image_write_png_bmp(tmp_path):
    import struct
    import zlib
    w, h = 37, 23
    film = _film(w, h)
    want = _u8(_flipped(film, w, h))
    assert _write(tmp_path / "a.png", w, h, film, 1) == 0
    data = (tmp_path / "a.png").read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(typ + body)
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    assert ihdr == (w, h, 8, 6, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, w * 4 + 1)
    assert np.all(raw[:, 0] == 0)
    np.testing.assert_array_equal(raw[:, 1:].reshape(h, w, 4), want)
    # BMP: 24-bit BGR rows bottom to top, padded to 4 bytes
    assert _write(tmp_path / "a.bmp", w, h, film, 1) == 0
    b = (tmp_path / "a.bmp").read_bytes()
    assert b[:2] == b"BM" and struct.unpack("<iiHH", b[18:30]) == (w, h, 1, 24)
    row = (w * 3 + 3) & ~3
    px = np.frombuffer(b[54:], np.uint8).reshape(h, row)[::-1, :w * 3].reshape(h, w, 3)
    np.testing.assert_array_equal(px[..., ::-1], want[..., :3])


def test_image_write_hdr_pfm(tmp_path):
    w, h = 19, 11
    film = np.abs(_film(w, h))
    assert _write(tmp_path / "a.hdr", w, h, film, 1) == 0
    d = (tmp_path / "a.hdr").read_bytes()
    head, _, body = d.partition(b"\n\n")
    assert head.startswith(b"#?RADIANCE")
    dims, _, px = body.partition(b"\n")
    assert dims == f"-Y {h} +X {w}".encode()
    e = np.frombuffer(px, np.uint8).reshape(h, w, 4).astype(np.float64)
    got = np.where(e[..., 3:] > 0, (e[..., :3] + 0.5) * np.ldexp(1.0, e[..., 3:].astype(int) - 136), 0.0)
    want = _flipped(film, w, h)[..., :3]
    big = want.max(-1, keepdims=True)
    assert np.all(np.abs(got - want) <= big / 128 + 1e-30)
    # PFM: float RGB, rows bottom to top (film order), x mirrored with flip
    head = f"PF\n{w} {h}\n-1.0\n".encode()
    assert _write(tmp_path / "a.pfm", w, h, film, 1) == 0
    p = (tmp_path / "a.pfm").read_bytes()
    assert p.startswith(head)
    rgb = np.frombuffer(p[len(head):], np.float32).reshape(h, w, 3)
    np.testing.assert_array_equal(rgb, film.reshape(h, w, 4)[:, ::-1, :3])
    assert _write(tmp_path / "b.pfm", w, h, film, 0) == 0
    rgb0 = np.frombuffer((tmp_path / "b.pfm").read_bytes()[len(head):], np.float32)
    np.testing.assert_array_equal(rgb0.reshape(h, w, 3), film.reshape(h, w, 4)[..., :3])


def test_image_write_rejects_other_formats(tmp_path):
    film = _film(4, 4)
    assert _write(tmp_path / "a.tga", 4, 4, film, 1) == 9  # SRT_ERR_UNSUPPORTED
    assert _write(tmp_path / "a.png", 0, 4, film, 1) == 1  # SRT_ERR_ARG


def test_cli_usage_and_missing_config(tmp_path):
    import subprocess
    cli = os.path.join(ROOT, "srt_gb300", "srt")
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "-c config.json" in r.stdout
    r = subprocess.run([cli, "-c", str(tmp_path / "missing.json")], capture_output=True, text=True)
    assert r.returncode == 1 and "Failed to open file" in r.stderr
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1
