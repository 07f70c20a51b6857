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
    cfg = b'{"render": {"resolution": [4, 4]}, "passes": [], "scene": {"model": "cornell_box.obj"}}'
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
