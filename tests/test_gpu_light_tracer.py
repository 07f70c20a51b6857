"""The LightTracer pass (src/shader/integrator/light_tracer.cu:57-175) on the
GPU against the oracle's restatement (GPU only).

Both trace the same light paths from the same per-launch-index curand
streams; the GPU adds splats with float atomics in whatever order they
arrive, the oracle sums them in double, and the two libraries' cosf / sinf
may differ in the last bit, which very rarely moves a path.  So most
pixels agree to 1e-3 and the image sums agree to 0.5 %.
"""
import json

import numpy as np
import pytest

from oracle import oracle as O
from srt_gb300 import pt_params

pytestmark = pytest.mark.gpu


def _lt(cuda, sa, w, h, p):
    import ctypes as C
    import torch
    import srt_gb300 as S
    sa.camera.aspect = w / h
    sc = S.Scene(sa)
    film = torch.full((w * h, 4), -1.0, dtype=torch.float32, device=cuda)
    st = S._capi.PtStats()
    S.check(S.lib().srt_lt_render(sc.handle, w, h, C.c_void_p(film.data_ptr()), C.byref(p), C.byref(st), None))
    torch.cuda.synchronize()
    return film.cpu().numpy(), st


@pytest.mark.parametrize("cfg", [dict(spp=16, max_depth=16, rr_depth=4, seed=11),
                                 dict(spp=4, max_depth=3, rr_depth=1, seed=2147480000)])
def test_light_tracer_matches_oracle(cuda, cfg):
    import srt_gb300 as S
    w, h = 32, 24
    sa = S.procedural("cornell")
    p = pt_params(cfg["spp"], cfg["max_depth"], cfg["rr_depth"], 1, 1, cfg["seed"])
    film, st = _lt(cuda, sa, w, h, p)
    of, cnt = O.OracleScene(sa.desc()).light_trace(w, h, p)
    assert np.all(film[:, 3] == 1.0)
    assert st.samples == w * h * cfg["spp"] and st.stack_overflows == 0
    assert abs(st.closest_rays - cnt[0]) <= 0.01 * cnt[0] + 2
    assert abs(st.shadow_rays - cnt[1]) <= 0.01 * cnt[1] + 2
    g = film[:, :3].astype(np.float64)
    rel = np.abs(g - of).max(1) / np.maximum(np.abs(of).max(1), 1e-6)
    assert np.mean(rel < 1e-3) > 0.9, np.mean(rel < 1e-3)
    assert abs(g.sum() - of.sum()) < 0.005 * of.sum()


def test_light_tracer_edge_cases(cuda):
    import ctypes as C
    import torch
    import srt_gb300 as S
    # no area light: the film is only cleared
    sa = S.procedural("cornell")
    for m in sa.materials:
        m.intensity = 0.0
    film, st = _lt(cuda, sa, 8, 6, pt_params(4, 8, 3, 1, 1, 1))
    assert np.all(film == np.array([0, 0, 0, 1], np.float32)) and st.closest_rays == 0
    # Camera::get_xy supports the perspective camera only
    sa = S.procedural("cornell")
    sa.camera.type = S.CAMERA_ORTHOGRAPHIC
    sc = S.Scene(sa)
    f = torch.zeros((48, 4), dtype=torch.float32, device=cuda)
    p = pt_params(1, 4, 3, 1, 1, 1)
    assert S.lib().srt_lt_render(sc.handle, 8, 6, C.c_void_p(f.data_ptr()), C.byref(p), None, None) == 9


def test_light_tracer_pass_through_the_renderer(cuda):
    import srt_gb300 as S
    w, h = 32, 24
    cfg = {"render": {"resolution": [w, h]},
           "passes": [{"name": "LightTracer", "params": {"samples_per_pixel": 32, "max_depth": 16, "rr_depth": 4}},
                      {"name": "Accumulate", "params": {}}],
           "scene": {"model": "procedural:cornell",
                     "camera": {"type": "perspective", "position": [0, 0, 3.5], "target": [0, 0, 0],
                                "up": [0, 1, 0], "fov": 40}}}
    r = S.Renderer(json.dumps(cfg))
    r.run(4)
    film = r.film()
    sa = S.procedural("cornell")
    sa.camera.aspect = w / h
    of, _ = O.OracleScene(sa.desc()).light_trace(w, h, pt_params(128, 16, 4, 1, 1, 77))
    assert abs(film[:, :3].mean() - of.mean()) < 0.05 * of.mean()
