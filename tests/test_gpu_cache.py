"""Radiance cache in the tracer (GPU only): online training on the tracer's
own paths, queries at the second vertex, per-cell plain fallback, and the
gain over plain path tracing at equal samples.

The error is measured against a high-spp plain render accumulated in FP64; the
relMSE is the reference's definition (((x - r) / (r + 1e-6))^2 averaged over
RGB, largest 0.1 % discarded, src/utils/metrics.h:30-34, measure.cu:46-49).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import golden, scene_from_npz
from oracle import oracle as O
from srt_gb300 import pt_params

pytestmark = pytest.mark.gpu

W = H = 64


def _setup(S, cuda):
    arr = scene_from_npz(golden("scene"))
    arr.set_aspect(W / H)
    scene = S.Scene(arr)
    pt = S.PathTracer(scene, W, H)
    mlp = C.c_void_p()
    S.check(S.lib().srt_mlp_create(11, C.byref(mlp)))
    lo = (C.c_float * 3)(-1.05, -1.05, -1.05)
    hi = (C.c_float * 3)(1.05, 1.05, 1.05)
    S.check(S.lib().srt_mlp_set_box(mlp, lo, hi))
    return arr, scene, pt, mlp


def _reference(S, scene, cuda, frames=32, spp=128):
    """Plain render, frames accumulated in FP64."""
    import torch
    pt = S.PathTracer(scene, W, H)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    acc = np.zeros((W * H, 4), np.float64)
    for f in range(frames):
        pt.render(film, pt_params(spp, 8, 3, 1, 1, 90000 + f))
        torch.cuda.synchronize()
        acc += film.cpu().numpy()
    return (acc / frames).astype(np.float32)


def _cached_frame(S, pt, film, mlp, seed, train=1, stats=None):
    p = pt_params(1, 8, 3, 1, 1, seed)
    cp = S._capi.CacheParams(1024, 4, 1e-2, 0.5, 8, train)  # one training pixel in 4
    st = S._capi.CacheStats()
    S.check(S.lib().srt_pt_render_cached(pt.handle, C.c_void_p(film.data_ptr()), C.byref(p), mlp, C.byref(cp),
                                         C.byref(st), None))
    return st


def test_cache_trains_and_queries(cuda):
    import torch
    import srt_gb300 as S
    arr, scene, pt, mlp = _setup(S, cuda)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    losses, queries = [], []
    for f in range(60):
        st = _cached_frame(S, pt, film, mlp, 1000 + f)
        losses.append(st.loss)
        queries.append(st.queries)
        assert st.train_vertices > 0
    torch.cuda.synchronize()
    img = film.cpu().numpy()
    assert np.all(np.isfinite(img)) and np.all(img[:, 3] == 1.0)
    # no cell is measured before the first training frame: that frame is traced plainly
    assert queries[0] == 0
    # once the cells are measured, the non-training pixels whose bounce ray hits
    # a wall (most of those not lost through the open front) end with a query
    assert min(queries[-10:]) > 0.25 * W * H
    assert np.mean(losses[-10:]) < np.mean(losses[:3])
    S.lib().srt_mlp_destroy(mlp)


def test_cache_gain_over_plain_at_equal_samples(cuda):
    """After online training, 8 cached 1-spp frames have a clearly lower
    relMSE against the FP64 reference than 8 plain 1-spp frames, and the
    cached image is not biased by more than a few percent overall."""
    import torch
    import srt_gb300 as S
    arr, scene, pt, mlp = _setup(S, cuda)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    for f in range(200):  # training frames
        _cached_frame(S, pt, film, mlp, 2000 + f)
    ref = _reference(S, scene, cuda)
    n = 8
    acc_c = np.zeros((W * H, 4))
    acc_p = np.zeros((W * H, 4))
    plain = S.PathTracer(scene, W, H)
    film_p = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    for f in range(n):
        _cached_frame(S, pt, film, mlp, 5000 + f, train=0)
        plain.render(film_p, pt_params(1, 8, 3, 1, 1, 5000 + f))
        torch.cuda.synchronize()
        acc_c += film.cpu().numpy()
        acc_p += film_p.cpu().numpy()
    rel_c, _ = O.metric((acc_c / n).astype(np.float32), ref, S.METRIC_RELMSE, 0.1)
    rel_p, _ = O.metric((acc_p / n).astype(np.float32), ref, S.METRIC_RELMSE, 0.1)
    assert rel_c < 0.85 * rel_p, (rel_c, rel_p)
    ratio = (acc_c / n)[:, :3].sum() / ref[:, :3].sum()
    assert abs(ratio - 1.0) < 0.05, ratio
    S.lib().srt_mlp_destroy(mlp)


def test_plain_render_after_cached_render_is_unchanged(cuda):
    """The same PathTracer handle renders plainly again (the cache kernel
    sees a plain job and does nothing): result equal to a fresh handle's."""
    import torch
    import srt_gb300 as S
    arr, scene, pt, mlp = _setup(S, cuda)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    _cached_frame(S, pt, film, mlp, 7)
    pt.render(film, pt_params(4, 8, 3, 1, 1, 77))
    fresh = S.PathTracer(scene, W, H)
    film2 = torch.zeros((W * H, 4), dtype=torch.float32, device=cuda)
    fresh.render(film2, pt_params(4, 8, 3, 1, 1, 77))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(film.cpu().numpy(), film2.cpu().numpy())
    S.lib().srt_mlp_destroy(mlp)
