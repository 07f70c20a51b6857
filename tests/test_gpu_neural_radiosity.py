"""The NeuralRadiosity pass (src/passes/npr/neural_radiosity.cu,
src/shader/npr/nr_lhs.cu, nr_rhs.cu) on the GPU against the oracle (GPU only).

The LHS / RHS raygen follows the oracle's streams (mask, base, weight and
network inputs per pixel).  The network runs in BF16 with FP32
accumulation on the GPU and in exact sums over BF16-rounded weights and
activations in the oracle; a hidden activation that lands next to a BF16
rounding boundary can round the other way, so outputs agree to about 2 %.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cornell(w, h):
    """The Cornell box with the room's triangles wound to face inwards: the
    RHS raygen takes the hit normal as it comes (no flip towards the
    viewer, nr_rhs.cu:83-118), so outward-facing walls would reject every
    BSDF sample."""
    import srt_gb300 as S
    sa = S.procedural("cornell")
    for m in sa.meshes[:3]:
        m["indices"] = np.ascontiguousarray(m["indices"][:, [0, 2, 1]])
    sa.camera.aspect = w / h
    return sa


def _trace(cuda, sc, w, h, type_, seed):
    import torch
    import srt_gb300 as S
    n = w * h
    mask = torch.zeros(n, dtype=torch.uint8, device=cuda)
    base = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    weight = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    inputs = torch.zeros((n, 12), dtype=torch.float32, device=cuda)
    S.check(S.lib().srt_nr_trace(sc.handle, w, h, type_, seed, C.c_void_p(mask.data_ptr()),
                                 C.c_void_p(base.data_ptr()), C.c_void_p(weight.data_ptr()),
                                 C.c_void_p(inputs.data_ptr()), None))
    torch.cuda.synchronize()
    return mask.cpu().numpy(), base.cpu().numpy(), weight.cpu().numpy(), inputs.cpu().numpy()


@pytest.mark.parametrize("type_", [0, 1])
def test_nr_trace_matches_oracle(cuda, type_):
    import srt_gb300 as S
    w, h = 40, 30
    sa = _cornell(w, h)
    sc = S.Scene(sa)
    gm, gb, gw, gi = _trace(cuda, sc, w, h, type_, 1234)
    om, ob, ow, oi = O.OracleScene(sa.desc()).nr_trace(w, h, type_, 1234)
    same = gm == om
    assert same.mean() > 0.98, same.mean()
    assert (gm == 0).sum() > 0.3 * w * h  # the network is asked for most pixels

    def close(a, b):
        return np.abs(a - b).max(1) <= 1e-4 * np.maximum(1.0, np.abs(b).max(1))
    ok = close(gb, ob) & close(gi, oi) & (close(gw, ow) if type_ == 1 else True)
    assert (ok & same).mean() > 0.95, (ok & same).mean()


def _net(cuda, seed=3, grid_scale=0.5):
    import srt_gb300 as S
    h = C.c_void_p()
    S.check(S.lib().srt_nr_create(seed, C.byref(h)))
    n = S.lib().srt_nr_num_params()
    p = np.zeros(n, np.float32)
    S.check(S.lib().srt_nr_get_params(h, p.ctypes.data_as(C.c_void_p)))
    # features large enough for the grid to matter in the output
    grid = n - (256 * 96 + 3 * 256 * 256 + 16 * 256)
    rng = np.random.default_rng(seed)
    p[:grid] = (rng.random(grid, dtype=np.float32) * 2 - 1) * grid_scale
    S.check(S.lib().srt_nr_set_params(h, p.ctypes.data_as(C.c_void_p)))
    return h, p


def _infer(cuda, h, inputs):
    import torch
    import srt_gb300 as S
    x = torch.from_numpy(np.ascontiguousarray(inputs, np.float32)).to(cuda)
    y = torch.zeros((len(inputs), 16), dtype=torch.float32, device=cuda)
    S.check(S.lib().srt_nr_infer(h, C.c_void_p(x.data_ptr()), len(inputs), C.c_void_p(y.data_ptr()), None))
    torch.cuda.synchronize()
    return y.cpu().numpy()[:, :3]


def test_nr_network_matches_oracle(cuda):
    import srt_gb300 as S
    h, p = _net(cuda)
    rng = np.random.default_rng(9)
    n = 5000
    pos = rng.random((n, 3), dtype=np.float32) * 2 - 1
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nm = rng.normal(size=(n, 3))
    nm /= np.linalg.norm(nm, axis=1, keepdims=True)
    col = rng.random((n, 3))
    inputs = np.concatenate([pos, (d + 1) / 2, (nm + 1) / 2, col], 1).astype(np.float32)
    g = _infer(cuda, h, inputs)
    o = O.nr_infer(p, inputs)
    scale = np.abs(o).max()
    assert scale > 1e-3
    err = np.abs(g - o)
    assert np.all(err <= 0.02 * scale + 0.02 * np.abs(o)), float((err / (0.02 * scale + 0.02 * np.abs(o))).max())
    # the grid is in play: moving the positions changes the output
    g2 = _infer(cuda, h, np.concatenate([pos * 0.5, inputs[:, 3:]], 1))
    assert np.abs(g2 - g).mean() > 0.01 * np.abs(g).mean()
    S.lib().srt_nr_destroy(h)


@pytest.mark.parametrize("type_", [0, 1])
def test_nr_render_matches_oracle(cuda, type_):
    import torch
    import srt_gb300 as S
    w, h = 32, 24
    sa = _cornell(w, h)
    sc = S.Scene(sa)
    net, p = _net(cuda, seed=5, grid_scale=0.2)
    seeds = (C.c_int32 * 2)(77, 1234567)
    film = torch.full((w * h, 4), -1.0, dtype=torch.float32, device=cuda)
    S.check(S.lib().srt_nr_render(sc.handle, net, w, h, type_, 2, seeds, C.c_void_p(film.data_ptr()), None))
    torch.cuda.synchronize()
    g = film.cpu().numpy()
    osc = O.OracleScene(sa.desc())
    acc = np.zeros((w * h, 3), np.float64)
    for s in seeds:
        m, b, wt, inp = osc.nr_trace(w, h, type_, s)
        y = O.nr_infer(p, inp)
        if type_ == 0:
            r = np.where(m[:, None] == 1, b, y)
        else:
            r = b + np.where(m[:, None] == 0, wt * y, 0.0)
        acc += r
    o = acc / 2
    assert np.all(g[:, 3] == 1.0)
    err = np.abs(g[:, :3] - o).max(1)
    scale = np.abs(o).max()
    assert np.mean(err <= 0.03 * scale) > 0.95, np.mean(err <= 0.03 * scale)
    S.lib().srt_nr_destroy(net)


def test_nr_pass_and_model_file(cuda, tmp_path):
    import json
    import srt_gb300 as S
    h, p = _net(cuda, seed=8)
    S.check(S.lib().srt_nr_save(h, str(tmp_path / "nr.bin").encode()))
    h2 = C.c_void_p()
    S.check(S.lib().srt_nr_create(99, C.byref(h2)))
    S.check(S.lib().srt_nr_load(h2, str(tmp_path / "nr.bin").encode()))
    q = np.zeros_like(p)
    S.check(S.lib().srt_nr_get_params(h2, q.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(p, q)
    (tmp_path / "bad.bin").write_bytes(b"not a model")
    assert S.lib().srt_nr_load(h2, str(tmp_path / "bad.bin").encode()) == 8
    w, hh = 24, 16
    cfg = {"render": {"resolution": [w, hh]},
           "passes": [{"name": "NeuralRadiosity",
                       "params": {"type": "RHS", "samples_per_pixel": 2, "model_path": str(tmp_path / "nr.bin")}}],
           "scene": {"model": "procedural:cornell",
                     "camera": {"type": "perspective", "position": [0, 0, 3.5], "target": [0, 0, 0],
                                "up": [0, 1, 0], "fov": 40}}}
    r = S.Renderer(json.dumps(cfg))
    r.run(1)
    film = r.film()
    assert np.all(np.isfinite(film)) and np.all(film[:, 3] == 1.0) and film[:, :3].max() > 0
    S.lib().srt_nr_destroy(h)
    S.lib().srt_nr_destroy(h2)
