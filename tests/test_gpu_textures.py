"""Textures on the GPU against the oracle (GPU only).

The kernels read textures through CUDA texture objects set up as the
reference sets them up (Scene::build_gscene_textures, scene.cu:92-139):
bilinear filtering, wrap addressing, sRGB decode of 8-bit texels.  The
oracle computes the same lookups exactly; the hardware quantises the
filter weights to 1/256 and decodes sRGB from a table, so a lookup may
differ from the oracle by up to

    spread / 128 + 0.005 * max|texel| + 1e-6

where spread and max are taken over the four texels the lookup blends
(measured on a GB300: 200,000 lookups per format stay within 0.96 of it).
Renders use the oracle's per-pixel streams, so paths agree except where a
texture difference moves a Russian-roulette decision.
"""
import ctypes as C
import json

import numpy as np
import pytest

from oracle import oracle as O
from srt_gb300 import pt_params

pytestmark = pytest.mark.gpu


def _lookup_bound(tex, uv):
    """The tolerance above for each lookup (texels decoded as the oracle does)."""
    t = tex.astype(np.float64)
    if tex.dtype == np.uint8:
        c = t / 255.0
        t = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
        t[..., 3] = c[..., 3]
    H, W = tex.shape[:2]
    x = uv[:, 0].astype(np.float64)
    y = uv[:, 1].astype(np.float64)
    xb = (x - np.floor(x)) * W - 0.5
    yb = (y - np.floor(y)) * H - 0.5
    i0 = np.floor(xb).astype(int) % W
    j0 = np.floor(yb).astype(int) % H
    q = np.stack([t[j0, i0], t[j0, (i0 + 1) % W], t[(j0 + 1) % H, i0], t[(j0 + 1) % H, (i0 + 1) % W]], 0)
    return (q.max(0) - q.min(0)) / 128.0 + 0.005 * np.abs(q).max(0) + 1e-6


def _empty_scene():
    import srt_gb300 as S
    sa = S.SceneArrays()
    sa.camera.fov, sa.camera.aspect, sa.camera.focal = 40.0, 1.0, 1.0
    sa.camera.position[:] = [0.0, 0.0, 3.0]
    sa.camera.up[:] = [0.0, 1.0, 0.0]
    return sa


def test_texture_lookups_vs_oracle(cuda):
    import torch
    import srt_gb300 as S
    rng = np.random.default_rng(41)
    sa = _empty_scene()
    sa.textures = [rng.integers(0, 256, size=(5, 7, 4), dtype=np.uint8),
                   (rng.random((6, 9, 4), dtype=np.float32) * 4 - 1).astype(np.float32),
                   rng.integers(0, 256, size=(64, 32, 4), dtype=np.uint8)]
    sc = S.Scene(sa)
    osc = O.OracleScene(sa.desc())
    uv = (rng.random((50000, 2), dtype=np.float32) * 5 - 2).astype(np.float32)
    for k, tex in enumerate(sa.textures):
        u = torch.from_numpy(uv).to(cuda)
        out = torch.empty((len(uv), 4), dtype=torch.float32, device=cuda)
        S.check(S.lib().srt_scene_texture_lookup(sc.handle, k, C.c_void_p(u.data_ptr()), len(uv),
                                                 C.c_void_p(out.data_ptr()), None))
        g = out.cpu().numpy()
        o = osc.texture_lookup(k, uv)
        bound = _lookup_bound(tex, uv)
        ratio = np.abs(g - o) / bound
        assert ratio.max() <= 1.0, (k, float(ratio.max()))
    with pytest.raises(S.SrtError):
        S.check(S.lib().srt_scene_texture_lookup(sc.handle, 3, C.c_void_p(u.data_ptr()), 1,
                                                 C.c_void_p(out.data_ptr()), None))


def _textured_cornell(env=True):
    """The Cornell box with a checker colour texture on the white walls
    (texcoords that wrap), a normal map on the red wall, an emission texture
    on the lamp (barycentric texcoords), tangents on the tall box and a
    "uvmap" environment seen through the open front."""
    import srt_gb300 as S
    rng = np.random.default_rng(42)
    sa = S.procedural("cornell")
    room = sa.meshes[0]
    v = room["vertices"]
    room["texcoords"] = np.stack([v[:, 0] + v[:, 2] * 0.5, v[:, 1] * 1.5 + 0.25], -1).astype(np.float32)
    red = sa.meshes[1]
    red["texcoords"] = np.stack([red["vertices"][:, 2], red["vertices"][:, 1]], -1).astype(np.float32)
    box = sa.meshes[3]
    t = np.array([1.0, 0.3, 0.2], np.float32)
    box["tangents"] = np.tile(t / np.linalg.norm(t), (len(box["vertices"]), 1)).astype(np.float32)
    checker = np.zeros((8, 8, 4), np.uint8)
    checker[..., 3] = 255
    checker[(np.add.outer(np.arange(8), np.arange(8)) % 2) == 0, :3] = [230, 220, 200]
    checker[(np.add.outer(np.arange(8), np.arange(8)) % 2) == 1, :3] = [60, 90, 140]
    bumps = np.zeros((4, 4, 4), np.uint8)
    bumps[..., 0] = 255
    bumps[..., 1] = rng.integers(0, 120, size=(4, 4))
    bumps[..., 2] = rng.integers(0, 120, size=(4, 4))
    bumps[..., 3] = 255
    lamp = (rng.random((3, 3, 4), dtype=np.float32) * 0.5 + 0.6).astype(np.float32)
    sa.textures = [checker, bumps, lamp]
    mt = [(-1, -1)] * len(sa.materials)
    mt[0] = (0, -1)
    mt[1] = (-1, 1)
    light_mat = [i for i, m in enumerate(sa.materials) if m.intensity > 0][0]
    mt[light_mat] = (2, -1)
    sa.material_textures = mt
    if env:
        yy, xx = np.mgrid[0:8, 0:16].astype(np.float32)
        sky = np.stack([0.3 + 0.2 * np.sin(xx / 2.5), 0.4 + 0.1 * yy / 8, 0.6 + 0.0 * xx, np.ones_like(xx)], -1)
        sa.textures.append(sky.astype(np.float32))
        sa.env_map = 3
    return sa


def _render(cuda, sa, w, h, params):
    import torch
    import srt_gb300 as S
    sa.camera.aspect = w / h
    pt = S.PathTracer(S.Scene(sa), w, h)
    film = torch.full((w * h, 4), -1.0, dtype=torch.float32, device=cuda)
    pt.render(film, params)
    torch.cuda.synchronize()
    return film.cpu().numpy(), pt.stats()


@pytest.mark.parametrize("nee", [1, 0])
def test_textured_cornell_vs_oracle_streams(cuda, nee):
    w, h = 24, 20
    sa = _textured_cornell()
    p = pt_params(16, 8, 3, nee, nee, 777)
    film, st = _render(cuda, sa, w, h, p)
    of, _, _, cnt = O.OracleScene(sa.desc()).render(w, h, p)
    assert st["samples"] == cnt[0] and st["stack_overflows"] == 0
    g, o = film[:, :3].astype(np.float64), of[:, :3].astype(np.float64)
    rel = np.abs(g - o).max(1) / np.maximum(np.abs(o).max(1), 1e-3)
    assert np.mean(rel < 0.02) > 0.85, np.mean(rel < 0.02)
    assert abs(g.mean() - o.mean()) < 0.01 * o.mean()
    # the textures are in play: the same scene without them renders differently
    plain = _textured_cornell(env=False)
    plain.material_textures = None
    pf, _ = _render(cuda, plain, w, h, p)
    assert abs(pf[:, :3].mean() - g.mean()) > 0.02 * g.mean()


def test_environment_map_vs_oracle(cuda):
    """Every camera ray misses: the film is the "uvmap" lookup of the
    primary rays (EnvironmentLight::emission, light.h:27-41)."""
    w, h = 32, 16
    sa = _empty_scene()
    yy, xx = np.mgrid[0:32, 0:64].astype(np.float32)
    sky = np.stack([1.0 + np.sin(xx / 5.0), 0.5 + yy / 32.0, np.cos(yy / 7.0) ** 2, np.ones_like(xx)], -1)
    sa.textures = [sky.astype(np.float32)]
    sa.env_map = 0
    sa.camera.fov = 100.0
    p = pt_params(4, 4, 3, 0, 0, 5)  # no area light: no next-event estimation
    film, _ = _render(cuda, sa, w, h, p)
    of, _, _, _ = O.OracleScene(sa.desc()).render(w, h, p)
    assert np.abs(film[:, :3] - of[:, :3]).max() <= 0.01 * np.abs(sky).max() + 1e-6
    assert film[:, :3].std() > 0.05  # the map varies over the picture


def test_renderer_obj_with_textures_and_uvmap(cuda, tmp_path):
    """A textured OBJ beside its config with a "uvmap" environment, through
    the JSON renderer, against the oracle on the same imported arrays."""
    import srt_gb300 as S
    rng = np.random.default_rng(43)
    albedo = rng.integers(40, 250, size=(4, 6, 4), dtype=np.uint8)
    albedo[..., 3] = 255
    S.image_write(tmp_path / "albedo.png", (albedo / 255.0).astype(np.float32).reshape(-1, 4), 6, 4, flip=False)
    sky = (rng.random((8, 16, 4), dtype=np.float32) * 0.5 + 0.25).astype(np.float32)
    S.image_write(tmp_path / "sky.exr", sky.reshape(-1, 4), 16, 8, flip=False)
    (tmp_path / "room.mtl").write_text("newmtl wall\nKd 0.7 0.7 0.7\nmap_Kd albedo.png\n"
                                       "newmtl lamp\nKd 0 0 0\nKe 8 8 8\n")
    (tmp_path / "room.obj").write_text(
        "mtllib room.mtl\n"
        "v -1 -1 -1\nv 1 -1 -1\nv 1 1 -1\nv -1 1 -1\nv -1 -1 1\nv 1 -1 1\n"
        "v -0.3 0.99 -0.3\nv 0.3 0.99 -0.3\nv 0.3 0.99 0.3\nv -0.3 0.99 0.3\n"
        "vt 0 0\nvt 2 0\nvt 2 2\nvt 0 2\n"
        "o walls\nusemtl wall\nf 1/1 2/2 3/3 4/4\nf 1/1 5/4 6/3 2/2\n"
        "o lamp\nusemtl lamp\nf 7 8 9 10\n")
    cam = {"type": "perspective", "position": [0, 0, 3.5], "target": [0, 0, 0], "up": [0, 1, 0], "fov": 45}
    cfg = {"render": {"resolution": [32, 24]},
           "passes": [{"name": "PathTracer", "params": {"samples_per_pixel": 64, "max_depth": 6, "rr_depth": 3}},
                      {"name": "Accumulate", "params": {}}],
           "scene": {"model": "room.obj", "camera": cam, "environment": {"type": "uvmap", "path": "sky.exr"}}}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    r = S.Renderer(path=str(tmp_path / "cfg.json"))
    r.run(2)
    film = r.film()
    sa = S.import_scene(str(tmp_path / "room.obj"))
    assert len(sa.textures) == 1 and sa.material_textures[0] == (0, -1)
    sky_read, _, _ = S.image_read(tmp_path / "sky.exr", flip=False)
    sa.textures.append(sky_read.reshape(8, 16, 4))
    sa.env_map = 1
    sa.camera.type = S.CAMERA_PERSPECTIVE
    sa.camera.position[:] = [0, 0, 3.5]
    sa.camera.target[:] = [0, 0, 0]
    sa.camera.up[:] = [0, 1, 0]
    sa.camera.fov = 45.0
    sa.camera.aspect = 32 / 24
    of, _, _, _ = O.OracleScene(sa.desc()).render(32, 24, pt_params(128, 6, 3, 1, 1, 1234))
    assert abs(film[:, :3].mean() - of[:, :3].mean()) < 0.03 * of[:, :3].mean()
