"""Imported scene files rendered on the GPU against the oracle (GPU only).

The Cornell box of the procedural generator is written out as a pbrt file
(binary and ascii plymesh, trianglemesh with and without normals, a conductor
and a coated-diffuse box as separate shapes under their own world Transform,
the lamp as an AreaLightSource inside an attribute block, a camera given by
its Transform) and as OBJ + MTL, read back with srt_import_scene, and
rendered by the PathTracer with the same per-pixel streams as the oracle.
The renderer and the `srt` command find the files next to their config.
"""
import json
import os
import struct
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from srt_gb300 import pt_params

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nums(a):
    return " ".join(repr(float(x)) for x in np.asarray(a).reshape(-1))


def _pbrt_lookat(eye, look, up, mirror=False):
    """pbrt's LookAt camera-from-world, listed column by column as pbrt does,
    after an optional Scale -1 1 1."""
    eye, look, up = (np.asarray(a, np.float64) for a in (eye, look, up))
    d = (look - eye) / np.linalg.norm(look - eye)
    right = np.cross(up / np.linalg.norm(up), d)
    right /= np.linalg.norm(right)
    wfc = np.eye(4)
    wfc[:3, 0], wfc[:3, 1], wfc[:3, 2], wfc[:3, 3] = right, np.cross(d, right), d, eye
    m = np.linalg.inv(wfc)
    if mirror:
        m = np.diag([-1.0, 1.0, 1.0, 1.0]) @ m
    return m.T.reshape(16)


def _face_normals(v, f):
    n = np.zeros_like(v)
    for a, b, c in f:
        g = np.cross(v[b] - v[a], v[c] - v[a])
        g /= np.linalg.norm(g)
        for k in (a, b, c):
            n[k] = g
    return n


def _cornell():
    import srt_gb300 as S
    return S.procedural("cornell")


def _ply_binary(path, v, f, n):
    hdr = ("ply\nformat binary_little_endian 1.0\n"
           f"element vertex {len(v)}\nproperty float x\nproperty float y\nproperty float z\n"
           "property float nx\nproperty float ny\nproperty float nz\n"
           f"element face {len(f)}\nproperty list uchar int vertex_indices\nend_header\n")
    body = b"".join(struct.pack("<6f", *v[i], *n[i]) for i in range(len(v)))
    body += b"".join(struct.pack("<B3i", 3, *map(int, t)) for t in f)
    path.write_bytes(hdr.encode() + body)


def _ply_ascii(path, v, f):
    path.write_text("ply\nformat ascii 1.0\n"
                    f"element vertex {len(v)}\nproperty float x\nproperty float y\nproperty float z\n"
                    f"element face {len(f)}\nproperty list uchar int vertex_indices\nend_header\n"
                    + "".join(f"{a!r} {b!r} {c!r}\n" for a, b, c in v.tolist())
                    + "".join(f"3 {a} {b} {c}\n" for a, b, c in f.tolist()))


def write_cornell_pbrt(folder, film, mirror=False):
    c = _cornell()
    folder.mkdir(parents=True, exist_ok=True)
    (folder / "meshes").mkdir(exist_ok=True)
    mats = c.materials
    lines = ['Integrator "volpath" "integer maxdepth" [ 8 ]',
             f'Transform [ {_nums(_pbrt_lookat([0, 0, 3.5], [0, 0, 0], [0, 1, 0], mirror))} ]',
             'Sampler "zsobol" "integer pixelsamples" [ 16 ]',
             f'Film "rgb" "integer xresolution" [ {film[0]} ] "integer yresolution" [ {film[1]} ]',
             'Camera "perspective" "float fov" [ 40 ]', "WorldBegin"]
    for k in range(3):
        lines.append(f'MakeNamedMaterial "m{k}" "string type" [ "diffuse" ] "rgb reflectance" [ {_nums(mats[k].base_color)} ]')
    boxes = 0
    for i, (mid, xf) in enumerate(c.instances):
        m = c.meshes[mid]
        mat_id = m["material"]
        x4 = np.vstack([np.asarray(xf, np.float64).reshape(3, 4), [0, 0, 0, 1]])
        v, f = m["vertices"], m["indices"]
        shape = (f'Shape "trianglemesh" "integer indices" [ {" ".join(map(str, f.reshape(-1)))} ] '
                 f'"point3 P" [ {_nums(v)} ]')
        if mat_id == 0:  # floor, ceiling and back wall
            _ply_binary(folder / "meshes" / "room.ply", v, f, _face_normals(v.astype(np.float64), f))
            lines += [f'Transform [ {_nums(x4.T)} ]', 'NamedMaterial "m0"', 'Shape "plymesh" "string filename" "meshes/room.ply"']
        elif mat_id in (1, 2):  # red and green walls
            lines += [f'Transform [ {_nums(x4.T)} ]', f'NamedMaterial "m{mat_id}"',
                      shape + f' "normal N" [ {_nums(_face_normals(v.astype(np.float64), f))} ]']
        elif mats[mat_id].intensity == 0:  # the two boxes
            mat = ('Material "conductor" "float roughness" [ 0.2 ]' if boxes == 0 else
                   'Material "coateddiffuse" "rgb reflectance" [ 0.725 0.725 0.725 ] "float roughness" [ 0.3 ]')
            boxes += 1
            lines += [f'Transform [ {_nums(x4.T)} ]', mat, shape]
        else:
            le = np.asarray(mats[mat_id].emission_color[:]) * mats[mat_id].intensity
            _ply_ascii(folder / "meshes" / "lamp.ply", v, f)
            lines += ["AttributeBegin", f'  Transform [ {_nums(x4.T)} ]',
                      '  Material "diffuse" "rgb reflectance" [ 0 0 0 ]',
                      f'  AreaLightSource "diffuse" "rgb L" [ {_nums(le)} ]',
                      '  Shape "plymesh" "string filename" [ "meshes/lamp.ply" ]', "AttributeEnd"]
    (folder / "box.pbrt").write_text("\n".join(lines) + "\n")
    return folder / "box.pbrt"


def write_cornell_obj(folder):
    c = _cornell()
    folder.mkdir(parents=True, exist_ok=True)
    mtl, obj, base = [], ["mtllib box.mtl"], 1
    for k, m in enumerate(c.materials):
        le = np.asarray(m.emission_color[:]) * m.intensity
        mtl += [f"newmtl m{k}", f"Kd {_nums(m.base_color)}", f"Ke {_nums(le)}", "Ni 1.5", "Pr 0.5"]
    for i, (mid, xf) in enumerate(c.instances):
        m = c.meshes[mid]
        x = np.asarray(xf, np.float64).reshape(3, 4)
        v = m["vertices"].astype(np.float64) @ x[:, :3].T + x[:, 3]
        obj += [f"o part{i}", f"usemtl m{m['material']}"] + [f"v {_nums(p)}" for p in v]
        obj += [f"f {a + base} {b + base} {cc + base}" for a, b, cc in m["indices"].tolist()]
        base += len(v)
    (folder / "box.mtl").write_text("\n".join(mtl) + "\n")
    (folder / "box.obj").write_text("\n".join(obj) + "\n")
    return folder / "box.obj"


def _render(cuda, sa, w, h, params):
    import torch
    import srt_gb300 as S
    pt = S.PathTracer(S.Scene(sa), w, h)
    film = torch.full((w * h, 4), -1.0, dtype=torch.float32, device=cuda)
    pt.render(film, params)
    torch.cuda.synchronize()
    return film.cpu().numpy(), pt.stats()


@pytest.mark.parametrize("mirror", [False, True])
def test_imported_pbrt_matches_oracle_streams(cuda, tmp_path, mirror):
    import srt_gb300 as S
    w, h = 24, 20
    sa = S.import_scene(str(write_cornell_pbrt(tmp_path, (w, h), mirror)))
    assert sa.resolution == (w, h) and len(sa.instances) == 6
    assert (sa.camera.type & S._capi.CAMERA_MIRROR_X) == (0 if mirror else S._capi.CAMERA_MIRROR_X)
    assert sa.meshes[0]["normals"] is not None
    p = pt_params(16, 8, 3, 1, 1, 4321)
    film, st = _render(cuda, sa, w, h, p)
    of, _, _, cnt = O.OracleScene(sa.desc()).render(w, h, p)
    assert np.all(film[:, 3] == 1.0) and st["stack_overflows"] == 0
    assert st["samples"] == w * h * 16 == cnt[0]
    d = np.abs(film[:, :3] - of[:, :3]).max(1)
    same = d <= 1e-4 * np.maximum(1.0, np.abs(of[:, :3]).max(1))
    assert np.mean(same) > 0.9, np.mean(same)
    assert abs(st["closest_rays"] - cnt[1]) <= 0.01 * cnt[1] + 2


def test_pbrt_scale_minus_one_mirrors_the_picture(cuda, tmp_path):
    """A pbrt `Scale -1 1 1` camera sees the scene mirrored left to right."""
    import srt_gb300 as S
    w, h, spp = 16, 12, 256
    p = pt_params(spp, 6, 3, 1, 1, 99)
    a, _ = _render(cuda, S.import_scene(str(write_cornell_pbrt(tmp_path / "a", (w, h), False))), w, h, p)
    b, _ = _render(cuda, S.import_scene(str(write_cornell_pbrt(tmp_path / "b", (w, h), True))), w, h, p)
    a = a[:, :3].reshape(h, w, 3)
    b = b[:, :3].reshape(h, w, 3)
    # the red and the green wall sit on opposite sides of the picture
    left, right = a[:, : w // 4, 0].mean(), a[:, -(w // 4):, 0].mean()
    assert max(left, right) > 1.5 * min(left, right)
    # per-column colour profiles: b is a mirrored left to right
    assert abs(b.mean() - a.mean()) < 0.05 * a.mean()
    assert np.corrcoef(b.mean(0).reshape(-1), a[:, ::-1].mean(0).reshape(-1))[0, 1] > 0.98
    rg_a, rg_b = (a[..., 0] - a[..., 1]).mean(0), (b[..., 0] - b[..., 1]).mean(0)
    q = w // 4
    side_a, side_b = rg_a[:q].mean() - rg_a[-q:].mean(), rg_b[:q].mean() - rg_b[-q:].mean()
    assert side_a * side_b < 0 and abs(side_b) > 0.5 * abs(side_a)
    assert np.corrcoef(rg_b, rg_a[::-1])[0, 1] > 0.9


def test_renderer_loads_pbrt_next_to_its_config(cuda, tmp_path):
    import srt_gb300 as S
    write_cornell_pbrt(tmp_path / "scenes", (32, 24))
    cfg = {"render": {"type": "image"},
           "passes": [{"name": "PathTracer", "params": {"samples_per_pixel": 64, "max_depth": 8, "rr_depth": 3}},
                      {"name": "Accumulate", "params": {}}],
           "scene": {"model": "scenes/box.pbrt"}}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    r = S.Renderer(path=str(tmp_path / "cfg.json"))
    assert (r.width, r.height) == (32, 24)  # the pbrt Film size stands in for the unset resolution
    r.run(2)
    film = r.film()
    sa = S.import_scene(str(tmp_path / "scenes" / "box.pbrt"))
    of, _, _, _ = O.OracleScene(sa.desc()).render(32, 24, pt_params(128, 8, 3, 1, 1, 999))
    assert abs(film[:, :3].mean() - of[:, :3].mean()) < 0.03 * of[:, :3].mean()
    # a render.resolution overrides the Film and sets the camera aspect
    cfg["render"]["resolution"] = [20, 10]
    (tmp_path / "cfg2.json").write_text(json.dumps(cfg))
    r2 = S.Renderer(path=str(tmp_path / "cfg2.json"))
    assert (r2.width, r2.height) == (20, 10)


def test_renderer_obj_with_camera_block(cuda, tmp_path):
    import srt_gb300 as S
    write_cornell_obj(tmp_path)
    cam = {"type": "perspective", "position": [0, 0, 3.5], "target": [0, 0, 0], "up": [0, 1, 0], "fov": 40}
    cfg = {"render": {"resolution": [32, 24]},
           "passes": [{"name": "PathTracer", "params": {"samples_per_pixel": 64, "max_depth": 8, "rr_depth": 3}},
                      {"name": "Accumulate", "params": {}}],
           "scene": {"model": "box.obj", "camera": cam}}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    r = S.Renderer(path=str(tmp_path / "cfg.json"))
    r.run(2)
    film = r.film()
    sa = S.import_scene(str(tmp_path / "box.obj"))
    assert len(sa.meshes) == 6
    sa.camera = _cornell().camera
    sa.camera.aspect = 32 / 24
    of, _, _, _ = O.OracleScene(sa.desc()).render(32, 24, pt_params(128, 8, 3, 1, 1, 999))
    assert abs(film[:, :3].mean() - of[:, :3].mean()) < 0.03 * of[:, :3].mean()


def test_cli_renders_a_pbrt_scene(cuda, tmp_path):
    write_cornell_pbrt(tmp_path / "scenes", (30, 20))
    cfg = {"render": {"type": "image", "output": "out.pfm"},
           "passes": [{"name": "PathTracer", "params": {"samples_per_pixel": 8, "max_depth": 8, "rr_depth": 3}}],
           "scene": {"model": "scenes/box.pbrt"}}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    cli = os.path.join(ROOT, "srt_gb300", "srt")
    r = subprocess.run([cli, "-c", str(tmp_path / "cfg.json")], capture_output=True, text=True, cwd="/")
    assert r.returncode == 0, r.stderr
    data = (tmp_path / "out.pfm").read_bytes()
    head = b"PF\n30 20\n-1.0\n"
    assert data.startswith(head)
    img = np.frombuffer(data[len(head):], np.float32)
    assert img.size == 30 * 20 * 3 and np.all(np.isfinite(img)) and img.max() > 0.1
