"""Scene files into host arrays (srt_import_scene), no GPU needed.

pbrt: the PBRTParser subset (src/importer/pbrtparse.cu) — camera frame,
film size, materials, area lights written into the attribute block's
material, instances, trianglemesh and plymesh (ascii and binary).  The
camera is pinned against the reference's own parse_options + camera code
(tests/golden/pbrt_camera.npz, written by tests/golden/make_golden.py).
OBJ + MTL: the reference's Assimp path (src/importer/assimp.cu:17-131) —
one mesh per object and material run, one material copy per mesh,
ai_convert's parameter mapping over the OBJ reader's defaults.
"""
import os
import struct

import numpy as np
import pytest

import srt_gb300 as S
from helpers import golden
from oracle import oracle as O

FILMS = {"front": (400, 300), "above": (320, 180), "tilted": (100, 100), "mirrored": (300, 200)}
TRI = 'Shape "trianglemesh" "integer indices" [ 0 1 2 ] "point3 P" [ 0 0 0 1 0 0 0 1 0 ]\n'


def _nums(a):
    return " ".join(repr(float(x)) for x in np.asarray(a).reshape(-1))


@pytest.mark.parametrize("name", sorted(FILMS))
def test_pbrt_camera_matches_reference(tmp_path, name):
    z = golden("pbrt_camera")
    w, h = FILMS[name]
    fov = float(z[f"{name}_fov_aspect"][0])
    assert abs(w / h - float(z[f"{name}_fov_aspect"][1])) < 1e-6
    f = tmp_path / "cam.pbrt"
    f.write_text(f'Integrator "path" "integer maxdepth" [ 5 ]\n'
                 f'Transform [ {_nums(z[name + "_m16"])} ]\n'
                 f'Sampler "halton" "integer pixelsamples" [ 16 ]\n'
                 f'PixelFilter "gaussian"\n'
                 f'Film "rgb" "integer xresolution" [ {w} ] "integer yresolution" [ {h} ] "string filename" "x.exr"\n'
                 f'Camera "perspective" "float fov" [ {fov!r} ]\n'
                 f'WorldBegin\nMaterial "diffuse"\n{TRI}')
    s = S.import_scene(str(f))
    assert s.resolution == (w, h)
    rays = O.camera_rays(s.camera, z["xy"])
    np.testing.assert_allclose(rays, z[f"{name}_rays"], rtol=0, atol=1e-6)


def _write_ply_binary(path, v, n, faces, face_count_type="B", extra_uv=True):
    props = ["x", "y", "z"] + (["nx", "ny", "nz"] if n is not None else []) + (["u", "v"] if extra_uv else [])
    hdr = "ply\nformat binary_little_endian 1.0\ncomment written by a test\n"
    hdr += f"element vertex {len(v)}\n" + "".join(f"property float {p}\n" for p in props)
    ctype = {"B": "uchar", "i": "int"}[face_count_type]
    hdr += f"element face {len(faces)}\nproperty list {ctype} int vertex_indices\nend_header\n"
    body = b""
    for i in range(len(v)):
        vals = list(v[i]) + (list(n[i]) if n is not None else []) + ([0.25, 0.75] if extra_uv else [])
        body += struct.pack(f"<{len(vals)}f", *vals)
    for fc in faces:
        body += struct.pack(f"<{face_count_type}{len(fc)}i", len(fc), *fc)
    path.write_bytes(hdr.encode() + body)


FLOOR_V = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
FLOOR_F = [(0, 2, 1), (0, 3, 2)]


def test_pbrt_scene_contents(tmp_path):
    _write_ply_binary(tmp_path / "floor.ply", FLOOR_V, np.tile([0, 1, 0], (4, 1)), FLOOR_F)
    (tmp_path / "meshes").mkdir()
    (tmp_path / "meshes" / "lamp.ply").write_text(
        "ply\nformat ascii 1.0\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
        "element face 2\nproperty list uchar int vertex_indices\nend_header\n"
        + "".join(" ".join(str(c) for c in p) + "\n" for p in FLOOR_V)
        + "".join("3 " + " ".join(map(str, fc)) + "\n" for fc in FLOOR_F))
    xf = np.array([[2, 0, 0, 0.5], [0, 2, 0, 1], [0, 0, 2, -1], [0, 0, 0, 1]], np.float64)
    (tmp_path / "s.pbrt").write_text(f"""# a pbrt-v4 style scene
Film "rgb" "integer xresolution" [ 64 ] "integer yresolution" [ 48 ]
Camera "perspective" "float fov" [ 35 ]
WorldBegin
MakeNamedMaterial "Floor" "string type" [ "diffuse" ] "rgb reflectance" [ 0.5 0.6 0.7 ]
MakeNamedMaterial "Metal" "string type" [ "conductor" ] "float uroughness" [ 0.2 ] "float vroughness" [ 0.4 ]
MakeNamedMaterial "Glass" "string type" [ "dielectric" ] "float eta" [ 1.33 ]
MakeNamedMaterial "Skin" "string type" [ "diffusetransmission" ]
MakeNamedMaterial "Light" "string type" [ "diffuse" ] "rgb reflectance" [ 0 0 0 ]
MakeNamedMedium "fog" "string type" [ "homogeneous" ]
NamedMaterial "Floor"
Shape "plymesh" "string filename" [ "floor.ply" ]
Transform [ {_nums(xf.T)} ]
NamedMaterial "Metal"
Shape "trianglemesh" "integer indices" [ 0 1 2 ] "point3 P" [ 0 0 0 1 0 0 0 1 0 ]
    "normal N" [ 0 0 1 0 0 1 0 0 1 ]
AttributeBegin
  Transform [ 1 0 0 0 0 1 0 0 0 0 1 0 0 3 0 1 ]
  NamedMaterial "Light"
  AreaLightSource "diffuse" "rgb L" [ 3 4 12 ]
  Shape "plymesh" "string filename" "meshes/lamp.ply"
AttributeEnd
AttributeBegin
  MediumInterface "" "fog"
AttributeEnd
NamedMaterial "Glass"
{TRI}NamedMaterial "Skin"
{TRI}Material "coateddiffuse" "rgb reflectance" [ 0.1 0.2 0.3 ] "float roughness" [ 0 ]
{TRI}""")
    s = S.import_scene(str(tmp_path / "s.pbrt"))
    assert s.resolution == (64, 48)
    assert abs(s.camera.aspect - 64 / 48) < 1e-6 and s.camera.fov == 35.0
    # no Transform before WorldBegin: the identity frame, which is right-handed
    assert s.camera.type == S.CAMERA_PERSPECTIVE
    assert list(s.camera.position) == [0, 0, 0] and list(s.camera.target) == [0, 0, 1]
    # materials: five named, one anonymous
    m = s.materials
    assert len(m) == 6
    assert m[0].bxdf.type == S.BXDF_DIFFUSE and np.allclose(list(m[0].base_color), [0.5, 0.6, 0.7])
    assert m[1].bxdf.type == S.BXDF_DISNEY and m[1].bxdf.metallic == 1.0
    assert np.isclose(m[1].bxdf.roughness, 0.3) and list(m[1].base_color) == [1, 1, 1]
    assert m[2].bxdf.type == S.BXDF_DIELECTRIC and np.isclose(m[2].bxdf.ior, 1.33)
    assert m[3].bxdf.type == S.BXDF_DIFFUSE_TRANSMISSION and list(m[3].base_color) == [1, 1, 1]
    assert m[4].intensity == pytest.approx(13.0)
    assert np.allclose(list(m[4].emission_color), [3 / 13, 4 / 13, 12 / 13])
    assert m[5].bxdf.clearcoat == pytest.approx(0.8) and m[5].bxdf.clearcoatGloss == 1.0
    assert m[5].bxdf.roughness == pytest.approx(0.001)
    for k in range(4):
        assert m[k].intensity == 0.0
    # meshes and instances, in the order the file gives them
    assert [mm["material"] for mm in s.meshes] == [0, 1, 4, 2, 3, 5]
    assert len(s.instances) == 6 and [i for i, _ in s.instances] == [0, 1, 2, 3, 4, 5]
    np.testing.assert_array_equal(s.meshes[0]["vertices"], FLOOR_V)
    np.testing.assert_array_equal(s.meshes[0]["indices"], FLOOR_F)
    np.testing.assert_array_equal(s.meshes[0]["normals"], np.tile([0, 1, 0], (4, 1)))
    assert s.meshes[2]["normals"] is None
    np.testing.assert_array_equal(s.meshes[1]["normals"], np.tile([0, 0, 1], (3, 1)))
    np.testing.assert_allclose(s.instances[0][1].reshape(3, 4), np.eye(4)[:3])
    # world Transform: Transpose of the 16 numbers read row by row
    np.testing.assert_allclose(s.instances[1][1].reshape(3, 4), xf[:3])
    np.testing.assert_allclose(s.instances[2][1].reshape(3, 4)[:, 3], [0, 3, 0])
    # after AttributeEnd the world transform is the one set before the block
    np.testing.assert_allclose(s.instances[3][1].reshape(3, 4), xf[:3])


def test_obj_mtl_mapping(tmp_path):
    (tmp_path / "m.mtl").write_text("""newmtl red
Kd 0.8 0.1 0.1
Ni 1.45
Pr 0.3
Pm 0.2
Ps 0.4
Pc 0.5
Pcr 0.25
aniso 0.6
newmtl lamp
Kd 0 0 0
Ks 0.2 0.3 0.4
Ke 3 4 0
newmtl plain
""")
    (tmp_path / "m.obj").write_text("""# quad, triangle and pentagon
mtllib m.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 1.5 0
vn 0 0 1
vt 0 0
o quad
usemtl red
f 1/1/1 2/1/1 3/1/1 4/1/1
usemtl lamp
f 1 2 3
usemtl red
f -4 -3 -2
o pentagon
usemtl plain
f 1 2 3 5 4
usemtl missing
f 1 2 3
""")
    s = S.import_scene(str(tmp_path / "m.obj"))
    assert s.resolution == (0, 0)
    # object "quad": red, lamp, red again (a new mesh each time); object
    # "pentagon": plain, then a name the library lacks
    assert len(s.meshes) == 5 and len(s.materials) == 5
    assert [mm["material"] for mm in s.meshes] == [0, 1, 2, 3, 4]
    red, lamp, red2, plain, missing = s.materials
    assert np.allclose(list(red.base_color), [0.8, 0.1, 0.1])
    assert (red.bxdf.type, red.intensity) == (S.BXDF_DISNEY, 0.0)
    b = red.bxdf
    assert np.allclose([b.ior, b.roughness, b.metallic, b.sheen, b.clearcoat, b.clearcoatGloss, b.anisotropic],
                       [1.45, 0.3, 0.2, 0.4, 0.5, 0.25, 0.6])
    assert np.allclose([b.subsurface, b.specular, b.specularTint, b.sheenTint, b.specTrans], [0, 0.5, 0, 0, 0])
    assert bytes(red2) == bytes(red)
    # black Kd falls back to Ks; Ke becomes intensity |Ke| and a unit colour
    assert np.allclose(list(lamp.base_color), [0.2, 0.3, 0.4])
    assert lamp.intensity == pytest.approx(5.0) and np.allclose(list(lamp.emission_color), [0.6, 0.8, 0.0])
    # the OBJ reader's defaults: Kd 0.6, ior 1.0; ai_convert's: roughness 0.5
    for mm in (plain, missing):
        assert np.allclose(list(mm.base_color), [0.6] * 3)
        assert mm.bxdf.ior == 1.0 and mm.bxdf.roughness == 0.5 and mm.bxdf.clearcoatGloss == pytest.approx(0.001)
    q = s.meshes[0]
    np.testing.assert_array_equal(q["indices"], [[0, 1, 2], [0, 2, 3]])
    np.testing.assert_array_equal(q["normals"], np.tile([0, 0, 1], (4, 1)))
    assert s.meshes[1]["normals"] is None
    np.testing.assert_array_equal(s.meshes[2]["vertices"], [[1, 0, 0], [1, 1, 0], [0, 1, 0]])
    pent = s.meshes[3]
    np.testing.assert_array_equal(pent["indices"], [[0, 1, 2], [0, 2, 3], [0, 3, 4]])
    np.testing.assert_array_equal(pent["vertices"][3], [0.5, 1.5, 0])
    assert all(np.allclose(x.reshape(3, 4), np.eye(4)[:3]) for _, x in s.instances)


def test_lone_ply(tmp_path):
    _write_ply_binary(tmp_path / "f.ply", FLOOR_V, None, FLOOR_F, face_count_type="i", extra_uv=False)
    s = S.import_scene(str(tmp_path / "f.ply"))
    assert len(s.meshes) == 1 and s.meshes[0]["normals"] is None
    np.testing.assert_array_equal(s.meshes[0]["indices"], FLOOR_F)
    assert np.allclose(list(s.materials[0].base_color), [0.6] * 3)


PBRT_HEAD = 'Film "rgb" "integer xresolution" [ 8 ] "integer yresolution" [ 8 ]\nCamera "perspective" "float fov" [ 40 ]\n'


@pytest.mark.parametrize("name,text,status", [
    ("tex.pbrt", PBRT_HEAD + 'WorldBegin\nTexture "checks" "spectrum" "imagemap" "string filename" "a.png"\n', 1),
    ("texclass.pbrt", PBRT_HEAD + 'WorldBegin\nTexture "c" "spectrum" "checkerboard" "float uscale" 4\n', 9),
    ("uvsize.pbrt", PBRT_HEAD + 'WorldBegin\nMaterial "diffuse"\n'
     'Shape "trianglemesh" "integer indices" [ 0 1 2 ] "point3 P" [ 0 0 0 1 0 0 0 1 0 ] "point2 uv" [ 0 0 1 ]\n', 8),
    ("token.pbrt", PBRT_HEAD + 'LookAt 0 0 0 0 0 1 0 1 0\nWorldBegin\n', 9),
    ("world.pbrt", PBRT_HEAD + 'WorldBegin\nMaterial "diffuse"\nShape "sphere" "float radius" 1\n', 9),
    ("mat.pbrt", PBRT_HEAD + 'WorldBegin\nMaterial "measured"\n', 9),
    ("nomat.pbrt", PBRT_HEAD + 'WorldBegin\n' + TRI, 8),
    ("noworld.pbrt", PBRT_HEAD, 8),
    ("index.pbrt", PBRT_HEAD + 'WorldBegin\nMaterial "diffuse"\n'
     'Shape "trianglemesh" "integer indices" [ 0 1 3 ] "point3 P" [ 0 0 0 1 0 0 0 1 0 ]\n', 8),
    ("noply.pbrt", PBRT_HEAD + 'WorldBegin\nMaterial "diffuse"\nShape "plymesh" "string filename" "none.ply"\n', 1),
    ("quads.ply", None, 9),
    ("badface.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n", 8),
    ("scene.gltf", "{}", 9),
])
def test_import_errors(tmp_path, name, text, status):
    f = tmp_path / name
    if name == "quads.ply":
        _write_ply_binary(f, FLOOR_V, None, [(0, 1, 2, 3)], extra_uv=False)
    else:
        f.write_text(text)
    with pytest.raises(S.SrtError) as e:
        S.import_scene(str(f))
    assert e.value.status == status, str(e.value)
    with pytest.raises(S.SrtError) as e:
        S.import_scene(str(tmp_path / "absent.pbrt"))
    assert e.value.status == 1


def test_renderer_needs_a_camera_for_obj(tmp_path):
    """Renderer::load_scene (renderer.cu:125-147): obj scenes carry no
    camera, so the config must give one (checked before any GPU work)."""
    (tmp_path / "t.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    (tmp_path / "c.json").write_text('{"render": {"resolution": [8, 8]}, "passes": [], "scene": {"model": "t.obj"}}')
    with pytest.raises(S.SrtError, match="No camera specified"):
        S.Renderer(path=str(tmp_path / "c.json"))
    with pytest.raises(S.SrtError) as e:  # relative to the working directory, not the config's
        S.Renderer({"render": {"resolution": [8, 8]}, "passes": [], "scene": {"model": "t.obj"}})
    assert e.value.status == 1


def _png(path, px):
    """An RGBA8 PNG through the library's writer (values are 8-bit already)."""
    h, w = px.shape[:2]
    S.image_write(path, (px.astype(np.float32) / 255.0).reshape(-1, 4), w, h, flip=False)


def test_pbrt_textures_uv_and_tangents(tmp_path):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, size=(3, 4, 4), dtype=np.uint8)
    (tmp_path / "tex").mkdir()
    _png(tmp_path / "tex" / "wood.png", img)
    hdr = np.abs(rng.random((2, 5, 4), dtype=np.float32))
    S.image_write(tmp_path / "tex" / "sky.pfm", hdr.reshape(-1, 4), 5, 2, flip=False)
    _write_ply_binary(tmp_path / "uv.ply", FLOOR_V, None, FLOOR_F, extra_uv=True)
    (tmp_path / "t.pbrt").write_text(PBRT_HEAD + """WorldBegin
Texture "wood" "spectrum" "imagemap" "string filename" [ "tex/wood.png" ]
Texture "sky" "spectrum" "imagemap" "string filename" "tex/sky.pfm"
Material "diffuse" "texture reflectance" "wood"
Shape "trianglemesh" "integer indices" [ 0 1 2 ] "point3 P" [ 0 0 0 1 0 0 0 1 0 ]
    "point2 uv" [ 0 0 1 0 0 1 ] "float3 tangent" [ 1 0 0 1 0 0 1 0 0 ]
MakeNamedMaterial "m" "string type" "conductor" "texture reflectance" "sky"
NamedMaterial "m"
Shape "plymesh" "string filename" "uv.ply"
Material "diffuse" "texture reflectance" "nosuch"
""" + TRI)
    s = S.import_scene(str(tmp_path / "t.pbrt"))
    assert len(s.textures) == 2
    # Image::load_from_file(path, false, true): rows flipped, columns kept
    assert s.textures[0].dtype == np.uint8 and np.array_equal(s.textures[0], img[::-1])
    assert s.textures[1].dtype == np.float32 and np.array_equal(s.textures[1][..., :3], hdr[..., :3])
    assert s.material_textures == [(0, -1), (1, -1), (-1, -1)]
    np.testing.assert_array_equal(s.meshes[0]["texcoords"], [[0, 0], [1, 0], [0, 1]])
    np.testing.assert_array_equal(s.meshes[0]["tangents"], np.tile([1, 0, 0], (3, 1)))
    np.testing.assert_array_equal(s.meshes[1]["texcoords"], np.tile([0.25, 0.75], (4, 1)))
    assert s.meshes[2]["texcoords"] is None and s.env_map is None


def test_obj_textures_and_flipped_uvs(tmp_path):
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, size=(2, 3, 4), dtype=np.uint8)
    nrm = rng.integers(0, 256, size=(4, 2, 4), dtype=np.uint8)
    (tmp_path / "maps").mkdir()
    _png(tmp_path / "maps" / "albedo.png", img)
    _png(tmp_path / "maps" / "normal.png", nrm)
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 1 1 1\nmap_Kd -s 1 1 1 maps\\albedo.png\nnorm maps/normal.png\n"
                                    "newmtl b\nKd 0.5 0.5 0.5\nmap_Kd maps/albedo.png\nnewmtl c\nKd 0.2 0.2 0.2\n")
    (tmp_path / "m.obj").write_text("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n"
                                    "vt 0 0\nvt 1 0\nvt 1 1\nvt 0.25 0.75\n"
                                    "usemtl a\nf 1/1 2/2 3/3 4/4\nusemtl b\nf 1/4 2/4 3/4\nusemtl c\nf 1 2 3\n")
    s = S.import_scene(str(tmp_path / "m.obj"))
    # textures loaded once each, unflipped (load_from_file(filename))
    assert len(s.textures) == 2
    assert np.array_equal(s.textures[0], img) and np.array_equal(s.textures[1], nrm)
    assert s.material_textures == [(0, 1), (0, -1), (-1, -1)]
    # aiProcess_FlipUVs: v -> 1 - v
    np.testing.assert_allclose(s.meshes[0]["texcoords"], [[0, 1], [1, 1], [1, 0], [0.25, 0.25]])
    np.testing.assert_allclose(s.meshes[1]["texcoords"], np.tile([0.25, 0.25], (3, 1)))
    assert s.meshes[2]["texcoords"] is None


# the reference's own example model, where $SRT_REFERENCE_ROOT names a reference tree
REF_EXAMPLE = os.path.join(os.environ.get("SRT_REFERENCE_ROOT") or "/nonexistent",
                           "example", "cornell_box_obj", "cornell_box.obj")


@pytest.mark.skipif(not os.path.exists(REF_EXAMPLE), reason="the reference tree is not present")
def test_reference_example_cornell_obj():
    """The reference's own example model (example/cornell_box_obj): one mesh
    per group as Assimp makes them, the MTL mapped by ai_convert, the lamp's
    Ke (17, 12, 4) as intensity |Ke| with a unit colour."""
    s = S.import_scene(REF_EXAMPLE)
    assert len(s.meshes) == 8 and len(s.materials) == 8
    kd = [list(np.round(m.base_color[:], 3)) for m in s.materials]
    assert kd[:5] == [[0.725, 0.71, 0.68]] * 3 + [[0.14, 0.45, 0.091], [0.63, 0.065, 0.05]]
    lights = [m for m in s.materials if m.intensity > 0]
    assert len(lights) == 1
    le = np.array(lights[0].emission_color[:]) * lights[0].intensity
    np.testing.assert_allclose(le, [17, 12, 4], rtol=1e-6)
    assert np.allclose(list(lights[0].base_color), [0.78] * 3)
    assert [m.bxdf.ior for m in s.materials][:5] == [1.0, 1.0, 1.0, 1.5, 1.5]
    # 2 triangles per wall quad, 12 per box, 2 for the lamp
    assert [len(m["indices"]) for m in s.meshes] == [2, 2, 2, 2, 2, 12, 12, 2]
