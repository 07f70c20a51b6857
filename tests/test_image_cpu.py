"""Film images on disk, no GPU needed: the OpenEXR writer against files the
reference's own image code wrote (tinyexr as Image::save_exr calls it,
src/scene/texture.cu:69-130), the readers against what the reference's
Image::load_from_file (texture.cu:170-217) read back from those files, and
the flips of save_to_file / load_from_file(path, true, true).  Fixtures:
tests/golden/image.npz and img_*.exr / img_stb.hdr, written by
tests/golden/make_golden.py.
"""
import ctypes as C
import os
import struct
import zlib

import numpy as np
import pytest

import srt_gb300 as S
from helpers import GOLDEN, golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_IMG = os.path.join(ROOT, "oracle", "_ref", "libsrtimg.so")


def _fixture(name):
    return os.path.join(GOLDEN, name)


def _same(a, b):
    """Bitwise-equal float arrays (NaN payloads included)."""
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def _exr_halves(data, n):
    """The n half values of channel B of a one-row, uncompressed EXR."""
    return np.frombuffer(data[-2 * 4 * n:], np.uint16)[:n]


def test_exr_writer_matches_the_reference_bytes(tmp_path):
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    S.image_write(tmp_path / "a.exr", z["src"], w, h, flip=False)
    assert (tmp_path / "a.exr").read_bytes() == open(_fixture("img_none.exr"), "rb").read()


def test_half_rounding_matches_the_reference(tmp_path):
    """Ties round away from zero, overflow goes to infinity, float
    denormals to zero, NaN to 0x7e00 with its sign."""
    z = golden("image")
    v = z["half_in"]
    probe = np.zeros((len(v), 4), np.float32)
    probe[:, 2] = v
    S.image_write(tmp_path / "p.exr", probe, len(v), 1, flip=False)
    got = _exr_halves((tmp_path / "p.exr").read_bytes(), len(v))
    bad = np.nonzero(got != z["half_out"])[0]
    assert len(bad) == 0, [(float(v[i]), hex(got[i]), hex(z["half_out"][i])) for i in bad[:8]]
    # spot checks of the rule itself
    assert z["half_out"][list(v).index(np.float32(65520.0))] == 0x7c00
    assert z["half_out"][list(v).index(np.float32(2.0**-25))] == 0x0001


@pytest.mark.parametrize("name", ["none", "rle", "zips", "zip"])
def test_exr_reader_matches_the_reference(name):
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    px, rw, rh = S.image_read(_fixture(f"img_{name}.exr"), flip=False)
    assert (rw, rh) == (w, h)
    assert _same(px, z[f"{name}_decoded"])
    # load_from_file(path, true, true): mirrored in x and y
    px, _, _ = S.image_read(_fixture(f"img_{name}.exr"), flip=True)
    assert _same(px.reshape(h, w, 4), z[f"{name}_decoded"].reshape(h, w, 4)[::-1, ::-1])


def test_hdr_reader_matches_stbi_loadf(tmp_path):
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    px, rw, rh = S.image_read(_fixture("img_stb.hdr"), flip=False)  # run-length scanlines (stb)
    assert (rw, rh) == (w, h) and _same(px, z["stb_hdr_decoded"])
    # our flat-scanline writer encodes each pixel as stb does
    S.image_write(tmp_path / "o.hdr", np.abs(z["src"]), w, h, flip=False)
    ours, _, _ = S.image_read(tmp_path / "o.hdr", flip=False)
    assert _same(ours, z["stb_hdr_decoded"])


@pytest.mark.parametrize("ext", ["exr", "pfm", "hdr"])
def test_write_then_read_with_flip_returns_the_film(tmp_path, ext):
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    film = np.abs(z["src"]) if ext == "hdr" else z["src"]
    S.image_write(tmp_path / f"f.{ext}", film, w, h, flip=True)
    back, _, _ = S.image_read(tmp_path / f"f.{ext}", flip=True)
    unflipped, _, _ = S.image_read(tmp_path / f"f.{ext}", flip=False)
    if ext == "exr":
        # half precision: within half an ulp (2^-11 relative, 2^-25 absolute near zero)
        assert np.all(np.abs(back - film) <= np.abs(film) * 2.0**-11 + 2.0**-25)
    elif ext == "pfm":
        assert _same(back[:, :3], film[:, :3]) and np.all(back[:, 3] == 1.0)
        # PFM rows are stored bottom to top, so the file is only mirrored in x
        assert _same(unflipped.reshape(h, w, 4)[:, ::-1, :3], film.reshape(h, w, 4)[..., :3])
    else:
        # RGBE shares one exponent: each channel is exact to 1/256 of the pixel's largest
        tol = film[:, :3].max(1, keepdims=True) / 128.0
        assert np.all(np.abs(back[:, :3] - film[:, :3]) <= tol)
    if ext != "pfm":
        assert _same(unflipped.reshape(h, w, 4)[::-1, ::-1], back.reshape(h, w, 4))


def _exr_zip_file(path, px, w, h, level, lines=16, compression=3):
    """A ZIP / ZIPS OpenEXR written here with Python's zlib at `level` (stored,
    fixed-Huffman and dynamic-Huffman deflate blocks), float channels."""
    def attr(name, typ, val):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(val)) + val
    chl = b"".join(n + b"\0" + struct.pack("<iiii", 2, 0, 1, 1) for n in (b"A", b"B", b"G", b"R")) + b"\0"
    head = b"\x76\x2f\x31\x01" + struct.pack("<I", 2)
    head += attr("channels", "chlist", chl) + attr("compression", "compression", bytes([compression]))
    head += attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    head += attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    head += attr("lineOrder", "lineOrder", b"\0") + b"\0"
    img = px.reshape(h, w, 4)
    chunks = []
    for y0 in range(0, h, lines):
        raw = b"".join(img[y, :, c].astype("<f4").tobytes() for y in range(y0, min(h, y0 + lines)) for c in (3, 2, 1, 0))
        t = np.frombuffer(raw, np.uint8)
        inter = np.empty_like(t)
        half = (len(t) + 1) // 2
        inter[:half], inter[half:] = t[0::2], t[1::2]
        pred = inter.astype(np.int16)
        pred[1:] = (inter[1:].astype(np.int16) - inter[:-1].astype(np.int16) + 128) & 0xff
        comp = zlib.compress(pred.astype(np.uint8).tobytes(), level)
        chunks.append(struct.pack("<ii", y0, len(comp)) + comp)
    table, off = b"", len(head) + 8 * len(chunks)
    for c in chunks:
        table += struct.pack("<Q", off)
        off += len(c)
    path.write_bytes(head + table + b"".join(chunks))


@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("compression,lines", [(3, 16), (2, 1)])
def test_exr_zip_deflate_block_types(tmp_path, level, compression, lines):
    rng = np.random.default_rng(level)
    w, h = 45, 40
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    px = np.stack([xx * 0.25, yy, rng.random((h, w), dtype=np.float32), np.ones_like(xx)], -1).reshape(-1, 4)
    _exr_zip_file(tmp_path / "z.exr", px.astype(np.float32), w, h, level, lines, compression)
    got, gw, gh = S.image_read(tmp_path / "z.exr", flip=False)
    assert (gw, gh) == (w, h) and _same(got, px)


def test_image_read_errors(tmp_path):
    with pytest.raises(S.SrtError) as e:
        S.image_read(_fixture("img_piz.exr"))
    assert e.value.status == 9 and "compression 4" in str(e.value)
    data = open(_fixture("img_zip.exr"), "rb").read()
    (tmp_path / "t.exr").write_bytes(data[:len(data) // 2])
    with pytest.raises(S.SrtError) as e:
        S.image_read(tmp_path / "t.exr")
    assert e.value.status == 8
    bad = bytearray(data)
    bad[-20] ^= 0x5a  # inside the last compressed chunk
    (tmp_path / "c.exr").write_bytes(bytes(bad))
    with pytest.raises(S.SrtError) as e:
        S.image_read(tmp_path / "c.exr")
    assert e.value.status == 8
    tiled = bytearray(open(_fixture("img_none.exr"), "rb").read())
    tiled[5] |= 0x02  # version flags: tiled
    (tmp_path / "tiled.exr").write_bytes(bytes(tiled))
    with pytest.raises(S.SrtError) as e:
        S.image_read(tmp_path / "tiled.exr")
    assert e.value.status == 9
    S.image_write(tmp_path / "a.png", np.zeros((4, 4), np.float32), 2, 2)
    with pytest.raises(S.SrtError) as e:
        S.image_read(tmp_path / "a.png")
    assert e.value.status == 9
    with pytest.raises(S.SrtError) as e:
        S.image_read(tmp_path / "missing.exr")
    assert e.value.status == 1


@pytest.mark.skipif(not os.path.exists(REF_IMG), reason="reference image library not built here")
def test_live_cross_check_with_the_reference_image_code(tmp_path):
    """Where the reference tree is present: random sizes and bit patterns
    through tinyexr and through ours, both ways."""
    R = C.CDLL(REF_IMG)
    rng = np.random.default_rng(77)
    for w, h in ((1, 1), (13, 7), (200, 3)):
        px = rng.integers(0, 2**32, size=w * h * 4, dtype=np.uint64).astype(np.uint32).view(np.float32).copy()
        S.image_write(tmp_path / "o.exr", px, w, h, flip=False)
        assert R.ref_save_exr(str(tmp_path / "r.exr").encode(), w, h, px.ctypes.data_as(C.c_void_p), 0) == 0
        assert (tmp_path / "o.exr").read_bytes() == (tmp_path / "r.exr").read_bytes()
        smooth = np.repeat(np.linspace(-2, 9, w * h, dtype=np.float32), 4)
        for comp in (0, 1, 2, 3):
            assert R.ref_save_exr(str(tmp_path / "c.exr").encode(), w, h, smooth.ctypes.data_as(C.c_void_p), comp) == 0
            ours, _, _ = S.image_read(tmp_path / "c.exr", flip=False)
            ww, hh = C.c_int(), C.c_int()
            ref = np.zeros((w * h, 4), np.float32)
            assert R.ref_load_float_image(str(tmp_path / "c.exr").encode(), C.byref(ww), C.byref(hh),
                                          ref.ctypes.data_as(C.c_void_p)) == 0
            assert _same(ours, ref)


PNG_NAMES = ["g1", "g2", "g4", "g8", "g16", "rgb8", "rgb16", "rgb8i", "p1", "p4", "p8", "ga8", "ga16", "rgba8",
             "rgba16", "rgba8i", "g8t", "rgb8t"]


@pytest.mark.parametrize("name", PNG_NAMES)
def test_png_decoder_matches_stbi_load(name):
    """Every colour type and bit depth, palettes, tRNS keys, Adam7 and all
    five filter types, against the reference's stbi_load(.., 4)."""
    z = np.load(os.path.join(GOLDEN, "png.npz"))
    px, w, h = S.image_read_rgba8(_fixture(f"png_{name}.png"), flip=False)
    assert (w, h) == (13, 11)
    assert np.array_equal(px, z[name])


def test_rgba8_reader_flips_and_own_writers(tmp_path):
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    film = z["src"]
    want = (np.clip(film, 0.0, 1.0) * np.float32(255.0)).astype(np.uint8)  # Image::f_to_u
    want[~(film > 0)] = 0
    for ext in ("png", "bmp"):
        S.image_write(tmp_path / f"o.{ext}", film, w, h, flip=False)
        px, rw, rh = S.image_read_rgba8(tmp_path / f"o.{ext}", flip=False)
        assert (rw, rh) == (w, h)
        assert np.array_equal(px[:, :3], want[:, :3])
        if ext == "png":
            assert np.array_equal(px[:, 3], want[:, 3])
        xy, _, _ = S.image_read_rgba8(tmp_path / f"o.{ext}", flip="xy")
        y, _, _ = S.image_read_rgba8(tmp_path / f"o.{ext}", flip="y")
        assert np.array_equal(xy.reshape(h, w, 4), px.reshape(h, w, 4)[::-1, ::-1])
        assert np.array_equal(y.reshape(h, w, 4), px.reshape(h, w, 4)[::-1])
    with pytest.raises(S.SrtError) as e:
        S.image_read_rgba8(_fixture("img_none.exr"))
    assert e.value.status == 9
    (tmp_path / "x.tga").write_bytes(bytes(64))
    with pytest.raises(S.SrtError) as e:
        S.image_read_rgba8(tmp_path / "x.tga")
    assert e.value.status == 9


@pytest.mark.skipif(not os.path.exists(REF_IMG), reason="reference image library not built here")
def test_png_bmp_written_by_stb_read_like_stbi(tmp_path):
    R = C.CDLL(REF_IMG)
    z = golden("image")
    w, h = (int(x) for x in z["size"])
    src = np.ascontiguousarray(z["src"])
    for kind, ext in ((1, "png"), (2, "bmp")):
        p = str(tmp_path / f"s.{ext}").encode()
        assert R.ref_save_stb(p, kind, w, h, src.ctypes.data_as(C.c_void_p)) == 0
        ref = np.zeros((w * h, 4), np.uint8)
        ww, hh = C.c_int(), C.c_int()
        assert R.ref_load_u8_image(p, C.byref(ww), C.byref(hh), ref.ctypes.data_as(C.c_void_p)) == 0
        ours, _, _ = S.image_read_rgba8(tmp_path / f"s.{ext}", flip=False)
        assert np.array_equal(ours, ref)


@pytest.mark.parametrize("name", ["q100", "q75", "grey90"])
def test_jpeg_decoder_close_to_stbi_load(name):
    """Baseline JPEGs written by the reference's stb_image_write: our exact
    IDCT and triangle chroma filter stay within 2 levels of stbi_load's
    integer IDCT and upsampler."""
    z = np.load(os.path.join(GOLDEN, "jpg.npz"))
    px, w, h = S.image_read_rgba8(_fixture(f"jpg_{name}.jpg"), flip=False)
    assert (w, h) == (37, 29)
    d = np.abs(px.astype(int) - z[name].astype(int))
    assert d.max() <= 2 and d.mean() < 0.5, (d.max(), d.mean())


def test_jpeg_writer_round_trip(tmp_path):
    """srt_image_write(.jpg) is save_ldr's stbi_write_jpg(.., 100): baseline,
    4:4:4, Annex K tables at quality 100; it reads back within 2 levels."""
    z = np.load(os.path.join(GOLDEN, "jpg.npz"))
    src = z["src"]
    h, w = src.shape[:2]
    S.image_write(tmp_path / "o.jpg", (src / 255.0).astype(np.float32).reshape(-1, 4), w, h, flip=False)
    data = (tmp_path / "o.jpg").read_bytes()
    assert data[:2] == b"\xff\xd8" and data[-2:] == b"\xff\xd9" and b"\xff\xc0" in data
    want = ((src / 255.0).astype(np.float32) * np.float32(255.0)).astype(np.uint8).reshape(-1, 4)
    px, _, _ = S.image_read_rgba8(tmp_path / "o.jpg", flip=False)
    assert np.abs(px[:, :3].astype(int) - want[:, :3]).max() <= 2
    # progressive and truncated files
    prog = bytearray(data)
    k = prog.index(b"\xff\xc0")
    prog[k + 1] = 0xC2
    (tmp_path / "p.jpg").write_bytes(bytes(prog))
    with pytest.raises(S.SrtError) as e:
        S.image_read_rgba8(tmp_path / "p.jpg")
    assert e.value.status == 9
    (tmp_path / "t.jpg").write_bytes(data[:40])
    with pytest.raises(S.SrtError) as e:
        S.image_read_rgba8(tmp_path / "t.jpg")
    assert e.value.status == 8


@pytest.mark.skipif(not os.path.exists(REF_IMG), reason="reference image library not built here")
def test_jpeg_writer_read_by_stbi(tmp_path):
    R = C.CDLL(REF_IMG)
    z = np.load(os.path.join(GOLDEN, "jpg.npz"))
    src = z["src"]
    h, w = src.shape[:2]
    S.image_write(tmp_path / "o.jpg", (src / 255.0).astype(np.float32).reshape(-1, 4), w, h, flip=False)
    ref = np.zeros((w * h, 4), np.uint8)
    ww, hh = C.c_int(), C.c_int()
    assert R.ref_load_u8_image(str(tmp_path / "o.jpg").encode(), C.byref(ww), C.byref(hh),
                               ref.ctypes.data_as(C.c_void_p)) == 0
    want = ((src / 255.0).astype(np.float32) * np.float32(255.0)).astype(np.uint8).reshape(-1, 4)
    assert np.abs(ref[:, :3].astype(int) - want[:, :3]).max() <= 2
