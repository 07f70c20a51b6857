"""The Measure pass (src/passes/postprocess/measure.{h,cu}) on the GPU with a
reference image on disk: an EXR the renderer itself saved (Image::save_to_file
flips x and y; Measure's load_from_file(path, true, true) flips them back),
the printed trimmed-mean error against the oracle's metric, and the pass's
"option" (Reference / Error) against the oracle's per-pixel errors.
"""
import re

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CAM = {"type": "perspective", "position": [0, 0, 3.5], "target": [0, 0, 0], "up": [0, 1, 0], "fov": 40}


def _cfg(passes, w=32, h=24):
    return {"render": {"type": "image", "resolution": [w, h]},
            "passes": [{"name": "PathTracer", "params": {"samples_per_pixel": 16, "max_depth": 8, "rr_depth": 3}}]
            + passes,
            "scene": {"model": "procedural:cornell", "camera": CAM}}


def test_measure_view_kernel_vs_oracle(cuda):
    import torch
    import srt_gb300 as S
    rng = np.random.default_rng(31)
    n = 70001
    film = (rng.random((n, 4), dtype=np.float32) * 2).astype(np.float32)
    ref = (rng.random((n, 4), dtype=np.float32) + 0.01).astype(np.float32)
    r = torch.from_numpy(ref).to(cuda)
    for t in range(4):
        _, err = O.metric(film, ref, t, 0.0)
        x = torch.from_numpy(film).to(cuda)
        S.film_measure_view(x, r, t, S._capi.MEASURE_ERROR)
        got = x.cpu().numpy()
        np.testing.assert_allclose(got[:, 0], err, rtol=2e-6, atol=1e-9)
        assert np.array_equal(got[:, 0], got[:, 1]) and np.array_equal(got[:, 0], got[:, 2]) and np.all(got[:, 3] == 1)
    x = torch.from_numpy(film).to(cuda)
    S.film_measure_view(x, r, 0, S._capi.MEASURE_REFERENCE)
    got = x.cpu().numpy()
    assert np.array_equal(got[:, :3], ref[:, :3]) and np.all(got[:, 3] == 1)
    x = torch.from_numpy(film).to(cuda)
    S.film_measure_view(x, r, 0, S._capi.MEASURE_NONE)
    assert np.array_equal(x.cpu().numpy(), film)
    with pytest.raises(S.SrtError):
        S.film_measure_view(x, r, 0, 3)


def test_measure_pass_against_a_saved_exr(cuda, tmp_path, capfd):
    import srt_gb300 as S
    w, h = 32, 24
    a = S.Renderer(_cfg([]))
    a.run(1)
    film_a = a.film()
    a.save(tmp_path / "ref.exr")
    a.close()
    ref, rw, rh = S.image_read(tmp_path / "ref.exr", flip=True)
    assert (rw, rh) == (w, h)
    # the saved picture is the film to half precision, in film order after the flip
    assert np.all(np.abs(ref[:, :3] - film_a[:, :3]) <= np.abs(film_a[:, :3]) * 2.0**-11 + 2.0**-25)
    capfd.readouterr()
    b = S.Renderer(_cfg([{"name": "Measure", "params": {"ref_path": str(tmp_path / "ref.exr"), "type": "RelMSE",
                                                         "discard": 0.1}}]))
    b.run(1)
    film_b = b.film()
    out = capfd.readouterr().out
    m = re.search(r"RelMSE error: (\S+)", out)
    assert m, out
    want, _ = O.metric(film_b, ref, S._capi.METRIC_RELMSE, 0.1)
    assert abs(float(m.group(1)) - want) <= 1e-5 * abs(want) + 1e-12, (m.group(1), want)
    # the frame seed comes from one generator per process (random_int), so this frame is a new sample
    assert not np.array_equal(film_b, film_a) and want > 0.0
    for option in ("Error", "Reference"):
        # a disabled PathTracer leaves the film as allocated (zero), which Measure then reads
        cfg = _cfg([{"name": "Measure", "params": {"ref_path": str(tmp_path / "ref.exr"), "type": "MAPE",
                                                    "option": option}}])
        cfg["passes"][0]["enable"] = False
        c = S.Renderer(cfg)
        c.run(1)
        got = c.film()
        if option == "Error":
            _, err = O.metric(np.zeros_like(ref), ref, S._capi.METRIC_MAPE, 0.1)
            np.testing.assert_allclose(got[:, 0], err, rtol=2e-6, atol=1e-12)
        else:
            assert np.array_equal(got[:, :3], ref[:, :3]) and np.all(got[:, 3] == 1)


def test_measure_rejects_wrong_references(cuda, tmp_path):
    import srt_gb300 as S
    S.image_write(tmp_path / "small.exr", np.ones((8 * 8, 4), np.float32), 8, 8)
    S.image_write(tmp_path / "ldr.png", np.ones((32 * 24, 4), np.float32), 32, 24)
    for name in ("small.exr", "ldr.png", "absent.exr"):
        with pytest.raises(S.SrtError, match="reference image size or format not match"):
            S.Renderer(_cfg([{"name": "Measure", "params": {"ref_path": str(tmp_path / name)}}]))
    with pytest.raises(S.SrtError, match="no ref_path"):
        S.Renderer(_cfg([{"name": "Measure", "params": {}}]))
