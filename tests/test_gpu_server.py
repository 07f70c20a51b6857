"""Render serving (continuous batching) on the GPU.

Every pixel of every job has its own curand stream and its samples are
accumulated in order, so a job's film is bit-identical whether it runs
alone or packed with other jobs into the shared wavefront queues.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import golden, scene_from_npz
from srt_gb300 import pt_params

pytestmark = pytest.mark.gpu


def _alone(S, scene, w, h, params, cuda):
    import torch
    pt = S.PathTracer(scene, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device=cuda)
    pt.render(film, params)
    torch.cuda.synchronize()
    return film.cpu().numpy()


class Films:
    """Caller-owned device films handed to the server."""

    def __init__(self, cuda):
        self.cuda, self.films = cuda, {}

    def new(self, n):
        import torch
        f = torch.full((n, 4), -1.0, dtype=torch.float32, device=self.cuda)
        return f

    def host(self, f):
        import torch
        torch.cuda.synchronize()
        return f.cpu().numpy()


def _scenes(S):
    cornell = scene_from_npz(golden("scene"))
    spheres = S.procedural("spheres", seed=5, n_spheres=6, subdiv=3)
    return cornell, spheres


def test_mixed_jobs_equal_alone(cuda):
    import srt_gb300 as S
    cornell, spheres = _scenes(S)
    jobs = [  # (arrays, w, h, spp, depth, seed)
        (cornell, 40, 30, 8, 8, 11),
        (spheres, 64, 36, 4, 16, 12),
        (cornell, 17, 23, 16, 5, 13),
        (spheres, 32, 32, 1, 16, 14),
        (cornell, 96, 64, 2, 8, 15),
    ]
    scenes, films = {}, []
    F = Films(cuda)
    srv = S.Server(hbm_budget_bytes=8 << 30, max_paths=1 << 16, max_jobs=8, iterations_per_step=4)
    ids = []
    for k, (arr, w, h, spp, md, seed) in enumerate(jobs):
        arr.set_aspect(w / h)
        key = (id(arr), w, h)
        scenes[key] = S.Scene(arr)  # camera aspect of this job
        film = F.new(w * h) if k % 2 == 0 else None  # even jobs: caller film, odd: server-owned
        films.append(film)
        ids.append(srv.submit(scenes[key], w, h, pt_params(spp, md, 3, 1, 1, seed), film=film))
    srv.drain(300)
    infos = [srv.info(j) for j in ids]
    assert all(i["state"] == 2 for i in infos)
    # continuous batching: jobs overlapped on the device
    assert sum(1 for a in infos for b in infos if a is not b and a["admit_s"] < b["done_s"] and b["admit_s"] < a["done_s"]) > 0
    import torch
    for (arr, w, h, spp, md, seed), jid, info, film in zip(jobs, ids, infos, films):
        if film is None:  # server-owned film: copy it out (accumulate with weight 1 into zeros)
            ptr = srv.film_ptr(jid)
            assert ptr
            film = torch.zeros((w * h, 4), dtype=torch.float32, device=cuda)
            S.check(S.lib().srt_film_accumulate(C.c_void_p(ptr), C.c_void_p(film.data_ptr()), w * h, 0, None))
        got = F.host(film)
        ref = _alone(S, scenes[(id(arr), w, h)], w, h, pt_params(spp, md, 3, 1, 1, seed), cuda)
        np.testing.assert_array_equal(got, ref)
        ft = srv.frame_times(jid)
        assert len(ft) == spp and all(a <= b for a, b in zip(ft, ft[1:]))
        assert info["submit_s"] <= info["admit_s"] <= info["first_frame_s"] <= info["done_s"]
        srv.release(jid)


def test_admission_waits_for_budget_and_slots(cuda):
    import srt_gb300 as S
    cornell, _ = _scenes(S)
    cornell.set_aspect(1.0)
    scene = S.Scene(cornell)
    # room for one 64x64 job's paths at a time: the others queue and are admitted later
    srv = S.Server(hbm_budget_bytes=4 << 30, max_paths=64 * 64, max_jobs=4, iterations_per_step=2)
    F = Films(cuda)
    fl = [F.new(64 * 64) for _ in range(3)]
    ids = [srv.submit(scene, 64, 64, pt_params(4, 6, 3, 1, 1, 100 + k), film=fl[k]) for k in range(3)]
    r, q = srv.step()
    assert r == 1 and q == 2
    srv.drain(300)
    infos = [srv.info(j) for j in ids]
    assert all(i["state"] == 2 for i in infos)
    assert infos[1]["admit_s"] >= infos[0]["done_s"] and infos[2]["admit_s"] >= infos[1]["done_s"]
    for k, jid in enumerate(ids):
        got = F.host(fl[k])
        ref = _alone(S, scene, 64, 64, pt_params(4, 6, 3, 1, 1, 100 + k), cuda)
        np.testing.assert_array_equal(got, ref)
    with pytest.raises(S.SrtError) as e:
        srv.submit(scene, 128, 128, pt_params(1, 4, 3, 1, 1, 0))  # more paths than the engine holds
    assert e.value.status == 5


def test_jobs_arriving_while_others_run(cuda):
    import srt_gb300 as S
    cornell, spheres = _scenes(S)
    cornell.set_aspect(1.0)
    spheres.set_aspect(1.0)
    sc1, sc2 = S.Scene(cornell), S.Scene(spheres)
    srv = S.Server(hbm_budget_bytes=8 << 30, max_paths=1 << 16, max_jobs=16, iterations_per_step=2)
    F = Films(cuda)
    f1, f2 = F.new(48 * 48), F.new(48 * 48)
    first = srv.submit(sc1, 48, 48, pt_params(32, 8, 3, 1, 1, 7), film=f1)
    srv.step()
    late = srv.submit(sc2, 48, 48, pt_params(4, 16, 4, 1, 1, 8), film=f2)
    srv.drain(300)
    a, b = srv.info(first), srv.info(late)
    assert b["admit_s"] < a["done_s"]  # admitted while the first job was still on the GPU
    np.testing.assert_array_equal(F.host(f2), _alone(S, sc2, 48, 48, pt_params(4, 16, 4, 1, 1, 8), cuda))
    np.testing.assert_array_equal(F.host(f1), _alone(S, sc1, 48, 48, pt_params(32, 8, 3, 1, 1, 7), cuda))


def test_slot_of_a_finished_cached_job_is_emptied(cuda):
    """A cached job finishes and frees its state; jobs admitted after it
    reuse that memory and the freed slot.  The cache kernels visit every
    slot, so the finished job's record must no longer point at its state:
    the later plain job's film stays bit-identical to a lone render and the
    later cached job completes with finite pixels."""
    import srt_gb300 as S
    cornell, _ = _scenes(S)
    cornell.set_aspect(1.0)
    scene = S.Scene(cornell)
    mlp = C.c_void_p()
    S.check(S.lib().srt_mlp_create(3, C.byref(mlp)))
    S.check(S.lib().srt_mlp_set_box(mlp, (C.c_float * 3)(-1.05, -1.05, -1.05), (C.c_float * 3)(1.05, 1.05, 1.05)))
    srv = S.Server(hbm_budget_bytes=4 << 30, max_paths=1 << 14, max_jobs=2, iterations_per_step=2)
    F = Films(cuda)
    fa, fb, fc = F.new(64 * 64), F.new(64 * 64), F.new(64 * 64)
    a = srv.submit(scene, 64, 64, pt_params(2, 8, 3, 1, 1, 21), film=fa, cache=mlp)
    srv.drain(300)
    assert srv.info(a)["state"] == 2
    b = srv.submit(scene, 64, 64, pt_params(4, 8, 3, 1, 1, 22), film=fb)
    c = srv.submit(scene, 64, 64, pt_params(3, 8, 3, 1, 1, 23), film=fc, cache=mlp)
    srv.drain(300)
    assert srv.info(b)["state"] == 2 and srv.info(c)["state"] == 2
    np.testing.assert_array_equal(F.host(fb), _alone(S, scene, 64, 64, pt_params(4, 8, 3, 1, 1, 22), cuda))
    for f in (fa, fc):
        img = F.host(f)
        assert np.all(np.isfinite(img)) and np.all(img[:, 3] == 1.0)
    del srv
    S.lib().srt_mlp_destroy(mlp)


def test_cached_jobs_equal_alone_and_in_the_mix(cuda):
    """Cached jobs (frozen network) give the same film alone and packed with
    plain and other cached jobs: each job's queries, fallback and film
    updates touch only its own pixels and state."""
    import srt_gb300 as S
    cornell, spheres = _scenes(S)
    cornell.set_aspect(1.0)
    spheres.set_aspect(1.0)
    sc1, sc2 = S.Scene(cornell), S.Scene(spheres)
    nets = []
    for seed, arr in ((4, cornell), (5, spheres)):
        verts = np.concatenate([m["vertices"] for m in arr.meshes])
        lo, hi = verts.min(0) - 0.05, verts.max(0) + 0.05
        h = C.c_void_p()
        S.check(S.lib().srt_mlp_create(seed, C.byref(h)))
        S.check(S.lib().srt_mlp_set_box(h, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi)))
        nets.append(h)
    jobs = [(sc1, 48, 4, 8, 31, nets[0]), (sc2, 40, 2, 16, 32, nets[1]), (sc1, 32, 3, 8, 33, None),
            (sc2, 24, 5, 16, 34, nets[1])]

    def run(subset):
        srv = S.Server(hbm_budget_bytes=4 << 30, max_paths=1 << 15, max_jobs=8, iterations_per_step=3)
        F = Films(cuda)
        films = []
        for sc, w, spp, md, seed, net in subset:
            f = F.new(w * w)
            films.append(f)
            srv.submit(sc, w, w, pt_params(spp, md, 3, 1, 1, seed), film=f, cache=net)
        srv.drain(300)
        out = [F.host(f) for f in films]
        srv.close()
        return out

    mixed = run(jobs)
    for k, job in enumerate(jobs):
        alone = run([job])[0]
        np.testing.assert_array_equal(mixed[k], alone)
        assert np.all(np.isfinite(alone)) and np.all(alone[:, 3] == 1.0)
    for h in nets:
        S.lib().srt_mlp_destroy(h)


def test_online_training_jobs_train_the_network(cuda):
    """A cached job that trains online: one pixel in 1 + npix / 16384 traces
    full paths for its first sample and, when the job's first progressive
    frame completes, the network takes Adam steps on the recorded vertices.
    The job completes with finite pixels, the network's parameters change,
    and a frozen cached job served after it leaves them as they are; a plain
    job in the same mix stays bit-identical to a lone render."""
    import srt_gb300 as S
    cornell, _ = _scenes(S)
    cornell.set_aspect(1.0)
    scene = S.Scene(cornell)
    mlp = C.c_void_p()
    S.check(S.lib().srt_mlp_create(9, C.byref(mlp)))
    S.check(S.lib().srt_mlp_set_box(mlp, (C.c_float * 3)(-1.05, -1.05, -1.05), (C.c_float * 3)(1.05, 1.05, 1.05)))
    n = S._capi.SRT_MLP_PARAMS if hasattr(S._capi, "SRT_MLP_PARAMS") else 23552
    before = np.zeros(n, np.float32)
    S.check(S.lib().srt_mlp_get_params(mlp, before.ctypes.data_as(S._capi.f32p)))
    srv = S.Server(hbm_budget_bytes=4 << 30, max_paths=1 << 16, max_jobs=4, iterations_per_step=4)
    F = Films(cuda)
    ft, fp = F.new(128 * 128), F.new(64 * 64)
    t = srv.submit(scene, 128, 128, pt_params(4, 8, 3, 1, 1, 41), film=ft, cache=mlp, cache_train=True)
    p = srv.submit(scene, 64, 64, pt_params(4, 8, 3, 1, 1, 42), film=fp)
    srv.drain(300)
    assert srv.info(t)["state"] == 2 and srv.info(p)["state"] == 2
    img = F.host(ft)
    assert np.all(np.isfinite(img)) and np.all(img[:, 3] == 1.0) and img[:, :3].mean() > 0.0
    np.testing.assert_array_equal(F.host(fp), _alone(S, scene, 64, 64, pt_params(4, 8, 3, 1, 1, 42), cuda))
    after = np.zeros(n, np.float32)
    S.check(S.lib().srt_mlp_get_params(mlp, after.ctypes.data_as(S._capi.f32p)))
    assert np.all(np.isfinite(after)) and not np.array_equal(before, after)
    # a frozen job does not change the network
    ff = F.new(64 * 64)
    f = srv.submit(scene, 64, 64, pt_params(2, 8, 3, 1, 1, 43), film=ff, cache=mlp)
    srv.drain(300)
    assert srv.info(f)["state"] == 2
    again = np.zeros(n, np.float32)
    S.check(S.lib().srt_mlp_get_params(mlp, again.ctypes.data_as(S._capi.f32p)))
    np.testing.assert_array_equal(after, again)
    srv.close()
    S.lib().srt_mlp_destroy(mlp)
