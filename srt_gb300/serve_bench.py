"""Render-serving load test: Poisson job arrivals against one GB300.

Each job draws its resolution from {256^2, 512^2, 1024^2, 1920x1080}, its
spp from {1, 4, 16, 64}, its scene from {Cornell box, 5.2M-triangle spheres
scene} (several seeds of each, built once and kept resident) and plain or
radiance-cache rendering 50/50 (the cache network of each scene is trained
beforehand with srt_pt_render_cached; half of the cached jobs keep training
it online on their own paths, the other half use it frozen).  Jobs are
admitted under the HBM budget as slots and queue capacity free up, and
their rays share the wavefront queues.

    python -m srt_gb300.serve_bench --rates 5,10,20,50,100,200 --duration 30

prints one JSON line per rate: p50/p99 job latency (submit -> done),
p50/p99 latency of the first progressive frame (submit -> frame 1), p50/p99
of each job's mean interval between progressive frames, completed jobs and
Msamples/s.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
SPPS = [1, 4, 16, 64]


def build_scenes(S, n_variants=2, spheres=64, subdiv=6, cache_frames=60):
    """Resident scenes and one trained (then frozen) cache network per scene."""
    import torch
    out = []
    for v in range(n_variants):
        for name in ("cornell", "spheres"):
            arr = S.procedural(name, seed=1 + v, n_spheres=spheres, subdiv=subdiv)
            arr.set_aspect(1.0)
            scene = S.Scene(arr)
            verts = np.concatenate([m["vertices"] for m in arr.meshes])
            lo, hi = verts.min(0) - 0.05, verts.max(0) + 0.05
            mlp = C.c_void_p()
            S.check(S.lib().srt_mlp_create(100 + v, C.byref(mlp)))
            S.check(S.lib().srt_mlp_set_box(mlp, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi)))
            pt = S.PathTracer(scene, 256, 256)
            film = torch.zeros((256 * 256, 4), dtype=torch.float32, device="cuda")
            cp = S._capi.CacheParams(8192, 4, 1e-2, 0.5, 16, 1)
            st = S._capi.CacheStats()
            for f in range(cache_frames):
                p = S.pt_params(1, 8 if name == "cornell" else 16, 3 if name == "cornell" else 4, 1, 1, 7000 + f)
                S.check(S.lib().srt_pt_render_cached(pt.handle, C.c_void_p(film.data_ptr()), C.byref(p), mlp,
                                                     C.byref(cp), C.byref(st), None))
            out.append({"name": name, "scene": scene, "mlp": mlp, "depth": 8 if name == "cornell" else 16,
                        "rr": 3 if name == "cornell" else 4})
    return out


def run_rate(S, scenes, rate, duration, seed=0, budget_gb=150, max_paths=1 << 24, drain_s=120.0):
    rng = np.random.default_rng(seed)
    srv = S.Server(hbm_budget_bytes=int(budget_gb) << 30, max_paths=max_paths, max_jobs=512,
                   iterations_per_step=8)
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        w, h = RESOLUTIONS[rng.integers(len(RESOLUTIONS))]
        spp = SPPS[rng.integers(len(SPPS))]
        sc = scenes[rng.integers(len(scenes))]
        cached = bool(rng.integers(2))
        online = cached and bool(rng.integers(2))
        arrivals.append((t, w, h, spp, sc, cached, online))
    jobs = []
    t0 = srv.now()
    i = 0
    while True:
        now = srv.now() - t0
        while i < len(arrivals) and arrivals[i][0] <= now:
            _, w, h, spp, sc, cached, online = arrivals[i]
            p = S.pt_params(spp, sc["depth"], sc["rr"], 1, 1, 1000 + i)
            jid = srv.submit(sc["scene"], w, h, p, cache=sc["mlp"] if cached else None, cache_train=online)
            jobs.append((jid, w * h * spp, cached, online))
            i += 1
        running, queued = srv.step()
        if i >= len(arrivals) and running == 0 and queued == 0:
            break
        if now > duration + drain_s:
            break
        if running == 0 and queued == 0 and i < len(arrivals):
            time.sleep(max(0.0, min(0.002, arrivals[i][0] - now)))
    wall = srv.now() - t0
    lat, first, interval, samples, done, cached_done, online_done = [], [], [], 0, 0, 0, 0
    for jid, ns, cached, online in jobs:
        info = srv.info(jid)
        if info["state"] == 2:
            done += 1
            cached_done += int(cached)
            online_done += int(online)
            samples += ns
            lat.append(info["done_s"] - info["submit_s"])
            # progressive frames: latency of the first one, and the job's mean
            # interval between frames (the host observes frames once per step)
            ft = srv.frame_times(jid)
            first.append(ft[0] - info["submit_s"])
            if len(ft) > 1:
                interval.append((ft[-1] - ft[0]) / (len(ft) - 1))
            srv.release(jid)
    srv.close()
    pct = lambda a, q: float(np.quantile(a, q)) if len(a) else None
    return {"rate_jobs_per_s": rate, "duration_s": duration, "submitted": len(jobs), "completed": done,
            "cached_completed": cached_done, "cached_online_training_completed": online_done,
            "wall_s": round(wall, 3),
            "p50_job_s": pct(lat, 0.5), "p99_job_s": pct(lat, 0.99),
            "p50_first_frame_s": pct(first, 0.5), "p99_first_frame_s": pct(first, 0.99),
            "p50_frame_interval_s": pct(interval, 0.5), "p99_frame_interval_s": pct(interval, 0.99),
            "msamples_per_s": round(samples / wall / 1e6, 2) if wall > 0 else None}


def main():
    import srt_gb300 as S
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="5,10,20,50,100,200")
    ap.add_argument("--duration", type=float, default=30.0)
    ap.add_argument("--variants", type=int, default=2)
    args = ap.parse_args()
    scenes = build_scenes(S, n_variants=args.variants)
    for r in [float(x) for x in args.rates.split(",")]:
        print(json.dumps(run_rate(S, scenes, r, args.duration)), flush=True)


if __name__ == "__main__":
    main()
