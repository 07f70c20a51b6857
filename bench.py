"""Headline benchmark: plain wavefront path tracing of the 5.2M-triangle
scene (64 displaced icospheres of 81,920 triangles, ground quad, four quad
lights, constant environment 0.05) at 1920x1080, 64 spp, max depth 16,
Russian roulette from depth 4, NEE + MIS, per-pixel curand streams.

One step = one PathTracer frame (w*h*spp samples).  `value` is Msamples/s
with the scene resident in HBM; `e2e` is the same metric through the C ABI
with the frame parameters handed over from host memory and the film read
back to pinned host memory every step.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Multi-GPU runs (torchrun) render independent replicas: each rank renders
the full frame, value = all ranks' samples / max rank time (weak scaling).
`--impl reference` times the reference's path-tracing algorithm on the
host cores (the oracle's CPU restatement) on a bounded crop.

Extra keys: `roofline` for the kernel with the most device time in a
timed profile frame (CUDA events around the production kernels; the work
per ray from a second frame of the same seed with the counting traversal
kernels), `traffic` scaled from the DRAM bytes per ray of one ncu capture
(profiles/<kernel>_dram.json); `cache` (learned-cache time to the plain
tracer's 64-spp relMSE, 1280x720), `serving` (a 10 s Poisson run at 20
jobs/s), `bxdf` (the Disney BSDF batch of 2^20 points), `cornell` (the
Cornell box at 512x512, 16 spp, depth 8), `cpu_baseline`.  `--no-cache`, `--no-serving`,
`--no-cpu-baseline` skip those parts; `--profile-case` runs the short
case the ncu captures use.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s and p50/p99 job latency at equal relMSE vs plain tracer, 1 GB300"
W, H, SPP, MAX_DEPTH, RR_DEPTH, SEED = 1920, 1080, 64, 16, 4, 1
N_SPHERES, SUBDIV = 64, 6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 8:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        finally:
            try:
                os.remove(self.path)
            except OSError:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_max(x, world, device):
    """Largest value over the ranks (the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_scene(S):
    arrays = S.procedural("spheres", seed=SEED, n_spheres=N_SPHERES, subdiv=SUBDIV)
    arrays.set_aspect(W / H)
    return arrays


def cpu_baseline(arrays, steps=1, budget_s=20.0):
    """The oracle's megakernel restatement on the host cores, on a crop of
    the same frame (bounded to about `budget_s` seconds of CPU work)."""
    from oracle import oracle as O
    import srt_gb300 as S
    threads = os.cpu_count() or 1
    osc = O.OracleScene(arrays.desc())
    t0 = time.perf_counter()
    osc.build_bvh()
    build_s = time.perf_counter() - t0
    # calibrate on a small crop, then size the crop to the budget
    cw = ch = 32
    spp = 1
    p = S.pt_params(spp, MAX_DEPTH, RR_DEPTH, 1, 1, SEED)
    x0, y0 = (W - cw) // 2, (H - ch) // 2
    t0 = time.perf_counter()
    osc.render(W, H, p, crop=(x0, y0, cw, ch), threads=threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    rate = cw * ch * spp / dt
    target = rate * budget_s / max(1, steps)
    side = int(max(32, min(512, (target / 4) ** 0.5)))
    spp = 4
    x0, y0 = (W - side) // 2, (H - side) // 2
    p = S.pt_params(spp, MAX_DEPTH, RR_DEPTH, 1, 1, SEED)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        osc.render(W, H, p, crop=(x0, y0, side, side), threads=threads)
        times.append(time.perf_counter() - t0)
    value = side * side * spp * len(times) / sum(times) / 1e6
    return {"value": round(value, 4), "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"centre crop {side}x{side} of the {W}x{H} frame, {spp} spp, depth {MAX_DEPTH}, "
                      f"oracle CPU BVH (build {build_s:.1f}s, not timed), {threads} threads"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import srt_gb300 as S
    arrays = build_scene(S)
    steps = max(1, args.steps)
    cb = cpu_baseline(arrays, steps=steps, budget_s=min(60.0, 12.0 * steps))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(None), "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(info):
    d = {"workload": "5.2M-triangle synthetic scene (64 icospheres subdiv 6, value-noise displaced), "
                     "plain wavefront PT FP32", "width": W, "height": H, "spp": SPP, "max_depth": MAX_DEPTH,
         "rr_depth": RR_DEPTH, "nee": True, "mis": True, "rng": "curand XORWOW per pixel",
         "l2": "scene larger than L2 (no flush between steps)"}
    if info:
        d["triangles"] = info["num_triangles"]
        d["scene_mb"] = round(info["device_bytes"] / 2 ** 20, 1)
        d["bvh_nodes"] = info["num_nodes"]
        d["bvh_build_s"] = round(info["build_ms"] / 1000, 2)
    return d


def measured_traffic(kernel, rays_per_launch):
    """DRAM bytes per launch of `kernel` scaled from one ncu capture: the
    per-ray dram__bytes_read.sum + dram__bytes_write.sum of a captured launch
    (profiles/<kernel>_dram.json, written from the capture) times the rays of
    an average benchmark launch."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", f"{kernel}_dram.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        d = json.load(f)
    return int(d["dram_bytes_per_ray"] * rays_per_launch), d["capture"]


def bxdf_eval_bench(S, n=1 << 20, launches=20, cpu=True):
    """Disney BSDF batch (sample + f + pdf, GMaterial::sample) on n = 2^20
    shading points generated in device memory from the PCG32 streams of
    the config-0 definition; kernel time from CUDA events per launch with
    L2 flushed between launches.  Algorithmic bytes per point = inputs
    (normal, wo, colour: 36 B; 12 parameters: 48 B; 2 uniforms: 8 B) +
    outputs (wi, f: 24 B; pdf, delta: 8 B) = 124 B.  CPU baseline: the
    oracle's FP32 restatement (bit-identical to the reference's bxdf.h on
    the golden vectors) on all host threads."""
    import torch
    dev = torch.device("cuda")
    f32 = dict(dtype=torch.float32, device=dev)
    normal, wo, color = (torch.empty((n, 3), **f32) for _ in range(3))
    params, rnd = torch.empty((n, 12), **f32), torch.empty((n, 2), **f32)
    wi, f = torch.empty((n, 3), **f32), torch.empty((n, 3), **f32)
    pdf, delta = torch.empty(n, **f32), torch.empty(n, dtype=torch.int32, device=dev)
    S.bxdf_generate(0, normal, wo, color, params, rnd, wi, f, pdf)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MB > L2
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(launches)]
    for _ in range(3):
        S.bxdf_sample(S.BXDF_DISNEY, normal, wo, color, params, rnd, wi, f, pdf, delta)
    for a, b in evs:
        flush.fill_(1.0)
        a.record()
        S.bxdf_sample(S.BXDF_DISNEY, normal, wo, color, params, rnd, wi, f, pdf, delta)
        b.record()
    torch.cuda.synchronize()
    ms = statistics.median(a.elapsed_time(b) for a, b in evs)
    peak, peak_kind = peaks()
    gbs = 124.0 * n / (ms / 1e3) / 1e9
    out = {"workload": "Disney BSDF sample + f + pdf, 2^20 points (config-0 inputs, PCG32 per point)",
           "mpoints_per_s": round(n / (ms / 1e3) / 1e6, 1), "kernel_ms": round(ms, 4),
           "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "peak_kind": peak_kind,
                        "unit": "GB/s", "frac": round(gbs / peak, 4), "alg_bytes_per_point": 124},
           "l2": "flushed (256 MB write) before every launch"}
    if cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        nrm, w_o, col, prm, r4 = O.bxdf_inputs(0, n)
        t0 = time.perf_counter()
        O.bxdf_sample(32, S.BXDF_DISNEY, nrm, w_o, col, prm, r4[:, :2].copy(), threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(n / dt / 1e6, 2), "unit": "Mpoints/s", "cores": threads,
                               "kind": "port", "sample": "the same 2^20 points, oracle FP32 BxDF"}
    return out


def cornell_eval(S, steps=10, warmup=3, cpu=True):
    """The Cornell box at 512x512, 16 spp, depth 8, Russian roulette from
    depth 3, NEE with MIS: the small-scene configuration (36 triangles, the
    BVH stays in L1/L2, so traversal is latency-bound).  Kernel time from CUDA
    events around `steps` renders on the launching stream; the scene is tiny,
    so there is no L2 flush.  CPU baseline: the oracle's megakernel
    restatement on all host threads, whole frame."""
    import torch
    w = h = 512
    spp, depth, rr = 16, 8, 3
    arrays = S.procedural("cornell")
    arrays.set_aspect(1.0)
    scene = S.Scene(arrays)
    pt = S.PathTracer(scene, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    p = S.pt_params(spp, depth, rr, 1, 1, SEED)
    for i in range(warmup):
        p.seed = SEED + 100 + i
        pt.render(film, p, stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for i in range(steps):
        p.seed = SEED + i
        pt.render(film, p, stream)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    st = pt.stats()
    out = {"workload": "Cornell box, 36 triangles, 512x512, 16 spp, depth 8, rr 3, NEE + MIS",
           "msamples_per_s": round(w * h * spp / (ms / 1e3) / 1e6, 1), "ms_per_frame": round(ms, 3),
           "closest_rays_per_frame": st["closest_rays"], "shadow_rays_per_frame": st["shadow_rays"]}
    if cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        osc = O.OracleScene(arrays.desc(), bvh=True)
        t0 = time.perf_counter()
        osc.render(w, h, p, threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(w * h * spp / dt / 1e6, 3), "unit": "Msamples/s", "cores": threads,
                               "kind": "port", "sample": "whole 512x512 frame at 16 spp, oracle CPU BVH"}
    pt.close()
    return out


def relmse(S, x, ref):
    """Reference relMSE (metrics.h:30-34, largest 0.1 % dropped) on the GPU."""
    import torch
    return S.film_metric(torch.from_numpy(x).cuda(), torch.from_numpy(ref).cuda(), S.METRIC_RELMSE, 0.1)


def cache_eval(S, arrays, scene, frames=256, w=1280, h=720, ref_frames=64, ref_spp=64):
    """Learned-cache workload: 1280x720, 1 spp per frame for `frames` frames
    with online training on 2^16 paths per frame; relMSE of the accumulated
    image against a 4096-spp plain render accumulated in FP64, and the wall
    time the cached form needs to reach the plain tracer's 64-spp relMSE."""
    import ctypes as C
    import numpy as np
    import torch
    arrays.set_aspect(w / h)
    S.check(S.lib().srt_scene_set_camera(scene.handle, C.byref(arrays.camera)))
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    plain = S.PathTracer(scene, w, h)
    # reference: 64 frames x 64 spp accumulated in FP64
    acc = np.zeros((w * h, 4), np.float64)
    for f in range(ref_frames):
        plain.render(film, S.pt_params(ref_spp, MAX_DEPTH, RR_DEPTH, 1, 1, 50000 + f))
        torch.cuda.synchronize()
        acc += film.cpu().numpy()
    ref = (acc / ref_frames).astype(np.float32)
    # plain 64 spp: relMSE and wall time
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain.render(film, S.pt_params(64, MAX_DEPTH, RR_DEPTH, 1, 1, 777))
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    rel_plain = relmse(S, film.cpu().numpy(), ref)
    # cached: progressive 1-spp frames, network trained online
    verts = np.concatenate([m["vertices"] for m in arrays.meshes])
    lo, hi = verts.min(0) - 0.05, verts.max(0) + 0.05
    mlp = C.c_void_p()
    S.check(S.lib().srt_mlp_create(1, C.byref(mlp)))
    S.check(S.lib().srt_mlp_set_box(mlp, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi)))
    pt = S.PathTracer(scene, w, h)
    cp = S._capi.CacheParams(1 << 16, 4, 1e-2, 0.5, 16, 1)
    st = S._capi.CacheStats()
    accd = torch.zeros((w * h, 4), dtype=torch.float64, device="cuda")
    # the first FP64 accumulate loads torch's kernels (over a second on a fresh process): not frame time
    accd += film.double()
    accd.zero_()
    torch.cuda.synchronize()
    t_total, t_reach, curve = 0.0, None, []
    queries = fallback = 0
    for f in range(frames):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p = S.pt_params(1, MAX_DEPTH, RR_DEPTH, 1, 1, 9000 + f)
        S.check(S.lib().srt_pt_render_cached(pt.handle, C.c_void_p(film.data_ptr()), C.byref(p), mlp,
                                             C.byref(cp), C.byref(st), None))
        accd += film.double()
        torch.cuda.synchronize()
        t_total += time.perf_counter() - t0
        queries += st.queries
        fallback += st.fallback_queries
        if (f + 1) in (1, 2, 4, 8, 16, 32, 64, 128, 256) or (t_reach is None and (f + 1) % 8 == 0):
            r = relmse(S, (accd / (f + 1)).float().cpu().numpy(), ref)
            curve.append((f + 1, round(t_total, 4), r))
            if t_reach is None and r <= rel_plain:
                t_reach = t_total
    S.lib().srt_mlp_destroy(mlp)
    arrays.set_aspect(W / H)
    S.check(S.lib().srt_scene_set_camera(scene.handle, C.byref(arrays.camera)))
    return {"workload": f"{w}x{h}, 1 spp/frame x {frames} frames, online training on 2^16 paths/frame",
            "reference": f"{ref_frames * ref_spp}-spp plain render accumulated in FP64",
            "plain_64spp": {"relmse": rel_plain, "wall_s": round(t_plain, 4)},
            "cached": {"relmse_final": curve[-1][2], "wall_s": round(t_total, 4), "frames": frames,
                       "relmse_curve": curve,
                       "fallback_fraction": round(fallback / max(1, queries + fallback), 4)},
            "time_to_plain64_relmse_s": None if t_reach is None else round(t_reach, 4),
            "speedup_vs_plain64": None if t_reach is None else round(t_plain / t_reach, 3)}


def serving_eval(S, scene_big, rate=20.0, duration=10.0):
    """Short serving run (Poisson arrivals at `rate` jobs/s for `duration` s)."""
    from srt_gb300 import serve_bench as SB
    scenes = SB.build_scenes(S, n_variants=1, cache_frames=30)
    out = SB.run_rate(S, scenes, rate, duration)
    out["mix"] = "res {256^2,512^2,1024^2,1920x1080} x spp {1,4,16,64} x {cornell, 5.2M spheres} x {plain, cached}"
    return out


def profile_case():
    """The benchmark scene (392 MB resident, larger than L2) at 1920x1080,
    for ncu.  Frame A: 1 spp with max depth 2, so the first closest-hit
    launch traces the 2,073,600 camera rays and the second the first-bounce
    rays (their count is printed), the first shadow launch the NEE rays of
    the primary hits.  Frame B: 1 spp at the benchmark's depth.  A few
    hundred launches in all; run it with SRT_NO_GRAPH=1 so that ncu sees the
    same kernels as separate launches."""
    import torch
    import srt_gb300 as S
    arrays = build_scene(S)
    scene = S.Scene(arrays)
    pt = S.PathTracer(scene, W, H)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    pt.render(film, S.pt_params(1, 2, RR_DEPTH, 1, 1, 0))
    torch.cuda.synchronize()
    a = pt.stats()
    pt.render(film, S.pt_params(1, MAX_DEPTH, RR_DEPTH, 1, 1, 1))
    torch.cuda.synchronize()
    b = pt.stats()
    print(json.dumps({"profile_case": "1920x1080x1spp",
                      "frame_a": {"max_depth": 2, "camera_rays": W * H,
                                  "bounce_rays": a["closest_rays"] - W * H, "shadow_rays": a["shadow_rays"]},
                      "frame_b": {"max_depth": MAX_DEPTH, "closest_rays": b["closest_rays"],
                                  "shadow_rays": b["shadow_rays"], "iterations": b["iterations"]}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cache", action="store_true", help="skip the learned-cache workload")
    ap.add_argument("--no-serving", action="store_true", help="skip the short serving run")
    ap.add_argument("--profile-case", action="store_true",
                    help="short run of the same scene (1 spp, two frames) for ncu captures")
    args = ap.parse_args()
    if args.profile_case:
        profile_case()
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    import srt_gb300 as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    arrays = build_scene(S)
    scene = S.Scene(arrays)
    info = scene.info()
    pt = S.PathTracer(scene, W, H)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    params = S.pt_params(SPP, MAX_DEPTH, RR_DEPTH, 1, 1, SEED)

    for i in range(args.warmup):
        params.seed = SEED + 1000 + i
        pt.render(film, params, stream)
    barrier()

    # ---- device-resident timed region ----------------------------------
    launches = 0
    with Clocks(local) as clk:
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for i in range(args.steps):
            params.seed = SEED + i
            pt.render(film, params, stream)
            launches += pt.stats()["kernel_launches"]
        ev1.record()
        barrier()
    ms = ev0.elapsed_time(ev1)
    ms = dist_max(ms, world, dev)
    samples = W * H * SPP * args.steps * world
    value = samples / (ms / 1e3) / 1e6
    clocks = clk.summary()

    # ---- end to end through the C ABI with host buffers -----------------
    host_film = torch.empty((W * H, 4), dtype=torch.float32, pin_memory=True)
    h2d = C_PARAM_BYTES = 32 + 48  # srt_pt_params + srt_camera_desc handed over per frame
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        params.seed = SEED + 500 + i
        scene.set_camera(arrays.camera)
        pt.render(film, params, stream)
        host_film.copy_(film, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = samples / dist_max(e2e_s, world, dev) / 1e6

    # ---- two profiled frames of the same seed (identical rays): one with
    # the counting traversal kernels for the work per ray, one with event
    # timestamps around the production kernels for their durations -------
    params.seed = SEED + 900
    pt.set_profiling(1)
    pt.render(film, params, stream)
    st = pt.stats()
    pt.set_profiling(2)
    pt.render(film, params, stream)
    st_t = pt.stats()
    pt.set_profiling(0)
    names = ["k_closest", "k_shade", "k_shadow", "k_regen", "k_advance"]
    kms = dict(zip(names, st_t["kernel_ms"]))
    top = max(kms, key=kms.get)
    # algorithmic bytes: per ray the ray (24 B) in and the hit (16 B) out, plus
    # the BVH nodes (128 B) and triangles (48 B) the traversal fetches
    if top == "k_shadow":
        rays, nodes, tris = st["shadow_rays"], st["shadow_nodes"], st["shadow_tris"]
        per_ray = 44
    else:
        rays, nodes, tris = st["closest_rays"], st["closest_nodes"], st["closest_tris"]
        per_ray = 40
    alg_bytes = rays * per_ray + nodes * 128 + tris * 48
    iters = max(1, st["iterations"])
    traffic, traffic_src = measured_traffic(top, rays / iters)
    achieved = alg_bytes / (kms[top] / 1e3) / 1e9 if kms[top] > 0 else 0.0
    peak, peak_kind = peaks()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_dict(info),
            "clocks": clocks,
            "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": W * H * 16},
            "gpu_launches": int(launches),
            "mrays_per_s": round((st["closest_rays"] + st["shadow_rays"]) / (ms / args.steps / 1e3) / 1e6, 1),
            "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "traffic_source": traffic_src, "launches": iters,
                         "per_launch_ms": round(kms[top] / iters, 4),
                         "alg_bytes_per_launch": int(alg_bytes / iters),
                         "nodes_per_ray": round(nodes / max(rays, 1), 2),
                         "tris_per_ray": round(tris / max(rays, 1), 2),
                         "shadow_nodes_per_ray": round(st["shadow_nodes"] / max(st["shadow_rays"], 1), 2),
                         "shadow_tris_per_ray": round(st["shadow_tris"] / max(st["shadow_rays"], 1), 2)},
            "profile_frame": {"kernel_ms": {k: round(v, 2) for k, v in kms.items()},
                              "closest_rays": st["closest_rays"], "shadow_rays": st["shadow_rays"],
                              "iterations": st["iterations"]},
        }
        line["bxdf"] = bxdf_eval_bench(S, cpu=not args.no_cpu_baseline)
        line["cornell"] = cornell_eval(S, cpu=not args.no_cpu_baseline)
        if not args.no_cache:
            line["cache"] = cache_eval(S, arrays, scene)
        if not args.no_serving:
            line["serving"] = serving_eval(S, scene)
            line["p50_job_latency_s"] = line["serving"]["p50_job_s"]
            line["p99_job_latency_s"] = line["serving"]["p99_job_s"]
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(arrays, steps=1, budget_s=20.0)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
