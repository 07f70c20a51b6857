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
host cores (the oracle's CPU restatement, which loads only the oracle
library) on a seeded uniform sample of the frame's pixels at the full 64 spp.

Extra keys: `roofline` for the kernel with the most device time in a
timed profile frame (CUDA events around the production kernels): achieved =
the per-ray bytes of the scope table (40 B ray + hit, plus the BVH traffic
measured by ncu, profiles/<kernel>_dram.json) / launch time, with the
logical node-and-triangle fetch figure beside it (`l2_level`) and the ncu
counters that bound the kernel (`limiter`); `cache` (learned-cache time to
the plain tracer's 64-spp relMSE, 1280x720), `serving` (Poisson arrivals at
several rates under a 150 GB budget), `bxdf` (the Disney BSDF batch of 2^20
points, with its FP64 parity), `cornell` (the Cornell box at 512x512, 16 spp,
depth 8, with its roofline), `mlp` (the two networks' tcgen05 kernels on
2,073,600 rows against the measured bf16 GEMM rate), `cpu_baseline`.  `--no-cache`, `--no-serving`,
`--no-cpu-baseline` skip those parts; `--profile-case spheres|cornell` runs
the short case the ncu captures use.
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


def tensor_peak():
    """Dense bf16 TFLOP/s of a cuBLAS GEMM timed alone (burst)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


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


def cpu_baseline(steps=1, budget_s=20.0, warmup=0):
    """The oracle's megakernel restatement (path_tracer.cu:50-169, own CPU
    BVH) on all host cores, on a seeded uniform sample of the frame's pixels
    at the full 64 spp and depth 16, so a sample's cost follows the frame's
    mix of environment and surface pixels.  The scene is built inside the
    oracle library from the same generator source: no CUDA library is
    loaded.  About `budget_s` seconds of CPU work in all."""
    import numpy as np
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    osc = O.OracleScene.procedural("spheres", seed=SEED, n_spheres=N_SPHERES, subdiv=SUBDIV, aspect=W / H, bvh=True)
    build_s = time.perf_counter() - t0
    order = np.random.default_rng(SEED).permutation(W * H).astype(np.int32)
    # calibrate on 1024 pixels, then size the per-step sample to the budget
    t0 = time.perf_counter()
    osc.render_pixels(W, H, O.pt_params(SPP, MAX_DEPTH, RR_DEPTH, 1, 1, SEED), order[:1024], threads=threads)
    rate = 1024 * SPP / max(time.perf_counter() - t0, 1e-3)
    npix = int(max(1024, min(W * H, rate * budget_s / max(1, steps + warmup) / SPP)))
    pix = np.sort(order[:npix])
    for i in range(warmup):
        osc.render_pixels(W, H, O.pt_params(SPP, MAX_DEPTH, RR_DEPTH, 1, 1, SEED + 2000 + i), pix, threads=threads)
    times = []
    for i in range(steps):
        t0 = time.perf_counter()
        osc.render_pixels(W, H, O.pt_params(SPP, MAX_DEPTH, RR_DEPTH, 1, 1, SEED + i), pix, threads=threads)
        times.append(time.perf_counter() - t0)
    value = npix * SPP * len(times) / sum(times) / 1e6
    return {"value": round(value, 4), "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{npix} pixels drawn uniformly (seeded) from the {W}x{H} frame, {SPP} spp each, depth "
                      f"{MAX_DEPTH}, per step; oracle CPU BVH (build {build_s:.1f}s, not timed), {threads} threads"}


def run_reference(args, rank, world):
    """The reference arm: the oracle's CPU restatement of the path tracer on
    the host cores, same metric and workload (a bounded pixel sample per
    step).  Only rank 0 works; nothing of the CUDA library is loaded."""
    if rank != 0:
        return
    steps = max(1, args.steps)
    warmup = min(1, max(0, args.warmup))
    cb = cpu_baseline(steps=steps, budget_s=min(120.0, 6.0 * (steps + warmup)), warmup=warmup)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(), "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict():
    """The workload definition, identical in both arms."""
    return {"workload": "5.2M-triangle synthetic scene (64 icospheres subdiv 6, value-noise displaced), "
                        "plain wavefront PT FP32", "width": W, "height": H, "spp": SPP, "max_depth": MAX_DEPTH,
            "rr_depth": RR_DEPTH, "nee": True, "mis": True, "rng": "curand XORWOW per pixel",
            "l2": "scene larger than L2 (no flush between steps)"}


def scene_dict(info):
    return {"triangles": info["num_triangles"], "scene_mb": round(info["device_bytes"] / 2 ** 20, 1),
            "bvh_nodes": info["num_nodes"], "bvh_build_s": round(info["build_ms"] / 1000, 2)}


def profile_record(name):
    """One ncu capture's summary (profiles/<name>_dram.json): DRAM bytes per
    ray (dram__bytes_read.sum + dram__bytes_write.sum of a captured launch /
    its rays) and the counters that bound the kernel."""
    path = os.path.join(ROOT, "profiles", f"{name}_dram.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def bxdf_fp64_parity(S, O, normal, wo, color, params, rnd):
    """The kernel's f and pdf at its own sampled direction against the FP64
    evaluation of the same formulas (the oracle's FP64 restatement) on
    device inputs: fraction of sampled points beyond 1e-5 relative and the
    error quantiles; the reference's own FP32 formulas (the oracle's FP32
    restatement, bit-identical to the reference's bxdf.h on the golden
    vectors) measured the same way beside it."""
    import numpy as np
    import torch
    n = normal.shape[0]
    dev = normal.device
    wi = torch.empty((n, 3), dtype=torch.float32, device=dev)
    f = torch.empty((n, 3), dtype=torch.float32, device=dev)
    pdf = torch.empty(n, dtype=torch.float32, device=dev)
    delta = torch.empty(n, dtype=torch.int32, device=dev)
    S.bxdf_sample(S.BXDF_DISNEY, normal, wo, color, params, rnd, wi, f, pdf, delta)
    torch.cuda.synchronize()
    h = [t.cpu().numpy() for t in (normal, wo, color, params, rnd, wi, f, pdf)]
    nrm, w_o, col, prm, r2, wi_, f_, pdf_ = h

    def rel(fa, pa, fb, pb):
        ef = (np.abs(fa - fb) / np.maximum(np.abs(fb), 1e-20)).max(1)
        return np.maximum(ef, np.abs(pa - pb) / np.maximum(np.abs(pb), 1e-20))

    ok = pdf_ > 0
    f64, p64 = O.bxdf_eval_pdf(64, S.BXDF_DISNEY, nrm, w_o, col, prm, wi_.astype(np.float64))
    r = rel(f_[ok], pdf_[ok], f64[ok], p64[ok])
    w32, f32, p32, _ = O.bxdf_sample(32, S.BXDF_DISNEY, nrm, w_o, col, prm, r2, threads=os.cpu_count() or 1)
    ok32 = p32 > 0
    f64b, p64b = O.bxdf_eval_pdf(64, S.BXDF_DISNEY, nrm, w_o, col, prm, w32)
    rr = rel(f32[ok32], p32[ok32], f64b[ok32], p64b[ok32])
    q = [0.5, 0.9, 0.99, 0.999]
    return {"sampled_points": int(ok.sum()), "frac_beyond_1e-5": round(float(np.mean(r > 1e-5)), 5),
            "rel_err_quantiles": {str(k): float(v) for k, v in zip(q, np.quantile(r, q))},
            "reference_fp32_frac_beyond_1e-5": round(float(np.mean(rr > 1e-5)), 5)}


def bxdf_eval_bench(S, n=1 << 20, launches=20, cpu=True):
    """Disney BSDF batch (sample + f + pdf, GMaterial::sample) on n = 2^20
    shading points generated in device memory from the PCG32 streams of
    the config-0 definition; kernel time from CUDA events per launch with
    L2 flushed between launches.  Algorithmic bytes per point = inputs
    (normal, wo, colour: 36 B; 12 parameters: 48 B; 2 uniforms: 8 B) +
    outputs (wi, f: 24 B; pdf, delta: 8 B) = 124 B.  CPU leg: the oracle's
    FP32 restatement (bit-identical to the reference's bxdf.h on the golden
    vectors) on all host threads, and the FP64 parity of the kernel's
    values on the same points (world frame) and with the shading frame
    exact (normal = +z)."""
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
        import numpy as np
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        nrm, w_o, col, prm, r4 = O.bxdf_inputs(0, n)
        t0 = time.perf_counter()
        O.bxdf_sample(32, S.BXDF_DISNEY, nrm, w_o, col, prm, r4[:, :2].copy(), threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(n / dt / 1e6, 2), "unit": "Mpoints/s", "cores": threads,
                               "kind": "port", "sample": "the same 2^20 points, oracle FP32 BxDF"}
        par = {"world_frame": bxdf_fp64_parity(S, O, normal, wo, color, params, rnd)}
        # exact shading frame: normal = +z, wo uniform on the upper hemisphere
        g = np.random.default_rng(11)
        v = g.normal(size=(n, 3))
        v[:, 2] = np.abs(v[:, 2]) + 1e-3
        v = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
        nz = torch.zeros((n, 3), **f32)
        nz[:, 2] = 1.0
        par["local_frame"] = bxdf_fp64_parity(S, O, nz, torch.from_numpy(v).to(dev), color, params, rnd)
        out["fp64_parity"] = par
    return out


def mlp_eval(S, n=1920 * 1080, reps=10):
    """The two networks' tensor-core kernels (tcgen05.mma, accumulators in
    tensor memory) on n rows.  NeuralRadiosity's network 96 -> 256 x 4 -> 16
    (srt_nr_infer: the encoding kernel and the fused five-layer kernel, each
    timed with the handle's profiling events) and the radiance cache's
    96 -> 64 x 5 -> 16 (srt_mlp_infer, features built in the kernel; CUDA
    events).  FLOPs per row = 2 * sum(in * out) over the layers; roofline
    against the measured dense bf16 GEMM rate."""
    import ctypes as C
    import torch
    L = S.lib()
    peak, kind = tensor_peak()
    dev = torch.device("cuda")
    out = {}
    nr = C.c_void_p()
    S.check(L.srt_nr_create(7, C.byref(nr)))
    x = torch.rand((n, 12), device=dev)
    y = torch.empty((n, 16), device=dev)
    S.check(L.srt_nr_set_profiling(nr, 1))
    st = S._capi.NrStats()
    enc, net = [], []
    for i in range(reps + 3):
        S.check(L.srt_nr_infer(nr, C.c_void_p(x.data_ptr()), n, C.c_void_p(y.data_ptr()), None))
        S.check(L.srt_nr_get_stats(nr, C.byref(st)))
        if i >= 3:
            enc.append(st.encode_ms)
            net.append(st.network_ms)
    L.srt_nr_destroy(nr)
    flops = 2.0 * n * (96 * 256 + 3 * 256 * 256 + 256 * 16)
    ms = statistics.median(net)
    tf = flops / (ms / 1e3) / 1e12
    out["neural_radiosity"] = {"rows": n, "network_ms": round(ms, 4), "encode_ms": round(statistics.median(enc), 4),
                               "roofline": {"bound": "tensor", "kernel": "k_umma_mlp_stream<NrNetTask>", "achieved": round(tf, 1),
                                            "peak": peak, "peak_kind": kind, "unit": "TFLOP/s",
                                            "frac": round(tf / peak, 4), "flops_per_row": flops / n}}
    mlp = C.c_void_p()
    S.check(L.srt_mlp_create(3, C.byref(mlp)))
    rec = torch.rand((n, 16), device=dev)
    o4 = torch.empty((n, 4), device=dev)
    call = lambda: S.check(L.srt_mlp_infer(mlp, C.c_void_p(rec.data_ptr()), n, C.c_void_p(o4.data_ptr()), None))
    for _ in range(3):
        call()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in evs:
        a.record()
        call()
        b.record()
    torch.cuda.synchronize()
    L.srt_mlp_destroy(mlp)
    ms2 = statistics.median(a.elapsed_time(b) for a, b in evs)
    flops2 = 2.0 * n * (96 * 64 + 4 * 64 * 64 + 64 * 16)
    tf2 = flops2 / (ms2 / 1e3) / 1e12
    out["radiance_cache"] = {"rows": n, "kernel_ms": round(ms2, 4),
                             "roofline": {"bound": "tensor", "kernel": "k_umma_mlp<MlpInferTask>", "achieved": round(tf2, 1),
                                          "peak": peak, "peak_kind": kind, "unit": "TFLOP/s",
                                          "frac": round(tf2 / peak, 4), "flops_per_row": flops2 / n}}
    return out


# the profiling slots of srt_pt_stats.kernel_ms
KERNELS = ["k_trace", "k_shade", "k_order", "k_regen", "k_advance"]
# queue bytes a closest-hit ray moves in k_trace (origin 16 B, direction 16 B,
# job word 4 B in; hit record 16 B out)
CLOSEST_QUEUE_BYTES = 52


def kernel_bytes(st, hist, npix):
    """Algorithmic bytes of one frame's wavefront iterations per kernel, from
    their exact counts (the iteration history: the finishing kernel's rays
    are not in it) and the queue layout (wavefront.cuh): R closest rays (H of
    them hits), Sh shadow rays, N samples ended over npix pixels.
      k_trace: per closest ray 32 B of ray + 4 B job word in, 16 B hit out;
        per shadow ray 48 B in + 32 B radiance update (BVH nodes and
        triangles are not included: they come from ncu's DRAM bytes where the
        scene exceeds L2)
      k_order: 4 B in, 4 B out per ray
      k_shade: order index 4 B + hit 16 B + path state 72 B in per ray; per
        hit the triangle 48 B, instance 16 B, material 80 B; per shadow ray
        the light triangle 48 B in and the shadow record 48 B out; 72 B out
        per continuing path and per next-sample camera ray, 8 B done record
        and 16 B radiance record read per ended sample, 32 B radiance update
        per miss
      k_regen: done record 8 B + radiance 32 B + film 32 B per sample"""
    R, Hh, Sh, N = (int(hist[:, k].sum()) for k in (0, 1, 3, 4))
    return {"k_trace": R * CLOSEST_QUEUE_BYTES + Sh * 80,
            "k_shade": (R * 92 + Hh * 144 + Sh * 96 + (R - N) * 72 + N * 24 + max(0, N - npix) * 72
                        + (R - Hh) * 32),
            "k_order": R * 8,
            "k_regen": N * 72,
            "k_advance": 0}


def cornell_eval(S, steps=10, warmup=3, cpu=True):
    """The Cornell box at 512x512, 16 spp, depth 8, Russian roulette from
    depth 3, NEE with MIS: the small-scene configuration (36 triangles, the
    BVH stays in L1/L2, so traversal is latency-bound).  Kernel time from CUDA
    events around `steps` renders on the launching stream; the scene is tiny,
    so there is no L2 flush.  Roofline: the kernel with the most device time
    in a timed profile frame (event timestamps around the production
    kernels), achieved = its algorithmic bytes (kernel_bytes) / its time.
    CPU baseline: the oracle's megakernel restatement on all host threads,
    whole frame."""
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
    hist = pt.iteration_counts()
    # one frame of the same seed with timestamps around the production kernels
    p.seed = SEED
    pt.set_profiling(2)
    pt.render(film, p, stream)
    st_p = pt.stats()
    kms = dict(zip(KERNELS, st_p["kernel_ms"]))
    pt.set_profiling(0)
    top = max(kms, key=kms.get)
    alg = kernel_bytes(st, hist, w * h)
    peak, peak_kind = peaks()
    achieved = alg[top] / (kms[top] / 1e3) / 1e9
    iters = max(1, st["iterations"])
    rec = profile_record(f"cornell_{top}")
    traffic = None
    if rec:
        # DRAM bytes per algorithmic byte of the captured launch, scaled to the average launch
        traffic = int(rec["dram_bytes_per_alg_byte"] * (alg[top] / iters))
    out = {"workload": "Cornell box, 36 triangles, 512x512, 16 spp, depth 8, rr 3, NEE + MIS",
           "msamples_per_s": round(w * h * spp / (ms / 1e3) / 1e6, 1), "ms_per_frame": round(ms, 3),
           "closest_rays_per_frame": st["closest_rays"], "shadow_rays_per_frame": st["shadow_rays"],
           "iterations": st["iterations"], "tail_paths": st["tail_paths"],
           "profile_frame_kernel_ms": dict({k: round(v, 3) for k, v in kms.items()},
                                           k_finish=round(st_p["tail_ms"], 3)),
           "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak,
                        "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                        "traffic": traffic, "traffic_source": rec["capture"] if rec else None,
                        "launches": iters, "per_launch_ms": round(kms[top] / iters, 5),
                        "alg_bytes_per_launch": int(alg[top] / iters),
                        "limiter": rec.get("limiter") if rec else None,
                        "alg_bytes_per_sample": round(sum(alg.values()) / (w * h * spp), 1)}}
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


def cache_bound(S, scene, ref, w, h, frames=128):
    """Upper bound on the time-to-quality speedup of ANY cache that ends
    paths at the second vertex, measured on this scene.  A perfect cache
    returns the exact expected radiance at the second vertex: it removes
    the variance of everything after it and the cost of tracing it, but
    keeps the variance of the path prefix (camera ray, emission and NEE at
    the first vertex: the estimator with max depth 1, its terms assumed not
    negatively correlated with the rest) and costs at least the prefix.
    Per-pixel variances from `frames` independent 1-spp frames of the full
    estimator and of the prefix; their trimmed (largest 0.1 % dropped) mean
    relMSE contribution per sample against the FP64 reference gives the
    variance ratio r, so the perfect cache needs 64 r samples to reach the
    plain 64-spp relMSE; cost per sample from 64-spp frames at max depth 16
    (plain) and 1 (prefix, optimistic: the second-vertex ray is not even
    traced).  Bound = (t_plain / t_prefix per sample) / r."""
    import numpy as np
    import torch
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    pt = S.PathTracer(scene, w, h)
    refd = torch.from_numpy(ref[:, :3]).cuda().double()
    den = (refd + 1e-6) ** 2

    def rel_per_sample(depth, flags=0):
        s1 = torch.zeros((w * h, 3), dtype=torch.float64, device="cuda")
        s2 = torch.zeros_like(s1)
        for f in range(frames):
            pt.render(film, S.pt_params(1, depth, RR_DEPTH, 1, 1, 30000 + f, flags=flags))
            x = film[:, :3].double()
            s1 += x
            s2 += x * x
        var = (s2 - s1 * s1 / frames) / (frames - 1)
        e = (var / den).mean(1)
        keep = int(e.numel() * 0.999)
        return float(torch.sort(e).values[:keep].mean())

    def per_sample_ms(depth, flags=0):
        pt.render(film, S.pt_params(64, depth, RR_DEPTH, 1, 1, 777, flags=flags))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(3):
            pt.render(film, S.pt_params(64, depth, RR_DEPTH, 1, 1, 778 + i, flags=flags))
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / 3 / 64 * 1e3

    nee1 = S._capi.PT_NEE_FIRST_VERTEX_ONLY
    e_full, e1, e2, ep = (rel_per_sample(MAX_DEPTH), rel_per_sample(1), rel_per_sample(2),
                          rel_per_sample(2, nee1))
    t_full, t1, t2, tp = per_sample_ms(MAX_DEPTH), per_sample_ms(1), per_sample_ms(2), per_sample_ms(2, nee1)
    r1, r2, rp = e1 / e_full, e2 / e_full, ep / e_full
    pt.close()
    # the prefix a second-vertex cache keeps: depth 2 with next-event
    # estimation at the first vertex only (the cache replaces the second
    # vertex's light sample and everything after it, but a ray that reaches
    # a light at the second vertex adds its MIS-weighted emission); depth 1
    # and depth 2 with both light samples bracket it
    return {"frames_for_variance": frames, "relmse_per_sample_plain": e_full,
            "relmse_per_sample_prefix": ep, "relmse_per_sample_depth1": e1, "relmse_per_sample_depth2": e2,
            "variance_ratio_prefix": round(rp, 4), "variance_ratio_depth1": round(r1, 4),
            "variance_ratio_depth2": round(r2, 4),
            "samples_a_perfect_cache_needs": round(64 * rp, 1),
            "ms_per_sample_plain_depth16": round(t_full, 4), "ms_per_sample_prefix": round(tp, 4),
            "ms_per_sample_depth1": round(t1, 4), "ms_per_sample_depth2": round(t2, 4),
            "max_speedup_any_second_vertex_cache": round((t_full / tp) / rp, 3)}


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
    bound = cache_bound(S, scene, ref, w, h)
    arrays.set_aspect(W / H)
    S.check(S.lib().srt_scene_set_camera(scene.handle, C.byref(arrays.camera)))
    return {"workload": f"{w}x{h}, 1 spp/frame x {frames} frames, online training on 2^16 paths/frame",
            "reference": f"{ref_frames * ref_spp}-spp plain render accumulated in FP64",
            "plain_64spp": {"relmse": rel_plain, "wall_s": round(t_plain, 4)},
            "cached": {"relmse_final": curve[-1][2], "wall_s": round(t_total, 4), "frames": frames,
                       "relmse_curve": curve,
                       "fallback_fraction": round(fallback / max(1, queries + fallback), 4)},
            "time_to_plain64_relmse_s": None if t_reach is None else round(t_reach, 4),
            "speedup_vs_plain64": None if t_reach is None else round(t_plain / t_reach, 3),
            "bound": bound}


def serving_eval(S, rates=(5.0, 20.0, 50.0), duration=30.0):
    """Render serving (config 4): Poisson arrivals at each rate for
    `duration` s under a 150 GB HBM budget, the job mix of serve_bench
    (resolution, spp, scene, plain / cached); p50 / p99 job latency, first
    progressive frame and frame interval, and Msamples/s per rate."""
    from srt_gb300 import serve_bench as SB
    scenes = SB.build_scenes(S, n_variants=1, cache_frames=30)
    table = [SB.run_rate(S, scenes, r, duration) for r in rates]
    return {"mix": "res {256^2,512^2,1024^2,1920x1080} x spp {1,4,16,64} x {cornell, 5.2M spheres} x "
                   "{plain, cached (network trained beforehand; half of the cached jobs train it online, half frozen)}",
            "budget_gb": 150, "duration_s": duration, "rates": table}


def profile_case(which="spheres"):
    """Short cases for ncu.  spheres: the benchmark scene (392 MB resident,
    larger than L2) at 1920x1080.  Frame A: 1 spp with max depth 2, so the
    first closest-hit launch traces the 2,073,600 camera rays and the second
    the first-bounce rays (their count is printed), the first shadow launch
    the NEE rays of the primary hits.  Frame B: 1 spp at the benchmark's
    depth.  cornell: one frame of the Cornell workload (512x512, 16 spp,
    depth 8).  Every kernel is launched directly (no graph), so ncu sees each
    launch; a few hundred launches in all."""
    import torch
    import srt_gb300 as S
    if which == "mlp":
        # the two networks' tensor-core kernels on 262,144 random rows: three
        # NeuralRadiosity inferences (encoding + fused network), then three
        # radiance-cache inferences
        import ctypes as C
        L = S.lib()
        n = 262144
        nr, mlp = C.c_void_p(), C.c_void_p()
        S.check(L.srt_nr_create(7, C.byref(nr)))
        S.check(L.srt_mlp_create(3, C.byref(mlp)))
        x = torch.rand((n, 12), device="cuda")
        y = torch.empty((n, 16), device="cuda")
        rec = torch.rand((n, 16), device="cuda")
        o4 = torch.empty((n, 4), device="cuda")
        for _ in range(3):
            S.check(L.srt_nr_infer(nr, C.c_void_p(x.data_ptr()), n, C.c_void_p(y.data_ptr()), None))
        for _ in range(3):
            S.check(L.srt_mlp_infer(mlp, C.c_void_p(rec.data_ptr()), n, C.c_void_p(o4.data_ptr()), None))
        torch.cuda.synchronize()
        ok = bool(torch.isfinite(y).all()) and bool(torch.isfinite(o4).all())
        L.srt_nr_destroy(nr)
        L.srt_mlp_destroy(mlp)
        print(json.dumps({"profile_case": "mlp 262144 rows", "finite": ok}))
        return
    if which == "cache":
        # radiance-cache frames of the learned-cache workload (1280x720, 1 spp,
        # online training on 2^16 paths per frame), every kernel launched directly
        import ctypes as C
        import numpy as np
        w, h = 1280, 720
        arrays = build_scene(S)
        arrays.set_aspect(w / h)
        scene = S.Scene(arrays)
        verts = np.concatenate([m["vertices"] for m in arrays.meshes])
        lo, hi = verts.min(0) - 0.05, verts.max(0) + 0.05
        mlp = C.c_void_p()
        S.check(S.lib().srt_mlp_create(1, C.byref(mlp)))
        S.check(S.lib().srt_mlp_set_box(mlp, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi)))
        pt = S.PathTracer(scene, w, h)
        pt.set_launch_mode(S.LAUNCH_DIRECT)
        film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
        cp = S._capi.CacheParams(1 << 16, 4, 1e-2, 0.5, 16, 1)
        st = S._capi.CacheStats()
        rows = []
        for f in range(8):
            p = S.pt_params(1, MAX_DEPTH, RR_DEPTH, 1, 1, 9000 + f)
            S.check(S.lib().srt_pt_render_cached(pt.handle, C.c_void_p(film.data_ptr()), C.byref(p), mlp,
                                                 C.byref(cp), C.byref(st), None))
            rows.append({"queries": st.queries, "fallback": st.fallback_queries, "train_vertices": st.train_vertices})
        torch.cuda.synchronize()
        S.lib().srt_mlp_destroy(mlp)
        print(json.dumps({"profile_case": "cache 1280x720 8 frames", "frames": rows}))
        return
    if which == "cornell":
        arrays = S.procedural("cornell")
        arrays.set_aspect(1.0)
        scene = S.Scene(arrays)
        pt = S.PathTracer(scene, 512, 512)
        pt.set_launch_mode(S.LAUNCH_DIRECT)
        film = torch.zeros((512 * 512, 4), dtype=torch.float32, device="cuda")
        pt.render(film, S.pt_params(16, 8, 3, 1, 1, SEED))
        torch.cuda.synchronize()
        st = pt.stats()
        hist = pt.iteration_counts()
        print(json.dumps({"profile_case": "cornell 512x512x16spp", "closest_rays": st["closest_rays"],
                          "shadow_rays": st["shadow_rays"], "iterations": st["iterations"],
                          "per_iteration": hist[:8].tolist(),
                          "kernel_bytes": kernel_bytes(st, hist, 512 * 512)}))
        return
    arrays = build_scene(S)
    scene = S.Scene(arrays)
    pt = S.PathTracer(scene, W, H)
    pt.set_launch_mode(S.LAUNCH_DIRECT)
    film = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    pt.render(film, S.pt_params(1, 2, RR_DEPTH, 1, 1, 0))
    torch.cuda.synchronize()
    a = pt.stats()
    ha = pt.iteration_counts()
    pt.render(film, S.pt_params(1, MAX_DEPTH, RR_DEPTH, 1, 1, 1))
    torch.cuda.synchronize()
    b = pt.stats()
    print(json.dumps({"profile_case": "1920x1080x1spp",
                      "frame_a": {"max_depth": 2, "camera_rays": W * H,
                                  "bounce_rays": a["closest_rays"] - W * H, "shadow_rays": a["shadow_rays"],
                                  # the second k_trace launch: iteration 0's shadow rays and iteration 1's rays
                                  "k_trace_launch_2": {"shadow_rays": int(ha[0, 3]), "closest_rays": int(ha[1, 0])}},
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
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sweep")
    ap.add_argument("--serving-rates", default="5,20,50", help="Poisson arrival rates (jobs/s) of the sweep")
    ap.add_argument("--serving-duration", type=float, default=30.0, help="seconds of arrivals per rate")
    ap.add_argument("--profile-case", nargs="?", const="spheres", default=None, choices=["spheres", "cornell", "cache", "mlp"],
                    help="short run for ncu captures (direct launches)")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
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
    h2d = 32 + 48  # srt_pt_params + srt_camera_desc handed over per frame
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
    hist = pt.iteration_counts()
    pt.set_profiling(2)
    pt.render(film, params, stream)
    st_t = pt.stats()
    pt.set_profiling(0)
    kms = dict(zip(KERNELS, st_t["kernel_ms"]))
    top = max(kms, key=kms.get)
    iters = max(1, st["iterations"])
    # k_trace traces both kinds of ray; the traversal counters include the
    # finishing kernel's rays: scale them to the rays of the wavefront
    # iterations (whose launches are timed here)
    rc, rs = int(hist[:, 0].sum()), int(hist[:, 3].sum())
    wc = rc / max(st["closest_rays"], 1)
    ws = rs / max(st["shadow_rays"], 1)
    rays = rc + rs
    nodes = st["closest_nodes"] * wc + st["shadow_nodes"] * ws
    tris = st["closest_tris"] * wc + st["shadow_tris"] * ws
    per_ray = (rc * 40 + rs * 44) / max(rays, 1)  # ray and hit (closest), ray and tmax (shadow)
    queue = (rc * CLOSEST_QUEUE_BYTES + rs * 80) / max(rays, 1)
    peak, peak_kind = peaks()
    # algorithmic bytes per ray (the scope table): the ray and its hit
    # (per_ray) plus the BVH traffic ncu measured in DRAM per ray (its DRAM
    # bytes per ray less the queue bytes the kernel moves per ray)
    rec = profile_record(top)
    launch_ms = kms[top] / iters
    rays_per_launch = rays / iters
    roof = {"bound": "hbm", "kernel": top, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "launches": iters, "per_launch_ms": round(launch_ms, 4)}
    if rec:
        # BVH bytes per ray measured in DRAM (the capture's DRAM bytes less its queue traffic)
        bvh = rec.get("bvh_dram_bytes_per_ray", max(0.0, rec["dram_bytes_per_ray"] - queue))
        alg_per_ray = per_ray + bvh
        achieved = alg_per_ray * rays_per_launch / (launch_ms / 1e3) / 1e9
        roof.update({"achieved": round(achieved, 1), "frac": round(achieved / peak, 4),
                     "traffic": int((queue + bvh) * rays_per_launch),
                     "traffic_source": rec["capture"], "alg_bytes_per_ray": round(alg_per_ray, 1),
                     "alg_bytes_per_launch": int(alg_per_ray * rays_per_launch),
                     "limiter": rec.get("limiter")})
    # the logical figure: every node (128 B) and triangle (48 B) the traversal
    # fetches, wherever it is served from (L1, L2 or DRAM)
    logical = rays * per_ray + nodes * 128 + tris * 48
    l2_gbs = logical / iters / (launch_ms / 1e3) / 1e9
    roof["l2_level"] = {"alg_bytes_per_launch": int(logical / iters), "achieved": round(l2_gbs, 1),
                        "frac_of_hbm_peak": round(l2_gbs / peak, 4),
                        "nodes_per_ray": round(st["closest_nodes"] / max(st["closest_rays"], 1), 2),
                        "tris_per_ray": round(st["closest_tris"] / max(st["closest_rays"], 1), 2),
                        "shadow_nodes_per_ray": round(st["shadow_nodes"] / max(st["shadow_rays"], 1), 2),
                        "shadow_tris_per_ray": round(st["shadow_tris"] / max(st["shadow_rays"], 1), 2)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_dict(), "scene": scene_dict(info),
            "clocks": clocks,
            "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": W * H * 16},
            "gpu_launches": int(launches),
            "mrays_per_s": round((st["closest_rays"] + st["shadow_rays"]) / (ms / args.steps / 1e3) / 1e6, 1),
            "roofline": roof,
            "profile_frame": {"kernel_ms": dict({k: round(v, 2) for k, v in kms.items()},
                                                k_finish=round(st_t["tail_ms"], 2)),
                              "closest_rays": st["closest_rays"], "shadow_rays": st["shadow_rays"],
                              "iterations": st["iterations"], "tail_paths": st["tail_paths"],
                              "wavefront_closest_rays": int(hist[:, 0].sum()),
                              "wavefront_shadow_rays": int(hist[:, 3].sum())},
        }
        line["bxdf"] = bxdf_eval_bench(S, cpu=not args.no_cpu_baseline)
        line["cornell"] = cornell_eval(S, cpu=not args.no_cpu_baseline)
        line["mlp"] = mlp_eval(S)
        if not args.no_cache:
            line["cache"] = cache_eval(S, arrays, scene)
        if not args.no_serving:
            rates = [float(x) for x in args.serving_rates.split(",") if x]
            line["serving"] = serving_eval(S, rates, args.serving_duration)
            # headline latencies: the lowest rate of the sweep at or above 20 jobs/s, else the highest
            pick = [r for r in line["serving"]["rates"] if r["rate_jobs_per_s"] >= 20.0]
            row = pick[0] if pick else line["serving"]["rates"][-1]
            line["p50_job_latency_s"] = row["p50_job_s"]
            line["p99_job_latency_s"] = row["p99_job_s"]
            line["serving_latency_rate_jobs_per_s"] = row["rate_jobs_per_s"]
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(steps=1, budget_s=20.0)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
