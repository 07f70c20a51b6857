"""CUDA kernels against the CPU oracle, through the C ABI (GPU only).

Tolerances: kernels and oracle both compute in FP32 without multiply-add
contraction; they differ only where the device's sin/cos/pow/log differ from
the host libm by an ulp, so BSDF values agree within 1e-5 relative at
>= 99.5% of the points (98% for the ill-conditioned refraction lobe);
integer results (RNG words, primitive ids away from edges, sample counts)
must be equal.
"""
import numpy as np
import pytest

from helpers import golden, rel_err, scene_from_npz
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def test_rng_tape_matches_host_curand(cuda):
    import torch
    import srt_gb300 as S
    for seed in (0, 12345, 2147483000):  # the last wraps seed + idx past INT32_MAX
        out = torch.empty((3000, 9), dtype=torch.float32, device=cuda)
        S.rng_tape(seed, 3000, 9, out)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), O.curand_tape(seed, 3000, 9))


def _run_bxdf(cuda, type_, normal, wo, color, params, rnd2):
    import torch
    import srt_gb300 as S
    n = len(normal)
    d = {k: _t(v, cuda) for k, v in dict(normal=normal, wo=wo, color=color, params=params, rnd=rnd2).items()}
    wi = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    f = torch.zeros_like(wi)
    pdf = torch.zeros(n, dtype=torch.float32, device=cuda)
    delta = torch.zeros(n, dtype=torch.int32, device=cuda)
    S.bxdf_sample(type_, d["normal"], d["wo"], d["color"], d["params"], d["rnd"], wi, f, pdf, delta)
    torch.cuda.synchronize()
    return wi.cpu().numpy(), f.cpu().numpy(), pdf.cpu().numpy(), delta.cpu().numpy(), d


@pytest.mark.parametrize("name", ["disney", "disney_trans", "diffuse", "diffuse_transmission", "dielectric"])
def test_bxdf_sample_vs_reference_fp32(cuda, name):
    z = golden("bxdf")
    t, p = int(z[f"{name}_type"]), z[f"{name}_params"]
    wi, f, pdf, delta, _ = _run_bxdf(cuda, t, z["normal"], z["wo"], z["color"], p, z["rnd4"][:, :2].copy())
    ref_wi, ref_pdf = z[f"{name}_wi"], z[f"{name}_pdf"]
    np.testing.assert_array_equal(delta, z[f"{name}_delta"])
    both = (pdf > 0) & (ref_pdf > 0)
    # rejection decisions agree except at float ties
    assert np.mean((pdf > 0) == (ref_pdf > 0)) > 0.999
    # same lobe + direction: wi agrees to a few ulps (device sin/cos/pow/log differ by an ulp)
    close = np.abs(wi - ref_wi).max(1) < 1e-5
    assert np.mean(close[both]) > 0.998
    if t == 2:
        return  # thin dielectric: f = colour, pdf = 1 (delta)
    # sampled values against the reference's FP32 values for the same draws; the
    # refraction lobe is ill-conditioned near the critical angle, so an ulp of
    # difference in a device sin/cos/pow moves f and pdf by more there
    sel = both & close
    r = np.maximum(rel_err(f[sel], z[f"{name}_f"][sel], 1e-20).max(1), rel_err(pdf[sel], ref_pdf[sel], 1e-20))
    need = 0.98 if name == "disney_trans" else 0.995
    assert np.median(r) < 1e-6 and np.mean(r < 1e-5) > need, np.quantile(r, [0.5, 0.99, 0.999])


def test_disney_vs_fp64(cuda):
    """f and pdf at the kernel's own sampled direction against an FP64
    evaluation of the same formulas; the kernel is no further from FP64
    than the reference's own FP32 build is."""
    normal, wo, color, params, rnd4 = O.bxdf_inputs(1000, 1 << 16)
    wi, f, pdf, delta, _ = _run_bxdf(cuda, 3, normal, wo, color, params, rnd4[:, :2].copy())
    ok = pdf > 0
    f64, p64 = O.bxdf_eval_pdf(64, 3, normal, wo, color, params, wi.astype(np.float64))
    r_gpu = np.maximum(rel_err(f[ok], f64[ok], 1e-20).max(1), rel_err(pdf[ok], p64[ok], 1e-20))
    w32, f32, p32, _ = O.bxdf_sample(32, 3, normal, wo, color, params, rnd4[:, :2].copy())
    ok32 = p32 > 0
    f64b, p64b = O.bxdf_eval_pdf(64, 3, normal, wo, color, params, w32)
    r_ref = np.maximum(rel_err(f32[ok32], f64b[ok32], 1e-20).max(1), rel_err(p32[ok32], p64b[ok32], 1e-20))
    frac_gpu, frac_ref = np.mean(r_gpu > 1e-5), np.mean(r_ref > 1e-5)
    assert frac_gpu <= frac_ref + 0.005, (frac_gpu, frac_ref)
    assert np.median(r_gpu) < 1e-6


def test_disney_local_frame_vs_fp64(cuda):
    """With the shading frame exact (normal = +z, so world and local
    coordinates coincide), the kernel's Disney f and pdf at its own sampled
    direction are within 1e-5 relative of the FP64 evaluation of the same
    formulas for at least 99 % of the points; the rest are peaked GTR2 lobes
    (alpha down to 0.001) where one FP32 ulp in the half vector moves D by
    more."""
    normal, _, color, params, rnd4 = O.bxdf_inputs(7000, 1 << 16)
    normal[:] = (0.0, 0.0, 1.0)
    rng = np.random.default_rng(11)
    wo = rng.normal(size=(len(normal), 3))
    wo[:, 2] = np.abs(wo[:, 2]) + 1e-3
    wo = (wo / np.linalg.norm(wo, axis=1, keepdims=True)).astype(np.float32)
    wi, f, pdf, delta, _ = _run_bxdf(cuda, 3, normal, wo, color, params, rnd4[:, :2].copy())
    ok = pdf > 0
    f64, p64 = O.bxdf_eval_pdf(64, 3, normal, wo, color, params, wi.astype(np.float64))
    r = np.maximum(rel_err(f[ok], f64[ok], 1e-20).max(1), rel_err(pdf[ok], p64[ok], 1e-20))
    frac = np.mean(r < 1e-5)
    print(f"Disney, exact local frame: {frac:.4%} of {ok.sum()} sampled points within 1e-5 of FP64")
    assert frac > 0.99, (frac, np.quantile(r, [0.5, 0.99, 0.999]))


def test_bxdf_eval_kernel(cuda):
    import torch
    import srt_gb300 as S
    z = golden("bxdf")
    for name in ("disney", "disney_trans", "diffuse", "diffuse_transmission"):
        t, p = int(z[f"{name}_type"]), z[f"{name}_params"]
        n = len(p)
        d = {k: _t(v, cuda) for k, v in dict(normal=z["normal"], wo=z["wo"], color=z["color"], params=p,
                                              rnd=z["rnd4"][:, :2].copy(), wi=z["wi_rand"]).items()}
        f = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
        pdf = torch.zeros(n, dtype=torch.float32, device=cuda)
        S.bxdf_eval(t, d["normal"], d["wo"], d["color"], d["params"], d["rnd"], d["wi"], f, pdf)
        torch.cuda.synchronize()
        r = np.maximum(rel_err(f.cpu().numpy(), z[f"{name}_eval_f"], 1e-20).max(1),
                       rel_err(pdf.cpu().numpy(), z[f"{name}_eval_pdf"], 1e-20))
        assert np.mean(r < 1e-5) > 0.999, (name, np.quantile(r, [0.99, 0.999]))


def test_bxdf_generator_matches_oracle(cuda):
    import torch
    import srt_gb300 as S
    n, first = 5000, 777
    bufs = {"normal": (n, 3), "wo": (n, 3), "color": (n, 3), "params": (n, 12), "rnd": (n, 2), "wi": (n, 3),
            "f": (n, 3), "pdf": (n,)}
    t = {k: torch.zeros(v, dtype=torch.float32, device=cuda) for k, v in bufs.items()}
    S.bxdf_generate(first, t["normal"], t["wo"], t["color"], t["params"], t["rnd"], t["wi"], t["f"], t["pdf"])
    torch.cuda.synchronize()
    nn, wo, c, p, r4 = O.bxdf_inputs(first, n)
    np.testing.assert_array_equal(t["color"].cpu().numpy(), c)      # raw uniforms: exact
    np.testing.assert_array_equal(t["params"].cpu().numpy(), p)
    np.testing.assert_array_equal(t["rnd"].cpu().numpy(), r4[:, :2])
    np.testing.assert_allclose(t["normal"].cpu().numpy(), nn, atol=2e-6)
    np.testing.assert_allclose(t["wo"].cpu().numpy(), wo, atol=2e-6)


def _random_rays(n, lo, hi, seed, tmin=1e-3):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, np.full((n, 1), tmin, np.float32), d, np.full((n, 1), 1e16, np.float32)], 1)


def _check_hits(sc, osc, rays, cuda):
    import torch
    hits = torch.zeros((len(rays), 4), dtype=torch.float32, device=cuda)
    sc.trace_closest(_t(rays, cuda), hits)
    torch.cuda.synchronize()
    g = hits.cpu().numpy()
    o, edge = osc.trace_closest(rays)
    pg, po = g[:, 3].view(np.int32), o[:, 3].view(np.int32)
    safe = edge > 1e-4
    tie = (po >= 0) & (pg >= 0) & (np.abs(g[:, 0] - o[:, 0]) <= 1e-5 * np.abs(o[:, 0]))
    mismatch = (pg != po) & ~tie
    assert np.sum(mismatch & safe) == 0, np.sum(mismatch & safe)
    hit = (pg == po) & (po >= 0)
    rt = rel_err(g[hit, 0], o[hit, 0], 1e-6)
    assert np.quantile(rt, 0.999) < 1e-5 and rt.max() < 1e-2, (np.quantile(rt, 0.999), rt.max())
    assert np.quantile(np.abs(g[hit, 1:3] - o[hit, 1:3]), 0.999) < 1e-5
    return np.mean(mismatch)


def test_trace_cornell_vs_brute_force(cuda):
    import torch
    import srt_gb300 as S
    s = golden("scene")
    sa = scene_from_npz(s)
    sc = S.Scene(sa)
    osc = O.OracleScene(sa.desc())
    rays = _random_rays(20000, -0.99, 0.99, 4)
    frac = _check_hits(sc, osc, rays, cuda)
    print(f"Cornell: primitive-id mismatch rate {frac:.2e} (only rays within 1e-4 of an edge may differ)")
    # shadow rays toward random points: visibility must agree away from edges
    rays[:, 7] = np.random.default_rng(9).uniform(0.1, 3.0, len(rays)).astype(np.float32)
    vis = torch.zeros(len(rays), dtype=torch.int32, device=cuda)
    sc.trace_shadow(_t(rays, cuda), vis)
    torch.cuda.synchronize()
    ov = osc.trace_shadow(rays)
    _, edge = osc.trace_closest(rays)
    safe = edge > 1e-4
    assert np.all(vis.cpu().numpy()[safe] == ov[safe])


def test_trace_spheres_vs_oracle(cuda):
    import srt_gb300 as S
    sa = S.procedural("spheres", seed=3, n_spheres=6, subdiv=3)
    sc = S.Scene(sa)
    info = sc.info()
    assert info["num_triangles"] == 6 * 1280 + 2 + 8
    osc = O.OracleScene(sa.desc(), bvh=True)
    rays = _random_rays(30000, -12.0, 12.0, 5)
    frac = _check_hits(sc, osc, rays, cuda)
    print(f"spheres: primitive-id mismatch rate {frac:.2e} (only rays within 1e-4 of an edge may differ)")
    assert frac < 1e-3


def test_prim_to_instance(cuda):
    import srt_gb300 as S
    s = golden("scene")
    sa = scene_from_npz(s)
    sc = S.Scene(sa)
    base = 0
    for i, (mid, _) in enumerate(sa.instances):
        nf = len(sa.meshes[mid]["indices"])
        assert sc.prim_to_instance(base) == (i, 0)
        assert sc.prim_to_instance(base + nf - 1) == (i, nf - 1)
        base += nf
    with pytest.raises(S.SrtError):
        sc.prim_to_instance(base)
