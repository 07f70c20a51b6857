"""Radiance-cache network kernels against the FP64 oracle (GPU only).

The kernels round inputs, weights and activations to BF16 and accumulate
in FP32; the oracle evaluates the same network in FP64 on the BF16-rounded
weights.  Tolerances follow from BF16's 8-bit mantissa: outputs within
5 % (|log ratio| < 0.05) for 99 % of queries; weight gradients within 5 %
(cosine > 0.999) of an FP64 evaluation that rounds where the kernels round,
and cosine > 0.99 against the exact FP64 gradient.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

LO, HI = np.array([-2.0, -1.0, -3.0]), np.array([2.0, 3.0, 1.0])


def _records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 16), np.float32)
    r[:, 0:3] = rng.uniform(LO, HI, (n, 3))
    r[:, 3] = rng.uniform(0.05, 1.0, n)
    nn = rng.normal(size=(n, 3))
    r[:, 4:7] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    r[:, 8:11] = wo / np.linalg.norm(wo, axis=1, keepdims=True)
    r[:, 12:15] = rng.random((n, 3))
    return r


def _target(rec):
    p = rec[:, 0:3]
    base = 0.6 + 0.35 * np.sin(2.0 * p[:, 0:1]) * np.cos(1.5 * p[:, 1:2]) + 0.2 * rec[:, 12:15] * rec[:, 5:6] ** 2
    t = np.zeros((len(rec), 4), np.float32)
    t[:, :3] = np.maximum(base, 0.02)
    return t


def _mlp(S, seed=3):
    h = C.c_void_p()
    S.check(S.lib().srt_mlp_create(seed, C.byref(h)))
    lo = (C.c_float * 3)(*LO)
    hi = (C.c_float * 3)(*HI)
    S.check(S.lib().srt_mlp_set_box(h, lo, hi))
    return h


def _params(S, h):
    p = np.zeros(M.PARAMS, np.float32)
    S.check(S.lib().srt_mlp_get_params(h, p.ctypes.data_as(C.POINTER(C.c_float))))
    return p


def test_inference_matches_fp64(cuda):
    import torch
    import srt_gb300 as S
    h = _mlp(S)
    ws = [M.bf16(w) for w in M.split(_params(S, h))]
    rec = _records(5000, 1)
    out = torch.zeros((5000, 4), dtype=torch.float32, device=cuda)
    rec_d = torch.from_numpy(rec).to(cuda)  # held until the kernel has run
    S.check(S.lib().srt_mlp_infer(h, C.c_void_p(rec_d.data_ptr()), 5000, C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()[:, :3]
    want = M.predict(ws, M.encode(rec, LO, HI))
    d = np.abs(np.log(got) - np.log(want))
    assert np.quantile(d, 0.99) < 0.05, np.quantile(d, [0.5, 0.99, 1.0])
    S.lib().srt_mlp_destroy(h)


def test_gradient_matches_fp64(cuda):
    import torch
    import srt_gb300 as S
    h = _mlp(S, seed=5)
    ws = [M.bf16(w) for w in M.split(_params(S, h))]
    n = 4096
    rec = _records(n, 2)
    tgt = _target(rec)
    g = np.zeros(M.PARAMS, np.float32)
    loss = C.c_float()
    # device copies stay referenced across the call: a temporary's block would
    # be handed to the next upload before the kernels read it
    rec_d, tgt_d = torch.from_numpy(rec).to(cuda), torch.from_numpy(tgt).to(cuda)
    S.check(S.lib().srt_mlp_gradient(h, C.c_void_p(rec_d.data_ptr()), C.c_void_p(tgt_d.data_ptr()), n,
                                     g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss), None))
    x = M.encode(rec, LO, HI)
    ol, og = M.loss_and_grad(ws, x, tgt)                       # exact FP64
    el, eg = M.loss_and_grad(ws, x, tgt, emulate_bf16=True)    # FP64 with the kernels' BF16 roundings
    assert abs(loss.value - ol) < 0.05 * ol
    gpu = M.split(g)

    def cmp(a, b):
        cos = np.sum(a * b) / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
        return cos, np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)

    for l in range(M.LAYERS):
        cos, rel = cmp(gpu[l], eg[l])
        assert cos > 0.999 and rel < 0.05, ("bf16-emulating oracle", l, cos, rel)
        cos, rel = cmp(gpu[l], og[l])
        assert cos > 0.99, ("exact oracle", l, cos, rel)
    S.lib().srt_mlp_destroy(h)


def test_training_reduces_loss(cuda):
    import torch
    import srt_gb300 as S
    h = _mlp(S, seed=9)
    n = 1 << 14
    losses = []
    for step in range(400):
        rec = _records(n, 100 + step)
        tgt = _target(rec)
        loss = C.c_float()
        rec_d, tgt_d = torch.from_numpy(rec).to(cuda), torch.from_numpy(tgt).to(cuda)
        S.check(S.lib().srt_mlp_train_step(h, C.c_void_p(rec_d.data_ptr()), C.c_void_p(tgt_d.data_ptr()), n, 1e-2,
                                           C.byref(loss), None))
        losses.append(loss.value)
    assert np.mean(losses[-20:]) < 0.2 * np.mean(losses[:5]), (losses[:5], losses[-5:])
    # held-out queries: the trained network predicts the function
    rec = _records(4000, 7)
    out = torch.zeros((4000, 4), dtype=torch.float32, device=cuda)
    rec_d = torch.from_numpy(rec).to(cuda)
    S.check(S.lib().srt_mlp_infer(h, C.c_void_p(rec_d.data_ptr()), 4000, C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    rel = np.abs(out.cpu().numpy()[:, :3] - _target(rec)[:, :3]) / _target(rec)[:, :3]
    assert np.median(rel) < 0.1
    S.lib().srt_mlp_destroy(h)


def test_bounded_wait_reports_a_timeout_and_the_device_stays_usable(cuda):
    """The tensor-core kernels' waits on their mbarriers are bounded: a wait
    on a phase that nothing completes (a self-test kernel) gives up after its
    limit and comes back as SRT_ERR_TIMEOUT; the next calls work normally."""
    import ctypes as C
    import time
    import torch
    import srt_gb300 as S
    L = S.lib()
    t0 = time.perf_counter()
    assert L.srt_selftest_wait_timeout(2_000_000) == 4  # SRT_ERR_TIMEOUT after 2 ms
    assert time.perf_counter() - t0 >= 0.002
    assert "gave up" in L.srt_last_error().decode()
    assert L.srt_selftest_wait_timeout(10) == 1  # out of range
    # the context is intact: a network inference and a render still run
    mlp = C.c_void_p()
    S.check(L.srt_mlp_create(1, C.byref(mlp)))
    rec = torch.rand((1000, 16), device=cuda)
    out = torch.zeros((1000, 4), device=cuda)
    S.check(L.srt_mlp_infer(mlp, C.c_void_p(rec.data_ptr()), 1000, C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    L.srt_mlp_destroy(mlp)
