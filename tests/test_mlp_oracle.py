"""The FP64 network oracle's gradient against central finite differences
(CPU): pins the oracle that the CUDA kernels' gradients are checked against."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    ws = [rng.normal(scale=np.sqrt(2.0 / w.shape[1]), size=w.shape) for w in M.split(np.zeros(M.PARAMS))]
    ws[-1][3:] = 0.0
    ws[-1] *= 0.1
    n = 64
    rec = np.zeros((n, 16))
    rec[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    rec[:, 3] = rng.uniform(0.05, 1, n)
    rec[:, 4:7] = rng.normal(size=(n, 3))
    rec[:, 8:11] = rng.normal(size=(n, 3))
    rec[:, 12:15] = rng.random((n, 3))
    x = M.encode(rec, [-1, -1, -1], [1, 1, 1])
    y = rng.uniform(0.1, 2.0, (n, 4))
    loss, grads = M.loss_and_grad(ws, x, y)
    # the loss's denominator is a stop-gradient: hold it at the base point
    p0 = M.predict(ws, x)
    den = p0 * p0 + 0.01
    eps = 1e-6
    for l in range(M.LAYERS):
        for _ in range(6):
            o = rng.integers(0, 3 if l == M.LAYERS - 1 else ws[l].shape[0])
            i = rng.integers(0, ws[l].shape[1])
            wp = [w.copy() for w in ws]
            wm = [w.copy() for w in ws]
            wp[l][o, i] += eps
            wm[l][o, i] -= eps
            fd = (M.loss_and_grad(wp, x, y, den)[0] - M.loss_and_grad(wm, x, y, den)[0]) / (2 * eps)
            assert abs(fd - grads[l][o, i]) <= 1e-6 + 1e-4 * abs(fd), (l, o, i, fd, grads[l][o, i])


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159], np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and abs(r[3] + 3.140625) < 1e-9
