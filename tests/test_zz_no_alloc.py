"""srt_film_metric_noalloc through the C ABI (GPU only).

This entry point is for callers that cannot allocate device memory when
they measure a film (a serving loop that reserved its whole HBM budget, or
code that must not let cudaMalloc synchronise the device mid-frame): its
scratch is a fixed array in device memory instead of a caller buffer.  It
must return what srt_film_metric returns with an allocated scratch, on
consecutive calls that reuse the same array, and refuse sizes beyond the
array.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(S, x, ref, type_, discard):
    out = C.c_float()
    S.check(S.lib().srt_film_metric_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(ref.data_ptr()), x.shape[0],
                                            type_, discard, C.byref(out), None))
    return out.value


def test_noalloc_metric_matches_allocating_entry_point(cuda):
    import torch
    import srt_gb300 as S
    rng = np.random.default_rng(123)
    # calls in a row on different films: each must not see the previous one's
    # state; the last case fills the array exactly (the error region and the
    # select state behind it must both fit at the limit)
    cases = [(1920 * 1080, S.METRIC_RELMSE, 0.1), (300001, S.METRIC_MSE, 2.5), (1 << 21, S.METRIC_SMAPE, 0.1)]
    for n, type_, discard in cases:
        ref = torch.from_numpy((rng.random((n, 4), dtype=np.float32) + 0.05)).to(cuda)
        x = torch.from_numpy((rng.random((n, 4), dtype=np.float32) * 2.0)).to(cuda)
        want = S.film_metric(x, ref, type_, discard)
        got = _noalloc(S, x, ref, type_, discard)
        assert np.isfinite(got)
        assert abs(got - want) <= 1e-6 * abs(want), (n, type_, got, want)


def test_noalloc_metric_rejects_oversize(cuda):
    import torch
    import srt_gb300 as S
    n = (1 << 21) + 1
    x = torch.zeros((n, 4), dtype=torch.float32, device=cuda)
    with pytest.raises(S.SrtError) as e:
        _noalloc(S, x, x, S.METRIC_MSE, 0.1)
    assert e.value.status == 1 and "2097152" in str(e.value)


def test_noalloc_metric_everything_discarded(cuda):
    """discard = 100 keeps no pixel: both entry points return NaN (the
    reference divides an empty sum by zero) without touching the array."""
    import torch
    import srt_gb300 as S
    x = torch.ones((1000, 4), dtype=torch.float32, device=cuda)
    assert np.isnan(S.film_metric(x, x, S.METRIC_MSE, 100.0))
    assert np.isnan(_noalloc(S, x, x, S.METRIC_MSE, 100.0))
    # and the array still serves a normal call afterwards (MSE over RGB)
    ref = x * 0.5
    assert abs(_noalloc(S, x, ref, S.METRIC_MSE, 0.0) - 0.25) < 1e-6
