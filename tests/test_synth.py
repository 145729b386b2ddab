"""CPU tests of the per-job observations of the batched and served workloads
(synth.job_tracks): every job its own array, whole baseline tracks,
float-representable coordinates inside the fill radius, reproducible."""
import numpy as np
import pytest

import synth

torch = pytest.importorskip("torch")


def test_job_tracks_shape_range_and_reproducibility():
    for N, n, seed in ((256, 10000, 1), (2048, 333333, 2), (512, 5000, 3)):
        uv, v = synth.job_tracks(N, n, seed)
        assert uv.shape == (n, 2) and v.shape == (n,)
        assert uv.dtype == torch.float64 and v.dtype == torch.complex64
        a = uv.numpy()
        assert np.array_equal(a, a.astype(np.float32).astype(np.float64))
        r = np.hypot(a[:, 0] - N / 2, a[:, 1] - N / 2)
        assert r.max() <= 0.9 * N / 2 * np.sqrt(2) + 1e-6
        assert np.abs(a - N / 2).max() <= 0.9 * N / 2 + 1e-3
        uv2, v2 = synth.job_tracks(N, n, seed)
        assert torch.equal(uv, uv2) and torch.equal(v, v2)


def test_jobs_have_their_own_arrays():
    """Two seeds give different antenna layouts (different tracks), and a
    job is made of whole tracks: consecutive samples of a baseline move by
    less than a cell."""
    a, _ = synth.job_tracks(1024, 2080 * 5, 11)
    b, _ = synth.job_tracks(1024, 2080 * 5, 12)
    assert not torch.equal(a, b)
    t = a.numpy().reshape(5, 2080, 2)
    step = np.abs(np.diff(t, axis=1)).max()
    assert step < 1.0
