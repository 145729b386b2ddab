"""gg_grid_device_noalloc: the allocation-free moving-window entry point.

It exists for callers that must not allocate device memory while they run --
a real-time ingest that reserves all of its GPU memory at start-up (an
allocation can block on the device or fail mid-observation), or a plugin in a
host framework that owns the device memory pool.  Its scratch is a fixed
array inside libgg.so.  These tests call it through the C ABI and compare its
grid with the context-based gg_grid_device on two calls in a row with
different jobs (the shared scratch must be cleared between calls), and check
that jobs larger than the fixed scratch are refused.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import gpugrid as gg
import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-6  # FP32 compensated accumulation, as for the other FP32 paths


def _entry():
    f = gg.LIB.gg_grid_device_noalloc
    f.argtypes = [ctypes.POINTER(gg.gg_options), ctypes.POINTER(gg.gg_job),
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _inputs(N, S, npts, seed):
    uv, vals = synth.tracks(N, nant=32, ntime=300, npts=npts, seed=seed)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    return (torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
            torch.from_numpy(gcf.reshape(-1)).cuda())


def test_noalloc_matches_context_entry_point_twice():
    assert torch.cuda.is_available(), "GPU test"
    f = _entry()
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED)
    stream = torch.cuda.current_stream()
    with gg.Context(0) as ctx:
        # two different jobs back to back; the second one is smaller on the
        # grid but denser, so stale scratch from the first would show up
        for N, S, npts, seed in ((1024, 8, 200000, 1), (512, 16, 150000, 2)):
            d_uv, d_vals, d_gcf = _inputs(N, S, npts, seed)
            ref = torch.empty(N * N, dtype=torch.complex64, device="cuda")
            ctx.grid(o, ref, d_uv, d_vals, d_gcf, N, S)
            out = torch.full((N * N,), float("nan"), dtype=torch.complex64, device="cuda")
            job = gg.Context.make_job(out, d_uv, d_vals, d_gcf, N, S)
            st = f(ctypes.byref(o.c()), ctypes.byref(job),
                   ctypes.c_void_p(stream.cuda_stream))
            assert st == gg.OK, gg.LIB.gg_last_error().decode()
            torch.cuda.synchronize()
            scale = ref.abs().max().item()
            assert scale > 0
            err = (out - ref).abs().max().item() / scale
            assert err <= TOL, err


def test_noalloc_rejects_jobs_beyond_its_scratch():
    assert torch.cuda.is_available(), "GPU test"
    f = _entry()
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED)
    d_uv, d_vals, d_gcf = _inputs(512, 8, (1 << 18) + 1, 3)
    out = torch.empty(512 * 512, dtype=torch.complex64, device="cuda")
    job = gg.Context.make_job(out, d_uv, d_vals, d_gcf, 512, 8)
    assert f(ctypes.byref(o.c()), ctypes.byref(job), None) == gg.ERR_ARG
    assert "exceeds" in gg.LIB.gg_last_error().decode()
    job = gg.Context.make_job(out, d_uv[:1000], d_vals[:1000], d_gcf, 8192, 8)
    assert f(ctypes.byref(o.c()), ctypes.byref(job), None) == gg.ERR_ARG
    assert "exceeds" in gg.LIB.gg_last_error().decode()
