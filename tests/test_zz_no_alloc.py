"""gg_grid_device_noalloc: the allocation-free moving-window entry point.

It exists for callers that must not allocate device memory while they run --
a real-time ingest that reserves all of its GPU memory at start-up (an
allocation can block on the device or fail mid-observation), or a plugin in a
host framework that owns the device memory pool.  Its scratch is a fixed
array inside libgg.so.  These tests call it through the C ABI and compare its
grid with the context-based gg_grid_device and with the CPU oracle on two
calls in a row with different jobs (the shared scratch must be cleared
between calls), over the GCF kinds, grid types, layouts and tile-sorted
input it accepts; they check that device-side failures are readable after
the call (gg_read_flags with a null context) and that jobs beyond the fixed
scratch are refused.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

import gpugrid as gg
import oracle as O
import synth
from helpers import cell_err, planar_from_grid, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-6        # FP32 compensated accumulation, normwise, as for the other FP32 paths
CELL_TOL = 1e-6   # and per cell


def pairs(c):
    c = np.asarray(c).reshape(-1)
    return np.stack([c.real, c.imag], -1).astype(np.float64)


def _inputs(N, S, npts, seed, sort_tiles=False):
    uv, vals = synth.tracks(N, nant=32, ntime=300, npts=npts, seed=seed)
    if sort_tiles:   # grouped by 32-cell uv tile, ascending, as input_sorted requires
        order = synth.tile_sort(uv, N, 32, S)
        uv, vals = np.ascontiguousarray(uv[order]), np.ascontiguousarray(vals[order])
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    return uv, vals, gcf


def _grid_both(N, S, uv, vals, gcf, o, out_dtype):
    """(no-alloc grid, context grid), both planar (2, 1, N, N) float64"""
    d_uv, d_vals = torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda()
    d_gcf = torch.from_numpy(gcf.reshape(-1)).cuda()
    planar = o.layout == gg.LAYOUT_PLANAR
    res = []
    with gg.Context(0) as ctx:
        ref = torch.empty(N * N, dtype=out_dtype, device="cuda")
        ctx.grid(o, ref, d_uv, d_vals, d_gcf, N, S)
        torch.cuda.synchronize()
        assert ctx.read_flags() == [0, 0, 0, 0]
    out = torch.full((N * N,), float("nan"), dtype=out_dtype, device="cuda")
    job = gg.Context.make_job(out, d_uv, d_vals,
                              d_gcf if o.gcf_kind == gg.GCF_TABLE else None, N, S)
    gg.grid_device_noalloc(o, job)
    torch.cuda.synchronize()
    assert gg.noalloc_flags() == [0, 0, 0, 0]
    for t in (out, ref):
        host = torch.view_as_real(t).reshape(-1).cpu().numpy()
        res.append(planar_from_grid(host, 1, N, planar))
    return res


@pytest.mark.parametrize("gcf_kind,out,layout,input_sorted", [
    (gg.GCF_TABLE, "c64", gg.LAYOUT_INTERLEAVED, False),
    (gg.GCF_GAUSSIAN, "c64", gg.LAYOUT_INTERLEAVED, False),
    (gg.GCF_TABLE, "c128", gg.LAYOUT_PLANAR, False),
    (gg.GCF_TABLE, "c64", gg.LAYOUT_PLANAR, True),
])
def test_noalloc_matches_context_entry_point_and_oracle_twice(gcf_kind, out, layout,
                                                              input_sorted):
    assert torch.cuda.is_available(), "GPU test"
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=layout,
                   gcf_kind=gcf_kind, input_sorted=input_sorted)
    odt = torch.complex64 if out == "c64" else torch.complex128
    # two different jobs back to back; the second one is smaller on the grid
    # but denser, so stale scratch from the first would show up
    for N, S, npts, seed in ((1024, 8, 200000, 1), (512, 16, 150000, 2)):
        uv, vals, gcf = _inputs(N, S, npts, seed, sort_tiles=input_sorted)
        got, ctx_grid = _grid_both(N, S, uv, vals, gcf, o, odt)
        scale = np.abs(ctx_grid).max()
        assert scale > 0
        assert np.abs(got - ctx_grid).max() / scale <= TOL
        ref = O.grid_pz(uv, pairs(vals), pairs(gcf), N, S, nthreads=16)
        mag = O.grid_mag(uv, pairs(vals), pairs(gcf), N, S, nthreads=16)
        assert rel_err(got, ref) <= TOL
        assert cell_err(got, ref, mag)[0] <= CELL_TOL


def test_noalloc_dense_tile_merges_items():
    """One dense uv tile, cut into many work items: their partial sub-grids
    meet in the array's merge slots; per-cell error as for one item."""
    N, S, n = 64, 8, 1 << 18
    rng = np.random.default_rng(3)
    uv = synth.fr(rng.uniform(36, 60, size=(n, 2)))      # inside one 32-cell tile
    vals = (1.0 + 0.5 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))).astype(
        np.complex64)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED)
    for _ in range(2):
        got, ctx_grid = _grid_both(N, S, uv, vals, gcf, o, torch.complex64)
        ref = O.grid_pz(uv, pairs(vals), pairs(gcf), N, S, nthreads=16)
        mag = O.grid_mag(uv, pairs(vals), pairs(gcf), N, S, nthreads=16)
        assert rel_err(got, ref) <= TOL
        assert cell_err(got, ref, mag)[0] <= CELL_TOL


def test_noalloc_reports_device_flags():
    """Device-side failures are read after the call with gg_read_flags on a
    null context: input declared tile-sorted that is not (the call grids
    nothing), and a flag raised from the host (a one-thread kernel behind
    the gridding, standing in for an expired bounded wait).  The next call
    clears them."""
    assert torch.cuda.is_available(), "GPU test"
    N, S = 256, 8
    uv, vals, gcf = _inputs(N, S, 20000, 4)
    rng = np.random.default_rng(4)
    perm = rng.permutation(len(uv))
    d_uv = torch.from_numpy(np.ascontiguousarray(uv[perm])).cuda()
    d_vals = torch.from_numpy(np.ascontiguousarray(vals[perm])).cuda()
    d_gcf = torch.from_numpy(gcf.reshape(-1)).cuda()
    out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    job = gg.Context.make_job(out, d_uv, d_vals, d_gcf, N, S)
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, input_sorted=True)
    gg.grid_device_noalloc(o, job)
    f = gg.noalloc_flags()
    assert f[2] == 1 and f[1] == 0, f
    assert torch.count_nonzero(out).item() == 0     # nothing gridded
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED)
    gg.inject_device_flags(gg.DEVFLAG_TIMEOUT, 1)
    try:
        gg.grid_device_noalloc(o, job)
        f = gg.noalloc_flags()
    finally:
        gg.inject_device_flags(0, 0)
    assert f == [0, 1, 0, 0], f
    gg.grid_device_noalloc(o, job)
    assert gg.noalloc_flags() == [0, 0, 0, 0]
    assert torch.count_nonzero(out).item() > 0


def test_noalloc_rejects_jobs_beyond_its_scratch():
    assert torch.cuda.is_available(), "GPU test"
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED)
    uv, vals, gcf = _inputs(512, 8, (1 << 18) + 1, 3)
    d_uv, d_vals = torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda()
    d_gcf = torch.from_numpy(gcf.reshape(-1)).cuda()
    out = torch.empty(512 * 512, dtype=torch.complex64, device="cuda")

    def refused(job, opts=o):
        with pytest.raises(gg.GridError) as e:
            gg.grid_device_noalloc(opts, job)
        assert e.value.code == gg.ERR_ARG
        return str(e.value)

    assert "exceeds" in refused(gg.Context.make_job(out, d_uv, d_vals, d_gcf, 512, 8))
    assert "exceeds" in refused(gg.Context.make_job(out, d_uv[:1000], d_vals[:1000], d_gcf,
                                                    8192, 8))
    # oversample 16 with support 32: 16*16*32*32 = 262144 taps > 65536
    big = torch.zeros(16 * 16 * 32 * 32, dtype=torch.complex64, device="cuda")
    o16 = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, oversample=16)
    assert "exceeds" in refused(gg.Context.make_job(out, d_uv[:1000], d_vals[:1000], big,
                                                    512, 32), o16)
    assert "polarisation" in refused(gg.Context.make_job(out, d_uv[:1000], d_vals[:1000],
                                                         d_gcf, 512, 8),
                                     gg.Options(mode=gg.MODE_WINDOW, polarizations=2))
