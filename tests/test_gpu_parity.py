"""GPU parity of the CUDA gridder against the CPU oracle (gridCPU_pz
restatement pinned to the reference's own output) -- all calls go through
the C ABI of libgg.so.

Tolerances, two metrics:
  normwise  max |gpu - oracle| / max |oracle| over the grid
  per cell  max over cells of |gpu - oracle| / sum |v| |w| at that cell (the
            oracle's magnitude sum of the cell's additions, O.grid_mag): the
            forward error of each cell's sum, the quantity a summation error
            bound is stated in; unlike the normwise figure it is not diluted
            by the largest cells of the grid (the reference's own check,
            grid.cu:495-500, is per cell too, absolute 1e-6)

                                                        normwise  per cell
  FP64 values, complex128 grid .......................... 1e-12    1e-12
  FP32 values, compensated (two-sum hi/lo) accumulation ... 1e-6     CELL_TOL
  FP32 values, plain FP32 accumulation .................... 2e-6     CELL_TOL
  on-the-fly Gaussian GCF (FP32 expf vs FP64 table) ....... 1e-6     as its
                                                                    accumulation
Index work (cell and oversample index, DEBUG1 footprints, bookmarks) is
compared bit-exactly.
"""
import ctypes

import numpy as np
import pytest

import gpugrid as gg
import oracle as O
import synth
from helpers import (GOLDEN_CASES, cell_err, load_golden, planar_from_grid, rel_err,
                     to_complex)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = {"zz": 1e-12, "zc": 1e-6, "cc": 2e-6, "cc_comp": 1e-6}
# per-cell forward error bounds (units of u = 2^-24 = 5.96e-8): compensated
# sums carry the error of one short register run (at most 32 records) plus a
# few roundings -- into the FP32 grid, and of the few partial sums a cell
# receives from neighbouring tiles; plain FP32 sums grow with the number of
# terms of a cell
CELL_TOL = {"zz": 1e-12, "zc": 1e-6, "cc_comp": 1e-6, "cc": 1e-5}
MODES = {"scatter": gg.MODE_SCATTER, "gather": gg.MODE_GATHER, "window": gg.MODE_WINDOW}


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gg.Context(0)
    yield c
    c.close()


def run(ctx, opts, uv, vals, gcf, N, S, prec, uv_dtype=np.float64, stream=None):
    """Grid on the device; returns (planar float64 grid (2,P,N,N), flags)."""
    vdt = np.complex128 if prec == "zz" else np.complex64
    odt = torch.complex64 if prec.startswith("cc") else torch.complex128
    P = opts.polarizations
    d_uv = torch.from_numpy(np.ascontiguousarray(uv, uv_dtype)).cuda()
    d_vals = torch.from_numpy(np.ascontiguousarray(vals, vdt)).cuda()
    d_gcf = (torch.from_numpy(np.ascontiguousarray(gcf, vdt).reshape(-1)).cuda()
             if gcf is not None else None)
    out = torch.full((P * N * N,), float("nan"), dtype=odt, device="cuda")
    ctx.grid(opts, out, d_uv, d_vals, d_gcf, N, S)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    planar = opts.layout == gg.LAYOUT_PLANAR or (
        opts.layout == gg.LAYOUT_REFERENCE and opts.mode == gg.MODE_WINDOW)
    host = torch.view_as_real(out).reshape(-1).cpu().numpy()
    return planar_from_grid(host, P, N, planar), flags


def oracle_for(uv, vals, gcf, N, S, P=1, G=8, debug1=False):
    """oracle on exactly the values the GPU saw (vals/gcf complex arrays)"""
    return O.grid_pz(uv, to_pairs(vals), to_pairs(gcf), N, S, pols=P, gcf_grid=G,
                     debug1=debug1, nthreads=8)


def to_pairs(c):
    c = np.asarray(c).reshape(-1)
    return np.stack([c.real, c.imag], -1).astype(np.float64)


def check(out, prec, uv, vals, gcf, N, S, P=1, G=8, ref=None, gcfinx=None, norm_tol=None,
          cell_tol=None):
    """Both metrics of out (planar (2,P,N,N)) against the oracle on exactly
    the GPU's inputs (vals/gcf complex arrays; gcf may be a table stack with
    gcfinx); returns (normwise, per-cell max, per-cell rms)."""
    if ref is None:
        ref = oracle_for(uv, vals, gcf, N, S, P=P, G=G)
    mag = O.grid_mag(uv, to_pairs(vals), to_pairs(gcf), N, S, pols=P, gcf_grid=G,
                     gcfinx=gcfinx, nthreads=8)
    ne = rel_err(out, ref)
    cmax, crms = cell_err(out, ref, mag)
    nt = TOL[prec] if norm_tol is None else norm_tol
    ct = CELL_TOL[prec] if cell_tol is None else cell_tol
    assert ne <= nt and cmax <= ct, dict(prec=prec, normwise=ne, cell_max=cmax, cell_rms=crms)
    return ne, cmax, crms


def opts_for(mode, prec, **kw):
    acc = gg.ACC_COMPENSATED if prec in ("zc", "cc_comp") else gg.ACC_PLAIN
    return gg.Options(mode=MODES[mode], accum=acc, **kw)


# ---------------------------------------------------------------------------
# golden fixtures (the reference's own output) -- every method and precision
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["zz", "zc", "cc", "cc_comp"])
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if not c.startswith("debug1")])
def test_golden(ctx, name, mode, prec):
    g = load_golden(name)
    N, S, P = g["N"], g["S"], g["P"]
    vals = to_complex(g["vals"])
    gcf = to_complex(g["gcf"])
    if prec != "zz":
        vals = vals.astype(np.complex64)
        gcf = gcf.astype(np.complex64)
    out, flags = run(ctx, opts_for(mode, prec, polarizations=P), g["uv"], vals, gcf, N, S, prec)
    assert flags == [0, 0, 0, 0]
    if prec == "zz":
        assert rel_err(out, g["out"]) <= TOL["zz"]
    check(out, prec, g["uv"], vals, gcf, N, S, P=P)


@pytest.mark.parametrize("prec", ["zz", "cc_comp", "cc"])
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_debug1_footprint_bit_exact(ctx, mode, prec):
    """DEBUG1 (Defines.h:78): every tap adds (1, visibility index); the grid
    holds hit counts and index sums, exact integers in FP32 and FP64."""
    g = load_golden("debug1_n64_s8")
    N, S = g["N"], g["S"]
    o = opts_for(mode, prec, gcf_kind=gg.GCF_COUNT)
    vals = np.zeros(len(g["uv"]), np.complex128)
    out, flags = run(ctx, o, g["uv"], vals, None, N, S, prec)
    assert flags == [0, 0, 0, 0]
    assert np.array_equal(out, g["out"])


# ---------------------------------------------------------------------------
# index step and binning (bit-exact)
# ---------------------------------------------------------------------------
def test_vis2ints_bit_exact_fp64(ctx):
    rng = np.random.default_rng(7)
    uv = rng.uniform(-40, 9000, size=(200000, 2))
    uv[:100000] = uv[:100000].astype(np.float32)  # half float-representable
    k = np.arange(1, 2001, dtype=np.float64)
    uv[-2000:, 0] = k - 1e-9                           # just below integers
    uv[-2000:, 1] = k + 1e-9
    d = torch.from_numpy(uv).cuda()
    got = gg.vis2ints(d).cpu().numpy()
    assert np.array_equal(got, O.vis2ints(uv))


def test_vis2ints_bit_exact_fp32(ctx):
    rng = np.random.default_rng(8)
    uv32 = rng.uniform(-100, 30000, size=(100000, 2)).astype(np.float32)
    got = gg.vis2ints(torch.from_numpy(uv32).cuda()).cpu().numpy()
    assert np.array_equal(got, O.vis2ints(uv32.astype(np.float64)))


def test_vis2ints_bit_exact_near_zero_and_half(ctx):
    """The FP32 index step where u - floorf(u) rounds (-1/2 < u < 0) and
    around it: values on both sides of -1/2, -1/4, -1/8, 0 and -1, tiny
    negatives whose 1 + u rounds to 1 (oversample index G), negative
    multiples of 1/G and signed zeros, as float and as float-representable
    double coordinates, bit-exact with the oracle."""
    rng = np.random.default_rng(12)
    f32 = np.float32
    special = [0.0, -0.0, -1e-30, -1e-10, -2.0 ** -25, -2.0 ** -24, -0.5, -1.0, -1.5, 0.5,
               -0.125, -0.375, -0.625, -0.875, -0.25, -2.0 ** -149 * 1e30]
    near = []
    for x in (-0.5, -0.25, -0.125, -1.0, -2.0, 0.0, 0.125):
        v = f32(x)
        for _ in range(4):
            v = np.nextafter(v, f32(-np.inf))
            near.append(v)
        v = f32(x)
        for _ in range(4):
            v = np.nextafter(v, f32(np.inf))
            near.append(v)
    dense = rng.uniform(-1.0, 0.0, 100000).astype(f32)
    mult = -(np.arange(1, 800, dtype=f32) / f32(8)) + rng.choice([-1, 0, 1], 799).astype(f32) * f32(2.0 ** -26)
    vals = np.concatenate([np.array(special, f32), np.array(near, f32), dense, mult.astype(f32)])
    uv32 = np.stack([vals, vals[::-1]], -1).astype(f32)
    ref = O.vis2ints(uv32.astype(np.float64))
    got32 = gg.vis2ints(torch.from_numpy(np.ascontiguousarray(uv32)).cuda()).cpu().numpy()
    assert np.array_equal(got32, ref)
    got64 = gg.vis2ints(torch.from_numpy(uv32.astype(np.float64)).cuda()).cpu().numpy()
    assert np.array_equal(got64, ref)


@pytest.mark.parametrize("T", [8, 32])
@pytest.mark.parametrize("input_sorted", [False, True])
def test_bin_bookmarks(ctx, input_sorted, T):
    N, S = 512, 8
    uv, _ = synth.uniform(30000, 0, N, seed=9)
    if input_sorted:
        uv = uv[synth.tile_sort(uv, N, T)]
    o = gg.Options(tile=T, input_sorted=input_sorted)
    bm, order = ctx.bin(o, torch.from_numpy(uv).cuda(), N, S)
    bm, order = bm.cpu().numpy(), order.cpu().numpy()
    pk = O.vis2ints(uv)
    tile = (pk[:, 1] // 8 // T) * (N // T) + pk[:, 0] // 8 // T
    srt = np.argsort(tile, kind="stable")
    expect = O.set_bookmarks(pk[srt], T, N // T)
    assert np.array_equal(bm, expect)
    kept = bm[-1]
    assert kept == len(uv)
    assert np.array_equal(np.sort(order[:kept]), np.arange(len(uv)))
    assert np.array_equal(tile[order[:kept]], np.sort(tile))
    if input_sorted:
        assert np.array_equal(order[:kept], np.arange(len(uv)))
    assert ctx.read_flags() == [0, 0, 0, 0]


def test_unsorted_input_detected(ctx):
    N, S = 256, 8
    uv, vals = synth.uniform(5000, 0, N, seed=10)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    out = np.zeros(gg.padded_size(N, S), np.complex64)
    o = gg.Options(mode=gg.MODE_WINDOW, input_sorted=True)
    with pytest.raises(gg.GridError) as e:
        gg.grid_host(o, out, uv.astype(np.float32).view(np.complex64).reshape(-1).copy(),
                     vals, len(uv), N, gcf, S)
    assert e.value.code == gg.ERR_UNSORTED


@pytest.mark.parametrize("mode", ["window", "gather"])
def test_unsorted_flag_does_not_block_later_calls(ctx, mode):
    """Device entry point: a call whose declared-sorted input is unsorted
    raises the (sticky) unsorted flag and grids nothing; the next call on the
    same context, made before the flags are read, still grids in full."""
    N, S = 256, 8
    uv, vals = synth.uniform(5000, 8, N - 8, seed=11)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    d_uv, d_v = torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda()
    d_g = torch.from_numpy(gcf.reshape(-1)).cuda()
    out = torch.full((N * N,), float("nan"), dtype=torch.complex64, device="cuda")
    layout = gg.LAYOUT_INTERLEAVED
    ctx.grid(gg.Options(mode=MODES[mode], input_sorted=True, layout=layout),
             out, d_uv, d_v, d_g, N, S)
    ctx.grid(gg.Options(mode=MODES[mode], accum=gg.ACC_COMPENSATED, layout=layout),
             out, d_uv, d_v, d_g, N, S)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    assert flags[2] == 1 and flags[1] == 0  # unsorted seen, no wait timed out
    host = torch.view_as_real(out).reshape(-1).cpu().numpy()
    check(planar_from_grid(host, 1, N, False), "cc_comp", uv, vals, gcf, N, S)


def test_out_of_table_index_dropped_and_counted(ctx):
    """u right below an integer is not float-representable: the CPU gridder's
    oversample index becomes -1 (outside its table); the GPU path drops the
    visibility and counts it instead of reading outside the table."""
    N, S = 64, 8
    uv = np.array([[20.5, 20.5], [30.0 - 1e-9, 30.25], [40.5, 40.5]])
    vals = np.ones(3, np.complex128)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    for mode in MODES:
        out, flags = run(ctx, opts_for(mode, "zz"), uv, vals, gcf, N, S, "zz")
        assert flags[0] == 1
        ref = oracle_for(uv[[0, 2]], vals[[0, 2]], gcf, N, S)
        assert rel_err(out, ref) <= 1e-12


# ---------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_empty_and_offgrid_inputs_give_zero_grid(ctx, mode):
    N, S = 96, 8
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    for uv in (np.zeros((0, 2)), np.array([[-10.0, 5.0], [200.0, 3.0], [5.0, 104.5]])):
        vals = np.ones(len(uv), np.complex64)
        out, flags = run(ctx, opts_for(mode, "cc_comp"), uv, vals, gcf, N, S, "cc_comp")
        assert flags == [0, 0, 0, 0]
        assert np.array_equal(out, np.zeros_like(out))


@pytest.mark.parametrize("S", [4, 8, 16, 32])
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_supports_and_ragged_grid(ctx, mode, S):
    N = 100  # not a multiple of the 32-cell tile
    uv, vals = synth.uniform(3000, -S, N + S, seed=S)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    out, flags = run(ctx, opts_for(mode, "cc_comp"), uv, vals, gcf, N, S, "cc_comp")
    assert flags == [0, 0, 0, 0]
    check(out, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_corners_and_single_visibility(ctx, mode):
    N, S = 64, 16
    uv = np.array([[0.0, 0.0], [63.875, 63.875], [0.5, 63.5], [63.5, 0.25], [31.0, 32.0]])
    vals = np.array([1 + 2j, -3 + 1j, 0.5 - 0.5j, 2j, 1], np.complex128)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    out, _ = run(ctx, opts_for(mode, "zz"), uv, vals, gcf, N, S, "zz")
    assert rel_err(out, oracle_for(uv, vals, gcf, N, S)) <= 1e-12
    for k in range(len(uv)):
        out, _ = run(ctx, opts_for(mode, "zz"), uv[k:k + 1], vals[k:k + 1], gcf, N, S, "zz")
        assert rel_err(out, oracle_for(uv[k:k + 1], vals[k:k + 1], gcf, N, S)) <= 1e-12


@pytest.mark.parametrize("G", [1, 4, 16])
def test_other_oversampling(ctx, G):
    N, S = 128, 8
    uv, vals = synth.uniform(4000, 0, N, seed=G)
    g1 = synth.gaussian_gcf_1d(S, oversample=G)
    gcf = synth.gcf_table(g1)
    for mode in MODES:
        out, _ = run(ctx, opts_for(mode, "zz", oversample=G), uv,
                     vals.astype(np.complex128), gcf, N, S, "zz")
        assert rel_err(out, oracle_for(uv, vals, gcf, N, S, G=G)) <= 1e-12


@pytest.mark.parametrize("layout", [gg.LAYOUT_INTERLEAVED, gg.LAYOUT_PLANAR])
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_layouts_and_float_coordinates(ctx, mode, layout):
    N, S = 128, 8
    uv, vals = synth.uniform(5000, 0, N, seed=11)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    o = opts_for(mode, "cc_comp", layout=layout)
    out, _ = run(ctx, o, uv, vals, gcf, N, S, "cc_comp", uv_dtype=np.float32)
    check(out, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_gaussian_on_the_fly(ctx, mode):
    """COMPUTE_GCF: the GPU evaluates the separable Gaussian in FP32; the
    oracle gets the FP64 table of the same function."""
    for N, S in ((128, 8), (128, 32)):
        uv, vals = synth.uniform(6000, 0, N, seed=S)
        gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
        o = opts_for(mode, "cc_comp", gcf_kind=gg.GCF_GAUSSIAN)
        out, _ = run(ctx, o, uv, vals, None, N, S, "cc_comp")
        check(out, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_output_is_overwritten_not_accumulated(ctx, mode):
    N, S = 64, 8
    uv, vals = synth.uniform(500, 0, N, seed=12)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    a, _ = run(ctx, opts_for(mode, "cc"), uv, vals, gcf, N, S, "cc")
    b, _ = run(ctx, opts_for(mode, "cc"), uv, vals, gcf, N, S, "cc")
    assert np.isfinite(a).all() and np.allclose(a, b, rtol=0, atol=1e-6 * np.abs(a).max())


# ---------------------------------------------------------------------------
# batches of jobs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_batch_equals_single_jobs(ctx, mode):
    rng = np.random.default_rng(13)
    specs = [(64, 8, 300), (256, 16, 5000), (96, 8, 0), (128, 16, 2000), (512, 8, 20000)]
    o = opts_for(mode, "cc_comp")
    jobs, keep, inputs = [], [], []
    for k, (N, S, n) in enumerate(specs):
        uv, vals = synth.uniform(n, -S, N + S, seed=100 + k)
        gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(),
             torch.full((N * N,), float("nan"), dtype=torch.complex64, device="cuda")]
        keep.append(d)
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S, npts=n))
        inputs.append((uv, vals, gcf))
    ctx.grid_batch(o, jobs)
    torch.cuda.synchronize()
    assert ctx.read_flags() == [0, 0, 0, 0]
    for (N, S, n), d, (uv, vals, gcf) in zip(specs, keep, inputs):
        host = torch.view_as_real(d[3]).reshape(-1).cpu().numpy()
        out = planar_from_grid(host, 1, N, mode == "window")
        check(out, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("accum,autotune", [("cc_comp", False), ("cc", False),
                                            ("cc_comp", True)])
def test_batch_of_track_jobs_matches_oracle(ctx, accum, autotune):
    """Batched moving-window gridding of dense uv-track jobs (whole baseline
    tracks at 2080 samples over +-4 h, several grid sides and both supports,
    one job overfilling its grid so that edge tiles hold clamped mains):
    every job against the oracle."""
    rng = np.random.default_rng(31)
    o = opts_for("window", accum, layout=gg.LAYOUT_INTERLEAVED, autotune=autotune)
    if autotune:
        gg.autotune_clear()
    specs = [(256, 8, 1.0), (256, 16, 0.9), (512, 8, 0.9), (512, 16, 1.05),
             (1024, 8, 0.9), (1024, 16, 0.9), (128, 16, 1.2), (512, 8, 0.6)]
    jobs, keep, inputs = [], [], []
    for k, (N, S, fill) in enumerate(specs):
        uv, vals = synth.tracks(N, nant=24, ntime=2080, npts=None, fill=fill, seed=300 + k)
        n = int(rng.integers(20000, len(uv)))
        off = int(rng.integers(0, len(uv) - n + 1))
        uv, vals = np.ascontiguousarray(uv[off:off + n]), np.ascontiguousarray(vals[off:off + n])
        gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(),
             torch.full((N * N,), float("nan"), dtype=torch.complex64, device="cuda")]
        keep.append(d)
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S))
        inputs.append((uv, vals, gcf, oracle_for(uv, vals, gcf, N, S)))
    for rep in range(2):  # the second launch reuses the workspace (and the tuning)
        ctx.grid_batch(o, jobs)
        torch.cuda.synchronize()
        assert ctx.read_flags() == [0, 0, 0, 0]
        for (N, S, _), d, (uv, vals, gcf, ref) in zip(specs, keep, inputs):
            host = torch.view_as_real(d[3]).reshape(-1).cpu().numpy()
            check(planar_from_grid(host, 1, N, False), accum, uv, vals, gcf, N, S, ref=ref)
        if autotune:
            report = gg.autotune_report()
            if rep == 0:
                first = report
            # one entry per support class, chosen once
            assert len(report.splitlines()) == 2 and report == first
            assert "support 8 " in report and "support 16 " in report


@pytest.mark.parametrize("mode,prec", [("scatter", "cc_comp"), ("window", "cc_comp"),
                                       ("window", "cc"), ("window", "zz")])
def test_per_visibility_gcf_tables(ctx, mode, prec):
    """A table per visibility (w-plane / baseline GCFs, the reference's
    vis.gcfinx): two jobs in one batch with 3 and 5 tables (one complex),
    dense tracks, indices outside the stack dropped and counted; against the
    oracle's per-visibility restatement."""
    vdt = np.complex128 if prec == "zz" else np.complex64
    o = opts_for(mode, prec, layout=gg.LAYOUT_INTERLEAVED)
    keep, jobs, refs, dropped = [], [], [], 0
    for k, (N, S, ntab) in enumerate([(256, 8, 3), (512, 16, 5)]):
        uv, vals = synth.tracks(N, nant=16, ntime=800, npts=None, seed=400 + k,
                                vals_dtype=vdt)
        rng = np.random.default_rng(500 + k)
        idx = rng.integers(0, ntab, len(uv)).astype(np.int32)
        idx[::211] = ntab          # outside the stack
        dropped += int((idx == ntab).sum())
        tabs = [synth.gcf_table(synth.gaussian_gcf_1d(S, sigma=S / 4 + 0.3 * t)).astype(vdt)
                for t in range(ntab)]
        tabs[1] = (tabs[1] * np.exp(0.9j)).astype(vdt)
        stack = np.concatenate([t.reshape(-1) for t in tabs])
        odt = torch.complex128 if prec == "zz" else torch.complex64
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(stack).cuda(),
             torch.full((N * N,), float("nan"), dtype=odt, device="cuda"),
             torch.from_numpy(idx).cuda()]
        keep.append(d)
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S, gcf_index=d[4],
                                        n_gcf=ntab))
        refs.append((N, S, uv, vals, stack, idx,
                     O.grid_pz_gcfinx(uv, vals, idx, stack, N, S, nthreads=8)))
    ctx.grid_batch(o, jobs)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    assert flags[0] == dropped and flags[1:] == [0, 0, 0]
    for (N, S, uv, vals, stack, idx, ref), d in zip(refs, keep):
        host = torch.view_as_real(d[3]).reshape(-1).cpu().numpy()
        check(planar_from_grid(host, 1, N, False), prec, uv, vals, stack, N, S, ref=ref,
              gcfinx=idx)


@pytest.mark.parametrize("imag", [0.0, 1e-3])
def test_real_and_nearly_real_tables(ctx, imag):
    """The moving window takes a real-factor path when a table has no
    imaginary part (detected on the device); a table with a single small
    imaginary entry must take the complex path.  Both against the oracle."""
    N, S = 512, 16
    uv, vals = synth.tracks(N, nant=16, ntime=2000, npts=None, seed=77)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    gcf[27, 7, 9] += np.complex64(1j * imag)
    o = opts_for("window", "cc_comp", layout=gg.LAYOUT_INTERLEAVED)
    got, flags = run(ctx, o, uv, vals, gcf, N, S, "cc_comp")
    assert flags == [0, 0, 0, 0]
    check(got, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("prec", ["cc_comp", "zz"])
@pytest.mark.parametrize("mode", ["scatter", "window"])
def test_compute_gcf_phase_factor(ctx, prec, mode):
    """GG_GCF_WPHASE, the reference scatter kernel's COMPUTE_GCF factor
    (grid_gpu.cu:103-108, 137-147), against its oracle restatement; any
    requested method grids it by scatter.  FP32 sine/cosine of the phase on
    the device vs libm on the host: 1e-5."""
    S, N = 16, 256
    uv, vals = synth.uniform(20000, 2, N - 2, seed=91,
                             vals_dtype=np.complex128 if prec == "zz" else np.complex64)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    gcf.reshape(-1)[S * (S - 1) // 2 - 1] = 0.4 + 0.9j   # (T, w)
    gcf = gcf.astype(np.complex128 if prec == "zz" else np.complex64)
    o = opts_for(mode, prec, layout=gg.LAYOUT_INTERLEAVED, gcf_kind=gg.GCF_WPHASE)
    got, flags = run(ctx, o, uv, vals, gcf, N, S, prec)
    assert flags == [0, 0, 0, 0]
    want = O.grid_pz_wphase(uv, to_pairs(vals), to_pairs(gcf), N, S, nthreads=8)
    assert rel_err(got, want) <= 1e-5
    mag = O.grid_mag(uv, to_pairs(vals), to_pairs(gcf), N, S, wphase=True, nthreads=8)
    assert cell_err(got, want, mag)[0] <= 1e-5


def test_compute_gcf_dropin_host_entry(ctx):
    """The drop-in entry with COMPUTE_GCF set globally (as -D__COMPUTE_GCF
    does through grid_gpu.cuh): padded output, reference semantics."""
    S, N = 8, 128
    uv, vals = synth.uniform(5000, 2, N - 2, seed=92, vals_dtype=np.complex128)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    gcf.reshape(-1)[S * (S - 1) // 2 - 1] = 1.5 + 0.25j
    gg.set_global_options(gg.Options(gcf_kind=gg.GCF_WPHASE))
    try:
        out = np.zeros(gg.padded_size(N, S), np.complex128)
        in_ = np.ascontiguousarray(uv[:, 0] + 1j * uv[:, 1])
        gg.gridGPU(out, in_, vals, len(uv), N, np.ascontiguousarray(gcf.reshape(-1)), S)
    finally:
        gg.set_global_options(gg.Options())
    h = gg.grid_head(N, S)
    grid = out[h:h + N * N].reshape(N, N)
    want = O.grid_pz_wphase(uv, to_pairs(vals), to_pairs(gcf), N, S)
    got = np.stack([grid.real, grid.imag]).reshape(2, 1, N, N)
    assert rel_err(got, want) <= 1e-5


def test_per_visibility_gcf_rejected_by_gather(ctx):
    N, S = 64, 8
    d = [torch.zeros((10, 2), dtype=torch.float64, device="cuda"),
         torch.zeros(10, dtype=torch.complex64, device="cuda"),
         torch.zeros(64 * S * S * 2, dtype=torch.complex64, device="cuda"),
         torch.zeros(N * N, dtype=torch.complex64, device="cuda"),
         torch.zeros(10, dtype=torch.int32, device="cuda")]
    j = gg.Context.make_job(d[3], d[0], d[1], d[2], N, S, gcf_index=d[4], n_gcf=2)
    with pytest.raises(gg.GridError) as e:
        ctx.grid_batch(opts_for("gather", "cc_comp"), [j])
    assert e.value.code == gg.ERR_ARG and "gcf_index" in str(e.value)


# ---------------------------------------------------------------------------
# drop-in host entry points (padded buffers, reference semantics)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
@pytest.mark.parametrize("inst", ["zz", "zc", "cc"])
def test_gridGPU_dropin_padded(ctx, mode, inst):
    g = load_golden("gauss_n128_s16")
    N, S = g["N"], g["S"]
    it = np.complex128 if inst == "zz" else np.complex64
    ot = np.complex64 if inst == "cc" else np.complex128
    gg.set_global_options(gg.Options(mode=MODES[mode],
                                     accum=gg.ACC_COMPENSATED if inst != "zz" else gg.ACC_PLAIN))
    try:
        uvc = np.ascontiguousarray(to_complex(g["uv"]).astype(it))
        vals = np.ascontiguousarray(to_complex(g["vals"]).astype(it))
        gcf = np.ascontiguousarray(to_complex(g["gcf"]).astype(it))
        out = np.full(gg.padded_size(N, S), 7 + 7j, ot)
        gg.gridGPU(out, uvc, vals, len(uvc), N, gcf, S)
    finally:
        gg.set_global_options(gg.Options())
    h = gg.grid_head(N, S)
    assert np.all(out[:h] == 0) and np.all(out[h + N * N:] == 0)
    head = out[h:h + N * N]
    if mode == "window":   # planar, like grid_kernel_window (grid_gpu.cu:524-525)
        r = head.view(np.float64 if ot == np.complex128 else np.float32)
        grid = np.stack([r[:N * N], r[N * N:]]).reshape(2, 1, N, N)
    else:
        grid = np.stack([head.real, head.imag]).reshape(2, 1, N, N)
    if inst == "zz":
        assert rel_err(grid, g["out"]) <= 1e-12
    else:
        check(grid, "zc" if inst == "zc" else "cc_comp",
              g["uv"].astype(np.float32).astype(np.float64), vals, gcf, N, S)


def test_convgrid_python3(ctx):
    g = load_golden("gauss_n64_s8")
    N, S = g["N"], g["S"]
    flat_uv = g["uv"].reshape(-1).tolist()
    vals = list(to_complex(g["vals"]))
    gcf = list(to_complex(g["gcf"]))
    grid = gg.convgrid(flat_uv, len(g["uv"]), vals, N, gcf, 8, S)
    assert grid.shape == (N, N)
    ref = g["out"][0, 0] + 1j * g["out"][1, 0]
    assert np.abs(grid - ref).max() <= 1e-12 * np.abs(ref).max()


# ---------------------------------------------------------------------------
# full-size workloads: size-independent properties
# ---------------------------------------------------------------------------
def _device_inputs(uv, vals, gcf):
    return (torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
            torch.from_numpy(gcf.reshape(-1)).cuda())


def test_tracks_4096_all_methods_agree_and_match_oracle_sample(ctx):
    """gather / moving-window workload (4096^2, 2^22 visibilities on uv
    tracks, S=8): the three methods agree; a 1/16 sample of the visibilities
    is checked against the oracle."""
    N, S = 4096, 8
    uv, vals = synth.tracks(N, npts=1 << 22, seed=21)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    d_uv, d_vals, d_gcf = _device_inputs(uv, vals, gcf)
    outs = {}
    for mode in MODES:
        o = opts_for(mode, "cc_comp", layout=gg.LAYOUT_INTERLEAVED)
        out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
        ctx.grid(o, out, d_uv, d_vals, d_gcf, N, S)
        outs[mode] = out
    torch.cuda.synchronize()
    ref = outs["window"]
    scale = ref.abs().max().item()
    for mode in ("scatter", "gather"):
        assert (outs[mode] - ref).abs().max().item() <= 1e-6 * scale
    sub = slice(0, None, 16)
    o = opts_for("window", "cc_comp", layout=gg.LAYOUT_INTERLEAVED)
    out = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    ctx.grid(o, out, *_device_inputs(np.ascontiguousarray(uv[sub]),
                                     np.ascontiguousarray(vals[sub]), gcf), N, S)
    host = torch.view_as_real(out).reshape(-1).cpu().numpy()
    got = planar_from_grid(host, 1, N, False)
    check(got, "cc_comp", uv[sub], vals[sub], gcf, N, S)


@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_linearity_and_checksum_large(ctx, mode):
    """grid(a*v1 + b*v2) = a*grid(v1) + b*grid(v2), and the grid sum equals
    sum_n v_n * (sum of the visibility's GCF taps) for on-grid footprints."""
    N, S = 2048, 16
    rng = np.random.default_rng(22)
    uv, v1 = synth.disk(1 << 20, N, seed=22)
    v2 = synth.normal_vals(rng, len(uv))
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    o = opts_for(mode, "cc_comp", layout=gg.LAYOUT_INTERLEAVED)
    res = []
    for v in (v1, v2, (2 * v1.astype(np.complex128) - 3 * v2).astype(np.complex64)):
        out = torch.empty(N * N, dtype=torch.complex128, device="cuda")
        d_uv, d_v, d_g = _device_inputs(uv, v, gcf)
        ctx.grid(o, out, d_uv, d_v, d_g, N, S)
        res.append(out)
    torch.cuda.synchronize()
    a, b, c = (r.cpu().numpy() for r in res)
    lin = 2 * a - 3 * b
    assert np.abs(c - lin).max() <= 1e-6 * np.abs(c).max()
    pk = O.vis2ints(uv)
    sx, sy = pk[:, 0] % 8, pk[:, 1] % 8
    tapsum = gcf.reshape(64, S, S).sum(axis=(1, 2)).astype(np.complex128)
    expect = (v1.astype(np.complex128) * tapsum[sy * 8 + sx]).sum()
    bound = (np.abs(v1) * np.abs(tapsum[sy * 8 + sx])).sum()
    assert abs(a.sum() - expect) <= 1e-6 * bound


@pytest.mark.parametrize("S,W", [(4, 0), (8, 1), (8, 2), (16, 1), (16, 2), (16, 4), (32, 4)])
def test_window_8_cell_tiles(ctx, S, W):
    """The moving window on 8-cell uv tiles (more, smaller sub-grids): a
    ragged grid with visibilities past every edge, against the oracle."""
    N = 100
    uv, vals = synth.uniform(6000, -S, N + S, seed=40 + S + W)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    o = opts_for("window", "cc_comp", tile=8, group_warps=W)
    out, flags = run(ctx, o, uv, vals, gcf, N, S, "cc_comp")
    assert flags == [0, 0, 0, 0]
    check(out, "cc_comp", uv, vals, gcf, N, S)


@pytest.mark.parametrize("T", [16, 32])
@pytest.mark.parametrize("prec", ["cc", "cc_comp"])
def test_window_support_32_four_warp_groups(ctx, prec, T):
    """Support 32 with four-warp groups (eight residue rows per thread), plain
    and compensated FP32 sums, ragged grid, against the oracle."""
    N, S = 200, 32
    uv, vals = synth.uniform(4000, -S, N + S, seed=60 + T)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    o = opts_for("window", prec, tile=T, group_warps=4)
    out, flags = run(ctx, o, uv, vals, gcf, N, S, prec)
    assert flags == [0, 0, 0, 0]
    check(out, prec, uv, vals, gcf, N, S)


# ---------------------------------------------------------------------------
# accumulate: add into the present grid (device entry points)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("layout", [gg.LAYOUT_INTERLEAVED, gg.LAYOUT_PLANAR])
@pytest.mark.parametrize("prec", ["zz", "cc_comp"])
@pytest.mark.parametrize("mode", ["scatter", "gather", "window"])
def test_accumulate_adds_into_the_present_grid(ctx, mode, prec, layout):
    """options.accumulate = 1: the gridded values are added to what `out`
    holds (a random grid here, in the layout's own memory order), for every
    method, FP64 and compensated FP32, both layouts, two polarisations; the
    autotuner does not run (its trials would write the outputs)."""
    N, S, P = 128, 8, 2
    uv, vals = synth.tracks(N, nant=16, ntime=200, npts=30000, seed=31)
    rng = np.random.default_rng(32)
    vals = (rng.standard_normal(len(uv) * P) + 1j * rng.standard_normal(len(uv) * P))
    vdt = np.complex128 if prec == "zz" else np.complex64
    vals = vals.astype(vdt)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(vdt)
    odt = torch.complex128 if prec == "zz" else torch.complex64
    o = opts_for(mode, prec, layout=layout, polarizations=P, accumulate=True, autotune=1)
    base = (rng.standard_normal(P * N * N) + 1j * rng.standard_normal(P * N * N))
    out = torch.from_numpy(base.astype(np.complex128)).to(odt).cuda()
    start = torch.view_as_real(out).reshape(-1).cpu().numpy().copy()
    ctx.grid(o, out, torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(), N, S)
    torch.cuda.synchronize()
    assert ctx.read_flags() == [0, 0, 0, 0]
    planar = layout == gg.LAYOUT_PLANAR
    got = planar_from_grid(torch.view_as_real(out).reshape(-1).cpu().numpy(), P, N, planar)
    ref = oracle_for(uv, vals, gcf, N, S, P=P) + planar_from_grid(start, P, N, planar)
    assert rel_err(got, ref) <= (1e-12 if prec == "zz" else 1e-6)


def test_accumulate_batch_twice_is_two_grids(ctx):
    """A batched window call with accumulate = 1 run twice into the same
    (zeroed) outputs gives twice the grid of each job."""
    jobs, keep, refs = [], [], []
    for k, (N, S) in enumerate([(128, 8), (256, 16), (64, 8)]):
        uv, vals = synth.tracks(N, nant=12, ntime=150, npts=20000, seed=40 + k)
        gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(),
             torch.zeros(N * N, dtype=torch.complex64, device="cuda")]
        keep.append(d)
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S))
        refs.append(2.0 * oracle_for(uv, vals, gcf, N, S))
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED, accumulate=True)
    ctx.grid_batch(o, jobs)
    ctx.grid_batch(o, jobs)
    torch.cuda.synchronize()
    assert ctx.read_flags() == [0, 0, 0, 0]
    for d, ref, j in zip(keep, refs, jobs):
        N = j.img_dim
        got = planar_from_grid(torch.view_as_real(d[3]).reshape(-1).cpu().numpy(), 1, N, False)
        assert rel_err(got, ref) <= 1e-6
