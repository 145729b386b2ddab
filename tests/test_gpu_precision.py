"""Accuracy of FP32 gridding where rounding errors are largest, measured per
cell: |gpu - oracle| / sum |v| |w| at every cell (the oracle's magnitude sum
of that cell's additions), beside the normwise figure.  Calls go through the
C ABI of libgg.so.

* the precision form at reduced size: uniform-disk uv, 1% outliers at 1e3
  amplitude, support 32, GCF computed on the fly -- compensated FP32 meets
  the per-cell bound, plain FP32 accumulation does not;
* one dense 8-cell uv tile cut into hundreds of work items: the partial
  sub-grids of the items are merged exactly (FP64 merge slots), so the
  per-cell error does not grow with the number of items, for complex64 and
  complex128 grids, two polarisations, planar and interleaved layouts,
  per-visibility tables and batches.
"""
import numpy as np
import pytest

import gpugrid as gg
import oracle as O
import synth
from helpers import cell_err, planar_from_grid, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

U = 2.0 ** -24                     # unit roundoff of FP32
# compensated FP32, per cell: 10 u.  Measured on GB300: 3.7-4.6 u on the
# precision form (most of it the FP32 evaluation of the Gaussian GCF), 0.8 u
# on the dense tile; plain FP32 accumulation reaches 24 u on the precision form
CELL_COMP = 10 * U
NORM_COMP = 1e-6


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gg.Context(0)
    yield c
    c.close()


def pairs(c):
    c = np.asarray(c).reshape(-1)
    return np.stack([c.real, c.imag], -1).astype(np.float64)


def grid_dev(ctx, o, uv, vals, gcf, N, S, out_dtype, P=1, gcf_index=None, n_gcf=0):
    d_uv = torch.from_numpy(np.ascontiguousarray(uv)).cuda()
    d_v = torch.from_numpy(np.ascontiguousarray(vals)).cuda()
    d_g = None if gcf is None else torch.from_numpy(np.ascontiguousarray(gcf).reshape(-1)).cuda()
    out = torch.full((P * N * N,), float("nan"), dtype=out_dtype, device="cuda")
    d_i = None if gcf_index is None else torch.from_numpy(gcf_index).cuda()
    job = gg.Context.make_job(out, d_uv, d_v, d_g, N, S, gcf_index=d_i, n_gcf=n_gcf)
    ctx.grid_job(o, job)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    planar = o.layout == gg.LAYOUT_PLANAR
    host = torch.view_as_real(out).reshape(-1).cpu().numpy()
    return planar_from_grid(host, P, N, planar), flags


# ---------------------------------------------------------------------------
# precision form (uniform disk, 1% outliers at 1e3, S=32, on-the-fly GCF)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def disk_case():
    N, S, n = 1024, 32, 1 << 19
    uv, vals = synth.disk(n, N, seed=5, outlier_frac=0.01, outlier_amp=1e3)
    g1 = synth.gaussian_gcf_1d(S)
    tab = synth.gcf_table(g1)
    ref = O.grid_pz(uv, pairs(vals), pairs(tab), N, S, nthreads=16)
    mag = O.grid_mag(uv, pairs(vals), pairs(tab), N, S, nthreads=16)
    return dict(N=N, S=S, uv=uv, vals=vals, ref=ref, mag=mag)


@pytest.mark.parametrize("mode,out", [("window", "c64"), ("window", "c128"),
                                      ("scatter", "c64"), ("gather", "c64")])
def test_precision_form_compensated_meets_per_cell_bound(ctx, disk_case, mode, out):
    c = disk_case
    o = gg.Options(mode=gg.MODES[mode], accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED, gcf_kind=gg.GCF_GAUSSIAN)
    odt = torch.complex64 if out == "c64" else torch.complex128
    got, flags = grid_dev(ctx, o, c["uv"], c["vals"], None, c["N"], c["S"], odt)
    assert flags == [0, 0, 0, 0]
    cmax, crms = cell_err(got, c["ref"], c["mag"])
    ne = rel_err(got, c["ref"])
    print(f"\n{mode} {out} compensated: normwise {ne:.3e} per-cell max {cmax:.3e} "
          f"rms {crms:.3e} ({cmax / U:.1f} u)")
    assert ne <= NORM_COMP and cmax <= CELL_COMP, (ne, cmax, crms)


def test_precision_form_plain_fp32_misses_the_bound(ctx, disk_case):
    """The same job with plain FP32 accumulation: its worst cells carry more
    error than the compensated bound allows -- the stress the outliers were
    put there for, visible per cell."""
    c = disk_case
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_PLAIN, layout=gg.LAYOUT_INTERLEAVED,
                   gcf_kind=gg.GCF_GAUSSIAN)
    got, flags = grid_dev(ctx, o, c["uv"], c["vals"], None, c["N"], c["S"], torch.complex64)
    assert flags == [0, 0, 0, 0]
    cmax, crms = cell_err(got, c["ref"], c["mag"])
    print(f"\nwindow c64 plain: normwise {rel_err(got, c['ref']):.3e} per-cell max "
          f"{cmax:.3e} rms {crms:.3e} ({cmax / U:.1f} u)")
    assert cmax > CELL_COMP, cmax


# ---------------------------------------------------------------------------
# one dense tile cut into many work items
# ---------------------------------------------------------------------------
def dense_tile(n, seed, pols=1):
    """n visibilities whose main cells all fall in the 8-cell uv tile (3, 3)
    of a 64^2 grid; values with a positive mean (partial sums of one sign,
    where merge roundings add up)."""
    rng = np.random.default_rng(seed)
    uv = synth.fr(rng.uniform(24, 32, size=(n, 2)))
    v = 1.0 + 0.5 * (rng.standard_normal(n * pols) + 1j * rng.standard_normal(n * pols))
    return uv, v.astype(np.complex64)


@pytest.mark.parametrize("out,layout,P", [("c64", gg.LAYOUT_INTERLEAVED, 1),
                                          ("c64", gg.LAYOUT_PLANAR, 2),
                                          ("c128", gg.LAYOUT_INTERLEAVED, 1)])
def test_dense_tile_many_items_error_independent_of_item_count(ctx, out, layout, P):
    N, S, n, chunk = 64, 8, 1 << 18, 1024          # 256 work items in one tile
    uv, vals = dense_tile(n, 7, P)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    ref = O.grid_pz(uv, pairs(vals), pairs(gcf), N, S, pols=P, nthreads=16)
    mag = O.grid_mag(uv, pairs(vals), pairs(gcf), N, S, pols=P, nthreads=16)
    odt = torch.complex64 if out == "c64" else torch.complex128
    errs = {}
    for ch in (chunk, 1 << 20):                    # 256 items vs. one item
        o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=layout,
                       tile=8, window_chunk=ch, polarizations=P)
        got, flags = grid_dev(ctx, o, uv, vals, gcf, N, S, odt, P=P)
        assert flags == [0, 0, 0, 0]
        errs[ch] = cell_err(got, ref, mag)
        print(f"\ndense tile {out} P={P} records/item {ch}: per-cell max {errs[ch][0]:.3e} "
              f"({errs[ch][0] / U:.1f} u) rms {errs[ch][1]:.3e}")
        assert rel_err(got, ref) <= NORM_COMP
        assert errs[ch][0] <= CELL_COMP, errs[ch]
    # merging 256 partial sub-grids costs at most a few roundings more than one
    assert errs[chunk][0] <= errs[1 << 20][0] + 8 * U, errs


def test_dense_tile_per_visibility_tables_and_batch(ctx):
    """Dense tiles in a batch with per-visibility tables (a merge slot per
    (tile, table) bin) and a job with a complex128 grid beside complex64
    ones."""
    S, n = 8, 150000
    jobs, keep, checks = [], [], []
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                   layout=gg.LAYOUT_INTERLEAVED, tile=8, window_chunk=1024)
    for k, (N, ntab, odt) in enumerate([(64, 3, torch.complex64), (64, 1, torch.complex128),
                                        (96, 2, torch.complex64)]):
        uv, vals = dense_tile(n, 20 + k)
        rng = np.random.default_rng(30 + k)
        idx = rng.integers(0, ntab, n).astype(np.int32)
        tabs = [synth.gcf_table(synth.gaussian_gcf_1d(S, sigma=2 + 0.3 * t)).astype(np.complex64)
                for t in range(ntab)]
        stack = np.concatenate([t.reshape(-1) for t in tabs])
        d = [torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(stack).cuda(),
             torch.full((N * N,), float("nan"), dtype=odt, device="cuda"),
             torch.from_numpy(idx).cuda()]
        keep.append(d)
        jobs.append(gg.Context.make_job(d[3], d[0], d[1], d[2], N, S,
                                        gcf_index=d[4] if ntab > 1 else None,
                                        n_gcf=ntab if ntab > 1 else 0))
        ref = O.grid_pz_gcfinx(uv, vals, idx, stack, N, S, nthreads=16)
        mag = O.grid_mag(uv, pairs(vals), pairs(stack), N, S, gcfinx=idx, nthreads=16)
        checks.append((N, ref, mag))
    ctx.grid_batch(o, jobs)
    torch.cuda.synchronize()
    assert ctx.read_flags() == [0, 0, 0, 0]
    for (N, ref, mag), d in zip(checks, keep):
        host = torch.view_as_real(d[3]).reshape(-1).cpu().numpy()
        got = planar_from_grid(host, 1, N, False)
        cmax, _ = cell_err(got, ref, mag)
        assert rel_err(got, ref) <= NORM_COMP and cmax <= CELL_COMP, (N, cmax)
