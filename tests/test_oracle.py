"""CPU tests of the oracle itself: before the oracle checks the GPU path, it
is pinned against outputs of the reference's own CPU gridder (golden
fixtures made by tests/golden/make_golden.py from grid.cu's gridCPU_pz) and,
where the reference checkout is present, against that code directly."""
import numpy as np
import pytest

import oracle as O
import synth
from helpers import GOLDEN_CASES, load_golden

REF_TAGS = ["64_8_1_double", "64_8_4_double", "64_32_1_double",
            "128_16_1_double", "256_8_1_double", "64_8_1_double_dbg"]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_port_matches_golden_bit_exact(name):
    g = load_golden(name)
    out = O.grid_pz(g["uv"], g["vals"], g["gcf"], g["N"], g["S"], pols=g["P"],
                    debug1=g["debug1"])
    assert np.array_equal(out, g["out"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_multithreaded_port_bit_identical(name):
    g = load_golden(name)
    a = O.grid_pz(g["uv"], g["vals"], g["gcf"], g["N"], g["S"], pols=g["P"],
                  debug1=g["debug1"])
    b = O.grid_pz(g["uv"], g["vals"], g["gcf"], g["N"], g["S"], pols=g["P"],
                  debug1=g["debug1"], nthreads=7)
    assert np.array_equal(a, b)


def test_golden_has_clipped_and_offgrid_visibilities():
    g = load_golden("gauss_n64_s8")
    uv = g["uv"]
    assert (uv < 0).any() and (uv >= g["N"]).any()
    # DEBUG1: every hit count is an integer, and the footprint total is the
    # number of on-grid taps
    d = load_golden("debug1_n64_s8")
    counts = d["out"][0, 0]
    assert np.array_equal(counts, np.round(counts))
    S, N = d["S"], d["N"]
    m = np.floor(d["uv"]).astype(int)
    taps = 0
    for mx, my in m:
        xs = np.arange(mx - S // 2 + 1, mx + S // 2 + 1)
        ys = np.arange(my - S // 2 + 1, my + S // 2 + 1)
        taps += ((xs >= 0) & (xs < N)).sum() * ((ys >= 0) & (ys < N)).sum()
    assert counts.sum() == taps


@pytest.mark.parametrize("tag", REF_TAGS)
def test_port_matches_reference_code(tag):
    if not O.ref_available(tag):
        pytest.skip("reference checkout not compiled here (oracle/_ref)")
    R = O.RefLib(tag)
    N, S, P = R.img, R.gcf_dim, R.pols
    rng = np.random.default_rng(hash(tag) % 1000)
    uv = rng.uniform(-S, N + S, size=(900, 2)).astype(np.float32).astype(np.float64)
    vals = rng.standard_normal((900 * P, 2))
    gcf, _ = O.gaussian_gcf(S)
    assert np.array_equal(R.grid(uv, vals, gcf),
                          O.grid_pz(uv, vals, gcf, N, S, pols=P, debug1=bool(R.debug1)))


def test_reference_nonsense_gcf_and_harness_inputs():
    if not O.ref_available("64_8_1_double"):
        pytest.skip("reference checkout not compiled here (oracle/_ref)")
    R = O.RefLib("64_8_1_double")
    uv, vals = R.harness_inputs(500)
    g = R.init_gcf()
    assert np.array_equal(R.grid(uv, vals, g), O.grid_pz(uv, vals, g, 64, 8))


def test_index_step_formulas_agree_on_float_representable():
    rng = np.random.default_rng(3)
    uv = rng.uniform(-50, 5000, size=(20000, 2)).astype(np.float32).astype(np.float64)
    uv[:10] = [[0, 0], [1, 1], [-1, -1], [7.875, 7.999], [4095.875, 0.125],
               [-0.125, -7.5], [2.5, 3.5], [100, 200], [1e-3, 1e-3], [-1e-3, 5]]
    uv[:10] = uv[:10].astype(np.float32).astype(np.float64)
    a = O.vis2ints(uv)
    b = O.vis2ints(uv, gpu_formula=True)
    assert np.array_equal(a, b)
    m = np.floor(uv).astype(np.int64)
    s = np.floor(8 * (uv - m)).astype(np.int64)
    assert np.array_equal(a, (m * 8 + s).astype(np.int32))


def test_index_step_follows_cpu_formula_below_integer():
    # u just below an integer, not float-representable: the CPU gridder's
    # floorf((float)u) rounds up, so its oversample index is -1 while the
    # all-double GPU driver formula gives 7 (grid.cu:159 vs grid_gpu.cu:118)
    u = np.array([[99.99999999, 10.5]])
    a = O.vis2ints(u)
    b = O.vis2ints(u, gpu_formula=True)
    assert a[0, 0] == 99 * 8 - 1
    assert b[0, 0] == 99 * 8 + 7


def test_bookmarks_are_lower_bounds():
    rng = np.random.default_rng(4)
    N, T = 256, 32
    uv = rng.uniform(0, N, size=(5000, 2)).astype(np.float32).astype(np.float64)
    pk = O.vis2ints(uv)
    tile = (pk[:, 1] // 8 // T) * (N // T) + pk[:, 0] // 8 // T
    order = np.argsort(tile, kind="stable")
    bm = O.set_bookmarks(pk[order], T, N // T)
    expect = np.searchsorted(tile[order], np.arange(N // T * N // T + 1), "left")
    assert np.array_equal(bm, expect)


def test_gaussian_gcf_is_separable_and_peaks_at_centre():
    tab, g1 = O.gaussian_gcf(16)
    assert tab.shape == (64, 16, 16)
    assert np.allclose(tab.imag, 0)
    # sub-kernel 0: sample distance a - 0 is zero at a' = S/2 - 1
    assert g1[0].argmax() == 16 // 2 - 1 and g1[0].max() == 1.0
    t2 = O.gcf_from_1d(g1)
    assert np.array_equal(tab, t2)


def test_oracle_per_visibility_tables():
    """gridCPU_pz with a table per visibility (vis.gcfinx): one table is the
    plain oracle bit for bit; several tables = the sum of per-table grids;
    indices outside the stack are skipped."""
    uv, v = synth.uniform(4000, 4, 60, seed=11)
    S = 8
    tabs = [synth.gcf_table(synth.gaussian_gcf_1d(S, sigma=sg)) for sg in (1.5, 2.0, 2.5)]
    tabs[1] = tabs[1] * np.exp(0.7j)  # a complex table
    stack = np.concatenate([t.reshape(-1) for t in tabs])
    one = O.grid_pz_gcfinx(uv, v, np.zeros(len(uv), np.int32), tabs[0].reshape(-1), 64, S)
    assert np.array_equal(one, O.grid_pz(uv, v, tabs[0], 64, S))
    idx = (np.arange(len(uv)) * 7 % 3).astype(np.int32)
    idx[::97] = 5
    idx[1::101] = -1
    got = O.grid_pz_gcfinx(uv, v, idx, stack, 64, S, nthreads=4)
    want = sum(O.grid_pz(uv[idx == k], v[idx == k], tabs[k], 64, S) for k in range(3))
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_oracle_wphase_factor_is_the_reference_formula():
    """COMPUTE_GCF restatement: with T = 0 the factor is the constant
    (sin 2 pi w, cos 2 pi w) in float, i.e. the plain oracle with a constant
    table; with T != 0 it depends on the sub-pixel position only."""
    S, G, N = 8, 8, 64
    uv, v = synth.uniform(2000, 6, 58, seed=5)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    off = S * (S - 1) // 2 - 1
    w = 0.123
    gcf.reshape(-1)[off] = 0.0 + 1j * w
    p1 = np.float32(2 * 3.1415926 * w)
    const = np.full(G * G * S * S, complex(np.sin(p1), np.cos(p1)))
    got = O.grid_pz_wphase(uv, v, gcf, N, S, nthreads=2)
    want = O.grid_pz(uv, v, const, N, S)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    # T != 0: two visibilities with the same sub-pixel offset get the same factor
    gcf.reshape(-1)[off] = 3.0 + 1j * w
    one = np.array([[20.25, 30.5]])
    two = np.array([[20.25, 30.5], [40.25, 10.5]])
    a = O.grid_pz_wphase(one, np.array([1.0 + 0j]), gcf, N, S)
    b = O.grid_pz_wphase(two, np.array([1.0 + 0j, 0j]), gcf, N, S)
    assert np.array_equal(a, b)


def _cdot(a, b):
    """<a, b> = sum conj(a) * b over complex arrays"""
    return np.vdot(np.asarray(a).ravel(), np.asarray(b).ravel())


@pytest.mark.parametrize("S,P,n_gcf", [(4, 1, 1), (8, 2, 3), (16, 1, 2), (32, 1, 1)])
def test_degrid_oracle_is_the_adjoint_of_the_gridder(S, P, n_gcf):
    """<grid(v), g> = <v, degrid(g)> for random complex tables (no symmetry),
    visibilities past every edge of a ragged grid and per-visibility tables,
    with the gridding side the reference-pinned gridCPU_pz restatement."""
    rng = np.random.default_rng(S * 10 + P)
    N, n, G = 61, 700, 8
    uv = synth.fr(rng.uniform(-S, N + S, size=(n, 2)))
    v = (rng.standard_normal((n, P)) + 1j * rng.standard_normal((n, P)))
    tabs = rng.standard_normal((n_gcf * G * G * S * S, 2))
    idx = rng.integers(0, n_gcf, n).astype(np.int32)
    g = rng.standard_normal((2, P, N, N))
    grid = O.grid_pz_gcfinx(uv, v.reshape(-1), idx, tabs, N, S, pols=P)
    d = O.degrid_pz(uv, g, tabs, N, S, pols=P, gcfinx=idx)
    lhs = _cdot(grid[0] + 1j * grid[1], g[0] + 1j * g[1])
    rhs = _cdot(v, d)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_degrid_oracle_drops_out_of_range_indices_and_is_thread_independent():
    N, S = 64, 8
    rng = np.random.default_rng(3)
    uv = synth.fr(rng.uniform(0, N, size=(500, 2)))
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S))
    g = rng.standard_normal((2, 1, N, N))
    idx = np.zeros(500, np.int32)
    idx[::7] = 1  # outside a stack of one table
    d1 = O.degrid_pz(uv, g, gcf, N, S, gcfinx=idx)
    d4 = O.degrid_pz(uv, g, gcf, N, S, gcfinx=idx, nthreads=4)
    assert np.array_equal(d1, d4)
    assert np.all(d1[::7] == 0) and np.all(d1[1::7] != 0)
    # a visibility far off the grid touches no cell
    far = synth.fr(np.array([[-40.0, 10.0], [10.0, N + 40.0]]))
    assert np.all(O.degrid_pz(far, g, gcf, N, S) == 0)


def _pairs(c):
    c = np.asarray(c).reshape(-1)
    return np.stack([c.real, c.imag], -1).astype(np.float64)


@pytest.mark.parametrize("n_gcf", [1, 3])
def test_magnitude_grid_bounds_every_cell(n_gcf):
    """The per-cell magnitude sum (denominator of the per-cell error) covers
    exactly the additions of the gridder: |grid| <= mag at every cell, mag is
    zero exactly where no tap lands, it equals the grid for positive real
    values and tables, and it does not depend on the thread count."""
    N, S, P = 96, 8, 2
    rng = np.random.default_rng(41)
    uv, _ = synth.uniform(3000, -S, N + S, seed=41)
    vals = (rng.standard_normal(len(uv) * P) + 1j * rng.standard_normal(len(uv) * P))
    tabs = np.concatenate([
        (synth.gcf_table(synth.gaussian_gcf_1d(S, sigma=2 + t)) * np.exp(0.7j * t)).reshape(-1)
        for t in range(n_gcf)])
    idx = rng.integers(0, n_gcf, len(uv)).astype(np.int32)
    grid = O.grid_pz_gcfinx(uv, _pairs(vals), idx, _pairs(tabs), N, S, pols=P)
    mag = O.grid_mag(uv, _pairs(vals), tabs, N, S, pols=P, gcfinx=idx)
    assert mag.shape == (P, N, N)
    assert np.all(np.hypot(grid[0], grid[1]) <= mag * (1 + 1e-12))
    ones = O.grid_pz_gcfinx(uv, np.ones((len(uv) * P, 2)) * [1, 0], idx, np.abs(_pairs(tabs)),
                            N, S, pols=P)
    assert np.array_equal(mag > 0, ones[0] > 0)
    assert np.array_equal(mag, O.grid_mag(uv, _pairs(vals), tabs, N, S, pols=P, gcfinx=idx,
                                          nthreads=7))
    pos = np.abs(vals).astype(np.complex128)
    absg = np.abs(tabs).astype(np.complex128)
    g2 = O.grid_pz_gcfinx(uv, _pairs(pos), idx, _pairs(absg), N, S, pols=P)
    m2 = O.grid_mag(uv, _pairs(pos), absg, N, S, pols=P, gcfinx=idx)
    assert np.allclose(g2[0], m2, rtol=1e-14, atol=0) and not g2[1].any()


def test_cell_error_metric():
    """cell_err: |a - ref| / mag per cell; an error where nothing was gridded
    is infinite; cells with mag 0 and no error are left out."""
    from helpers import cell_err
    ref = np.zeros((2, 1, 4, 4))
    mag = np.zeros((1, 4, 4))
    ref[0, 0, 1, 1], mag[0, 1, 1] = 1.0, 2.0
    a = ref.copy()
    a[1, 0, 1, 1] = 1e-3
    mx, rms = cell_err(a, ref, mag)
    assert mx == pytest.approx(5e-4) and rms == pytest.approx(5e-4)
    a[0, 0, 0, 0] = 1e-30
    assert cell_err(a, ref, mag)[0] == float("inf")
