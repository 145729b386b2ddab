"""GPU tests of degridding (the adjoint of the gridder), through the C ABI.

The oracle's degridder is checked on the CPU to be the exact adjoint of the
reference-pinned gridding oracle (tests/test_oracle.py); here the GPU
degridder is compared with it, normwise (max |gpu - oracle| / max |oracle|):
  FP64 values ............................................. 1e-12
  FP32 values, compensated lane sums ...................... 1e-6
  FP32 values, plain FP32 sums ............................ 2e-6
and, at the size of the 4096^2 track workload, the GPU degridder is checked
against the GPU gridder through <grid(v), g> = <v, degrid(g)>.
"""
import numpy as np
import pytest

import gpugrid as gg
import oracle as O
import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = {"zz": 1e-12, "cc_comp": 1e-6, "cc": 2e-6}


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gg.Context(0)
    yield c
    c.close()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def device_grid(g_planar, layout, dtype):
    """planar (2, P, N, N) float64 -> device tensor in the requested layout"""
    c = g_planar[0] + 1j * g_planar[1]
    if layout == gg.LAYOUT_PLANAR:
        real = torch.from_numpy(np.ascontiguousarray(g_planar.reshape(-1)))
        real = real.to(torch.float64 if dtype == torch.complex128 else torch.float32)
        return real.cuda()
    return torch.from_numpy(c.reshape(-1).astype(np.complex128)).to(dtype).cuda()


def degrid_gpu(ctx, opts, uv, g_planar, gcf, N, S, P, vals_dtype, grid_dtype,
               gcf_index=None, n_gcf=1):
    d_uv = torch.from_numpy(np.ascontiguousarray(uv)).cuda()
    d_grid = device_grid(g_planar, opts.layout, grid_dtype)
    out = torch.full((len(uv) * P,), float("nan"), dtype=vals_dtype, device="cuda")
    d_gcf = (torch.from_numpy(np.ascontiguousarray(gcf).reshape(-1)).to(vals_dtype).cuda()
             if gcf is not None else None)
    d_idx = torch.from_numpy(gcf_index).cuda() if gcf_index is not None else None
    if opts.layout == gg.LAYOUT_PLANAR:
        # the planar grid is a real tensor: describe it by its complex type
        job = gg.Context.make_job(d_grid, d_uv, out, d_gcf, N, S, gcf_index=d_idx, n_gcf=n_gcf)
        job.out_type = gg.C128 if grid_dtype == torch.complex128 else gg.C64
        import ctypes
        s = torch.cuda.current_stream()
        gg._check(gg.LIB.gg_degrid_device(ctx._h, ctypes.byref(opts.c()), ctypes.byref(job),
                                          ctypes.c_void_p(s.cuda_stream)))
    else:
        ctx.degrid(opts, d_grid, d_uv, out, d_gcf, N, S, gcf_index=d_idx, n_gcf=n_gcf)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(len(uv), P), ctx.read_flags()


@pytest.mark.parametrize("S", [4, 8, 16, 32])
@pytest.mark.parametrize("prec", ["cc", "cc_comp", "zz"])
def test_degrid_matches_oracle(ctx, S, prec):
    """ragged grid, visibilities past every edge, a complex table with no
    symmetry, FP32 or FP64 values"""
    rng = np.random.default_rng(S)
    N, n = 100, 3000
    uv = synth.fr(rng.uniform(-S, N + S, size=(n, 2)))
    tab = rng.standard_normal((64 * S * S, 2))
    g = rng.standard_normal((2, 1, N, N))
    vdt = torch.complex128 if prec == "zz" else torch.complex64
    if prec != "zz":  # the GPU sees FP32 table and grid: give the oracle the same
        tab = tab.astype(np.float32).astype(np.float64)
        g = g.astype(np.float32).astype(np.float64)
    acc = gg.ACC_COMPENSATED if prec == "cc_comp" else gg.ACC_PLAIN
    o = gg.Options(accum=acc, layout=gg.LAYOUT_INTERLEAVED)
    got, flags = degrid_gpu(ctx, o, uv, g, tab[:, 0] + 1j * tab[:, 1], N, S, 1, vdt, vdt)
    assert flags == [0, 0, 0, 0]
    ref = O.degrid_pz(uv, g, tab, N, S)
    assert rel(got, ref) <= TOL[prec], rel(got, ref)


@pytest.mark.parametrize("layout", [gg.LAYOUT_INTERLEAVED, gg.LAYOUT_PLANAR])
def test_degrid_layouts_polarisations_and_table_stack(ctx, layout):
    """two polarisations, a stack of three tables selected per visibility
    (one index outside the stack: zero and counted), FP64 grid with FP32
    values, both grid layouts"""
    rng = np.random.default_rng(5)
    N, S, P, n = 128, 8, 2, 4000
    uv = synth.fr(rng.uniform(0, N, size=(n, 2)))
    tabs = rng.standard_normal((3 * 64 * S * S, 2)).astype(np.float32).astype(np.float64)
    idx = rng.integers(0, 3, n).astype(np.int32)
    idx[17] = 3
    g = rng.standard_normal((2, P, N, N))
    o = gg.Options(accum=gg.ACC_COMPENSATED, layout=layout, polarizations=P)
    got, flags = degrid_gpu(ctx, o, uv, g, tabs[:, 0] + 1j * tabs[:, 1], N, S, P,
                            torch.complex64, torch.complex128, gcf_index=idx, n_gcf=3)
    assert flags[0] == 1
    ref = O.degrid_pz(uv, g, tabs, N, S, pols=P, gcfinx=idx)
    assert np.all(got[17] == 0)
    assert rel(got, ref) <= TOL["cc_comp"]


def test_degrid_gaussian_on_the_fly(ctx):
    N, S = 96, 16
    rng = np.random.default_rng(6)
    uv = synth.fr(rng.uniform(0, N, size=(2000, 2)))
    g = rng.standard_normal((2, 1, N, N)).astype(np.float32).astype(np.float64)
    tab = synth.gcf_table(synth.gaussian_gcf_1d(S))
    o = gg.Options(accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED,
                   gcf_kind=gg.GCF_GAUSSIAN)
    got, flags = degrid_gpu(ctx, o, uv, g, None, N, S, 1, torch.complex64, torch.complex64)
    assert flags == [0, 0, 0, 0]
    assert rel(got, O.degrid_pz(uv, g, tab, N, S)) <= TOL["cc_comp"]


def test_degrid_is_the_adjoint_of_the_gpu_gridder_at_full_size(ctx):
    """<grid(v), g> = <v, degrid(g)> with the GPU on both sides: the 4096^2
    track workload (2^22 visibilities, S=8), FP32 compensated arithmetic"""
    N, S = 4096, 8
    uv, vals = synth.tracks(N, npts=1 << 22, seed=3)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    d_uv = torch.from_numpy(uv).cuda()
    d_v = torch.from_numpy(vals).cuda()
    d_g = torch.from_numpy(gcf.reshape(-1)).cuda()
    grid = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED)
    ctx.grid(o, grid, d_uv, d_v, d_g, N, S)
    gen = torch.Generator(device="cuda").manual_seed(7)
    probe = torch.randn(N * N, dtype=torch.complex64, device="cuda", generator=gen)
    back = torch.empty_like(d_v)
    ctx.degrid(o, probe, d_uv, back, d_g, N, S)
    torch.cuda.synchronize()
    assert ctx.read_flags() == [0, 0, 0, 0]
    lhs = torch.vdot(grid.to(torch.complex128), probe.to(torch.complex128)).item()
    rhs = torch.vdot(d_v.to(torch.complex128), back.to(torch.complex128)).item()
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
