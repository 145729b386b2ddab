"""GPU tests of the grid -> dirty image step (centred inverse 2-D DFT of
every polarisation plane, in place, through the C ABI; cuFFT underneath).
The check is numpy's FFT of the same grid:
  image = N^2 * fftshift(ifft2(ifftshift(grid)))
normwise (max |gpu - numpy| / max |numpy|): complex64 1e-5, complex128 1e-12.
"""
import numpy as np
import pytest

import gpugrid as gg
import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gg.Context(0)
    yield c
    c.close()


def numpy_image(g):
    n = g.shape[-1]
    ax = (-2, -1)
    return n * n * np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=ax), axes=ax), axes=ax)


@pytest.mark.parametrize("dtype,tol", [(np.complex64, 1e-5), (np.complex128, 1e-12)])
@pytest.mark.parametrize("N,P", [(256, 1), (96, 2)])
def test_image_matches_numpy(ctx, dtype, tol, N, P):
    rng = np.random.default_rng(N + P)
    g = (rng.standard_normal((P, N, N)) + 1j * rng.standard_normal((P, N, N))).astype(dtype)
    d = torch.from_numpy(g.reshape(-1).copy()).cuda()
    ctx.grid_to_image(d, N, P)
    got = d.cpu().numpy().reshape(P, N, N)
    ref = numpy_image(g.astype(np.complex128))
    assert np.abs(got - ref).max() / np.abs(ref).max() <= tol


def test_point_source_images_at_its_position(ctx):
    """grid the visibilities of a unit point source at pixel offset (l0, m0)
    from the centre with a narrow Gaussian GCF; the dirty image peaks there"""
    N, S, l0, m0 = 256, 8, 9, -6
    uv, _ = synth.tracks(N, nant=24, ntime=400, npts=None, seed=4)
    u = uv[:, 0] - N / 2
    v = uv[:, 1] - N / 2
    vals = np.exp(-2j * np.pi * (u * l0 + v * m0) / N).astype(np.complex64)
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
    grid = torch.empty(N * N, dtype=torch.complex64, device="cuda")
    o = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED)
    ctx.grid(o, grid, torch.from_numpy(uv).cuda(), torch.from_numpy(vals).cuda(),
             torch.from_numpy(gcf.reshape(-1)).cuda(), N, S)
    ctx.grid_to_image(grid, N)
    img = np.abs(grid.cpu().numpy().reshape(N, N))
    m, l = np.unravel_index(np.argmax(img), img.shape)
    assert (l - N // 2, m - N // 2) == (l0, m0)


def test_odd_image_size_rejected(ctx):
    d = torch.zeros(63 * 63, dtype=torch.complex64, device="cuda")
    with pytest.raises(gg.GridError) as e:
        ctx.grid_to_image(d, 63)
    assert e.value.code == gg.ERR_ARG
