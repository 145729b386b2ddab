"""Seeded synthetic visibilities with the shapes of the benchmark workloads.

No public dataset exists for this path; these generators stand in for it.
Coordinates are FP64 grid-pixel positions rounded to float32-representable
values, the convention of the reference harness (grid.cu:446, computed in
float), under which the cell/oversample index step is exact on every path.

* ``uniform``  -- u,v uniform in [lo, hi) (plain-scatter workload: 1024^2,
                  2^18 visibilities, support 16)
* ``tracks``   -- realistic uv tracks: antennas uniform in a disk, all
                  baselines, hour-angle samples at a declination, scaled to
                  fill a fraction of the grid (gather / moving-window
                  workload: 4096^2, 64 antennas, 2016 baselines x 2080 samples
                  over +-4 h at dec -30 deg, 90% fill, padded to 2^22)
* ``disk``     -- uniform density in a disk, N(0,1) values with a fraction of
                  outliers (precision workload: 8192^2, 2^24, 1% at 1e3)
* ``gaussian_gcf`` -- the separable Gaussian table, sigma = S/4
"""
from __future__ import annotations

import math

import numpy as np


def fr(a) -> np.ndarray:
    """float32-representable float64"""
    return np.asarray(a, np.float32).astype(np.float64)


def normal_vals(rng, n: int, dtype=np.complex64, outlier_frac: float = 0.0,
                outlier_amp: float = 1e3) -> np.ndarray:
    v = (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    if outlier_frac > 0:
        k = int(round(n * outlier_frac))
        idx = rng.choice(n, size=k, replace=False)
        ph = rng.uniform(0, 2 * np.pi, size=k)
        v[idx] = outlier_amp * np.exp(1j * ph)
    return v.astype(dtype)


def uniform(npts: int, lo: float, hi: float, seed: int = 0,
            vals_dtype=np.complex64, pols: int = 1):
    rng = np.random.default_rng(seed)
    uv = fr(rng.uniform(lo, hi, size=(npts, 2)))
    vals = normal_vals(rng, npts * pols, vals_dtype)
    return uv, vals


def _antennas(rng, nant: int, radius_m: float) -> np.ndarray:
    r = radius_m * np.sqrt(rng.uniform(0, 1, nant))
    th = rng.uniform(0, 2 * np.pi, nant)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(nant)], axis=1)


def tracks(img_dim: int = 4096, nant: int = 64, ntime: int = 2080,
           ha_hours: float = 4.0, dec_deg: float = -30.0, fill: float = 0.9,
           radius_m: float = 1000.0, npts: int | None = 1 << 22,
           seed: int = 0, vals_dtype=np.complex64):
    """uv tracks of all nant*(nant-1)/2 baselines over hour angles
    [-ha, ha]; (u,v) in pixels centred at img_dim/2, the longest projected
    baseline at fill*img_dim/2.  Visibilities are baseline-major, time-minor;
    when npts exceeds nbl*ntime the first baselines get extra samples past
    the end of the track, when it is smaller the tail is cut."""
    rng = np.random.default_rng(seed)
    ant = _antennas(rng, nant, radius_m)
    i, j = np.triu_indices(nant, k=1)
    bl = ant[j] - ant[i]                                  # (nbl, 3) metres
    nbl = bl.shape[0]
    total = nbl * ntime if npts is None else npts
    extra = max(0, total - nbl * ntime)
    ha = np.linspace(-ha_hours, ha_hours, ntime) * (np.pi / 12.0)
    dha = ha[1] - ha[0] if ntime > 1 else 0.0
    dec = math.radians(dec_deg)
    sd, cd = math.sin(dec), math.cos(dec)

    def uvw(b, h):
        sh, ch = np.sin(h), np.cos(h)
        u = sh * b[..., 0] + ch * b[..., 1]
        v = -sd * ch * b[..., 0] + sd * sh * b[..., 1] + cd * b[..., 2]
        return u, v

    u, v = uvw(bl[:, None, :], ha[None, :])               # (nbl, ntime)
    u, v = u.reshape(-1), v.reshape(-1)
    if extra:
        k = np.arange(extra)
        b = bl[k % nbl]
        h = ha[-1] + dha * (1 + k // nbl)
        ue, ve = uvw(b, h)
        u, v = np.concatenate([u, ue]), np.concatenate([v, ve])
    u, v = u[:total], v[:total]
    scale = fill * (img_dim / 2) / max(np.abs(u).max(), np.abs(v).max())
    uv = fr(np.stack([img_dim / 2 + u * scale, img_dim / 2 + v * scale], axis=1))
    vals = normal_vals(rng, total, vals_dtype)
    return uv, vals


def disk(npts: int, img_dim: int, fill: float = 0.9, seed: int = 0,
         outlier_frac: float = 0.0, outlier_amp: float = 1e3,
         vals_dtype=np.complex64):
    rng = np.random.default_rng(seed)
    r = fill * (img_dim / 2) * np.sqrt(rng.uniform(0, 1, npts))
    th = rng.uniform(0, 2 * np.pi, npts)
    uv = fr(np.stack([img_dim / 2 + r * np.cos(th),
                      img_dim / 2 + r * np.sin(th)], axis=1))
    vals = normal_vals(rng, npts, vals_dtype, outlier_frac, outlier_amp)
    return uv, vals


def tile_sort(uv: np.ndarray, img_dim: int, tile: int = 32, gcf_dim: int = 8,
              oversample: int = 8):
    """Stable order grouping visibilities by uv tile (of the main cell,
    clamped into the grid as the device binning does); returns the
    permutation."""
    m = np.floor(uv).astype(np.int64)
    m = np.clip(m, 0, img_dim - 1)
    ntx = (img_dim + tile - 1) // tile
    key = (m[:, 1] // tile) * ntx + (m[:, 0] // tile)
    return np.argsort(key, kind="stable")


def job_tracks(img_dim: int, nvis: int, seed: int, device="cpu", nant: int = 64,
               ntime: int = 2080, ha_hours: float = 4.0, dec_deg: float = -30.0,
               fill: float = 0.9, radius_m: float = 1000.0):
    """One request's own observation (the batched and served workloads): an
    array of nant antennas at random positions in a disk of radius_m -- its
    own layout, drawn from `seed` -- of which ceil(nvis / ntime) baselines,
    picked at random, are tracked over ntime hour angles in [-ha, ha] at
    declination dec_deg; (u, v) in pixels centred at img_dim / 2, scaled so
    that the array's longest baseline spans fill * img_dim / 2 (the largest
    |u|, |v| any of its tracks can reach); float-representable coordinates;
    complex64 N(0, 1) values.  Baseline-major, time-minor, cut to nvis.
    Computed with torch on `device` (the layout and the baseline choice on
    the host from `seed`, the values from a generator of `device` seeded
    with it).  Returns (uv float64 (nvis, 2), vals complex64 (nvis,))
    tensors on `device`."""
    import torch
    g = torch.Generator().manual_seed(int(seed))
    r = radius_m * torch.sqrt(torch.rand(nant, generator=g, dtype=torch.float64))
    th = 2 * math.pi * torch.rand(nant, generator=g, dtype=torch.float64)
    ax, ay = r * torch.cos(th), r * torch.sin(th)
    i, j = torch.triu_indices(nant, nant, 1)
    bx, by = ax[j] - ax[i], ay[j] - ay[i]
    lmax = float(torch.sqrt(bx * bx + by * by).max())
    nbl = min(bx.numel(), -(-int(nvis) // ntime))
    pick = torch.randperm(bx.numel(), generator=g)[:nbl]
    bx, by = bx[pick].to(device), by[pick].to(device)
    ha = torch.linspace(-ha_hours, ha_hours, ntime, dtype=torch.float64,
                        device=device) * (math.pi / 12.0)
    sd = math.sin(math.radians(dec_deg))
    sh, ch = torch.sin(ha)[None, :], torch.cos(ha)[None, :]
    u = sh * bx[:, None] + ch * by[:, None]
    v = -sd * ch * bx[:, None] + sd * sh * by[:, None]
    scale = fill * (img_dim / 2) / lmax
    uv = torch.stack([img_dim / 2 + u.reshape(-1) * scale,
                      img_dim / 2 + v.reshape(-1) * scale], dim=1)[:nvis]
    uv = uv.float().double().contiguous()
    gd = torch.Generator(device=device).manual_seed(int(seed))
    vals = torch.randn(int(nvis), 2, generator=gd, device=device, dtype=torch.float32)
    return uv, torch.view_as_complex(vals.contiguous())


def request_specs(n: int, seed: int = 0, sides=(256, 512, 1024, 2048),
                  supports=(8, 16), nvis_min: float = 1e4, nvis_max: float = 1e6,
                  log10_mean: float = 5.0, log10_sd: float = 0.5):
    """Job / request shapes of the batched and served workloads: grid side
    uniform over `sides`, support uniform over `supports`, visibility count
    lognormal (log10 ~ N(log10_mean, log10_sd)) clipped to [nvis_min,
    nvis_max].  Each job's visibilities come from job_tracks."""
    rng = np.random.default_rng(seed)
    side = rng.choice(np.asarray(sides), n)
    S = rng.choice(np.asarray(supports), n)
    nvis = np.clip(10.0 ** rng.normal(log10_mean, log10_sd, n), nvis_min,
                   nvis_max).astype(np.int64)
    return {"side": side.astype(np.int64), "S": S.astype(np.int64), "nvis": nvis}


def gaussian_gcf_1d(gcf_dim: int, oversample: int = 8,
                    sigma: float | None = None) -> np.ndarray:
    """[G][S] factors g(a' - S/2 + 1 - s/G), g(x) = exp(-x^2 / (2 sigma^2))"""
    if sigma is None:
        sigma = gcf_dim / 4.0
    s = np.arange(oversample)[:, None]
    a = np.arange(gcf_dim)[None, :]
    x = (a - gcf_dim // 2 + 1) - s / oversample
    return np.exp(-(x * x) / (2.0 * sigma * sigma))


def gcf_table(g1: np.ndarray) -> np.ndarray:
    """complex128 [G*G, S, S] table from 1-D factors (exact products)."""
    G, S = g1.shape
    t = g1[None, :, None, :] * g1[:, None, :, None]       # [sy, sx, b', a']
    return t.reshape(G * G, S, S).astype(np.complex128)
