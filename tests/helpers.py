"""Shared test helpers: golden fixtures, error metrics, oracle calls."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    """(uv (n,2) f64, vals (n*P,2) f64, gcf (G*G*S*S,2) f64, out (2,P,N,N), meta)"""
    import oracle as O
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "g1" in z:
        g = O.gcf_from_1d(z["g1"])
        gcf = np.stack([g.real, g.imag], -1).reshape(-1, 2)
    else:
        gcf = z["gcf"]
    N, S, P, dbg = (int(x) for x in z["meta"])
    return dict(uv=z["uv"], vals=z["vals"], gcf=gcf, out=z["out"], N=N, S=S,
                P=P, debug1=bool(dbg), g1=z["g1"] if "g1" in z else None)


def rel_err(a, ref):
    """max |a - ref| / max |ref| over all cells (normwise relative error)"""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.abs(ref).max()
    return float(np.abs(a - ref).max() / (den if den > 0 else 1.0))


def cell_err(a, ref, mag):
    """Per-cell forward error of a planar grid a (2, P, N, N) against the
    oracle ref: |a - ref| (complex modulus) / mag at every cell, mag the
    oracle's sum of |val| * |w| over that cell's additions (O.grid_mag,
    shape (P, N, N)).  Returns (max, rms) over the cells with mag > 0; a
    nonzero value at a cell with mag == 0 counts as an infinite error."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    mag = np.asarray(mag, np.float64).reshape(a.shape[1:])
    d = np.hypot(a[0] - ref[0], a[1] - ref[1])
    hit = mag > 0
    if np.any(d[~hit] != 0):
        return float("inf"), float("inf")
    if not hit.any():
        return 0.0, 0.0
    e = d[hit] / mag[hit]
    return float(e.max()), float(np.sqrt((e * e).mean()))


def rms_rel_err(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.sqrt((ref ** 2).sum())
    return float(np.sqrt(((a - ref) ** 2).sum()) / (den if den > 0 else 1.0))


def to_complex(pairs):
    pairs = np.asarray(pairs)
    return pairs[..., 0] + 1j * pairs[..., 1]


def planar_from_grid(grid, P, N, layout_planar):
    """device grid (flat, complex or real) -> planar (2, P, N, N) float64"""
    g = np.asarray(grid)
    if np.iscomplexobj(g):
        g = g.reshape(P, N, N)
        return np.stack([g.real, g.imag]).astype(np.float64)
    g = g.reshape(-1).astype(np.float64)
    if layout_planar:
        return g.reshape(2, P, N, N)
    c = g.reshape(P, N, N, 2)
    return np.moveaxis(c, -1, 0)
