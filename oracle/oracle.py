"""CPU oracle loader -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only to check or time the reference
algorithm; the GPU gridder never calls it.

Two libraries are wrapped:

* ``liboracle.so``  -- ``grid_oracle.c``, a plain-C restatement of the
  reference's CPU gridder ``gridCPU_pz`` (grid.cu:140-193), of the index step
  (grid.cu:159-163, vis2ints grid_gpu.cu:352-365) and of ``set_bookmarks``
  (grid_gpu.cu:366-390).  Builds anywhere with ``make -C oracle``.
* ``_ref/libref_<N>_<S>_<P>_<prec>[_dbg].so`` -- the reference's own grid.cu
  compiled from its checkout (``make -C oracle ref``), one library per
  compile-time size class.  Present only where the reference checkout is.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_sz = ctypes.c_size_t


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, if asked, the reference libraries)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"] + (["ref"] if ref else []),
                   check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_grid_pz.argtypes = [_dp, _dp, _dp, _sz, _sz, _dp, _sz,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_grid_pz_mt.argtypes = L.oracle_grid_pz.argtypes + [ctypes.c_int]
        L.oracle_grid_pz_gcfinx.argtypes = [_dp, _dp, _dp, _ip, _sz, _sz, _dp, ctypes.c_int,
                                            _sz, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int]
        L.oracle_grid_pz_wphase.argtypes = [_dp, _dp, _dp, _sz, _sz, _dp, _sz, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int]
        L.oracle_grid_mag_pz.argtypes = [_dp, _dp, _dp, _ip, _sz, _sz, _dp, ctypes.c_int, _sz,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_degrid_pz.argtypes = [_dp, _dp, _dp, _ip, _sz, _sz, _dp, ctypes.c_int, _sz,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_vis2ints.argtypes = [_dp, _sz, ctypes.c_int, _ip]
        L.oracle_vis2ints_gpu_formula.argtypes = [_dp, _sz, ctypes.c_int, _ip]
        L.oracle_set_bookmarks.argtypes = [_ip, _sz, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, _ip]
        L.oracle_gaussian_gcf.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double]
        L.oracle_gcf_from_1d.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int]
        for f in (L.oracle_grid_pz, L.oracle_grid_pz_mt, L.oracle_grid_pz_gcfinx,
                  L.oracle_grid_pz_wphase, L.oracle_grid_mag_pz, L.oracle_degrid_pz,
                  L.oracle_vis2ints,
                  L.oracle_vis2ints_gpu_formula, L.oracle_set_bookmarks,
                  L.oracle_gaussian_gcf, L.oracle_gcf_from_1d):
            f.restype = None
        _LIB = L
    return _LIB


def _as_pairs(a) -> np.ndarray:
    """complex or (...,2) real array -> contiguous float64 (n,2)."""
    a = np.asarray(a)
    if np.iscomplexobj(a):
        a = np.stack([a.real, a.imag], axis=-1)
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 2)


def grid_pz(uv, vals, gcf, img_dim: int, gcf_dim: int, pols: int = 1,
            gcf_grid: int = 8, debug1: bool = False, nthreads: int = 1,
            out: np.ndarray | None = None) -> np.ndarray:
    """Grid like gridCPU_pz; returns the planar grid, shape (2, P, N, N)
    (real plane then imaginary plane).  ``out`` (same shape) accumulates."""
    uv = _as_pairs(uv)
    vals = _as_pairs(vals)
    gcf = _as_pairs(gcf)
    npts = uv.shape[0]
    assert vals.shape[0] == npts * pols
    assert gcf.shape[0] == gcf_grid * gcf_grid * gcf_dim * gcf_dim
    if out is None:
        out = np.zeros((2, pols, img_dim, img_dim), np.float64)
    assert out.flags.c_contiguous and out.dtype == np.float64
    args = (_ptr(out), _ptr(uv), _ptr(vals), npts, img_dim, _ptr(gcf),
            gcf_dim, gcf_grid, pols, int(debug1))
    if nthreads > 1:
        lib().oracle_grid_pz_mt(*args, nthreads)
    else:
        lib().oracle_grid_pz(*args)
    return out


def grid_pz_gcfinx(uv, vals, gcfinx, gcfs, img_dim: int, gcf_dim: int, pols: int = 1,
                   gcf_grid: int = 8, nthreads: int = 1) -> np.ndarray:
    """gridCPU_pz with a table per visibility: visibility n reads table
    gcfinx[n] of the stack ``gcfs`` (n_gcf tables of G*G*S*S complex);
    indices outside [0, n_gcf) are skipped.  Returns (2, P, N, N)."""
    uv = _as_pairs(uv)
    vals = _as_pairs(vals)
    tabs = _as_pairs(gcfs)
    per = gcf_grid * gcf_grid * gcf_dim * gcf_dim
    assert tabs.shape[0] % per == 0
    n_gcf = tabs.shape[0] // per
    npts = uv.shape[0]
    idx = np.ascontiguousarray(gcfinx, np.int32)
    assert idx.shape == (npts,) and vals.shape[0] == npts * pols
    out = np.zeros((2, pols, img_dim, img_dim), np.float64)
    lib().oracle_grid_pz_gcfinx(_ptr(out), _ptr(uv), _ptr(vals), _ptr(idx, _ip), npts, img_dim,
                                _ptr(tabs), n_gcf, gcf_dim, gcf_grid, pols, 0, max(1, nthreads))
    return out


def grid_mag(uv, vals, gcf, img_dim: int, gcf_dim: int, pols: int = 1,
             gcf_grid: int = 8, gcfinx=None, wphase: bool = False,
             nthreads: int = 1) -> np.ndarray:
    """Per-cell magnitude sums sum |val| * |w| over the additions gridCPU_pz
    makes into each cell (same taps, tables and COMPUTE_GCF factor): the
    denominator of the per-cell forward error.  ``gcf`` is one table or a
    stack selected by ``gcfinx``.  Returns (P, N, N) float64."""
    uv = _as_pairs(uv)
    vals = _as_pairs(vals)
    tabs = _as_pairs(gcf)
    per = gcf_grid * gcf_grid * gcf_dim * gcf_dim
    assert tabs.shape[0] % per == 0
    n_gcf = tabs.shape[0] // per
    npts = uv.shape[0]
    assert vals.shape[0] == npts * pols
    idx = None if gcfinx is None else np.ascontiguousarray(gcfinx, np.int32)
    assert idx is None or idx.shape == (npts,)
    out = np.zeros((pols, img_dim, img_dim), np.float64)
    lib().oracle_grid_mag_pz(_ptr(out), _ptr(uv), _ptr(vals),
                             None if idx is None else _ptr(idx, _ip), npts, img_dim,
                             _ptr(tabs), n_gcf, gcf_dim, gcf_grid, pols, int(wphase),
                             max(1, nthreads))
    return out


def degrid_pz(uv, grid, gcf, img_dim: int, gcf_dim: int, pols: int = 1,
              gcf_grid: int = 8, gcfinx=None, nthreads: int = 1) -> np.ndarray:
    """Degridding, the adjoint of grid_pz / grid_pz_gcfinx: visibility n, plane
    p gets the sum over its on-grid taps of grid[p][y][x] * conj(w), w the
    gridder's table entry for that tap.  ``grid`` is planar (2, P, N, N)
    (real planes, then imaginary planes), ``gcf`` one table or a stack of
    tables selected by ``gcfinx``.  Returns complex128 values, shape
    (npts, P); visibilities with an oversample or table index out of range
    get zero."""
    uv = _as_pairs(uv)
    tabs = _as_pairs(gcf)
    per = gcf_grid * gcf_grid * gcf_dim * gcf_dim
    assert tabs.shape[0] % per == 0
    n_gcf = tabs.shape[0] // per
    npts = uv.shape[0]
    g = np.ascontiguousarray(grid, np.float64)
    assert g.shape == (2, pols, img_dim, img_dim)
    out = np.zeros((npts * pols, 2), np.float64)
    idx = None if gcfinx is None else np.ascontiguousarray(gcfinx, np.int32)
    assert idx is None or idx.shape == (npts,)
    lib().oracle_degrid_pz(_ptr(out), _ptr(g), _ptr(uv),
                           None if idx is None else _ptr(idx, _ip), npts, img_dim, _ptr(tabs),
                           n_gcf, gcf_dim, gcf_grid, pols, max(1, nthreads))
    return (out[:, 0] + 1j * out[:, 1]).reshape(npts, pols)


def grid_pz_wphase(uv, vals, gcf, img_dim: int, gcf_dim: int, pols: int = 1,
                   gcf_grid: int = 8, nthreads: int = 1) -> np.ndarray:
    """gridCPU_pz with the reference scatter kernel's COMPUTE_GCF factor: every
    tap of a visibility gets (sin phi, cos phi), (T, w) taken from the entry
    S(S-1)/2-1 of ``gcf``.  Returns (2, P, N, N)."""
    uv = _as_pairs(uv)
    vals = _as_pairs(vals)
    gcf = _as_pairs(gcf)
    npts = uv.shape[0]
    out = np.zeros((2, pols, img_dim, img_dim), np.float64)
    lib().oracle_grid_pz_wphase(_ptr(out), _ptr(uv), _ptr(vals), npts, img_dim, _ptr(gcf),
                                gcf_dim, gcf_grid, pols, max(1, nthreads))
    return out


def vis2ints(uv, gcf_grid: int = 8, gpu_formula: bool = False) -> np.ndarray:
    uv = _as_pairs(uv)
    out = np.empty((uv.shape[0], 2), np.int32)
    f = lib().oracle_vis2ints_gpu_formula if gpu_formula else lib().oracle_vis2ints
    f(_ptr(uv), uv.shape[0], gcf_grid, _ptr(out, _ip))
    return out


def set_bookmarks(packed, blocksize: int, blockgrid: int,
                  gcf_grid: int = 8) -> np.ndarray:
    packed = np.ascontiguousarray(packed, np.int32).reshape(-1, 2)
    bm = np.full(blockgrid * blockgrid + 1, -1, np.int32)
    lib().oracle_set_bookmarks(_ptr(packed, _ip), packed.shape[0], gcf_grid,
                               blocksize, blockgrid, _ptr(bm, _ip))
    return bm


def gaussian_gcf(gcf_dim: int, sigma: float | None = None, gcf_grid: int = 8):
    """(table complex128 [G*G, S, S], g1 float64 [G, S]); sigma defaults to
    S/4, the separable Gaussian of the benchmark workloads."""
    if sigma is None:
        sigma = gcf_dim / 4.0
    tab = np.empty((gcf_grid * gcf_grid, gcf_dim, gcf_dim, 2), np.float64)
    g1 = np.empty((gcf_grid, gcf_dim), np.float64)
    lib().oracle_gaussian_gcf(_ptr(tab), _ptr(g1), gcf_dim, gcf_grid, sigma)
    return tab[..., 0] + 1j * tab[..., 1], g1


def gcf_from_1d(g1: np.ndarray) -> np.ndarray:
    g1 = np.ascontiguousarray(g1, np.float64)
    G, S = g1.shape
    tab = np.empty((G * G, S, S, 2), np.float64)
    lib().oracle_gcf_from_1d(_ptr(tab), _ptr(g1), S, G)
    return tab[..., 0] + 1j * tab[..., 1]


# ---------------------------------------------------------------------------
# the reference's own code, compiled by ``make -C oracle ref``
# ---------------------------------------------------------------------------

def ref_available(tag: str) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libref_{tag}.so"))


class RefLib:
    """One compile-time size class of the reference's grid.cu."""

    def __init__(self, tag: str):
        path = os.path.join(HERE, "_ref", f"libref_{tag}.so")
        self.L = ctypes.CDLL(path)
        p = (ctypes.c_int * 7)()
        self.L.ref_params(p)
        (self.img, self.gcf_dim, self.gcf_grid, self.pols, in_sz, out_sz,
         self.debug1) = list(p)
        self.in_dtype = np.float64 if in_sz == 16 else np.float32
        vp = ctypes.c_void_p
        self.L.ref_gridCPU_pz.argtypes = [vp, vp, vp, _sz, _sz, vp, _sz]
        self.L.ref_init_gcf.argtypes = [vp, _sz]
        for f in ("ref_sort_sub", "ref_sort_main", "ref_sort_grid"):
            getattr(self.L, f).argtypes = [vp, _sz]
        self.L.ref_harness_inputs.argtypes = [vp, vp, _sz]

    def _in(self, a):
        return np.ascontiguousarray(_as_pairs(a), self.in_dtype)

    def grid(self, uv, vals, gcf) -> np.ndarray:
        """gridCPU_pz into a zeroed padded buffer, as grid.cu:484-487 does;
        returns the planar grid (2, P, N, N) read from the unpadded head."""
        N, S, P = self.img, self.gcf_dim, self.pols
        uv, vals, gcf = self._in(uv), self._in(vals), self._in(gcf)
        npts = uv.shape[0]
        padded = np.zeros(((N * N + 2 * N * S + 2 * S) * P, 2), np.float64)
        head = padded[N * S + S:]
        self.L.ref_gridCPU_pz(head.ctypes.data, uv.ctypes.data,
                              vals.ctypes.data, npts, N, gcf.ctypes.data, S)
        flat = head.reshape(-1)[: 2 * P * N * N]
        return flat.reshape(2, P, N, N).copy()

    def init_gcf(self) -> np.ndarray:
        S, G = self.gcf_dim, self.gcf_grid
        g = np.zeros((G * G * S * S, 2), self.in_dtype)
        self.L.ref_init_gcf(g.ctypes.data, S)
        return g

    def harness_inputs(self, npts: int):
        uv = np.zeros((npts, 2), self.in_dtype)
        vals = np.zeros((npts * self.pols, 2), self.in_dtype)
        self.L.ref_harness_inputs(uv.ctypes.data, vals.ctypes.data, npts)
        return uv, vals

    def sort(self, uv, how: str) -> np.ndarray:
        uv = self._in(uv).copy()
        getattr(self.L, f"ref_sort_{how}")(uv.ctypes.data, uv.shape[0])
        return uv
