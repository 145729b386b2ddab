"""Python host side of the GB300 gridder: a ctypes binding of libgg.so.

Mirrors the reference's interfaces for the gridding path:

* ``gridGPU(out, in_, in_vals, npts, img_dim, gcf, gcf_dim)`` -- the drop-in
  entry point (grid_gpu.cuh:30-32) on host numpy arrays: padded ``out``,
  un-offset ``gcf``, dispatch on the element types of the three explicit
  instantiations (grid_gpu.cu:820-825).
* ``convgrid(in_, npts, in_vals, img_size, gcf, Qpx, gcf_dim)`` -- the Python
  module function of GPUGrid.cpp:124-164, for Python 3, returning the
  img_size x img_size grid (the reference returned an npts-sized buffer).
* ``Context.grid(...)`` -- device-resident gridding of torch CUDA tensors on
  the current torch stream (no host copies), and ``Context.grid_batch``.

Compile-time switches of the reference (Defines.h, Makefile) are the fields
of ``Options``.  There is no CPU fallback: importing this module fails when
libgg.so is missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgg.so")

# ---- constants of include/gg.h --------------------------------------------
OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_UNSORTED, ERR_BUDGET, ERR_TIMEOUT, \
    ERR_CANCELLED, ERR_STATE = range(9)
C64, C128 = 0, 1
MODE_SCATTER, MODE_GATHER, MODE_WINDOW, MODE_AUTO = range(4)
LAYOUT_INTERLEAVED, LAYOUT_PLANAR, LAYOUT_REFERENCE = range(3)
ACC_PLAIN, ACC_COMPENSATED = range(2)
GCF_TABLE, GCF_GAUSSIAN, GCF_COUNT, GCF_WPHASE = range(4)
DEVFLAG_INDEX, DEVFLAG_TIMEOUT, DEVFLAG_UNSORTED, DEVFLAG_BOUNDS = 1, 2, 4, 8

MODES = {"scatter": MODE_SCATTER, "gather": MODE_GATHER,
         "window": MODE_WINDOW, "auto": MODE_AUTO}


class GridError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gg error {code}: {msg}")
        self.code = code


class gg_options(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("accum", ctypes.c_int32), ("gcf_kind", ctypes.c_int32),
                ("oversample", ctypes.c_int32),
                ("polarizations", ctypes.c_int32), ("tile", ctypes.c_int32),
                ("input_sorted", ctypes.c_int32),
                ("gcf_sigma", ctypes.c_double),
                ("window_chunk", ctypes.c_int32),
                ("group_warps", ctypes.c_int32),
                ("autotune", ctypes.c_int32),
                ("accumulate", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 4)]


class gg_job(ctypes.Structure):
    _fields_ = [("out", ctypes.c_void_p), ("uv", ctypes.c_void_p),
                ("vals", ctypes.c_void_p), ("gcf", ctypes.c_void_p),
                ("npts", ctypes.c_int64), ("img_dim", ctypes.c_int64),
                ("gcf_dim", ctypes.c_int64), ("uv_type", ctypes.c_int32),
                ("vals_type", ctypes.c_int32), ("out_type", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("gcf_sigma", ctypes.c_double),
                ("gcf_index", ctypes.c_void_p), ("n_gcf", ctypes.c_int64),
                ("reserved", ctypes.c_int64 * 2)]


REQ_INPUTS_ON_DEVICE, REQ_OUT_ON_DEVICE, REQ_KEEP_RESIDENT = 1, 2, 4
# the server times autotuner trials only during its first batches
SERVER_TUNE_BATCHES = 32


class gg_server_config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("streams", ctypes.c_int32),
                ("max_batch_jobs", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("max_batch_vis", ctypes.c_int64), ("hbm_budget_bytes", ctypes.c_int64),
                ("options", gg_options), ("reserved", ctypes.c_int64 * 4)]


class gg_request(ctypes.Structure):
    _fields_ = [("uv", ctypes.c_void_p), ("vals", ctypes.c_void_p),
                ("out", ctypes.c_void_p), ("npts", ctypes.c_int64),
                ("img_dim", ctypes.c_int64), ("gcf_dim", ctypes.c_int64),
                ("uv_type", ctypes.c_int32), ("vals_type", ctypes.c_int32),
                ("out_type", ctypes.c_int32), ("gcf_id", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("reserved", ctypes.c_int64 * 3)]


class gg_result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("device_flags", ctypes.c_int32),
                ("latency_s", ctypes.c_double), ("queue_s", ctypes.c_double),
                ("device_out", ctypes.c_void_p)]


class gg_server_stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in
                ("submitted", "completed", "failed", "rejected", "cancelled",
                 "batches", "visibilities")] + \
               [(n, ctypes.c_double) for n in
                ("span_s", "p50_latency_s", "p99_latency_s", "mean_latency_s",
                 "mean_batch_jobs")] + \
               [("hbm_in_use", ctypes.c_int64), ("hbm_peak", ctypes.c_int64)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64, sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
    P = ctypes.POINTER
    sig = {
        "gg_abi_version": ([], ctypes.c_int),
        "gg_last_error": ([], ctypes.c_char_p),
        "gg_default_options": ([P(gg_options)], ctypes.c_int),
        "gg_set_global_options": ([P(gg_options)], ctypes.c_int),
        "gg_get_global_options": ([P(gg_options)], ctypes.c_int),
        "gg_gridGPU_zz": ([vp, vp, vp, sz, sz, vp, sz], ctypes.c_int),
        "gg_gridGPU_zc": ([vp, vp, vp, sz, sz, vp, sz], ctypes.c_int),
        "gg_gridGPU_cc": ([vp, vp, vp, sz, sz, vp, sz], ctypes.c_int),
        "gg_grid_host": ([P(gg_options), ctypes.c_int, vp, ctypes.c_int, vp,
                          ctypes.c_int, vp, sz, sz, vp, sz], ctypes.c_int),
        "gg_create": ([P(vp), ctypes.c_int], ctypes.c_int),
        "gg_destroy": ([vp], ctypes.c_int),
        "gg_reserve": ([vp, P(gg_options), i64, i64, i64, i32], ctypes.c_int),
        "gg_workspace_bytes": ([vp, P(sz)], ctypes.c_int),
        "gg_grid_device": ([vp, P(gg_options), P(gg_job), vp], ctypes.c_int),
        "gg_degrid_device": ([vp, P(gg_options), P(gg_job), vp], ctypes.c_int),
        "gg_grid_to_image": ([vp, vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, vp],
                             ctypes.c_int),
        "gg_grid_batch": ([vp, P(gg_options), P(gg_job), i32, vp], ctypes.c_int),
        "gg_read_flags": ([vp, vp, P(i32)], ctypes.c_int),
        "gg_profile_enable": ([vp, ctypes.c_int], ctypes.c_int),
        "gg_profile_last": ([vp, P(ctypes.c_double)], ctypes.c_int),
        "gg_kernel_launches": ([P(i64)], ctypes.c_int),
        "gg_vis2ints": ([ctypes.c_int, vp, i64, i32, vp, vp], ctypes.c_int),
        "gg_bin": ([vp, P(gg_options), ctypes.c_int, vp, i64, i64, i64, vp, vp,
                    vp], ctypes.c_int),
        "gg_plan_create": ([vp, P(gg_options), P(gg_job), i32, P(vp)], ctypes.c_int),
        "gg_plan_launch": ([vp, vp], ctypes.c_int),
        "gg_plan_read_flags": ([vp, vp, P(i32)], ctypes.c_int),
        "gg_plan_destroy": ([vp], ctypes.c_int),
        "gg_server_default_config": ([P(gg_server_config)], ctypes.c_int),
        "gg_server_create": ([P(vp), P(gg_server_config)], ctypes.c_int),
        "gg_server_add_gcf": ([vp, vp, i32, i64, P(i32)], ctypes.c_int),
        "gg_server_submit": ([vp, P(gg_request), P(i64)], ctypes.c_int),
        "gg_server_submit_schedule": ([vp, P(gg_request), P(ctypes.c_double), i64,
                                       P(i64)], ctypes.c_int),
        "gg_server_wait": ([vp, i64, ctypes.c_double, P(gg_result)], ctypes.c_int),
        "gg_server_release": ([vp, i64], ctypes.c_int),
        "gg_server_cancel": ([vp, i64], ctypes.c_int),
        "gg_server_get_stats": ([vp, P(gg_server_stats), ctypes.c_int], ctypes.c_int),
        "gg_server_drain": ([vp, ctypes.c_double], ctypes.c_int),
        "gg_server_destroy": ([vp], ctypes.c_int),
        "gg_autotune_clear": ([], ctypes.c_int),
        "gg_selftest_wait_timeout": ([vp, vp], ctypes.c_int),
        "gg_debug_inject_alloc_failures": ([i32], ctypes.c_int),
        "gg_debug_inject_device_flags": ([i32, i32], ctypes.c_int),
        "gg_grid_device_noalloc": ([P(gg_options), P(gg_job), vp], ctypes.c_int),
        "gg_autotune_report": ([ctypes.c_char_p, sz], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


LIB = _load()


def _check(code: int) -> None:
    if code != OK:
        raise GridError(code, LIB.gg_last_error().decode(errors="replace"))


@dataclass
class Options:
    """The reference's compile-time switches as run-time fields."""
    mode: int = MODE_SCATTER            # Makefile GATHER= / MOVING_WINDOW=
    layout: int = LAYOUT_REFERENCE
    accum: int = ACC_PLAIN
    gcf_kind: int = GCF_TABLE           # COMPUTE_GCF=1 -> GCF_WPHASE (or GCF_GAUSSIAN)
    oversample: int = 8                 # GCF_GRID
    polarizations: int = 1              # POLARIZATIONS
    tile: int = 0                       # 0: chosen by method and support
    input_sorted: bool = False
    gcf_sigma: float = 0.0
    window_chunk: int = 0
    group_warps: int = 0                # moving window: warps per sub-grid
    autotune: int = 0                   # moving window: tile / warps / chunk by timing
                                        # (1: time new size classes, 2: reuse choices)
    accumulate: bool = False            # device entry points: add into `out`

    def c(self) -> gg_options:
        o = gg_options()
        _check(LIB.gg_default_options(ctypes.byref(o)))
        mode = MODES.get(self.mode, self.mode) if isinstance(self.mode, str) else self.mode
        o.mode, o.layout, o.accum, o.gcf_kind = mode, self.layout, self.accum, self.gcf_kind
        o.oversample, o.polarizations, o.tile = self.oversample, self.polarizations, self.tile
        o.input_sorted = int(bool(self.input_sorted))
        o.gcf_sigma, o.window_chunk = self.gcf_sigma, self.window_chunk
        o.group_warps = self.group_warps
        o.autotune = int(self.autotune)
        o.accumulate = int(bool(self.accumulate))
        return o


def set_global_options(opts: Options) -> None:
    """Options used by gridGPU / convgrid (the Defines.h of a build)."""
    _check(LIB.gg_set_global_options(ctypes.byref(opts.c())))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def padded_size(img_dim: int, gcf_dim: int, pols: int = 1) -> int:
    """Elements of gridGPU's output buffer (grid.cu:290)."""
    return (img_dim * img_dim + 2 * img_dim * gcf_dim + 2 * gcf_dim) * pols


def grid_head(img_dim: int, gcf_dim: int) -> int:
    """Element offset of the grid inside the padded buffer (grid_gpu.cu:732)."""
    return img_dim * gcf_dim + gcf_dim


def gridGPU(out: np.ndarray, in_: np.ndarray, in_vals: np.ndarray, npts: int,
            img_dim: int, gcf: np.ndarray, gcf_dim: int) -> None:
    """Drop-in gridGPU on host arrays; dtypes pick the instantiation:
    complex128 out/in -> <double2,double2>, complex128 out + complex64 in ->
    <double2,float2>, complex64 out/in -> <float2,float2>.  `in_` holds
    (u, v) as the real/imaginary parts of a complex array (CmplxType in[])."""
    for a in (out, in_, in_vals, gcf):
        if not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
    ot, it = out.dtype, in_.dtype
    if in_vals.dtype != it or gcf.dtype != it:
        raise TypeError("in, in_vals and gcf must share one dtype (CmplxType)")
    if ot == np.complex128 and it == np.complex128:
        f = LIB.gg_gridGPU_zz
    elif ot == np.complex128 and it == np.complex64:
        f = LIB.gg_gridGPU_zc
    elif ot == np.complex64 and it == np.complex64:
        f = LIB.gg_gridGPU_cc
    else:
        raise TypeError(f"no gridGPU instantiation for out={ot}, in={it}")
    _check(f(_ptr(out), _ptr(in_), _ptr(in_vals), npts, img_dim, _ptr(gcf), gcf_dim))


def grid_host(opts: Options, out: np.ndarray, uv: np.ndarray, vals: np.ndarray,
              npts: int, img_dim: int, gcf: np.ndarray | None, gcf_dim: int) -> None:
    """gg_grid_host: host buffers with explicit options and independent
    coordinate / value types."""
    def t(a):
        return C128 if a.dtype in (np.complex128, np.float64) else C64
    _check(LIB.gg_grid_host(ctypes.byref(opts.c()), t(out), _ptr(out), t(uv), _ptr(uv),
                            t(vals), _ptr(vals), npts, img_dim,
                            _ptr(gcf) if gcf is not None else None, gcf_dim))


def convgrid(in_, npts: int, in_vals, img_size: int, gcf, Qpx: int,
             gcf_dim: int) -> np.ndarray:
    """GPUGrid.convgrid (GPUGrid.cpp:124-164) for Python 3.

    in_: 2*npts floats (u0, v0, u1, v1, ...); in_vals: npts complex; gcf:
    Qpx*Qpx*gcf_dim*gcf_dim complex.  Returns the complex128 grid
    (img_size, img_size).  Qpx is the oversampling factor (the reference
    ignored it and used GCF_GRID)."""
    uv = np.ascontiguousarray(np.asarray(in_, np.float64).reshape(npts, 2))
    uvc = uv[:, 0] + 1j * uv[:, 1]
    vals = np.ascontiguousarray(np.asarray(in_vals, np.complex128).reshape(-1))
    g = np.ascontiguousarray(np.asarray(gcf, np.complex128).reshape(-1))
    o = Options()
    LIBo = gg_options()
    _check(LIB.gg_get_global_options(ctypes.byref(LIBo)))
    o.mode, o.layout, o.accum, o.gcf_kind = LIBo.mode, LIBo.layout, LIBo.accum, LIBo.gcf_kind
    o.polarizations, o.tile = LIBo.polarizations, LIBo.tile
    o.oversample = int(Qpx)
    o.layout = LAYOUT_INTERLEAVED
    out = np.zeros(padded_size(img_size, gcf_dim, o.polarizations), np.complex128)
    grid_host(o, out, np.ascontiguousarray(uvc), vals, npts, img_size, g, gcf_dim)
    h = grid_head(img_size, gcf_dim)
    return out[h:h + img_size * img_size].reshape(img_size, img_size).copy()


# ---------------------------------------------------------------------------
# device-resident API on torch tensors
# ---------------------------------------------------------------------------

def _ttype(t) -> int:
    import torch
    if t.dtype in (torch.complex128, torch.float64):
        return C128
    if t.dtype in (torch.complex64, torch.float32):
        return C64
    raise TypeError(f"unsupported dtype {t.dtype}")


class Context:
    """A gg_context on one device: owns the workspace reused across calls."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(LIB.gg_create(ctypes.byref(self._h), device))
        self.device = device

    def close(self) -> None:
        if self._h:
            LIB.gg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def make_job(out, uv, vals, gcf, img_dim: int, gcf_dim: int,
                 npts: int | None = None, gcf_sigma: float = 0.0,
                 gcf_index=None, n_gcf: int = 1) -> gg_job:
        """gg_job over device tensors.  gcf_index (int32, one per visibility)
        selects one of n_gcf consecutive [G*G][S][S] tables at gcf."""
        j = gg_job()
        j.out = out.data_ptr()
        j.uv = uv.data_ptr() if uv is not None else None
        j.vals = vals.data_ptr() if vals is not None else None
        j.gcf = gcf.data_ptr() if gcf is not None else None
        j.npts = int(npts if npts is not None else (uv.numel() // 2 if uv.dtype.is_floating_point else uv.numel()))
        j.img_dim, j.gcf_dim = img_dim, gcf_dim
        j.uv_type = _ttype(uv) if uv is not None else C128
        j.vals_type = _ttype(vals) if vals is not None else C64
        j.out_type = _ttype(out)
        j.gcf_sigma = gcf_sigma
        if gcf_index is not None:
            j.gcf_index = gcf_index.data_ptr()
            j.n_gcf = int(n_gcf)
        return j

    def grid_job(self, opts: Options, job: gg_job, stream=None) -> None:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(LIB.gg_grid_device(self._h, ctypes.byref(opts.c()), ctypes.byref(job),
                                  ctypes.c_void_p(s.cuda_stream)))

    def grid(self, opts: Options, out, uv, vals, gcf, img_dim: int, gcf_dim: int,
             stream=None, gcf_sigma: float = 0.0) -> None:
        """Grid device tensors into `out` (overwritten) on the current stream."""
        self.grid_job(opts, self.make_job(out, uv, vals, gcf, img_dim, gcf_dim,
                                          gcf_sigma=gcf_sigma), stream)

    def degrid(self, opts: Options, grid, uv, vals_out, gcf, img_dim: int, gcf_dim: int,
               stream=None, gcf_sigma: float = 0.0, gcf_index=None, n_gcf: int = 1) -> None:
        """Degrid (the adjoint of grid): vals_out (npts*P complex, written)
        gets, per visibility and plane, the sum over its on-grid taps of
        grid * conj(table entry).  grid: P planes of N*N complex (planar when
        opts.layout is LAYOUT_PLANAR, else interleaved)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        job = self.make_job(grid, uv, vals_out, gcf, img_dim, gcf_dim, gcf_sigma=gcf_sigma,
                            gcf_index=gcf_index, n_gcf=n_gcf)
        _check(LIB.gg_degrid_device(self._h, ctypes.byref(opts.c()), ctypes.byref(job),
                                    ctypes.c_void_p(s.cuda_stream)))

    def grid_to_image(self, grid, img_dim: int, pols: int = 1, stream=None) -> None:
        """In place: each of the `pols` interleaved N*N complex planes of the
        device tensor `grid` becomes its dirty image (centred inverse 2-D
        DFT, no normalisation; N even).  Synchronises the stream."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(LIB.gg_grid_to_image(self._h, ctypes.c_void_p(grid.data_ptr()), img_dim, pols,
                                    _ttype(grid), ctypes.c_void_p(s.cuda_stream)))

    def grid_batch(self, opts: Options, jobs: list[gg_job], stream=None) -> None:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        arr = (gg_job * len(jobs))(*jobs)
        _check(LIB.gg_grid_batch(self._h, ctypes.byref(opts.c()), arr, len(jobs),
                                 ctypes.c_void_p(s.cuda_stream)))

    def read_flags(self, stream=None) -> list[int]:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        f = (ctypes.c_int32 * 4)()
        _check(LIB.gg_read_flags(self._h, ctypes.c_void_p(s.cuda_stream), f))
        return list(f)

    def profile(self, on: bool = True) -> None:
        _check(LIB.gg_profile_enable(self._h, int(on)))

    def profile_last(self) -> tuple[float, float, float]:
        """(set-up+binning ms, gridding-kernel ms, whole-call ms) of the last
        call, timed with CUDA events on its stream."""
        ms = (ctypes.c_double * 3)()
        _check(LIB.gg_profile_last(self._h, ms))
        return ms[0], ms[1], ms[2]

    def reserve(self, opts: Options, max_npts: int, max_img_dim: int,
                max_gcf_dim: int, vals_type: int = C64) -> None:
        _check(LIB.gg_reserve(self._h, ctypes.byref(opts.c()), max_npts, max_img_dim,
                              max_gcf_dim, vals_type))

    def workspace_bytes(self) -> int:
        n = ctypes.c_size_t()
        _check(LIB.gg_workspace_bytes(self._h, ctypes.byref(n)))
        return n.value

    def bin(self, opts: Options, uv, img_dim: int, gcf_dim: int, stream=None):
        """(bookmarks, order) device tensors of gg_bin."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        npts = uv.shape[0]
        ntx = (img_dim + opts.tile - 1) // opts.tile
        bm = torch.empty(ntx * ntx + 1, dtype=torch.int32, device=uv.device)
        order = torch.full((npts,), -1, dtype=torch.int32, device=uv.device)
        _check(LIB.gg_bin(self._h, ctypes.byref(opts.c()), _ttype(uv), uv.data_ptr(),
                          npts, img_dim, gcf_dim, bm.data_ptr(), order.data_ptr(),
                          ctypes.c_void_p(s.cuda_stream)))
        return bm, order


class Plan:
    """A batch of jobs fixed once (gg_plan_create); launch() only enqueues
    memsets and kernels, so it can be captured into a CUDA graph."""

    def __init__(self, ctx: Context, opts: Options, jobs: list[gg_job]):
        self._h = ctypes.c_void_p()
        arr = (gg_job * len(jobs))(*jobs)
        _check(LIB.gg_plan_create(ctx._h, ctypes.byref(opts.c()), arr, len(jobs),
                                  ctypes.byref(self._h)))
        self.ctx = ctx

    def launch(self, stream=None) -> None:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.ctx.device)
        _check(LIB.gg_plan_launch(self._h, ctypes.c_void_p(s.cuda_stream)))

    def read_flags(self, stream=None) -> list[int]:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.ctx.device)
        f = (ctypes.c_int32 * 4)()
        _check(LIB.gg_plan_read_flags(self._h, ctypes.c_void_p(s.cuda_stream), f))
        return list(f)

    def close(self) -> None:
        if self._h:
            LIB.gg_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """gg_server: admission by HBM budget and continuous batching."""

    def __init__(self, device: int = 0, streams: int = 2, max_batch_jobs: int = 256,
                 max_batch_vis: int = 1 << 26, hbm_budget: float = 150e9,
                 options: Options | None = None):
        cfg = gg_server_config()
        _check(LIB.gg_server_default_config(ctypes.byref(cfg)))
        cfg.device, cfg.streams = device, streams
        cfg.max_batch_jobs, cfg.max_batch_vis = max_batch_jobs, max_batch_vis
        cfg.hbm_budget_bytes = int(hbm_budget)
        if options is not None:
            cfg.options = options.c()
        self._h = ctypes.c_void_p()
        _check(LIB.gg_server_create(ctypes.byref(self._h), ctypes.byref(cfg)))

    def add_gcf(self, table: np.ndarray) -> int:
        t = np.ascontiguousarray(table)
        gid = ctypes.c_int32()
        vt = C128 if t.dtype == np.complex128 else C64
        S = t.shape[-1]
        _check(LIB.gg_server_add_gcf(self._h, t.ctypes.data, vt, S, ctypes.byref(gid)))
        return gid.value

    @staticmethod
    def request(uv_ptr, vals_ptr, out_ptr, npts, img_dim, gcf_dim, gcf_id=-1,
                flags=0, uv_type=C128, vals_type=C64, out_type=C64) -> gg_request:
        r = gg_request()
        r.uv, r.vals, r.out = uv_ptr, vals_ptr, out_ptr
        r.npts, r.img_dim, r.gcf_dim = npts, img_dim, gcf_dim
        r.uv_type, r.vals_type, r.out_type = uv_type, vals_type, out_type
        r.gcf_id, r.flags = gcf_id, flags
        return r

    def submit(self, req: gg_request) -> int:
        t = ctypes.c_int64()
        _check(LIB.gg_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def submit_schedule(self, reqs: list[gg_request], offsets_s) -> np.ndarray:
        n = len(reqs)
        arr = (gg_request * n)(*reqs)
        off = np.ascontiguousarray(offsets_s, np.float64)
        tickets = np.zeros(n, np.int64)
        _check(LIB.gg_server_submit_schedule(
            self._h, arr, off.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
            tickets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return tickets

    def wait(self, ticket: int, timeout: float = -1.0, check: bool = True) -> gg_result:
        """The request's result; a failed request raises GridError unless
        ``check`` is false (then its ``status`` and ``device_flags`` tell)."""
        r = gg_result()
        st = LIB.gg_server_wait(self._h, ticket, timeout, ctypes.byref(r))
        if check or st == ERR_TIMEOUT and r.status == OK:
            _check(st)
        return r

    def release(self, ticket: int) -> None:
        _check(LIB.gg_server_release(self._h, ticket))

    def cancel(self, ticket: int) -> None:
        _check(LIB.gg_server_cancel(self._h, ticket))

    def stats(self, reset: bool = False) -> dict:
        s = gg_server_stats()
        _check(LIB.gg_server_get_stats(self._h, ctypes.byref(s), int(reset)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def drain(self, timeout: float = -1.0) -> None:
        _check(LIB.gg_server_drain(self._h, timeout))

    def close(self) -> None:
        if self._h:
            LIB.gg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def autotune_report() -> str:
    """the autotuner's choices so far, one line per size class"""
    buf = ctypes.create_string_buffer(1 << 16)
    _check(LIB.gg_autotune_report(buf, len(buf)))
    return buf.value.decode()


def autotune_clear() -> None:
    _check(LIB.gg_autotune_clear())


def inject_device_flags(bits: int, count: int = 1) -> None:
    """Test hook: the next ``count`` served batches / allocation-free calls get
    the GG_DEVFLAG_* ``bits`` raised in their device flag word (by a host-side
    kernel launch behind their gridding, before the flags are read back)."""
    _check(LIB.gg_debug_inject_device_flags(bits, count))


def grid_device_noalloc(opts: Options, job: gg_job, stream=None) -> None:
    """gg_grid_device_noalloc: moving-window gridding with the library's fixed
    scratch array (no allocation); asynchronous on the torch stream."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    _check(LIB.gg_grid_device_noalloc(ctypes.byref(opts.c()), ctypes.byref(job),
                                      ctypes.c_void_p(s.cuda_stream)))


def noalloc_flags(stream=None) -> list[int]:
    """flag counters of the last allocation-free call on the current device
    (gg_read_flags with a null context; synchronises the stream)"""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    f = (ctypes.c_int32 * 4)()
    _check(LIB.gg_read_flags(None, ctypes.c_void_p(s.cuda_stream), f))
    return list(f)


def kernel_launches() -> int:
    """kernels launched by libgg in this process so far"""
    n = ctypes.c_int64()
    _check(LIB.gg_kernel_launches(ctypes.byref(n)))
    return n.value


def vis2ints(uv, oversample: int = 8, stream=None):
    """gg_vis2ints on a (npts, 2) float64/float32 CUDA tensor -> int32 (npts, 2)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream(uv.device)
    out = torch.empty((uv.shape[0], 2), dtype=torch.int32, device=uv.device)
    _check(LIB.gg_vis2ints(_ttype(uv), uv.data_ptr(), uv.shape[0], oversample,
                           out.data_ptr(), ctypes.c_void_p(s.cuda_stream)))
    return out
