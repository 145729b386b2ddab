#!/usr/bin/env python3
"""Benchmark of the GB300 gridder; prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                    [--impl ours|reference]

Workloads (seeded synthetic visibilities with each configuration's shapes):

  served10k   (default) a stream of 10,000 gridding requests -- grid side
              uniform in {256,512,1024,2048}, support 8 or 16, visibility count
              lognormal in [1e4, 1e6], uv tracks -- through the request server
              (HBM-budget admission, continuous batching over CUDA streams,
              grids and GCF tables resident).  A step = the whole stream
              submitted at once (saturation); an arrival-rate sweep (Poisson)
              reports p50/p99 latency; the same stream through plain per-request
              launches is timed for comparison.
  batch256    256 such jobs in one batched plan captured in a CUDA graph.
  tracks4096  one 4096^2 job, 2^22 visibilities on uv tracks, support 8.
  uniform1024 one 1024^2 FP64 job, 2^18 uniform visibilities, support 16.
  disk8192    one 8192^2 job, 2^24 visibilities in a disk with 1% outliers,
              support 32, GCF computed on the fly.

`value` is Mvis/s with the inputs resident in HBM; `e2e` is the same metric
with the inputs copied from pinned host memory and the grids copied back,
inside the timed region, through the library's public API.

--impl reference times the reference's CPU gridder (gridCPU_pz, grid.cu:
140-193) on the host cores -- the C restatement in oracle/ split over all
host threads in row bands, bit-identical to the single-threaded reference --
on a bounded sample of the same workload.
Under torchrun each rank runs its own replica (independent jobs, weak
scaling); rank 0 prints the line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("ska-gpu-grid_gb300", "oracle"):
    sys.path.insert(0, os.path.join(ROOT, sub))

import numpy as np  # noqa: E402

METRIC = ("gridded Mvis/s batched+served vs plain kernel at <=1e-6 rel err; "
          "p50/p99 latency")
FALLBACK_HBM_GBS = 6800.0

STREAM_DESC = ("grid side uniform in {256,512,1024,2048}; support 8 or 16, "
               "oversample 8; visibility count lognormal (log10 ~ N(5, 0.5)) "
               "clipped to [1e4, 1e6]; every job its own observation with the "
               "tracks4096 geometry: its own 64 antennas at random positions in "
               "a 2 km disk, whole tracks of a random choice of its 2016 "
               "baselines, 2080 samples over +-4 h, dec -30 deg, the longest "
               "baseline at 90% fill; complex64 N(0,1) values; FP32 "
               "u,v (float2, as the reference's FP32 instantiation "
               "gridGPU<float2,float2> takes them); complex64 grids; FP32 "
               "compensated accumulation; "
               "tabulated separable Gaussian GCFs resident on the device")

WORKLOADS = {
    "served10k": dict(kind="served", n=10000, streams=3, max_batch_jobs=512,
                      max_batch_vis=1 << 26, budget=150e9,
                      desc="10,000 Poisson-arrival gridding requests: " + STREAM_DESC +
                           "; HBM admission budget 150 GB"),
    "batch256": dict(kind="batch", n=256,
                     desc="256 independent gridding jobs in one batched "
                          "launch captured in a CUDA graph: " + STREAM_DESC),
    "tracks4096": dict(
        kind="single", N=4096, S=8, npts=1 << 22, gen="tracks", vals="c64", out="c64",
        uv="f32", mode="auto", accum="comp", presort=True,
        desc=("4096^2 complex64 grid; 2^22 visibilities on uv tracks (64 "
              "antennas in a 2 km disk, 2016 baselines x 2080 hour angles over "
              "+-4 h at dec -30 deg, 90% fill, +1024 to 2^22); complex64 N(0,1) "
              "values; FP32 u,v (float2, as gridGPU<float2,float2> takes them); "
              "support 8, oversample 8; presorted into 32x32 uv tiles; FP32 "
              "compensated accumulation")),
    "uniform1024": dict(
        kind="single", N=1024, S=16, npts=1 << 18, gen="uniform", vals="c128", out="c128",
        mode="scatter", accum="plain",
        desc=("1024^2 complex128 grid; 2^18 visibilities uniform in "
              "[16, 1008); complex128 N(0,1) values; support 16, oversample 8; "
              "FP64 scatter")),
    "disk8192": dict(
        kind="single", N=8192, S=32, npts=1 << 24, gen="disk", vals="c64", out="c128",
        mode="auto", accum="comp", gcf="gauss", precision_study=True, check_window=1024,
        desc=("8192^2 grid (complex128 output of FP32 compensated "
              "accumulation); 2^24 visibilities, uniform disk; N(0,1) values "
              "with 1% outliers at 1e3; support 32, oversample 8; GCF computed "
              "on the fly")),
}
WORKLOADS["degrid4096"] = dict(
    kind="degrid", N=4096, S=8, npts=1 << 22, gen="tracks", vals="c64", out="c64",
    mode="window", accum="comp", presort=True,
    desc=("degridding (the gridder's adjoint) of the tracks4096 visibilities from "
          "their own 4096^2 complex64 grid: 2^22 predicted complex64 values, "
          "support 8, oversample 8, tabulated Gaussian GCF, FP32 compensated "
          "lane sums"))
DEFAULT_WORKLOAD = "served10k"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def pairs(c):
    c = np.asarray(c).reshape(-1)
    return np.stack([c.real, c.imag], -1).astype(np.float64)


class nvtx_range:
    """an NVTX range around a region (a profiler can select the launches in
    it: ncu --nvtx --nvtx-include "gg_profiled/"); a no-op without NVTX"""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        try:
            import torch
            torch.cuda.nvtx.range_push(self.name)
            self.on = True
        except Exception:
            self.on = False

    def __exit__(self, *exc):
        if self.on:
            import torch
            torch.cuda.nvtx.range_pop()


def max_over_ranks(x, dist, dev=None):
    """the largest value of x over all ranks (x unchanged without a process
    group): every rank's timed region ends when the slowest rank's does"""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64,
                     device=dev if dev is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, world, seconds):
    """whole-job throughput of `world` replicas that each processed
    units_per_rank in `seconds` (the max over ranks), in millions per second"""
    return world * units_per_rank / seconds / 1e6


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.f:
            return None
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                rows.append((float(p[1]), float(p[2]), float(p[3]), p[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return None
        load = [r for r in rows if r[2] > 150.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3])
                          if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in load),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(load)}


def peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_from_profile(tag):
    """dram bytes per launch recorded from an ncu capture (profiles/)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", f"{tag}.txt")):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


_RED = {}


def red_peaks(dev):
    """FP32 global-reduction rates of this GPU (libgg_probe.so), once per run:
    red.global.add.v2.f32 / .f32 per second over an L2-resident array (32 MB),
    an HBM-sized one (2 GB) and 1024 contended cells."""
    if _RED:
        return _RED
    try:
        lib = ctypes.CDLL(os.path.join(ROOT, "ska-gpu-grid_gb300", "libgg_probe.so"))
        lib.gg_probe_red_rate.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        for name, cells, v2, pat in (("v2_coalesced_l2", 1 << 22, 1, 0),
                                     ("v2_scattered_l2", 1 << 22, 1, 1),
                                     ("v2_scattered_hbm", 1 << 28, 1, 1),
                                     ("v2_contended_1024", 1 << 10, 1, 1),
                                     ("f32_scattered_l2", 1 << 22, 0, 1)):
            r = ctypes.c_double()
            if lib.gg_probe_red_rate(dev, cells, v2, pat, ctypes.byref(r)) == 0:
                _RED[name] = round(r.value / 1e9, 2)
    except OSError:
        pass
    return _RED


def roofline(kernel, alg_bytes, kern_ms, tag, taps=None, dev=0):
    hbm, kind = peaks()
    achieved = alg_bytes / (kern_ms / 1e3) / 1e9
    out = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": hbm,
           "unit": "GB/s", "frac": round(achieved / hbm, 4), "peak_kind": f"{kind} (copy)",
           "traffic": traffic_from_profile(tag), "algorithmic_bytes_per_launch": int(alg_bytes)}
    red = red_peaks(dev)
    if taps and red.get("v2_scattered_l2"):
        rate = taps / (kern_ms / 1e3) / 1e9
        out["atomic"] = {
            "tap_updates_per_s_G": round(rate, 1),
            "red_v2_peak_G_per_s": red["v2_scattered_l2"],
            "frac": round(rate / red["v2_scattered_l2"], 3),
            "note": "grid-tap updates per second of the kernel vs the measured L2 rate of "
                    "scattered red.global.add.v2.f32, which bounds a scatter gridder "
                    "(one reduction per tap)",
            "measured_red_rates_G_per_s": red}
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement of gridCPU_pz on the host cores
# ---------------------------------------------------------------------------
# The CPU sample of a workload -- the same in the line's cpu_baseline and in
# the reference arm (--impl reference): for the request stream and the batch,
# the first whole jobs up to CPU_SAMPLE_VIS visibilities; for a single job, a
# prefix of its visibilities (smaller for support 32, whose taps cost 4x).
CPU_SAMPLE_VIS = 3_500_000


def stream_seed(kind, rank=0):
    return (7 if kind == "served" else 17) + rank


def cpu_sample(w, rank=0):
    """(jobs [(uv, vals, gcf, N, S)], description) of the workload's CPU sample"""
    if w["kind"] == "single":
        uv, vals, gcf = make_single(w, seed=1000 + rank)
        m = min(len(uv), (1 << 18) if w["S"] >= 32 else (1 << 20))
        return ([(uv[:m], vals[:m], gcf, w["N"], w["S"])],
                f"the first {m} visibilities of the workload")
    st = JobStream(w["n"], stream_seed(w["kind"], rank))
    jobs, vis = [], 0
    for i in range(w["n"]):
        N, S, n = st.shape(i)
        if jobs and vis + n > CPU_SAMPLE_VIS:
            break
        uv, vals = st.host_job(i)
        jobs.append((uv, vals, st.gcfs[S], N, S))
        vis += n
    return jobs, f"the first {len(jobs)} jobs of the stream ({vis} visibilities)"


def cpu_rate(jobs, threads=None):
    """Grids the sample once on the host cores (the oracle restatement of
    gridCPU_pz over all threads in row bands); returns (Mvis/s,
    visibilities, seconds, threads)."""
    import oracle as O
    threads = threads or os.cpu_count() or 1
    vis, spent = 0, 0.0
    for uv, vals, gcf, N, S in jobs:
        t0 = time.perf_counter()
        O.grid_pz(uv, pairs(vals), pairs(gcf), N, S, nthreads=threads)
        spent += time.perf_counter() - t0
        vis += len(uv)
    return vis / spent / 1e6, vis, spent, threads


def cpu_baseline(w, rank=0):
    jobs, desc = cpu_sample(w, rank)
    v, n, t, c = cpu_rate(jobs)
    return {"value": round(v, 4), "unit": "Mvis/s", "cores": c, "kind": "port",
            "sample": f"{desc}, {t:.2f} s; gridCPU_pz restatement (oracle/grid_oracle.c) "
                      f"over {c} row bands, bit-identical to the single-threaded reference"}


# ---------------------------------------------------------------------------
# shared pieces of the batched and served workloads
# ---------------------------------------------------------------------------
class JobStream:
    """The jobs of the batched and served workloads: shapes from
    synth.request_specs (grid side, support, visibility count), and for every
    job its own observation -- its own random 64-antenna array, tracks of a
    random choice of its baselines (synth.job_tracks, seeded with the job's
    index) -- generated with torch on the GPU when there is one, else on the
    host, once per job and kept."""

    def __init__(self, n, seed, device=None):
        import synth
        import torch
        self.specs = synth.request_specs(n, seed=seed + 1)
        self.seed = seed
        self.n = n
        self.device = device or ("cuda" if torch.cuda.is_available() else "cpu")
        self.gcfs = {S: synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(np.complex64)
                     for S in (8, 16)}
        self.dev = {}

    def shape(self, i):
        return (int(self.specs["side"][i]), int(self.specs["S"][i]),
                int(self.specs["nvis"][i]))

    def total_vis(self, n=None):
        return int(self.specs["nvis"][: self.n if n is None else n].sum())

    def device_job(self, i):
        """(uv float32 (n, 2), vals complex64 (n,)) tensors on the device; the
        coordinates are generated float-representable, so the float32 copy
        is exact"""
        if i not in self.dev:
            import synth
            N, _, n = self.shape(i)
            uv, v = synth.job_tracks(N, n, self.seed * 100003 + i, self.device)
            self.dev[i] = (uv.float().contiguous(), v)
        return self.dev[i]

    def generate(self, n=None):
        for i in range(self.n if n is None else n):
            self.device_job(i)

    def ptrs(self, i):
        uv, v = self.device_job(i)
        return uv.data_ptr(), v.data_ptr()

    def host_job(self, i):
        uv, v = self.device_job(i)
        return uv.cpu().numpy(), v.cpu().numpy()

    def device_bytes(self):
        return sum(uv.numel() * 4 + v.numel() * 8 for uv, v in self.dev.values())


ACC_NOTE = ("max_rel / rms_rel: normwise, |gpu - oracle| / max |oracle| (max) and "
            "||gpu - oracle|| / ||oracle|| (rms) over the grid; cell_max / cell_rms: per "
            "cell, |gpu - oracle| / sum |v||w| of the cell's additions (forward error of "
            "each cell's sum), over the cells that receive any")


class ErrAcc:
    """normwise and per-cell error of grids against the FP64 oracle,
    accumulated over several grids (planar (2, P, N, N) float64 each)"""

    def __init__(self):
        self.worst = self.num = self.den = 0.0
        self.cmax = self.csq = 0.0
        self.cells = 0

    def add(self, got, ref, mag):
        self.worst = max(self.worst, float(np.abs(got - ref).max() /
                                           max(np.abs(ref).max(), 1e-300)))
        self.num += float(((got - ref) ** 2).sum())
        self.den += float((ref ** 2).sum())
        d = np.hypot(got[0] - ref[0], got[1] - ref[1])
        hit = mag > 0
        if np.any(d[~hit] != 0):
            self.cmax = float("inf")
        e = d[hit] / mag[hit]
        if e.size:
            self.cmax = max(self.cmax, float(e.max()))
            self.csq += float((e * e).sum())
            self.cells += int(e.size)

    def result(self, **extra):
        r = {"max_rel": self.worst, "rms_rel": (self.num / max(self.den, 1e-300)) ** 0.5,
             "cell_max": self.cmax,
             "cell_rms": (self.csq / max(self.cells, 1)) ** 0.5}
        r.update(extra)
        r["reference"] = "FP64 oracle (gridCPU_pz restatement)"
        return r


def oracle_pair(uv, vals, gcf, N, S):
    """(planar FP64 grid, per-cell magnitude sums) of the oracle"""
    import oracle as O
    t = os.cpu_count() or 1
    return (O.grid_pz(uv, pairs(vals), pairs(gcf), N, S, nthreads=t),
            O.grid_mag(uv, pairs(vals), pairs(gcf), N, S, nthreads=t))


def window_reference(uv, vals, gcf, N, S, x0, y0, B):
    """Oracle of the B x B window [x0, x0+B) x [y0, y0+B) of an N^2 grid:
    every visibility whose footprint can reach the window, shifted by an
    integer offset (exact in FP64 and keeping u, v float-representable, so
    main and oversample indices shift exactly) onto a (B + 2S)^2 grid.
    Returns (ref, mag) of the window, planar (2, 1, B, B) and (1, B, B)."""
    m = np.floor(uv)
    keep = ((m[:, 0] >= x0 - S) & (m[:, 0] < x0 + B + S) &
            (m[:, 1] >= y0 - S) & (m[:, 1] < y0 + B + S))
    sub = uv[keep] - np.array([x0 - S, y0 - S], np.float64)
    ref, mag = oracle_pair(sub, vals[keep], gcf, B + 2 * S, S)
    return ref[:, :, S:S + B, S:S + B], mag[:, S:S + B, S:S + B], int(keep.sum())


def check_sample(grids, st, idx):
    """normwise and per-cell error of device grids vs the FP64 oracle"""
    acc = ErrAcc()
    for i, g in zip(idx, grids):
        uv, vals = st.host_job(i)
        N, S, _ = st.shape(i)
        ref, mag = oracle_pair(uv, vals, st.gcfs[S], N, S)
        got = np.stack([g.real, g.imag]).reshape(2, 1, N, N).astype(np.float64)
        acc.add(got, ref, mag)
    return acc.result(jobs_checked=len(idx), metrics=ACC_NOTE)


def stream_jobs(st, n, dev):
    """The first n jobs of a stream as batch jobs on device inputs: (jobs,
    grids, gcf tensors)."""
    import torch
    import gpugrid as gg
    dg = {S: torch.from_numpy(st.gcfs[S].reshape(-1)).to(dev) for S in (8, 16)}
    jobs, grids = [], []
    for i in range(n):
        N, S, nv = st.shape(i)
        pu, pv = st.ptrs(i)
        grids.append(torch.empty(N * N, dtype=torch.complex64, device=dev))
        j = gg.gg_job()
        j.out, j.uv, j.vals, j.gcf = grids[-1].data_ptr(), pu, pv, dg[S].data_ptr()
        j.npts, j.img_dim, j.gcf_dim = nv, N, S
        j.uv_type, j.vals_type, j.out_type = gg.C64, gg.C64, gg.C64
        jobs.append(j)
    return jobs, grids, dg


def profile_served_batch(args, st, opts, dev, local_rank):
    """--profile-batch: only the served line's roofline batch (the first 256
    requests in one batched call; only their inputs are generated, about 1
    GB), launched 3 times and once more inside the NVTX range gg_profiled --
    a case a profiler captures launch by launch.  Prints the kernel time and
    the algorithmic bytes of that launch."""
    import torch
    import gpugrid as gg
    n = min(256, st.n)
    jobs, grids, _ = stream_jobs(st, n, dev)
    ctx = gg.Context(local_rank)
    ctx.profile(True)
    for _ in range(3):
        ctx.grid_batch(opts, jobs)
    with nvtx_range("gg_profiled"):
        ctx.grid_batch(opts, jobs)
    _, kern_ms, _ = ctx.profile_last()
    torch.cuda.synchronize()
    nv = sum(j.npts for j in jobs)
    alg = nv * 16 + sum(2 * 8 * j.img_dim * j.img_dim for j in jobs)
    return {"profile_batch": f"first {n} requests of {args.workload}", "visibilities": nv,
            "window_kernels_ms": round(kern_ms, 4), "algorithmic_bytes": int(alg),
            "flags": ctx.read_flags(), "autotune": gg.autotune_report().splitlines()}


def cudart():
    f = ctypes.CDLL("libcudart.so.13")
    f.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    f.cudaMemcpy.restype = ctypes.c_int
    return f


# ---------------------------------------------------------------------------
# served stream of 10,000 requests -- the headline
# ---------------------------------------------------------------------------
def run_served(args, rank, world, local_rank, dist):
    import torch
    import gpugrid as gg
    w = WORKLOADS[args.workload]
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n = w["n"]
    js = JobStream(n, stream_seed("served", rank), dev)
    specs, gcfs = js.specs, js.gcfs
    total_vis = js.total_vis()
    opts = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                      layout=gg.LAYOUT_INTERLEAVED, autotune=True)
    if args.profile_batch:
        return profile_served_batch(args, js, opts, dev, local_rank)
    t_gen = time.perf_counter()
    js.generate()
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen
    srv = gg.Server(device=local_rank, streams=w["streams"], max_batch_jobs=w["max_batch_jobs"],
                    max_batch_vis=w["max_batch_vis"], hbm_budget=w["budget"], options=opts)
    gids = {S: srv.add_gcf(gcfs[S]) for S in (8, 16)}
    flags = gg.REQ_INPUTS_ON_DEVICE | gg.REQ_KEEP_RESIDENT
    reqs = []
    for i in range(n):
        N, S, nv = js.shape(i)
        pu, pv = js.ptrs(i)
        reqs.append(gg.Server.request(pu, pv, None, nv, N, S, gids[S], flags=flags,
                                      uv_type=gg.C64))

    def stream(offsets, keep=()):
        """submit all requests at the given arrival offsets; wait, release;
        returns (server span seconds, stats, kept grids)"""
        srv.stats(reset=True)
        tickets = srv.submit_schedule(reqs, offsets)
        kept = {}
        for k, t in enumerate(tickets):
            r = srv.wait(int(t), timeout=600)
            if k in keep:
                N = int(specs["side"][k])
                h = np.empty(N * N, np.complex64)
                cudart().cudaMemcpy(h.ctypes.data, ctypes.c_void_p(r.device_out), h.nbytes, 2)
                kept[k] = h
            srv.release(int(t))
        st = srv.stats()
        return st["span_s"], st, kept

    zeros = np.zeros(n)
    for _ in range(args.warmup):
        stream(zeros)
    # timed saturation passes (all arrivals at t=0); L2: the inputs (43 GB,
    # every request its own) exceed it
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = gg.kernel_launches()
    spans, stats = [], []
    with ClockSampler(local_rank) as clk:
        for _ in range(args.steps):
            span, st, _ = stream(zeros)
            spans.append(span)
            stats.append(st)
        torch.cuda.synchronize()
    launches = gg.kernel_launches() - l0
    total_s = sum(spans)
    total_s = max_over_ranks(total_s, dist, dev)
    value = replica_rate(total_vis * args.steps, world, total_s)

    # arrival-rate sweep (Poisson) up to saturation
    rng = np.random.default_rng(11)
    cap_rps = n / (total_s / args.steps)
    sweep = []
    for frac in (0.25, 0.5, 0.75, 0.9):
        rate = frac * cap_rps
        offs = np.cumsum(rng.exponential(1.0 / rate, n))
        span, st, _ = stream(offs)
        sweep.append({"load": frac, "rate_req_per_s": round(rate, 1),
                      "Mvis_per_s": round(total_vis / span / 1e6, 1),
                      "p50_ms": round(1e3 * st["p50_latency_s"], 3),
                      "p99_ms": round(1e3 * st["p99_latency_s"], 3),
                      "mean_batch_jobs": round(st["mean_batch_jobs"], 2)})
    sat = stats[-1]
    sweep.append({"load": "saturation (all at t=0)", "Mvis_per_s": round(value / world, 1),
                  "p50_ms": round(1e3 * sat["p50_latency_s"], 3),
                  "p99_ms": round(1e3 * sat["p99_latency_s"], 3),
                  "mean_batch_jobs": round(sat["mean_batch_jobs"], 2)})

    # accuracy on a sample of requests, from the server's resident grids
    sample = list(range(0, n, max(1, n // 12)))[:12]
    _, _, kept = stream(zeros, keep=set(sample))
    acc = check_sample([kept[i] for i in sample], js, sample) \
        if rank == 0 and not args.no_check else None

    # plain per-request launches on one stream (no batching)
    ctx = gg.Context(local_rank)
    outs = {N: torch.empty(N * N, dtype=torch.complex64, device=dev) for N in (256, 512, 1024, 2048)}
    dg = {S: torch.from_numpy(gcfs[S].reshape(-1)).to(dev) for S in (8, 16)}
    plain = {}
    for label, o in (("plain_scatter_per_request",
                      gg.Options(mode=gg.MODE_SCATTER, accum=gg.ACC_PLAIN,
                                 layout=gg.LAYOUT_INTERLEAVED)),
                     ("window_per_request",
                      gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                                 layout=gg.LAYOUT_INTERLEAVED))):
        jobs = []
        for i in range(n):
            N, S, nv = js.shape(i)
            pu, pv = js.ptrs(i)
            j = gg.gg_job()
            j.out, j.uv, j.vals, j.gcf = outs[N].data_ptr(), pu, pv, dg[S].data_ptr()
            j.npts, j.img_dim, j.gcf_dim = nv, N, S
            j.uv_type, j.vals_type, j.out_type = gg.C64, gg.C64, gg.C64
            jobs.append(j)
        for j in jobs[:50]:
            ctx.grid_job(o, j)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for j in jobs:
            ctx.grid_job(o, j)
        e1.record()
        torch.cuda.synchronize()
        plain[label] = round(total_vis / (e0.elapsed_time(e1) / 1e3) / 1e6, 1)

    # kernel-level roofline: the first 256 requests as one profiled batch
    ctx.profile(True)
    jobs, grid_out, _ = stream_jobs(js, min(256, n), dev)
    for _ in range(3):
        ctx.grid_batch(opts, jobs)
    with nvtx_range("gg_profiled"):
        ctx.grid_batch(opts, jobs)
    _, kern_ms, _ = ctx.profile_last()
    nv = sum(j.npts for j in jobs)
    alg = nv * 16 + sum(2 * 8 * j.img_dim * j.img_dim for j in jobs)
    taps = sum(j.npts * j.gcf_dim * j.gcf_dim for j in jobs)
    roof = roofline("window_kernel", alg, kern_ms, "window_served256", taps, local_rank)

    # e2e: host requests through the server's host path -- inputs copied in
    # from pinned host memory and every grid copied back to pinned host
    # memory by the server.  The client owns RING pinned output buffers per
    # grid side and reuses one only after the request that last used it is
    # complete (a bounded number of requests in flight, as a real client with
    # bounded host memory runs).
    e2e = None
    if not args.no_e2e:
        import collections
        import torch as _t
        # every request's inputs in pinned host memory (copied once from the
        # generated device inputs, outside the timed passes)
        h_uv = _t.empty((total_vis, 2), dtype=_t.float32).pin_memory()
        h_v = _t.empty(total_vis, dtype=_t.complex64).pin_memory()
        hoff, o = [], 0
        for i in range(n):
            uvd, vd = js.device_job(i)
            h_uv[o:o + len(uvd)].copy_(uvd)
            h_v[o:o + len(vd)].copy_(vd)
            hoff.append(o)
            o += len(uvd)
        torch.cuda.synchronize()
        sides = sorted({int(x) for x in specs["side"]})
        RING = args.e2e_ring
        hout = {N: [_t.empty(N * N, dtype=_t.complex64).pin_memory() for _ in range(RING)]
                for N in sides}
        hreqs, hbuf = [], []
        used = {N: 0 for N in sides}
        for i in range(n):
            N, S, nv_ = js.shape(i)
            b = used[N] % RING
            used[N] += 1
            hbuf.append((N, b))
            hreqs.append(gg.Server.request(h_uv.data_ptr() + hoff[i] * 8,
                                           h_v.data_ptr() + hoff[i] * 8,
                                           hout[N][b].data_ptr(), nv_, N, S, gids[S], flags=0,
                                           uv_type=gg.C64))

        def host_pass():
            owner = {}                       # (side, buffer) -> ticket using it
            fifo = collections.deque()
            for k in range(n):
                key = hbuf[k]
                if key in owner:             # wait until the buffer is free
                    while True:
                        t, kk = fifo.popleft()
                        srv.wait(t, timeout=600)
                        srv.release(t)
                        owner.pop(kk, None)
                        if kk == key:
                            break
                t = srv.submit(hreqs[k])
                owner[key] = t
                fifo.append((t, key))
            for t, _ in fifo:
                srv.wait(t, timeout=600)
                srv.release(t)

        host_pass()                          # warm-up (pins, pool growth)
        reps = max(1, min(args.steps, 3))
        t_all = 0.0
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            host_pass()
            t_all += time.perf_counter() - t0
        if rank == 0 and not args.no_check:
            # the last pass's grids in the buffers of the last requests
            last = {}
            for k in range(n):
                last[hbuf[k]] = k
            ks = sorted(last.values())[-4:]
            acc_h = check_sample([hout[hbuf[k][0]][hbuf[k][1]].numpy().copy() for k in ks],
                                 js, ks)
            assert acc_h["max_rel"] < 1e-6, acc_h
        t_all = max_over_ranks(t_all, dist, dev)
        e2e = {"value": round(replica_rate(total_vis * reps, world, t_all), 3), "unit": "Mvis/s",
               "h2d_bytes_per_step": int(total_vis * 16),
               "d2h_bytes_per_step": int(sum(8 * int(N) * int(N) for N in specs["side"])),
               "ms_per_step": round(1e3 * t_all / reps, 3),
               "api": "gg_server_* (C ABI): host requests, inputs copied in from pinned "
                      "host memory and every grid copied back to pinned host memory by "
                      f"the server; the client reuses {RING} pinned output buffers per "
                      "grid side as their requests complete",
               "copy_bound_note": "the pass moves h2d + d2h bytes over the host link "
                                  "(measured here: about 190 GB/s device-to-host alone, "
                                  "340 GB/s both directions at once)"}
    srv.close()

    if rank != 0:
        return None
    best_plain = max(plain.values())
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total_s / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators with the workload's shapes)",
        "config": {"workload": f"{args.workload}: {w['desc']}",
                   "visibilities_per_step": total_vis, "requests": n,
                   "server": {"streams": w["streams"], "max_batch_jobs": w["max_batch_jobs"],
                              "hbm_budget_bytes": int(w["budget"]), "method": "window"},
                   "l2": f"inputs ({js.device_bytes() / 1e9:.1f} GB, every request its own "
                         f"observation) exceed L2",
                   "input_generation_s": round(t_gen, 2),
                   "timing": "server clock from first arrival to last grid ready, "
                             "per pass; device synchronised around the passes",
                   "autotune": gg.autotune_report().splitlines(),
                   "parallelism": f"replicas x{world}"},
        "plain_per_request_Mvis_per_s": plain,
        "speedup_vs_best_plain": round(value / world / best_plain, 2),
        "latency_sweep": sweep,
        "accuracy": acc,
        "roofline": roof,
        "cpu_baseline": cpu_baseline(w, rank),
        "e2e": e2e,
        "gpu_launches": int(launches),
    }
    clocks = clk.summary()
    if clocks:
        res["clocks"] = clocks
    return res


# ---------------------------------------------------------------------------
# batched plan of 256 jobs in a CUDA graph
# ---------------------------------------------------------------------------
def run_batch(args, rank, world, local_rank, dist):
    import torch
    import gpugrid as gg
    w = WORKLOADS[args.workload]
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n = w["n"]
    if args.profile_small:
        # a small case of the same kernel for detailed profiler captures:
        # the first 64 jobs (about 1.5 GB on the device)
        n = 64
    js = JobStream(n, stream_seed("batch", rank), dev)
    specs, gcfs = js.specs, js.gcfs
    total_vis = js.total_vis()
    opts = gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                      layout=gg.LAYOUT_INTERLEAVED, autotune=True)
    jobs, outs, _ = stream_jobs(js, n, dev)
    ctx = gg.Context(local_rank)
    plan = gg.Plan(ctx, opts, jobs)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan.launch(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.launch(s)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        g.replay()
    torch.cuda.synchronize()
    flags = plan.read_flags()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = gg.kernel_launches()
    cs = torch.cuda.current_stream()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            ev[k][0].record(cs)
            g.replay()
            ev[k][1].record(cs)
        torch.cuda.synchronize()
    # graph replays launch the captured kernels without the library's counter
    launches = (gg.kernel_launches() - l0) or None
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms = max_over_ranks(total_ms, dist, dev)
    value = replica_rate(total_vis * args.steps, world, total_ms / 1e3)
    # number of kernels in one replay: count a direct (uncaptured) launch
    l1 = gg.kernel_launches()
    plan.launch()
    torch.cuda.synchronize()
    per_step = gg.kernel_launches() - l1
    launches = per_step * args.steps
    # accuracy on a sample of jobs
    sample = list(range(0, n, max(1, n // 12)))[:12]
    acc = check_sample([outs[i].cpu().numpy() for i in sample], js, sample) \
        if rank == 0 and not args.no_check else None
    # plain per-job launches
    plain = {}
    for label, o in (("plain_scatter_per_job",
                      gg.Options(mode=gg.MODE_SCATTER, accum=gg.ACC_PLAIN,
                                 layout=gg.LAYOUT_INTERLEAVED)),
                     ("window_per_job",
                      gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                                 layout=gg.LAYOUT_INTERLEAVED))):
        for j in jobs[:20]:
            ctx.grid_job(o, j)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for j in jobs:
            ctx.grid_job(o, j)
        e1.record()
        torch.cuda.synchronize()
        plain[label] = round(total_vis / (e0.elapsed_time(e1) / 1e3) / 1e6, 1)
    ctx.profile(True)
    ctx.grid_batch(opts, jobs)
    with nvtx_range("gg_profiled"):
        ctx.grid_batch(opts, jobs)
    _, kern_ms, _ = ctx.profile_last()
    alg = total_vis * 16 + sum(2 * 8 * j.img_dim * j.img_dim for j in jobs)
    taps = sum(j.npts * j.gcf_dim * j.gcf_dim for j in jobs)
    roof = roofline("window_kernel", alg, kern_ms, "window_batch256", taps, local_rank)
    # e2e through the server's host path: one batch of host requests
    e2e = None
    if not args.no_e2e:
        h_uv = torch.empty((total_vis, 2), dtype=torch.float32).pin_memory()
        h_v = torch.empty(total_vis, dtype=torch.complex64).pin_memory()
        hoff, o = [], 0
        for i in range(n):
            uvd, vd = js.device_job(i)
            h_uv[o:o + len(uvd)].copy_(uvd)
            h_v[o:o + len(vd)].copy_(vd)
            hoff.append(o)
            o += len(uvd)
        torch.cuda.synchronize()
        houts = [torch.empty(int(N) * int(N), dtype=torch.complex64).pin_memory().numpy()
                 for N in specs["side"]]
        # host path: 3 stream slots, batches of up to 16 jobs, so that copies of
        # one batch overlap the gridding of another (64: 2-5 % slower)
        srv = gg.Server(device=local_rank, streams=3, max_batch_jobs=16, options=opts)
        gids = {S: srv.add_gcf(gcfs[S]) for S in (8, 16)}
        reqs = []
        for i in range(n):
            N, S, nv_ = js.shape(i)
            reqs.append(gg.Server.request(h_uv.data_ptr() + hoff[i] * 8,
                                          h_v.data_ptr() + hoff[i] * 8,
                                          houts[i].ctypes.data, nv_, N, S, gids[S],
                                          uv_type=gg.C64))
        zeros = np.zeros(n)
        for _ in range(2):
            for t in srv.submit_schedule(reqs, zeros):
                srv.wait(int(t), timeout=600)
                srv.release(int(t))
        reps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(reps):
            for t in srv.submit_schedule(reqs, zeros):
                srv.wait(int(t), timeout=600)
                srv.release(int(t))
        t_all = time.perf_counter() - t0
        srv.close()
        t_all = max_over_ranks(t_all, dist, dev)
        e2e = {"value": round(replica_rate(total_vis * reps, world, t_all), 3), "unit": "Mvis/s",
               "h2d_bytes_per_step": int(total_vis * 16),
               "d2h_bytes_per_step": int(sum(8 * int(N) * int(N) for N in specs["side"])),
               "ms_per_step": round(1e3 * t_all / reps, 3),
               "api": "gg_server_* (C ABI) with host input and output buffers (3 stream "
                      "slots, batches of up to 16 jobs)"}
    if rank != 0:
        return None
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators with the workload's shapes)",
        "config": {"workload": f"{args.workload}: {w['desc']}",
                   "visibilities_per_step": total_vis, "jobs": n,
                   "l2": "flushed before every timed step (256 MiB write)",
                   "launch": "one gg_plan_launch captured in a CUDA graph, replayed",
                   "autotune": gg.autotune_report().splitlines(),
                   "parallelism": f"replicas x{world}"},
        "plain_per_job_Mvis_per_s": plain,
        "speedup_vs_best_plain": round(value / world / max(plain.values()), 2),
        "flags": flags, "accuracy": acc, "roofline": roof,
        "cpu_baseline": cpu_baseline(w, rank),
        "e2e": e2e, "gpu_launches": int(launches),
    }
    clocks = clk.summary()
    if clocks:
        res["clocks"] = clocks
    return res


# ---------------------------------------------------------------------------
# single job (uniform1024, tracks4096, disk8192)
# ---------------------------------------------------------------------------
def make_single(w, seed):
    import synth
    N, S, n = w["N"], w["S"], w["npts"]
    vdt = np.complex64 if w["vals"] == "c64" else np.complex128
    if w["gen"] == "tracks":
        uv, vals = synth.tracks(N, npts=n, seed=seed, vals_dtype=vdt)
    elif w["gen"] == "disk":
        uv, vals = synth.disk(n, N, seed=seed, outlier_frac=0.01, vals_dtype=vdt)
    else:
        uv, vals = synth.uniform(n, S, N - S, seed=seed, vals_dtype=vdt)
    if w.get("presort"):
        # the data format of the workload: grouped into 32x32 uv tiles; the
        # gridder still bins on the device at its own tile size
        perm = synth.tile_sort(uv, N, 32)
        uv, vals = np.ascontiguousarray(uv[perm]), np.ascontiguousarray(vals[perm])
    gcf = synth.gcf_table(synth.gaussian_gcf_1d(S)).astype(vdt)
    return uv, vals, gcf


def single_options(w):
    import gpugrid as gg
    return gg.Options(
        mode=gg.MODES[w["mode"]],
        accum=gg.ACC_COMPENSATED if w["accum"] == "comp" else gg.ACC_PLAIN,
        gcf_kind=gg.GCF_GAUSSIAN if w.get("gcf") == "gauss" else gg.GCF_TABLE,
        layout=gg.LAYOUT_INTERLEAVED, autotune=True)


def run_single(args, rank, world, local_rank, dist):
    import torch
    import gpugrid as gg
    import oracle as O
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = WORKLOADS[args.workload]
    if args.method:
        w = dict(w, mode=args.method)
    N, S, n = w["N"], w["S"], w["npts"]
    uv, vals, gcf = make_single(w, seed=1000 + rank)
    o = single_options(w)
    odt = torch.complex64 if w["out"] == "c64" else torch.complex128
    # float2 coordinates for the FP32 workloads (exact: generated
    # float-representable); the oracle reads the same values in FP64
    uv_in = uv.astype(np.float32) if w.get("uv") == "f32" else uv
    d_uv = torch.from_numpy(uv_in).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    d_gcf = torch.from_numpy(gcf.reshape(-1)).to(dev)
    out = torch.empty(N * N, dtype=odt, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ctx = gg.Context(local_rank)
    ctx.profile(True)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        ctx.grid(o, out, d_uv, d_vals, d_gcf, N, S)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    err = None
    if rank == 0 and not args.no_check:
        B = w.get("check_window")
        if B:
            # the oracle of a central B x B window: every visibility that can
            # reach it, on a shifted (B + 2S)^2 grid
            x0 = y0 = N // 2 - B // 2
            ref, mag, nsub = window_reference(uv, vals, gcf, N, S, x0, y0, B)
            checked = (f"central {B}x{B} window of the grid (cells [{x0}, {x0 + B})^2), "
                       f"against the oracle of the {nsub} visibilities that reach it")
        else:
            x0 = y0 = 0
            B = N
            ref, mag = oracle_pair(uv, vals, gcf, N, S)
            checked = f"whole grid, all {n} visibilities"

        def error_of(opts, grid=out):
            ctx.grid(opts, grid, d_uv, d_vals, d_gcf, N, S)
            got = torch.view_as_real(grid).reshape(N, N, 2)[y0:y0 + B, x0:x0 + B]
            got = got.cpu().numpy().astype(np.float64)
            a = ErrAcc()
            a.add(np.moveaxis(got, -1, 0).reshape(2, 1, B, B), ref, mag)
            return a.result()

        err = error_of(o)
        err["checked"] = checked
        err["metrics"] = ACC_NOTE
        if w.get("precision_study") and w["vals"] == "c64":
            # the precision form: the same visibilities with plain FP32 sums,
            # into the workload's complex128 grid and into a complex64 grid
            plain = single_options(dict(w, accum="plain"))
            out64 = torch.empty(N * N, dtype=torch.complex64, device=dev)
            err["by_accumulation"] = {
                "complex128_grid": {"fp32_compensated": error_of(o),
                                    "fp32_plain": error_of(plain)},
                "complex64_grid": {"fp32_compensated": error_of(o, out64),
                                   "fp32_plain": error_of(plain, out64)}}
            del out64
        del ref, mag
    start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kern_ms, bin_ms = [], []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = gg.kernel_launches()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xff)            # evict L2 (untimed)
            start[k].record(stream)
            with nvtx_range("gg_profiled" if k == args.steps - 1 else "gg_step"):
                ctx.grid(o, out, d_uv, d_vals, d_gcf, N, S)
            end[k].record(stream)
            b, g_ms, _ = ctx.profile_last()
            kern_ms.append(g_ms)
            bin_ms.append(b)
        torch.cuda.synchronize()
    launches = gg.kernel_launches() - l0
    total_ms = sum(s.elapsed_time(e) for s, e in zip(start, end))
    total_ms = max_over_ranks(total_ms, dist, dev)
    e2e = None
    if not args.no_e2e:
        cuv = uv_in.view(np.complex64 if uv_in.dtype == np.float32 else np.complex128)
        pin_uv = torch.from_numpy(cuv.reshape(-1)).pin_memory().numpy()
        pin_vals = torch.from_numpy(vals).pin_memory().numpy()
        pin_gcf = torch.from_numpy(gcf.reshape(-1)).pin_memory().numpy()
        pin_out = torch.zeros(gg.padded_size(N, S), dtype=odt).pin_memory().numpy()
        for _ in range(max(1, args.warmup)):
            gg.grid_host(o, pin_out, pin_uv, pin_vals, n, N, pin_gcf, S)
        ts = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gg.grid_host(o, pin_out, pin_uv, pin_vals, n, N, pin_gcf, S)
            ts.append(time.perf_counter() - t0)
        e2e_s = sum(ts)
        e2e_s = max_over_ranks(e2e_s, dist, dev)
        e2e = {"value": round(replica_rate(n * args.steps, world, e2e_s), 3), "unit": "Mvis/s",
               "h2d_bytes_per_step": int(pin_uv.nbytes + pin_vals.nbytes + pin_gcf.nbytes),
               "d2h_bytes_per_step": int(N * N * pin_out.itemsize),
               "ms_per_step": round(1e3 * e2e_s / args.steps, 4),
               "api": "gg_grid_host (C ABI, pinned host buffers)"}
    if rank != 0:
        return None
    value = replica_rate(n * args.steps, world, total_ms / 1e3)
    vb = 8 if w["vals"] == "c64" else 16
    ob = 8 if w["out"] == "c64" else 16
    mode_name = {0: "scatter", 1: "gather", 2: "window", 3: "window"}[o.mode]
    if mode_name == "scatter":
        alg = n * (16 + vb) + 2 * N * N * ob
    elif mode_name == "gather":
        alg = n * (8 + vb) + N * N * ob
    else:
        alg = n * (8 + vb) + 2 * N * N * ob
    mean_kern = statistics.mean(kern_ms)
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mvis/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if w["vals"] == "c64" else "f64",
        "data": "synthetic (seeded generators with the workload's shapes)",
        "config": {"workload": f"{args.workload}: {w['desc']}", "method": mode_name,
                   "l2": "flushed before every timed step (256 MiB write)",
                   "img_dim": N, "gcf_dim": S, "oversample": 8, "visibilities": n,
                   "autotune": gg.autotune_report().splitlines(),
                   "parallelism": f"replicas x{world}"},
        "tap_updates_per_s": round(value * 1e6 * S * S, 1),
        "phase_ms": {"setup_and_binning": round(statistics.mean(bin_ms), 4),
                     "gridding_kernel": round(mean_kern, 4)},
        "accuracy": err, "flags": flags,
        "roofline": roofline(f"{mode_name}_kernel", alg, mean_kern,
                             f"{mode_name}_{args.workload}", n * S * S, local_rank),
        "cpu_baseline": cpu_baseline(w, rank),
        "e2e": e2e, "gpu_launches": int(launches),
    }
    clocks = clk.summary()
    if clocks:
        res["clocks"] = clocks
    return res


# ---------------------------------------------------------------------------
# degridding (the gridder's adjoint) of one job
# ---------------------------------------------------------------------------
def run_degrid(args, rank, world, local_rank, dist):
    import torch
    import gpugrid as gg
    import oracle as O
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = WORKLOADS[args.workload]
    N, S, n = w["N"], w["S"], w["npts"]
    uv, vals, gcf = make_single(w, seed=1000 + rank)
    ctx = gg.Context(local_rank)
    d_uv = torch.from_numpy(uv).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    d_gcf = torch.from_numpy(gcf.reshape(-1)).to(dev)
    # the grid to sample: the workload's own visibilities gridded
    grid = torch.empty(N * N, dtype=torch.complex64, device=dev)
    ctx.grid(gg.Options(mode=gg.MODE_WINDOW, accum=gg.ACC_COMPENSATED,
                        layout=gg.LAYOUT_INTERLEAVED), grid, d_uv, d_vals, d_gcf, N, S)
    o = gg.Options(accum=gg.ACC_COMPENSATED, layout=gg.LAYOUT_INTERLEAVED)
    out = torch.empty(n, dtype=torch.complex64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        ctx.degrid(o, grid, d_uv, out, d_gcf, N, S)
    torch.cuda.synchronize()
    flags = ctx.read_flags()
    err = None
    if rank == 0 and not args.no_check:
        nchk = 1 << 18
        g = grid.cpu().numpy()
        planar = np.stack([g.real, g.imag]).reshape(2, 1, N, N).astype(np.float64)
        ref = O.degrid_pz(uv[:nchk], planar, pairs(gcf), N, S, nthreads=os.cpu_count())[:, 0]
        got = out[:nchk].cpu().numpy().astype(np.complex128)
        err = {"max_rel": float(np.abs(got - ref).max() / np.abs(ref).max()),
               "visibilities_checked": nchk,
               "reference": "FP64 degridding restatement (adjoint of the gridCPU_pz "
                            "restatement, checked by <grid(v), g> = <v, degrid(g)>)"}
        del planar, ref
    start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = gg.kernel_launches()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xff)            # evict L2 (untimed)
            start[k].record(stream)
            with nvtx_range("gg_profiled" if k == args.steps - 1 else "gg_step"):
                ctx.degrid(o, grid, d_uv, out, d_gcf, N, S)
            end[k].record(stream)
        torch.cuda.synchronize()
    launches = gg.kernel_launches() - l0
    times = [s_.elapsed_time(e_) for s_, e_ in zip(start, end)]
    total_ms = max_over_ranks(sum(times), dist, dev)
    e2e = None
    if not args.no_e2e:
        # host buffers through the public API: coordinates and grid copied in
        # from pinned memory, predicted values copied back, every step
        pin_uv = torch.from_numpy(uv).pin_memory()
        pin_grid = grid.cpu().pin_memory()
        pin_out = torch.empty(n, dtype=torch.complex64).pin_memory()
        d_uv2, d_grid2 = torch.empty_like(d_uv), torch.empty_like(grid)
        ts = []
        for k in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d_uv2.copy_(pin_uv, non_blocking=True)
            d_grid2.copy_(pin_grid, non_blocking=True)
            ctx.degrid(o, d_grid2, d_uv2, out, d_gcf, N, S)
            pin_out.copy_(out, non_blocking=True)
            torch.cuda.synchronize()
            if k >= args.warmup:
                ts.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(sum(ts), dist, dev)
        e2e = {"value": round(replica_rate(n * args.steps, world, e2e_s), 3), "unit": "Mvis/s",
               "h2d_bytes_per_step": int(pin_uv.numel() * 8 + pin_grid.numel() * 8),
               "d2h_bytes_per_step": int(n * 8),
               "ms_per_step": round(1e3 * e2e_s / args.steps, 4),
               "api": "gpugrid.Context.degrid over gg_degrid_device, pinned host buffers"}
    if rank != 0:
        return None
    value = replica_rate(n * args.steps, world, total_ms / 1e3)
    mean_ms = statistics.mean(times)
    alg = n * (16 + 8) + N * N * 8       # coordinates in, values out, grid read once
    # CPU baseline: the oracle degridder over all host threads on a prefix
    threads = os.cpu_count() or 1
    g = grid.cpu().numpy()
    planar = np.stack([g.real, g.imag]).reshape(2, 1, N, N).astype(np.float64)
    m = 1 << 16
    while True:
        t0 = time.perf_counter()
        O.degrid_pz(uv[:m], planar, pairs(gcf), N, S, nthreads=threads)
        cs = time.perf_counter() - t0
        if cs * 4 > args.cpu_budget or m >= n:
            break
        m = min(n, m * 4)
    res = {
        "metric": "degridded Mvis/s (predicted visibilities per second)",
        "value": round(value, 3), "unit": "Mvis/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators with the workload's shapes)",
        "config": {"workload": f"{args.workload}: {w['desc']}",
                   "l2": "flushed before every timed step (256 MiB write)",
                   "img_dim": N, "gcf_dim": S, "oversample": 8, "visibilities": n,
                   "parallelism": f"replicas x{world}"},
        "tap_reads_per_s": round(value * 1e6 * S * S, 1),
        "accuracy": err, "flags": flags,
        "roofline": roofline("degrid_kernel", alg, mean_ms, f"degrid_{args.workload}",
                             None, local_rank),
        "cpu_baseline": {"value": round(m / cs / 1e6, 4), "unit": "Mvis/s", "cores": threads,
                         "kind": "port",
                         "sample": f"first {m} visibilities ({cs:.1f} s), the degridding "
                                   f"restatement over {threads} threads"},
        "e2e": e2e, "gpu_launches": int(launches),
    }
    clocks = clk.summary()
    if clocks:
        res["clocks"] = clocks
    return res


# ---------------------------------------------------------------------------
# reference arm: the reference CPU gridder on the host cores
# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return None
    import oracle as O
    w = WORKLOADS[args.workload]
    if w["kind"] == "degrid":
        return {"impl": "reference",
                "unavailable": "the reference has no degridder (it grids only)"}
    threads = os.cpu_count() or 1
    # every step grids the workload's CPU sample -- the same sample as the
    # cpu_baseline of the GPU arm's line
    jobs, desc = cpu_sample(w)
    desc_n = (w["npts"] if w["kind"] == "single"
              else JobStream(w["n"], stream_seed(w["kind"])).total_vis())

    def step():
        _, vis, t, _ = cpu_rate(jobs, threads)
        return vis, t
    for _ in range(args.warmup):
        step()
    tot_v, tot_t = 0, 0.0
    for _ in range(args.steps):
        v, dt = step()
        tot_v += v
        tot_t += dt
    val = tot_v / tot_t / 1e6
    return {
        "metric": METRIC, "value": round(val, 4), "unit": "Mvis/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * tot_t / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generators with the workload's shapes)",
        "config": {"workload": f"{args.workload}: {w['desc']}", "visibilities_per_pass": desc_n},
        "cpu_baseline": {"value": round(val, 4), "unit": "Mvis/s", "cores": threads,
                         "kind": "port",
                         "sample": f"every step: {desc}; gridCPU_pz restatement "
                                   f"(oracle/grid_oracle.c) over {threads} row bands, "
                                   f"bit-identical to the single-threaded reference"},
        "e2e": {"value": round(val, 4), "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# the other configurations, compact, in the default line
# ---------------------------------------------------------------------------
SUB_CONFIGS = (("uniform1024", None), ("tracks4096", None), ("tracks4096", "scatter"),
               ("tracks4096", "gather"), ("disk8192", None), ("batch256", None))


def compact(res):
    """the figures of a full result line that the default line carries for
    the other configurations"""
    keep = ("value", "unit", "ms_per_step", "steps", "dtype", "speedup_vs_best_plain",
            "plain_per_job_Mvis_per_s", "tap_updates_per_s", "phase_ms", "flags",
            "gpu_launches")
    out = {k: res[k] for k in keep if k in res}
    out["workload"] = res["config"]["workload"]
    if "method" in res["config"]:
        out["method"] = res["config"]["method"]
    acc = res.get("accuracy")
    if acc:
        out["accuracy"] = {k: v for k, v in acc.items() if k not in ("metrics", "reference")}
    if res.get("e2e"):
        out["e2e"] = {k: res["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step",
                                                 "d2h_bytes_per_step", "ms_per_step")}
    r = res.get("roofline") or {}
    out["roofline"] = {k: r.get(k) for k in ("kernel", "achieved", "peak", "frac", "traffic")}
    cb = res.get("cpu_baseline") or {}
    out["cpu_baseline"] = {k: cb.get(k) for k in ("value", "cores", "sample")}
    if res.get("clocks"):
        out["clocks"] = {k: res["clocks"][k] for k in ("sm_mhz", "sm_max_mhz", "reasons")}
    return out


def run_configs(args, rank, world, local_rank, dist):
    """BASELINE configurations 1-4 at a few steps each (the default line's
    headline is configuration 5, the served stream)"""
    import copy
    out = {}
    for name, method in SUB_CONFIGS:
        a = copy.copy(args)
        a.workload, a.method = name, method
        a.steps, a.warmup = min(args.steps, 5), 3
        kind = WORKLOADS[name]["kind"]
        fn = {"batch": run_batch, "single": run_single}[kind]
        t0 = time.perf_counter()
        res = fn(a, rank, world, local_rank, dist)
        if res is not None:
            key = name + (f"_{method}" if method else "")
            out[key] = compact(res)
            out[key]["bench_wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=8.0,
                    help="degrid4096: seconds of CPU degridding for its CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--profile-small", action="store_true",
                    help="batch256: 64 jobs from 2 observations per grid side, a case small "
                         "enough for multi-pass profiler captures")
    ap.add_argument("--method", choices=["scatter", "gather", "window"], default=None,
                    help="single-job workloads: grid with this method instead of the "
                         "workload's own")
    ap.add_argument("--e2e-ring", type=int, default=256,
                    help="served10k e2e: pinned host output buffers per grid side that the "
                         "client cycles through (requests in flight <= 4 x this)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="served10k: only its roofline batch (the first 256 requests in one "
                         "batched call), for profiler captures")
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload: leave out the compact results of the other "
                         "configurations")
    args = ap.parse_args()
    if args.warmup < 3:
        log("bench: warm-up below 3 steps; using 3")
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        if world > 1:
            import torch
            import torch.distributed as td
            torch.cuda.set_device(local_rank)
            td.init_process_group("nccl")
            dist = td
        kind = WORKLOADS[args.workload]["kind"]
        fn = {"served": run_served, "batch": run_batch, "single": run_single,
              "degrid": run_degrid}[kind]
        res = fn(args, rank, world, local_rank, dist)
        if (args.workload == DEFAULT_WORKLOAD and world == 1 and not args.no_configs
                and args.method is None and not args.profile_batch):
            sub = run_configs(args, rank, world, local_rank, dist)
            if res is not None:
                res["configs"] = sub
                res["configs_note"] = (
                    "BASELINE configurations 1-4 measured in the same run, min(steps, 5) "
                    "timed steps each after 3 warm-up steps; every entry keeps the fields "
                    "of its own full line (python bench.py --workload NAME)")
        if dist:
            dist.destroy_process_group()
    if res is not None and rank == 0:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
