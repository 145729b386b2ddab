#!/usr/bin/env python3
"""Benchmark of the GB300 gridder; prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                    [--impl ours|reference]

A step is one gridding pass over one batch of synthetic visibilities with the
inputs resident in HBM (value), or, for e2e, the same pass through the C ABI
(gg_grid_host) from pinned host buffers, host->device copies and the
device->host grid copy included.  L2 is flushed (256 MiB write) before every
timed step; steps are timed with CUDA events on the launching stream.

--impl reference times the reference's CPU gridder (gridCPU_pz, grid.cu:
140-193) on the host cores: the C restatement in oracle/ split over all host
threads in row bands (bit-identical to the single-threaded reference), on a
bounded sample of the same workload.
Under torchrun each rank grids its own replica of the workload (independent
jobs, weak scaling); rank 0 prints the line with the max time over ranks.
"""
from __future__ import annotations

import argparse
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

WORKLOADS = {
    # gather / moving-window workload
    "tracks4096": dict(
        N=4096, S=8, npts=1 << 22, gen="tracks", vals="c64", out="c64",
        mode="auto", accum="comp", presort=True, input_sorted=False,
        desc=("4096^2 complex64 grid; 2^22 visibilities on uv tracks (64 "
              "antennas in a 2 km disk, 2016 baselines x 2080 hour angles over "
              "+-4 h at dec -30 deg, 90% fill, +1024 to 2^22); complex64 N(0,1) "
              "values; FP64 u,v; support 8, oversample 8; presorted into 32x32 "
              "uv tiles; FP32 compensated accumulation")),
    # plain scatter workload (FP64, the CPU-reference-runs case)
    "uniform1024": dict(
        N=1024, S=16, npts=1 << 18, gen="uniform", vals="c128", out="c128",
        mode="scatter", accum="plain", input_sorted=False,
        desc=("1024^2 complex128 grid; 2^18 visibilities uniform in "
              "[16, 1008); complex128 N(0,1) values; support 16, oversample 8; "
              "FP64 scatter")),
    # precision workload
    "disk8192": dict(
        N=8192, S=32, npts=1 << 24, gen="disk", vals="c64", out="c128",
        mode="auto", accum="comp", input_sorted=False, gcf="gauss",
        desc=("8192^2 grid (complex128 output of FP32 compensated "
              "accumulation); 2^24 visibilities, uniform disk; N(0,1) values "
              "with 1% outliers at 1e3; support 32, oversample 8; GCF computed "
              "on the fly")),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def make_inputs(w, seed):
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
    g1 = synth.gaussian_gcf_1d(S)
    gcf = synth.gcf_table(g1).astype(vdt)
    return uv, vals, gcf


def options(w):
    import gpugrid as gg
    return gg.Options(
        mode=gg.MODES[w["mode"]],
        accum=gg.ACC_COMPENSATED if w["accum"] == "comp" else gg.ACC_PLAIN,
        gcf_kind=gg.GCF_GAUSSIAN if w.get("gcf") == "gauss" else gg.GCF_TABLE,
        layout=gg.LAYOUT_INTERLEAVED, input_sorted=w.get("input_sorted", False))


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
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_from_profile(kernel_tag):
    """dram bytes per launch recorded from an ncu capture (profiles/)."""
    p = os.path.join(ROOT, "profiles", f"{kernel_tag}.txt")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of gridCPU_pz)
# ---------------------------------------------------------------------------
def cpu_grid_rate(w, uv, vals, gcf, budget_s=8.0, threads=None):
    """Mvis/s of the CPU gridder on a bounded sample, all host threads."""
    import oracle as O
    threads = threads or os.cpu_count() or 1
    N, S = w["N"], w["S"]
    pairs = lambda c: np.stack([c.real, c.imag], -1).astype(np.float64).reshape(-1, 2)
    g = pairs(gcf.reshape(-1))
    n = min(len(uv), 1 << 14)
    t0 = time.perf_counter()
    O.grid_pz(uv[:n], pairs(vals[:n]), g, N, S, nthreads=threads)
    dt = time.perf_counter() - t0
    per = dt / n
    n2 = int(min(len(uv), max(n, budget_s / max(per, 1e-12))))
    t0 = time.perf_counter()
    O.grid_pz(uv[:n2], pairs(vals[:n2]), g, N, S, nthreads=threads)
    dt = time.perf_counter() - t0
    return n2 / dt / 1e6, n2, dt, threads


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank, dist):
    import torch
    import gpugrid as gg
    import oracle as O
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = WORKLOADS[args.workload]
    N, S, n = w["N"], w["S"], w["npts"]
    uv, vals, gcf = make_inputs(w, seed=1000 + rank)
    o = options(w)
    odt = torch.complex64 if w["out"] == "c64" else torch.complex128
    d_uv = torch.from_numpy(uv).to(dev)
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

    # accuracy of this exact output against the FP64 oracle (rank 0)
    err = None
    if rank == 0 and not args.no_check:
        pairs = lambda c: np.stack([c.real, c.imag], -1).astype(np.float64).reshape(-1, 2)
        nchk = n if N <= 4096 else n // 16
        if nchk < n:
            ctx.grid(o, out, d_uv[:nchk], d_vals[:nchk], d_gcf, N, S)
        ref = O.grid_pz(uv[:nchk], pairs(vals[:nchk]), pairs(gcf.reshape(-1)), N, S,
                        nthreads=os.cpu_count())
        got = torch.view_as_real(out).reshape(N, N, 2).cpu().numpy().astype(np.float64)
        d = np.abs(got[..., 0] - ref[0, 0]).max(), np.abs(got[..., 1] - ref[1, 0]).max()
        den = max(np.abs(ref).max(), 1e-300)
        rms = np.sqrt(((got[..., 0] - ref[0, 0]) ** 2 + (got[..., 1] - ref[1, 0]) ** 2).sum()
                      / (ref ** 2).sum())
        err = {"max_rel": float(max(d) / den), "rms_rel": float(rms),
               "visibilities_checked": int(nchk)}
        del ref, got

    # timed region
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
            ctx.grid(o, out, d_uv, d_vals, d_gcf, N, S)
            end[k].record(stream)
            b, g_ms, _ = ctx.profile_last()
            kern_ms.append(g_ms)
            bin_ms.append(b)
        torch.cuda.synchronize()
    launches = gg.kernel_launches() - l0
    step_ms = [s.elapsed_time(e) for s, e in zip(start, end)]
    total_ms = sum(step_ms)
    if dist:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()

    # e2e through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin_uv = torch.from_numpy(uv.view(np.complex128).reshape(-1)).pin_memory().numpy()
        pin_vals = torch.from_numpy(vals).pin_memory().numpy()
        pin_gcf = torch.from_numpy(gcf.reshape(-1)).pin_memory().numpy()
        pdt = np.complex64 if w["out"] == "c64" else np.complex128
        pin_out = torch.zeros(gg.padded_size(N, S), dtype=odt).pin_memory().numpy()
        assert pin_out.dtype == pdt
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
        if dist:
            t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = pin_uv.nbytes + pin_vals.nbytes + pin_gcf.nbytes
        d2h = N * N * np.dtype(pdt).itemsize
        e2e = {"value": round(world * n * args.steps / e2e_s / 1e6, 3), "unit": "Mvis/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": round(1e3 * e2e_s / args.steps, 4),
               "api": "gg_grid_host (C ABI, pinned host buffers)"}

    if rank != 0:
        return None

    value = world * n * args.steps / (total_ms / 1e3) / 1e6
    hbm, hbm_kind = peaks()
    vb = 8 if w["vals"] == "c64" else 16
    ob = 8 if w["out"] == "c64" else 16
    mean_kern = statistics.mean(kern_ms)
    # gridding-kernel algorithmic bytes per launch: staged records (8-byte
    # packed index + value) + one read and one write of the grid by the
    # flush reductions (window), the plain stores (gather), or the per-tap
    # reductions' footprint (scatter: inputs 16 B uv + value per visibility)
    mode_name = {0: "scatter", 1: "gather", 2: "window", 3: "window"}[o.mode]
    if mode_name == "scatter":
        alg = n * (16 + vb) + 2 * N * N * ob
    elif mode_name == "gather":
        alg = n * (8 + vb) + N * N * ob
    else:
        alg = n * (8 + vb) + 2 * N * N * ob
    achieved = alg / (mean_kern / 1e3) / 1e9
    tag = f"{mode_name}_{args.workload}"
    traffic = traffic_from_profile(tag)
    cpu_v, cpu_n, cpu_dt, cpu_threads = cpu_grid_rate(w, uv, vals, gcf, budget_s=args.cpu_budget)
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mvis/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if w["vals"] == "c64" else "f64",
        "data": "synthetic (seeded generators, shapes of the workload)",
        "config": {"workload": f"{args.workload}: {w['desc']}",
                   "method": mode_name, "l2": "flushed before every timed step (256 MiB write)",
                   "img_dim": N, "gcf_dim": S, "oversample": 8, "visibilities": n,
                   "parallelism": f"replicas x{world}"},
        "tap_updates_per_s": round(value * 1e6 * S * S, 1),
        "phase_ms": {"setup_and_binning": round(statistics.mean(bin_ms), 4),
                     "gridding_kernel": round(mean_kern, 4)},
        "accuracy": err, "flags": flags,
        "roofline": {"bound": "hbm", "kernel": f"{mode_name}_kernel",
                     "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_kind": f"{hbm_kind} (copy)",
                     "traffic": traffic, "algorithmic_bytes_per_launch": int(alg)},
        "cpu_baseline": {"value": round(cpu_v, 4), "unit": "Mvis/s", "cores": cpu_threads,
                         "kind": "port",
                         "sample": f"first {cpu_n} of {n} visibilities of the same "
                                   f"workload, gridCPU_pz restatement over "
                                   f"{cpu_threads} row bands ({cpu_dt:.1f} s)"},
        "e2e": e2e,
        "gpu_launches": int(launches),
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
    w = WORKLOADS[args.workload]
    uv, vals, gcf = make_inputs(w, seed=1000)
    threads = os.cpu_count() or 1
    # size a step to ~budget seconds
    rate, n_s, _, _ = cpu_grid_rate(w, uv, vals, gcf, budget_s=1.0, threads=threads)
    n_step = int(min(len(uv), max(1 << 12, rate * 1e6 * args.cpu_budget / max(args.steps, 1))))
    import oracle as O
    pairs = lambda c: np.stack([c.real, c.imag], -1).astype(np.float64).reshape(-1, 2)
    g = pairs(gcf.reshape(-1))
    pv = pairs(vals[:n_step])
    for _ in range(args.warmup):
        O.grid_pz(uv[:n_step], pv, g, w["N"], w["S"], nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.grid_pz(uv[:n_step], pv, g, w["N"], w["S"], nthreads=threads)
    dt = time.perf_counter() - t0
    v = n_step * args.steps / dt / 1e6
    return {
        "metric": METRIC, "value": round(v, 4), "unit": "Mvis/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generators, shapes of the workload)",
        "config": {"workload": f"{args.workload}: {w['desc']}", "img_dim": w["N"],
                   "gcf_dim": w["S"], "oversample": 8, "visibilities": w["npts"]},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mvis/s", "cores": threads,
                         "kind": "port",
                         "sample": f"first {n_step} of {w['npts']} visibilities per step; "
                                   f"gridCPU_pz restatement (oracle/grid_oracle.c) over "
                                   f"{threads} row bands, bit-identical to the "
                                   f"single-threaded reference"},
        "e2e": {"value": round(v, 4), "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="tracks4096", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=8.0,
                    help="seconds of CPU gridding for the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true")
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
        res = run_ours(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
    if res is not None and rank == 0:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
