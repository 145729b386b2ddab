"""Build libgg.so (the gridder's C ABI) in-tree for sm_103a.

    python ska-gpu-grid_gb300/build.py [--force] [--debug]

Each CUDA translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -lineinfo -O3), then linked into
``ska-gpu-grid_gb300/libgg.so`` against the shared CUDA runtime.  Object files
go to ``ska-gpu-grid_gb300/_build/``.  Rebuilds only what changed.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgg.so")
# measurement helper of the benchmark (reduction-rate probe), a separate library
PROBE_SRC = "gg_probe.cu"
PROBE_LIB = os.path.join(HERE, "libgg_probe.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["gg_api.cu", "gg_bin.cu", "gg_scatter.cu", "gg_window.cu",
           "gg_gather.cu", "gg_noalloc.cu", "gg_server.cu", "gg_degrid.cu", "gg_image.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"),
              "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(debug: bool) -> list[str]:
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
         "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]
    if debug:
        f += ["-DGG_DEBUG=1"]
    return f + ARCH


def _digest(paths: list[str], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def build(force: bool = False, debug: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))] + [os.path.join(INCLUDE, "gg.h")]
    flags = _flags(debug)
    hdr = _digest(headers, " ".join(flags))
    objs, jobs = [], []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        tag = _digest([sp], hdr)
        obj = os.path.join(BUILD, f"{src[:-3]}.{tag}.o")
        objs.append(obj)
        if force or not os.path.exists(obj):
            jobs.append((sp, obj))
    nv = nvcc()

    def compile_one(job):
        sp, obj = job
        cmd = [nv, "-c", sp, "-o", obj + ".tmp"] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(sp)}:\n"
                               f"{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        return r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for msg in ex.map(compile_one, jobs):
                if verbose and msg:
                    print(msg, file=sys.stderr)
    link_tag = _digest(objs, "link")
    stamp = os.path.join(BUILD, "libgg.stamp")
    if (force or jobs or not os.path.exists(LIB) or not os.path.exists(stamp)
            or open(stamp).read() != link_tag):
        cmd = [nv, "-shared", "-o", LIB + ".tmp"] + objs + ARCH + [
            "-cudart", "shared", "-ldl", "-Xlinker", "-soname=libgg.so"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
        with open(stamp, "w") as fh:
            fh.write(link_tag)
    # the probe library
    psrc = os.path.join(CSRC, PROBE_SRC)
    ptag = _digest([psrc], " ".join(flags))
    pobj = os.path.join(BUILD, f"gg_probe.{ptag}.o")
    if force or not os.path.exists(pobj) or not os.path.exists(PROBE_LIB):
        compile_one((psrc, pobj))
        cmd = [nv, "-shared", "-o", PROBE_LIB + ".tmp", pobj] + ARCH + ["-cudart", "shared"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(PROBE_LIB + ".tmp", PROBE_LIB)
    # drop stale objects of earlier source versions
    keep = set(objs) | {pobj}
    for f in os.listdir(BUILD):
        p = os.path.join(BUILD, f)
        if f.endswith(".o") and p not in keep:
            os.remove(p)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--debug", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.debug, a.verbose))
