"""The C++ drop-in header on the GPU: a reference-style caller (the call of
grid.cu:481) compiled against include/grid_gpu.cuh once per method macro
(none = scatter, __GATHER, __MOVING_WINDOW) with POLARIZATIONS=4 and
GCF_GRID=8, calling all three instantiations of the template (grid_gpu.cu:
820-825) on host buffers.  Its padded outputs are compared with the golden
fixture made from the reference's own gridCPU_pz (complex128 inputs) and with
the oracle on the float-converted inputs (complex64 inputs; the global
options are the reference's defaults, plain accumulation)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import gpugrid as gg
import oracle as O
from helpers import ROOT, cell_err, load_golden, rel_err

pytestmark = pytest.mark.gpu

CALLER = r'''
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "grid_gpu.cuh"

static std::vector<double> load(const std::string &path, size_t n) {
  std::vector<double> v(n);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(double), n, f) != n) std::exit(2);
  std::fclose(f);
  return v;
}

template <class C> static std::vector<C> as(const std::vector<double> &d) {
  std::vector<C> c(d.size() / 2);
  for (size_t i = 0; i < c.size(); ++i) {
    c[i].x = d[2 * i];
    c[i].y = d[2 * i + 1];
  }
  return c;
}

// one instantiation: the reference's call, gridGPU(out, in, in_vals, npts,
// IMG_SIZE, gcf, GCF_DIM), on host buffers; the padded output written back
// as doubles
template <class O, class I>
static int run(const std::string &dir, const char *tag, size_t npts, size_t N, size_t S) {
  std::vector<I> in = as<I>(load(dir + "/in.bin", 2 * npts));
  std::vector<I> vals = as<I>(load(dir + "/vals.bin", 2 * npts * POLARIZATIONS));
  std::vector<I> gcf = as<I>(load(dir + "/gcf.bin", 2 * GCF_GRID * GCF_GRID * S * S));
  const size_t pad = (N * N + 2 * N * S + 2 * S) * POLARIZATIONS;
  std::vector<O> out(pad);
  for (auto &o : out) o.x = o.y = 7;  // overwritten, not accumulated
  gridGPU(out.data(), in.data(), vals.data(), npts, N, gcf.data(), S);
  if (gg_last_status() != GG_OK) return 1;
  std::vector<double> d(2 * pad);
  for (size_t i = 0; i < pad; ++i) {
    d[2 * i] = out[i].x;
    d[2 * i + 1] = out[i].y;
  }
  FILE *f = std::fopen((dir + "/out_" + tag + ".bin").c_str(), "wb");
  if (!f || std::fwrite(d.data(), sizeof(double), d.size(), f) != d.size()) return 3;
  std::fclose(f);
  return 0;
}

int main(int argc, char **argv) {
  if (argc != 5) return 4;
  const std::string dir = argv[1];
  const size_t npts = std::strtoull(argv[2], 0, 10), N = std::strtoull(argv[3], 0, 10),
               S = std::strtoull(argv[4], 0, 10);
  int st = run<double2, double2>(dir, "zz", npts, N, S);
  if (!st) st = run<double2, float2>(dir, "zc", npts, N, S);
  if (!st) st = run<float2, float2>(dir, "cc", npts, N, S);
  return st;
}
'''


@pytest.fixture(scope="module")
def golden():
    return load_golden("gauss_n64_s8_p4")


@pytest.mark.parametrize("macro", [None, "__GATHER", "__MOVING_WINDOW"])
def test_cpp_template_dropin_runs_on_gpu(tmp_path, golden, macro):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    g = golden
    N, S, P = g["N"], g["S"], g["P"]
    assert P == 4
    (tmp_path / "caller.cpp").write_text(CALLER)
    exe = tmp_path / "caller"
    cmd = [gxx, "-std=c++14", "-O1", str(tmp_path / "caller.cpp"), "-o", str(exe),
           "-DPOLARIZATIONS=4", "-DGCF_GRID=8", "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", os.path.abspath(gg.LIB_PATH),
           "-Wl,-rpath," + os.path.dirname(os.path.abspath(gg.LIB_PATH))]
    if macro:
        cmd.insert(4, "-D" + macro)
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    uv, vals, gcf = g["uv"], g["vals"], g["gcf"]
    for name, a in (("in", uv), ("vals", vals), ("gcf", gcf)):
        np.ascontiguousarray(a, np.float64).tofile(tmp_path / f"{name}.bin")
    r = subprocess.run([str(exe), str(tmp_path), str(len(uv)), str(N), str(S)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)

    head = N * S + S
    planar = macro == "__MOVING_WINDOW"   # the reference's window kernel writes planar
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    ref32 = O.grid_pz(f32(uv), f32(vals), f32(gcf), N, S, pols=P, nthreads=8)
    mag32 = O.grid_mag(f32(uv), f32(vals), f32(gcf), N, S, pols=P, nthreads=8)
    for tag in ("zz", "zc", "cc"):
        d = np.fromfile(tmp_path / f"out_{tag}.bin", np.float64).reshape(-1, 2)
        pad = (N * N + 2 * N * S + 2 * S) * P
        assert d.shape[0] == pad
        # zeroed outside the grid, everything overwritten
        assert not d[:head].any() and not d[head + P * N * N:].any()
        grid = d[head:head + P * N * N]
        if planar:
            # re[P][N][N] then im[P][N][N]: the caller wrote the output's
            # scalars back in memory order
            got = grid.reshape(-1).reshape(2, P, N, N)
        else:
            got = np.moveaxis(grid.reshape(P, N, N, 2), -1, 0)
        if tag == "zz":
            assert rel_err(got, g["out"]) <= 1e-12
        else:
            assert rel_err(got, ref32) <= 2e-6
            assert cell_err(got, ref32, mag32)[0] <= 1e-5
