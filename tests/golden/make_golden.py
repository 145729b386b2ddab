"""Generate the golden fixtures in this directory from the reference's OWN
CPU gridder (grid.cu's gridCPU_pz, compiled by ``make -C oracle ref`` from the
reference checkout).  Run where that checkout exists:

    python tests/golden/make_golden.py

Each ``<case>.npz`` holds the inputs and the reference's planar output grid
(real plane then imaginary plane, shape (2, P, N, N)):

    uv      float64 (npts, 2)      grid-pixel coordinates (float-representable)
    vals    float64 (npts*P, 2)    complex values (re, im)
    g1      float64 (8, S)         1-D Gaussian factors (Gaussian cases), or
    gcf     float64 (64*S*S, 2)    the full table (the reference's init_gcf)
    out     float64 (2, P, N, N)   gridCPU_pz output
    meta    int64  [N, S, P, debug1]

The GCF of the Gaussian cases is rebuilt by tests as an exact product of the
stored 1-D factors, so no libm result is needed to reproduce the inputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402


def fr(a):
    """round to float32-representable float64 values"""
    return np.asarray(a, np.float32).astype(np.float64)


def save(name, **kw):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **kw)
    print("wrote", name, {k: np.asarray(v).shape for k, v in kw.items()})


def gauss_case(name, tag, npts, lo, hi, seed, sigma=None):
    R = O.RefLib(tag)
    N, S, P = R.img, R.gcf_dim, R.pols
    rng = np.random.default_rng(seed)
    uv = fr(rng.uniform(lo, hi, size=(npts, 2)))
    vals = rng.standard_normal((npts * P, 2))
    _, g1 = O.gaussian_gcf(S, sigma)
    gcf = O.gcf_from_1d(g1)
    out = R.grid(uv, vals, gcf)
    save(name, uv=uv, vals=vals, g1=g1, out=out,
         meta=np.array([N, S, P, R.debug1], np.int64))


def main():
    O.build(ref=True)
    # the reference harness's own inputs (srand(1541617), grid.cu:444-452)
    # with its own "nonsense" GCF (init_gcf, grid.cu:72-85); u,v span the
    # whole grid, so footprints are clipped at all four edges
    R = O.RefLib("64_8_1_double")
    uv, vals = R.harness_inputs(1000)
    gcf = R.init_gcf()
    save("ref_harness_n64_s8", uv=uv, vals=vals, gcf=gcf,
         out=R.grid(uv, vals, gcf), meta=np.array([64, 8, 1, 0], np.int64))
    # same inputs after the reference's GATHER-mode host sort (comp_grid,
    # grid.cu:256-276): only uv is permuted, in_vals stays as generated
    uvs = R.sort(uv, "grid")
    save("ref_harness_sorted_n64_s8", uv=uvs, vals=vals, gcf=gcf,
         out=R.grid(uvs, vals, gcf), meta=np.array([64, 8, 1, 0], np.int64))
    # Gaussian GCF, coordinates past every edge (partial and fully clipped
    # footprints, negative u,v)
    gauss_case("gauss_n64_s8", "64_8_1_double", 700, -6.0, 70.0, 11)
    gauss_case("gauss_n128_s16", "128_16_1_double", 1500, 8.0, 120.0, 12)
    gauss_case("gauss_n64_s32", "64_32_1_double", 200, -10.0, 74.0, 13)
    gauss_case("gauss_n64_s8_p4", "64_8_4_double", 400, 0.0, 64.0, 14)
    # DEBUG1 footprint mode: out = (hit count, sum of visibility indices)
    gauss_case("debug1_n64_s8", "64_8_1_double_dbg", 300, -4.0, 68.0, 16)


if __name__ == "__main__":
    main()
