// Pieces shared by the three gridding kernels.
#pragma once
#include "gg_common.cuh"
#include "gg_internal.h"

namespace gg {

// Per-launch parameters every gridding kernel receives by value.
struct KParams {
  const JobDesc *jobs;
  const WorkItem *items;
  const int *nitems;
  int *item_next;
  int *flags;
  // nonzero when this call's binning found input declared tile-sorted to be
  // unsorted (its sorted records then have holes); null without binning
  const int *holes;
  const int64_t *vis_base;
  const int *tile_base;
  int64_t total_vis;
  int njobs;
  int total_tiles;
  int P;
  int T;        // uv tile side, uniform within a launch
  int G;        // oversampling, uniform within a launch
  float sigma;  // GAUSS sigma, uniform within a launch
  int accumulate;  // gather: add each finished cell into the grid
  // moving window, compensated FP32 into complex64 grids: FP64 merge slots
  // of the tiles cut into several work items (base null: none)
  MergeSlots merge;
};

// GCF value of tap (a', b') of sub-kernel (sx, sy); KIND 0 table, 1 Gaussian
// computed on the fly, 2 the reference's per-visibility COMPUTE_GCF factor
template <int S, int KIND, typename VT>
struct GcfSrc;

// tabulated: the reference's [G*G][S][S] layout (grid.cu:169-172)
template <int S, typename VT>
struct GcfSrc<S, 0, VT> {
  using VT2 = typename vec2_of<VT>::type;
  const VT2 *tab;
  int G;
  __device__ __forceinline__ void value(int sx, int sy, int ap, int bp, VT &gr,
                                        VT &gi) const {
    VT2 g = __ldg(tab + ((size_t)(sy * G + sx) * S + bp) * S + ap);
    gr = g.x;
    gi = g.y;
  }
};

// COMPUTE_GCF: separable Gaussian from per-CTA 1-D factors g1[s*S + a'],
// evaluated in the prologue with expf (real, imaginary part zero)
template <int S, typename VT>
struct GcfSrc<S, 1, VT> {
  const float *g1;
  __device__ __forceinline__ void value(int sx, int sy, int ap, int bp, VT &gr,
                                        VT &gi) const {
    gr = (VT)(g1[sx * S + ap] * g1[sy * S + bp]);
    gi = (VT)0;
  }
};

// COMPUTE_GCF as the reference's scatter kernel evaluates it: one factor per
// visibility (set by the caller from wphase_factor), the same for every tap
template <int S, typename VT>
struct GcfSrc<S, 2, VT> {
  float fr, fi;
  __device__ __forceinline__ void value(int, int, int, int, VT &gr, VT &gi) const {
    gr = (VT)fr;
    gi = (VT)fi;
  }
};

// The factor of GcfSrc<S, 2>: (T, w) = the centre-offset table entry; dx, dy
// in double then float, the rest in float, each step rounded as written
// (no contraction), sine and cosine from the device library.
__device__ __forceinline__ float2 wphase_factor(double u, double v, int mx, int sx, int my,
                                                int sy, int G, double T, double w) {
  const float p1 = (float)(2 * 3.1415926 * w);
  const float p2 = (float)((double)p1 * T);
  const float dx = (float)(__dadd_rn(__dadd_rn((double)mx, -u), sx * 1.0 / G));
  const float dy = (float)(__dadd_rn(__dadd_rn((double)my, -v), sy * 1.0 / G));
  const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  const float ph = __fsub_rn(p1, __fmul_rn(p2, r));
  float s, c;
  sincosf(ph, &s, &c);
  return make_float2(s, c);
}

// g1[s][a'] = exp(-(a' - S/2 + 1 - s/G)^2 / (2 sigma^2)) in FP32, rows of
// `row` entries (row = 2S repeats each row once: g1[s][a' + S] = g1[s][a'])
__device__ __forceinline__ void gauss_fill(float *g1, int S, int G, float sigma,
                                           int tid, int nt, int row = 0) {
  if (row == 0) row = S;
  const float inv = 1.0f / (2.0f * sigma * sigma);
  for (int i = tid; i < G * row; i += nt) {
    int s = i / row, ap = (i % row) % S;
    float x = (float)(ap - S / 2 + 1) - (float)s / (float)G;
    g1[i] = expf(-(x * x) * inv);
  }
}

// Adds a finished cell value into the output grid (type from the job)
__device__ __forceinline__ void out_red(const JobDesc &J, size_t cell, int p,
                                        int P, double re, double im) {
  size_t NN = (size_t)J.N * J.N;
  if (J.out_f64) grid_red<double>((double *)J.out, cell, p, P, NN, J.planar, re, im);
  else grid_red<float>((float *)J.out, cell, p, P, NN, J.planar, re, im);
}

template <class ACC>
__device__ __forceinline__ void out_red_acc(const JobDesc &J, size_t cell,
                                            int p, int P, const ACC &a) {
  size_t NN = (size_t)J.N * J.N;
  if (J.out_f64)
    grid_red<double>((double *)J.out, cell, p, P, NN, J.planar, a.dre(), a.dim());
  else
    grid_red<float>((float *)J.out, cell, p, P, NN, J.planar, (double)a.fre(),
                    (double)a.fim());
}

}  // namespace gg
