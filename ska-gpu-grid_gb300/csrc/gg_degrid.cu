// Degridding: the adjoint of the gridder.  The reference has no degridder;
// this one keeps its gridder's conventions (grid.cu:157-191 for the index
// step, the tap window (-S/2, S/2] and the table entry of a tap) so that
// degridding with the same table is the exact adjoint of gridding:
//
//   vals[n][p] = sum over the on-grid taps of n of grid[p][y][x] * conj(w)
//
// and <grid(v), g> = <v, degrid(g)> for <a, b> = sum conj(a) b.
//
// Each visibility is summed by S lanes, one footprint column each (32/S
// visibilities per warp), so no atomics and no binning are needed: the lanes
// of a visibility read contiguous cells of one row per step, and
// consecutive visibilities on a uv track read overlapping footprints
// through L1/L2.  S lanes rather than a whole warp per visibility: the
// per-visibility work (index step, reduction) is spread over S taps per lane
// (a whole warp on a support-8 visibility measured 330 warp instructions per
// visibility, two taps per lane).
// FP32 values: plain FP32 sums, or with GG_ACC_COMPENSATED a two-sum (hi, lo)
// pair per lane that the warp reduction carries; FP64 values: FP64 sums.
#include <type_traits>

#include "gg_kernels.cuh"

namespace gg {

namespace {

__device__ __forceinline__ bool uv_step(const void *uv, int uv_f64, int64_t n, int G, int &mx,
                                        int &sx, int &my, int &sy) {
  if (uv_f64) {
    const double2 c = __ldg(reinterpret_cast<const double2 *>(uv) + n);
    const bool a = index_step(c.x, G, mx, sx);
    const bool b = index_step(c.y, G, my, sy);
    return a && b;
  }
  const float2 c = __ldg(reinterpret_cast<const float2 *>(uv) + n);
  const bool a = index_step(c.x, G, mx, sx);
  const bool b = index_step(c.y, G, my, sy);
  return a && b;
}

template <typename GT, typename VT>
__device__ __forceinline__ void load_cell(const DegridLaunch &d, size_t NN, int p, size_t cell,
                                          VT &cr, VT &ci) {
  const GT *g = reinterpret_cast<const GT *>(d.grid);
  if (d.planar) {
    cr = (VT)__ldg(g + (size_t)p * NN + cell);
    ci = (VT)__ldg(g + (size_t)(d.P + p) * NN + cell);
  } else {
    using GT2 = typename vec2_of<GT>::type;
    const GT2 v = __ldg(reinterpret_cast<const GT2 *>(g) + (size_t)p * NN + cell);
    cr = (VT)v.x;
    ci = (VT)v.y;
  }
}

// running sum of one lane: plain, or a (hi, lo) two-sum pair
template <typename VT, bool COMP> struct LaneSum {
  VT h = 0, l = 0;
  __device__ __forceinline__ void add(VT t) {
    if constexpr (COMP) {
      float s, e;
      two_sum(h, t, s, e);
      h = s;
      l = __fadd_rn(l, e);
    } else {
      h += t;
    }
  }
  // adds the partner lane's pair (hi sums two-summed, lo sums added)
  __device__ __forceinline__ void merge(VT oh, VT ol) {
    if constexpr (COMP) {
      float s, e;
      two_sum(h, oh, s, e);
      h = s;
      l = __fadd_rn(__fadd_rn(l, ol), e);
    } else {
      h += oh;
    }
  }
  __device__ __forceinline__ VT value() const {
    if constexpr (COMP) return __fadd_rn(h, l);
    return h;
  }
};

template <int S, typename VT, typename GT, int GK, bool COMP>
__global__ void __launch_bounds__(256, 4) degrid_kernel(DegridLaunch d) {
  using VT2 = typename vec2_of<VT>::type;
  constexpr int TT = S * S;
  constexpr int LPV = S;        // lanes per visibility: one footprint column each
  constexpr int VPW = 32 / LPV; // visibilities per warp
  __shared__ float g1[GK == 1 ? 64 * S : 1];
  if constexpr (GK == 1) {
    gauss_fill(g1, S, d.G, d.sigma, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, sl = lane % LPV, sv = lane / LPV;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const size_t NN = (size_t)d.N * d.N;
  const VT2 *tabs = reinterpret_cast<const VT2 *>(d.gcf);
  for (int64_t n0 = warp * VPW; n0 < d.npts; n0 += nwarps * VPW) {
    const int64_t n = n0 + sv;
    const bool valid = n < d.npts;
    int mx = 0, sx = 0, my = 0, sy = 0, tab = 0;
    bool ok = false;
    if (valid) {
      ok = uv_step(d.uv, d.uv_f64, n, d.G, mx, sx, my, sy) && (unsigned)sx < (unsigned)d.G &&
           (unsigned)sy < (unsigned)d.G;
      if (ok && d.gcf_index) {
        tab = __ldg(d.gcf_index + n);
        ok = (unsigned)tab < (unsigned)d.n_gcf;
      }
      if (!ok && sl == 0) atomicAdd(&d.flags[FLAG_INDEX], 1);
    }
    const VT2 *w = tabs && ok ? tabs + ((size_t)tab * d.G * d.G + (size_t)sy * d.G + sx) * TT : tabs;
    // this lane's column of the footprint
    const int ap = sl, x = mx + ap - S / 2 + 1;
    const bool xin = ok && (unsigned)x < (unsigned)d.N;
    for (int p = 0; p < d.P; ++p) {
      LaneSum<VT, COMP> sr, si;
      if (xin) {
#pragma unroll 8
        for (int bp = 0; bp < S; ++bp) {
          const int y = my + bp - S / 2 + 1;
          if ((unsigned)y < (unsigned)d.N) {
            VT wr, wi;
            if constexpr (GK == 1) {
              wr = (VT)(g1[sx * S + ap] * g1[sy * S + bp]);
              wi = (VT)0;
            } else {
              const VT2 e = __ldg(w + bp * S + ap);
              wr = e.x;
              wi = e.y;
            }
            VT cr, ci;
            load_cell<GT, VT>(d, NN, p, (size_t)y * d.N + x, cr, ci);
            // grid * conj(w)
            sr.add(cr * wr + ci * wi);
            si.add(ci * wr - cr * wi);
          }
        }
      }
#pragma unroll
      for (int o = LPV / 2; o > 0; o >>= 1) {
        const VT rh = __shfl_xor_sync(0xffffffffu, sr.h, o);
        const VT rl = __shfl_xor_sync(0xffffffffu, sr.l, o);
        const VT ih = __shfl_xor_sync(0xffffffffu, si.h, o);
        const VT il = __shfl_xor_sync(0xffffffffu, si.l, o);
        sr.merge(rh, rl);
        si.merge(ih, il);
      }
      if (valid && sl == 0) {
        VT2 out;
        out.x = sr.value();
        out.y = si.value();
        reinterpret_cast<VT2 *>(d.vals)[(size_t)n * d.P + p] = out;
      }
    }
  }
}

template <int S, typename VT, typename GT>
cudaError_t degrid_kinds(const DegridLaunch &d, unsigned blocks, cudaStream_t s) {
  constexpr bool F32 = std::is_same<VT, float>::value;
  if (d.gauss) {
    if (F32 && d.compensated) degrid_kernel<S, VT, GT, 1, F32><<<blocks, 256, 0, s>>>(d);
    else degrid_kernel<S, VT, GT, 1, false><<<blocks, 256, 0, s>>>(d);
  } else {
    if (F32 && d.compensated) degrid_kernel<S, VT, GT, 0, F32><<<blocks, 256, 0, s>>>(d);
    else degrid_kernel<S, VT, GT, 0, false><<<blocks, 256, 0, s>>>(d);
  }
  count_launch();
  return cudaGetLastError();
}

template <int S>
cudaError_t degrid_types(const DegridLaunch &d, unsigned blocks, cudaStream_t s) {
  if (d.vals_f64)
    return d.grid_f64 ? degrid_kinds<S, double, double>(d, blocks, s)
                      : degrid_kinds<S, double, float>(d, blocks, s);
  return d.grid_f64 ? degrid_kinds<S, float, double>(d, blocks, s)
                    : degrid_kinds<S, float, float>(d, blocks, s);
}

}  // namespace

cudaError_t launch_degrid(const DegridLaunch &d, cudaStream_t s) {
  if (d.npts <= 0) return cudaSuccess;
  const int vpw = 32 / d.S;
  const int64_t warps = (d.npts + vpw - 1) / vpw;
  const int64_t b = (warps + 7) / 8;
  const int64_t cap = (int64_t)d.sm_count * 4;  // resident CTAs (64 registers)
  const unsigned blocks = (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
  switch (d.S) {
    case 4: return degrid_types<4>(d, blocks, s);
    case 8: return degrid_types<8>(d, blocks, s);
    case 16: return degrid_types<16>(d, blocks, s);
    case 32: return degrid_types<32>(d, blocks, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gg
