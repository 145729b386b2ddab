// Scatter gridding (the reference's default method, grid_kernel
// grid_gpu.cu:95-173 and grid_kernel_small_gcf :254-327), rebuilt for sm_103a.
//
// Every tap is added into the grid in HBM/L2 by the memory system itself:
// native red.global.add.v2.f32 (one 8-byte complex per tap) or
// red.global.add.f64, instead of the reference's CAS retry loops
// (atomicAddWrap, grid_gpu.cu:53-90; the FP32 path there is always a CAS
// loop).  The small-support kernel's unsynchronised += (grid_gpu.cu:309-310)
// is a data race and has no counterpart here.
//
// A CTA takes 256 consecutive visibilities: every thread loads one (u,v) as a
// 128-bit vector, performs the FP64 index step once, and parks the packed
// indices and values in shared memory; each warp then walks the visibilities
// with its lanes spread over the S*S taps, so a warp's reductions hit
// consecutive cells of a footprint row.
//
// Compensated mode (complex64 output): the hi grid is updated with
// atom.global.v2.f32.add, which returns the previous value; two_sum of
// (previous, term) is the exact rounding error, reduced into a lo grid that
// a final pass folds into the output.  With complex128 output the FP32 terms
// are reduced with red.global.add.f64, which is at least as accurate.
#include "gg_kernels.cuh"

namespace gg {

constexpr int kScatterThreads = 256;

__device__ __forceinline__ int find_job_v(const int64_t *base, int njobs,
                                          int64_t g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int S, class ACC, int GK>
__global__ void __launch_bounds__(kScatterThreads)
    scatter_kernel(KParams kp) {
  constexpr bool GAUSS = GK == 1, WPHASE = GK == 2;
  using VT = typename ACC::VT;
  using VT2 = typename vec2_of<VT>::type;
  constexpr int NT = kScatterThreads, H = S / 2;
  extern __shared__ __align__(16) unsigned char smem[];
  int4 *rec = reinterpret_cast<int4 *>(smem);                   // mx, my, sx|sy<<8, job (-1 = skip)
  VT2 *sval = reinterpret_cast<VT2 *>(smem + NT * sizeof(int4));  // [NT][P]
  float *g1 = reinterpret_cast<float *>(smem + NT * sizeof(int4) +
                                        (size_t)NT * kp.P * sizeof(VT2));
  // WPHASE: the per-visibility factor, beside the record
  float2 *sfac = reinterpret_cast<float2 *>(smem + NT * sizeof(int4) +
                                            (size_t)NT * kp.P * sizeof(VT2) + 64 * S * 4);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int P = kp.P;
  if constexpr (GAUSS) gauss_fill(g1, S, kp.G, kp.sigma, tid, NT);
  const int64_t vb0 = kp.njobs > 1 ? __ldg(kp.vis_base) : 0;

  for (int64_t c0 = (int64_t)blockIdx.x * NT; c0 < kp.total_vis;
       c0 += (int64_t)gridDim.x * NT) {
    __syncthreads();  // previous chunk fully consumed
    {
      const int64_t t = c0 + tid;
      int4 r = make_int4(0, 0, 0, -1);
      if (t < kp.total_vis) {
        int j = 0;
        int64_t n = t;
        if (kp.njobs > 1) {
          const int64_t g = t + vb0;
          j = find_job_v(kp.vis_base, kp.njobs, g);
          n = g - __ldg(kp.vis_base + j);
        }
        const JobDesc &J = kp.jobs[j];
        int mx, sx, my, sy;
        bool ok;
        if (J.uv_f64) {
          double2 c = __ldg(reinterpret_cast<const double2 *>(J.uv) + n);
          ok = index_step(c.x, J.G, mx, sx) & index_step(c.y, J.G, my, sy);
        } else {
          float2 c = __ldg(reinterpret_cast<const float2 *>(J.uv) + n);
          ok = index_step(c.x, J.G, mx, sx) & index_step(c.y, J.G, my, sy);
        }
        if (ok && ((unsigned)sx >= (unsigned)J.G || (unsigned)sy >= (unsigned)J.G)) {
          ok = false;
          atomicAdd(&kp.flags[FLAG_INDEX], 1);
        } else if (!ok) {
          atomicAdd(&kp.flags[FLAG_INDEX], 1);
        }
        int tab = 0;
        if (ok && J.gcf_index) {
          tab = __ldg(J.gcf_index + n);
          if ((unsigned)tab >= (unsigned)J.n_gcf) {
            ok = false;
            atomicAdd(&kp.flags[FLAG_INDEX], 1);
          }
        }
        if (ok && mx + H >= 0 && mx - H + 1 < J.N && my + H >= 0 && my - H + 1 < J.N) {
          // sx, sy < 64 (8 bits each), table index < 32768
          r = make_int4(mx, my, sx | (sy << 8) | (tab << 16), j);
          const VT2 *v = reinterpret_cast<const VT2 *>(J.vals) + n * P;
          for (int p = 0; p < P; ++p) sval[tid * P + p] = __ldg(v + p);
          if constexpr (WPHASE) {
            // (T, w) at the centre offset S(S-1)/2-1 of the table
            const VT2 tw = __ldg(reinterpret_cast<const VT2 *>(J.gcf) + (S * (S - 1) / 2 - 1));
            double u, vv;
            if (J.uv_f64) {
              const double2 c = __ldg(reinterpret_cast<const double2 *>(J.uv) + n);
              u = c.x;
              vv = c.y;
            } else {
              const float2 c = __ldg(reinterpret_cast<const float2 *>(J.uv) + n);
              u = c.x;
              vv = c.y;
            }
            sfac[tid] = wphase_factor(u, vv, mx, sx, my, sy, J.G, (double)tw.x, (double)tw.y);
          }
        }
      }
      rec[tid] = r;
    }
    __syncthreads();
    for (int q = warp; q < NT; q += NT / 32) {
      const int4 r = rec[q];
      if (r.w < 0) continue;
      const JobDesc &J = kp.jobs[r.w];
      const int N = J.N;
      const size_t NN = (size_t)N * N;
      const int sx = r.z & 0xff, sy = (r.z >> 8) & 0xff, tab = r.z >> 16;
      GcfSrc<S, GK, VT> gsrc;
      if constexpr (GAUSS) {
        gsrc.g1 = g1;
      } else if constexpr (WPHASE) {
        gsrc.fr = sfac[q].x;
        gsrc.fi = sfac[q].y;
      } else {
        gsrc.tab = reinterpret_cast<const VT2 *>(J.gcf) + (size_t)tab * J.G * J.G * S * S;
        gsrc.G = J.G;
      }
      for (int tap = lane; tap < S * S; tap += 32) {
        const int ap = tap % S, bp = tap / S;
        const int gx = r.x - H + 1 + ap, gy = r.y - H + 1 + bp;
        if ((unsigned)gx >= (unsigned)N || (unsigned)gy >= (unsigned)N) continue;
        const size_t cell = (size_t)gy * N + gx;
        VT gr, gi;
        gsrc.value(sx, sy, ap, bp, gr, gi);
        for (int p = 0; p < P; ++p) {
          const VT2 v = sval[q * P + p];
          VT tr, ti;
          if constexpr (GAUSS) {
            tr = v.x * gr;
            ti = v.y * gr;
          } else {
            cmul<VT>(v.x, v.y, gr, gi, tr, ti);
          }
          if constexpr (std::is_same<ACC, AccComp>::value) {
            if (J.out_f64) {
              grid_red<double>((double *)J.out, cell, p, P, NN, J.planar, (double)tr,
                               (double)ti);
            } else {
              float *hi = (float *)J.out;
              const size_t c = (size_t)p * NN + cell;
              float er, ei, s;
              if (J.planar) {
                float o = atomicAdd(hi + c, (float)tr);
                two_sum(o, (float)tr, s, er);
                o = atomicAdd(hi + (size_t)P * NN + c, (float)ti);
                two_sum(o, (float)ti, s, ei);
                if (er != 0.f) red_add(J.lo + c, er);
                if (ei != 0.f) red_add(J.lo + (size_t)P * NN + c, ei);
              } else {
                float2 o = atom_add_v2(hi + 2 * c, (float)tr, (float)ti);
                two_sum(o.x, (float)tr, s, er);
                two_sum(o.y, (float)ti, s, ei);
                if (er != 0.f || ei != 0.f) red_add_v2(J.lo + 2 * c, er, ei);
              }
            }
          } else {
            if (J.out_f64)
              grid_red<double>((double *)J.out, cell, p, P, NN, J.planar, (double)tr,
                               (double)ti);
            else
              grid_red<float>((float *)J.out, cell, p, P, NN, J.planar, (double)tr,
                              (double)ti);
          }
        }
      }
    }
  }
}

template <int S, class ACC, int GK>
static cudaError_t scatter_launch(const KParams &kp, int sm_count, cudaStream_t s) {
  using VT2 = typename vec2_of<typename ACC::VT>::type;
  size_t smem = kScatterThreads * sizeof(int4) +
                (size_t)kScatterThreads * kp.P * sizeof(VT2) + 64 * S * 4 +
                (GK == 2 ? kScatterThreads * sizeof(float2) : 0);
  auto kern = scatter_kernel<S, ACC, GK>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kScatterThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t chunks = (kp.total_vis + kScatterThreads - 1) / kScatterThreads;
  int64_t grid = (int64_t)sm_count * per_sm;
  if (grid > chunks) grid = chunks;
  if (grid < 1) return cudaSuccess;
  kern<<<(unsigned)grid, kScatterThreads, smem, s>>>(kp);
  count_launch();
  return cudaGetLastError();
}

template <int S>
static cudaError_t scatter_dispatch(const GridLaunch &g, const KParams &kp,
                                    cudaStream_t s) {
  // GCF source: 0 table, 1 Gaussian on the fly, 2 COMPUTE_GCF phase factor
  const int gk = g.wphase ? 2 : (g.gauss ? 1 : 0);
#define GG_SC(ACCT)                                                      \
  return gk == 2 ? scatter_launch<S, ACCT, 2>(kp, g.sm_count, s)         \
                 : (gk == 1 ? scatter_launch<S, ACCT, 1>(kp, g.sm_count, s) \
                            : scatter_launch<S, ACCT, 0>(kp, g.sm_count, s))
  if (g.vals_f64) GG_SC(AccF64);
  if (g.accum == GG_ACC_COMPENSATED) GG_SC(AccComp);
  GG_SC(AccF32);
#undef GG_SC
}

cudaError_t launch_scatter(const GridLaunch &g, cudaStream_t s) {
  KParams kp{};
  kp.jobs = g.jobs;
  kp.flags = g.flags;
  kp.njobs = g.njobs;
  kp.vis_base = g.vis_base;
  kp.total_vis = g.total_vis;
  kp.P = g.P;
  kp.T = g.tile;
  kp.G = g.G;
  kp.sigma = g.sigma;
  switch (g.S) {
    case 4: return scatter_dispatch<4>(g, kp, s);
    case 8: return scatter_dispatch<8>(g, kp, s);
    case 16: return scatter_dispatch<16>(g, kp, s);
    case 32: return scatter_dispatch<32>(g, kp, s);
  }
  return cudaErrorInvalidValue;
}

__global__ void comp_finalize_kernel(float *out, const float *lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __fadd_rn(out[i], lo[i]);
}

cudaError_t launch_comp_finalize(float *out, const float *lo, int64_t n,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  comp_finalize_kernel<<<(unsigned)b, 256, 0, s>>>(out, lo, n);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gg
