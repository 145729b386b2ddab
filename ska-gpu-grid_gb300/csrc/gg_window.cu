// Moving-window gridding (the reference's MOVING_WINDOW method,
// grid_kernel_window, grid_gpu.cu:504-673), rebuilt for sm_103a.
//
// The reference gives each thread a fixed residue (x mod S, y mod S), keeps a
// register sum while the target cell of consecutive (sorted) visibilities is
// unchanged and flushes it with a global CAS atomic when the cell changes.
// Here:
//  * a persistent CTA pulls work items -- slices of one uv tile's sorted
//    visibilities -- from a device queue, so dense tiles are split across SMs
//    and sparse ones are packed together;
//  * every CTA owns a (T+S-1)^2 shared-memory sub-grid covering its tile plus
//    the footprint halo; register sums are flushed there (FP32 compensated
//    hi/lo when requested) and the sub-grid is flushed to HBM ONCE per item,
//    with native vector reductions and only for cells that were touched;
//  * residue threads: S*S of them own distinct residues, so within one
//    visibility group no two threads ever write the same cell; with S*S <
//    256, several groups split each staged chunk and flush with shared
//    atomics instead;
//  * visibility records (packed indices + values) are staged in shared memory
//    by 1-D TMA bulk copies, double-buffered on two mbarriers.
// Items too sparse to pay for zeroing and flushing the sub-grid flush each
// register sum straight to HBM instead.
#include "gg_kernels.cuh"

namespace gg {

constexpr int kWinChunk = 512;

template <class ACC> struct Cell;
template <> struct Cell<AccF32> { float re, im; };
template <> struct Cell<AccComp> { float hr, hi, lr, li; };
template <> struct Cell<AccF64> { double re, im; };

__device__ __forceinline__ void cell_add(Cell<AccF32> *c, const AccF32 &a,
                                         bool exclusive) {
  if (exclusive) {
    c->re = __fadd_rn(c->re, a.re);
    c->im = __fadd_rn(c->im, a.im);
  } else {
    atomicAdd(&c->re, a.re);
    atomicAdd(&c->im, a.im);
  }
}
__device__ __forceinline__ void cell_add(Cell<AccComp> *c, const AccComp &a,
                                         bool exclusive) {
  float s, e;
  if (exclusive) {
    two_sum(c->hr, a.hr, s, e);
    c->hr = s;
    c->lr = __fadd_rn(c->lr, __fadd_rn(e, a.lr));
    two_sum(c->hi, a.hi_, s, e);
    c->hi = s;
    c->li = __fadd_rn(c->li, __fadd_rn(e, a.li));
  } else {
    // the shared-memory atomic returns the old value; two_sum recovers the
    // exact rounding error of the addition the hardware just performed
    float old = atomicAdd(&c->hr, a.hr);
    two_sum(old, a.hr, s, e);
    atomicAdd(&c->lr, __fadd_rn(e, a.lr));
    old = atomicAdd(&c->hi, a.hi_);
    two_sum(old, a.hi_, s, e);
    atomicAdd(&c->li, __fadd_rn(e, a.li));
  }
}
__device__ __forceinline__ void cell_add(Cell<AccF64> *c, const AccF64 &a,
                                         bool exclusive) {
  if (exclusive) {
    c->re = __dadd_rn(c->re, a.re);
    c->im = __dadd_rn(c->im, a.im);
  } else {
    atomicAdd(&c->re, a.re);
    atomicAdd(&c->im, a.im);
  }
}

__device__ __forceinline__ void cell_load(const Cell<AccF32> &c, AccF32 &a) {
  a.re = c.re; a.im = c.im;
}
__device__ __forceinline__ void cell_load(const Cell<AccComp> &c, AccComp &a) {
  a.hr = c.hr; a.hi_ = c.hi; a.lr = c.lr; a.li = c.li;
}
__device__ __forceinline__ void cell_load(const Cell<AccF64> &c, AccF64 &a) {
  a.re = c.re; a.im = c.im;
}

template <int S, class ACC>
struct WinShape {
  using VT = typename ACC::VT;
  using VT2 = typename vec2_of<VT>::type;
  static constexpr int NRES = S * S;
  static constexpr int NT = NRES > 256 ? NRES : 256;
  static constexpr int V = NT / NRES;
  static constexpr int IDX_BUF = kWinChunk * 8 + 16;
  static constexpr int VAL_BUF = kWinChunk * (int)sizeof(VT2) + 16;
  // bytes: 2 mbarriers (pad 16) + 2 idx buffers + 2 value buffers + 1-D GCF
  // factors (64 x S floats max) + the sub-grid
  static size_t smem(int T) {
    int R = T + S - 1;
    return 16 + 2 * IDX_BUF + 2 * VAL_BUF + 64 * S * 4 +
           (size_t)R * R * sizeof(Cell<ACC>);
  }
};

template <int S, class ACC, bool GAUSS>
__global__ void __launch_bounds__(WinShape<S, ACC>::NT)
    window_kernel(KParams kp) {
  using Sh = WinShape<S, ACC>;
  using VT = typename ACC::VT;
  using VT2 = typename Sh::VT2;
  using CellT = Cell<ACC>;
  constexpr int NRES = Sh::NRES, NT = Sh::NT, V = Sh::V, K = kWinChunk;
  constexpr int H = S / 2;

  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  unsigned char *idxbuf[2] = {smem + 16, smem + 16 + Sh::IDX_BUF};
  unsigned char *valbuf[2] = {smem + 16 + 2 * Sh::IDX_BUF,
                              smem + 16 + 2 * Sh::IDX_BUF + Sh::VAL_BUF};
  float *g1 = reinterpret_cast<float *>(smem + 16 + 2 * Sh::IDX_BUF + 2 * Sh::VAL_BUF);
  CellT *region = reinterpret_cast<CellT *>(
      smem + 16 + 2 * Sh::IDX_BUF + 2 * Sh::VAL_BUF + 64 * S * 4);
  __shared__ int s_item;
  __shared__ int s_abort;

  const int tid = threadIdx.x;
  const int res = tid % NRES, grp = tid / NRES;
  const int rx = res % S, ry = res / S;
  const int P = kp.P, T = kp.T, R = T + S - 1;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  uint32_t uses0 = 0, uses1 = 0;  // completed phases of each buffer barrier
  if constexpr (GAUSS) gauss_fill(g1, S, kp.G, kp.sigma, tid, NT);
  const int nitems = *kp.nitems;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(kp.item_next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems || s_abort) break;
    const WorkItem w = kp.items[it];
    const JobDesc &J = kp.jobs[w.job];
    const int N = J.N, G = J.G, log2G = J.log2G;
    const int tx = w.bin % J.ntx, ty = w.bin / J.ntx;
    const int ox = tx * T - H + 1, oy = ty * T - H + 1;  // sub-grid origin
    const int n = w.end - w.start;
    const bool direct = (long long)n * NRES * 4 < (long long)R * R;
    const VT2 *vals_base = reinterpret_cast<const VT2 *>(J.vals);
    GcfSrc<S, GAUSS, VT> gsrc;
    if constexpr (GAUSS) {
      gsrc.g1 = g1;
    } else {
      gsrc.tab = reinterpret_cast<const VT2 *>(J.gcf);
      gsrc.G = G;
    }
    const int nchunks = (n + K - 1) / K;

    for (int p = 0; p < P; ++p) {
      const VT2 *vplane = vals_base + (size_t)p * J.vstride;
      auto issue = [&](int c, int b) {
        int s0 = w.start + c * K;
        int e0 = min(w.end, s0 + K);
        size_t i0 = (size_t)s0 * 8, i1 = (size_t)e0 * 8;
        size_t v0 = (size_t)s0 * sizeof(VT2), v1 = (size_t)e0 * sizeof(VT2);
        uint32_t bytes = (uint32_t)(((i1 + 15) & ~(size_t)15) - (i0 & ~(size_t)15)) +
                         (uint32_t)(((v1 + 15) & ~(size_t)15) - (v0 & ~(size_t)15));
        fence_proxy_async();
        mbar_expect_tx(&bar[b], bytes);
        stage_span(idxbuf[b], reinterpret_cast<const char *>(J.idx), i0, i1, &bar[b]);
        stage_span(valbuf[b], reinterpret_cast<const char *>(vplane), v0, v1, &bar[b]);
      };
      if (!direct)
        for (int i = tid; i < R * R; i += NT) region[i] = CellT{};
      if (tid == 0) {
        issue(0, 0);
        if (nchunks > 1) issue(1, 1);
      }
      __syncthreads();

      int cur = -1;
      ACC acc;
      acc.zero();
      auto flush = [&]() {
        if (direct) out_red_acc(J, (size_t)cur, p, P, acc);
        else cell_add(region + cur, acc, V == 1);
      };
      for (int c = 0; c < nchunks; ++c) {
        const int b = c & 1;
        const uint32_t parity = (b == 0 ? uses0 : uses1) & 1;
        if (!mbar_wait(&bar[b], parity, kp.flags)) s_abort = 1;
        if (b == 0) ++uses0; else ++uses1;
        __syncthreads();
        if (s_abort) break;
        const int s0 = w.start + c * K;
        const int m = min(K, w.end - s0);
        const int2 *ib = reinterpret_cast<const int2 *>(idxbuf[b] + (((size_t)s0 * 8) & 15));
        const VT2 *vb = reinterpret_cast<const VT2 *>(valbuf[b] + (((size_t)s0 * sizeof(VT2)) & 15));
        const int r0 = (grp * m) / V, r1 = ((grp + 1) * m) / V;
        for (int r = r0; r < r1; ++r) {
          const int2 pk = ib[r];
          const VT2 v = vb[r];
          const int mx = unpack_main(pk.x, log2G), sx = unpack_sub(pk.x, log2G);
          const int my = unpack_main(pk.y, log2G), sy = unpack_sub(pk.y, log2G);
          const int fx0 = mx - H + 1, fy0 = my - H + 1;
          const int ap = (rx - fx0) & (S - 1), bp = (ry - fy0) & (S - 1);
          const int gx = fx0 + ap, gy = fy0 + bp;
          bool on = (unsigned)gx < (unsigned)N && (unsigned)gy < (unsigned)N;
          int lc = -1;
          if (on) {
            if (direct) {
              lc = gy * N + gx;
            } else {
              int lx = gx - ox, ly = gy - oy;
              if ((unsigned)lx < (unsigned)R && (unsigned)ly < (unsigned)R) {
                lc = ly * R + lx;
              } else {
                atomicOr(&kp.flags[FLAG_BOUNDS], 1);
                on = false;
              }
            }
          }
          if (lc != cur) {
            if (cur >= 0) flush();
            cur = lc;
            acc.zero();
          }
          if (on) {
            VT gr, gi, tr, ti;
            gsrc.value(sx, sy, ap, bp, gr, gi);
            if constexpr (GAUSS) {
              tr = v.x * gr;
              ti = v.y * gr;
            } else {
              cmul<VT>(v.x, v.y, gr, gi, tr, ti);
            }
            acc.add(tr, ti);
          }
        }
        __syncthreads();  // buffer b fully consumed
        if (tid == 0 && c + 2 < nchunks) issue(c + 2, b);
      }
      if (cur >= 0 && !s_abort) flush();
      __syncthreads();
      if (!direct && !s_abort) {
        for (int i = tid; i < R * R; i += NT) {
          const int gx = ox + i % R, gy = oy + i / R;
          if ((unsigned)gx >= (unsigned)N || (unsigned)gy >= (unsigned)N) continue;
          ACC a;
          cell_load(region[i], a);
          if (a.nonzero()) out_red_acc(J, (size_t)gy * N + gx, p, P, a);
        }
      }
      __syncthreads();
      if (s_abort) break;
    }
  }
  // A timed-out copy may still be in flight: drain both barriers (bounded)
  // before the CTA's shared memory is released.
  if (s_abort && tid == 0) {
    mbar_wait(&bar[0], uses0 & 1, nullptr);
    mbar_wait(&bar[1], uses1 & 1, nullptr);
  }
}

size_t window_smem_bytes_t(int S, int accum, int vals_f64, int T) {
  switch (S) {
#define GG_WS(SV)                                                        \
  case SV:                                                               \
    if (vals_f64) return WinShape<SV, AccF64>::smem(T);                  \
    if (accum == GG_ACC_COMPENSATED) return WinShape<SV, AccComp>::smem(T); \
    return WinShape<SV, AccF32>::smem(T);
    GG_WS(4) GG_WS(8) GG_WS(16) GG_WS(32)
#undef GG_WS
  }
  return 0;
}

template <int S, class ACC, bool GAUSS>
static cudaError_t win_launch(const KParams &kp, int sm_count, cudaStream_t s) {
  using Sh = WinShape<S, ACC>;
  size_t smem = Sh::smem(kp.T);
  auto kern = window_kernel<S, ACC, GAUSS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Sh::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<sm_count * per_sm, Sh::NT, smem, s>>>(kp);
  count_launch();
  return cudaGetLastError();
}

template <int S>
static cudaError_t win_dispatch(const GridLaunch &g, const KParams &kp,
                                cudaStream_t s) {
  if (g.vals_f64)
    return g.gauss ? win_launch<S, AccF64, true>(kp, g.sm_count, s)
                   : win_launch<S, AccF64, false>(kp, g.sm_count, s);
  if (g.accum == GG_ACC_COMPENSATED)
    return g.gauss ? win_launch<S, AccComp, true>(kp, g.sm_count, s)
                   : win_launch<S, AccComp, false>(kp, g.sm_count, s);
  return g.gauss ? win_launch<S, AccF32, true>(kp, g.sm_count, s)
                 : win_launch<S, AccF32, false>(kp, g.sm_count, s);
}

cudaError_t launch_window(const GridLaunch &g, cudaStream_t s) {
  KParams kp{};
  kp.jobs = g.jobs;
  kp.items = g.items;
  kp.nitems = g.nitems;
  kp.item_next = g.item_next;
  kp.flags = g.flags;
  kp.njobs = g.njobs;
  kp.P = g.P;
  kp.T = g.tile;
  kp.G = g.G;
  kp.sigma = g.sigma;
  switch (g.S) {
    case 4: return win_dispatch<4>(g, kp, s);
    case 8: return win_dispatch<8>(g, kp, s);
    case 16: return win_dispatch<16>(g, kp, s);
    case 32: return win_dispatch<32>(g, kp, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gg
