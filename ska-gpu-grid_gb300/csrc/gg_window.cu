// Moving-window gridding (the reference's MOVING_WINDOW method,
// grid_kernel_window, grid_gpu.cu:504-673), rebuilt for sm_103a.
//
// The reference gives each thread a fixed residue (x mod S, y mod S) of the
// support, keeps a register sum while the target cell of consecutive (sorted)
// visibilities is unchanged and flushes it with a global CAS atomic when the
// cell changes.  The property that makes this work is kept and pushed further:
// a cell (x, y) is only ever reached through residue (x mod S, y mod S), so
// the thread that owns that residue is the only one that ever touches it.
//
//  * Work is split into independent groups of W warps.  Each group owns a
//    private (T+S-1)^2 shared-memory sub-grid covering one uv tile plus the
//    footprint halo, its own double-buffered TMA staging area and mbarriers,
//    and pulls work items (slices of one tile's sorted visibilities) from the
//    device queue on its own: groups never wait for each other.
//  * Inside a group every thread owns Q = S*S/(32 W) residues of one column.
//    For each residue it keeps a register sum while the target cell stays the
//    same and, when it changes, adds the sum into the sub-grid.  Ownership
//    makes that read-modify-write exclusive: no atomics, and no
//    synchronisation between visibilities.  One-warp groups, whose lanes
//    step through the records together, own taps instead on interior tiles
//    (fixed table offsets, a __syncwarp per run), which halves the table's
//    L1 footprint.
//  * FP32 sums are compensated: sub-grid cells hold a (hi, lo) pair per
//    component, updated with Knuth's TwoSum on the packed (re, im) pair
//    (f32x2 instructions) whenever a register run is added in; register runs
//    are cut after kRunMax records, which bounds their plain-FP32 error.
//  * Visibility records (both main cells in one word + the sub-kernel index,
//    and the values) stream through shared memory by 1-D TMA bulk copies,
//    double-buffered, as one continuous stream across work items (the next
//    item is claimed early and its first chunk prefetched while the current
//    one is gridded).
//  * Records come in runs with an unchanged footprint origin.  The first
//    record of a run works out the target cells and adds every register sum
//    into its cell (the Q read-modify-writes of a thread issued together);
//    the rest of the run goes through a fast loop
//    that only loads GCF values (two records ahead of their use, at fixed
//    strides in a row-doubled copy of the table) and accumulates.  Tables
//    without imaginary parts (flagged on the device) take a real-factor
//    variant.
//  * Once per item the sub-grid is flushed to HBM with native vector
//    reductions (touched cells only) and zeroed as it is read.  Items too
//    sparse to pay for that flush, and edge tiles (whose clamped mains may
//    reach outside the sub-grid), take a bounds-checked one-stage loop; the
//    sparse ones send each register sum straight to HBM.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "gg_kernels.cuh"

namespace gg {

// ---- per-thread running sums and sub-grid cells -------------------------------
// MODE 0: plain FP32      sum u64 (re, im)          cell float2
// MODE 1: compensated     sums u64 hi, lo           cell float4 {hi, lo}
// MODE 2: FP64            sums double re, im        cell double2
template <int MODE> struct WinAcc;
template <> struct WinAcc<0> {
  using VT = float;
  using CellT = float2;
  u64 s;
  __device__ __forceinline__ CellT merged(const CellT o) const {
    return upk2(add2(pk2(o.x, o.y), s));
  }
  __device__ __forceinline__ void zero() { s = 0ull; }
  __device__ __forceinline__ void add(u64 t) { s = add2(s, t); }
  __device__ __forceinline__ void fma(u64 v, u64 g) { s = fma2(v, g, s); }
  __device__ __forceinline__ void into(CellT *c) const {
    const float2 o = *c;
    *c = upk2(add2(pk2(o.x, o.y), s));
  }
  __device__ __forceinline__ void out(const JobDesc &J, size_t cell, int p, int P) const {
    const float2 v = upk2(s);
    out_red(J, cell, p, P, (double)v.x, (double)v.y);
  }
};
// Compensated: a register run of at most kRunMax records is summed plainly in
// FP32 and every run is added into a two-sum (hi, lo) cell, so the rounding
// error is that of one short run per cell plus O(u^2) terms, not O(n u).
template <> struct WinAcc<1> {
  using VT = float;
  using CellT = float4;
  u64 s;
  __device__ __forceinline__ CellT merged(const CellT o) const {
    u64 e;
    const u64 h = two_sum2(pk2(o.x, o.y), s, e);
    const float2 hf = upk2(h), lf = upk2(add2(pk2(o.z, o.w), e));
    return make_float4(hf.x, hf.y, lf.x, lf.y);
  }
  __device__ __forceinline__ void zero() { s = 0ull; }
  __device__ __forceinline__ void add(u64 t) { s = add2(s, t); }
  __device__ __forceinline__ void fma(u64 v, u64 g) { s = fma2(v, g, s); }
  __device__ __forceinline__ void into(CellT *c) const {
    const float4 o = *c;
    u64 e;
    const u64 h = two_sum2(pk2(o.x, o.y), s, e);
    const float2 hf = upk2(h), lf = upk2(add2(pk2(o.z, o.w), e));
    *c = make_float4(hf.x, hf.y, lf.x, lf.y);
  }
  __device__ __forceinline__ void out(const JobDesc &J, size_t cell, int p, int P) const {
    const float2 v = upk2(s);
    out_red(J, cell, p, P, (double)v.x, (double)v.y);
  }
};
template <> struct WinAcc<2> {
  using VT = double;
  using CellT = double2;
  double re, im;
  __device__ __forceinline__ CellT merged(const CellT o) const {
    return make_double2(__dadd_rn(o.x, re), __dadd_rn(o.y, im));
  }
  __device__ __forceinline__ void zero() { re = im = 0.0; }
  // adds v * g for packed FP32 pairs (v complex, g = (r, r) real factor)
  __device__ __forceinline__ void fma(u64 v, u64 g) {
    const float2 a = upk2(v), b = upk2(g);
    add((double)a.x * b.x, (double)a.y * b.x);
  }
  __device__ __forceinline__ void add(double tr, double ti) {
    re = __dadd_rn(re, tr);
    im = __dadd_rn(im, ti);
  }
  __device__ __forceinline__ void into(CellT *c) const {
    const double2 o = *c;
    *c = make_double2(__dadd_rn(o.x, re), __dadd_rn(o.y, im));
  }
  __device__ __forceinline__ void out(const JobDesc &J, size_t cell, int p, int P) const {
    out_red(J, cell, p, P, re, im);
  }
};

__device__ __forceinline__ bool cell_nonzero(const float2 &c) { return c.x != 0.f || c.y != 0.f; }
__device__ __forceinline__ bool cell_nonzero(const float4 &c) {
  return c.x != 0.f || c.y != 0.f || c.z != 0.f || c.w != 0.f;
}
__device__ __forceinline__ bool cell_nonzero(const double2 &c) { return c.x != 0.0 || c.y != 0.0; }

// flush of a finished sub-grid cell into the output grid (reduction)
__device__ __forceinline__ void out_cell(const JobDesc &J, size_t cell, int p,
                                         int P, const float2 &c) {
  out_red(J, cell, p, P, (double)c.x, (double)c.y);
}
__device__ __forceinline__ void out_cell(const JobDesc &J, size_t cell, int p,
                                         int P, const float4 &c) {
  // complex128 grid: hi+lo exactly; complex64 grid: hi+lo rounded once
  if (J.out_f64)
    out_red(J, cell, p, P, (double)c.x + (double)c.z, (double)c.y + (double)c.w);
  else
    out_red(J, cell, p, P, (double)__fadd_rn(c.x, c.z), (double)__fadd_rn(c.y, c.w));
}
__device__ __forceinline__ void out_cell(const JobDesc &J, size_t cell, int p,
                                         int P, const double2 &c) {
  out_red(J, cell, p, P, c.x, c.y);
}

// exact (hi + lo in FP64) addition of a compensated sub-grid cell into a merge
// slot cell; the other cell types never reach a slot
__device__ __forceinline__ void merge_cell(double2 *d, const float4 &c) {
  red_add(&d->x, (double)c.x + (double)c.z);
  red_add(&d->y, (double)c.y + (double)c.w);
}
__device__ __forceinline__ void merge_cell(double2 *, const float2 &) {}
__device__ __forceinline__ void merge_cell(double2 *, const double2 &) {}

// ---- configuration ----------------------------------------------------------------
constexpr int kWinThreads = 256;
// longest register run (records) of the compensated mode: a run of L terms
// carries at most about L/2 units in the last place of relative error
constexpr int kRunMax = 32;

// warps per sub-grid group chosen when the caller leaves it open, by support
// and tile (measured on the track and disk workloads: one-warp groups for
// support 8 on 8-cell tiles, where their sub-grids are small enough for three
// CTAs per SM; two warps otherwise for supports 8 and 16; four for 32)
__host__ __device__ constexpr int win_default_warps(int S, int T) {
  return S >= 32 ? 4 : (S >= 16 ? 2 : (S >= 8 ? (T <= 8 ? 1 : 2) : 1));
}

template <int S, int W> struct WinCfg {
  static constexpr int NGT = 32 * W;                         // threads per group
  static constexpr int Q = (S * S + NGT - 1) / NGT;          // residues per thread
  // records per chunk (staging buffers).  48 for S=16: two CTAs of one-warp
  // groups on 8-cell tiles then take 159.5 KB of shared memory, under the
  // 164 KB carveout, which leaves 92 KB of L1 for the 64 KB of table rows the
  // tap-owning lanes read (64 records per chunk left 60 KB: 5 % slower)
  static constexpr int K = S >= 32 ? 512 : (S >= 16 ? 48 : 128);
  static constexpr int GROUPS = kWinThreads / NGT;

};

template <int S, int W, int MODE, bool GAUSS>
struct WinLayout {
  using Cfg = WinCfg<S, W>;
  using VT2 = typename vec2_of<typename WinAcc<MODE>::VT>::type;
  using CellT = typename WinAcc<MODE>::CellT;
  static constexpr int IDX_BUF = Cfg::K * 8 + 16;
  static constexpr int VAL_BUF = Cfg::K * (int)sizeof(VT2) + 16;
  // 1-D Gaussian factors (computed GCF only): doubled rows, G <= 64
  static constexpr int G1_BYTES = GAUSS ? 64 * 2 * S * 4 : 0;
  // per group: 2 mbarriers (16 B), 2 index buffers, 2 value buffers, sub-grid
  __host__ __device__ static size_t group_bytes(int T) {
    const size_t R = (size_t)T + S - 1;
    return (16 + 2 * IDX_BUF + 2 * VAL_BUF + R * R * sizeof(CellT) + 15) & ~(size_t)15;
  }
  __host__ __device__ static size_t cta_bytes(int T) {
    return G1_BYTES + Cfg::GROUPS * group_bytes(T);
  }
};

__device__ __forceinline__ void group_sync(int gid, int nthreads) {
  if (nthreads == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(nthreads) : "memory");
  }
}

// Resident CTAs per SM the register allocation is held to: as many as the
// shared memory of the configuration allows at the default tile (16) -- for
// one-warp groups of supports 8 and 16, at the 8-cell tile -- where the
// compiler then fits the loop (one-warp support-16 groups with a few spilled
// bytes, measured faster than one CTA per SM); FP64 sums get one fewer.
// Support 32 with four-warp groups: two CTAs only for plain FP32 sums, whose
// float2 cells let two CTAs' sub-grids fit an SM.
__host__ __device__ constexpr int win_min_ctas(int S, int W, int MODE) {
  return S <= 4 ? 2
         : S <= 8 ? (W == 1 ? (MODE == 2 ? 2 : 3) : (MODE == 2 ? 3 : 4))
         : S <= 16 ? (W == 1 ? (MODE == 2 ? 1 : 2) : (MODE == 2 ? 2 : 3))
                   : (W == 8 || MODE == 0 ? 2 : 1);
}

template <int S, int W, int MODE, bool GAUSS>
__global__ void __launch_bounds__(kWinThreads, win_min_ctas(S, W, MODE))
    window_kernel(KParams kp) {
  using Cfg = WinCfg<S, W>;
  using L = WinLayout<S, W, MODE, GAUSS>;
  using ACC = WinAcc<MODE>;
  using VT2 = typename L::VT2;
  using CellT = typename L::CellT;
  constexpr int NGT = Cfg::NGT, Q = Cfg::Q, K = Cfg::K, GROUPS = Cfg::GROUPS;
  constexpr int H = S / 2;
  // Input declared tile-sorted but found unsorted by this call's binning:
  // the sorted records have holes (never written) and the call fails with
  // GG_ERR_UNSORTED -- grid nothing.
  if (kp.holes && *kp.holes) return;

  extern __shared__ __align__(16) unsigned char smem[];
  float *g1 = reinterpret_cast<float *>(smem);
  const int tid = threadIdx.x;
  const int gid = tid / NGT, gt = tid % NGT;
  const int P = kp.P, T = kp.T, R = T + S - 1;
  const size_t gbytes = L::group_bytes(T);
  unsigned char *gbase_p = smem + L::G1_BYTES + gid * gbytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(gbase_p);
  unsigned char *const idx0 = gbase_p + 16;
  unsigned char *const val0 = gbase_p + 16 + 2 * L::IDX_BUF;
  CellT *region = reinterpret_cast<CellT *>(gbase_p + 16 + 2 * L::IDX_BUF + 2 * L::VAL_BUF);
  __shared__ int s_item[GROUPS], s_next[GROUPS], s_abort[GROUPS];

  // residues of this thread: r = gt + k*NGT -> column rx (the same for every
  // k, NGT being a multiple of S), rows ry[k]
  const int rx = gt % S;
  int ry[Q];
  bool rv[Q];
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const int r = gt + k * NGT;
    rv[k] = r < S * S;
    ry[k] = r / S;
  }
  const int nitems = *kp.nitems;
  const bool leader = gt == 0;
  // One-warp groups on interior tiles own taps instead of residues: thread
  // gt adds the taps (rx, ry[k]) of every footprint, so its table offsets are
  // the same for every record -- only the first S rows of each row-doubled
  // sub-kernel are read, half the L1 footprint of the rotating offsets (for
  // support 16, 64 KB instead of 128 KB beside two CTAs' sub-grids) -- and
  // its cells move with the footprint.  A cell then passes from lane to lane
  // across footprint moves, ordered by __syncwarp.  Wider groups, whose
  // warps run apart, keep residue ownership (no cell shared by threads).
  // Each cell still receives the same register sums in the same order.
  constexpr bool TAPS = W == 1 && S * S % NGT == 0;

  if (leader) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort[gid] = 0;
    const int a = atomicAdd(kp.item_next, 1);
    s_item[gid] = a;
    s_next[gid] = a < nitems ? atomicAdd(kp.item_next, 1) : nitems;
  }
  if constexpr (GAUSS) gauss_fill(g1, S, kp.G, kp.sigma, tid, kWinThreads, 2 * S);
  for (int i = gt; i < R * R; i += NGT) region[i] = CellT{};
  __syncthreads();

  // Chunk stream of this group: chunk g lives in buffer g&1, whose (g>>1)-th
  // use completes barrier phase (g>>1)&1.  The leader keeps two in flight,
  // looking one (item, plane) ahead.
  int gfirst = 0;  // stream number of the current (item, plane)'s first chunk
  int issued = 0, waited = 0;
  int item = s_item[gid], next = s_next[gid];

  auto issue = [&](int g, int it, int c, int p) {
    const WorkItem wi = kp.items[it];
    const int s0 = wi.start + c * K;
    const int e0 = min(wi.end, s0 + K);
    const JobDesc &J = kp.jobs[wi.job];
    const VT2 *vplane = reinterpret_cast<const VT2 *>(J.vals) + (size_t)p * J.vstride;
    const size_t i0 = (size_t)s0 * 8, i1 = (size_t)e0 * 8;
    const size_t v0 = (size_t)s0 * sizeof(VT2), v1 = (size_t)e0 * sizeof(VT2);
    const uint32_t bytes = (uint32_t)(((i1 + 15) & ~(size_t)15) - (i0 & ~(size_t)15)) +
                           (uint32_t)(((v1 + 15) & ~(size_t)15) - (v0 & ~(size_t)15));
    const int b = g & 1;
    fence_proxy_async();
    mbar_expect_tx(&bar[b], bytes);
    stage_span(idx0 + b * L::IDX_BUF, reinterpret_cast<const char *>(J.idx), i0, i1, &bar[b]);
    stage_span(val0 + b * L::VAL_BUF, reinterpret_cast<const char *>(vplane), v0, v1, &bar[b]);
  };

  int p = 0;  // polarisation plane of the current (item, plane)
  while (item < nitems) {
    const WorkItem w = kp.items[item];
    const JobDesc &J = kp.jobs[w.job];
    const int N = J.N, log2G = J.log2G;
    // bin = uv tile * n_gcf + table index (per-visibility GCF tables)
    const int tile = J.n_gcf > 1 ? w.bin / J.n_gcf : w.bin;
    const int tab = w.bin - tile * J.n_gcf;
    const int tx = tile % J.ntx, ty = tile / J.ntx;
    const int ox = tx * T - H + 1, oy = ty * T - H + 1;  // sub-grid origin
    const int n = w.end - w.start;
    const int nch = (n + K - 1) / K;
    // FP64 merge slot of a tile cut into several items (compensated FP32 into
    // a complex64 grid): the item's sub-grid is added into it exactly
    double2 *const mslot = MODE == 1 && kp.merge.base && w.slot >= 0
                               ? kp.merge.base + (size_t)w.slot * kp.merge.cells + (size_t)p * R * R
                               : nullptr;
    const bool direct = !mslot && (long long)n * S * S < (long long)R * R;
    // what follows in the stream: the next plane of this item, or the next item
    const int nxt_item = p + 1 < P ? item : next;
    const int nxt_p = p + 1 < P ? p + 1 : 0;
    int nxt_chunks = 0;
    if (nxt_item < nitems) {
      const WorkItem w2 = kp.items[nxt_item];
      nxt_chunks = (w2.end - w2.start + K - 1) / K;
    }
    auto issue_next = [&](int limit) {
      while (issued < gfirst + nch + nxt_chunks && issued < limit) {
        const int c = issued - gfirst;
        if (c < nch) issue(issued, item, c, p);
        else issue(issued, nxt_item, c - nch, nxt_p);
        ++issued;
      }
    };
    if (leader) issue_next(gfirst + 2);

    const VT2 *gtab = reinterpret_cast<const VT2 *>(J.gcf) + (size_t)tab * J.G * J.G * 2 * S * S;
    // FP32 table without imaginary parts: the real-factor fast path
    const bool real_tab = !GAUSS && MODE != 2 && J.gcf_real && J.gcf_imag && *J.gcf_imag == 0;
    const float *const greal =
        real_tab ? J.gcf_real + (size_t)tab * J.G * J.G * 2 * S * S : nullptr;
    const int G = J.G;
    // tiles on the border of the grid hold the clamped mains, whose
    // footprints may leave the sub-grid
    const bool edge = tx == 0 || ty == 0 || tx == J.ntx - 1 || ty == J.ntx - 1;
    ACC acc[Q];
    int cur[Q];
    // footprint origin of the last record, this thread's column in it and
    // the offset of its first tap in a sub-kernel of the row-doubled table
    int pfx = INT_MIN, pfy = INT_MIN, pax = 0, pofs = 0, pkm = -1;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      acc[k].zero();
      cur[k] = -1;
    }
    int run = 0;  // records in the current register runs (compensated mode)
    auto flush_runs = [&]() {
      run = 0;
#pragma unroll
      for (int k = 0; k < Q; ++k)
        if (cur[k] >= 0) {
          if (direct) acc[k].out(J, (size_t)cur[k], p, P);
          else acc[k].into(region + cur[k]);
          acc[k].zero();
        }
    };

    for (int c = 0; c < nch; ++c) {
      const int g = gfirst + c, b = g & 1;
      if (mbar_wait(&bar[b], (g >> 1) & 1, kp.flags)) waited = g + 1;
      else s_abort[gid] = 1;
      group_sync(gid, NGT);
      if (s_abort[gid]) break;
      const int s0 = w.start + c * K;
      const int m = min(K, w.end - s0);
      const int2 *ib = reinterpret_cast<const int2 *>(idx0 + b * L::IDX_BUF + (((size_t)s0 * 8) & 15));
      const VT2 *vb = reinterpret_cast<const VT2 *>(val0 + b * L::VAL_BUF +
                                                    (((size_t)s0 * sizeof(VT2)) & 15));
      // Interior tiles.  Records come in runs whose footprint origin does
      // not move (the same target cell for every residue); the slow step
      // handles the first record of a run (target cells, flushes of the
      // register sums whose cell changed), the fast loop only adds records
      // while the origin stays put.  Both decisions are uniform over the
      // group.  The fast loop is unrolled by two with two register stages:
      // it decodes record r+1 and issues its GCF loads before adding record
      // r, so that a record's load latency is hidden behind the previous one.
      using GT = typename vec2_of<typename ACC::VT>::type;
      // The GCF table seen here repeats every sub-kernel's rows once
      // ([G*G][2S][S]): this thread's Q taps of a record, rows b0 + k*D mod S,
      // then sit at fixed strides k*D*S from its first tap.
      constexpr int D = NGT / S;
      auto load_g = [&](GT (&g)[Q], int sub) {
        if constexpr (GAUSS) {
          const int sx = sub & (G - 1), sy = sub >> log2G;
          const float gxf = g1[sx * 2 * S + pax];
          const float *gy = g1 + sy * 2 * S + pofs;
#pragma unroll
          for (int k = 0; k < Q; ++k) {
            g[k].x = (typename ACC::VT)(gxf * gy[k * D]);
            g[k].y = 0;
          }
        } else {
          const GT *gp = reinterpret_cast<const GT *>(gtab) + sub * (2 * S * S) + pofs;
#pragma unroll
          for (int k = 0; k < Q; ++k) g[k] = __ldg(gp + k * D * S);
        }
      };
      auto accum = [&](const GT (&g)[Q], const VT2 v) {
        u64 vrr = 0, vsn = 0, vv = 0;
        if constexpr (MODE != 2) {
          vv = pk2((float)v.x, (float)v.y);
          vrr = pk2((float)v.x, (float)v.x);
          vsn = pk2(-(float)v.y, (float)v.y);
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
          if (S * S % NGT != 0 && !rv[k]) continue;
          if constexpr (MODE == 2) {
            acc[k].add(v.x * g[k].x - v.y * g[k].y, v.x * g[k].y + g[k].x * v.y);
          } else if constexpr (GAUSS) {
            acc[k].add(mul2(vv, pk2((float)g[k].x, (float)g[k].x)));
          } else {
            acc[k].add(fma2(vrr, pk2((float)g[k].x, (float)g[k].y),
                            mul2(vsn, pk2((float)g[k].y, (float)g[k].x))));
          }
        }
      };
      // One step of the fast loop: add record r (stage a).  Record r+1 is in
      // stage b and continues the run when `nb`.  Record r+2 is decoded and
      // loaded into stage c whether or not it continues the run (index
      // clamped to the chunk; a wasted load at a run's end costs less than
      // a branch around it), and `nc` says whether it does: same footprint
      // origin and inside `mr`, the chunk end or the run-length limit.
      // Loads run two records ahead of their use.
      //
      // RG: the item's table has no imaginary part (checked on the device
      // when the row-doubled copy is made): the stages hold the real parts
      // only (half the table bytes) and a tap is one fused multiply-add of
      // the complex value by the real factor.
      auto run_interior = [&](auto real_tag) {
        constexpr bool RG = decltype(real_tag)::value;
        using GS = typename std::conditional<RG, float, GT>::type;
        auto load = [&](GS (&g)[Q], int sub) {
          if constexpr (RG && MODE != 2) {
            const float *gp = greal + sub * (2 * S * S) + pofs;
#pragma unroll
            for (int k = 0; k < Q; ++k) g[k] = __ldg(gp + k * D * S);
          } else {
            load_g(g, sub);
          }
        };
        auto add_rec = [&](const GS (&g)[Q], const VT2 v) {
          if constexpr (RG && MODE != 2) {
            const u64 vv = pk2((float)v.x, (float)v.y);
#pragma unroll
            for (int k = 0; k < Q; ++k) {
              if (S * S % NGT != 0 && !rv[k]) continue;
              acc[k].fma(vv, pk2(g[k], g[k]));
            }
          } else {
            accum(g, v);
          }
        };
        auto step = [&](int r, int mr, const GS (&ga)[Q], const VT2 va, GS (&gc)[Q], VT2 &vc,
                        bool &nc) {
          const int r2 = min(r + 2, m - 1);
          const int2 q = ib[r2];
          vc = vb[r2];
          nc = q.x == pkm && r + 2 < mr;
          load(gc, q.y);
          add_rec(ga, va);
        };
        int r = 0;
        while (r < m) {
          // slow step: record r opens a run
          const int2 pk = ib[r];
          VT2 va = vb[r], vb1, vc1;
          const int fx0 = (int)((unsigned)pk.x & 0xffffu) - kWinMainBias - H + 1;
          const int fy0 = (int)((unsigned)pk.x >> 16) - kWinMainBias - H + 1;
          if constexpr (TAPS) __syncwarp();  // other lanes' cell updates seen
          if (MODE == 1 && run >= kRunMax) flush_runs();
          if (fx0 != pfx || fy0 != pfy) {
            pfx = fx0;
            pfy = fy0;
            pax = TAPS ? rx : (rx - fx0) & (S - 1);
            const int b0 = TAPS ? ry[0] : (ry[0] - fy0) & (S - 1);
            pofs = GAUSS ? b0 : b0 * S + pax;
            const int lx = fx0 + pax - ox;
            if constexpr (S * S % NGT == 0) {
              // Every register sum goes to its cell on a footprint move,
              // changed or not: the Q read-modify-writes of a thread are
              // issued together (distinct cells, no aliasing) instead of one
              // branch per residue, which a warp takes whenever any lane's
              // cell changed -- on most moves.  Adding a sum into a cell that
              // stays current only splits a register run.  A sum with no
              // cell yet is zero and goes to its new cell.
              int cc[Q], lcs[Q];
              CellT cv[Q];
#pragma unroll
              for (int k = 0; k < Q; ++k) {
                const int bp = (b0 + k * D) & (S - 1);
                lcs[k] = (fy0 + bp - oy) * R + lx;
                cc[k] = cur[k] >= 0 ? cur[k] : lcs[k];
                cv[k] = region[cc[k]];
              }
#pragma unroll
              for (int k = 0; k < Q; ++k) region[cc[k]] = acc[k].merged(cv[k]);
#pragma unroll
              for (int k = 0; k < Q; ++k) {
                cur[k] = lcs[k];
                acc[k].zero();
              }
            } else {
#pragma unroll
              for (int k = 0; k < Q; ++k) {
                const int bp = (b0 + k * D) & (S - 1);
                const int lc = (S * S % NGT == 0 || rv[k]) ? (fy0 + bp - oy) * R + lx : -1;
                if (lc != cur[k]) {
                  if (cur[k] >= 0) acc[k].into(region + cur[k]);
                  cur[k] = lc;
                  acc[k].zero();
                }
              }
            }
          }
          // the main cells of this run and the last record the run may reach
          pkm = pk.x;
          const int r0 = r;
          const int mr = MODE == 1 ? min(m, r0 + (kRunMax - run)) : m;
          GS ga[Q], gb[Q], gc[Q];
          load(ga, pk.y);
          const int r1 = min(r + 1, m - 1);
          const int2 q = ib[r1];
          vb1 = vb[r1];
          bool nb = q.x == pkm && r + 1 < mr, nc, na;
          load(gb, q.y);
          // fast loop over the rest of the run, three rotating stages
          for (;;) {
            step(r++, mr, ga, va, gc, vc1, nc);
            if (!nb) break;
            step(r++, mr, gb, vb1, ga, va, na);
            if (!nc) break;
            step(r++, mr, gc, vc1, gb, vb1, nb);
            if (!na) break;
          }
          run += r - r0;
        }
      };
      // Edge tiles and sparse items (a small share of the taps) take a plain
      // one-stage loop with bounds tests: it keeps the register footprint of
      // the kernel at that of the interior path.
      auto run_checked = [&]() {
        const int LIM = direct ? N : R;
        const int bx = direct ? 0 : ox, by = direct ? 0 : oy;
        for (int r = 0; r < m; ++r) {
          if (MODE == 1 && ++run >= kRunMax) flush_runs();
          const int2 pk = ib[r];
          const VT2 v = vb[r];
          const int mx = (int)((unsigned)pk.x & 0xffffu) - kWinMainBias;
          const int my = (int)((unsigned)pk.x >> 16) - kWinMainBias;
          const int sx = pk.y & (G - 1), sy = pk.y >> log2G;
          const int fx0 = mx - H + 1, fy0 = my - H + 1;
          const int ap = (rx - fx0) & (S - 1);
          const int lx = fx0 + ap - bx;
          const bool xin = (unsigned)lx < (unsigned)LIM;
#pragma unroll
          for (int k = 0; k < Q; ++k) {
            const int bp = (ry[k] - fy0) & (S - 1);
            const int ly = fy0 + bp - by;
            const bool in = (S * S % NGT == 0 || rv[k]) && xin && (unsigned)ly < (unsigned)LIM;
            const int lc = in ? ly * LIM + lx : -1;
            if (lc != cur[k]) {
              if (cur[k] >= 0) {
                if (direct) acc[k].out(J, (size_t)cur[k], p, P);
                else acc[k].into(region + cur[k]);
              }
              cur[k] = lc;
              acc[k].zero();
            }
            if (lc < 0) continue;
            GT g;
            if constexpr (GAUSS) {
              g.x = (typename ACC::VT)(g1[sx * 2 * S + ap] * g1[sy * 2 * S + bp]);
              g.y = 0;
            } else {
              g = __ldg(reinterpret_cast<const GT *>(gtab) + (sy * G + sx) * (2 * S * S) +
                        bp * S + ap);
            }
            if constexpr (MODE == 2) {
              acc[k].add(v.x * g.x - v.y * g.y, v.x * g.y + g.x * v.y);
            } else {
              const u64 vrr = pk2((float)v.x, (float)v.x), vsn = pk2(-(float)v.y, (float)v.y);
              acc[k].add(fma2(vrr, pk2((float)g.x, (float)g.y),
                              mul2(vsn, pk2((float)g.y, (float)g.x))));
            }
          }
        }
      };
      if (direct || edge) {
        run_checked();
      } else {
        if constexpr (!GAUSS && MODE != 2) {
          if (real_tab) run_interior(std::true_type{});
          else run_interior(std::false_type{});
        } else {
          run_interior(std::false_type{});
        }
      }
      group_sync(gid, NGT);  // buffer b consumed by the whole group
      if (leader) issue_next(g + 3);
    }
    if (s_abort[gid]) break;
    if constexpr (TAPS) __syncwarp();
#pragma unroll
    for (int k = 0; k < Q; ++k)
      if (cur[k] >= 0) {
        if (direct) acc[k].out(J, (size_t)cur[k], p, P);
        else acc[k].into(region + cur[k]);
      }
    if (!direct) {
      group_sync(gid, NGT);  // all register sums are in the sub-grid
      // walk cell i = gt, gt + NGT, ... keeping its (x, y) by increments (R
      // is not a power of two: no division per cell)
      const int sdx = NGT % R, sdy = NGT / R;
      int cx = gt % R, cy = gt / R;
      for (int i = gt; i < R * R; i += NGT) {
        const CellT cv = region[i];
        if (cell_nonzero(cv)) {
          region[i] = CellT{};
          if (mslot) {
            merge_cell(mslot + i, cv);
          } else {
            const int gx = ox + cx, gy = oy + cy;
            if ((unsigned)gx < (unsigned)N && (unsigned)gy < (unsigned)N)
              out_cell(J, (size_t)gy * N + gx, p, P, cv);
          }
        }
        cx += sdx;
        cy += sdy;
        if (cx >= R) {
          cx -= R;
          ++cy;
        }
      }
    }
    // advance the stream: next plane of this item, or the next item
    gfirst += nch;
    if (p + 1 < P) {
      ++p;
    } else {
      p = 0;
      if (leader) {
        s_item[gid] = next;
        s_next[gid] = next < nitems ? atomicAdd(kp.item_next, 1) : nitems;
      }
      group_sync(gid, NGT);
      item = s_item[gid];
      next = s_next[gid];
    }
    group_sync(gid, NGT);  // sub-grid zeroed before the next item's updates
  }
  // A timed-out copy may still be in flight: drain this group's barriers
  // (bounded) before the CTA's shared memory is released.
  if (s_abort[gid] && leader)
    for (int g = waited; g < issued; ++g) mbar_wait(&bar[g & 1], (g >> 1) & 1, nullptr);
}

template <int S, int W, int MODE, bool GAUSS>
static cudaError_t win_launch(const KParams &kp, int sm_count, cudaStream_t s) {
  using L = WinLayout<S, W, MODE, GAUSS>;
  const size_t smem = L::cta_bytes(kp.T);
  auto kern = window_kernel<S, W, MODE, GAUSS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWinThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<sm_count * per_sm, kWinThreads, smem, s>>>(kp);
  count_launch();
  return cudaGetLastError();
}

template <int S, int W>
static cudaError_t win_modes(const GridLaunch &g, const KParams &kp, cudaStream_t s) {
  if (g.vals_f64)
    return g.gauss ? win_launch<S, W, 2, true>(kp, g.sm_count, s)
                   : win_launch<S, W, 2, false>(kp, g.sm_count, s);
  if (g.accum == GG_ACC_COMPENSATED)
    return g.gauss ? win_launch<S, W, 1, true>(kp, g.sm_count, s)
                   : win_launch<S, W, 1, false>(kp, g.sm_count, s);
  return g.gauss ? win_launch<S, W, 0, true>(kp, g.sm_count, s)
                 : win_launch<S, W, 0, false>(kp, g.sm_count, s);
}

// supported (support, warps per group): Q = S*S/(32 W) residues per thread
// between 1 and 8
static int win_warps(int S, int requested, int T) {
  int w = requested > 0 ? requested : win_default_warps(S, T);
  switch (S) {
    case 4: return 1;
    case 8: return w >= 2 ? 2 : 1;
    case 16: return w >= 4 ? 4 : (w >= 2 ? 2 : 1);
    case 32: return w >= 8 ? 8 : 4;
  }
  return w;
}

size_t window_smem_bytes(int S, int accum, int vals_f64, int T, int group_warps, int gauss) {
  const int mode = vals_f64 ? 2 : (accum == GG_ACC_COMPENSATED ? 1 : 0);
  const int w = win_warps(S, group_warps, T);
#define GG_WSG(SV, WV, MV)                                                 \
  return gauss ? WinLayout<SV, WV, MV, true>::cta_bytes(T)                 \
               : WinLayout<SV, WV, MV, false>::cta_bytes(T)
#define GG_WS(SV, WV)                                                      \
  do {                                                                     \
    if (mode == 2) GG_WSG(SV, WV, 2);                                      \
    if (mode == 1) GG_WSG(SV, WV, 1);                                      \
    GG_WSG(SV, WV, 0);                                                     \
  } while (0)
  switch (S) {
    case 4: GG_WS(4, 1);
    case 8:
      if (w == 2) GG_WS(8, 2);
      GG_WS(8, 1);
    case 16:
      if (w == 4) GG_WS(16, 4);
      if (w == 2) GG_WS(16, 2);
      GG_WS(16, 1);
    case 32:
      if (w == 8) GG_WS(32, 8);
      GG_WS(32, 4);
  }
#undef GG_WS
#undef GG_WSG
  return 0;
}

__global__ void __launch_bounds__(256)
    gcf_double_rows_kernel(const unsigned char *src, unsigned char *dst, int S, int GG,
                           int elem_bytes, float *dst_real, int *has_imag) {
  const int64_t per = 2ll * S * S, n = (int64_t)GG * per;
  bool imag = false;
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
    const int64_t sk = i / per;
    const int rem = (int)(i % per), b = rem / S, a = rem % S;
    const int64_t j = (sk * S + (b % S)) * S + a;
    if (elem_bytes == 16) {
      reinterpret_cast<double2 *>(dst)[i] = reinterpret_cast<const double2 *>(src)[j];
    } else {
      const float2 v = reinterpret_cast<const float2 *>(src)[j];
      reinterpret_cast<float2 *>(dst)[i] = v;
      if (dst_real) {
        dst_real[i] = v.x;
        imag |= v.y != 0.f;
      }
    }
  }
  if (imag && has_imag) atomicOr(has_imag, 1);
}

cudaError_t launch_gcf_double_rows(const void *src, void *dst, int S, int G, int ntab,
                                   int elem_bytes, cudaStream_t s, float *dst_real,
                                   int *has_imag) {
  const int64_t n = 2ll * ntab * G * G * S * S;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1184);
  gcf_double_rows_kernel<<<blocks, 256, 0, s>>>((const unsigned char *)src, (unsigned char *)dst,
                                                 S, ntab * G * G, elem_bytes,
                                                 elem_bytes == 8 ? dst_real : nullptr, has_imag);
  count_launch();
  return cudaGetLastError();
}

// Self-test of the bounded wait: an mbarrier that expects one arrival which
// never comes.  Every thread waits on it with mbar_wait, gives up after the
// wait limit and raises the timeout flag; no copy is in flight, so nothing is
// left behind.
__global__ void __launch_bounds__(32) selftest_wait_kernel(int *flags) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncwarp();
  mbar_wait(&bar, 0, flags);
}

cudaError_t launch_selftest_wait(int *flags, cudaStream_t s) {
  selftest_wait_kernel<<<1, 32, 0, s>>>(flags);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_window(const GridLaunch &g, cudaStream_t s) {
  KParams kp{};
  kp.jobs = g.jobs;
  kp.items = g.items;
  kp.nitems = g.nitems;
  kp.item_next = g.item_next;
  kp.flags = g.flags;
  kp.holes = g.holes;
  kp.njobs = g.njobs;
  kp.P = g.P;
  kp.T = g.tile;
  kp.G = g.G;
  kp.sigma = g.sigma;
  kp.merge = g.accum == GG_ACC_COMPENSATED && !g.vals_f64 ? g.merge : MergeSlots{};
  const int w = win_warps(g.S, g.group_warps, g.tile);
  switch (g.S) {
    case 4: return win_modes<4, 1>(g, kp, s);
    case 8: return w == 2 ? win_modes<8, 2>(g, kp, s) : win_modes<8, 1>(g, kp, s);
    case 16:
      return w == 4 ? win_modes<16, 4>(g, kp, s)
                    : (w == 2 ? win_modes<16, 2>(g, kp, s) : win_modes<16, 1>(g, kp, s));
    case 32: return w == 8 ? win_modes<32, 8>(g, kp, s) : win_modes<32, 4>(g, kp, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gg
