// Index step and uv-tile binning on the device.
//
// Replaces, for the binned methods, the reference's host-side qsort by uv tile
// (comp_grid, grid.cu:256-276, dispatch grid.cu:467-475), vis2ints
// (grid_gpu.cu:352-365) and set_bookmarks (grid_gpu.cu:366-390):
//
//   bin_count    index step per visibility (bit-exact with grid.cu:159-163),
//                packed main*G+sub pair, global uv-tile key, tile histogram
//   scan         exclusive prefix sum of the histogram = bookmarks
//   bin_scatter  places every kept visibility at its sorted position and
//                copies its packed indices and values there (SoA planes), so
//                the gridding kernels stream each tile contiguously
//
// All kernels work on a batch of jobs sharing one global visibility index
// space and one global tile space; a single job is a batch of one.
#include <algorithm>
#include <climits>
#include <cstring>

#include "gg_kernels.cuh"

namespace gg {

__device__ __forceinline__ int find_job64(const int64_t *base, int njobs,
                                          int64_t g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}
// Job of visibility g when the warp's first visibility g0 (<= g) belongs to
// job j0: jobs are contiguous in g, so the search is done once per warp with
// uniform loads and each lane only steps forward past job ends.
__device__ __forceinline__ int job_from(const int64_t *base, int njobs, int j0, int64_t g) {
  int j = j0;
  while (j + 1 < njobs && __ldg(base + j + 1) <= g) ++j;
  return j;
}

__device__ __forceinline__ int find_job32(const int *base, int njobs, int g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Contiguous slice [w0, w1) of the visibilities for this warp (multiples of
// 32 apart), walked 32 at a time: the job of the slice's first visibility is
// found once and then only advanced, where a grid-stride walk would search
// the job table (dependent loads) on every step.
struct WarpSlice {
  int64_t w0, w1;
  __device__ WarpSlice(int64_t total) {
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t per = ((total + nwarps - 1) / nwarps + 31) & ~(int64_t)31;
    w0 = min(total, wid * per);
    w1 = min(total, w0 + per);
  }
};
__device__ __forceinline__ int advance_job(const int64_t *base, int njobs, int j, int64_t g) {
  while (j + 1 < njobs && __ldg(base + j + 1) <= g) ++j;
  return j;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// index step of visibility n of a uv array of either precision
__device__ __forceinline__ bool uv_index(const void *uv, int uv_f64, int64_t n,
                                         int G, int &mx, int &sx, int &my,
                                         int &sy) {
  if (uv_f64) {
    double2 c = __ldg((const double2 *)uv + n);
    bool a = index_step(c.x, G, mx, sx);
    bool b = index_step(c.y, G, my, sy);
    return a && b;
  }
  float2 c = __ldg((const float2 *)uv + n);
  bool a = index_step(c.x, G, mx, sx);
  bool b = index_step(c.y, G, my, sy);
  return a && b;
}

__global__ void __launch_bounds__(256)
    vis2ints_kernel(int uv_f64, const void *uv, int64_t npts, int G,
                    int2 *packed, int *flags) {
  for (int64_t n = blockIdx.x * 256ll + threadIdx.x; n < npts;
       n += (int64_t)gridDim.x * 256) {
    int mx, sx, my, sy;
    if (uv_index(uv, uv_f64, n, G, mx, sx, my, sy)) {
      packed[n] = make_int2(mx * G + sx, my * G + sy);
    } else {
      packed[n] = make_int2(INT_MIN, INT_MIN);
      atomicAdd(&flags[FLAG_INDEX], 1);
    }
  }
}

// Pass 1.  Every visibility of every job: index step, drop rules, tile key,
// warp-aggregated histogram increment.
//  * a visibility whose oversample index falls outside [0,G) would address
//    outside the GCF table in the reference; it is dropped and counted
//  * a visibility whose footprint misses the grid contributes nothing and is
//    dropped silently (the reference skips all of its taps, grid.cu:174-176)
//  * mains left/right of the grid are clamped into the edge tile: all of
//    their on-grid taps still lie inside that tile's window region
__global__ void __launch_bounds__(256) bin_count_kernel(BinBuffers b) {
  const int lane = threadIdx.x & 31;
  const WarpSlice ws(b.total_vis);
  int jw = b.njobs == 1 || ws.w0 >= ws.w1 ? 0 : find_job64(b.vis_base, b.njobs, ws.w0);
  for (int64_t base = ws.w0; base < ws.w1; base += 32) {
    int64_t g = base + lane;
    bool valid = g < ws.w1;
    int key = -1;
    bool bad = false;
    if (b.njobs > 1) jw = advance_job(b.vis_base, b.njobs, jw, base);
    if (valid) {
      int j = b.njobs == 1 ? 0 : job_from(b.vis_base, b.njobs, jw, g);
      const BinJob &J = b.jobs[j];
      int mx, sx, my, sy;
      int2 pk = make_int2(INT_MIN, INT_MIN);
      bool ok = uv_index(J.uv, J.uv_f64, g - J.vis_base, J.G, mx, sx, my, sy);
      if (ok && ((unsigned)sx >= (unsigned)J.G || (unsigned)sy >= (unsigned)J.G))
        ok = false;
      int gi = 0;
      if (ok && J.gcf_index) {
        gi = __ldg(J.gcf_index + (g - J.vis_base));
        if ((unsigned)gi >= (unsigned)J.n_gcf) ok = false;
      }
      bad = !ok;
      if (ok) {
        pk = make_int2(mx * J.G + sx, my * J.G + sy);
        const int h = J.S >> 1;
        if (mx + h >= 0 && mx - h + 1 < J.N && my + h >= 0 && my - h + 1 < J.N) {
          int cx = min(max(mx, 0), J.N - 1) >> J.log2T;
          int cy = min(max(my, 0), J.N - 1) >> J.log2T;
          key = J.tile_base + (cy * J.ntx + cx) * J.n_gcf + gi;
        }
      }
      b.packed[g] = pk;
      b.key[g] = key;
      if (b.kept_pos) b.kept_pos[g] = key >= 0 ? 1 : 0;
    }
    unsigned badm = __ballot_sync(0xffffffffu, bad);
    if (badm && lane == 0) atomicAdd(&b.flags[FLAG_INDEX], __popc(badm));
    unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(peers) - 1)
      atomicAdd(&b.bookmarks[key], __popc(peers));
  }
}

// Pass 3.  Sorted position of every kept visibility; copy of its packed
// indices (and of its values, one plane per polarisation).
//   generic:       position = bookmarks[key] + claim on cursor[key]
//                  (one atomic per run of equal keys within a warp)
//   input_sorted:  position = number of kept visibilities before it, which
//                  keeps input order; a visibility landing outside its own
//                  tile's range proves the input was not tile-sorted
__global__ void __launch_bounds__(256) bin_scatter_kernel(BinBuffers b) {
  const int lane = threadIdx.x & 31;
  const WarpSlice ws(b.total_vis);
  int jw = b.njobs == 1 || ws.w0 >= ws.w1 ? 0 : find_job64(b.vis_base, b.njobs, ws.w0);
  for (int64_t base = ws.w0; base < ws.w1; base += 32) {
    int64_t g = base + lane;
    bool valid = g < ws.w1;
    int key = valid ? b.key[g] : -1;
    // What is copied does not depend on the sorted position: its loads (the
    // packed indices and the first value plane) are issued before the
    // position's atomic, so that their latency overlaps it.
    if (b.njobs > 1) jw = advance_job(b.vis_base, b.njobs, jw, base);
    const BinJob *J = nullptr;
    int64_t n = 0;
    int2 pk = make_int2(0, 0);
    float2 v8 = make_float2(0.f, 0.f);
    double2 v16 = make_double2(0.0, 0.0);
    if (key >= 0) {
      J = b.jobs + (b.njobs == 1 ? 0 : job_from(b.vis_base, b.njobs, jw, g));
      n = g - J->vis_base;
      pk = b.packed[g];
      if (b.vals_bytes == 8) v8 = __ldg((const float2 *)J->vals + n * b.P);
      else v16 = __ldg((const double2 *)J->vals + n * b.P);
    }
    int pos = -1;
    if (b.input_sorted) {
      if (key >= 0) {
        pos = b.kept_pos[g];
        if (pos < b.bookmarks[key] || pos >= b.bookmarks[key + 1]) {
          atomicOr(&b.flags[FLAG_UNSORTED], 1);
          b.bookmarks[b.total_tiles + 1] = 1;  // this call's records have holes
          pos = -1;
        }
      }
    } else {
      unsigned peers = __match_any_sync(0xffffffffu, key);
      int leader = __ffs(peers) - 1;
      int start = 0;
      if (key >= 0 && lane == leader)
        start = atomicAdd(&b.cursor[key], __popc(peers));
      start = __shfl_sync(0xffffffffu, start, leader);
      if (key >= 0) pos = start + __popc(peers & lanemask_lt());
    }
    if (pos >= 0) {
      b.sorted_idx[pos] = b.window_records
                              ? window_record(pk.x >> J->log2G, pk.x & (J->G - 1),
                                              pk.y >> J->log2G, pk.y & (J->G - 1), J->G)
                              : pk;
      if (b.vals_bytes == 8) {
        const float2 *v = (const float2 *)J->vals + n * b.P;
        float2 *o = (float2 *)b.sorted_vals;
        o[pos] = v8;
        for (int p = 1; p < b.P; ++p) o[p * b.vstride + pos] = __ldg(v + p);
      } else {
        const double2 *v = (const double2 *)J->vals + n * b.P;
        double2 *o = (double2 *)b.sorted_vals;
        o[pos] = v16;
        for (int p = 1; p < b.P; ++p) o[p * b.vstride + pos] = __ldg(v + p);
      }
      if (b.order) b.order[pos] = (int)g;
    }
  }
}

// ---- exclusive scan ---------------------------------------------------------
constexpr int kScanThreads = 256, kScanPer = 8,
              kScanBlock = kScanThreads * kScanPer;

__global__ void __launch_bounds__(kScanThreads)
    scan_block_kernel(int *d, int64_t n, int *bsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t base = blockIdx.x * (int64_t)kScanBlock + threadIdx.x * kScanPer;
  int v[kScanPer];
  if (base + kScanPer <= n) {
    int4 a = *reinterpret_cast<const int4 *>(d + base);
    int4 c = *reinterpret_cast<const int4 *>(d + base + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = c.x; v[5] = c.y; v[6] = c.z; v[7] = c.w;
  } else {
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) v[i] = base + i < n ? d[base + i] : 0;
  }
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i) {
    int t = v[i];
    v[i] = s;
    s += t;
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  __shared__ int wsum[kScanThreads / 32];
  __shared__ int total;
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int x = lane < kScanThreads / 32 ? wsum[lane] : 0;
    int xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane < kScanThreads / 32) wsum[lane] = xi - x;
    if (lane == 31) total = xi;
  }
  __syncthreads();
  int off = wsum[warp] + incl - s;
  if (base + kScanPer <= n) {
    int4 a = make_int4(v[0] + off, v[1] + off, v[2] + off, v[3] + off);
    int4 c = make_int4(v[4] + off, v[5] + off, v[6] + off, v[7] + off);
    *reinterpret_cast<int4 *>(d + base) = a;
    *reinterpret_cast<int4 *>(d + base + 4) = c;
  } else {
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
      if (base + i < n) d[base + i] = v[i] + off;
  }
  if (bsum && threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_add_kernel(int *d, int64_t n, const int *boff) {
  int add = boff[blockIdx.x];
  int64_t base = blockIdx.x * (int64_t)kScanBlock;
  for (int i = threadIdx.x; i < kScanBlock; i += kScanThreads)
    if (base + i < n) d[base + i] += add;
}

static int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

size_t scan_tmp_ints(int64_t n) {
  size_t t = 0;
  while (n > kScanBlock) {
    n = cdiv(n, kScanBlock);
    t += (size_t)((n + 7) & ~7ll) + 8;
  }
  return t + 8;
}

cudaError_t scan_exclusive(int *d, int64_t n, int *tmp, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t nb = cdiv(n, kScanBlock);
  scan_block_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(d, n, nb > 1 ? tmp : nullptr);
  count_launch();
  if (nb > 1) {
    cudaError_t e = scan_exclusive(tmp, nb, tmp + ((nb + 7) & ~7ll) + 8, s);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(d, n, tmp);
    count_launch();
  }
  return cudaGetLastError();
}

// ---- driver -----------------------------------------------------------------
static unsigned grid_for(int64_t n) {
  int64_t b = cdiv(n, 256);
  return (unsigned)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

cudaError_t launch_vis2ints(int uv_f64, const void *uv, int64_t npts, int G,
                            int2 *packed, int *flags, cudaStream_t s) {
  if (npts <= 0) return cudaSuccess;
  vis2ints_kernel<<<grid_for(npts), 256, 0, s>>>(uv_f64, uv, npts, G, packed,
                                                 flags);
  count_launch();
  return cudaGetLastError();
}

cudaError_t run_binning(const BinBuffers &b, cudaStream_t s) {
  cudaError_t e;
  e = cudaMemsetAsync(b.bookmarks, 0, sizeof(int) * (size_t)(b.total_tiles + 2), s);
  if (e != cudaSuccess) return e;
  if (b.total_vis > 0) {
    bin_count_kernel<<<grid_for(b.total_vis), 256, 0, s>>>(b);
    count_launch();
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = scan_exclusive(b.bookmarks, b.total_tiles + 1, b.scan_tmp, s)) != cudaSuccess)
    return e;
  if (b.input_sorted) {
    if ((e = scan_exclusive(b.kept_pos, b.total_vis, b.scan_tmp, s)) != cudaSuccess)
      return e;
  } else {
    e = cudaMemcpyAsync(b.cursor, b.bookmarks, sizeof(int) * (size_t)b.total_tiles,
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  if (b.total_vis > 0) {
    bin_scatter_kernel<<<grid_for(b.total_vis), 256, 0, s>>>(b);
    count_launch();
  }
  return cudaGetLastError();
}

// ---- work items ---------------------------------------------------------------

// inclusive warp prefix sum
__device__ __forceinline__ int warp_incl_sum(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  return v;
}

__global__ void __launch_bounds__(256)
    make_items_kernel(const int *bm, const int *tile_base, const int *job_class,
                      int njobs, int total_tiles, ClassChunks chunks, WorkItem *items,
                      int64_t class_cap, int *counters, const JobDesc *jobs, ClassSlots slots,
                      int *heavy_counters, int *flags) {
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * 256 + (threadIdx.x & ~31); base < total_tiles;
       base += gridDim.x * 256) {
    int t = base + lane;
    int k = 0, s0 = 0, e0 = 0, j = 0, cls = 0, chunk = 1;
    if (t < total_tiles) {
      s0 = bm[t];
      e0 = bm[t + 1];
      j = njobs == 1 ? 0 : find_job32(tile_base, njobs, t);
      cls = job_class ? job_class[j] : 0;
      chunk = chunks.c[cls];
      k = (e0 - s0 + chunk - 1) / chunk;
    }
#pragma unroll
    for (int c = 0; c < kMaxClasses; ++c) {
      int kc = (cls == c) ? k : 0;
      int incl = warp_incl_sum(kc, lane);
      int tot = __shfl_sync(0xffffffffu, incl, 31);
      int start = 0;
      if (lane == 0 && tot) start = atomicAdd(&counters[c], tot);
      start = __shfl_sync(0xffffffffu, start, 0);
      // a merge slot for a tile cut into several items (complex64 grids of
      // classes with slots)
      const MergeSlots &ms = slots.m[c];
      int slot = -1;
      if (ms.base != nullptr) {  // uniform over the warp
        const int need = kc > 1 && !jobs[j].out_f64 ? 1 : 0;
        const int hin = warp_incl_sum(need, lane);
        const int htot = __shfl_sync(0xffffffffu, hin, 31);
        int h0 = 0;
        if (lane == 0 && htot) h0 = atomicAdd(&heavy_counters[c], htot);
        h0 = __shfl_sync(0xffffffffu, h0, 0);
        if (need) {
          slot = h0 + hin - 1;
          if (slot >= ms.cap) {
            atomicOr(&flags[FLAG_BOUNDS], 1);
            slot = -1;
          } else {
            ms.desc[slot] = make_int2(j, t - tile_base[j]);
          }
        }
      }
      if (kc) {
        WorkItem *dst = items + c * class_cap + start + (incl - kc);
        int local = t - tile_base[j];
        for (int i = 0; i < kc; ++i) {
          WorkItem w;
          w.job = j;
          w.bin = local;
          w.start = s0 + i * chunk;
          w.end = min(e0, s0 + (i + 1) * chunk);
          w.slot = slot;
          w.pad_[0] = w.pad_[1] = w.pad_[2] = 0;
          dst[i] = w;
        }
      }
    }
  }
}

cudaError_t launch_make_items(const int *bookmarks, const int *tile_base,
                              const int *job_class, int njobs, int total_tiles,
                              ClassChunks chunk, WorkItem *items, int64_t class_cap,
                              int *counters, cudaStream_t s, const JobDesc *jobs,
                              const ClassSlots *slots, int *heavy_counters, int *flags) {
  if (total_tiles <= 0) return cudaSuccess;
  ClassSlots cs{};
  if (slots && jobs && heavy_counters && flags) cs = *slots;
  for (int c = 0; c < kMaxClasses; ++c)
    if (cs.m[c].cap <= 0) cs.m[c].base = nullptr;
  make_items_kernel<<<grid_for(total_tiles), 256, 0, s>>>(
      bookmarks, tile_base, job_class, njobs, total_tiles, chunk, items,
      class_cap, counters, jobs, cs, heavy_counters, flags);
  count_launch();
  return cudaGetLastError();
}

// ---- FP64 merge slots of tiles cut into several work items ---------------------

__global__ void __launch_bounds__(256)
    merge_zero_kernel(double2 *base, int cells, int cap, const int *count) {
  const int64_t n = (int64_t)min(*count, cap) * cells;
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
    base[i] = make_double2(0.0, 0.0);
}

cudaError_t launch_merge_zero(const MergeSlots &m, const int *heavy_counter, int sm_count,
                              cudaStream_t s) {
  if (!m.base || m.cap <= 0) return cudaSuccess;
  merge_zero_kernel<<<sm_count * 4, 256, 0, s>>>(m.base, m.cells, m.cap, heavy_counter);
  count_launch();
  return cudaGetLastError();
}

// one CTA per slot (grid-stride over slots): cells of the slot's R x R
// sub-grid (P planes), origin at the tile's corner minus the halo
__global__ void __launch_bounds__(256)
    merge_finalize_kernel(MergeSlots m, const int *count, const JobDesc *jobs, int S, int T,
                          int P) {
  const int n = min(*count, m.cap);
  const int R = T + S - 1, H = S / 2;
  for (int sl = blockIdx.x; sl < n; sl += gridDim.x) {
    const int2 d = m.desc[sl];
    const JobDesc &J = jobs[d.x];
    const int tile = J.n_gcf > 1 ? d.y / J.n_gcf : d.y;
    const int ox = (tile % J.ntx) * T - H + 1, oy = (tile / J.ntx) * T - H + 1;
    const double2 *src = m.base + (size_t)sl * m.cells;
    for (int i = threadIdx.x; i < P * R * R; i += 256) {
      const double2 v = src[i];
      if (v.x == 0.0 && v.y == 0.0) continue;
      const int p = i / (R * R), c = i - p * R * R;
      const int gx = ox + c % R, gy = oy + c / R;
      if ((unsigned)gx < (unsigned)J.N && (unsigned)gy < (unsigned)J.N)
        out_red(J, (size_t)gy * J.N + gx, p, P, v.x, v.y);
    }
  }
}

cudaError_t launch_merge_finalize(const MergeSlots &m, const int *heavy_counter,
                                  const JobDesc *jobs, int S, int T, int P, int sm_count,
                                  cudaStream_t s) {
  if (!m.base || m.cap <= 0) return cudaSuccess;
  merge_finalize_kernel<<<sm_count * 8, 256, 0, s>>>(m, heavy_counter, jobs, S, T, P);
  count_launch();
  return cudaGetLastError();
}

__global__ void inject_flags_kernel(int *flags, int bits) {
  for (int f = 0; f < 4; ++f)
    if (bits & (1 << f)) atomicOr(&flags[f], 1);
}

cudaError_t launch_inject_flags(int *flags, int bits, cudaStream_t s) {
  inject_flags_kernel<<<1, 1, 0, s>>>(flags, bits);
  count_launch();
  return cudaGetLastError();
}

// ---- table upload through kernel parameters -------------------------------------
// A launch carries its parameters with it (copied by the driver at the call),
// so tables sent this way never wait on a copy engine behind the bulk
// transfers of other streams, and the host buffer is free once the call
// returns.
constexpr int kUploadChunk = 16384;  // bytes per launch (parameters: up to 32 KB)
struct UploadChunk {
  uint4 *dst;
  int n16;  // 16-byte words in this chunk
  uint4 data[kUploadChunk / 16];
};

__global__ void __launch_bounds__(256) upload_kernel(const __grid_constant__ UploadChunk p) {
  for (int i = threadIdx.x; i < p.n16; i += 256) p.dst[i] = p.data[i];
}

cudaError_t launch_upload(void *dst, const void *src, size_t bytes, cudaStream_t s) {
  if (bytes % 16 || (uintptr_t)dst % 16) return cudaErrorInvalidValue;
  static thread_local UploadChunk p;  // 16 KB: off the stack
  for (size_t o = 0; o < bytes; o += kUploadChunk) {
    const size_t n = std::min<size_t>(kUploadChunk, bytes - o);
    p.dst = reinterpret_cast<uint4 *>(static_cast<char *>(dst) + o);
    p.n16 = (int)(n / 16);
    memcpy(p.data, static_cast<const char *>(src) + o, n);
    upload_kernel<<<1, 256, 0, s>>>(p);
    count_launch();
  }
  return cudaGetLastError();
}

// ---- DEBUG1 footprint inputs --------------------------------------------------
__global__ void count_inputs_kernel(void *vals, int vals_f64, int64_t npts,
                                    int P, void *gcf, int64_t gcf_elems) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < npts * P; i += stride) {
    int64_t n = i / P;
    if (vals_f64) ((double2 *)vals)[i] = make_double2(1.0, (double)n);
    else ((float2 *)vals)[i] = make_float2(1.f, (float)n);
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < gcf_elems; i += stride) {
    if (vals_f64) ((double2 *)gcf)[i] = make_double2(1.0, 0.0);
    else ((float2 *)gcf)[i] = make_float2(1.f, 0.f);
  }
}

cudaError_t launch_count_inputs(void *vals, int vals_f64, int64_t npts, int P,
                                void *gcf, int64_t gcf_elems, cudaStream_t s) {
  count_inputs_kernel<<<grid_for(npts * P > gcf_elems ? npts * P : gcf_elems),
                        256, 0, s>>>(vals, vals_f64, npts, P, gcf, gcf_elems);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gg
