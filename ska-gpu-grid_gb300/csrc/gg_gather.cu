// Gather gridding (the reference's GATHER method, grid_kernel_gather,
// grid_gpu.cu:391-503), rebuilt for sm_103a.
//
// One CTA per 32x32-cell output tile; every thread owns 4 cells (one column,
// 4 consecutive rows: warp w owns the row band 4w..4w+3 of the tile) and
// sums, in registers, every tap that lands on them.  The visibilities come
// from the tile's own uv bin and its 8 neighbours (a footprint reaches at
// most S/2 <= 32 cells past its bin): each bin is streamed through shared
// memory by 1-D TMA bulk copies, and every warp compacts, with ballots, the
// records of a chunk whose footprint overlaps its own band into a list of its
// own -- a footprint of S rows reaches about S/4 + 1 of the 8 bands, and a
// warp never visits the records that miss it.  The chunks of a tile's 9 bins
// (and of the CTA's next planes and tiles) form one stream through
// kGatherStages buffers with a full and an empty mbarrier each: a buffer is
// refilled once every warp has released it, so the warps of a tile drift
// apart by a few chunks (track segments give the row bands unequal shares)
// instead of meeting at a barrier after every chunk.
// Each output cell is then written exactly once with a plain store: no
// atomics, no pre-zeroed grid, and a fixed summation order per cell.
#include <type_traits>

#include "gg_kernels.cuh"

namespace gg {

constexpr int kGatherChunk = 512;
// FP32 values: every cell keeps a packed (re, im) register run, added into a
// compensated (hi, lo) pair by TwoSum after at most this many records (a cell
// receives at most one tap per record), so a tap costs one or two packed
// fused multiply-adds instead of a two-sum per component
constexpr int kGatherRun = 32;
constexpr int kGatherTile = 32;
constexpr int kGatherThreads = 256;

// chunk buffers in flight per CTA
constexpr int kGatherStages = 4;

template <typename VT2>
struct GatherShape {
  static constexpr int HEAD = 16 * kGatherStages;  // full and empty mbarriers
  static constexpr int IDX_BUF = kGatherChunk * 8 + 16;
  static constexpr int VAL_BUF = kGatherChunk * (int)sizeof(VT2) + 16;
  // per-warp lists of record indices (16 bits: a chunk has at most 512)
  static constexpr int LIST_BYTES = (kGatherThreads / 32) * kGatherChunk * 2;
  static constexpr size_t smem(int S) {
    return HEAD + kGatherStages * (IDX_BUF + VAL_BUF) + LIST_BYTES + 64 * S * 4;
  }
};

__device__ __forceinline__ int find_job_t(const int *base, int njobs, int g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int S, class ACC, bool GAUSS>
__global__ void __launch_bounds__(kGatherThreads)
    gather_kernel(KParams kp) {
  using VT = typename ACC::VT;
  using VT2 = typename vec2_of<VT>::type;
  using Sh = GatherShape<VT2>;
  constexpr bool F32 = std::is_same<VT, float>::value;
  constexpr bool COMP = std::is_same<ACC, AccComp>::value;
  constexpr int K = kGatherChunk, H = S / 2, TT = kGatherTile;
  // unsorted input declared sorted: holes in this call's sorted records, the
  // call fails with GG_ERR_UNSORTED -- grid nothing
  if (kp.holes && *kp.holes) return;
  extern __shared__ __align__(16) unsigned char smem[];
  // per stage: a "full" barrier (the chunk's bulk copies landed) and an
  // "empty" barrier (every warp is done with the buffer)
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + kGatherStages;
  unsigned char *const idx0 = smem + Sh::HEAD;
  unsigned char *const val0 = smem + Sh::HEAD + kGatherStages * Sh::IDX_BUF;
  unsigned short *wlist = reinterpret_cast<unsigned short *>(
      smem + Sh::HEAD + kGatherStages * (Sh::IDX_BUF + Sh::VAL_BUF)) + (threadIdx.x >> 5) * K;
  float *g1 = reinterpret_cast<float *>(smem + Sh::HEAD + kGatherStages * (Sh::IDX_BUF + Sh::VAL_BUF) +
                                        Sh::LIST_BYTES);
  __shared__ int s_abort;
  // the bins of the current tile (its own and the 8 around it; empty ranges
  // for bins off the grid)
  __shared__ int s_beg[9], s_end[9];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = kGatherThreads / 32;
  if (tid == 0) {
    for (int b = 0; b < kGatherStages; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], NW);
    }
    fence_mbar_init();
    s_abort = 0;
  }
  if constexpr (GAUSS) gauss_fill(g1, S, kp.G, kp.sigma, tid, kGatherThreads);
  __syncthreads();
  const int P = kp.P;
  // One stream of chunks per CTA, through all its tiles and planes: chunk g
  // of the stream uses buffer g % kGatherStages.  Thread 0 issues up to
  // kGatherStages - 1 chunks ahead of its own warp, reusing a buffer once
  // every warp has released it, so the warps of a tile drift apart by up to
  // that many chunks instead of meeting at a barrier after every chunk.
  uint32_t consumed = 0;  // chunks this warp has taken from the stream
  uint32_t issued = 0;    // thread 0: chunks issued

  for (int t = blockIdx.x; t < kp.total_tiles; t += gridDim.x) {
    // tiles of the launch's jobs are numbered from tile_base[0]
    int j = 0, lt = t;
    if (kp.njobs > 1) {
      const int tg = t + __ldg(kp.tile_base);
      j = find_job_t(kp.tile_base, kp.njobs, tg);
      lt = tg - __ldg(kp.tile_base + j);
    }
    const JobDesc &J = kp.jobs[j];
    const int N = J.N, log2G = J.log2G, ntx = J.ntx;
    const int tx = lt % ntx, ty = lt / ntx;
    const int x0 = tx * TT, y0 = ty * TT;
    const int cx = x0 + lane, cy0 = y0 + 4 * warp;
    __syncthreads();  // every warp is done with the previous tile's bin ranges
    // a timed-out wait anywhere ends the CTA's work: read by every thread
    // after the barrier (where it was set before), so all leave together
    if (s_abort) break;
    if (tid < 9) {
      const int by = ty - 1 + tid / 3, bx = tx - 1 + tid % 3;
      int b0 = 0, b1 = 0;
      if (by >= 0 && by < ntx && bx >= 0 && bx < ntx) {
        b0 = __ldg(J.bookmarks + by * ntx + bx);
        b1 = __ldg(J.bookmarks + by * ntx + bx + 1);
      }
      s_beg[tid] = b0;
      s_end[tid] = b1;
    }
    __syncthreads();
    int nch[9], nchunks = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      nch[q] = (s_end[q] - s_beg[q] + K - 1) / K;
      nchunks += nch[q];
    }
    GcfSrc<S, GAUSS, VT> gsrc;
    if constexpr (GAUSS) {
      gsrc.g1 = g1;
    } else {
      gsrc.tab = reinterpret_cast<const VT2 *>(J.gcf);
      gsrc.G = J.G;
    }
    // complex64 table without imaginary parts (flagged on the device when
    // the real parts were copied, rows doubled: [G*G][2S][S]): a tap is one
    // float load and one packed fused multiply-add
    const float *const greal =
        F32 && !GAUSS && J.gcf_real && J.gcf_imag && *J.gcf_imag == 0 ? J.gcf_real : nullptr;
    // chunk c of this (tile, plane): bin q and its first record
    auto chunk_at = [&](int c, int &s0, int &m) {
      int q = 0;
      while (q < 8 && c >= nch[q]) {
        c -= nch[q];
        ++q;
      }
      s0 = s_beg[q] + c * K;
      m = min(K, s_end[q] - s0);
    };
    for (int p = 0; p < P; ++p) {
      const VT2 *vplane = reinterpret_cast<const VT2 *>(J.vals) + (size_t)p * J.vstride;
      ACC acc[4];                          // FP64 values
      u64 run2[4], hi2[4], lo2[4];         // FP32 values: run, compensated pair
      int since = 0;                       // records visited since the last merge
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        acc[k].zero();
        run2[k] = hi2[k] = lo2[k] = 0ull;
      }
      // add the register runs into the (hi, lo) pairs (compensated), or keep
      // them as the sums (plain FP32)
      auto merge_runs = [&]() {
        if constexpr (COMP) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            u64 e;
            hi2[k] = two_sum2(hi2[k], run2[k], e);
            lo2[k] = add2(lo2[k], e);
            run2[k] = 0ull;
          }
        }
        since = 0;
      };
      // thread 0: chunk c of this (tile, plane) into the stream, once every
      // warp has released the buffer it takes
      auto issue = [&](int c) {
        const int b = issued % kGatherStages;
        if (issued >= (uint32_t)kGatherStages &&
            !mbar_wait(&empty[b], (issued / kGatherStages - 1) & 1, kp.flags)) {
          s_abort = 1;
          return false;
        }
        int s0, m;
        chunk_at(c, s0, m);
        const size_t i0 = (size_t)s0 * 8, i1 = (size_t)(s0 + m) * 8;
        const size_t v0 = (size_t)s0 * sizeof(VT2), v1 = (size_t)(s0 + m) * sizeof(VT2);
        const uint32_t bytes = (uint32_t)(((i1 + 15) & ~(size_t)15) - (i0 & ~(size_t)15)) +
                               (uint32_t)(((v1 + 15) & ~(size_t)15) - (v0 & ~(size_t)15));
        fence_proxy_async();
        mbar_expect_tx(&full[b], bytes);
        stage_span(idx0 + b * Sh::IDX_BUF, reinterpret_cast<const char *>(J.idx), i0, i1, &full[b]);
        stage_span(val0 + b * Sh::VAL_BUF, reinterpret_cast<const char *>(vplane), v0, v1, &full[b]);
        ++issued;
        return true;
      };
      int nissued = 0;  // thread 0: chunks of this (tile, plane) issued
      for (int c = 0; c < nchunks; ++c) {
        if (tid == 0)
          while (nissued < nchunks && nissued < c + kGatherStages && !s_abort) {
            if (!issue(nissued)) break;
            ++nissued;
          }
        const int b = consumed % kGatherStages;
        if (!mbar_wait(&full[b], (consumed / kGatherStages) & 1, kp.flags)) s_abort = 1;
        ++consumed;
        if (s_abort) break;
        int s0, m;
        chunk_at(c, s0, m);
        const int2 *ib = reinterpret_cast<const int2 *>((idx0 + b * Sh::IDX_BUF) + (((size_t)s0 * 8) & 15));
        const VT2 *vb = reinterpret_cast<const VT2 *>((val0 + b * Sh::VAL_BUF) + (((size_t)s0 * sizeof(VT2)) & 15));
            // this warp's records: footprint (columns mx-H+1 .. mx+H, rows
            // my-H+1 .. my+H) overlapping the tile's columns and the warp's
            // rows cy0 .. cy0+3, in chunk order
            int base = 0;
            for (int r0 = 0; r0 < m; r0 += 32) {
              const int r = r0 + lane;
              bool keep = false;
              if (r < m) {
                const int2 pk = ib[r];
                const int mx = unpack_main(pk.x, log2G), my = unpack_main(pk.y, log2G);
                keep = (mx + H >= x0) && (mx - H + 1 < x0 + TT) &&
                       (my + H >= cy0) && (my - H + 1 <= cy0 + 3);
              }
              const unsigned bal = __ballot_sync(0xffffffffu, keep);
              if (keep) wlist[base + __popc(bal & ((1u << lane) - 1))] = (unsigned short)r;
              base += __popc(bal);
            }
            __syncwarp();
            for (int q = 0; q < base; ++q) {
              if constexpr (F32) {  // uniform over the warp
                if (++since > kGatherRun) merge_runs();
              }
              const int r = wlist[q];
              const int2 pk = ib[r];
              const int my = unpack_main(pk.y, log2G);
              const int mx = unpack_main(pk.x, log2G), sx = unpack_sub(pk.x, log2G);
              const int sy = unpack_sub(pk.y, log2G);
              const int ap = cx - (mx - H + 1);
              if ((unsigned)ap >= (unsigned)S) continue;
              const VT2 v = vb[r];
              if constexpr (F32 && !GAUSS) {
                if (greal) {  // uniform over the tile
                  const u64 vv = pk2(v.x, v.y);
                  const float *gp = greal + (size_t)(sy * J.G + sx) * (2 * S * S) + ap +
                                    (cy0 - (my - H + 1)) * S;
#pragma unroll
                  for (int k = 0; k < 4; ++k) {
                    const int bp = cy0 + k - (my - H + 1);
                    if ((unsigned)bp < (unsigned)S) {
                      const float g = __ldg(gp + k * S);
                      run2[k] = fma2(vv, pk2(g, g), run2[k]);
                    }
                  }
                  continue;
                }
              }
              if constexpr (F32) {
                const u64 vv = pk2(v.x, v.y), vrr = pk2(v.x, v.x), vsn = pk2(-v.y, v.y);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                  const int bp = cy0 + k - (my - H + 1);
                  if ((unsigned)bp < (unsigned)S) {
                    VT gr, gi;
                    gsrc.value(sx, sy, ap, bp, gr, gi);
                    if constexpr (GAUSS) {
                      run2[k] = fma2(vv, pk2(gr, gr), run2[k]);
                    } else {
                      // (vr gr - vi gi, vr gi + vi gr), two packed roundings
                      run2[k] = fma2(vrr, pk2(gr, gi), fma2(vsn, pk2(gi, gr), run2[k]));
                    }
                  }
                }
              } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                  const int bp = cy0 + k - (my - H + 1);
                  if ((unsigned)bp < (unsigned)S) {
                    VT gr, gi, tr, ti;
                    gsrc.value(sx, sy, ap, bp, gr, gi);
                    if constexpr (GAUSS) {
                      tr = v.x * gr;
                      ti = v.y * gr;
                    } else {
                      cmul<VT>(v.x, v.y, gr, gi, tr, ti);
                    }
                    acc[k].add(tr, ti);
                  }
                }
              }
            }
            __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);  // this warp is done with buffer b
      }
      if (s_abort) break;  // on to the next tile's barrier, where the CTA stops
      if constexpr (F32) merge_runs();
      // each cell written once: plain stores, coalesced along x
      const size_t NN = (size_t)N * N;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int cy = cy0 + k;
        if (cx < N && cy < N) {
          size_t cell = (size_t)cy * N + cx;
          double dre, dim;
          float fre, fim;
          if constexpr (F32) {
            // compensated: hi + lo (exact in FP64, rounded once in FP32);
            // plain: the register run holds the sum
            const float2 h = upk2(COMP ? hi2[k] : run2[k]), l = upk2(lo2[k]);
            dre = (double)h.x + (double)l.x;
            dim = (double)h.y + (double)l.y;
            fre = __fadd_rn(h.x, l.x);
            fim = __fadd_rn(h.y, l.y);
          } else {
            dre = acc[k].dre();
            dim = acc[k].dim();
            fre = acc[k].fre();
            fim = acc[k].fim();
          }
          if (kp.accumulate) {  // into the present value, rounded once
            if (J.out_f64)
              grid_add<double>((double *)J.out, cell, p, P, NN, J.planar, dre, dim);
            else
              grid_add<float>((float *)J.out, cell, p, P, NN, J.planar, dre, dim);
          } else if (J.out_f64) {
            grid_store<double>((double *)J.out, cell, p, P, NN, J.planar, dre, dim);
          } else {
            grid_store<float>((float *)J.out, cell, p, P, NN, J.planar, fre, fim);
          }
        }
      }
    }
  }
  // A timed-out wait may leave bulk copies in flight: thread 0 waits
  // (bounded) for the chunks it issued before the CTA's shared memory goes.
  if (s_abort && tid == 0)
    for (uint32_t g = issued > (uint32_t)kGatherStages ? issued - kGatherStages : 0; g < issued; ++g)
      mbar_wait(&full[g % kGatherStages], (g / kGatherStages) & 1, nullptr);
}

template <int S, class ACC, bool GAUSS>
static cudaError_t gather_launch(const KParams &kp, int sm_count, cudaStream_t s) {
  using VT2 = typename vec2_of<typename ACC::VT>::type;
  size_t smem = GatherShape<VT2>::smem(S);
  auto kern = gather_kernel<S, ACC, GAUSS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGatherThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = sm_count * per_sm;
  if (grid > kp.total_tiles) grid = kp.total_tiles;
  if (grid < 1) return cudaSuccess;
  kern<<<grid, kGatherThreads, smem, s>>>(kp);
  count_launch();
  return cudaGetLastError();
}

template <int S>
static cudaError_t gather_dispatch(const GridLaunch &g, const KParams &kp,
                                   cudaStream_t s) {
  if (g.vals_f64)
    return g.gauss ? gather_launch<S, AccF64, true>(kp, g.sm_count, s)
                   : gather_launch<S, AccF64, false>(kp, g.sm_count, s);
  if (g.accum == GG_ACC_COMPENSATED)
    return g.gauss ? gather_launch<S, AccComp, true>(kp, g.sm_count, s)
                   : gather_launch<S, AccComp, false>(kp, g.sm_count, s);
  return g.gauss ? gather_launch<S, AccF32, true>(kp, g.sm_count, s)
                 : gather_launch<S, AccF32, false>(kp, g.sm_count, s);
}

cudaError_t launch_gather(const GridLaunch &g, cudaStream_t s) {
  if (g.tile != kGatherTile) return cudaErrorInvalidValue;
  KParams kp{};
  kp.jobs = g.jobs;
  kp.flags = g.flags;
  kp.holes = g.holes;
  kp.njobs = g.njobs;
  kp.tile_base = g.tile_base;
  kp.total_tiles = g.total_tiles;
  kp.P = g.P;
  kp.T = g.tile;
  kp.G = g.G;
  kp.sigma = g.sigma;
  kp.accumulate = g.accumulate;
  switch (g.S) {
    case 4: return gather_dispatch<4>(g, kp, s);
    case 8: return gather_dispatch<8>(g, kp, s);
    case 16: return gather_dispatch<16>(g, kp, s);
    case 32: return gather_dispatch<32>(g, kp, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gg
