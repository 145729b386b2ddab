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
// warp never visits the records that miss it.  Warps synchronise only once
// per chunk (before its buffer is refilled).
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

template <typename VT2>
struct GatherShape {
  static constexpr int IDX_BUF = kGatherChunk * 8 + 16;
  static constexpr int VAL_BUF = kGatherChunk * (int)sizeof(VT2) + 16;
  // per-warp lists of record indices (16 bits: a chunk has at most 512)
  static constexpr int LIST_BYTES = (kGatherThreads / 32) * kGatherChunk * 2;
  static constexpr size_t smem(int S) {
    return 16 + 2 * IDX_BUF + 2 * VAL_BUF + LIST_BYTES + 64 * S * 4;
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
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  // double buffers, addressed arithmetically (buffer b at +b*size)
  unsigned char *const idx0 = smem + 16;
  unsigned char *const val0 = smem + 16 + 2 * Sh::IDX_BUF;
  unsigned short *wlist = reinterpret_cast<unsigned short *>(
      smem + 16 + 2 * Sh::IDX_BUF + 2 * Sh::VAL_BUF) + (threadIdx.x >> 5) * K;
  float *g1 = reinterpret_cast<float *>(smem + 16 + 2 * Sh::IDX_BUF + 2 * Sh::VAL_BUF +
                                        Sh::LIST_BYTES);
  __shared__ int s_abort;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  if constexpr (GAUSS) gauss_fill(g1, S, kp.G, kp.sigma, tid, kGatherThreads);
  __syncthreads();
  uint32_t uses0 = 0, uses1 = 0;
  const int P = kp.P;

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
      for (int by = max(ty - 1, 0); by <= min(ty + 1, ntx - 1); ++by)
        for (int bx = max(tx - 1, 0); bx <= min(tx + 1, ntx - 1); ++bx) {
          const int bin = by * ntx + bx;
          const int s_beg = __ldg(J.bookmarks + bin), s_end = __ldg(J.bookmarks + bin + 1);
          const int nchunks = (s_end - s_beg + K - 1) / K;
          auto issue = [&](int c, int b) {
            int s0 = s_beg + c * K, e0 = min(s_end, s0 + K);
            size_t i0 = (size_t)s0 * 8, i1 = (size_t)e0 * 8;
            size_t v0 = (size_t)s0 * sizeof(VT2), v1 = (size_t)e0 * sizeof(VT2);
            uint32_t bytes = (uint32_t)(((i1 + 15) & ~(size_t)15) - (i0 & ~(size_t)15)) +
                             (uint32_t)(((v1 + 15) & ~(size_t)15) - (v0 & ~(size_t)15));
            fence_proxy_async();
            mbar_expect_tx(&bar[b], bytes);
            stage_span((idx0 + b * Sh::IDX_BUF), reinterpret_cast<const char *>(J.idx), i0, i1, &bar[b]);
            stage_span((val0 + b * Sh::VAL_BUF), reinterpret_cast<const char *>(vplane), v0, v1, &bar[b]);
          };
          if (tid == 0 && nchunks > 0) {
            issue(0, 0);
            if (nchunks > 1) issue(1, 1);
          }
          for (int c = 0; c < nchunks; ++c) {
            const int b = c & 1;
            const uint32_t parity = (b == 0 ? uses0 : uses1) & 1;
            if (!mbar_wait(&bar[b], parity, kp.flags)) s_abort = 1;
            if (b == 0) ++uses0; else ++uses1;
            __syncthreads();
            if (s_abort) break;
            const int s0 = s_beg + c * K;
            const int m = min(K, s_end - s0);
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
            __syncthreads();  // buffer b consumed by every warp
            if (tid == 0 && c + 2 < nchunks) issue(c + 2, b);
          }
          if (s_abort) by = ntx;  // leave both bin loops
          if (s_abort) break;
        }
      if (s_abort) break;
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
    if (s_abort) break;
  }
  if (s_abort && tid == 0) {
    mbar_wait(&bar[0], uses0 & 1, nullptr);
    mbar_wait(&bar[1], uses1 & 1, nullptr);
  }
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
