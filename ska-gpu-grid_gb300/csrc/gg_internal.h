// Host-side launcher interfaces between the C ABI (gg_api.cu) and the
// kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gg_types.h"

namespace gg {

// process-wide count of kernel launches made by the library
void count_launch(int n = 1);
// records msg as the calling thread's gg_last_error() and returns code
int set_error(int code, const char *msg);

// One job of a binning pass.  Visibilities of all jobs of a batch live in one
// global index space: job j owns global indices [vis_base, vis_base+npts) and
// global uv tiles [tile_base, tile_base+ntiles).
struct BinJob {
  const void *uv;
  const void *vals;
  const int *gcf_index;  // per-visibility table index, or null
  int64_t vis_base;
  int64_t npts;
  int tile_base, ntiles;  // ntiles = ntx * ntx * n_gcf bins
  int N, S, G, log2G, log2T, ntx, P;
  int uv_f64;
  int n_gcf;
};

struct BinBuffers {
  const BinJob *jobs;      // device [njobs]
  const int64_t *vis_base; // device [njobs+1]
  const int *tile_base;    // device [njobs+1]
  int njobs;
  int64_t total_vis;       // sum of npts
  int total_tiles;         // sum of ntiles
  int vals_bytes;          // 8 (complex64) or 16 (complex128)
  int P;                   // polarisations (uniform over the batch)
  int2 *packed;            // [total_vis]
  int *key;                // [total_vis] global tile id or -1 (dropped)
  int *bookmarks;          // [total_tiles+1]: counts, then exclusive offsets;
                           // [total_tiles+1]: set when input declared sorted
                           // is not (records left unwritten)
  int *cursor;             // [total_tiles]
  int *scan_tmp;           // scratch for the multi-level scan
  int2 *sorted_idx;        // [total_vis + pad]
  void *sorted_vals;       // [P][vstride]
  int64_t vstride;
  int *order;              // [total_vis] or null
  int *flags;
  int input_sorted;
  int *kept_pos;           // [total_vis+1] (input_sorted only)
  // sorted record format: 0 = packed (main*G+sub) pairs (gather, gg_bin);
  // 1 = moving window: {main cells (my+64)<<16 | (mx+64), sub-kernel
  //     sy*G+sx} -- see window_record()
  int window_records;
};

// Sorted record of the moving-window kernel: both main cells in one word
// (offset by 64 so that clamped mains stay positive; 16 bits each hold
// img_dim up to 32768 plus the support) and the sub-kernel index.
constexpr int kWinMainBias = 64;
__host__ __device__ inline int2 window_record(int mx, int sx, int my, int sy, int G) {
  return make_int2((int)(((unsigned)(my + kWinMainBias) << 16) | (unsigned)(mx + kWinMainBias)),
                   sy * G + sx);
}

// index step only (vis2ints)
cudaError_t launch_vis2ints(int uv_f64, const void *uv, int64_t npts, int G,
                            int2 *packed, int *flags, cudaStream_t s);
// count, scan, scatter; leaves bookmarks = exclusive offsets [total_tiles+1]
cudaError_t run_binning(const BinBuffers &b, cudaStream_t s);
// exclusive scan of n ints in place; tmp needs scan_tmp_ints(n) ints
size_t scan_tmp_ints(int64_t n);
cudaError_t scan_exclusive(int *data, int64_t n, int *tmp, cudaStream_t s);

// Work items for the moving-window kernel: every non-empty tile of job j
// (global tiles tile_base..) is cut into slices of at most `chunk` sorted
// visibilities.  Items of jobs of S-class c go to items + c*class_cap,
// counted in counters[c].
// records per work item of each support class (index: class of the job)
constexpr int kMaxClasses = 4;
struct ClassChunks {
  int c[kMaxClasses];
};
// Merge slots per support class (cap 0 or base null: none).  A tile of a job
// with a complex64 grid that is cut into more than one item gets slot
// heavy_counters[c]++ of its class: every one of its items carries the slot,
// and desc[slot] = {job, tile-local bin}.  A slot index beyond the class's
// cap (the host sizes cap so that this cannot happen) raises FLAG_BOUNDS and
// leaves the tile on the plain reduction.
struct ClassSlots {
  MergeSlots m[kMaxClasses];
};
cudaError_t launch_make_items(const int *bookmarks, const int *tile_base,
                              const int *job_class, int njobs, int total_tiles,
                              ClassChunks chunk, WorkItem *items, int64_t class_cap,
                              int *counters, cudaStream_t s,
                              const JobDesc *jobs = nullptr, const ClassSlots *slots = nullptr,
                              int *heavy_counters = nullptr, int *flags = nullptr);
// Number of merge slots a class needs at most: tiles with more than `chunk`
// records, at most vis / (chunk + 1) of them.
inline int merge_slot_cap(int64_t vis, int chunk, int64_t tiles) {
  int64_t c = vis / ((int64_t)chunk + 1) + 1;
  if (c > tiles) c = tiles;
  return (int)c;
}
// Clears the slots a class took (heavy_counter on the device) before its
// window kernel adds into them.
cudaError_t launch_merge_zero(const MergeSlots &m, const int *heavy_counter, int sm_count,
                              cudaStream_t s);
// Rounds every slot of the class once into its job's grid (after the
// class's window kernel): cell values that are nonzero are reduced into the
// output with the grid's layout, cells outside the grid skipped.
cudaError_t launch_merge_finalize(const MergeSlots &m, const int *heavy_counter,
                                  const JobDesc *jobs, int S, int T, int P, int sm_count,
                                  cudaStream_t s);
// ORs `bits` (1 << FLAG_*) into flags[FLAG_*] on the stream: the host-side
// injection behind gg_debug_inject_device_flags.
cudaError_t launch_inject_flags(int *flags, int bits, cudaStream_t s);
// Copies `bytes` (a multiple of 16, dst 16-byte aligned) from host memory to
// dst on the stream through kernel parameters, 16 KB per launch: nothing
// waits on a copy engine, and src may be rewritten once the call returns.
cudaError_t launch_upload(void *dst, const void *src, size_t bytes, cudaStream_t s);
// flags of a context (device int32[64], see gg_read_flags)
int *context_flags(gg_context *c);
// Makes the batched calls of a context use `flags` (device int32[64], the
// caller zeroes words 0..7) instead of its own flag words, until reset with
// null: the request server gives every batch in flight its own words, read
// back after the batch's output copies while the slot runs its next batch.
void context_set_batch_flags(gg_context *c, int *flags);
// consumes one pending injection of gg_debug_inject_device_flags: returns
// its bits (0: none pending)
int injected_device_flags();
// gg_read_flags without a context: flags of the last allocation-free call on
// the current device (gg_noalloc.cu); synchronises the stream
int noalloc_read_flags(void *stream, int32_t out[4]);

// ---- gridding launches ----------------------------------------------------
struct GridLaunch {
  const JobDesc *jobs;     // device [njobs]
  int njobs;
  int S;                   // support of every job in this launch
  int accum;               // GG_ACC_*
  int vals_f64;
  int gauss;
  int wphase;              // scatter: the reference's COMPUTE_GCF factor
  float sigma;             // GAUSS: uniform over the launch
  int G;                   // oversampling, uniform over the launch
  int tile;                // uv tile side, uniform over the launch
  int group_warps;         // moving window: warps per sub-grid (0: by support)
  int accumulate;          // gather: add into the grid instead of storing
  int P;
  int *flags;
  const int *holes;        // binned methods: bookmarks[total_tiles + 1]
  int sm_count;
  // scatter: global visibility space
  const int64_t *vis_base; // device [njobs+1]
  int64_t total_vis;
  // window: work queue
  const WorkItem *items;
  const int *nitems;
  int *item_next;
  int64_t max_items;
  MergeSlots merge;        // the class's FP64 merge slots (base null: none)
  // gather: global tiles of the jobs in this launch
  const int *tile_base;    // device [njobs+1]
  int total_tiles;
};

// Degridding (adjoint of the gridder): one launch per job
struct DegridLaunch {
  const void *grid;        // device: P planes of N*N complex (grid_f64: double)
  void *vals;              // device: npts*P complex out (vals_f64: double)
  const void *uv;          // device: npts (u,v) pairs (uv_f64: double)
  const void *gcf;         // device: n_gcf tables [G*G][S][S] of the values' type; null: Gaussian
  const int *gcf_index;    // device, optional: table of each visibility
  int64_t npts;
  int N, S, G, P, n_gcf;
  int uv_f64, grid_f64, vals_f64;
  int planar;              // grid layout: planar (1) or interleaved (0)
  int gauss;               // GCF computed on the fly (separable Gaussian)
  int compensated;         // FP32 values: two-sum (hi, lo) lane sums
  float sigma;
  int *flags;
  int sm_count;
};
cudaError_t launch_degrid(const DegridLaunch &d, cudaStream_t s);
// centred inverse 2-D FFT of P interleaved planes in place (cuFFT, loaded at
// first use); 0 on success, else a message in err.  Synchronises s.
int image_inverse_fft(void *grid, int64_t N, int P, bool f64, int sm_count, cudaStream_t s,
                      std::string &err);

cudaError_t launch_scatter(const GridLaunch &g, cudaStream_t s);
cudaError_t launch_window(const GridLaunch &g, cudaStream_t s);
// one warp waiting on an mbarrier nobody completes (bounded-wait self-test)
cudaError_t launch_selftest_wait(int *flags, cudaStream_t s);
// test hook: the next n device allocations of the library fail (NOMEM);
// returns true (and consumes one) when the current allocation must fail
bool injected_alloc_failure();
// Row-doubled copy of ntab consecutive [G*G][S][S] GCF tables for the
// moving-window kernel: dst[s][b][a] = src[s][b mod S][a] for b < 2S, s over
// all ntab*G*G sub-kernels (elem_bytes 8 or 16).  With dst_real (complex64
// tables only) the real parts are written there too, and *has_imag (zeroed
// by the caller) is set when any imaginary part is nonzero.
cudaError_t launch_gcf_double_rows(const void *src, void *dst, int S, int G, int ntab,
                                   int elem_bytes, cudaStream_t s,
                                   float *dst_real = nullptr, int *has_imag = nullptr);
inline size_t gcf_double_rows_bytes(int S, int G, int elem_bytes) {
  return (size_t)elem_bytes * G * G * 2 * S * S;
}
cudaError_t launch_gather(const GridLaunch &g, cudaStream_t s);
// compensated scatter with complex64 output: out = fl(hi + lo)
cudaError_t launch_comp_finalize(float *out, const float *lo, int64_t n,
                                 cudaStream_t s);
// substitute inputs of the DEBUG1 footprint mode: vals[n*P+p] = (1, n),
// gcf = (1, 0) everywhere
cudaError_t launch_count_inputs(void *vals, int vals_f64, int64_t npts, int P,
                                void *gcf, int64_t gcf_elems, cudaStream_t s);
// smem bytes the window kernel needs (for occupancy sizing)
size_t window_smem_bytes(int S, int accum, int vals_f64, int T, int group_warps, int gauss);

}  // namespace gg
