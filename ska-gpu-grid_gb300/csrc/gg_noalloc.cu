// gg_grid_device_noalloc: the moving-window gridding path with every scratch
// buffer carved from one file-scope __device__ array instead of a context
// workspace, so that a call allocates nothing.
//
// Who needs it: callers that must not allocate device memory once they are
// running -- e.g. a real-time visibility ingest that reserves all of its GPU
// memory at start-up and forbids cudaMalloc in the data path (cudaMalloc can
// block on the device and can fail mid-observation), or a plugin loaded into
// a host framework that owns the device memory pool and does not let plugins
// allocate behind its back.  They pass inputs and outputs; the library
// supplies a fixed scratch area.
//
// Limits: at most kNoAllocMaxVis visibilities, img_dim up to 4096 with the
// default 32-cell tile (kNoAllocMaxTiles uv tiles), one polarisation,
// complex64 values, a GCF table of at most 65536 taps (G*G*S*S).  The array
// (kScratchBytes = 12206336 bytes, 11.6 MiB) is held by every GPU that loads
// this library until the process exits.
//
// Set-up: the first call on a device looks up the device address of the
// array with cudaGetSymbolAddress while that device is current, and caches
// it; make that first call before any stream capture.  All calls share the
// array, which keeps whatever the last call left in it: every call clears
// what must start at zero (histogram, counters, flags, merge slots, the
// output grid), and calls that overlap on the GPU (different streams, or
// different host threads) race on the scratch and corrupt each other's
// results.  The call's small tables travel as kernel parameters, so nothing
// on the stream reads host memory and the host never waits.  Device-side
// failures stay in the array's flag words until the next call:
// gg_read_flags(NULL, ...) reads them.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "gg_internal.h"

namespace gg {
namespace {

constexpr int64_t kNoAllocMaxVis = 1 << 18;
constexpr int kNoAllocMaxTiles = 16384;
constexpr int kNoAllocChunk = 2048;
constexpr int kNoAllocMaxDevices = 64;
constexpr int64_t kClassCap = kNoAllocMaxTiles + kNoAllocMaxVis / kNoAllocChunk + 2;

constexpr size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

// scratch layout (byte offsets)
constexpr size_t kOffJobs = 0;
constexpr size_t kOffBin = kOffJobs + al(sizeof(JobDesc));
constexpr size_t kOffVisBase = kOffBin + al(sizeof(BinJob));
constexpr size_t kOffTileBase = kOffVisBase + al(2 * sizeof(int64_t));
constexpr size_t kOffClass = kOffTileBase + al(2 * sizeof(int));
// flags [0, 8), item counters [8, 12), item claims [12, 16), merge slots
// taken [16, 20)
constexpr int kFlagInts = 32;
constexpr size_t kOffFlags = kOffClass + al(sizeof(int));
constexpr size_t kOffPacked = kOffFlags + al(kFlagInts * sizeof(int));
constexpr size_t kOffKey = kOffPacked + al(sizeof(int2) * (kNoAllocMaxVis + 1));
constexpr size_t kOffBm = kOffKey + al(sizeof(int) * (kNoAllocMaxVis + 1));
constexpr size_t kOffCursor = kOffBm + al(sizeof(int) * (kNoAllocMaxTiles + 8));
constexpr size_t kOffScan = kOffCursor + al(sizeof(int) * (kNoAllocMaxTiles + 8));
// scan scratch for up to max(tiles, vis)+1 entries: 2048-entry blocks
constexpr size_t kScanInts = (kNoAllocMaxVis + 1) / 2048 + 64;
constexpr size_t kOffKept = kOffScan + al(sizeof(int) * kScanInts);
constexpr size_t kOffSidx = kOffKept + al(sizeof(int) * (kNoAllocMaxVis + 8));
constexpr size_t kOffSvals = kOffSidx + al(sizeof(int2) * (kNoAllocMaxVis + 8));
constexpr size_t kOffItems = kOffSvals + al(sizeof(float2) * (kNoAllocMaxVis + 8) + 64);
// row-doubled copy of the GCF table read by the window kernel: up to
// kNoAllocMaxGcf sub-kernel taps (G*G*S*S), complex64
constexpr int64_t kNoAllocMaxGcf = 1 << 16;
constexpr size_t kOffGcf = kOffItems + al(sizeof(WorkItem) * kClassCap);  // one class
// FP64 merge slots of tiles cut into several work items (compensated
// accumulation into complex64 grids): a fixed area, divided into as many
// slots of the call's sub-grid size as fit; the records per work item grow
// when needed so that no more tiles than that are ever cut
constexpr size_t kMergeBytes = size_t(2) << 20;
constexpr int kMergeMaxSlots = 1024;
constexpr size_t kOffMerge = kOffGcf + al(sizeof(float2) * 2 * kNoAllocMaxGcf);
constexpr size_t kOffMergeDesc = kOffMerge + al(kMergeBytes);
constexpr size_t kScratchBytes = kOffMergeDesc + al(sizeof(int2) * kMergeMaxSlots);

// the size the header and the documentation state
static_assert(kScratchBytes == 12206336, "update the stated size of the allocation-free array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_ptr[kNoAllocMaxDevices];

int setup_scratch(char **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return GG_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return GG_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return GG_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = (char *)g_scratch_ptr[dev];
  return GG_OK;
}

int ilog2i(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

int noalloc_fail(int code, const char *m) { return set_error(code, m); }

// The call's device tables (job, binning job, bases, class) are kernel
// parameters written into the scratch by one thread, which also clears the
// flag and counter words: no host memory is read by the copy engine, so the
// call does not wait for earlier work on the stream.
__global__ void noalloc_setup_kernel(JobDesc D, BinJob B, int64_t n, int ntiles, char *ws) {
  *reinterpret_cast<JobDesc *>(ws + kOffJobs) = D;
  *reinterpret_cast<BinJob *>(ws + kOffBin) = B;
  int64_t *vb = reinterpret_cast<int64_t *>(ws + kOffVisBase);
  vb[0] = 0;
  vb[1] = n;
  int *tb = reinterpret_cast<int *>(ws + kOffTileBase);
  tb[0] = 0;
  tb[1] = ntiles;
  *reinterpret_cast<int *>(ws + kOffClass) = 0;
  int *flags = reinterpret_cast<int *>(ws + kOffFlags);
  for (int i = 0; i < kFlagInts; ++i) flags[i] = 0;
}

}  // namespace

// flags of the last allocation-free call on the current device (gg_read_flags
// with a null context): copied to the host after `stream` completes
int noalloc_read_flags(void *stream, int32_t out[4]) {
  char *ws = nullptr;
  if (int st = setup_scratch(&ws)) return noalloc_fail(st, "noalloc: cudaGetSymbolAddress failed");
  cudaStream_t s = (cudaStream_t)stream;
  int32_t h[4];
  if (cudaMemcpyAsync(h, ws + kOffFlags, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return noalloc_fail(GG_ERR_CUDA, "noalloc: reading the flags failed");
  for (int i = 0; i < 4; ++i) out[i] = h[i];
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" int gg_grid_device_noalloc(const gg_options *opt, const gg_job *job,
                                      void *stream) {
  if (!opt || !job) return noalloc_fail(GG_ERR_ARG, "noalloc: null argument");
  const int mode = opt->mode == GG_MODE_AUTO ? GG_MODE_WINDOW : opt->mode;
  if (mode != GG_MODE_WINDOW)
    return noalloc_fail(GG_ERR_ARG, "noalloc: only the moving-window method");
  if (opt->polarizations != 1)
    return noalloc_fail(GG_ERR_ARG, "noalloc: one polarisation only");
  if (opt->gcf_kind != GG_GCF_TABLE && opt->gcf_kind != GG_GCF_GAUSSIAN)
    return noalloc_fail(GG_ERR_ARG, "noalloc: GCF must be TABLE or GAUSSIAN");
  const int G = opt->oversample, T = opt->tile > 0 ? opt->tile : 32;
  if (G < 1 || G > 64 || (G & (G - 1)) || T < 16 || T > 256 || (T & (T - 1)))
    return noalloc_fail(GG_ERR_ARG, "noalloc: oversample / tile not a power of two in range");
  if (job->vals_type != GG_C64)
    return noalloc_fail(GG_ERR_ARG, "noalloc: complex64 values only");
  if ((job->uv_type != GG_C64 && job->uv_type != GG_C128) ||
      (job->out_type != GG_C64 && job->out_type != GG_C128))
    return noalloc_fail(GG_ERR_ARG, "noalloc: bad uv_type / out_type");
  const int64_t S = job->gcf_dim, N = job->img_dim, n = job->npts;
  if (S != 4 && S != 8 && S != 16 && S != 32)
    return noalloc_fail(GG_ERR_ARG, "noalloc: gcf_dim not in {4,8,16,32}");
  if (n < 0 || n > kNoAllocMaxVis)
    return noalloc_fail(GG_ERR_ARG,
                        "noalloc: npts exceeds the fixed scratch (max 262144 visibilities)");
  const int64_t ntx = (N + T - 1) / T;
  if (N < 1 || ntx * ntx > kNoAllocMaxTiles)
    return noalloc_fail(GG_ERR_ARG,
                        "noalloc: img_dim exceeds the fixed scratch (max 16384 uv tiles, "
                        "i.e. 4096 at tile 32)");
  if (job->gcf_index)
    return noalloc_fail(GG_ERR_ARG, "noalloc: per-visibility GCF tables are not supported");
  if (opt->gcf_kind == GG_GCF_TABLE && (int64_t)G * G * S * S > kNoAllocMaxGcf)
    return noalloc_fail(GG_ERR_ARG,
                        "noalloc: GCF table exceeds the fixed scratch (G*G*S*S at most 65536, "
                        "e.g. oversample 8 with support 32)");
  if (!job->out || (n > 0 && (!job->uv || !job->vals)) ||
      (opt->gcf_kind == GG_GCF_TABLE && !job->gcf))
    return noalloc_fail(GG_ERR_ARG, "noalloc: null buffer");

  // merge slots (compensated accumulation into a complex64 grid): as many as
  // the fixed area holds at this sub-grid size; records per item raised so
  // that fewer tiles than that are cut into several items
  int chunk = kNoAllocChunk, merge_cap = 0, merge_cells = 0;
  if (opt->accum == GG_ACC_COMPENSATED && job->out_type == GG_C64) {
    const int64_t R = T + S - 1;
    merge_cells = (int)(R * R);
    const int64_t fit = std::min<int64_t>(kMergeMaxSlots,
                                          (int64_t)(kMergeBytes / (sizeof(double2) * R * R)));
    if (fit < 2)
      return noalloc_fail(GG_ERR_ARG, "noalloc: tile + support too large for the merge area");
    // a tile of more than `chunk` records takes a slot: at most n/(chunk+1)
    const int64_t need = (n + fit - 2) / (fit - 1);
    chunk = (int)std::max<int64_t>(kNoAllocChunk, need);
    merge_cap = (int)fit;
  }

  char *ws = nullptr;
  int st = setup_scratch(&ws);
  if (st) return noalloc_fail(st, "noalloc: cudaGetSymbolAddress failed");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return noalloc_fail(GG_ERR_CUDA, "noalloc: device");
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return noalloc_fail(GG_ERR_CUDA, "noalloc: device attribute");

  // device tables, built on the host and copied into the scratch
  JobDesc D;
  std::memset(&D, 0, sizeof D);
  D.out = job->out;
  D.uv = job->uv;
  D.gcf = opt->gcf_kind == GG_GCF_TABLE ? (const void *)(ws + kOffGcf) : nullptr;
  D.idx = (const int2 *)(ws + kOffSidx);
  D.vals = ws + kOffSvals;
  D.bookmarks = (const int *)(ws + kOffBm);
  D.npts = n;
  D.vstride = kNoAllocMaxVis + 8;
  D.N = (int)N;
  D.S = (int)S;
  D.G = G;
  D.log2G = ilog2i(G);
  D.P = 1;
  D.T = T;
  D.log2T = ilog2i(T);
  D.ntx = (int)ntx;
  D.planar = opt->layout == GG_LAYOUT_PLANAR || opt->layout == GG_LAYOUT_REFERENCE;
  D.out_f64 = job->out_type == GG_C128;
  D.uv_f64 = job->uv_type == GG_C128;
  const double sg = job->gcf_sigma > 0 ? job->gcf_sigma
                                       : (opt->gcf_sigma > 0 ? opt->gcf_sigma : S / 4.0);
  D.sigma = (float)sg;
  D.n_gcf = 1;
  BinJob B;
  std::memset(&B, 0, sizeof B);
  B.uv = job->uv;
  B.vals = job->vals;
  B.vis_base = 0;
  B.npts = n;
  B.tile_base = 0;
  B.ntiles = (int)(ntx * ntx);
  B.n_gcf = 1;
  B.N = (int)N;
  B.S = (int)S;
  B.G = G;
  B.log2G = D.log2G;
  B.log2T = D.log2T;
  B.ntx = (int)ntx;
  B.P = 1;
  B.uv_f64 = D.uv_f64;
#define GG_NA(call)                                                        \
  do {                                                                     \
    if ((call) != cudaSuccess) return noalloc_fail(GG_ERR_CUDA, "noalloc: " #call); \
  } while (0)
  noalloc_setup_kernel<<<1, 1, 0, s>>>(D, B, n, (int)(ntx * ntx), ws);
  count_launch();
  GG_NA(cudaGetLastError());
  int *flags = (int *)(ws + kOffFlags);
  const size_t out_bytes = (size_t)(D.out_f64 ? 16 : 8) * N * N;
  if (!opt->accumulate) GG_NA(cudaMemsetAsync(job->out, 0, out_bytes, s));

  if (opt->gcf_kind == GG_GCF_TABLE)
    GG_NA(launch_gcf_double_rows(job->gcf, ws + kOffGcf, (int)S, G, 1, 8, s));

  BinBuffers b{};
  b.jobs = (const BinJob *)(ws + kOffBin);
  b.vis_base = (const int64_t *)(ws + kOffVisBase);
  b.tile_base = (const int *)(ws + kOffTileBase);
  b.njobs = 1;
  b.total_vis = n;
  b.total_tiles = (int)(ntx * ntx);
  b.vals_bytes = 8;
  b.P = 1;
  b.packed = (int2 *)(ws + kOffPacked);
  b.key = (int *)(ws + kOffKey);
  b.bookmarks = (int *)(ws + kOffBm);
  b.cursor = (int *)(ws + kOffCursor);
  b.scan_tmp = (int *)(ws + kOffScan);
  b.sorted_idx = (int2 *)(ws + kOffSidx);
  b.sorted_vals = ws + kOffSvals;
  b.vstride = kNoAllocMaxVis + 8;
  b.order = nullptr;
  b.flags = flags;
  b.input_sorted = opt->input_sorted ? 1 : 0;
  b.window_records = 1;
  b.kept_pos = b.input_sorted ? (int *)(ws + kOffKept) : nullptr;
  GG_NA(run_binning(b, s));

  WorkItem *items = (WorkItem *)(ws + kOffItems);
  ClassChunks chunks = {{chunk, chunk, chunk, chunk}};
  ClassSlots slots{};
  if (merge_cap > 0) {
    slots.m[0].base = (double2 *)(ws + kOffMerge);
    slots.m[0].desc = (int2 *)(ws + kOffMergeDesc);
    slots.m[0].cap = merge_cap;
    slots.m[0].cells = merge_cells;
  }
  GG_NA(launch_make_items(b.bookmarks, b.tile_base, (const int *)(ws + kOffClass), 1,
                          b.total_tiles, chunks, items, kClassCap, flags + 8, s,
                          (const JobDesc *)(ws + kOffJobs), &slots, flags + 16, flags));
  GG_NA(launch_merge_zero(slots.m[0], flags + 16, sms, s));
  GridLaunch g{};
  g.jobs = (const JobDesc *)(ws + kOffJobs);
  g.njobs = 1;
  g.S = (int)S;
  g.accum = opt->accum;
  g.vals_f64 = 0;
  g.gauss = opt->gcf_kind == GG_GCF_GAUSSIAN;
  g.sigma = (float)sg;
  g.G = G;
  g.tile = T;
  g.P = 1;
  g.flags = flags;
  g.holes = b.bookmarks + b.total_tiles + 1;
  g.sm_count = sms;
  g.items = items;
  g.nitems = flags + 8;
  g.item_next = flags + 12;
  g.max_items = kClassCap;
  g.merge = slots.m[0];
  GG_NA(launch_window(g, s));
  GG_NA(launch_merge_finalize(slots.m[0], flags + 16, (const JobDesc *)(ws + kOffJobs), (int)S, T,
                              1, sms, s));
  if (const int bits = injected_device_flags()) GG_NA(launch_inject_flags(flags, bits, s));
#undef GG_NA
  return GG_OK;
}
