// C ABI of the gridder (include/gg.h): contexts, plans, drop-in entry points.
//
// The reference's gridGPU (grid_gpu.cu:675-819) pins the caller's buffers,
// allocates and frees device memory on every call, zeroes the padded grid,
// launches one compile-time-selected method and copies the whole padded grid
// back, printing (not returning) any CUDA error.  Here a context owns every
// device buffer (grown on demand, reused across calls), a plan turns a batch
// of jobs into device tables once, and executing a plan only enqueues
// kernels and memsets on the caller's stream, so it can be captured into a
// CUDA graph.  Errors come back as status codes with a message.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gg_internal.h"

namespace gg {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int set_error(int code, const char *msg) {
  g_last_error = msg ? msg : "";
  return code;
}

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
static int cuda_fail(cudaError_t e, const char *what) {
  return fail(e == cudaErrorMemoryAllocation ? GG_ERR_NOMEM : GG_ERR_CUDA,
              "%s: %s", what, cudaGetErrorString(e));
}
#define GG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

static bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }
static int ilog2(int64_t v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}
static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// ---------------------------------------------------------------------------
// device buffer that only grows
// ---------------------------------------------------------------------------
static std::atomic<int> g_fail_allocs{0};
bool injected_alloc_failure() {
  int k = g_fail_allocs.load();
  while (k > 0)
    if (g_fail_allocs.compare_exchange_weak(k, k - 1)) return true;
  return false;
}

// gg_debug_inject_device_flags: flag bits and how many more served batches /
// allocation-free calls receive them
static std::mutex g_inject_mu;
static int g_inject_bits = 0, g_inject_count = 0;
int injected_device_flags() {
  std::lock_guard<std::mutex> lk(g_inject_mu);
  if (g_inject_count <= 0) return 0;
  --g_inject_count;
  return g_inject_bits;
}

struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  int ensure(size_t bytes) {
    if (bytes <= n) return GG_OK;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (injected_alloc_failure())
      return fail(GG_ERR_NOMEM, "cudaMalloc(workspace): injected allocation failure");
    size_t want = align256(bytes + bytes / 8);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMalloc(workspace)");
    }
    n = want;
    return GG_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};
struct HostBuf {
  void *p = nullptr;
  size_t n = 0;
  int ensure(size_t bytes) {
    if (bytes <= n) return GG_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    size_t want = align256(bytes + bytes / 8 + 4096);
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMallocHost(staging)");
    }
    n = want;
    return GG_OK;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace gg

using namespace gg;

// ---------------------------------------------------------------------------
// options
// ---------------------------------------------------------------------------
static gg_options default_opts() {
  gg_options o;
  memset(&o, 0, sizeof o);
  o.mode = GG_MODE_SCATTER;
  o.layout = GG_LAYOUT_REFERENCE;
  o.accum = GG_ACC_PLAIN;
  o.gcf_kind = GG_GCF_TABLE;
  o.oversample = 8;
  o.polarizations = 1;
  o.tile = 0;
  o.input_sorted = 0;
  o.gcf_sigma = 0.0;
  o.window_chunk = 0;
  return o;
}

static std::mutex g_opt_mu;
static gg_options g_global_opts = default_opts();

static int check_options(const gg_options *o) {
  if (!o) return fail(GG_ERR_ARG, "options: null");
  if (o->mode < GG_MODE_SCATTER || o->mode > GG_MODE_AUTO)
    return fail(GG_ERR_ARG, "options: mode %d unknown", o->mode);
  if (o->layout < GG_LAYOUT_INTERLEAVED || o->layout > GG_LAYOUT_REFERENCE)
    return fail(GG_ERR_ARG, "options: layout %d unknown", o->layout);
  if (o->accum != GG_ACC_PLAIN && o->accum != GG_ACC_COMPENSATED)
    return fail(GG_ERR_ARG, "options: accum %d unknown", o->accum);
  if (o->gcf_kind < GG_GCF_TABLE || o->gcf_kind > GG_GCF_WPHASE)
    return fail(GG_ERR_ARG, "options: gcf_kind %d unknown", o->gcf_kind);
  if (!is_pow2(o->oversample) || o->oversample > 64)
    return fail(GG_ERR_ARG, "options: oversample %d must be a power of two <= 64",
                o->oversample);
  if (o->polarizations < 1 || o->polarizations > kMaxPols)
    return fail(GG_ERR_ARG, "options: polarizations %d outside 1..%d",
                o->polarizations, kMaxPols);
  if (o->tile != 0 && (!is_pow2(o->tile) || o->tile < 8 || o->tile > 256))
    return fail(GG_ERR_ARG, "options: tile %d must be 0 or a power of two in 8..256",
                o->tile);
  if (o->window_chunk < 0) return fail(GG_ERR_ARG, "options: window_chunk < 0");
  if (o->group_warps != 0 && o->group_warps != 1 && o->group_warps != 2 &&
      o->group_warps != 4 && o->group_warps != 8)
    return fail(GG_ERR_ARG, "options: group_warps %d not in {0,1,2,4,8}", o->group_warps);
  if (o->autotune < 0 || o->autotune > 2)
    return fail(GG_ERR_ARG, "options: autotune %d not in {0,1,2}", o->autotune);
  if (o->accumulate != 0 && o->accumulate != 1)
    return fail(GG_ERR_ARG, "options: accumulate %d not in {0,1}", o->accumulate);
  return GG_OK;
}

// ---------------------------------------------------------------------------
// context and plan
// ---------------------------------------------------------------------------
struct Plan {
  // resolved launch configuration
  int mode = GG_MODE_WINDOW;
  int accum = GG_ACC_PLAIN;
  int vals_f64 = 0;
  int gauss = 0;
  float sigma = 0.f;
  int G = 8, P = 1, T = 32, chunk = 2048, group_warps = 0;
  int njobs = 0;
  int64_t total_vis = 0;
  int total_tiles = 0;
  int input_sorted = 0;
  int comp_lo = 0;  // compensated scatter with complex64 output
  struct ClassRange {
    int S, j0, j1;
    int64_t v0, v1;  // global vis range
    int t0, t1;      // global tile range
    int T, W, chunk; // tile, warps per sub-grid group (0: by support), records per item
  };
  std::vector<ClassRange> classes;
  std::vector<JobDesc> hjobs;
  std::vector<BinJob> hbin;
  std::vector<int64_t> hvis_base;
  std::vector<int> htile_base, hclass;
  std::vector<std::pair<void *, size_t>> zero_ranges;  // outputs to clear
  std::vector<std::pair<float *, int64_t>> finalize;   // (out, floats) comp scatter
  std::vector<std::pair<void *, int64_t>> count_fill;  // (vals, npts) DEBUG1
  // row-doubled GCF tables read by the moving-window kernel: source (null:
  // the DEBUG1 count table), workspace offset, support; per job (class
  // order) the offset of its copy, or SIZE_MAX
  struct GcfCopy {
    const void *src;
    size_t off;
    int S;
    int ntab;         // consecutive tables (per-visibility selection)
    size_t off_real;  // real parts (complex64 tables; 0: none)
  };
  size_t o_gcf_flags = 0;  // one int per copy: nonzero when a table has imaginary parts
  std::vector<size_t> hgcf_copy;  // per job (class order): index of its copy
  std::vector<GcfCopy> gcf_copies;
  std::vector<size_t> hgcf_off;
  // FP64 merge slots per support class (compensated FP32 moving window into
  // complex64 grids): offsets of the slots and their descriptors, slots and
  // double2 values per slot (0 slots: none)
  size_t o_merge[kMaxClasses] = {}, o_mdesc[kMaxClasses] = {};
  int merge_cap[kMaxClasses] = {}, merge_cells[kMaxClasses] = {};
  // workspace carve (offsets into the device workspace)
  size_t o_jobs, o_bin, o_visb, o_tileb, o_class, o_packed, o_key, o_bm,
      o_cursor, o_scan, o_sidx, o_svals, o_order, o_items, o_kept, o_lo,
      o_count_vals, o_count_gcf, ws_bytes;
  int64_t vstride = 0, class_cap = 0;
  size_t table_bytes = 0;  // bytes uploaded from staging (jobs..class)
  char *ws = nullptr;      // workspace the addresses are bound to
};

// Side stream of a moving-window launch: the output grids are zeroed there
// while the binning and the earlier support classes run on the main stream
// (the window kernels are issue bound and leave HBM nearly idle); each class
// waits only for the zeroing of its own grids.
struct AuxStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t done[kMaxClasses] = {};
  int init() {
    GG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    GG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (auto &e : done) GG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return GG_OK;
  }
  void release() {
    for (auto &e : done)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (s) cudaStreamDestroy(s);
    s = nullptr;
    fork = nullptr;
  }
};

struct gg_context {
  int device = 0;
  int sm_count = 152;
  std::mutex mu;
  DevBuf ws;        // plan workspace
  DevBuf flags;     // int32[16]: flags[0..7], item counters [8..11], item_next [12..15]
  int *batch_flags = nullptr;  // set by the server: the flag words of its batch
  HostBuf staging;  // pinned: device tables are uploaded from here
  cudaEvent_t upload_done = nullptr;  // staging may be rewritten after this
  cudaEvent_t exec_done = nullptr;    // workspace free after this
  cudaStream_t own = nullptr;         // stream of the host-path calls
  AuxStream aux;                      // zeroing beside moving-window launches
  // host-path device copies of the caller's buffers
  DevBuf h_uv, h_vals, h_gcf, h_out;
  Plan plan;
  // profiling: events around set-up+binning, gridding kernels, whole call
  int profile = 0;
  int prof_recorded = 0;
  cudaEvent_t prof[4] = {nullptr, nullptr, nullptr, nullptr};
};

int *gg::context_flags(gg_context *c) {
  return c->batch_flags ? c->batch_flags : (int *)c->flags.p;
}
void gg::context_set_batch_flags(gg_context *c, int *flags) { c->batch_flags = flags; }

static int ctx_init(gg_context *c, int device) {
  c->device = device;
  GG_CUDA(cudaSetDevice(device));
  int sms = 0;
  GG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  c->sm_count = sms;
  GG_CUDA(cudaEventCreateWithFlags(&c->upload_done, cudaEventDisableTiming));
  GG_CUDA(cudaEventCreateWithFlags(&c->exec_done, cudaEventDisableTiming));
  GG_CUDA(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
  if (int st = c->aux.init()) return st;
  for (auto &e : c->prof) GG_CUDA(cudaEventCreate(&e));
  int st = c->flags.ensure(64 * sizeof(int));
  if (st) return st;
  GG_CUDA(cudaMemset(c->flags.p, 0, 64 * sizeof(int)));
  return GG_OK;
}

static void ctx_release(gg_context *c) {
  cudaSetDevice(c->device);
  if (c->exec_done) cudaEventSynchronize(c->exec_done);
  c->ws.release();
  c->flags.release();
  c->h_uv.release();
  c->h_vals.release();
  c->h_gcf.release();
  c->h_out.release();
  c->staging.release();
  if (c->upload_done) cudaEventDestroy(c->upload_done);
  if (c->exec_done) cudaEventDestroy(c->exec_done);
  for (auto &e : c->prof)
    if (e) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  c->aux.release();
}

// GG_MODE_AUTO: the moving window for FP32 values (fastest at every size
// class measured: 1.5x scatter on the 4096^2 track workload, more on
// batches); the scatter for FP64 values, whose FP64 register arithmetic in
// the window kernel is slower on this GPU than FP64 L2 reductions (1024^2,
// S=16: 399 vs 218 Mvis/s)
static int resolve_mode(const gg_options *o, int S, int vals_f64) {
  // the COMPUTE_GCF phase factor is the reference scatter kernel's: scatter
  if (o->gcf_kind == GG_GCF_WPHASE) return GG_MODE_SCATTER;
  if (o->mode != GG_MODE_AUTO) return o->mode;
  (void)S;
  return vals_f64 ? GG_MODE_SCATTER : GG_MODE_WINDOW;
}

// Launch configuration of one support class of the moving window
struct ClassCfg {
  int T = 0, W = 0, chunk = 0;
};
using ClassCfgs = std::map<int, ClassCfg>;  // by support

// Autotuner cache: the configuration picked for a size class, keyed by
// support, arithmetic, polarisations, oversampling and the class's density
// (visibilities per 256 grid cells, as a power of two)
struct TuneKey {
  int S, accum, vals_f64, gauss, P, G, density;
  bool operator<(const TuneKey &o) const {
    return std::tie(S, accum, vals_f64, gauss, P, G, density) <
           std::tie(o.S, o.accum, o.vals_f64, o.gauss, o.P, o.G, o.density);
  }
};
struct TuneEntry {
  ClassCfg cfg;
  double ms_best = 0, ms_default = 0;
  int trials = 0;
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tune;

static bool tunable(const gg_options *o) {
  return o->tile == 0 && o->group_warps == 0 && o->window_chunk == 0;
}

// density class of the jobs of support S in a batch
static int density_class(const gg_job *jobs, int njobs, int S) {
  double vis = 0, area = 0;
  for (int j = 0; j < njobs; ++j)
    if (jobs[j].gcf_dim == S) {
      vis += (double)jobs[j].npts;
      area += (double)jobs[j].img_dim * (double)jobs[j].img_dim;
    }
  const double d = area > 0 ? vis * 256.0 / area : 0.0;
  int b = 0;
  while (b < 24 && d >= (double)(2ll << b)) ++b;
  return b;
}

static TuneKey tune_key(const gg_options *o, int vals_f64, int S, int density) {
  return {S, vals_f64 ? GG_ACC_PLAIN : o->accum, vals_f64, o->gcf_kind == GG_GCF_GAUSSIAN,
          o->polarizations, o->oversample, density};
}

// classes smaller than this are not timed when a choice for the same support
// and arithmetic exists (their trials are short and noisy); they take the
// choice of the nearest density instead
constexpr double kTuneMinVis = 1 << 23;

// the cached entry of `k`, or of the nearest density with the same other
// fields; null when there is none (caller holds g_tune_mu)
static const TuneEntry *tune_lookup(const TuneKey &k) {
  auto it = g_tune.find(k);
  if (it != g_tune.end()) return &it->second;
  const TuneEntry *best = nullptr;
  int dist = 1 << 30;
  for (const auto &kv : g_tune) {
    const TuneKey &o = kv.first;
    if (o.S != k.S || o.accum != k.accum || o.vals_f64 != k.vals_f64 || o.gauss != k.gauss ||
        o.P != k.P || o.G != k.G)
      continue;
    const int d = std::abs(o.density - k.density);
    if (d < dist) {
      dist = d;
      best = &kv.second;
    }
  }
  return best;
}

// Build the plan for a batch: validate, resolve, order jobs by support class,
// lay out the workspace.  No device work.  `force` fixes the configuration of
// support classes (autotuner trials).
static int plan_build(gg_context *c, const gg_options *opt, const gg_job *jobs,
                      int njobs, Plan &pl, const ClassCfgs *force = nullptr) {
  int st = check_options(opt);
  if (st) return st;
  if (njobs < 1) return fail(GG_ERR_ARG, "no jobs");
  if (!jobs) return fail(GG_ERR_ARG, "jobs: null");
  pl = Plan();
  pl.G = opt->oversample;
  pl.P = opt->polarizations;
  // per support class: tile, warps per sub-grid group, records per work item
  ClassCfgs cfgs;
  {
    int64_t maxS = 0;
    for (int j = 0; j < njobs; ++j) maxS = std::max<int64_t>(maxS, jobs[j].gcf_dim);
    const int m0 = resolve_mode(opt, (int)maxS, jobs[0].vals_type == GG_C128);
    const int vf64 = jobs[0].vals_type == GG_C128;
    for (int j = 0; j < njobs; ++j) {
      const int S = (int)jobs[j].gcf_dim;
      if (cfgs.count(S)) continue;
      // automatic tile: the moving window keeps one (T+S-1)^2 sub-grid per
      // warp group, so supports up to 16 use 8-cell tiles (small sub-grids,
      // many resident groups: measured fastest on every track workload);
      // gather needs 32; input declared tile-sorted: the caller's tiles are
      // the default 32
      ClassCfg cf;
      cf.T = opt->tile > 0 ? opt->tile
                           : (m0 == GG_MODE_WINDOW && S <= 16 && !opt->input_sorted ? 8 : 32);
      cf.W = opt->group_warps;
      cf.chunk = opt->window_chunk > 0 ? opt->window_chunk : 2048;
      if (m0 == GG_MODE_WINDOW && tunable(opt)) {
        if (force && force->count(S)) {
          cf = force->at(S);
        } else if (opt->autotune) {
          std::lock_guard<std::mutex> lk(g_tune_mu);
          const TuneEntry *e = tune_lookup(tune_key(opt, vf64, S, density_class(jobs, njobs, S)));
          if (e) cf = e->cfg;
        }
      }
      cfgs[S] = cf;
    }
    pl.T = cfgs.begin()->second.T;
    pl.chunk = cfgs.begin()->second.chunk;
    for (auto &kv : cfgs) pl.chunk = std::min(pl.chunk, kv.second.chunk);
    pl.group_warps = opt->group_warps;
  }
  pl.input_sorted = opt->input_sorted ? 1 : 0;
  pl.gauss = opt->gcf_kind == GG_GCF_GAUSSIAN;
  pl.accum = opt->accum;
  pl.njobs = njobs;
  const int vt = jobs[0].vals_type;
  if (vt != GG_C64 && vt != GG_C128) return fail(GG_ERR_ARG, "job 0: vals_type %d", vt);
  pl.vals_f64 = vt == GG_C128;
  const size_t vbytes = pl.vals_f64 ? 16 : 8;
  int mode = -1;
  double sigma = -1.0;
  // stable order by support
  std::vector<int> order(njobs);
  for (int j = 0; j < njobs; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return jobs[a].gcf_dim < jobs[b].gcf_dim;
  });
  int64_t vis = 0;
  int64_t tiles = 0;
  for (int k = 0; k < njobs; ++k) {
    const gg_job &J = jobs[order[k]];
    const int j = order[k];
    if (J.vals_type != vt)
      return fail(GG_ERR_ARG, "job %d: all jobs of a batch need the same vals_type", j);
    if (J.uv_type != GG_C64 && J.uv_type != GG_C128)
      return fail(GG_ERR_ARG, "job %d: uv_type %d", j, J.uv_type);
    if (J.out_type != GG_C64 && J.out_type != GG_C128)
      return fail(GG_ERR_ARG, "job %d: out_type %d", j, J.out_type);
    if (pl.vals_f64 && J.out_type != GG_C128)
      return fail(GG_ERR_ARG,
                  "job %d: complex128 values need a complex128 grid (the reference "
                  "instantiates gridGPU<double2,double2> only)", j);
    if (J.gcf_dim != 4 && J.gcf_dim != 8 && J.gcf_dim != 16 && J.gcf_dim != 32)
      return fail(GG_ERR_ARG, "job %d: gcf_dim %lld not in {4,8,16,32}", j,
                  (long long)J.gcf_dim);
    if (J.img_dim < 1 || J.img_dim > 32768)
      return fail(GG_ERR_ARG, "job %d: img_dim %lld outside 1..32768", j,
                  (long long)J.img_dim);
    if (J.npts < 0) return fail(GG_ERR_ARG, "job %d: npts < 0", j);
    if (!J.out) return fail(GG_ERR_ARG, "job %d: out is null", j);
    if (J.npts > 0 && (!J.uv || !J.vals))
      return fail(GG_ERR_ARG, "job %d: uv/vals null", j);
    if ((opt->gcf_kind == GG_GCF_TABLE || opt->gcf_kind == GG_GCF_WPHASE) && !J.gcf)
      return fail(GG_ERR_ARG, "job %d: TABLE and WPHASE GCFs need gcf", j);
    if (J.gcf_index) {
      if (opt->gcf_kind != GG_GCF_TABLE)
        return fail(GG_ERR_ARG, "job %d: gcf_index needs a TABLE GCF", j);
      if (J.n_gcf < 1 || J.n_gcf > 32768)
        return fail(GG_ERR_ARG, "job %d: n_gcf %lld outside 1..32768", j, (long long)J.n_gcf);
      if (opt->input_sorted)
        return fail(GG_ERR_ARG, "job %d: gcf_index with input_sorted is not supported", j);
    }
    const int m = resolve_mode(opt, (int)J.gcf_dim, J.vals_type == GG_C128);
    if (mode < 0) mode = m;
    if (m != mode) return fail(GG_ERR_ARG, "job %d: mixed methods in one batch", j);
    double sg = J.gcf_sigma > 0 ? J.gcf_sigma
                                : (opt->gcf_sigma > 0 ? opt->gcf_sigma : J.gcf_dim / 4.0);
    if (pl.gauss) {
      if (sigma < 0) sigma = sg;
      if (sg != sigma)
        return fail(GG_ERR_ARG, "job %d: on-the-fly GCF needs one sigma per batch", j);
      if (J.gcf_dim != jobs[order[0]].gcf_dim)
        return fail(GG_ERR_ARG, "on-the-fly GCF needs one support per batch");
    }
    const int T = cfgs[(int)J.gcf_dim].T;
    if (mode == GG_MODE_GATHER && T != 32)
      return fail(GG_ERR_ARG, "gather needs tile 32");
    if (mode == GG_MODE_GATHER && J.gcf_index)
      return fail(GG_ERR_ARG, "job %d: gcf_index: use the scatter or moving-window method", j);
    vis += J.npts;
    int ntx = (int)((J.img_dim + T - 1) / T);
    tiles += (int64_t)ntx * ntx * (J.gcf_index ? J.n_gcf : 1);
  }
  if (vis >= (1ll << 31) - 1024) return fail(GG_ERR_ARG, "batch has >= 2^31 visibilities");
  if (tiles >= (1ll << 30)) return fail(GG_ERR_ARG, "batch has too many uv tiles");
  pl.mode = mode;
  if (mode == GG_MODE_WINDOW) {
    for (int j = 0; j < njobs; ++j) {
      const ClassCfg &cf = cfgs[(int)jobs[j].gcf_dim];
      const size_t need = window_smem_bytes((int)jobs[j].gcf_dim, opt->accum, vt == GG_C128,
                                            cf.T, cf.W, opt->gcf_kind == GG_GCF_GAUSSIAN);
      if (need > 227 * 1024)
        return fail(GG_ERR_ARG,
                    "tile %d with support %lld needs %zu bytes of shared memory "
                    "(max 232448): use a smaller tile",
                    cf.T, (long long)jobs[j].gcf_dim, need);
    }
  }
  pl.sigma = (float)(sigma > 0 ? sigma : 0.0);
  pl.total_vis = vis;
  pl.total_tiles = (int)tiles;
  if (pl.vals_f64) pl.accum = GG_ACC_PLAIN;  // FP64 values: FP64 arithmetic
  const bool binned = mode != GG_MODE_SCATTER;

  // workspace layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  pl.o_jobs = take(sizeof(JobDesc) * njobs);
  pl.o_bin = take(sizeof(BinJob) * njobs);
  pl.o_visb = take(sizeof(int64_t) * (njobs + 1));
  pl.o_tileb = take(sizeof(int) * (njobs + 1));
  pl.o_class = take(sizeof(int) * njobs);
  pl.table_bytes = off;
  pl.vstride = vis + 8;
  pl.class_cap = tiles + vis / pl.chunk + njobs + 1;
  if (binned) {
    pl.o_packed = take(sizeof(int2) * (vis + 1));
    pl.o_key = take(sizeof(int) * (vis + 1));
    pl.o_bm = take(sizeof(int) * (tiles + 8));
    pl.o_cursor = take(sizeof(int) * (tiles + 8));
    pl.o_scan = take(sizeof(int) * scan_tmp_ints(std::max<int64_t>(tiles + 1, vis + 1)));
    pl.o_sidx = take(sizeof(int2) * (vis + 8));
    pl.o_svals = take(vbytes * pl.P * pl.vstride + 64);
    pl.o_order = 0;
    pl.o_kept = pl.input_sorted ? take(sizeof(int) * (vis + 8)) : 0;
    pl.o_items = mode == GG_MODE_WINDOW ? take(sizeof(WorkItem) * 4 * pl.class_cap) : 0;
  }
  const bool count = opt->gcf_kind == GG_GCF_COUNT;
  pl.o_count_vals = count ? take(vbytes * pl.P * (vis + 1)) : 0;
  int maxS = 0;
  for (int j = 0; j < njobs; ++j) maxS = std::max<int>(maxS, (int)jobs[j].gcf_dim);
  pl.o_count_gcf = count ? take(vbytes * pl.G * pl.G * maxS * maxS) : 0;
  pl.comp_lo = mode == GG_MODE_SCATTER && pl.accum == GG_ACC_COMPENSATED && !pl.vals_f64;
  size_t lo_total = 0;
  if (pl.comp_lo)
    for (int j = 0; j < njobs; ++j)
      if (jobs[j].out_type == GG_C64)
        lo_total += align256(8 * (size_t)pl.P * jobs[j].img_dim * jobs[j].img_dim);
  pl.o_lo = pl.comp_lo ? take(lo_total) : 0;
  pl.gcf_copies.clear();
  pl.hgcf_off.assign(njobs, SIZE_MAX);
  pl.hgcf_copy.assign(njobs, SIZE_MAX);
  // row-doubled copies of the tables (moving window), and for complex64
  // tables their real parts with a "has an imaginary part" flag (moving
  // window and gather take a real-factor path when it is clear)
  if ((mode == GG_MODE_WINDOW || (mode == GG_MODE_GATHER && !pl.vals_f64)) && !pl.gauss) {
    std::map<std::tuple<const void *, int, int>, size_t> seen;  // -> copy index
    for (int k = 0; k < njobs; ++k) {
      const gg_job &J = jobs[order[k]];
      const int ntab = J.gcf_index ? (int)J.n_gcf : 1;
      const std::tuple<const void *, int, int> key(count ? nullptr : J.gcf, (int)J.gcf_dim, ntab);
      auto it = seen.find(key);
      if (it == seen.end()) {
        const size_t o = take(gcf_double_rows_bytes((int)J.gcf_dim, pl.G, (int)vbytes) * ntab);
        // complex64 tables: also their real parts, for the real-factor path
        const size_t o_real =
            vbytes == 8 ? take(gcf_double_rows_bytes((int)J.gcf_dim, pl.G, 4) * ntab) : 0;
        it = seen.emplace(key, pl.gcf_copies.size()).first;
        pl.gcf_copies.push_back({std::get<0>(key), o, (int)J.gcf_dim, ntab, o_real});
      }
      pl.hgcf_copy[k] = it->second;
      pl.hgcf_off[k] = pl.gcf_copies[it->second].off;
    }
    pl.o_gcf_flags = take(sizeof(int) * (pl.gcf_copies.size() + 1));
  }
  // merge slots: classes in ascending support, like cfgs
  if (mode == GG_MODE_WINDOW && pl.accum == GG_ACC_COMPENSATED && !pl.vals_f64) {
    int ci = 0;
    for (const auto &kv : cfgs) {
      const int S = kv.first;
      int64_t cvis = 0, ctiles = 0;
      bool c64 = false;
      for (int j = 0; j < njobs; ++j)
        if (jobs[j].gcf_dim == S) {
          cvis += jobs[j].npts;
          const int64_t ntx = (jobs[j].img_dim + kv.second.T - 1) / kv.second.T;
          ctiles += ntx * ntx * (jobs[j].gcf_index ? jobs[j].n_gcf : 1);
          c64 |= jobs[j].out_type == GG_C64;
        }
      if (c64 && ci < kMaxClasses) {
        const int R = kv.second.T + S - 1;
        pl.merge_cap[ci] = merge_slot_cap(cvis, kv.second.chunk, ctiles);
        pl.merge_cells[ci] = pl.P * R * R;
        pl.o_merge[ci] = take(sizeof(double2) * (size_t)pl.merge_cap[ci] * pl.merge_cells[ci]);
        pl.o_mdesc[ci] = take(sizeof(int2) * (size_t)pl.merge_cap[ci]);
      }
      ++ci;
    }
  }
  pl.ws_bytes = off;

  // host tables in class order
  pl.hjobs.resize(njobs);
  pl.hbin.resize(njobs);
  pl.hvis_base.resize(njobs + 1);
  pl.htile_base.resize(njobs + 1);
  pl.hclass.resize(njobs);
  int64_t vb = 0;
  int tb = 0;
  size_t lo_off = 0;
  int64_t cnt_off = 0;
  for (int k = 0; k < njobs; ++k) {
    const gg_job &J = jobs[order[k]];
    const int S = (int)J.gcf_dim;
    if (pl.classes.empty() || pl.classes.back().S != S) {
      if (!pl.classes.empty()) {
        pl.classes.back().j1 = k;
        pl.classes.back().v1 = vb;
        pl.classes.back().t1 = tb;
      }
      const ClassCfg &cf = cfgs[S];
      pl.classes.push_back({S, k, k, vb, vb, tb, tb, cf.T, cf.W, cf.chunk});
    }
    const int T = pl.classes.back().T;
    const int N = (int)J.img_dim;
    const int ntx = (N + T - 1) / T;
    JobDesc &D = pl.hjobs[k];
    memset(&D, 0, sizeof D);
    D.out = J.out;
    D.uv = J.uv;
    D.vals = J.vals;
    D.gcf = J.gcf;
    D.npts = J.npts;
    D.vstride = pl.vstride;
    D.N = N;
    D.S = S;
    D.G = pl.G;
    D.log2G = ilog2(pl.G);
    D.P = pl.P;
    D.T = T;
    D.log2T = ilog2(T);
    D.ntx = ntx;
    int layout = opt->layout;
    if (layout == GG_LAYOUT_REFERENCE)
      layout = mode == GG_MODE_WINDOW ? GG_LAYOUT_PLANAR : GG_LAYOUT_INTERLEAVED;
    D.planar = layout == GG_LAYOUT_PLANAR;
    D.out_f64 = J.out_type == GG_C128;
    D.uv_f64 = J.uv_type == GG_C128;
    D.sigma = pl.sigma;
    D.gcf_index = J.gcf_index;
    D.n_gcf = J.gcf_index ? (int)J.n_gcf : 1;
    BinJob &B = pl.hbin[k];
    memset(&B, 0, sizeof B);
    B.uv = J.uv;
    B.vals = J.vals;
    B.vis_base = vb;
    B.npts = J.npts;
    B.tile_base = tb;
    B.ntiles = ntx * ntx * D.n_gcf;
    B.gcf_index = J.gcf_index;
    B.n_gcf = D.n_gcf;
    B.N = N;
    B.S = S;
    B.G = pl.G;
    B.log2G = D.log2G;
    B.log2T = D.log2T;
    B.ntx = ntx;
    B.P = pl.P;
    B.uv_f64 = D.uv_f64;
    pl.hvis_base[k] = vb;
    pl.htile_base[k] = tb;
    pl.hclass[k] = (int)pl.classes.size() - 1;
    const size_t out_bytes = (size_t)(D.out_f64 ? 16 : 8) * pl.P * N * N;
    // the binned scatter-type kernels add into the grid: cleared first unless
    // the caller accumulates into it (gather stores, or adds, every cell)
    if (mode != GG_MODE_GATHER && !opt->accumulate) pl.zero_ranges.push_back({J.out, out_bytes});
    if (pl.comp_lo && J.out_type == GG_C64) {
      // filled in once the workspace base is known (plan_bind)
      D.lo = reinterpret_cast<float *>(lo_off + 1);
      pl.finalize.push_back({(float *)J.out, (int64_t)2 * pl.P * N * N});
      lo_off += align256(out_bytes);
    }
    if (count) {
      pl.count_fill.push_back({reinterpret_cast<void *>(cnt_off), J.npts});
      cnt_off += J.npts * pl.P;
    }
    vb += J.npts;
    tb += ntx * ntx * D.n_gcf;
  }
  pl.classes.back().j1 = njobs;
  pl.classes.back().v1 = vb;
  pl.classes.back().t1 = tb;
  pl.hvis_base[njobs] = vb;
  pl.htile_base[njobs] = tb;
  return GG_OK;
}

// Fix device addresses for a workspace at `ws`; write the device tables
// (jobs, bin jobs, bases, classes) into `host` (pl.table_bytes bytes).
static void plan_bind(const gg_options *opt, Plan &pl, char *ws, char *host) {
  const bool binned = pl.mode != GG_MODE_SCATTER;
  const size_t vbytes = pl.vals_f64 ? 16 : 8;
  for (int k = 0; k < pl.njobs; ++k) {
    JobDesc &D = pl.hjobs[k];
    if (pl.comp_lo && D.lo) D.lo = (float *)(ws + pl.o_lo + ((size_t)D.lo - 1));
    if (opt->gcf_kind == GG_GCF_COUNT) {
      void *cv = ws + pl.o_count_vals +
                 vbytes * (size_t)reinterpret_cast<intptr_t>(pl.count_fill[k].first);
      D.vals = cv;
      pl.hbin[k].vals = cv;
      D.gcf = ws + pl.o_count_gcf;
    }
    if (pl.hgcf_off[k] != SIZE_MAX) {
      const auto &c = pl.gcf_copies[pl.hgcf_copy[k]];
      // the gather kernel reads the caller's [G*G][S][S] table (and the real
      // parts of the copy); the moving window reads the row-doubled copy
      if (pl.mode == GG_MODE_WINDOW) D.gcf = ws + c.off;
      D.gcf_real = c.off_real ? (const float *)(ws + c.off_real) : nullptr;
      D.gcf_imag = c.off_real ? (const int *)(ws + pl.o_gcf_flags) + pl.hgcf_copy[k] : nullptr;
    }
    if (binned) {
      D.idx = (const int2 *)(ws + pl.o_sidx);
      D.vals = ws + pl.o_svals;
      D.bookmarks = (const int *)(ws + pl.o_bm) + pl.htile_base[k];
    }
  }
  // count-mode fills: resolve to absolute addresses
  for (auto &f : pl.count_fill)
    f.first = ws + pl.o_count_vals + vbytes * (size_t)reinterpret_cast<intptr_t>(f.first);
  memcpy(host + pl.o_jobs, pl.hjobs.data(), sizeof(JobDesc) * pl.njobs);
  memcpy(host + pl.o_bin, pl.hbin.data(), sizeof(BinJob) * pl.njobs);
  memcpy(host + pl.o_visb, pl.hvis_base.data(), sizeof(int64_t) * (pl.njobs + 1));
  memcpy(host + pl.o_tileb, pl.htile_base.data(), sizeof(int) * (pl.njobs + 1));
  memcpy(host + pl.o_class, pl.hclass.data(), sizeof(int) * pl.njobs);
  pl.ws = ws;
}

// Profiling events of one enqueue (null: none)
struct ProfEvents {
  cudaEvent_t ev[4];
};

// Enqueue the whole computation on stream s: zeroing, binning, work queue,
// gridding kernels.  `upload` (host tables) is sent into the workspace first
// when given, through kernel parameters (launch_upload): a copy-engine
// transfer would queue behind other streams' input and output copies (one
// to two milliseconds per batch on a server moving host data), a launch does
// not, and the staging buffer is free again when the call returns
// (`upload_ev` is still recorded after it); a plan whose tables are already
// resident passes null, and then nothing here reads host memory, allocates
// or synchronises -- the sequence can be captured into a CUDA graph.
static int plan_enqueue(const gg_options *opt, const Plan &pl, int *flags, int sm_count,
                        cudaStream_t s, const void *upload, cudaEvent_t upload_ev,
                        const ProfEvents *prof, const AuxStream *aux) {
  char *ws = pl.ws;
  if (prof) GG_CUDA(cudaEventRecord(prof->ev[0], s));
  if (upload) {
    GG_CUDA(launch_upload(ws, upload, pl.table_bytes, s));
    if (upload_ev) GG_CUDA(cudaEventRecord(upload_ev, s));
  }
  const JobDesc *djobs = (const JobDesc *)(ws + pl.o_jobs);
  const int64_t *dvisb = (const int64_t *)(ws + pl.o_visb);
  const int *dtileb = (const int *)(ws + pl.o_tileb);
  const int *dclass = (const int *)(ws + pl.o_class);
  const size_t vbytes = pl.vals_f64 ? 16 : 8;

  // output zeroing: on the side stream, class by class, for the moving
  // window (jobs are in class order, one zero range each); else here
  const bool side = aux && aux->s && pl.mode == GG_MODE_WINDOW &&
                    pl.zero_ranges.size() == (size_t)pl.njobs &&
                    pl.classes.size() <= (size_t)kMaxClasses;
  if (side) {
    GG_CUDA(cudaEventRecord(aux->fork, s));
    GG_CUDA(cudaStreamWaitEvent(aux->s, aux->fork, 0));
    for (size_t ci = 0; ci < pl.classes.size(); ++ci) {
      for (int j = pl.classes[ci].j0; j < pl.classes[ci].j1; ++j)
        GG_CUDA(cudaMemsetAsync(pl.zero_ranges[j].first, 0, pl.zero_ranges[j].second, aux->s));
      GG_CUDA(cudaEventRecord(aux->done[ci], aux->s));
    }
  } else {
    for (auto &z : pl.zero_ranges) GG_CUDA(cudaMemsetAsync(z.first, 0, z.second, s));
  }
  if (pl.comp_lo) {
    size_t lo_bytes = pl.ws_bytes - pl.o_lo;
    GG_CUDA(cudaMemsetAsync(ws + pl.o_lo, 0, lo_bytes, s));
  }
  if (opt->gcf_kind == GG_GCF_COUNT) {
    int maxS = 0;
    for (auto &cl : pl.classes) maxS = std::max(maxS, cl.S);
    for (size_t k = 0; k < pl.count_fill.size(); ++k) {
      GG_CUDA(launch_count_inputs(pl.count_fill[k].first, pl.vals_f64,
                                  pl.count_fill[k].second, pl.P,
                                  k == 0 ? (void *)(ws + pl.o_count_gcf) : nullptr,
                                  k == 0 ? (int64_t)pl.G * pl.G * maxS * maxS : 0, s));
    }
  }
  if (!pl.gcf_copies.empty())
    GG_CUDA(cudaMemsetAsync(ws + pl.o_gcf_flags, 0, sizeof(int) * pl.gcf_copies.size(), s));
  for (size_t ci = 0; ci < pl.gcf_copies.size(); ++ci) {
    const auto &c = pl.gcf_copies[ci];
    GG_CUDA(launch_gcf_double_rows(c.src ? c.src : ws + pl.o_count_gcf, ws + c.off, c.S, pl.G,
                                   c.ntab, (int)vbytes, s,
                                   c.off_real ? (float *)(ws + c.off_real) : nullptr,
                                   (int *)(ws + pl.o_gcf_flags) + ci));
  }

  GridLaunch g{};
  g.accum = pl.accum;
  g.vals_f64 = pl.vals_f64;
  g.gauss = pl.gauss;
  g.wphase = opt->gcf_kind == GG_GCF_WPHASE;
  g.sigma = pl.sigma;
  g.G = pl.G;
  g.tile = pl.T;
  g.group_warps = pl.group_warps;
  g.accumulate = opt->accumulate;
  g.P = pl.P;
  g.flags = flags;
  g.sm_count = sm_count;

  if (pl.mode != GG_MODE_SCATTER) {
    BinBuffers b{};
    b.jobs = (const BinJob *)(ws + pl.o_bin);
    b.vis_base = dvisb;
    b.tile_base = dtileb;
    b.njobs = pl.njobs;
    b.total_vis = pl.total_vis;
    b.total_tiles = pl.total_tiles;
    b.vals_bytes = (int)vbytes;
    b.P = pl.P;
    b.packed = (int2 *)(ws + pl.o_packed);
    b.key = (int *)(ws + pl.o_key);
    b.bookmarks = (int *)(ws + pl.o_bm);
    b.cursor = (int *)(ws + pl.o_cursor);
    b.scan_tmp = (int *)(ws + pl.o_scan);
    b.sorted_idx = (int2 *)(ws + pl.o_sidx);
    b.sorted_vals = ws + pl.o_svals;
    b.vstride = pl.vstride;
    b.order = nullptr;
    b.flags = flags;
    b.input_sorted = pl.input_sorted;
    b.kept_pos = pl.input_sorted ? (int *)(ws + pl.o_kept) : nullptr;
    b.window_records = pl.mode == GG_MODE_WINDOW;
    GG_CUDA(run_binning(b, s));
    g.holes = b.bookmarks + pl.total_tiles + 1;
  }

  if (pl.mode == GG_MODE_WINDOW) {
    // item counters [8, 12), item claims [12, 16), merge slots taken [16, 20)
    GG_CUDA(cudaMemsetAsync(flags + 8, 0, 12 * sizeof(int), s));
    WorkItem *items = (WorkItem *)(ws + pl.o_items);
    ClassChunks chunks;
    ClassSlots slots{};
    for (int ci = 0; ci < kMaxClasses; ++ci) {
      chunks.c[ci] = ci < (int)pl.classes.size() ? pl.classes[ci].chunk : pl.chunk;
      if (pl.merge_cap[ci] > 0) {
        slots.m[ci].base = (double2 *)(ws + pl.o_merge[ci]);
        slots.m[ci].desc = (int2 *)(ws + pl.o_mdesc[ci]);
        slots.m[ci].cap = pl.merge_cap[ci];
        slots.m[ci].cells = pl.merge_cells[ci];
      }
    }
    GG_CUDA(launch_make_items((const int *)(ws + pl.o_bm), dtileb, dclass, pl.njobs,
                              pl.total_tiles, chunks, items, pl.class_cap, flags + 8, s,
                              djobs, &slots, flags + 16, flags));
    for (int ci = 0; ci < kMaxClasses; ++ci)
      GG_CUDA(launch_merge_zero(slots.m[ci], flags + 16 + ci, sm_count, s));
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[1], s));
    for (size_t ci = 0; ci < pl.classes.size(); ++ci) {
      const auto &cl = pl.classes[ci];
      g.jobs = djobs;
      g.njobs = pl.njobs;
      g.S = cl.S;
      g.tile = cl.T;
      g.group_warps = cl.W;
      g.items = items + ci * pl.class_cap;
      g.nitems = flags + 8 + ci;
      if (side) GG_CUDA(cudaStreamWaitEvent(s, aux->done[ci], 0));
      g.item_next = flags + 12 + ci;
      g.max_items = pl.class_cap;
      g.merge = slots.m[ci];
      GG_CUDA(launch_window(g, s));
      GG_CUDA(launch_merge_finalize(slots.m[ci], flags + 16 + ci, djobs, cl.S, cl.T, pl.P,
                                    sm_count, s));
    }
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[2], s));
  } else if (pl.mode == GG_MODE_GATHER) {
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[1], s));
    for (const auto &cl : pl.classes) {
      g.jobs = djobs + cl.j0;
      g.njobs = cl.j1 - cl.j0;
      g.S = cl.S;
      g.tile_base = dtileb + cl.j0;
      g.total_tiles = cl.t1 - cl.t0;
      GG_CUDA(launch_gather(g, s));
    }
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[2], s));
  } else {
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[1], s));
    for (const auto &cl : pl.classes) {
      g.jobs = djobs + cl.j0;
      g.njobs = cl.j1 - cl.j0;
      g.S = cl.S;
      g.vis_base = dvisb + cl.j0;
      g.total_vis = cl.v1 - cl.v0;
      GG_CUDA(launch_scatter(g, s));
    }
    if (prof) GG_CUDA(cudaEventRecord(prof->ev[2], s));
    if (pl.comp_lo) {
      for (int k = 0; k < pl.njobs; ++k) {
        const JobDesc &D = pl.hjobs[k];
        if (D.lo)
          GG_CUDA(launch_comp_finalize((float *)D.out, D.lo, 2ll * pl.P * D.N * D.N, s));
      }
    }
  }
  if (prof) GG_CUDA(cudaEventRecord(prof->ev[3], s));
  return GG_OK;
}

static int enqueue_jobs(gg_context *c, const gg_options *opt, const gg_job *jobs,
                        int njobs, cudaStream_t s, const ClassCfgs *force) {
  Plan &pl = c->plan;
  int st = plan_build(c, opt, jobs, njobs, pl, force);
  if (st) return st;
  // the workspace may be reallocated: earlier work on it must be finished
  if (pl.ws_bytes > c->ws.n) GG_CUDA(cudaEventSynchronize(c->exec_done));
  if ((st = c->ws.ensure(pl.ws_bytes))) return st;
  // pinned staging: the previous upload must have been consumed
  GG_CUDA(cudaEventSynchronize(c->upload_done));
  if ((st = c->staging.ensure(pl.table_bytes))) return st;
  plan_bind(opt, pl, (char *)c->ws.p, (char *)c->staging.p);
  GG_CUDA(cudaStreamWaitEvent(s, c->exec_done, 0));
  ProfEvents pe;
  for (int i = 0; i < 4; ++i) pe.ev[i] = c->prof[i];
  st = plan_enqueue(opt, pl, gg::context_flags(c), c->sm_count, s, c->staging.p,
                    c->upload_done, c->profile ? &pe : nullptr, &c->aux);
  if (st) return st;
  if (c->profile) c->prof_recorded = 1;
  GG_CUDA(cudaEventRecord(c->exec_done, s));
  return GG_OK;
}

// Autotuner.  For every support class of a moving-window batch whose size
// class has no entry yet, time candidate configurations on the class's own
// jobs (every pair of warps per sub-grid group and tile, then records per
// work item at the best pair; two launches each, the faster counted) and
// record the fastest.  The trials write the jobs' outputs, which the real
// launch then overwrites; they synchronise stream s.
static int autotune_batch(gg_context *c, const gg_options *opt, const gg_job *jobs, int njobs,
                          cudaStream_t s) {
  // trials write the outputs: none when the caller accumulates into them
  if (opt->autotune != 1 || opt->accumulate || !tunable(opt) || njobs < 1 || !jobs)
    return GG_OK;
  int maxS = 0;
  for (int j = 0; j < njobs; ++j) maxS = std::max<int>(maxS, (int)jobs[j].gcf_dim);
  if (resolve_mode(opt, maxS, jobs[0].vals_type == GG_C128) != GG_MODE_WINDOW) return GG_OK;
  const int vf64 = jobs[0].vals_type == GG_C128;
  cudaEvent_t e0, e1;
  GG_CUDA(cudaEventCreate(&e0));
  GG_CUDA(cudaEventCreate(&e1));
  int st = GG_OK;
  std::vector<int> supports;
  for (int j = 0; j < njobs; ++j)
    if (std::find(supports.begin(), supports.end(), (int)jobs[j].gcf_dim) == supports.end())
      supports.push_back((int)jobs[j].gcf_dim);
  for (int S : supports) {
    const TuneKey key = tune_key(opt, vf64, S, density_class(jobs, njobs, S));
    std::vector<gg_job> sub;
    double vis = 0;
    for (int j = 0; j < njobs; ++j)
      if (jobs[j].gcf_dim == S) {
        sub.push_back(jobs[j]);
        vis += (double)jobs[j].npts;
      }
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      if (g_tune.count(key)) continue;
      if (vis < kTuneMinVis && tune_lookup(key)) continue;
    }
    int trials = 0;
    // time one configuration; a configuration the plan rejects (shared
    // memory) counts as infinitely slow
    auto timeit = [&](const ClassCfg &cf) -> double {
      ClassCfgs f{{S, cf}};
      double best = 1e30;
      for (int rep = 0; rep < 2; ++rep) {
        if (cudaEventRecord(e0, s) != cudaSuccess) return 1e30;
        if (enqueue_jobs(c, opt, sub.data(), (int)sub.size(), s, &f) != GG_OK) return 1e30;
        float ms = 0.f;
        if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
          return 1e30;
        best = std::min(best, (double)ms);
      }
      ++trials;
      return best;
    };
    ClassCfg base;
    base.T = S <= 16 && !opt->input_sorted ? 8 : 32;
    base.W = 0;
    base.chunk = 2048;
    const double t_default = timeit(base);
    if (t_default >= 1e30) {
      st = fail(GG_ERR_CUDA, "autotune: the default configuration failed for support %d", S);
      break;
    }
    ClassCfg best = base;
    double t_best = t_default;
    auto consider = [&](ClassCfg cf) {
      const double t = timeit(cf);
      if (t < t_best) {
        t_best = t;
        best = cf;
      }
    };
    // warps per group and tile jointly (their best pair is not found one
    // coordinate at a time: one-warp groups win on 8-cell tiles and lose on
    // 16-cell ones); 8-cell tiles give smaller sub-grids and so more resident
    // groups, not tried for support 32
    static const int kWarps[] = {1, 2, 4, 8};
    const ClassCfg base_best = best;
    for (int w : kWarps) {
      if ((S == 4 && w != 1) || (S == 8 && w > 2) || (S == 16 && w > 4) || (S == 32 && w < 4))
        continue;
      for (int T : {8, 16, 32}) {
        if (opt->input_sorted && T != base_best.T) continue;
        if (T == 8 && S > 16) continue;
        ClassCfg cf = base_best;
        cf.W = w;
        cf.T = T;
        consider(cf);
      }
    }
    for (int ch : {1024, 4096}) {
      ClassCfg cf = best;
      cf.chunk = ch;
      consider(cf);
    }
    // a rejected trial configuration leaves its message: clear it
    g_last_error.clear();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    TuneEntry &e = g_tune[key];
    e.cfg = best;
    e.ms_best = t_best;
    e.ms_default = t_default;
    e.trials = trials;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

static int grid_jobs(gg_context *c, const gg_options *opt, const gg_job *jobs,
                     int njobs, cudaStream_t s) {
  GG_CUDA(cudaSetDevice(c->device));
  int st = check_options(opt);
  if (st) return st;
  if ((st = autotune_batch(c, opt, jobs, njobs, s))) return st;
  return enqueue_jobs(c, opt, jobs, njobs, s, nullptr);
}

// ---------------------------------------------------------------------------
// exported ABI
// ---------------------------------------------------------------------------
extern "C" {

int gg_abi_version(void) { return GG_ABI_VERSION; }
const char *gg_last_error(void) { return g_last_error.c_str(); }

int gg_default_options(gg_options *opt) {
  if (!opt) return fail(GG_ERR_ARG, "opt: null");
  *opt = default_opts();
  return GG_OK;
}
int gg_set_global_options(const gg_options *opt) {
  int st = check_options(opt);
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_opt_mu);
  g_global_opts = *opt;
  return GG_OK;
}
int gg_get_global_options(gg_options *opt) {
  if (!opt) return fail(GG_ERR_ARG, "opt: null");
  std::lock_guard<std::mutex> lk(g_opt_mu);
  *opt = g_global_opts;
  return GG_OK;
}

int gg_debug_inject_alloc_failures(int32_t count) {
  if (count < 0) return fail(GG_ERR_ARG, "count < 0");
  g_fail_allocs.store(count);
  return GG_OK;
}

int gg_debug_inject_device_flags(int32_t bits, int32_t count) {
  if (count < 0 || (bits & ~0xf)) return fail(GG_ERR_ARG, "bits outside 0..15 or count < 0");
  std::lock_guard<std::mutex> lk(g_inject_mu);
  g_inject_bits = bits;
  g_inject_count = bits ? count : 0;
  return GG_OK;
}

int gg_selftest_wait_timeout(gg_context *ctx, void *stream) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  int *flags = (int *)ctx->flags.p;
  GG_CUDA(cudaMemsetAsync(flags + FLAG_TIMEOUT, 0, sizeof(int), s));
  GG_CUDA(launch_selftest_wait(flags, s));
  int h = 0;
  GG_CUDA(cudaMemcpyAsync(&h, flags + FLAG_TIMEOUT, sizeof h, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  GG_CUDA(cudaMemsetAsync(flags + FLAG_TIMEOUT, 0, sizeof(int), s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (h) return fail(GG_ERR_TIMEOUT, "device wait gave up after its limit (expected)");
  return fail(GG_ERR_STATE, "device wait did not report a timeout");
}

int gg_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return GG_OK;
}

int gg_autotune_report(char *buf, size_t len) {
  if (!buf || len == 0) return fail(GG_ERR_ARG, "buf: null or empty");
  std::string r;
  char line[256];
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto &kv : g_tune) {
    const TuneKey &k = kv.first;
    const TuneEntry &e = kv.second;
    snprintf(line, sizeof line,
             "support %d accum %d f64 %d gauss %d pols %d G %d density 2^%d vis/256 cells: "
             "tile %d group_warps %d chunk %d (%.3f ms; default %.3f ms; %d trials)\n",
             k.S, k.accum, k.vals_f64, k.gauss, k.P, k.G, k.density, e.cfg.T, e.cfg.W,
             e.cfg.chunk, e.ms_best, e.ms_default, e.trials);
    r += line;
  }
  snprintf(buf, len, "%s", r.c_str());
  return GG_OK;
}

int gg_create(gg_context **ctx, int device) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  *ctx = nullptr;
  std::unique_ptr<gg_context> c(new (std::nothrow) gg_context);
  if (!c) return fail(GG_ERR_NOMEM, "context allocation");
  int st = ctx_init(c.get(), device);
  if (st) {
    ctx_release(c.get());
    return st;
  }
  *ctx = c.release();
  return GG_OK;
}

int gg_destroy(gg_context *ctx) {
  if (!ctx) return GG_OK;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx_release(ctx);
  }
  delete ctx;
  return GG_OK;
}

int gg_reserve(gg_context *ctx, const gg_options *opt, int64_t max_npts,
               int64_t max_img_dim, int64_t max_gcf_dim, int32_t vals_type) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_job j;
  memset(&j, 0, sizeof j);
  j.out = (void *)16;
  j.uv = (const void *)16;
  j.vals = (const void *)16;
  j.gcf = (const void *)16;
  j.npts = max_npts;
  j.img_dim = max_img_dim;
  j.gcf_dim = max_gcf_dim;
  j.uv_type = GG_C128;
  j.vals_type = vals_type;
  // complex64 grids of FP32 values need the larger workspace (the lo grid of
  // the compensated scatter, the merge slots of the moving window)
  j.out_type = vals_type == GG_C128 ? GG_C128 : GG_C64;
  Plan pl;
  int st = plan_build(ctx, opt, &j, 1, pl);
  if (st) return st;
  GG_CUDA(cudaEventSynchronize(ctx->exec_done));
  st = ctx->ws.ensure(pl.ws_bytes);
  if (st) return st;
  return ctx->staging.ensure(pl.table_bytes + 4096);
}

int gg_workspace_bytes(gg_context *ctx, size_t *bytes) {
  if (!ctx || !bytes) return fail(GG_ERR_ARG, "null argument");
  *bytes = ctx->ws.n;
  return GG_OK;
}

int gg_grid_device(gg_context *ctx, const gg_options *opt, const gg_job *job,
                   void *stream) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  std::lock_guard<std::mutex> lk(ctx->mu);
  return grid_jobs(ctx, opt, job, 1, (cudaStream_t)stream);
}

int gg_degrid_device(gg_context *ctx, const gg_options *opt, const gg_job *job,
                     void *stream) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  if (!job) return fail(GG_ERR_ARG, "job: null");
  int st = check_options(opt);
  if (st) return st;
  const gg_job &J = *job;
  if (J.gcf_dim != 4 && J.gcf_dim != 8 && J.gcf_dim != 16 && J.gcf_dim != 32)
    return fail(GG_ERR_ARG, "degrid: gcf_dim %lld not in {4,8,16,32}", (long long)J.gcf_dim);
  if (J.img_dim < 1 || J.img_dim > (1 << 16))
    return fail(GG_ERR_ARG, "degrid: img_dim %lld outside 1..65536", (long long)J.img_dim);
  if (J.npts < 0) return fail(GG_ERR_ARG, "degrid: npts < 0");
  for (int t : {J.uv_type, J.vals_type, J.out_type})
    if (t != GG_C64 && t != GG_C128) return fail(GG_ERR_ARG, "degrid: type %d", t);
  if (opt->gcf_kind != GG_GCF_TABLE && opt->gcf_kind != GG_GCF_GAUSSIAN)
    return fail(GG_ERR_ARG, "degrid: gcf_kind %d (table or Gaussian)", opt->gcf_kind);
  const bool gauss = opt->gcf_kind == GG_GCF_GAUSSIAN;
  if (J.npts > 0 && (!J.out || !J.uv || !J.vals || (!gauss && !J.gcf)))
    return fail(GG_ERR_ARG, "degrid: null device pointer");
  if (J.gcf_index && (gauss || J.n_gcf < 1 || J.n_gcf > 32768))
    return fail(GG_ERR_ARG, "degrid: gcf_index needs a table stack of 1..32768 tables");
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  DegridLaunch d{};
  d.grid = J.out;
  d.vals = const_cast<void *>(J.vals);
  d.uv = J.uv;
  d.gcf = gauss ? nullptr : J.gcf;
  d.gcf_index = J.gcf_index;
  d.npts = J.npts;
  d.N = (int)J.img_dim;
  d.S = (int)J.gcf_dim;
  d.G = opt->oversample;
  d.P = opt->polarizations;
  d.n_gcf = J.gcf_index ? (int)J.n_gcf : 1;
  d.uv_f64 = J.uv_type == GG_C128;
  d.grid_f64 = J.out_type == GG_C128;
  d.vals_f64 = J.vals_type == GG_C128;
  d.planar = opt->layout == GG_LAYOUT_PLANAR;
  d.gauss = gauss;
  d.compensated = opt->accum == GG_ACC_COMPENSATED;
  const double sg = J.gcf_sigma > 0 ? J.gcf_sigma
                                    : (opt->gcf_sigma > 0 ? opt->gcf_sigma : J.gcf_dim / 4.0);
  d.sigma = (float)sg;
  d.flags = (int *)ctx->flags.p;
  d.sm_count = ctx->sm_count;
  GG_CUDA(launch_degrid(d, (cudaStream_t)stream));
  return GG_OK;
}

int gg_grid_to_image(gg_context *ctx, void *grid, int64_t img_dim, int32_t pols,
                     int32_t grid_type, void *stream) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  if (!grid) return fail(GG_ERR_ARG, "grid: null");
  if (img_dim < 2 || img_dim > (1 << 15) || (img_dim & 1))
    return fail(GG_ERR_ARG, "image: img_dim %lld must be even, 2..32768", (long long)img_dim);
  if (pols < 1 || pols > kMaxPols) return fail(GG_ERR_ARG, "image: pols %d", pols);
  if (grid_type != GG_C64 && grid_type != GG_C128)
    return fail(GG_ERR_ARG, "image: grid_type %d", grid_type);
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  std::string err;
  if (image_inverse_fft(grid, img_dim, pols, grid_type == GG_C128, ctx->sm_count,
                        (cudaStream_t)stream, err))
    return fail(GG_ERR_CUDA, "image: %s", err.c_str());
  return GG_OK;
}

int gg_grid_batch(gg_context *ctx, const gg_options *opt, const gg_job *jobs,
                  int32_t njobs, void *stream) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  std::lock_guard<std::mutex> lk(ctx->mu);
  return grid_jobs(ctx, opt, jobs, njobs, (cudaStream_t)stream);
}

int gg_read_flags(gg_context *ctx, void *stream, int32_t flags[4]) {
  if (!flags) return fail(GG_ERR_ARG, "flags: null");
  // no context: the flags of the last allocation-free call on this device
  if (!ctx) return noalloc_read_flags(stream, flags);
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  int h[4];
  GG_CUDA(cudaMemcpyAsync(h, ctx->flags.p, sizeof h, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  GG_CUDA(cudaMemsetAsync(ctx->flags.p, 0, sizeof h, s));
  GG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < 4; ++i) flags[i] = h[i];
  return GG_OK;
}

}  // extern "C"

struct gg_plan {
  gg_context *ctx = nullptr;
  gg_options opt;
  Plan pl;
  DevBuf ws, flags;
  AuxStream aux;
};

extern "C" {

int gg_plan_create(gg_context *ctx, const gg_options *opt, const gg_job *jobs,
                   int32_t njobs, gg_plan **out) {
  if (!ctx || !out) return fail(GG_ERR_ARG, "null argument");
  *out = nullptr;
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  std::unique_ptr<gg_plan> p(new (std::nothrow) gg_plan);
  if (!p) return fail(GG_ERR_NOMEM, "plan allocation");
  p->ctx = ctx;
  if (!opt) return fail(GG_ERR_ARG, "opt: null");
  p->opt = *opt;
  int st = check_options(opt);
  if (st) return st;
  if ((st = autotune_batch(ctx, opt, jobs, njobs, ctx->own))) return st;
  GG_CUDA(cudaStreamSynchronize(ctx->own));
  st = plan_build(ctx, opt, jobs, njobs, p->pl);
  if (st) return st;
  if ((st = p->ws.ensure(p->pl.ws_bytes))) return st;
  if ((st = p->flags.ensure(64 * sizeof(int)))) {
    p->ws.release();
    return st;
  }
  if ((st = p->aux.init())) {
    p->ws.release();
    p->flags.release();
    p->aux.release();
    return st;
  }
  std::vector<char> tables(p->pl.table_bytes);
  plan_bind(opt, p->pl, (char *)p->ws.p, tables.data());
  cudaError_t e = cudaMemcpy(p->ws.p, tables.data(), p->pl.table_bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->flags.p, 0, 64 * sizeof(int));
  if (e != cudaSuccess) {
    p->ws.release();
    p->flags.release();
    p->aux.release();
    return cuda_fail(e, "plan upload");
  }
  *out = p.release();
  return GG_OK;
}

int gg_plan_launch(gg_plan *p, void *stream) {
  if (!p) return fail(GG_ERR_ARG, "plan: null");
  GG_CUDA(cudaSetDevice(p->ctx->device));
  return plan_enqueue(&p->opt, p->pl, (int *)p->flags.p, p->ctx->sm_count,
                      (cudaStream_t)stream, nullptr, nullptr, nullptr, &p->aux);
}

int gg_plan_read_flags(gg_plan *p, void *stream, int32_t flags[4]) {
  if (!p || !flags) return fail(GG_ERR_ARG, "null argument");
  GG_CUDA(cudaSetDevice(p->ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  int h[4];
  GG_CUDA(cudaMemcpyAsync(h, p->flags.p, sizeof h, cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  GG_CUDA(cudaMemsetAsync(p->flags.p, 0, sizeof h, s));
  GG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < 4; ++i) flags[i] = h[i];
  return GG_OK;
}

int gg_plan_destroy(gg_plan *p) {
  if (!p) return GG_OK;
  cudaSetDevice(p->ctx->device);
  cudaDeviceSynchronize();
  p->ws.release();
  p->flags.release();
  p->aux.release();
  delete p;
  return GG_OK;
}

int gg_profile_enable(gg_context *ctx, int on) {
  if (!ctx) return fail(GG_ERR_ARG, "ctx: null");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->profile = on ? 1 : 0;
  ctx->prof_recorded = 0;
  return GG_OK;
}

int gg_profile_last(gg_context *ctx, double ms[3]) {
  if (!ctx || !ms) return fail(GG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->profile || !ctx->prof_recorded)
    return fail(GG_ERR_STATE, "profiling off or no call recorded");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CUDA(cudaEventSynchronize(ctx->prof[3]));
  float a = 0, b = 0, t = 0;
  GG_CUDA(cudaEventElapsedTime(&a, ctx->prof[0], ctx->prof[1]));
  GG_CUDA(cudaEventElapsedTime(&b, ctx->prof[1], ctx->prof[2]));
  GG_CUDA(cudaEventElapsedTime(&t, ctx->prof[0], ctx->prof[3]));
  ms[0] = a;
  ms[1] = b;
  ms[2] = t;
  return GG_OK;
}

int gg_kernel_launches(int64_t *count) {
  if (!count) return fail(GG_ERR_ARG, "count: null");
  *count = (int64_t)g_launches.load();
  return GG_OK;
}

int gg_vis2ints(int uv_type, const void *uv, int64_t npts, int32_t oversample,
                int32_t *packed, void *stream) {
  if (npts < 0 || (npts > 0 && (!uv || !packed)))
    return fail(GG_ERR_ARG, "vis2ints: bad arguments");
  if (uv_type != GG_C64 && uv_type != GG_C128) return fail(GG_ERR_ARG, "uv_type");
  if (!is_pow2(oversample) || oversample > 64) return fail(GG_ERR_ARG, "oversample");
  static int *dflags = nullptr;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!dflags) {
      GG_CUDA(cudaMalloc(&dflags, 16 * sizeof(int)));
      GG_CUDA(cudaMemset(dflags, 0, 16 * sizeof(int)));
    }
  }
  GG_CUDA(launch_vis2ints(uv_type == GG_C128, uv, npts, oversample, (int2 *)packed,
                          dflags, (cudaStream_t)stream));
  return GG_OK;
}

int gg_bin(gg_context *ctx, const gg_options *opt, int uv_type, const void *uv,
           int64_t npts, int64_t img_dim, int64_t gcf_dim, int32_t *bookmarks,
           int32_t *order, void *stream) {
  if (!ctx || !bookmarks) return fail(GG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_options o = *opt;
  o.mode = GG_MODE_GATHER;
  o.gcf_kind = GG_GCF_GAUSSIAN;  // no table needed; nothing is gridded
  o.tile = opt->tile;
  gg_job j;
  memset(&j, 0, sizeof j);
  j.out = (void *)16;
  j.uv = uv;
  j.vals = uv;  // values are copied along but unused: reuse the uv array
  j.npts = npts;
  j.img_dim = img_dim;
  j.gcf_dim = gcf_dim;
  j.uv_type = uv_type;
  j.vals_type = GG_C64;
  j.out_type = GG_C64;
  if (o.tile != 32) o.mode = GG_MODE_WINDOW;
  Plan pl;
  int st = plan_build(ctx, &o, &j, 1, pl);
  if (st) return st;
  pl.P = 1;
  if (pl.ws_bytes > ctx->ws.n) GG_CUDA(cudaEventSynchronize(ctx->exec_done));
  size_t order_off = align256(pl.ws_bytes);
  pl.ws_bytes = order_off + align256(sizeof(int) * (npts + 8));
  if ((st = ctx->ws.ensure(pl.ws_bytes))) return st;
  GG_CUDA(cudaEventSynchronize(ctx->upload_done));
  if ((st = ctx->staging.ensure(pl.table_bytes))) return st;
  plan_bind(&o, pl, (char *)ctx->ws.p, (char *)ctx->staging.p);
  char *ws = (char *)ctx->ws.p;
  cudaStream_t s = (cudaStream_t)stream;
  GG_CUDA(cudaStreamWaitEvent(s, ctx->exec_done, 0));
  GG_CUDA(launch_upload(ws, ctx->staging.p, pl.table_bytes, s));
  GG_CUDA(cudaEventRecord(ctx->upload_done, s));
  BinBuffers b{};
  b.jobs = (const BinJob *)(ws + pl.o_bin);
  b.vis_base = (const int64_t *)(ws + pl.o_visb);
  b.tile_base = (const int *)(ws + pl.o_tileb);
  b.njobs = 1;
  b.total_vis = pl.total_vis;
  b.total_tiles = pl.total_tiles;
  b.vals_bytes = 8;
  b.P = 1;
  b.packed = (int2 *)(ws + pl.o_packed);
  b.key = (int *)(ws + pl.o_key);
  b.bookmarks = (int *)(ws + pl.o_bm);
  b.cursor = (int *)(ws + pl.o_cursor);
  b.scan_tmp = (int *)(ws + pl.o_scan);
  b.sorted_idx = (int2 *)(ws + pl.o_sidx);
  b.sorted_vals = ws + pl.o_svals;
  b.vstride = pl.vstride;
  b.order = (int *)(ws + order_off);
  b.flags = (int *)ctx->flags.p;
  b.input_sorted = pl.input_sorted;
  b.kept_pos = pl.input_sorted ? (int *)(ws + pl.o_kept) : nullptr;
  GG_CUDA(run_binning(b, s));
  GG_CUDA(cudaMemcpyAsync(bookmarks, b.bookmarks, sizeof(int) * (pl.total_tiles + 1),
                          cudaMemcpyDeviceToDevice, s));
  if (order)
    GG_CUDA(cudaMemcpyAsync(order, b.order, sizeof(int) * npts, cudaMemcpyDeviceToDevice, s));
  GG_CUDA(cudaEventRecord(ctx->exec_done, s));
  return GG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// host-buffer entry points (drop-in gridGPU)
// ---------------------------------------------------------------------------
static std::mutex g_host_mu;
static gg_context *g_host_ctx[64];

static int host_ctx(gg_context **out) {
  int dev = 0;
  GG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(GG_ERR_ARG, "device %d", dev);
  std::lock_guard<std::mutex> lk(g_host_mu);
  if (!g_host_ctx[dev]) {
    int st = gg_create(&g_host_ctx[dev], dev);
    if (st) return st;
  }
  *out = g_host_ctx[dev];
  return GG_OK;
}

extern "C" int gg_grid_host(const gg_options *opt, int out_type, void *out,
                            int uv_type, const void *uv, int vals_type,
                            const void *vals, size_t npts, size_t img_dim,
                            const void *gcf, size_t gcf_dim) {
  int st = check_options(opt);
  if (st) return st;
  if (!out) return fail(GG_ERR_ARG, "out: null");
  if (npts > 0 && (!uv || !vals)) return fail(GG_ERR_ARG, "in/in_vals: null");
  if ((opt->gcf_kind == GG_GCF_TABLE || opt->gcf_kind == GG_GCF_WPHASE) && !gcf)
    return fail(GG_ERR_ARG, "gcf: null");
  gg_context *c = nullptr;
  if ((st = host_ctx(&c))) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  GG_CUDA(cudaSetDevice(c->device));
  const size_t P = (size_t)opt->polarizations, G = (size_t)opt->oversample;
  const size_t N = img_dim, S = gcf_dim;
  const size_t uvb = uv_type == GG_C128 ? 16 : 8, vb = vals_type == GG_C128 ? 16 : 8;
  const size_t ob = out_type == GG_C128 ? 16 : 8;
  const size_t grid_elems = P * N * N;
  const size_t head = N * S + S;
  const size_t total = (N * N + 2 * N * S + 2 * S) * P;
  // wait for the previous host call to finish with the device copies
  GG_CUDA(cudaEventSynchronize(c->exec_done));
  if ((st = c->h_uv.ensure(uvb * (npts + 1)))) return st;
  if ((st = c->h_vals.ensure(vb * P * (npts + 1)))) return st;
  if ((st = c->h_gcf.ensure(vb * G * G * S * S + 16))) return st;
  if ((st = c->h_out.ensure(ob * grid_elems))) return st;
  cudaStream_t s = c->own;
  if (npts) {
    GG_CUDA(cudaMemcpyAsync(c->h_uv.p, uv, uvb * npts, cudaMemcpyHostToDevice, s));
    GG_CUDA(cudaMemcpyAsync(c->h_vals.p, vals, vb * P * npts, cudaMemcpyHostToDevice, s));
  }
  if (opt->gcf_kind == GG_GCF_TABLE || opt->gcf_kind == GG_GCF_WPHASE)
    GG_CUDA(cudaMemcpyAsync(c->h_gcf.p, gcf, vb * G * G * S * S, cudaMemcpyHostToDevice, s));
  gg_job j;
  memset(&j, 0, sizeof j);
  j.out = c->h_out.p;
  j.uv = c->h_uv.p;
  j.vals = c->h_vals.p;
  j.gcf = c->h_gcf.p;
  j.npts = (int64_t)npts;
  j.img_dim = (int64_t)N;
  j.gcf_dim = (int64_t)S;
  j.uv_type = uv_type;
  j.vals_type = vals_type;
  j.out_type = out_type;
  gg_options ho = *opt;
  ho.accumulate = 0;  // the device copy of the grid starts empty: overwrite
  st = grid_jobs(c, &ho, &j, 1, s);
  if (st) return st;
  char *o = (char *)out;
  GG_CUDA(cudaMemcpyAsync(o + ob * head, c->h_out.p, ob * grid_elems, cudaMemcpyDeviceToHost, s));
  memset(o, 0, ob * head);
  memset(o + ob * (head + grid_elems), 0, ob * (total - head - grid_elems));
  GG_CUDA(cudaStreamSynchronize(s));
  int h[4];
  GG_CUDA(cudaMemcpy(h, c->flags.p, sizeof h, cudaMemcpyDeviceToHost));
  GG_CUDA(cudaMemset(c->flags.p, 0, sizeof h));
  if (h[FLAG_TIMEOUT]) return fail(GG_ERR_TIMEOUT, "a bounded device wait expired");
  if (h[FLAG_UNSORTED])
    return fail(GG_ERR_UNSORTED, "input_sorted set but visibilities are not tile-sorted");
  if (h[FLAG_BOUNDS]) return fail(GG_ERR_STATE, "internal: sub-grid bounds check failed");
  return GG_OK;
}

static int host_typed(int out_type, void *out, int in_type, const void *in,
                      const void *vals, size_t npts, size_t img_dim,
                      const void *gcf, size_t gcf_dim) {
  gg_options o;
  {
    std::lock_guard<std::mutex> lk(g_opt_mu);
    o = g_global_opts;
  }
  return gg_grid_host(&o, out_type, out, in_type, in, in_type, vals, npts, img_dim,
                      gcf, gcf_dim);
}

extern "C" int gg_gridGPU_zz(double *out, const double *in, const double *in_vals,
                             size_t npts, size_t img_dim, const double *gcf,
                             size_t gcf_dim) {
  return host_typed(GG_C128, out, GG_C128, in, in_vals, npts, img_dim, gcf, gcf_dim);
}
extern "C" int gg_gridGPU_zc(double *out, const float *in, const float *in_vals,
                             size_t npts, size_t img_dim, const float *gcf,
                             size_t gcf_dim) {
  return host_typed(GG_C128, out, GG_C64, in, in_vals, npts, img_dim, gcf, gcf_dim);
}
extern "C" int gg_gridGPU_cc(float *out, const float *in, const float *in_vals,
                             size_t npts, size_t img_dim, const float *gcf,
                             size_t gcf_dim) {
  return host_typed(GG_C64, out, GG_C64, in, in_vals, npts, img_dim, gcf, gcf_dim);
}
