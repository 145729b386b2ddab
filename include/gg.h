/*
 * gg.h -- C ABI of the GB300 convolutional gridder (libgg.so).
 *
 * Plain pointers and sizes only.  Every function returns a status code
 * (GG_OK = 0); gg_last_error() gives the message of the last failure on the
 * calling thread.
 *
 * Reference interfaces replaced (paths within NVIDIA/SKA-gpu-grid):
 *   gridGPU<CmplxOutType,CmplxType>   grid_gpu.cuh:30-32, grid_gpu.cu:675-819,
 *                                     instantiations grid_gpu.cu:820-825
 *   vis2ints                          grid_gpu.cu:352-365
 *   set_bookmarks                     grid_gpu.cu:366-390
 *   Defines.h compile-time switches   Defines.h:57-77, Makefile:30-60
 *   GPUGrid.convgrid (Python 2)       GPUGrid.cpp:124-164
 *
 * Coordinates are in grid pixels (the caller centres them, as in grid.cu:446).
 * Taps of a visibility at main cell m cover m-S/2+1 .. m+S/2 on each axis
 * (grid.cu:167-168); taps outside [0, img_dim) are dropped.  The GCF table is
 * [G*G][S][S] complex, indexed [sub_y*G+sub_x][b'][a'] with a'=a+S/2-1.
 */
#ifndef GG_H
#define GG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GG_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define GG_OK 0
#define GG_ERR_ARG 1      /* invalid argument or unsupported combination     */
#define GG_ERR_CUDA 2     /* a CUDA runtime call failed                      */
#define GG_ERR_NOMEM 3    /* device or pinned-host allocation failed         */
#define GG_ERR_UNSORTED 4 /* input declared tile-sorted is not               */
#define GG_ERR_BUDGET 5   /* request larger than the server's HBM budget     */
#define GG_ERR_TIMEOUT 6  /* a bounded device or host wait expired           */
#define GG_ERR_CANCELLED 7
#define GG_ERR_STATE 8    /* object used after failure / in the wrong state  */

/* ---- element types ----------------------------------------------------- */
#define GG_C64 0  /* float2:  complex64,  or (u,v) as two floats             */
#define GG_C128 1 /* double2: complex128, or (u,v) as two doubles            */

/* ---- gridding method: the reference's compile-time GATHER= / MOVING_WINDOW=
 *      switches (Makefile:37-45) become a run-time field ------------------ */
#define GG_MODE_SCATTER 0 /* per-tap native red.global adds                  */
#define GG_MODE_GATHER 1  /* one output cell per thread over uv-tile bins    */
#define GG_MODE_WINDOW 2  /* register + shared-memory moving window per tile */
#define GG_MODE_AUTO 3    /* moving window for FP32 values, scatter for FP64
                             values (the faster on this GPU for each)        */

/* ---- output layout ----------------------------------------------------- */
#define GG_LAYOUT_INTERLEAVED 0 /* P planes of N*N (re,im) pairs             */
#define GG_LAYOUT_PLANAR 1      /* re[P][N][N] then im[P][N][N] (gridCPU_pz) */
#define GG_LAYOUT_REFERENCE 2   /* what gridGPU writes per method: planar for
                                   the moving window (grid_gpu.cu:524-525),
                                   interleaved otherwise (:162-163, :500)   */

/* ---- accumulation ------------------------------------------------------ */
#define GG_ACC_PLAIN 0       /* arithmetic in the values' precision         */
#define GG_ACC_COMPENSATED 1 /* FP32 two-sum hi/lo per cell (FP32 values)    */

/* ---- GCF source -------------------------------------------------------- */
#define GG_GCF_TABLE 0    /* tabulated [G*G][S][S] complex (init_gcf layout)  */
#define GG_GCF_GAUSSIAN 1 /* COMPUTE_GCF: separable exp(-x^2/(2 sigma^2)),
                             x = a - sub/G, evaluated on the device          */
#define GG_GCF_COUNT 2    /* DEBUG1 footprint mode (Defines.h:78): every tap
                             adds (1, visibility index)                     */
#define GG_GCF_WPHASE 3   /* COMPUTE_GCF as the reference's scatter kernel
                             computes it (grid_gpu.cu:103-108, 137-147):
                             every tap of a visibility gets (sin p, cos p),
                             p = p1 - p2*sqrt(dx^2 + dy^2) in FP32 with
                             p1 = 2*pi*w, p2 = p1*T, (T, w) = the table entry
                             at the centre offset S(S-1)/2-1 and dx = main_x
                             - u + sub_x/G; gridded by the scatter method   */

typedef struct gg_options {
  int32_t mode;          /* GG_MODE_*                                        */
  int32_t layout;        /* GG_LAYOUT_*                                      */
  int32_t accum;         /* GG_ACC_*                                         */
  int32_t gcf_kind;      /* GG_GCF_*                                         */
  int32_t oversample;    /* GCF_GRID: power of two, 1..64 (default 8)        */
  int32_t polarizations; /* POLARIZATIONS: 1..8 (default 1)                  */
  int32_t tile;          /* uv tile side in cells for binning, a power of
                            two in 8..256 (gather: 32); 0 = chosen by
                            method and support (default)                  */
  int32_t input_sorted;  /* 1: caller guarantees visibilities are grouped by
                            uv tile (of `tile` cells, 32 when tile is 0) in
                            ascending tile id (checked)                      */
  double gcf_sigma;      /* GG_GCF_GAUSSIAN: sigma in cells; 0 -> S/4        */
  int32_t window_chunk;  /* max visibilities per work item (0 -> default)    */
  int32_t group_warps;   /* moving window: warps sharing one sub-grid
                            (1, 2, 4 or 8; 0 -> chosen by support)           */
  int32_t autotune;      /* moving window with tile, group_warps and
                            window_chunk all 0: 1 = pick them per support
                            class by timing candidates on the first batch of
                            each size class (that call synchronises its
                            stream), then reuse the choice (process-wide).
                            The trials grid the batch itself (writing its
                            outputs, which the real launch then rewrites);
                            gg_plan_create runs them at creation, on the
                            inputs present then.  2 = reuse the choices
                            made so far (the nearest size class of the same
                            support and arithmetic; defaults when there is
                            none) and never time trials.                   */
  int32_t accumulate;    /* 1: add the gridded values into the present
                            contents of each job's `out` instead of
                            overwriting it (device entry points: summing
                            w-planes, facets or snapshots into one grid; the
                            host entry points and the request server always
                            overwrite).  Autotuner
                            trials, which write the outputs, are not run:
                            choices made so far are reused as with
                            autotune = 2.                                    */
  int32_t reserved[4];
} gg_options;

/* Defaults = the reference built with no Makefile switches: SCATTER,
 * REFERENCE layout, PLAIN, TABLE, G=8, P=1; automatic tile. */
int gg_default_options(gg_options *opt);

/* Process-wide options used by the drop-in gridGPU entry points below, the
 * run-time counterpart of Defines.h / Makefile switches. */
int gg_set_global_options(const gg_options *opt);
int gg_get_global_options(gg_options *opt);

/* Autotuner cache (see gg_options.autotune): forget every choice, or write a
 * text table of the choices made so far into buf (always NUL-terminated). */
int gg_autotune_clear(void);
int gg_autotune_report(char *buf, size_t len);

const char *gg_last_error(void);
int gg_abi_version(void);


/* ---- drop-in gridGPU: HOST buffers, reference semantics ----------------
 * out: (img_dim^2 + 2*img_dim*gcf_dim + 2*gcf_dim) * P elements; the grid is
 * written at element offset img_dim*gcf_dim + gcf_dim and everything else is
 * zeroed, i.e. out is overwritten, never accumulated (grid_gpu.cu:755-800).
 * in: npts (u,v); in_vals: npts*P complex; gcf: G*G*S*S complex, un-offset.
 * Unlike the reference these allocate nothing per call (a context owns the
 * device buffers), pin nothing, and report errors.                          */
int gg_gridGPU_zz(double *out, const double *in, const double *in_vals,
                  size_t npts, size_t img_dim, const double *gcf,
                  size_t gcf_dim); /* gridGPU<double2,double2> */
int gg_gridGPU_zc(double *out, const float *in, const float *in_vals,
                  size_t npts, size_t img_dim, const float *gcf,
                  size_t gcf_dim); /* gridGPU<double2,float2>  */
int gg_gridGPU_cc(float *out, const float *in, const float *in_vals,
                  size_t npts, size_t img_dim, const float *gcf,
                  size_t gcf_dim); /* gridGPU<float2,float2>   */

/* The same with explicit options and element types (uv_type and vals_type
 * may differ, e.g. FP64 coordinates with complex64 values). */
int gg_grid_host(const gg_options *opt, int out_type, void *out, int uv_type,
                 const void *uv, int vals_type, const void *vals, size_t npts,
                 size_t img_dim, const void *gcf, size_t gcf_dim);

/* ---- device-resident API ------------------------------------------------ */
typedef struct gg_context gg_context;

int gg_create(gg_context **ctx, int device);
int gg_destroy(gg_context *ctx);

/* ---- failure detection, tested without a GPU fault ---------------------
 * Every device-side wait of the library (mbarrier phases of the bulk copies)
 * gives up after a bounded time (0.5 s), raises the context's timeout flag
 * (gg_read_flags()[1]) and lets the kernel return.
 * gg_selftest_wait_timeout runs one warp that waits on an mbarrier nothing
 * completes; it returns GG_ERR_TIMEOUT when the wait gave up as designed
 * (the context stays usable) and GG_ERR_STATE otherwise.
 * gg_debug_inject_alloc_failures makes the next `count` device allocations
 * of the library fail with GG_ERR_NOMEM (0 switches it off): a test hook for
 * allocation-failure paths. */
int gg_selftest_wait_timeout(gg_context *ctx, void *stream);
int gg_debug_inject_alloc_failures(int32_t count);
/* Test hook for the reporting of device-side failures: the next `count`
 * served batches and allocation-free calls get the flag bits `bits`
 * (GG_DEVFLAG_*) raised in their device flag word by a one-thread kernel
 * enqueued after their gridding kernels and before their flags are read
 * back -- as if a kernel had raised them.  No fault and no device wait is
 * involved.  bits 0 switches it off. */
int gg_debug_inject_device_flags(int32_t bits, int32_t count);

/* Pre-size the context's device workspace for jobs up to these sizes so that
 * later calls allocate nothing (needed before CUDA-graph capture). */
int gg_reserve(gg_context *ctx, const gg_options *opt, int64_t max_npts,
               int64_t max_img_dim, int64_t max_gcf_dim, int32_t vals_type);
/* bytes of device workspace the context holds */
int gg_workspace_bytes(gg_context *ctx, size_t *bytes);

typedef struct gg_job {
  void *out;          /* device grid head: N*N*P complex of out_type; it is
                         overwritten (zeroed first) by the call            */
  const void *uv;     /* device: npts (u,v) pairs of uv_type              */
  const void *vals;   /* device: npts*P complex of vals_type              */
  const void *gcf;    /* device: G*G*S*S complex of vals_type (TABLE)     */
  int64_t npts;
  int64_t img_dim;
  int64_t gcf_dim;
  int32_t uv_type, vals_type, out_type;
  int32_t reserved0;
  double gcf_sigma;   /* overrides options.gcf_sigma when > 0             */
  const int32_t *gcf_index; /* device, optional (TABLE GCF, scatter or moving
                         window): per-visibility table index -- visibility n
                         uses table gcf_index[n] of n_gcf consecutive
                         [G*G][S][S] tables at gcf (a w-plane or baseline
                         GCF, the reference's vis.gcfinx, vis.h:17);
                         visibilities with an index outside [0, n_gcf) are
                         dropped and counted like bad indices             */
  int64_t n_gcf;      /* tables at gcf when gcf_index is set (1..32768)    */
  int64_t reserved[2];
} gg_job;

/* Grid one job on `stream` (a cudaStream_t; NULL = the legacy default
 * stream).  Asynchronous: returns after enqueueing. */
int gg_grid_device(gg_context *ctx, const gg_options *opt, const gg_job *job,
                   void *stream);

/* Degridding, the adjoint of gridding (no counterpart in the reference; it
 * keeps the gridder's index step, tap window (-S/2, S/2] and table layout):
 *   vals[n][p] = sum over the on-grid taps of visibility n of
 *                grid[p][y][x] * conj(gcf entry of the tap)
 * so that <grid(v), g> = <v, degrid(g)> for <a, b> = sum conj(a) b.  The
 * job's fields are read as for gg_grid_device except that `out` is the grid
 * to sample (read, out_type, opt->layout: GG_LAYOUT_PLANAR planar, every
 * other layout interleaved) and `vals` RECEIVES npts*P values (vals_type);
 * the table (or Gaussian) and gcf_index/n_gcf select the kernel as for
 * gridding.  Visibilities with an oversample or table index out of range get
 * zero and are counted (gg_read_flags()[0]).  FP32 values: plain FP32 sums,
 * or two-sum compensated ones with GG_ACC_COMPENSATED; FP64 values: FP64.
 * Asynchronous on `stream`; no workspace, no allocation. */
int gg_degrid_device(gg_context *ctx, const gg_options *opt, const gg_job *job,
                     void *stream);

/* Grid -> dirty image, in place: every one of the `pols` planes of an
 * interleaved N*N complex grid (grid_type GG_C64 / GG_C128) becomes
 *   image[m][l] = sum_{v,u} grid[v][u]
 *                 * exp(+2 pi i ((u-N/2)(l-N/2) + (v-N/2)(m-N/2)) / N)
 * (zero spatial frequency at cell (N/2, N/2), image centre at pixel
 * (N/2, N/2), no normalisation); N even, at most 32768.  No counterpart in
 * the reference.  Uses cuFFT, loaded at first use (GG_ERR_CUDA if it cannot
 * be); plans a transform per call and synchronises `stream`.  After an
 * error the grid's contents are unspecified. */
int gg_grid_to_image(gg_context *ctx, void *grid, int64_t img_dim, int32_t pols,
                     int32_t grid_type, void *stream);

/* Many independent jobs in one persistent launch over a device work queue of
 * (job, uv tile) items.  All jobs share opt, S-class and types. */
int gg_grid_batch(gg_context *ctx, const gg_options *opt, const gg_job *jobs,
                  int32_t njobs, void *stream);

/* ---- plans: a batch fixed once, launched many times ---------------------
 * gg_plan_create validates the jobs, allocates the plan's own workspace and
 * uploads its device tables (synchronously).  gg_plan_launch then only
 * enqueues memsets and kernels on `stream` -- no host copies, allocations
 * or synchronisation -- so it can be captured into a CUDA graph and
 * replayed; every launch re-reads the jobs' input buffers and overwrites
 * their outputs. */
typedef struct gg_plan gg_plan;
int gg_plan_create(gg_context *ctx, const gg_options *opt, const gg_job *jobs,
                   int32_t njobs, gg_plan **plan);
int gg_plan_launch(gg_plan *plan, void *stream);
/* the plan's flag counters, like gg_read_flags (synchronises the stream) */
int gg_plan_read_flags(gg_plan *plan, void *stream, int32_t flags[4]);
int gg_plan_destroy(gg_plan *plan);

/* Counters of the last completed calls on this context (synchronises the
 * stream, then clears them): [0] visibilities dropped because their
 * oversample index fell outside [0,G) (u not float-representable right below
 * an integer), [1] bounded-wait timeouts, [2] unsorted input detected (the
 * call gridded nothing), [3] an internal bounds check failed.
 * ctx NULL: the counters of the last gg_grid_device_noalloc call on the
 * current device (not cleared; the next such call clears them). */
int gg_read_flags(gg_context *ctx, void *stream, int32_t flags[4]);

/* Profiling (the reference's getElapsed event timer, grid_gpu.cu:38-44, made
 * per phase): when enabled, every grid call records CUDA events on its own
 * stream around the binning pass and around the gridding kernels. */
int gg_profile_enable(gg_context *ctx, int on);
/* Times in ms of the last grid call on ctx: [0] binning (index step, tile
 * sort, bookmarks, work queue), [1] gridding kernels, [2] whole call.
 * Waits for that call's last event. */
int gg_profile_last(gg_context *ctx, double ms[3]);
/* Kernels launched by this process through libgg so far. */
int gg_kernel_launches(int64_t *count);

/* vis2ints (grid_gpu.cu:352-365) on device buffers: packed[2n] = main_x*G +
 * sub_x, packed[2n+1] = main_y*G + sub_y, bit-exact with grid.cu:159-163. */
int gg_vis2ints(int uv_type, const void *uv, int64_t npts, int32_t oversample,
                int32_t *packed, void *stream);

/* Bin visibilities by uv tile of `tile` cells (the device replacement of the
 * reference's host sorts, grid.cu:467-475, and set_bookmarks).  On return
 * (device buffers):
 *   bookmarks[z] = first sorted position of tile z, z in [0, ntiles]
 *                  (ntiles = ceil(img_dim/tile)^2; set_bookmarks semantics)
 *   order[k]     = input index of the visibility at sorted position k
 * Visibilities whose footprint misses the grid are left out: bookmarks[ntiles]
 * is the number kept.  Within a tile, input order is kept when
 * opt->input_sorted is set; otherwise it is unspecified. */
int gg_bin(gg_context *ctx, const gg_options *opt, int uv_type, const void *uv,
           int64_t npts, int64_t img_dim, int64_t gcf_dim, int32_t *bookmarks,
           int32_t *order, void *stream);

/* ---- serving: continuous batching of gridding requests -----------------
 * A server owns `streams` batch slots (each a context with its own workspace
 * and CUDA stream) and a scheduler thread.  Requests are admitted in arrival
 * order while the HBM budget allows (grid + staged inputs + workspace share);
 * whenever a slot is free, every admitted request not yet started is
 * gridded in one batched launch there, so requests that arrive while others
 * are on the GPU overlap with them on the device.  Host inputs are copied in
 * on one server-wide input stream and grids copied out on one server-wide
 * output stream, ordered with the slot's kernels by events: a slot takes its
 * next batch as soon as its kernels finish, while earlier grids are still
 * being copied out.  Requests complete in launch order.  Latency = arrival
 * to grid ready (in host memory for host-bound requests). */
typedef struct gg_server gg_server;

#define GG_SERVER_TUNE_BATCHES 32
#define GG_REQ_INPUTS_ON_DEVICE 1 /* uv / vals are device pointers            */
#define GG_REQ_OUT_ON_DEVICE 2    /* out is a caller-owned device grid         */
#define GG_REQ_KEEP_RESIDENT 4    /* out unused: the grid stays on the device,
                                     owned by the server until release       */

typedef struct gg_server_config {
  int32_t device;
  int32_t streams;          /* batch slots in flight (default 2)            */
  int32_t max_batch_jobs;   /* per launch (default 256)                     */
  int32_t reserved0;
  int64_t max_batch_vis;    /* per launch (default 2^26)                    */
  int64_t hbm_budget_bytes; /* admission budget (default 150e9)             */
  gg_options options;       /* method, accumulation, ... of every request;
                               autotune 1 times trials only in the server's
                               first GG_SERVER_TUNE_BATCHES batches, later
                               batches run as autotune 2, so that no trial
                               lands on the latency path of a request
                               under load                                   */
  int64_t reserved[4];
} gg_server_config;

typedef struct gg_request {
  const void *uv;     /* host, or device with GG_REQ_INPUTS_ON_DEVICE        */
  const void *vals;
  void *out;          /* host grid (copied back), or a device grid with
                         GG_REQ_OUT_ON_DEVICE; layout as gg_grid_device     */
  int64_t npts, img_dim, gcf_dim;
  int32_t uv_type, vals_type, out_type;
  int32_t gcf_id;     /* table from gg_server_add_gcf; -1: options' GCF     */
  int32_t flags;      /* GG_REQ_*                                            */
  int32_t reserved0;
  int64_t reserved[3];
} gg_request;

/* device flag bits of a served batch (gg_result.device_flags) */
#define GG_DEVFLAG_INDEX 1    /* visibilities dropped: oversample or table
                                 index out of range (status stays GG_OK)   */
#define GG_DEVFLAG_TIMEOUT 2  /* a bounded device wait expired: the batch's
                                 requests fail with GG_ERR_TIMEOUT          */
#define GG_DEVFLAG_UNSORTED 4 /* input declared tile-sorted was not: the
                                 requests fail with GG_ERR_UNSORTED         */
#define GG_DEVFLAG_BOUNDS 8   /* an internal bounds check failed: the
                                 requests fail with GG_ERR_STATE            */

typedef struct gg_result {
  int32_t status;     /* GG_OK or GG_ERR_*                                  */
  int32_t device_flags; /* GG_DEVFLAG_* raised by the batch the request was
                         gridded in (the flags are per batch: a flag may come
                         from another request of the same batch)         */
  double latency_s;   /* arrival -> grid ready                              */
  double queue_s;     /* arrival -> launch                                  */
  void *device_out;   /* GG_REQ_KEEP_RESIDENT: the grid on the device       */
} gg_result;

typedef struct gg_server_stats {
  int64_t submitted, completed, failed, rejected, cancelled, batches;
  int64_t visibilities;      /* gridded by completed requests               */
  double span_s;             /* first arrival to last completion            */
  double p50_latency_s, p99_latency_s, mean_latency_s, mean_batch_jobs;
  int64_t hbm_in_use, hbm_peak;
} gg_server_stats;

int gg_server_default_config(gg_server_config *cfg);
int gg_server_create(gg_server **srv, const gg_server_config *cfg);
/* upload a GCF table once; requests refer to it by id */
int gg_server_add_gcf(gg_server *srv, const void *host_table, int32_t vals_type,
                      int64_t gcf_dim, int32_t *gcf_id);
/* non-blocking; GG_ERR_BUDGET if the request alone exceeds the budget */
int gg_server_submit(gg_server *srv, const gg_request *req, int64_t *ticket);
/* submits request i at (now + offsets_s[i]) from a server-side thread
 * (arrival traces, e.g. Poisson); tickets are assigned immediately */
int gg_server_submit_schedule(gg_server *srv, const gg_request *reqs,
                              const double *offsets_s, int64_t n,
                              int64_t *tickets);
/* GG_ERR_TIMEOUT when not complete within timeout_s (< 0: no limit) */
int gg_server_wait(gg_server *srv, int64_t ticket, double timeout_s,
                   gg_result *res);
/* forget a completed ticket, freeing its resident grid */
int gg_server_release(gg_server *srv, int64_t ticket);
/* cancel a request that has not been launched yet */
int gg_server_cancel(gg_server *srv, int64_t ticket);
int gg_server_get_stats(gg_server *srv, gg_server_stats *st, int reset);
/* wait until nothing is pending or in flight */
int gg_server_drain(gg_server *srv, double timeout_s);
int gg_server_destroy(gg_server *srv);

/* ---- allocation-free moving window -------------------------------------
 * No counterpart in the reference.  Grids one job like gg_grid_device with
 * the moving-window method, but every scratch buffer (tile histogram,
 * bookmarks, sorted visibilities, work queue, merge slots, counters) comes
 * from a fixed array compiled into libgg.so instead of an allocation.  It is
 * for callers that must not allocate device memory while they run: a
 * real-time ingest that reserves all of its GPU memory at start-up because
 * cudaMalloc can block on the device or fail mid-observation, or a plugin
 * inside a host framework that owns the device memory pool.  The caller
 * passes inputs and outputs (device pointers) as for gg_grid_device.
 * Limits, each rejected with GG_ERR_ARG: npts <= 262144; at most 16384 uv
 * tiles (img_dim <= 4096 at the default 32-cell tile); tile 0 (= 32) or a
 * power of two in 16..256; oversample a power of two in 1..64; one
 * polarisation; complex64 values; GCF TABLE of at most 65536 taps (G*G*S*S,
 * e.g. G 8 with S 32) or GAUSSIAN; no per-visibility tables (gcf_index).  The
 * array (12206336 bytes, 11.6 MiB) stays resident on every GPU that loads
 * libgg.so until the process exits.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current: make that first call
 * before any stream capture.  A call enqueues kernels and memsets only; it
 * reads no host memory on the stream and does not wait for it.  All calls
 * share the array and clear what must start at zero; calls that overlap on
 * the GPU (other streams or threads) race on it.  Device-side failures
 * (unsorted input declared sorted, an expired bounded wait, dropped
 * visibilities) are read with gg_read_flags(NULL, stream, flags) after the
 * call. */
int gg_grid_device_noalloc(const gg_options *opt, const gg_job *job,
                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GG_H */
