// Request server: admission by HBM budget and continuous batching of
// gridding requests over several CUDA streams (gg_server_* in gg.h).
//
// There is no counterpart in the reference, whose gridGPU serves one call at
// a time on the default stream.  Design:
//  * a scheduler thread owns `streams` slots; a slot = one gg_context (its
//    own workspace) + one CUDA stream.  Whenever a slot is free and requests
//    are pending, every pending request that fits the HBM budget (in arrival
//    order, up to the batch limits) is staged and gridded there in ONE
//    batched launch (gg_grid_batch: one binning pass and one persistent
//    window kernel per support over all of them);
//  * a batch is a three-stage pipeline: its input copies on the server's
//    input stream, its kernels on the slot's stream (waiting on an event),
//    its output copies and the read-back of its device flag words on the
//    server's output stream (waiting on an event behind the kernels).  The
//    slot takes its next batch as soon as the kernels finish, so host-bound
//    traffic keeps both directions of the host link busy;
//  * every batch in flight has its own device flag words (an entry of a
//    ring; the slot's context is pointed at it for the batch), so a slot's
//    next batch cannot clear flags not yet read back;
//  * staging uses stream-ordered allocation (cudaMallocAsync from the
//    device's memory pool) so that a batch allocates nothing synchronously;
//    inputs are freed behind the kernels, host-bound grids behind their
//    copies;
//  * host functions enqueued behind the kernels and behind the output stage
//    (cudaLaunchHostFunc) only flag the slot / the batch and wake the
//    scheduler, which frees slots, finishes requests in launch order,
//    returns their budget and wakes waiters;
//  * latency is measured from a request's arrival (its submit time, or its
//    scheduled time in a trace) to that completion.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gg_internal.h"

using gg::set_error;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { R_SCHEDULED = 0, R_PENDING, R_LAUNCHED, R_DONE, R_FAILED, R_CANCELLED };

struct Req {
  int64_t ticket = 0;
  gg_request r;
  double t_arrival = 0, t_launch = 0, t_done = 0;
  int state = R_SCHEDULED;
  int status = GG_OK;
  int device_flags = 0;       // GG_DEVFLAG_* of its batch
  int64_t bytes = 0;          // budget charged while admitted
  int64_t resident_bytes = 0; // part of `bytes` kept until release
  void *d_uv = nullptr, *d_vals = nullptr, *d_out = nullptr;
  bool own_uv = false, own_vals = false, own_out = false;
  cudaStream_t stream = nullptr;
};

// A slot = one gg_context (its own workspace) + one stream for the kernels
// of its current batch.  It is free again as soon as those kernels finish;
// the batch's output copies run on the server's output stream.
struct Slot {
  cudaStream_t s = nullptr;
  gg_context *ctx = nullptr;
  std::vector<Req *> batch;  // being admitted
  bool busy = false;         // its batch's kernels are queued or running
  bool free_again = false;   // set by the host function behind those kernels
  int64_t seq = 0;           // batches the server launched before this one
  struct gg_server *srv = nullptr;
};

// A batch from its launch until its requests complete (its output copies and
// the read-back of its device flag words have finished).
struct Batch {
  std::vector<Req *> reqs;
  int ring = -1;  // entry of the server's flag-word ring used by its kernels
  cudaEvent_t ev_in = nullptr, ev_compute = nullptr;
  int launch_status = GG_OK;
  bool done = false;  // set by the host function behind the output stage
  struct gg_server *srv = nullptr;
};

// flag-word ring: one entry (int32[64], the words a context's batched calls
// use) per batch in flight; the scheduler launches nothing while it is full
constexpr int kFlagRing = 1024;

int elem(int type) { return type == GG_C128 ? 16 : 8; }

}  // namespace

struct gg_server {
  gg_server_config cfg;
  Clock::time_point epoch;
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_feed;
  std::deque<Req *> pending;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  int64_t next_ticket = 1;
  int64_t used = 0, peak = 0;
  bool stop = false;
  std::vector<std::unique_ptr<Slot>> slots;
  // Pipeline: the input copies of every batch go on s_in, its kernels on its
  // slot's stream, its output copies on s_out, ordered by events.  One
  // stream per direction keeps each copy engine fed in launch order, and a
  // slot starts its next batch while earlier grids are still being copied
  // out (a slot kept until its copies end ran in lock-step with the others,
  // the output link idle 40 % of the time).
  cudaStream_t s_in = nullptr, s_out = nullptr;
  int *d_ring = nullptr;      // kFlagRing x 64 int32 (device)
  int32_t *h_ring = nullptr;  // kFlagRing x 4 int32 (pinned): words 0..3 read back
  std::vector<int> ring_free;
  std::vector<cudaEvent_t> ev_free;
  std::vector<std::unique_ptr<Batch>> inflight;  // launch order
  std::vector<void *> gcf_ptr;
  std::vector<int64_t> gcf_dim;
  std::vector<int> gcf_type;
  std::thread sched;
  // arrival-trace feeders; a finished one sets its flag and is joined by the
  // next gg_server_submit_schedule (or at destruction)
  struct Feeder {
    std::thread t;
    std::shared_ptr<std::atomic<bool>> finished;
  };
  std::vector<Feeder> feeders;
  std::mutex feeders_mu;  // guards `feeders` (client threads)
  int feeders_running = 0;
  int64_t n_launched = 0;  // batches launched since creation (not reset)
  // statistics
  int64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_rejected = 0,
          n_cancelled = 0, n_batches = 0, n_batch_jobs = 0, n_vis = 0;
  double first_arrival = -1, last_done = 0;
  std::vector<double> lat;

  double now() const {
    return std::chrono::duration<double>(Clock::now() - epoch).count();
  }
};

namespace {

// host functions (no CUDA calls): flag the event and wake the scheduler
void on_slot_free(void *p) {
  Slot *slot = static_cast<Slot *>(p);
  gg_server *srv = slot->srv;
  std::lock_guard<std::mutex> lk(srv->mu);
  slot->free_again = true;
  srv->cv_sched.notify_one();
}

void on_batch_done(void *p) {
  Batch *b = static_cast<Batch *>(p);
  gg_server *srv = b->srv;
  std::lock_guard<std::mutex> lk(srv->mu);
  b->done = true;
  srv->cv_sched.notify_one();
}

cudaEvent_t take_event(gg_server *srv) {
  if (!srv->ev_free.empty()) {
    cudaEvent_t e = srv->ev_free.back();
    srv->ev_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  return e;
}

// bytes a request holds on the device while admitted
int64_t estimate(const gg_server *srv, const gg_request &r) {
  const int64_t P = srv->cfg.options.polarizations;
  const int64_t N = r.img_dim, n = r.npts;
  const int64_t grid = (r.flags & GG_REQ_OUT_ON_DEVICE) ? 0 : elem(r.out_type) * P * N * N;
  const int64_t inputs =
      (r.flags & GG_REQ_INPUTS_ON_DEVICE) ? 0 : n * (elem(r.uv_type) + elem(r.vals_type) * P);
  const int64_t tiles = ((N + 15) / 16) * ((N + 15) / 16);
  int64_t ws = n * (8 + 4 + 8 + 4 + elem(r.vals_type) * P) + tiles * 16;
  // FP64 merge slots of tiles cut into several work items (compensated FP32
  // into a complex64 grid): at most one per 1025 records, each a sub-grid of
  // side T + S - 1 with tiles of up to 32 cells
  const gg_options &o = srv->cfg.options;
  if (o.accum == GG_ACC_COMPENSATED && r.vals_type == GG_C64 && r.out_type == GG_C64) {
    const int64_t R = 32 + r.gcf_dim - 1;
    ws += (n / 1025 + 1) * (R * R * 16 * P + 8);
  }
  return grid + inputs + ws + 4096;
}

int validate(const gg_server *srv, const gg_request &r) {
  if (r.npts < 0 || (r.npts > 0 && (!r.uv || !r.vals)))
    return set_error(GG_ERR_ARG, "server: request without inputs");
  if (r.img_dim < 1 || r.img_dim > 32768) return set_error(GG_ERR_ARG, "server: img_dim");
  if (r.gcf_dim != 4 && r.gcf_dim != 8 && r.gcf_dim != 16 && r.gcf_dim != 32)
    return set_error(GG_ERR_ARG, "server: gcf_dim not in {4,8,16,32}");
  if ((r.uv_type != GG_C64 && r.uv_type != GG_C128) ||
      (r.vals_type != GG_C64 && r.vals_type != GG_C128) ||
      (r.out_type != GG_C64 && r.out_type != GG_C128))
    return set_error(GG_ERR_ARG, "server: element type");
  if ((r.flags & GG_REQ_OUT_ON_DEVICE) && !r.out)
    return set_error(GG_ERR_ARG, "server: GG_REQ_OUT_ON_DEVICE without out");
  if (!(r.flags & (GG_REQ_OUT_ON_DEVICE | GG_REQ_KEEP_RESIDENT)) && !r.out)
    return set_error(GG_ERR_ARG, "server: no output (host out, device out or keep resident)");
  if (r.gcf_id >= 0) {
    if (r.gcf_id >= (int)srv->gcf_ptr.size())
      return set_error(GG_ERR_ARG, "server: unknown gcf_id");
    if (srv->gcf_dim[r.gcf_id] != r.gcf_dim || srv->gcf_type[r.gcf_id] != r.vals_type)
      return set_error(GG_ERR_ARG, "server: gcf_id does not match gcf_dim / vals_type");
  } else if (srv->cfg.options.gcf_kind == GG_GCF_TABLE) {
    return set_error(GG_ERR_ARG, "server: TABLE GCF needs a gcf_id");
  }
  return GG_OK;
}

void finish_batch(gg_server *srv, Batch *b) {
  const double t = srv->now();
  // device flags of the batch: a timeout, unsorted input or a failed bounds
  // check fails every request of the batch (its grids are incomplete);
  // dropped visibilities are reported and the requests succeed
  const int32_t *h = srv->h_ring + 4 * b->ring;
  const int bits = (h[gg::FLAG_INDEX] ? GG_DEVFLAG_INDEX : 0) |
                   (h[gg::FLAG_TIMEOUT] ? GG_DEVFLAG_TIMEOUT : 0) |
                   (h[gg::FLAG_UNSORTED] ? GG_DEVFLAG_UNSORTED : 0) |
                   (h[gg::FLAG_BOUNDS] ? GG_DEVFLAG_BOUNDS : 0);
  const int dev_status = h[gg::FLAG_TIMEOUT]    ? GG_ERR_TIMEOUT
                         : h[gg::FLAG_UNSORTED] ? GG_ERR_UNSORTED
                         : h[gg::FLAG_BOUNDS]   ? GG_ERR_STATE
                                                : GG_OK;
  for (Req *q : b->reqs) {
    q->device_flags = bits;
    if (q->state == R_LAUNCHED && q->status == GG_OK && dev_status != GG_OK) {
      q->status = dev_status;
      if (q->own_out && q->d_out) {  // a resident grid of a failed request
        cudaFreeAsync(q->d_out, srv->s_out);
        q->own_out = false;
        q->d_out = nullptr;
      }
    }
    if (q->state == R_LAUNCHED && q->status == GG_OK) {
      q->state = R_DONE;
      q->t_done = t;
      ++srv->n_completed;
      srv->n_vis += q->r.npts;
      srv->lat.push_back(t - q->t_arrival);
    } else {
      q->state = R_FAILED;
      q->t_done = t;
      q->resident_bytes = 0;  // a failed request keeps no grid
      ++srv->n_failed;
    }
    srv->used -= q->bytes - q->resident_bytes;
    q->bytes = q->resident_bytes;
  }
  srv->last_done = t;
  srv->ring_free.push_back(b->ring);
  if (b->ev_in) srv->ev_free.push_back(b->ev_in);
  if (b->ev_compute) srv->ev_free.push_back(b->ev_compute);
  srv->cv_done.notify_all();
}

// Stage and launch one batch on a slot (called without the lock): input
// copies on s_in, zeroing / binning / kernels on the slot's stream, output
// copies and the flag read-back on s_out.
void launch_batch(gg_server *srv, Slot *slot, Batch *b) {
  cudaSetDevice(srv->cfg.device);
  cudaStream_t s = slot->s, si = srv->s_in, so = srv->s_out;
  int *dflags = srv->d_ring + (size_t)64 * b->ring;
  std::vector<gg_job> jobs;
  jobs.reserve(b->reqs.size());
  int st = GG_OK;
  bool any_in = false;
  const int64_t P = srv->cfg.options.polarizations;
  for (Req *q : b->reqs) {
    const gg_request &r = q->r;
    q->stream = so;
    cudaError_t e = cudaSuccess;
    if (r.flags & GG_REQ_INPUTS_ON_DEVICE) {
      q->d_uv = const_cast<void *>(r.uv);
      q->d_vals = const_cast<void *>(r.vals);
    } else if (r.npts > 0) {
      const size_t bu = (size_t)r.npts * elem(r.uv_type);
      const size_t bv = (size_t)r.npts * elem(r.vals_type) * P;
      e = gg::injected_alloc_failure() ? cudaErrorMemoryAllocation
                                       : cudaMallocAsync(&q->d_uv, bu, si);
      if (e == cudaSuccess) {
        q->own_uv = true;
        e = cudaMallocAsync(&q->d_vals, bv, si);
      }
      if (e == cudaSuccess) {
        q->own_vals = true;
        any_in = true;
        e = cudaMemcpyAsync(q->d_uv, r.uv, bu, cudaMemcpyHostToDevice, si);
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(q->d_vals, r.vals, bv, cudaMemcpyHostToDevice, si);
    }
    if (e == cudaSuccess) {
      if (r.flags & GG_REQ_OUT_ON_DEVICE) {
        q->d_out = r.out;
      } else {
        e = gg::injected_alloc_failure()
                ? cudaErrorMemoryAllocation
                : cudaMallocAsync(&q->d_out, (size_t)elem(r.out_type) * P * r.img_dim * r.img_dim,
                                  s);
        if (e == cudaSuccess) q->own_out = true;
      }
    }
    if (e != cudaSuccess) {
      q->status = e == cudaErrorMemoryAllocation ? GG_ERR_NOMEM : GG_ERR_CUDA;
      st = q->status;
      break;
    }
    gg_job j;
    memset(&j, 0, sizeof j);
    j.out = q->d_out;
    j.uv = q->d_uv;
    j.vals = q->d_vals;
    j.gcf = r.gcf_id >= 0 ? srv->gcf_ptr[r.gcf_id] : nullptr;
    j.npts = r.npts;
    j.img_dim = r.img_dim;
    j.gcf_dim = r.gcf_dim;
    j.uv_type = r.uv_type;
    j.vals_type = r.vals_type;
    j.out_type = r.out_type;
    jobs.push_back(j);
  }
  if (any_in && (cudaEventRecord(b->ev_in, si) != cudaSuccess ||
                 cudaStreamWaitEvent(s, b->ev_in, 0) != cudaSuccess) &&
      st == GG_OK)
    st = GG_ERR_CUDA;
  // autotuner trials (which synchronise the slot's stream) only while the
  // server is young; afterwards the cached choices are reused
  gg_options opt = srv->cfg.options;
  if (opt.autotune == 1 && slot->seq >= GG_SERVER_TUNE_BATCHES) opt.autotune = 2;
  opt.accumulate = 0;  // every request gets a fresh grid
  if (st == GG_OK && cudaMemsetAsync(dflags, 0, 64 * sizeof(int), s) != cudaSuccess)
    st = GG_ERR_CUDA;
  if (st == GG_OK) {
    gg::context_set_batch_flags(slot->ctx, dflags);
    st = gg_grid_batch(slot->ctx, &opt, jobs.data(), (int32_t)jobs.size(), s);
    gg::context_set_batch_flags(slot->ctx, nullptr);
  }
  if (st == GG_OK) {
    if (const int inj = gg::injected_device_flags())
      if (gg::launch_inject_flags(dflags, inj, s) != cudaSuccess) st = GG_ERR_CUDA;
  }
  // inputs are read by this batch's kernels only
  for (Req *q : b->reqs) {
    if (q->own_uv) cudaFreeAsync(q->d_uv, s);
    if (q->own_vals) cudaFreeAsync(q->d_vals, s);
    q->own_uv = q->own_vals = false;
    q->d_uv = q->d_vals = nullptr;
  }
  if (cudaEventRecord(b->ev_compute, s) != cudaSuccess && st == GG_OK) st = GG_ERR_CUDA;
  if (cudaLaunchHostFunc(s, on_slot_free, slot) != cudaSuccess) {
    cudaStreamSynchronize(s);  // no callback: free the slot synchronously
    on_slot_free(slot);
  }
  // output stage, behind the kernels
  cudaStreamWaitEvent(so, b->ev_compute, 0);
  for (Req *q : b->reqs) {
    if (st != GG_OK && q->status == GG_OK) q->status = st;
    const gg_request &r = q->r;
    const bool host_out = !(r.flags & (GG_REQ_OUT_ON_DEVICE | GG_REQ_KEEP_RESIDENT));
    if (st == GG_OK && host_out && q->d_out)
      cudaMemcpyAsync(r.out, q->d_out, (size_t)elem(r.out_type) * P * r.img_dim * r.img_dim,
                      cudaMemcpyDeviceToHost, so);
    if (q->own_out && (host_out || st != GG_OK)) {
      cudaFreeAsync(q->d_out, so);
      q->own_out = false;
      q->d_out = nullptr;
    }
  }
  if (st == GG_OK && cudaMemcpyAsync(srv->h_ring + 4 * b->ring, dflags, 4 * sizeof(int32_t),
                                     cudaMemcpyDeviceToHost, so) != cudaSuccess) {
    st = GG_ERR_CUDA;
    for (Req *q : b->reqs)
      if (q->status == GG_OK) q->status = st;
  }
  b->launch_status = st;
  if (cudaLaunchHostFunc(so, on_batch_done, b) != cudaSuccess) {
    cudaStreamSynchronize(so);
    on_batch_done(b);
  }
}

void scheduler(gg_server *srv) {
  cudaSetDevice(srv->cfg.device);
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    for (auto &sl : srv->slots)
      if (sl->busy && sl->free_again) {
        sl->busy = false;
        sl->free_again = false;
      }
    // batches complete in launch order (one output stream)
    while (!srv->inflight.empty() && srv->inflight.front()->done) {
      finish_batch(srv, srv->inflight.front().get());
      srv->inflight.erase(srv->inflight.begin());
    }
    Slot *free_slot = nullptr;
    for (auto &sl : srv->slots)
      if (!sl->busy) {
        free_slot = sl.get();
        break;
      }
    if (free_slot && !srv->pending.empty() && !srv->ring_free.empty()) {
      // admit in arrival order while the budget and batch limits allow
      int64_t vis = 0;
      while (!srv->pending.empty() &&
             (int)free_slot->batch.size() < srv->cfg.max_batch_jobs) {
        Req *q = srv->pending.front();
        const int64_t b = estimate(srv, q->r);
        if (srv->used + b > srv->cfg.hbm_budget_bytes) break;
        if (!free_slot->batch.empty() && vis + q->r.npts > srv->cfg.max_batch_vis) break;
        srv->pending.pop_front();
        q->bytes = b;
        q->resident_bytes = (q->r.flags & GG_REQ_KEEP_RESIDENT)
                                ? (int64_t)elem(q->r.out_type) * srv->cfg.options.polarizations *
                                      q->r.img_dim * q->r.img_dim
                                : 0;
        srv->used += b;
        srv->peak = std::max(srv->peak, srv->used);
        q->state = R_LAUNCHED;
        q->t_launch = srv->now();
        vis += q->r.npts;
        free_slot->batch.push_back(q);
      }
      if (!free_slot->batch.empty()) {
        std::unique_ptr<Batch> nb(new Batch);
        Batch *b = nb.get();
        b->srv = srv;
        b->reqs.swap(free_slot->batch);
        b->ring = srv->ring_free.back();
        srv->ring_free.pop_back();
        for (int i = 0; i < 4; ++i) srv->h_ring[4 * b->ring + i] = 0;
        b->ev_in = take_event(srv);
        b->ev_compute = take_event(srv);
        srv->inflight.push_back(std::move(nb));
        free_slot->busy = true;
        free_slot->free_again = false;
        free_slot->seq = srv->n_launched++;
        ++srv->n_batches;
        srv->n_batch_jobs += (int64_t)b->reqs.size();
        if (!b->ev_in || !b->ev_compute) {
          // no events: fail the batch without launching anything
          for (Req *q : b->reqs) q->status = GG_ERR_CUDA;
          free_slot->busy = false;
          b->done = true;
          continue;
        }
        lk.unlock();
        launch_batch(srv, free_slot, b);
        lk.lock();
        continue;
      }
    }
    bool any_busy = !srv->inflight.empty();
    for (auto &sl : srv->slots) any_busy |= sl->busy;
    if (srv->stop && srv->pending.empty() && !any_busy && srv->feeders_running == 0) break;
    srv->cv_sched.wait(lk);
  }
}

void enqueue_locked(gg_server *srv, Req *q, double t_arrival) {
  q->t_arrival = t_arrival;
  q->state = R_PENDING;
  if (srv->first_arrival < 0 || t_arrival < srv->first_arrival) srv->first_arrival = t_arrival;
  srv->pending.push_back(q);
  srv->cv_sched.notify_one();
}

}  // namespace

extern "C" {

int gg_server_default_config(gg_server_config *cfg) {
  if (!cfg) return set_error(GG_ERR_ARG, "cfg: null");
  memset(cfg, 0, sizeof *cfg);
  cfg->device = 0;
  cfg->streams = 2;
  cfg->max_batch_jobs = 256;
  cfg->max_batch_vis = 1ll << 26;
  cfg->hbm_budget_bytes = 150000000000ll;
  gg_default_options(&cfg->options);
  cfg->options.mode = GG_MODE_WINDOW;
  cfg->options.accum = GG_ACC_COMPENSATED;
  cfg->options.layout = GG_LAYOUT_INTERLEAVED;
  return GG_OK;
}

int gg_server_create(gg_server **out, const gg_server_config *cfg) {
  if (!out || !cfg) return set_error(GG_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->streams < 1 || cfg->streams > 16) return set_error(GG_ERR_ARG, "streams 1..16");
  if (cfg->max_batch_jobs < 1 || cfg->max_batch_vis < 1 || cfg->hbm_budget_bytes < 1)
    return set_error(GG_ERR_ARG, "batch limits / budget must be positive");
  std::unique_ptr<gg_server> srv(new (std::nothrow) gg_server);
  if (!srv) return set_error(GG_ERR_NOMEM, "server allocation");
  srv->cfg = *cfg;
  srv->epoch = Clock::now();
  if (cudaSetDevice(cfg->device) != cudaSuccess) return set_error(GG_ERR_CUDA, "cudaSetDevice");
  // keep freed stream-ordered memory in the pool between batches
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, cfg->device) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  // everything made so far is released on a failure below
  auto undo = [&]() {
    for (auto &x : srv->slots) {
      gg_destroy(x->ctx);
      cudaStreamDestroy(x->s);
    }
    srv->slots.clear();
    if (srv->s_in) cudaStreamDestroy(srv->s_in);
    if (srv->s_out) cudaStreamDestroy(srv->s_out);
    if (srv->d_ring) cudaFree(srv->d_ring);
    if (srv->h_ring) cudaFreeHost(srv->h_ring);
  };
  for (int i = 0; i < cfg->streams; ++i) {
    std::unique_ptr<Slot> sl(new Slot);
    sl->srv = srv.get();
    int st = gg_create(&sl->ctx, cfg->device);
    if (st) {
      undo();
      return st;
    }
    if (cudaStreamCreateWithFlags(&sl->s, cudaStreamNonBlocking) != cudaSuccess) {
      gg_destroy(sl->ctx);
      undo();
      return set_error(GG_ERR_CUDA, "server: stream");
    }
    srv->slots.push_back(std::move(sl));
  }
  if (cudaStreamCreateWithFlags(&srv->s_in, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&srv->s_out, cudaStreamNonBlocking) != cudaSuccess) {
    undo();
    return set_error(GG_ERR_CUDA, "server: copy streams");
  }
  if (cudaMalloc(&srv->d_ring, sizeof(int) * 64 * kFlagRing) != cudaSuccess ||
      cudaMallocHost(&srv->h_ring, sizeof(int32_t) * 4 * kFlagRing) != cudaSuccess) {
    undo();
    return set_error(GG_ERR_NOMEM, "server: flag words");
  }
  for (int i = kFlagRing - 1; i >= 0; --i) srv->ring_free.push_back(i);
  gg_server *p = srv.release();
  p->sched = std::thread(scheduler, p);
  *out = p;
  return GG_OK;
}

int gg_server_add_gcf(gg_server *srv, const void *host_table, int32_t vals_type,
                      int64_t gcf_dim, int32_t *gcf_id) {
  if (!srv || !host_table || !gcf_id) return set_error(GG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  const int64_t G = srv->cfg.options.oversample;
  const size_t bytes = (size_t)elem(vals_type) * G * G * gcf_dim * gcf_dim;
  void *d = nullptr;
  cudaSetDevice(srv->cfg.device);
  if (cudaMalloc(&d, bytes) != cudaSuccess) return set_error(GG_ERR_NOMEM, "gcf table");
  if (cudaMemcpy(d, host_table, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return set_error(GG_ERR_CUDA, "gcf upload");
  }
  srv->gcf_ptr.push_back(d);
  srv->gcf_dim.push_back(gcf_dim);
  srv->gcf_type.push_back(vals_type);
  *gcf_id = (int32_t)srv->gcf_ptr.size() - 1;
  return GG_OK;
}

int gg_server_submit(gg_server *srv, const gg_request *req, int64_t *ticket) {
  if (!srv || !req || !ticket) return set_error(GG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->stop) return set_error(GG_ERR_STATE, "server is shutting down");
  int st = validate(srv, *req);
  if (st) return st;
  if (estimate(srv, *req) > srv->cfg.hbm_budget_bytes) {
    ++srv->n_rejected;
    return set_error(GG_ERR_BUDGET, "request larger than the server's HBM budget");
  }
  std::unique_ptr<Req> q(new Req);
  q->ticket = srv->next_ticket++;
  q->r = *req;
  Req *raw = q.get();
  srv->reqs[q->ticket] = std::move(q);
  ++srv->n_submitted;
  enqueue_locked(srv, raw, srv->now());
  *ticket = raw->ticket;
  return GG_OK;
}

int gg_server_submit_schedule(gg_server *srv, const gg_request *reqs,
                              const double *offsets_s, int64_t n, int64_t *tickets) {
  if (!srv || (n > 0 && (!reqs || !offsets_s || !tickets)))
    return set_error(GG_ERR_ARG, "null argument");
  std::vector<std::pair<double, Req *>> plan;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stop) return set_error(GG_ERR_STATE, "server is shutting down");
    const double t0 = srv->now();
    for (int64_t i = 0; i < n; ++i) {
      std::unique_ptr<Req> q(new Req);
      q->ticket = srv->next_ticket++;
      q->r = reqs[i];
      tickets[i] = q->ticket;
      int st = validate(srv, reqs[i]);
      if (!st && estimate(srv, reqs[i]) > srv->cfg.hbm_budget_bytes) {
        st = GG_ERR_BUDGET;
        ++srv->n_rejected;
      }
      ++srv->n_submitted;
      if (st) {
        q->state = R_FAILED;
        q->status = st;
        ++srv->n_failed;
      } else {
        plan.push_back({t0 + std::max(0.0, offsets_s[i]), q.get()});
      }
      srv->reqs[q->ticket] = std::move(q);
    }
    ++srv->feeders_running;
  }
  std::sort(plan.begin(), plan.end(),
            [](const std::pair<double, Req *> &a, const std::pair<double, Req *> &b) {
              return a.first < b.first;
            });
  // join the feeders of earlier traces that have finished
  std::lock_guard<std::mutex> flk(srv->feeders_mu);
  for (auto it = srv->feeders.begin(); it != srv->feeders.end();) {
    if (it->finished->load()) {
      it->t.join();
      it = srv->feeders.erase(it);
    } else {
      ++it;
    }
  }
  auto finished = std::make_shared<std::atomic<bool>>(false);
  std::thread feeder([srv, plan, finished]() {
    for (const auto &e : plan) {
      const auto when = srv->epoch + std::chrono::duration_cast<Clock::duration>(
                                         std::chrono::duration<double>(e.first));
      {
        // sleep to within ~100 us of the arrival (woken early on shutdown),
        // then spin for precision
        std::unique_lock<std::mutex> lk(srv->mu);
        srv->cv_feed.wait_until(lk, when - std::chrono::microseconds(100),
                                [srv] { return srv->stop; });
        if (srv->stop) break;
      }
      while (Clock::now() < when) {
      }
      std::lock_guard<std::mutex> lk(srv->mu);
      if (e.second->state == R_SCHEDULED) enqueue_locked(srv, e.second, e.first);
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    --srv->feeders_running;
    srv->cv_sched.notify_one();
    finished->store(true);
  });
  srv->feeders.push_back({std::move(feeder), finished});
  return GG_OK;
}

int gg_server_wait(gg_server *srv, int64_t ticket, double timeout_s, gg_result *res) {
  if (!srv) return set_error(GG_ERR_ARG, "server: null");
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->reqs.find(ticket);
  if (it == srv->reqs.end()) return set_error(GG_ERR_ARG, "unknown ticket");
  Req *q = it->second.get();
  auto finished = [q] { return q->state >= R_DONE; };
  if (timeout_s < 0) {
    srv->cv_done.wait(lk, finished);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
    return set_error(GG_ERR_TIMEOUT, "request not complete within the timeout");
  }
  if (res) {
    memset(res, 0, sizeof *res);
    res->status = q->state == R_CANCELLED ? GG_ERR_CANCELLED : q->status;
    res->device_flags = q->device_flags;
    res->latency_s = q->t_done - q->t_arrival;
    res->queue_s = q->t_launch > 0 ? q->t_launch - q->t_arrival : 0.0;
    res->device_out = (q->r.flags & GG_REQ_KEEP_RESIDENT) ? q->d_out : nullptr;
  }
  if (q->state == R_CANCELLED) return set_error(GG_ERR_CANCELLED, "request cancelled");
  if (q->status != GG_OK) return set_error(q->status, "request failed");
  return GG_OK;
}

int gg_server_release(gg_server *srv, int64_t ticket) {
  if (!srv) return set_error(GG_ERR_ARG, "server: null");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->reqs.find(ticket);
  if (it == srv->reqs.end()) return set_error(GG_ERR_ARG, "unknown ticket");
  Req *q = it->second.get();
  if (q->state < R_DONE) return set_error(GG_ERR_STATE, "request still in progress");
  if (q->own_out && q->d_out) {
    cudaSetDevice(srv->cfg.device);
    cudaFreeAsync(q->d_out, q->stream);
  }
  srv->used -= q->bytes;
  srv->reqs.erase(it);
  srv->cv_sched.notify_one();
  return GG_OK;
}

int gg_server_cancel(gg_server *srv, int64_t ticket) {
  if (!srv) return set_error(GG_ERR_ARG, "server: null");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->reqs.find(ticket);
  if (it == srv->reqs.end()) return set_error(GG_ERR_ARG, "unknown ticket");
  Req *q = it->second.get();
  if (q->state == R_PENDING) {
    srv->pending.erase(std::find(srv->pending.begin(), srv->pending.end(), q));
  } else if (q->state != R_SCHEDULED) {
    return set_error(GG_ERR_STATE, "request already launched or finished");
  }
  q->state = R_CANCELLED;
  q->t_done = srv->now();
  ++srv->n_cancelled;
  srv->cv_done.notify_all();
  return GG_OK;
}

int gg_server_get_stats(gg_server *srv, gg_server_stats *st, int reset) {
  if (!srv || !st) return set_error(GG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  memset(st, 0, sizeof *st);
  st->submitted = srv->n_submitted;
  st->completed = srv->n_completed;
  st->failed = srv->n_failed;
  st->rejected = srv->n_rejected;
  st->cancelled = srv->n_cancelled;
  st->batches = srv->n_batches;
  st->visibilities = srv->n_vis;
  st->span_s = srv->first_arrival >= 0 ? srv->last_done - srv->first_arrival : 0.0;
  st->mean_batch_jobs = srv->n_batches ? (double)srv->n_batch_jobs / srv->n_batches : 0.0;
  st->hbm_in_use = srv->used;
  st->hbm_peak = srv->peak;
  if (!srv->lat.empty()) {
    std::vector<double> v(srv->lat);
    auto pct = [&v](double q) {
      size_t k = (size_t)std::min<double>(v.size() - 1, std::max(0.0, q * (v.size() - 1) + 0.5));
      std::nth_element(v.begin(), v.begin() + k, v.end());
      return v[k];
    };
    st->p50_latency_s = pct(0.50);
    st->p99_latency_s = pct(0.99);
    double sum = 0;
    for (double x : srv->lat) sum += x;
    st->mean_latency_s = sum / srv->lat.size();
  }
  if (reset) {
    srv->n_submitted = srv->n_completed = srv->n_failed = srv->n_rejected = 0;
    srv->n_cancelled = srv->n_batches = srv->n_batch_jobs = srv->n_vis = 0;
    srv->first_arrival = -1;
    srv->last_done = 0;
    srv->lat.clear();
    srv->peak = srv->used;
  }
  return GG_OK;
}

int gg_server_drain(gg_server *srv, double timeout_s) {
  if (!srv) return set_error(GG_ERR_ARG, "server: null");
  std::unique_lock<std::mutex> lk(srv->mu);
  auto idle = [srv] {
    if (!srv->pending.empty() || srv->feeders_running || !srv->inflight.empty()) return false;
    for (auto &sl : srv->slots)
      if (sl->busy) return false;
    return true;
  };
  if (timeout_s < 0) {
    srv->cv_done.wait(lk, idle);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), idle)) {
    return set_error(GG_ERR_TIMEOUT, "server still busy after the timeout");
  }
  return GG_OK;
}

int gg_server_destroy(gg_server *srv) {
  if (!srv) return GG_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
    // requests whose arrival time has not come are dropped
    for (auto &kv : srv->reqs)
      if (kv.second->state == R_SCHEDULED) kv.second->state = R_CANCELLED;
    srv->cv_sched.notify_all();
    srv->cv_feed.notify_all();
  }
  {
    std::lock_guard<std::mutex> flk(srv->feeders_mu);
    for (auto &f : srv->feeders) f.t.join();
  }
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->cv_sched.notify_all();
  }
  srv->sched.join();
  cudaSetDevice(srv->cfg.device);
  for (auto &sl : srv->slots) cudaStreamSynchronize(sl->s);
  cudaStreamSynchronize(srv->s_in);
  cudaStreamSynchronize(srv->s_out);
  for (auto &kv : srv->reqs)
    if (kv.second->own_out && kv.second->d_out) cudaFree(kv.second->d_out);
  cudaDeviceSynchronize();
  for (auto &sl : srv->slots) {
    gg_destroy(sl->ctx);
    cudaStreamDestroy(sl->s);
  }
  cudaStreamDestroy(srv->s_in);
  cudaStreamDestroy(srv->s_out);
  cudaFree(srv->d_ring);
  cudaFreeHost(srv->h_ring);
  for (cudaEvent_t e : srv->ev_free) cudaEventDestroy(e);
  for (auto &b : srv->inflight) {
    if (b->ev_in) cudaEventDestroy(b->ev_in);
    if (b->ev_compute) cudaEventDestroy(b->ev_compute);
  }
  for (void *p : srv->gcf_ptr) cudaFree(p);
  delete srv;
  return GG_OK;
}

}  // extern "C"
