// Served path: continuous batching of independent structures under a device
// memory budget (gf_server_* in include/giraffe_gpu.h).
//
// One device allocation (the budget) backs every admitted batch through a
// first-fit arena, so admitting and retiring batches never calls cudaMalloc
// or cudaFree while other batches run.  Each batch ("wave") runs on its own
// stream from a fixed pool; its Newton passes are the batch path's captured
// pass graph, enqueued in chunks with a copy of the per-structure state and
// an event after each chunk.  Two chunks stay in flight per wave, so the
// device works while the host reads the older chunk's state.  A structure
// whose state reads DONE or ABORTED has its nodal result copied out on a
// separate stream (no kernel writes a finished structure's nodes again) into
// pinned staging, and is reported once that copy has landed; the wave's
// memory returns to the budget when its last structure is reported and no
// chunk of it is in flight.  Every host<->device copy of the served path
// goes through the pinned staging pool, because copies to or from pageable
// memory block the host until the device's other work lets them through,
// which stalls the polling loop behind long Shell_1 passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"

using namespace gf;
using namespace gfh;

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  gf_model_desc model;
  bool wide = false;  // Shell_1 structure (wide-band solver)
  double* out = nullptr;
  long long tag = 0;
  size_t bytes = 0;
  double t_submit = 0.0, t_admit = 0.0;
};

struct Wave {
  gf_batch* B = nullptr;
  int slot = -1;
  std::vector<Request> reqs;
  std::vector<char> reported;  // 0 running, 1 reported, 2 result copy pending
  int pending = 0;             // result copies not yet landed
  size_t reserved = 0;         // budget bytes set aside at admission
  int build_status = GF_OK;    // set by the builder thread
  std::string build_err;
  int inflight = 0;  // chunks enqueued and not yet read (0..2)
  int head = 0;      // buffer (0/1) of the oldest in-flight chunk
  bool finishing = false;
  long long passes = 0;
};

// Newton passes a wave may run before its unfinished structures are
// reported as timed out (the batch path's cap).
constexpr long long kMaxWavePasses = 4000000;  // default of max_wave_passes
// Slack added to each wave's size: the batch's own 256-byte roundings.
constexpr size_t kWaveSlack = 1 << 16;
// Pinned host staging shared by the uploads of new waves and the result
// copies; a copy that finds no room waits (results) or goes through
// pageable memory (uploads).
constexpr size_t kHostStage = (size_t)256 << 20;

// Handles of a retired Shell_1 wave kept until the device is idle:
// destroying an executable graph with conditional nodes waits for the
// device's other work, which would stall the polling loop behind the
// running waves.
struct Parked {
  cudaGraphExec_t graph = nullptr;
  cudaStream_t aux[GF_WB_STREAMS] = {};
  cudaEvent_t evt[GF_WB_EVENTS] = {};
};
// Parked handles beyond this many are destroyed at once, waiting or not.
constexpr size_t kMaxParked = 64;

// A finished structure's nodal result on its way to the caller: issued
// (host != nullptr) once staging room is free, reported when ev completes.
struct PendingResult {
  Wave* w = nullptr;
  int s = 0;
  StructState st{};
  char* host = nullptr;
  cudaEvent_t ev = nullptr;
};

}  // namespace

struct gf_server {
  gf_ctx* ctx = nullptr;
  gf_server_opts o{};
  void* arena_mem = nullptr;
  DevArena arena;
  std::vector<cudaStream_t> streams;  // one per wave slot
  std::vector<char> slot_busy;
  std::vector<cudaEvent_t> events;    // [slot][2]
  StructState* pin_state = nullptr;   // [slot][2][max_wave_structs], pinned
  int* pin_running = nullptr;         // [slot][2], pinned
  cudaStream_t copy_stream = nullptr;
  cudaStream_t capture_stream = nullptr;
  void* stage_mem = nullptr;  // pinned, kHostStage bytes
  DevArena stage;             // first-fit over stage_mem
  std::deque<PendingResult> pending;
  std::vector<Parked> parked;
  // Builder thread: builds admitted waves (batch build, uploads, graph
  // capture and instantiation, reset), so that the polling thread never
  // waits on them.  Instantiating a Shell_1 pass graph of thousands of
  // launches can take hundreds of milliseconds while other waves run.
  gf_ctx build_ctx;           // the builder's error text
  std::thread builder;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Wave*> jobs;     // admitted, to build
  std::vector<Wave*> built;   // built (or failed), to pick up
  bool stop = false;
  int building = 0;           // admitted waves not yet picked up (polling thread)
  size_t reserved = 0;        // their budget bytes (polling thread)
  std::deque<Request> queue;
  std::vector<Wave*> waves;
  std::deque<gf_server_result> done;
  long long passes = 0, launches = 0, reported = 0;
  int in_flight_structs = 0;
};

namespace {

// Slot kinds: with more than one slot, the upper third (at least one slot)
// takes Shell_1 waves and the rest beam waves.  A Shell_1 wave holds many
// plates at once (its LU kernels run them side by side) for seconds; beam
// waves are short and many.
bool slot_for_wide(const gf_server* S, int i) {
  int W = S->o.max_waves;
  return W > 1 && i >= W - std::max(1, W / 3);
}

StructState* state_buf(gf_server* S, int slot, int k) {
  return S->pin_state + ((size_t)slot * 2 + k) * S->o.max_wave_structs;
}

int* running_buf(gf_server* S, int slot, int k) { return S->pin_running + slot * 2 + k; }

void report(gf_server* S, Wave& w, int s, const StructState* st, int status) {
  const Request& r = w.reqs[s];
  gf_server_result res{};
  res.tag = r.tag;
  res.status = status;
  if (st) {
    res.stats.converged_steps = st->converged_number;
    res.stats.newton_iterations = st->total_it;
    res.stats.bisections = st->bisections;
    res.stats.aborted = st->phase == PH_ABORTED || st->aborted;
    res.stats.linear_solves = st->n_solves;
    res.stats.refine_sweeps = st->ir_sweeps;
    res.stats.fp64_fallbacks = st->ir_fallbacks;
  }
  double t = now_ms();
  res.queued_ms = r.t_admit - r.t_submit;
  res.total_ms = t - r.t_submit;
  S->done.push_back(res);
  w.reported[s] = 1;
  S->in_flight_structs--;
  S->reported++;
}

// Queues structure s's nodal result for copying out (its final state st).
void start_result(gf_server* S, Wave& w, int s, const StructState& st) {
  PendingResult p;
  p.w = &w;
  p.s = s;
  p.st = st;
  w.reported[s] = 2;
  w.pending++;
  S->pending.push_back(p);
}

// Issues the D->H copies of queued results while staging room lasts: the
// structure's nodes (position + rotation vector, 6 doubles each) and Q (9
// each) into pinned memory, then an event.
int issue_results(gf_server* S) {
  gf_ctx* ctx = S->ctx;
  for (PendingResult& p : S->pending) {
    if (p.host) continue;
    const StructInfo& inf = p.w->B->info[p.s];
    const size_t nn = (size_t)inf.n_nodes;
    if (!p.w->reqs[p.s].out || nn == 0) continue;  // nothing to copy; completed below
    char* h = static_cast<char*>(S->stage.alloc(sizeof(double) * 15 * nn));
    if (!h) break;  // keep arrival order: wait for room
    p.host = h;
    const Batch& b = p.w->B->b;
    double* hd = reinterpret_cast<double*>(h);
    GF_CK(cudaMemcpyAsync(hd, b.copy + (size_t)inf.node_off * 6, sizeof(double) * 6 * nn, cudaMemcpyDeviceToHost,
                          S->copy_stream));
    GF_CK(cudaMemcpyAsync(hd + 6 * nn, b.Qn + (size_t)inf.node_off * 9, sizeof(double) * 9 * nn,
                          cudaMemcpyDeviceToHost, S->copy_stream));
    GF_CK(cudaEventCreateWithFlags(&p.ev, cudaEventDisableTiming));
    GF_CK(cudaEventRecord(p.ev, S->copy_stream));
  }
  return GF_OK;
}

// Reports the results whose copies have landed (in order), interleaving
// them into the caller's arrays (15 doubles per node).
int complete_results(gf_server* S) {
  gf_ctx* ctx = S->ctx;
  while (!S->pending.empty()) {
    PendingResult& p = S->pending.front();
    Wave& w = *p.w;
    const Request& r = w.reqs[p.s];
    const size_t nn = (size_t)w.B->info[p.s].n_nodes;
    const bool copy = r.out && nn > 0;
    if (copy) {
      if (!p.host) break;
      cudaError_t q = cudaEventQuery(p.ev);
      if (q == cudaErrorNotReady) break;
      GF_CK(q);
      const double* x = reinterpret_cast<const double*>(p.host);
      const double* Q = x + 6 * nn;
      for (size_t i = 0; i < nn; ++i) {
        std::memcpy(r.out + 15 * i, x + 6 * i, 6 * sizeof(double));
        std::memcpy(r.out + 15 * i + 6, Q + 9 * i, 9 * sizeof(double));
      }
      S->stage.release(p.host);
      cudaEventDestroy(p.ev);
    }
    report(S, w, p.s, &p.st, GF_OK);
    w.pending--;
    S->pending.pop_front();
  }
  return GF_OK;
}

int enqueue_chunk(gf_server* S, Wave& w) {
  gf_ctx* ctx = S->ctx;
  cudaStream_t st = S->streams[w.slot];
  const int k = (w.head + w.inflight) & 1;
  const Batch& b = w.B->b;
  for (int p = 0; p < S->o.passes_per_chunk; ++p) {
    if (w.B->graph) {
      GF_CK(cudaGraphLaunch(w.B->graph, st));
    } else {
      launch_iteration(b, st);
      GF_CK(cudaGetLastError());
    }
  }
  GF_CK(cudaMemcpyAsync(running_buf(S, w.slot, k), b.running, sizeof(int), cudaMemcpyDeviceToHost, st));
  GF_CK(cudaMemcpyAsync(state_buf(S, w.slot, k), b.state, sizeof(StructState) * (size_t)b.n_struct,
                        cudaMemcpyDeviceToHost, st));
  GF_CK(cudaEventRecord(S->events[w.slot * 2 + k], st));
  w.inflight++;
  w.passes += S->o.passes_per_chunk;
  S->passes += S->o.passes_per_chunk;
  S->launches += (long long)S->o.passes_per_chunk * w.B->launches_per_pass;
  return GF_OK;
}

// Reads the oldest chunk if it has finished; reports structures that are done.
int read_chunk(gf_server* S, Wave& w, bool* progressed) {
  gf_ctx* ctx = S->ctx;
  *progressed = false;
  if (w.inflight == 0) return GF_OK;
  const int k = w.head;
  cudaError_t q = cudaEventQuery(S->events[w.slot * 2 + k]);
  if (q == cudaErrorNotReady) return GF_OK;
  GF_CK(q);
  const StructState* st = state_buf(S, w.slot, k);
  const int running = *running_buf(S, w.slot, k);
  for (int s = 0; s < (int)w.reqs.size(); ++s) {
    if (w.reported[s]) continue;
    if (st[s].phase == PH_DONE || st[s].phase == PH_ABORTED) start_result(S, w, s, st[s]);
  }
  w.head ^= 1;
  w.inflight--;
  if (running == 0) w.finishing = true;
  if (w.passes >= (S->o.max_wave_passes > 0 ? (long long)S->o.max_wave_passes : kMaxWavePasses)) {
    w.finishing = true;
    for (int s = 0; s < (int)w.reqs.size(); ++s)
      if (!w.reported[s]) report(S, w, s, &st[s], GF_ERR_TIMEOUT);
  }
  *progressed = true;
  return GF_OK;
}

void destroy_parked(Parked& p) {
  if (p.graph) cudaGraphExecDestroy(p.graph);
  for (auto& a : p.aux)
    if (a) cudaStreamDestroy(a);
  for (auto& e : p.evt)
    if (e) cudaEventDestroy(e);
}

// Destroys the parked handles (the device is idle, or too many wait).
void reap(gf_server* S) {
  for (Parked& p : S->parked) destroy_parked(p);
  S->parked.clear();
}

void retire(gf_server* S, size_t i) {
  Wave* w = S->waves[i];
  for (int s = 0; s < (int)w->reqs.size(); ++s)
    if (!w->reported[s]) report(S, *w, s, nullptr, GF_ERR_TIMEOUT);
  gf_batch* B = w->B;
  if (B->b.sh.loops_in_graph) {
    Parked p;
    std::swap(p.graph, B->graph);
    for (int k = 0; k < GF_WB_STREAMS; ++k) std::swap(p.aux[k], B->b.sh.aux[k]);
    for (int k = 0; k < GF_WB_EVENTS; ++k) std::swap(p.evt[k], B->b.sh.evt[k]);
    S->parked.push_back(p);
    if (S->parked.size() > kMaxParked) {
      destroy_parked(S->parked.front());
      S->parked.erase(S->parked.begin());
    }
  }
  gf_batch_destroy(B);  // returns its arena blocks
  S->slot_busy[w->slot] = 0;
  delete w;
  S->waves.erase(S->waves.begin() + (long)i);
}

// Forms one wave of one kind of structure, if a slot of that kind and the
// budget allow.  A wave holds structures of one kind (beam structures, or
// Shell_1 structures, whose pass is the long wide-band solve), taken in
// arrival order while they fit the free budget.
int admit_kind(gf_server* S, bool kind, bool* admitted) {
  gf_ctx* ctx = S->ctx;
  *admitted = false;
  bool any = false, wide_queued = false;
  for (const Request& r : S->queue) {
    any |= r.wide == kind;
    wide_queued |= r.wide;
  }
  if (!any) return GF_OK;
  // Shell_1 waves take the Shell_1 slots; beam waves take the beam slots,
  // and the Shell_1 slots too while no Shell_1 structure waits
  int slot = -1;
  for (int i = 0; i < S->o.max_waves && slot < 0; ++i) {
    if (S->slot_busy[i]) continue;
    bool ok = S->o.max_waves == 1 || (kind ? slot_for_wide(S, i) : (!slot_for_wide(S, i) || !wide_queued));
    if (ok) slot = i;
  }
  if (slot < 0) return GF_OK;
  const size_t used = S->arena.bytes_in_use() + S->reserved;
  const size_t free_bytes = used < S->arena.size ? S->arena.size - used : 0;
  size_t total = kWaveSlack;
  std::vector<int> pick;
  for (int i = 0; i < (int)S->queue.size() && (int)pick.size() < S->o.max_wave_structs; ++i) {
    const Request& r = S->queue[i];
    if (r.wide != kind) continue;
    if (total + r.bytes > free_bytes) break;
    total += r.bytes;
    pick.push_back(i);
  }
  const int take = (int)pick.size();
  if (take == 0) return GF_OK;
  Wave* w = new Wave();
  w->slot = slot;
  w->reserved = total;
  const double t = now_ms();
  for (int i : pick) {
    w->reqs.push_back(S->queue[i]);
    w->reqs.back().t_admit = t;
  }
  w->reported.assign(take, 0);
  for (int k = take - 1; k >= 0; --k) S->queue.erase(S->queue.begin() + pick[k]);
  S->slot_busy[slot] = 1;
  S->in_flight_structs += take;
  S->reserved += total;
  S->building++;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->jobs.push_back(w);
  }
  S->cv.notify_one();
  *admitted = true;
  return GF_OK;
}

// Builder thread: the device batch of one admitted wave, built and captured
// on the capture stream, reset on the wave's slot stream.
void build_wave(gf_server* S, Wave& w) {
  NvtxRange range("build wave");
  const int take = (int)w.reqs.size();
  std::vector<gf_model_desc> models(take);
  for (int i = 0; i < take; ++i) models[i] = w.reqs[i].model;
  gf_batch* B = new gf_batch();
  B->ctx = &S->build_ctx;
  gf_default_opts(&B->opts);
  B->opts.use_graph = 1;
  B->opts.precision = S->o.precision;
  B->arena = &S->arena;
  B->host_stage = &S->stage;
  B->stream = S->capture_stream;
  int r = build_batch(B, take, models.data());
  B->b.sh.loops_in_graph = 1;
  // the uploads must land before the staging blocks are reused
  if (cudaStreamSynchronize(S->capture_stream) != cudaSuccess && r == GF_OK) r = GF_ERR_CUDA;
  for (void* h : B->staged) S->stage.release(h);
  B->staged.clear();
  B->host_stage = nullptr;
  if (r == GF_OK) {
    B->launches_per_pass = count_launches_per_pass(B);
    r = ensure_graph(B);
  }
  if (r == GF_OK) {
    B->stream = S->streams[w.slot];
    r = batch_reset(B);
  }
  if (r != GF_OK) {
    w.build_err = S->build_ctx.err;
    gf_batch_destroy(B);
    w.build_status = r;
    return;
  }
  w.B = B;
}

void builder_main(gf_server* S) {
  cudaSetDevice(S->ctx->device);
  for (;;) {
    Wave* w = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv.wait(lk, [S] { return S->stop || !S->jobs.empty(); });
      if (S->stop) return;
      w = S->jobs.front();
      S->jobs.pop_front();
    }
    build_wave(S, *w);
    std::lock_guard<std::mutex> g(S->mu);
    S->built.push_back(w);
  }
}

// Takes over the waves the builder has finished: built ones start running;
// a failed one returns its structures to the head of the queue.  Running out
// of contiguous room is retried once a wave retires; with nothing running or
// building, the failure is the submitted structures' own and is returned.
int pickup(gf_server* S) {
  std::vector<Wave*> got;
  {
    std::lock_guard<std::mutex> g(S->mu);
    got.swap(S->built);
  }
  int r = GF_OK;
  for (Wave* w : got) {
    S->building--;
    S->reserved -= w->reserved;
    if (w->build_status == GF_OK) {
      w->B->ctx = S->ctx;
      S->waves.push_back(w);
      continue;
    }
    for (int k = (int)w->reqs.size() - 1; k >= 0; --k) S->queue.push_front(w->reqs[k]);
    S->slot_busy[w->slot] = 0;
    S->in_flight_structs -= (int)w->reqs.size();
    if (r == GF_OK && S->waves.empty() && S->building == 0) {
      S->ctx->err = w->build_err;
      r = w->build_status;
    }
    delete w;
  }
  return r;
}

int admit(gf_server* S, bool* admitted) {
  bool a = false, b = false;
  int r = admit_kind(S, false, &a);
  if (r == GF_OK) r = admit_kind(S, true, &b);
  *admitted = a || b;
  return r;
}

}  // namespace

extern "C" {

void gf_server_default_opts(gf_server_opts* o) {
  o->hbm_budget = (size_t)8 << 30;
  o->max_waves = 4;
  o->max_wave_structs = 128;
  o->passes_per_chunk = 4;
  o->max_wave_passes = 0;
  o->precision = GF_PREC_FP64;
}

gf_server* gf_server_create(gf_ctx* ctx, const gf_server_opts* opts) {
  if (!ctx) return nullptr;
  gf_server* S = new gf_server();
  S->ctx = ctx;
  if (opts) S->o = *opts; else gf_server_default_opts(&S->o);
  if (S->o.max_waves <= 0 || S->o.max_wave_structs <= 0 || S->o.passes_per_chunk <= 0 || S->o.hbm_budget == 0 ||
      (S->o.precision != GF_PREC_FP64 && S->o.precision != GF_PREC_MIXED)) {
    set_err(ctx, "gf_server_create: invalid options");
    delete S;
    return nullptr;
  }
  bool ok = cudaSetDevice(ctx->device) == cudaSuccess && cudaMalloc(&S->arena_mem, S->o.hbm_budget) == cudaSuccess;
  if (ok) S->arena.init(S->arena_mem, S->o.hbm_budget);
  const int W = S->o.max_waves;
  S->streams.assign(W, nullptr);
  S->slot_busy.assign(W, 0);
  S->events.assign(2 * W, nullptr);
  // beam waves run on high-priority streams, Shell_1 waves (long wide-band
  // passes) on low-priority ones, so chains keep their latency beside plates
  int prio_low = 0, prio_high = 0;
  if (ok) ok = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) == cudaSuccess;
  for (int i = 0; ok && i < W; ++i)
    ok = cudaStreamCreateWithPriority(&S->streams[i], cudaStreamNonBlocking,
                                      slot_for_wide(S, i) ? prio_low : prio_high) == cudaSuccess;
  for (int i = 0; ok && i < 2 * W; ++i)
    ok = cudaEventCreateWithFlags(&S->events[i], cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking) == cudaSuccess &&
       cudaStreamCreateWithFlags(&S->capture_stream, cudaStreamNonBlocking) == cudaSuccess &&
       cudaMallocHost(&S->pin_state, sizeof(StructState) * 2 * (size_t)W * S->o.max_wave_structs) == cudaSuccess &&
       cudaMallocHost(&S->pin_running, sizeof(int) * 2 * (size_t)W) == cudaSuccess &&
       cudaMallocHost(&S->stage_mem, kHostStage) == cudaSuccess;
  if (ok) S->stage.init(S->stage_mem, kHostStage);
  if (!ok) {
    set_err(ctx, "gf_server_create: device set-up failed (budget %zu bytes): %s", S->o.hbm_budget,
            cudaGetErrorString(cudaGetLastError()));
    gf_server_destroy(S);
    return nullptr;
  }
  S->build_ctx.device = ctx->device;
  S->build_ctx.stream = S->capture_stream;
  S->builder = std::thread(builder_main, S);
  return S;
}

void gf_server_destroy(gf_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  if (S->builder.joinable()) S->builder.join();
  for (Wave* w : S->jobs) delete w;
  S->jobs.clear();
  for (Wave* w : S->built) {
    if (w->B) gf_batch_destroy(w->B);
    delete w;
  }
  S->built.clear();
  for (cudaStream_t s : S->streams)
    if (s) cudaStreamSynchronize(s);
  if (S->copy_stream) cudaStreamSynchronize(S->copy_stream);
  for (PendingResult& p : S->pending)
    if (p.ev) cudaEventDestroy(p.ev);
  S->pending.clear();
  while (!S->waves.empty()) retire(S, S->waves.size() - 1);
  reap(S);
  for (cudaStream_t s : S->streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : S->events)
    if (e) cudaEventDestroy(e);
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  if (S->capture_stream) cudaStreamDestroy(S->capture_stream);
  if (S->pin_state) cudaFreeHost(S->pin_state);
  if (S->pin_running) cudaFreeHost(S->pin_running);
  if (S->stage_mem) cudaFreeHost(S->stage_mem);
  if (S->arena_mem) cudaFree(S->arena_mem);
  delete S;
}

int gf_server_submit(gf_server* S, const gf_model_desc* model, double* final_nodes, long long tag) {
  if (!S || !model) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  size_t bytes = 0;
  gf_solve_opts wo;  // the options the wave's batch is built with
  gf_default_opts(&wo);
  wo.precision = S->o.precision;
  int r = batch_device_bytes(ctx, 1, model, &wo, &bytes);
  if (r != GF_OK) return r;
  if (bytes + kWaveSlack > S->arena.size) {
    set_err(ctx, "gf_server_submit: structure needs %zu device bytes, the budget is %zu", bytes, S->arena.size);
    return GF_ERR_ARG;
  }
  Request q;
  q.model = *model;
  q.out = final_nodes;
  q.tag = tag;
  q.bytes = bytes;
  q.wide = model->n_shells > 0;
  q.t_submit = now_ms();
  S->queue.push_back(q);
  return GF_OK;
}

int gf_server_poll(gf_server* S, gf_server_result* results, int max_results, int* n_results) {
  if (!S) return GF_ERR_ARG;
  int r = pickup(S);
  if (r != GF_OK) return r;
  if ((r = complete_results(S)) != GF_OK) return r;
  // read finished chunks (every ready one), copy out finished structures,
  // retire waves whose structures are all reported
  for (size_t i = 0; i < S->waves.size(); ++i) {
    Wave& w = *S->waves[i];
    bool progressed = true;
    while (progressed && r == GF_OK) r = read_chunk(S, w, &progressed);
    if (r != GF_OK) return r;
  }
  if ((r = issue_results(S)) != GF_OK || (r = complete_results(S)) != GF_OK) return r;
  for (size_t i = 0; i < S->waves.size();) {
    Wave& w = *S->waves[i];
    if (w.finishing && w.inflight == 0 && w.pending == 0) {
      retire(S, i);
      continue;
    }
    ++i;
  }
  // admit what fits
  for (bool admitted = true; admitted;) {
    r = admit(S, &admitted);
    if (r != GF_OK) return r;
  }
  if ((r = pickup(S)) != GF_OK) return r;
  // keep two chunks in flight per running wave
  for (Wave* w : S->waves)
    while (!w->finishing && w->inflight < 2) {
      r = enqueue_chunk(S, *w);
      if (r != GF_OK) return r;
    }
  if (S->waves.empty() && S->building == 0 && !S->parked.empty()) reap(S);
  int n = 0;
  while (results && n < max_results && !S->done.empty()) {
    results[n++] = S->done.front();
    S->done.pop_front();
  }
  if (n_results) *n_results = n;
  return GF_OK;
}

int gf_server_get_status(const gf_server* S, gf_server_status* st) {
  if (!S || !st) return GF_ERR_ARG;
  std::memset(st, 0, sizeof(*st));
  st->queued = (int)S->queue.size();
  st->waves = (int)S->waves.size() + S->building;
  st->structures = S->in_flight_structs;
  st->budget_in_use = S->arena.bytes_in_use();
  st->passes = S->passes;
  st->launches = S->launches;
  st->reported = S->reported;
  return GF_OK;
}

}  // extern "C"
