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
// separate stream (no kernel writes a finished structure's nodes again) and
// is reported at once; the wave's memory returns to the budget when its last
// structure is done and no chunk of it is in flight.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <deque>
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
  std::vector<char> reported;
  int inflight = 0;  // chunks enqueued and not yet read (0..2)
  int head = 0;      // buffer (0/1) of the oldest in-flight chunk
  bool finishing = false;
  long long passes = 0;
};

// Newton passes a wave may run before its unfinished structures are
// reported as timed out (the batch path's cap).
constexpr long long kMaxWavePasses = 4000000;
// Slack added to each wave's size: the batch's own 256-byte roundings.
constexpr size_t kWaveSlack = 1 << 16;

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
  std::deque<Request> queue;
  std::vector<Wave*> waves;
  std::deque<gf_server_result> done;
  long long passes = 0, launches = 0, reported = 0;
  int in_flight_structs = 0;
};

namespace {

// Slot kinds: with more than one slot, the upper half (at least one slot)
// takes Shell_1 waves and the rest beam waves.
bool slot_for_wide(const gf_server* S, int i) {
  int W = S->o.max_waves;
  return W > 1 && i >= W - W / 2;
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
    res.stats.fp64_fallback = st->fp64_fallback;
  }
  double t = now_ms();
  res.queued_ms = r.t_admit - r.t_submit;
  res.total_ms = t - r.t_submit;
  S->done.push_back(res);
  w.reported[s] = 1;
  S->in_flight_structs--;
  S->reported++;
}

// Copies structure s's final nodal state (position + rotation vector, then
// Q row-major: 15 doubles per node) into the caller's array.
int copy_result(gf_server* S, Wave& w, int s) {
  gf_ctx* ctx = S->ctx;
  const StructInfo& inf = w.B->info[s];
  double* out = w.reqs[s].out;
  if (!out || inf.n_nodes == 0) return GF_OK;
  const Batch& b = w.B->b;
  GF_CK(cudaMemcpy2DAsync(out, 15 * sizeof(double), b.copy + (size_t)inf.node_off * 6, 6 * sizeof(double),
                          6 * sizeof(double), (size_t)inf.n_nodes, cudaMemcpyDeviceToHost, S->copy_stream));
  GF_CK(cudaMemcpy2DAsync(out + 6, 15 * sizeof(double), b.Qn + (size_t)inf.node_off * 9, 9 * sizeof(double),
                          9 * sizeof(double), (size_t)inf.n_nodes, cudaMemcpyDeviceToHost, S->copy_stream));
  GF_CK(cudaStreamSynchronize(S->copy_stream));
  return GF_OK;
}

int enqueue_chunk(gf_server* S, Wave& w) {
  gf_ctx* ctx = S->ctx;
  cudaStream_t st = S->streams[w.slot];
  const int k = (w.head + w.inflight) & 1;
  const Batch& b = w.B->b;
  for (int p = 0; p < S->o.passes_per_chunk; ++p) GF_CK(cudaGraphLaunch(w.B->graph, st));
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
    if (st[s].phase == PH_DONE || st[s].phase == PH_ABORTED) {
      int r = copy_result(S, w, s);
      if (r != GF_OK) return r;
      report(S, w, s, &st[s], GF_OK);
    }
  }
  w.head ^= 1;
  w.inflight--;
  if (running == 0) w.finishing = true;
  if (w.passes > kMaxWavePasses) {
    w.finishing = true;
    for (int s = 0; s < (int)w.reqs.size(); ++s)
      if (!w.reported[s]) report(S, w, s, &st[s], GF_ERR_TIMEOUT);
  }
  *progressed = true;
  return GF_OK;
}

void retire(gf_server* S, size_t i) {
  Wave* w = S->waves[i];
  for (int s = 0; s < (int)w->reqs.size(); ++s)
    if (!w->reported[s]) report(S, *w, s, nullptr, GF_ERR_TIMEOUT);
  gf_batch_destroy(w->B);  // returns its arena blocks
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
  size_t free_bytes = S->arena.size - S->arena.in_use;
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
  for (int i : pick) w->reqs.push_back(S->queue[i]);
  w->reported.assign(take, 0);
  std::vector<gf_model_desc> models(take);
  double t = now_ms();
  for (int i = 0; i < take; ++i) {
    models[i] = w->reqs[i].model;
    w->reqs[i].t_admit = t;
  }
  gf_batch* B = new gf_batch();
  B->ctx = ctx;
  gf_default_opts(&B->opts);
  B->opts.use_graph = 1;
  B->arena = &S->arena;
  // build and capture on the idle capture stream, then run on the slot's
  B->stream = S->capture_stream;
  int r = build_batch(B, take, models.data());
  // the uploads must land before the blocks are reused or the wave runs
  if (cudaStreamSynchronize(S->capture_stream) != cudaSuccess && r == GF_OK) r = GF_ERR_CUDA;
  if (r == GF_OK) {
    B->launches_per_pass = count_launches_per_pass(B);
    r = ensure_graph(B);
  }
  if (r != GF_OK) {
    gf_batch_destroy(B);
    delete w;
    // out of contiguous room: leave the queue as it is and retry when a
    // wave retires; anything else is an error of the submitted structures
    return S->waves.empty() ? r : GF_OK;
  }
  B->stream = S->streams[slot];
  r = batch_reset(B);
  if (r != GF_OK) {
    gf_batch_destroy(B);
    delete w;
    return r;
  }
  w->B = B;
  for (int k = take - 1; k >= 0; --k) S->queue.erase(S->queue.begin() + pick[k]);
  S->slot_busy[slot] = 1;
  S->in_flight_structs += take;
  S->waves.push_back(w);
  *admitted = true;
  return GF_OK;
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
  o->pad = 0;
}

gf_server* gf_server_create(gf_ctx* ctx, const gf_server_opts* opts) {
  if (!ctx) return nullptr;
  gf_server* S = new gf_server();
  S->ctx = ctx;
  if (opts) S->o = *opts; else gf_server_default_opts(&S->o);
  if (S->o.max_waves <= 0 || S->o.max_wave_structs <= 0 || S->o.passes_per_chunk <= 0 || S->o.hbm_budget == 0) {
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
       cudaMallocHost(&S->pin_running, sizeof(int) * 2 * (size_t)W) == cudaSuccess;
  if (!ok) {
    set_err(ctx, "gf_server_create: device set-up failed (budget %zu bytes): %s", S->o.hbm_budget,
            cudaGetErrorString(cudaGetLastError()));
    gf_server_destroy(S);
    return nullptr;
  }
  return S;
}

void gf_server_destroy(gf_server* S) {
  if (!S) return;
  for (cudaStream_t s : S->streams)
    if (s) cudaStreamSynchronize(s);
  while (!S->waves.empty()) retire(S, S->waves.size() - 1);
  for (cudaStream_t s : S->streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : S->events)
    if (e) cudaEventDestroy(e);
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  if (S->capture_stream) cudaStreamDestroy(S->capture_stream);
  if (S->pin_state) cudaFreeHost(S->pin_state);
  if (S->pin_running) cudaFreeHost(S->pin_running);
  if (S->arena_mem) cudaFree(S->arena_mem);
  delete S;
}

int gf_server_submit(gf_server* S, const gf_model_desc* model, double* final_nodes, long long tag) {
  if (!S || !model) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  size_t bytes = 0;
  int r = gf_batch_device_bytes(ctx, 1, model, &bytes);
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
  int r = GF_OK;
  // read finished chunks (every ready one), retire finished waves
  for (size_t i = 0; i < S->waves.size();) {
    Wave& w = *S->waves[i];
    bool progressed = true;
    while (progressed && r == GF_OK) r = read_chunk(S, w, &progressed);
    if (r != GF_OK) return r;
    if (w.finishing && w.inflight == 0) {
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
  // keep two chunks in flight per running wave
  for (Wave* w : S->waves)
    while (!w->finishing && w->inflight < 2) {
      r = enqueue_chunk(S, *w);
      if (r != GF_OK) return r;
    }
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
  st->waves = (int)S->waves.size();
  st->structures = S->in_flight_structs;
  st->budget_in_use = S->arena.in_use;
  st->passes = S->passes;
  st->launches = S->launches;
  st->reported = S->reported;
  return GF_OK;
}

}  // extern "C"
