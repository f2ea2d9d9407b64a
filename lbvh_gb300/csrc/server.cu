// Request server: device-resident BVHs, build / refit / trace requests served
// as they arrive by one dispatch thread and a pool of stream workers.
//
// Threads and ownership:
//   * submit() (any thread) appends to the inbox under the server mutex;
//   * the dispatch thread owns all scheduling state (per-scene queues,
//     resident scenes, the HBM account, worker assignment) and is the only
//     thread that changes it;
//   * a worker runs one job at a time on its own stream and context (copies,
//     launches through the public C ABI, then a context synchronize), touches
//     only the job and its own staging buffers, and hands the job back;
//   * a spill thread (own stream and context) copies evicted scenes to host
//     memory, in eviction order, and hands the dumps back the same way;
//   * wait_any() (any thread) takes finished requests from the done list.
// Device memory of resident scenes is allocated by the worker that builds
// it (stream-ordered) and freed by the dispatch thread on its own release
// stream once no running job reads it.
#include "../../include/lbvh_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

namespace {

constexpr size_t kTriBytes = 48, kRayBytes = 32, kHitBytes = 16, kNodeBytes = 32;

size_t
scene_bytes(size_t n)
{
  return 148 * n + (size_t(1) << 16); // triangles 48 + nodes 32 + traversal copy 64 + sorted codes 4, per triangle
}

struct Request
{
  uint64_t ticket = 0, seq = 0;
  int kind = 0;
  int64_t scene = 0;
  const float* data = nullptr;
  size_t rows = 0;
  void* hits = nullptr;
  double arrival = 0, start = 0;
};
using ReqPtr = std::shared_ptr<Request>;

struct BatchRef
{
  lbvh_batch* batch = nullptr;
  void* tris = nullptr;           // device triangles of all members (owned)
  std::vector<uint32_t> off;      // member offsets
  int members = 0;                // members still resident
};

struct Resident
{
  size_t n = 0, nbytes = 0;
  lbvh_bvh* bvh = nullptr;        // own tree, or nullptr for a batch member
  void* tris = nullptr;           // device triangles the own tree reads (owned)
  std::shared_ptr<BatchRef> batch;
  uint32_t index = 0;             // member index in the batch
  int busy = 0;                   // running jobs that read it
  uint64_t last_use = 0;          // LRU tick
  bool retired = false;           // out of residency, freed when busy drops to 0
};
using ResPtr = std::shared_ptr<Resident>;

// An evicted scene kept on the host: the raw dump of its tree.
struct Spilled
{
  size_t n = 0;                       // triangles
  std::vector<unsigned char> nodes;   // (n - 1) x 32-byte reference nodes
  std::vector<float> tris;            // n x 12 floats
  uint64_t last_use = 0;
  size_t bytes() const { return nodes.size() + 4 * tris.size(); }
};
using SpillPtr = std::shared_ptr<Spilled>;

struct Worker;

enum class JobKind
{
  build,
  batch_build,
  refit,
  trace,
  spill,  // copy an evicted scene to the host (the spill thread)
  reload  // load a spilled scene back onto the device
};

struct Job
{
  JobKind kind = JobKind::build;
  std::vector<ReqPtr> group;
  // prepared by the dispatcher
  std::vector<uint32_t> off;                    // batch build: member offsets; batched trace: ray offsets
  std::vector<std::pair<size_t, size_t>> spans; // trace: rows of each request in the launch
  std::vector<size_t> nbytes;                   // build: accounted bytes per request
  ResPtr res;                                   // refit / trace: the (first) scene read
  std::vector<ResPtr> used;                     // trace: every scene read, one per request
  size_t rays = 0;                              // trace: rays in the launch
  Worker* worker = nullptr;                     // the worker that runs it
  int64_t scene = 0;                            // spill / reload: the scene
  SpillPtr dump;                                // spill: filled; reload: read
  // results of the worker
  lbvh_bvh* bvh = nullptr;
  lbvh_batch* batch = nullptr;
  void* tris = nullptr;
  int status = LBVH_OK;
  std::string msg;
  double t_done = 0;
};
using JobPtr = std::shared_ptr<Job>;

struct Worker
{
  int index = 0;
  cudaStream_t stream = nullptr;
  lbvh_ctx* ctx = nullptr;
  std::thread thread;
  std::condition_variable cv;
  JobPtr job;                     // guarded by the server mutex
  bool quit = false;              // guarded by the server mutex
  bool busy = false;              // dispatch thread only
  void* rays = nullptr;           // device staging (worker only)
  size_t rays_cap = 0;
  void* hits = nullptr;
  size_t hits_cap = 0;
  std::atomic<uint32_t>* fail_allocs = nullptr; // the server's injected allocation failures
};

} // namespace

struct lbvh_server
{
  lbvh_server_config cfg{};
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_dispatch, cv_done;
  // guarded by mu
  std::vector<ReqPtr> inbox;
  std::vector<JobPtr> finished;
  std::deque<lbvh_request_done> done;
  std::vector<int64_t> resident_snapshot;
  uint64_t next_ticket = 1, next_seq = 0, submitted = 0, completed = 0;
  uint64_t coalesced = 0, evictions = 0, used_snapshot = 0;
  uint64_t spills = 0, reloads = 0, spilled_snapshot = 0, host_used_snapshot = 0;
  uint64_t cancelled = 0, expired = 0;
  std::deque<JobPtr> spill_jobs; // for the spill thread
  std::vector<uint64_t> cancels; // tickets to cancel if still queued
  bool dirty = false, stop = false;
  std::atomic<uint32_t> fail_allocs{ 0 }; // injected allocation failures still to come
  // dispatch thread only
  std::unordered_map<int64_t, std::deque<ReqPtr>> queues;
  std::unordered_map<int64_t, ResPtr> resident;
  std::unordered_set<int64_t> writing;
  std::vector<lbvh_request_done> outbox; // reports of this step
  std::unordered_map<int64_t, SpillPtr> spilled; // evicted scenes kept on the host
  std::unordered_set<int64_t> spilling;          // evictions being copied out
  size_t host_used = 0;
  uint64_t spill_inflight = 0;
  size_t used = 0;
  uint64_t tick = 0;
  cudaStream_t release_stream = nullptr;
  lbvh_ctx* release_ctx = nullptr;
  std::vector<std::unique_ptr<Worker>> workers;
  std::unique_ptr<Worker> spiller; // copies evicted scenes out, off the workers' streams
  std::thread dispatcher;

  double now() const
  {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// ---- completion ------------------------------------------------------------

// Queues a request's report; the dispatch thread publishes its reports after
// each step, once the state they describe (e.g. the resident set) is
// visible too.
void
complete(lbvh_server* s, const ReqPtr& r, int status, const std::string& msg, double t_done)
{
  lbvh_request_done d{};
  d.ticket = r->ticket;
  d.status = status;
  d.kind = r->kind;
  d.scene = r->scene;
  d.arrival = r->arrival;
  d.start = r->start;
  d.done = t_done;
  std::snprintf(d.message, sizeof(d.message), "%s", msg.c_str());
  s->outbox.push_back(d);
}

// ---- worker side -----------------------------------------------------------

bool
fail_job(Job& j, lbvh_ctx* ctx, int status, const char* what)
{
  j.status = status;
  j.msg = what;
  const char* m = ctx ? lbvh_ctx_last_error(ctx) : "";
  if (m && *m) {
    j.msg += ": ";
    j.msg += m;
  }
  return false;
}

bool
cuda_ok(Job& j, cudaError_t e, const char* what)
{
  if (e == cudaSuccess)
    return true;
  j.status = e == cudaErrorMemoryAllocation ? LBVH_ERR_OOM : LBVH_ERR_DEVICE;
  j.msg = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

// A worker's device allocation for request data. An injected failure
// (lbvh_server_inject_alloc_failures) is reported exactly as cudaMallocAsync
// reports an exhausted device.
cudaError_t
worker_malloc(Worker& w, void** p, size_t bytes)
{
  if (w.fail_allocs) {
    uint32_t k = w.fail_allocs->load();
    while (k > 0 && !w.fail_allocs->compare_exchange_weak(k, k - 1)) {
    }
    if (k > 0)
      return cudaErrorMemoryAllocation;
  }
  return cudaMallocAsync(p, bytes, w.stream);
}

#define W_CK(call, what)                                                                                               \
  do {                                                                                                                 \
    if (!cuda_ok(j, (call), what))                                                                                     \
      return false;                                                                                                    \
  } while (0)
#define W_LB(call, what)                                                                                               \
  do {                                                                                                                 \
    const int st_ = (call);                                                                                            \
    if (st_ != LBVH_OK)                                                                                                \
      return fail_job(j, w.ctx, st_, what);                                                                            \
  } while (0)

bool
grow(Job& j, Worker& w, void*& buf, size_t& cap, size_t bytes)
{
  if (bytes <= cap)
    return true;
  if (buf)
    W_CK(cudaFreeAsync(buf, w.stream), "staging free");
  buf = nullptr;
  cap = 0;
  const size_t want = std::max(bytes, size_t(1) << 20);
  W_CK(worker_malloc(w, &buf, want), "staging allocation");
  cap = want;
  return true;
}

bool
run_build(Worker& w, Job& j)
{
  const Request& r = *j.group[0];
  W_CK(worker_malloc(w, &j.tris, kTriBytes * r.rows), "triangle allocation");
  W_CK(cudaMemcpyAsync(j.tris, r.data, kTriBytes * r.rows, cudaMemcpyDefault, w.stream), "triangle upload");
  W_LB(lbvh_bvh_create(w.ctx, &j.bvh), "bvh create");
  W_LB(lbvh_build_triangles(w.ctx, static_cast<const float*>(j.tris), r.rows, 0, j.bvh), "build");
  // the traversal copy is made here, on this stream, so that traces on other
  // streams only ever read it
  W_LB(lbvh_bvh_prepare_trace(w.ctx, j.bvh), "prepare trace");
  return true;
}

bool
run_batch_build(Worker& w, Job& j)
{
  const size_t total = j.off.back();
  W_CK(worker_malloc(w, &j.tris, kTriBytes * total), "triangle allocation");
  for (size_t k = 0; k < j.group.size(); k++)
    W_CK(cudaMemcpyAsync(static_cast<char*>(j.tris) + kTriBytes * j.off[k], j.group[k]->data,
                         kTriBytes * j.group[k]->rows, cudaMemcpyDefault, w.stream),
         "triangle upload");
  W_LB(lbvh_batch_create(w.ctx, &j.batch), "batch create");
  W_LB(lbvh_batch_build_triangles(w.ctx, static_cast<const float*>(j.tris), total, j.off.data(), j.group.size(),
                                  j.batch),
       "batched build");
  W_LB(lbvh_batch_prepare_trace(w.ctx, j.batch), "prepare trace");
  return true;
}

bool
run_refit(Worker& w, Job& j)
{
  const Request& r = *j.group[0];
  lbvh_bvh* bvh = j.res->bvh;
  if (j.res->batch) { // a batch member first becomes its own tree (same nodes)
    const BatchRef& b = *j.res->batch;
    const uint32_t k = j.res->index;
    const size_t n = b.off[k + 1] - b.off[k];
    W_LB(lbvh_bvh_create(w.ctx, &j.bvh), "bvh create");
    void* nodes = nullptr;
    W_CK(worker_malloc(w, &nodes, kNodeBytes * (n - 1)), "node allocation");
    const float* mesh = reinterpret_cast<const float*>(static_cast<const char*>(b.tris) + kTriBytes * b.off[k]);
    int st = lbvh_batch_mesh_nodes(w.ctx, b.batch, k, nodes);
    if (st == LBVH_OK)
      st = lbvh_bvh_import_triangles(w.ctx, nodes, n - 1, mesh, j.bvh); // copies the nodes, checks the tree
    cudaFreeAsync(nodes, w.stream);
    W_LB(st, "batch member import");
    bvh = j.bvh;
  }
  W_CK(worker_malloc(w, &j.tris, kTriBytes * r.rows), "triangle allocation");
  W_CK(cudaMemcpyAsync(j.tris, r.data, kTriBytes * r.rows, cudaMemcpyDefault, w.stream), "triangle upload");
  W_LB(lbvh_refit_triangles(w.ctx, bvh, static_cast<const float*>(j.tris)), "refit");
  W_LB(lbvh_bvh_prepare_trace(w.ctx, bvh), "prepare trace");
  return true;
}

bool
run_trace(Worker& w, Job& j)
{
  const size_t m = j.rays;
  if (m == 0)
    return true;
  if (!grow(j, w, w.rays, w.rays_cap, kRayBytes * m) || !grow(j, w, w.hits, w.hits_cap, kHitBytes * m))
    return false;
  for (size_t k = 0; k < j.group.size(); k++) {
    const Request& r = *j.group[k];
    W_CK(cudaMemcpyAsync(static_cast<char*>(w.rays) + kRayBytes * j.spans[k].first, r.data, kRayBytes * r.rows,
                         cudaMemcpyDefault, w.stream),
         "ray upload");
  }
  const float* rays = static_cast<const float*>(w.rays);
  if (j.res->batch)
    W_LB(lbvh_batch_trace_triangles(w.ctx, j.res->batch->batch, rays, j.off.data(), m, w.hits), "batched trace");
  else
    W_LB(lbvh_trace_triangles(w.ctx, j.res->bvh, rays, m, w.hits), "trace");
  for (size_t k = 0; k < j.group.size(); k++) {
    const Request& r = *j.group[k];
    if (r.rows)
      W_CK(cudaMemcpyAsync(r.hits, static_cast<const char*>(w.hits) + kHitBytes * j.spans[k].first,
                           kHitBytes * r.rows, cudaMemcpyDefault, w.stream),
           "hit download");
  }
  return true;
}

bool
run_spill(Worker& w, Job& j)
{
  const Resident& r = *j.res;
  auto d = std::make_shared<Spilled>();
  d->n = r.n;
  d->nodes.resize(kNodeBytes * (r.n - 1));
  d->tris.resize(12 * r.n);
  if (r.batch) {
    const BatchRef& b = *r.batch;
    W_LB(lbvh_batch_mesh_nodes(w.ctx, b.batch, r.index, d->nodes.data()), "member node dump");
    W_CK(cudaMemcpyAsync(d->tris.data(), static_cast<const char*>(b.tris) + kTriBytes * b.off[r.index],
                         kTriBytes * r.n, cudaMemcpyDeviceToHost, w.stream),
         "member triangle dump");
  } else {
    W_LB(lbvh_bvh_nodes(w.ctx, r.bvh, d->nodes.data()), "node dump");
    W_LB(lbvh_bvh_primitives(w.ctx, r.bvh, d->tris.data()), "triangle dump");
  }
  j.dump = std::move(d);
  return true;
}

bool
run_reload(Worker& w, Job& j)
{
  const Spilled& d = *j.dump;
  W_LB(lbvh_bvh_create(w.ctx, &j.bvh), "bvh create");
  // host triangles are copied into memory the BVH owns; the tree is checked
  W_LB(lbvh_bvh_import_triangles(w.ctx, d.nodes.data(), d.n - 1, d.tris.data(), j.bvh), "reload");
  W_LB(lbvh_bvh_prepare_trace(w.ctx, j.bvh), "prepare trace");
  return true;
}

#undef W_CK
#undef W_LB

void
worker_loop(lbvh_server* s, Worker* w)
{
  cudaSetDevice(s->cfg.device);
  for (;;) {
    JobPtr job;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      w->cv.wait(lk, [&] { return w->job || w->quit; });
      if (!w->job)
        return;
      job = w->job;
    }
    Job& j = *job;
    bool ok = false;
    switch (j.kind) {
      case JobKind::build:
        ok = run_build(*w, j);
        break;
      case JobKind::batch_build:
        ok = run_batch_build(*w, j);
        break;
      case JobKind::refit:
        ok = run_refit(*w, j);
        break;
      case JobKind::trace:
        ok = run_trace(*w, j);
        break;
      case JobKind::spill:
        ok = run_spill(*w, j);
        break;
      case JobKind::reload:
        ok = run_reload(*w, j);
        break;
    }
    // waits for the stream and reads the context's device error word
    const int st = lbvh_ctx_synchronize(w->ctx);
    if (ok && st != LBVH_OK)
      fail_job(j, w->ctx, st, "device");
    j.t_done = s->now();
    std::lock_guard<std::mutex> lk(s->mu);
    w->job.reset();
    s->finished.push_back(job);
    s->dirty = true;
    s->cv_dispatch.notify_one();
  }
}

// The spill thread: takes spill jobs in order from the server's queue, on its
// own stream and context, and hands them back like a worker.
void
spill_loop(lbvh_server* s, Worker* w)
{
  cudaSetDevice(s->cfg.device);
  for (;;) {
    JobPtr job;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      w->cv.wait(lk, [&] { return !s->spill_jobs.empty() || w->quit; });
      if (s->spill_jobs.empty())
        return;
      job = s->spill_jobs.front();
      s->spill_jobs.pop_front();
    }
    bool ok = run_spill(*w, *job);
    const int st = lbvh_ctx_synchronize(w->ctx);
    if (ok && st != LBVH_OK)
      fail_job(*job, w->ctx, st, "device");
    job->t_done = s->now();
    std::lock_guard<std::mutex> lk(s->mu);
    s->finished.push_back(job);
    s->dirty = true;
    s->cv_dispatch.notify_one();
  }
}

// ---- dispatch side ---------------------------------------------------------

void
free_batch(lbvh_server* s, BatchRef& b)
{
  if (b.batch)
    lbvh_batch_destroy(s->release_ctx, b.batch);
  if (b.tris)
    cudaFreeAsync(b.tris, s->release_stream);
  b.batch = nullptr;
  b.tris = nullptr;
}

void
release(lbvh_server* s, Resident& r)
{
  s->used -= r.nbytes;
  if (r.batch) {
    if (--r.batch->members == 0)
      free_batch(s, *r.batch);
    r.batch.reset();
  } else {
    if (r.bvh)
      lbvh_bvh_destroy(s->release_ctx, r.bvh);
    if (r.tris)
      cudaFreeAsync(r.tris, s->release_stream);
    r.bvh = nullptr;
    r.tris = nullptr;
  }
}

// Takes a scene out of residency; its memory goes back once no running job
// reads it.
void
drop(lbvh_server* s, int64_t scene)
{
  auto it = s->resident.find(scene);
  if (it == s->resident.end())
    return;
  ResPtr r = it->second;
  s->resident.erase(it);
  r->retired = true;
  if (r->busy == 0)
    release(s, *r);
}

// Moves a resident scene out of the device budget towards the host: the
// spill thread copies its tree out, then its device memory is freed (no
// running job reads it: eviction picks idle scenes only).
void
start_spill(lbvh_server* s, int64_t scene)
{
  auto it = s->resident.find(scene);
  ResPtr r = it->second;
  s->resident.erase(it);
  s->used -= r->nbytes; // out of the budget now; its memory goes when the copy is done
  r->nbytes = 0;
  r->retired = true;
  s->spilling.insert(scene);
  s->spill_inflight++;
  auto job = std::make_shared<Job>();
  job->kind = JobKind::spill;
  job->res = r;
  job->scene = scene;
  std::lock_guard<std::mutex> lk(s->mu);
  s->spill_jobs.push_back(std::move(job));
  s->spiller->cv.notify_one();
}

void
evict(lbvh_server* s, int64_t scene)
{
  const ResPtr& r = s->resident.at(scene);
  const size_t dump = kNodeBytes * (r->n - 1) + kTriBytes * r->n;
  if (s->cfg.host_budget && dump <= s->cfg.host_budget)
    start_spill(s, scene);
  else
    drop(s, scene);
}

void
forget_spilled(lbvh_server* s, int64_t scene)
{
  auto it = s->spilled.find(scene);
  if (it == s->spilled.end())
    return;
  s->host_used -= it->second->bytes();
  s->spilled.erase(it);
}

bool
make_room(lbvh_server* s, size_t need, int64_t keep)
{
  if (s->used + need <= s->cfg.hbm_budget)
    return true;
  std::vector<std::pair<uint64_t, int64_t>> lru;
  for (auto& kv : s->resident)
    if (!kv.second->busy && kv.first != keep && !s->queues.count(kv.first) && !s->writing.count(kv.first))
      lru.emplace_back(kv.second->last_use, kv.first);
  std::sort(lru.begin(), lru.end());
  uint64_t evicted = 0;
  for (auto& e : lru) {
    if (s->used + need <= s->cfg.hbm_budget)
      break;
    evict(s, e.second);
    evicted++;
  }
  if (evicted) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->evictions += evicted;
  }
  return s->used + need <= s->cfg.hbm_budget;
}

bool
admissible(lbvh_server* s, const Request& r)
{
  if (s->writing.count(r.scene) || s->spilling.count(r.scene))
    return false;
  auto it = s->resident.find(r.scene);
  if (r.kind == LBVH_REQ_TRACE)
    return it != s->resident.end();
  if (r.kind == LBVH_REQ_REFIT)
    return it != s->resident.end() && it->second->busy == 0;
  return make_room(s, scene_bytes(r.rows), r.scene);
}

// Removes a group from the queues: for each scene it is a run from the front
// of that scene's queue, in queue order.
void
take(lbvh_server* s, const std::vector<ReqPtr>& group)
{
  const double t = s->now();
  for (const ReqPtr& r : group) {
    auto it = s->queues.find(r->scene);
    it->second.pop_front();
    if (it->second.empty())
      s->queues.erase(it);
    r->start = t;
  }
}

// `r` is a copy: the queue entry it came from is popped here.
void
reject(lbvh_server* s, ReqPtr r, int status, const std::string& msg)
{
  take(s, { r });
  complete(s, r, status, msg, s->now());
}

void
launch(lbvh_server* s, Worker* w, JobPtr job)
{
  w->busy = true;
  job->worker = w;
  std::lock_guard<std::mutex> lk(s->mu);
  w->job = std::move(job);
  w->cv.notify_one();
}

// Extends a group ending with the head of `scene`'s queue by the small traces
// queued right behind it (they read the same tree).
void
trace_run(lbvh_server* s, int64_t scene, std::vector<ReqPtr>& group)
{
  if (group.back()->rows > s->cfg.trace_batch_max_rays)
    return;
  const auto& q = s->queues[scene];
  for (size_t k = 1; k < q.size(); k++) {
    const ReqPtr& r = q[k];
    if (group.size() >= s->cfg.batch_max_requests || r->kind != LBVH_REQ_TRACE ||
        r->rows > s->cfg.trace_batch_max_rays)
      break;
    group.push_back(r);
  }
}

void
start_builds(lbvh_server* s, Worker* w, std::vector<ReqPtr> group)
{
  auto job = std::make_shared<Job>();
  job->kind = group.size() > 1 ? JobKind::batch_build : JobKind::build;
  job->off.push_back(0);
  for (const ReqPtr& r : group) {
    const size_t b = scene_bytes(r->rows);
    job->nbytes.push_back(b);
    job->off.push_back(uint32_t(job->off.back() + r->rows));
    s->used += b;
    s->writing.insert(r->scene);
  }
  if (group.size() > 1) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->coalesced += group.size();
  }
  job->group = std::move(group);
  launch(s, w, std::move(job));
}

void
start_refit(lbvh_server* s, Worker* w, const ReqPtr& r)
{
  auto job = std::make_shared<Job>();
  job->kind = JobKind::refit;
  job->group = { r };
  job->res = s->resident.at(r->scene);
  s->writing.insert(r->scene);
  launch(s, w, std::move(job));
}

// Loads a spilled scene back; its requests wait (the scene is "writing").
void
start_reload(lbvh_server* s, Worker* w, int64_t scene)
{
  auto job = std::make_shared<Job>();
  job->kind = JobKind::reload;
  job->scene = scene;
  job->dump = s->spilled.at(scene);
  s->used += scene_bytes(job->dump->n);
  s->writing.insert(scene);
  launch(s, w, std::move(job));
}

void
start_trace(lbvh_server* s, Worker* w, std::vector<ReqPtr> group)
{
  auto job = std::make_shared<Job>();
  job->kind = JobKind::trace;
  for (const ReqPtr& r : group) {
    ResPtr res = s->resident.at(r->scene);
    res->busy++;
    job->used.push_back(res);
  }
  job->res = job->used[0];
  job->spans.resize(group.size());
  if (!job->res->batch) { // traces of one tree, one after another
    size_t at = 0;
    for (size_t k = 0; k < group.size(); k++) {
      job->spans[k] = { at, at + group[k]->rows };
      at += group[k]->rows;
    }
    job->rays = at;
  } else { // rays grouped by member, in member order
    const size_t nm = job->res->batch->off.size() - 1;
    std::vector<size_t> per(nm + 1, 0);
    for (size_t k = 0; k < group.size(); k++)
      per[job->used[k]->index + 1] += group[k]->rows;
    for (size_t i = 0; i < nm; i++)
      per[i + 1] += per[i];
    job->off.assign(per.begin(), per.end());
    std::vector<size_t> cursor(per.begin(), per.end() - 1);
    for (size_t k = 0; k < group.size(); k++) {
      const uint32_t idx = job->used[k]->index;
      job->spans[k] = { cursor[idx], cursor[idx] + group[k]->rows };
      cursor[idx] += group[k]->rows;
    }
    job->rays = per[nm];
  }
  if (group.size() > 1) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->coalesced += group.size();
  }
  job->group = std::move(group);
  launch(s, w, std::move(job));
}

// Starts one job on a free worker; false when nothing could start.
bool
dispatch(lbvh_server* s)
{
  Worker* w = nullptr;
  for (auto& wp : s->workers)
    if (!wp->busy) {
      w = wp.get();
      break;
    }
  if (!w || s->queues.empty())
    return false;
  std::vector<std::pair<uint64_t, int64_t>> heads;
  heads.reserve(s->queues.size());
  for (auto& kv : s->queues)
    heads.emplace_back(kv.second.front()->seq, kv.first);
  std::sort(heads.begin(), heads.end());
  ReqPtr chosen;
  for (auto& h : heads) {
    const ReqPtr& r = s->queues[h.second].front();
    if (s->spilling.count(r->scene))
      continue; // its tree is being copied out; then it can be loaded back
    auto it = s->resident.find(r->scene);
    const bool known = it != s->resident.end() || s->writing.count(r->scene);
    if (r->kind != LBVH_REQ_BUILD && !known) {
      auto sp = s->spilled.find(r->scene);
      if (sp == s->spilled.end()) {
        reject(s, r, LBVH_ERR_NOT_RESIDENT, "scene " + std::to_string(r->scene) + " is not resident");
        return true;
      }
      if (make_room(s, scene_bytes(sp->second->n), r->scene)) {
        start_reload(s, w, r->scene);
        return true;
      }
      continue;
    }
    if (r->kind == LBVH_REQ_REFIT && it != s->resident.end() && !s->writing.count(r->scene) &&
        it->second->n != r->rows) {
      reject(s, r, LBVH_ERR_INVALID_ARG,
             "refit of scene " + std::to_string(r->scene) + " with " + std::to_string(r->rows) +
               " triangles; it was built with " + std::to_string(it->second->n));
      return true;
    }
    if (r->kind == LBVH_REQ_BUILD && r->rows < 2) {
      reject(s, r, LBVH_ERR_INVALID_ARG, "a build needs at least 2 triangles");
      return true;
    }
    if (admissible(s, *r)) {
      chosen = r;
      break;
    }
  }
  if (!chosen)
    return false;
  if (chosen->kind == LBVH_REQ_BUILD) {
    std::vector<ReqPtr> group{ chosen };
    if (chosen->rows <= s->cfg.batch_max_tris) {
      size_t total = chosen->rows, bytes = scene_bytes(chosen->rows);
      for (auto& h : heads) {
        if (group.size() >= s->cfg.batch_max_requests)
          break;
        const ReqPtr& r = s->queues[h.second].front();
        if (r == chosen || r->kind != LBVH_REQ_BUILD || r->rows < 2 || r->rows > s->cfg.batch_max_tris ||
            total + r->rows > LBVH_MAX_PRIMS || s->writing.count(r->scene) ||
            !make_room(s, bytes + scene_bytes(r->rows), r->scene)) // room for the whole group
          continue;
        total += r->rows;
        bytes += scene_bytes(r->rows);
        group.push_back(r);
      }
    }
    take(s, group);
    start_builds(s, w, std::move(group));
  } else if (chosen->kind == LBVH_REQ_REFIT) {
    take(s, { chosen });
    start_refit(s, w, chosen);
  } else {
    ResPtr res = s->resident.at(chosen->scene);
    std::vector<ReqPtr> group{ chosen };
    trace_run(s, chosen->scene, group);
    if (res->batch && chosen->rows <= s->cfg.trace_batch_max_rays) {
      for (auto& h : heads) {
        if (group.size() >= s->cfg.batch_max_requests)
          break;
        if (h.second == chosen->scene || s->writing.count(h.second))
          continue;
        auto it = s->resident.find(h.second);
        const ReqPtr& r = s->queues[h.second].front();
        if (it == s->resident.end() || it->second->batch != res->batch || r->kind != LBVH_REQ_TRACE ||
            r->rows > s->cfg.trace_batch_max_rays)
          continue;
        group.push_back(r);
        trace_run(s, h.second, group);
      }
    }
    take(s, group);
    start_trace(s, w, std::move(group));
  }
  return true;
}

void
free_job_outputs(lbvh_server* s, Job& j)
{
  if (j.bvh)
    lbvh_bvh_destroy(s->release_ctx, j.bvh);
  if (j.batch)
    lbvh_batch_destroy(s->release_ctx, j.batch);
  if (j.tris)
    cudaFreeAsync(j.tris, s->release_stream);
  j.bvh = nullptr;
  j.batch = nullptr;
  j.tris = nullptr;
}

// Applies a finished job to the scheduling state and reports its requests.
void
finish(lbvh_server* s, Job& j)
{
  const bool ok = j.status == LBVH_OK;
  switch (j.kind) {
    case JobKind::build:
    case JobKind::batch_build: {
      std::shared_ptr<BatchRef> ref;
      if (ok && j.kind == JobKind::batch_build) {
        ref = std::make_shared<BatchRef>();
        ref->batch = j.batch;
        ref->tris = j.tris;
        ref->off = j.off;
        ref->members = int(j.group.size());
      }
      for (size_t k = 0; k < j.group.size(); k++) {
        const ReqPtr& r = j.group[k];
        s->writing.erase(r->scene);
        if (!ok) {
          s->used -= j.nbytes[k];
          continue;
        }
        drop(s, r->scene); // the tree this build replaces
        forget_spilled(s, r->scene);
        auto res = std::make_shared<Resident>();
        res->n = r->rows;
        res->nbytes = j.nbytes[k];
        res->last_use = ++s->tick;
        if (ref) {
          res->batch = ref;
          res->index = uint32_t(k);
        } else {
          res->bvh = j.bvh;
          res->tris = j.tris;
        }
        s->resident[r->scene] = res;
      }
      if (!ok)
        free_job_outputs(s, j);
      break;
    }
    case JobKind::refit: {
      const ReqPtr& r = j.group[0];
      s->writing.erase(r->scene);
      ResPtr res = j.res;
      if (!ok) {
        free_job_outputs(s, j);
        drop(s, r->scene); // the tree may be half refitted
        break;
      }
      if (res->batch) { // the member leaves its batch for its own tree
        if (--res->batch->members == 0)
          free_batch(s, *res->batch);
        res->batch.reset();
        res->bvh = j.bvh;
      } else if (res->tris) {
        cudaFreeAsync(res->tris, s->release_stream); // the tree now reads the new triangles
      }
      res->tris = j.tris;
      res->last_use = ++s->tick;
      break;
    }
    case JobKind::spill: {
      s->spill_inflight--;
      s->spilling.erase(j.scene);
      release(s, *j.res); // the device copy goes (nothing of it was still counted)
      if (!ok || !j.dump)
        break; // the scene is gone, as a dropped one is
      const size_t b = j.dump->bytes();
      while (s->host_used + b > s->cfg.host_budget) { // drop the least recently used dumps
        auto lru = s->spilled.end();
        for (auto it = s->spilled.begin(); it != s->spilled.end(); ++it)
          if (!s->writing.count(it->first) && (lru == s->spilled.end() || it->second->last_use < lru->second->last_use))
            lru = it; // (a dump being loaded back stays)
        if (lru == s->spilled.end())
          break;
        forget_spilled(s, lru->first);
      }
      if (s->host_used + b <= s->cfg.host_budget) {
        j.dump->last_use = ++s->tick;
        s->spilled[j.scene] = j.dump;
        s->host_used += b;
        std::lock_guard<std::mutex> lk(s->mu);
        s->spills++;
      }
      break;
    }
    case JobKind::reload: {
      s->writing.erase(j.scene);
      const size_t nb = scene_bytes(j.dump->n);
      forget_spilled(s, j.scene);
      if (!ok) { // the dump did not load: the scene is gone
        s->used -= nb;
        free_job_outputs(s, j);
        break;
      }
      auto res = std::make_shared<Resident>();
      res->n = j.dump->n;
      res->nbytes = nb;
      res->bvh = j.bvh; // owns its triangles
      res->last_use = ++s->tick;
      s->resident[j.scene] = res;
      std::lock_guard<std::mutex> lk(s->mu);
      s->reloads++;
      break;
    }
    case JobKind::trace:
      for (const ResPtr& res : j.used) {
        res->busy--;
        res->last_use = ++s->tick;
        if (res->retired && res->busy == 0)
          release(s, *res);
      }
      break;
  }
  for (const ReqPtr& r : j.group)
    complete(s, r, j.status, j.msg, j.t_done);
}

bool
any_busy(const lbvh_server* s)
{
  if (s->spill_inflight)
    return true;
  for (const auto& w : s->workers)
    if (w->busy)
      return true;
  return false;
}

// Nothing runs and nothing waiting could start: the oldest waiting request
// never can (a build larger than what the budget frees).
void
unblock(lbvh_server* s)
{
  ReqPtr oldest;
  for (auto& kv : s->queues)
    if (!oldest || kv.second.front()->seq < oldest->seq)
      oldest = kv.second.front();
  if (oldest)
    reject(s, oldest, LBVH_ERR_BUDGET,
           "a build of " + std::to_string(oldest->rows) + " triangles does not fit the HBM budget of " +
             std::to_string(s->cfg.hbm_budget) + " bytes");
}

// Cancelled requests that have not started leave their queues and are
// reported; a ticket that is not queued (started, finished, unknown) is
// ignored.
void
cancel_queued(lbvh_server* s, const std::vector<uint64_t>& tickets)
{
  std::unordered_set<uint64_t> want(tickets.begin(), tickets.end());
  uint64_t k = 0;
  const double t = s->now();
  for (auto it = s->queues.begin(); it != s->queues.end();) {
    auto& q = it->second;
    for (auto r = q.begin(); r != q.end();) {
      if (want.count((*r)->ticket)) {
        complete(s, *r, LBVH_ERR_CANCELLED, "cancelled before it started", t);
        r = q.erase(r);
        k++;
      } else {
        ++r;
      }
    }
    it = q.empty() ? s->queues.erase(it) : std::next(it);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->cancelled += k;
}

// Requests still queued max_queue_s after their arrival fail. Queues are in
// arrival order, so only their fronts are looked at.
void
expire_queued(lbvh_server* s)
{
  if (s->cfg.max_queue_s <= 0)
    return;
  const double t = s->now();
  uint64_t k = 0;
  for (auto it = s->queues.begin(); it != s->queues.end();) {
    auto& q = it->second;
    while (!q.empty() && q.front()->arrival + s->cfg.max_queue_s <= t) {
      complete(s, q.front(), LBVH_ERR_EXPIRED,
               "not started within " + std::to_string(s->cfg.max_queue_s) + " s of its arrival", t);
      q.pop_front();
      k++;
    }
    it = q.empty() ? s->queues.erase(it) : std::next(it);
  }
  if (k) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->expired += k;
  }
}

// When the next queued request expires (server clock), or a negative value.
double
next_expiry(const lbvh_server* s)
{
  if (s->cfg.max_queue_s <= 0 || s->queues.empty())
    return -1.0;
  double t = -1.0;
  for (const auto& kv : s->queues) {
    const double e = kv.second.front()->arrival + s->cfg.max_queue_s;
    if (t < 0 || e < t)
      t = e;
  }
  return t;
}

void
dispatcher_loop(lbvh_server* s)
{
  cudaSetDevice(s->cfg.device);
  for (;;) {
    std::vector<ReqPtr> inbox;
    std::vector<JobPtr> fin;
    std::vector<uint64_t> cancels;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      while (!s->dirty) {
        if (s->stop && s->inbox.empty() && s->queues.empty() && !any_busy(s)) {
          for (auto& w : s->workers) {
            w->quit = true;
            w->cv.notify_one();
          }
          if (s->spiller) {
            s->spiller->quit = true;
            s->spiller->cv.notify_one();
          }
          return;
        }
        const double e = next_expiry(s); // queues are the dispatcher's own
        if (e < 0) {
          s->cv_dispatch.wait(lk);
        } else if (s->cv_dispatch.wait_for(lk, std::chrono::duration<double>(std::max(0.0, e - s->now()))) ==
                   std::cv_status::timeout) {
          s->dirty = true; // a queued request has expired
        }
      }
      s->dirty = false;
      inbox.swap(s->inbox);
      fin.swap(s->finished);
      cancels.swap(s->cancels);
    }
    for (ReqPtr& r : inbox)
      s->queues[r->scene].push_back(std::move(r));
    if (!cancels.empty())
      cancel_queued(s, cancels);
    expire_queued(s);
    for (JobPtr& j : fin) {
      if (j->worker) // spill jobs run on the spill thread
        j->worker->busy = false;
      finish(s, *j);
    }
    while (dispatch(s)) {
    }
    while (!s->queues.empty() && !any_busy(s))
      if (!dispatch(s))
        unblock(s);
    std::vector<int64_t> snap;
    snap.reserve(s->resident.size());
    for (auto& kv : s->resident)
      snap.push_back(kv.first);
    std::sort(snap.begin(), snap.end());
    std::lock_guard<std::mutex> lk(s->mu);
    s->resident_snapshot.swap(snap);
    s->used_snapshot = s->used;
    s->spilled_snapshot = s->spilled.size();
    s->host_used_snapshot = s->host_used;
    if (!s->outbox.empty()) {
      s->done.insert(s->done.end(), s->outbox.begin(), s->outbox.end());
      s->completed += s->outbox.size();
      s->outbox.clear();
      s->cv_done.notify_all();
    }
  }
}

void
destroy_all(lbvh_server* s)
{
  for (auto& w : s->workers) {
    if (w->thread.joinable())
      w->thread.join();
  }
  if (s->spiller && s->spiller->thread.joinable())
    s->spiller->thread.join();
  for (auto& kv : s->resident)
    release(s, *kv.second);
  s->resident.clear();
  s->spilled.clear();
  if (s->spiller) {
    if (s->spiller->ctx)
      lbvh_ctx_destroy(s->spiller->ctx);
    if (s->spiller->stream) {
      cudaStreamSynchronize(s->spiller->stream);
      cudaStreamDestroy(s->spiller->stream);
    }
  }
  for (auto& w : s->workers) {
    if (w->rays)
      cudaFreeAsync(w->rays, w->stream);
    if (w->hits)
      cudaFreeAsync(w->hits, w->stream);
    if (w->ctx)
      lbvh_ctx_destroy(w->ctx);
    if (w->stream) {
      cudaStreamSynchronize(w->stream);
      cudaStreamDestroy(w->stream);
    }
  }
  if (s->release_ctx)
    lbvh_ctx_destroy(s->release_ctx);
  if (s->release_stream) {
    cudaStreamSynchronize(s->release_stream);
    cudaStreamDestroy(s->release_stream);
  }
  delete s;
}

} // namespace

// ---- C ABI -------------------------------------------------------------------

extern "C" {

int
lbvh_server_create(const lbvh_server_config* cfg, lbvh_server** out)
{
  if (!cfg || !out)
    return LBVH_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->slots < 1 || cfg->slots > 64 || cfg->hbm_budget == 0 || !(cfg->max_queue_s >= 0))
    return LBVH_ERR_INVALID_ARG;
  if (cudaSetDevice(cfg->device) != cudaSuccess)
    return LBVH_ERR_DEVICE;
  lbvh_server* s = nullptr;
  try {
    s = new lbvh_server;
    s->cfg = *cfg;
    if (s->cfg.batch_max_requests < 1)
      s->cfg.batch_max_requests = 1;
    s->t0 = std::chrono::steady_clock::now();
    if (cudaStreamCreateWithFlags(&s->release_stream, cudaStreamNonBlocking) != cudaSuccess ||
        lbvh_ctx_create(cfg->device, s->release_stream, &s->release_ctx) != LBVH_OK) {
      destroy_all(s);
      return LBVH_ERR_DEVICE;
    }
    for (int k = 0; k < cfg->slots; k++) {
      auto w = std::make_unique<Worker>();
      w->index = k;
      w->fail_allocs = &s->fail_allocs;
      if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
          lbvh_ctx_create(cfg->device, w->stream, &w->ctx) != LBVH_OK) {
        s->workers.push_back(std::move(w));
        destroy_all(s);
        return LBVH_ERR_DEVICE;
      }
      // Workers build with the multi-kernel path only. The one-launch small
      // build is a thread-block cluster that needs up to 16 SMs, each with
      // about 162 KB of shared memory free, at the same moment; with the
      // other workers' kernels running on every SM it can wait long enough
      // to stall the whole request stream. The nodes are the same either way.
      if (lbvh_ctx_set_param(w->ctx, LBVH_PARAM_SMALL_BUILD_MAX, 0) != LBVH_OK) {
        s->workers.push_back(std::move(w));
        destroy_all(s);
        return LBVH_ERR_DEVICE;
      }
      s->workers.push_back(std::move(w));
    }
    {
      auto w = std::make_unique<Worker>();
      w->index = -1;
      const bool ok = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) == cudaSuccess &&
                      lbvh_ctx_create(cfg->device, w->stream, &w->ctx) == LBVH_OK;
      s->spiller = std::move(w);
      if (!ok) {
        destroy_all(s);
        return LBVH_ERR_DEVICE;
      }
    }
    for (auto& w : s->workers)
      w->thread = std::thread(worker_loop, s, w.get());
    s->spiller->thread = std::thread(spill_loop, s, s->spiller.get());
    s->dispatcher = std::thread(dispatcher_loop, s);
  } catch (...) { // thread or allocation failure
    if (s) {
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->dirty = true;
        for (auto& w : s->workers) {
          w->quit = true;
          w->cv.notify_one();
        }
        if (s->spiller) {
          s->spiller->quit = true;
          s->spiller->cv.notify_one();
        }
        s->cv_dispatch.notify_one();
      }
      if (s->dispatcher.joinable())
        s->dispatcher.join();
      destroy_all(s);
    }
    return LBVH_ERR_OOM;
  }
  *out = s;
  return LBVH_OK;
}

int
lbvh_server_submit(lbvh_server* s, int kind, int64_t scene, const float* data, size_t rows, void* hits,
                   uint64_t* ticket)
{
  if (!s || !ticket || kind < LBVH_REQ_BUILD || kind > LBVH_REQ_TRACE || (rows && !data) ||
      (kind == LBVH_REQ_TRACE && rows && !hits) || rows > LBVH_MAX_PRIMS)
    return LBVH_ERR_INVALID_ARG;
  auto r = std::make_shared<Request>();
  r->kind = kind;
  r->scene = scene;
  r->data = data;
  r->rows = rows;
  r->hits = hits;
  r->arrival = s->now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop)
    return LBVH_ERR_INVALID_ARG; // closed
  r->ticket = s->next_ticket++;
  r->seq = s->next_seq++;
  s->inbox.push_back(std::move(r));
  s->submitted++;
  s->dirty = true;
  s->cv_dispatch.notify_one();
  *ticket = s->next_ticket - 1;
  return LBVH_OK;
}

int
lbvh_server_cancel(lbvh_server* s, uint64_t ticket)
{
  if (!s)
    return LBVH_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->cancels.push_back(ticket);
  s->dirty = true;
  s->cv_dispatch.notify_one();
  return LBVH_OK;
}

int
lbvh_server_inject_alloc_failures(lbvh_server* s, uint32_t count)
{
  if (!s)
    return LBVH_ERR_INVALID_ARG;
  s->fail_allocs.store(count);
  return LBVH_OK;
}

int
lbvh_server_wait_any(lbvh_server* s, lbvh_request_done* out, size_t max, double timeout_s, size_t* n_out)
{
  if (!s || !out || !n_out || max == 0)
    return LBVH_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && timeout_s > 0)
    s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !s->done.empty(); });
  const size_t n = std::min(max, s->done.size());
  for (size_t k = 0; k < n; k++) {
    out[k] = s->done.front();
    s->done.pop_front();
  }
  *n_out = n;
  return LBVH_OK;
}

double
lbvh_server_clock(const lbvh_server* s)
{
  return s ? s->now() : 0.0;
}

int
lbvh_server_drain(lbvh_server* s)
{
  if (!s)
    return LBVH_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->completed == s->submitted; });
  return LBVH_OK;
}

int
lbvh_server_stats_get(lbvh_server* s, lbvh_server_stats* out)
{
  if (!s || !out)
    return LBVH_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->coalesced_requests = s->coalesced;
  out->evictions = s->evictions;
  out->resident_scenes = s->resident_snapshot.size();
  out->resident_bytes = s->used_snapshot;
  out->spills = s->spills;
  out->reloads = s->reloads;
  out->spilled_scenes = s->spilled_snapshot;
  out->spilled_bytes = s->host_used_snapshot;
  out->cancelled = s->cancelled;
  out->expired = s->expired;
  return LBVH_OK;
}

int
lbvh_server_resident(lbvh_server* s, int64_t* scenes, size_t cap, size_t* n_out)
{
  if (!s || !n_out || (cap && !scenes))
    return LBVH_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  const size_t n = std::min(cap, s->resident_snapshot.size());
  std::copy(s->resident_snapshot.begin(), s->resident_snapshot.begin() + n, scenes);
  *n_out = s->resident_snapshot.size();
  return LBVH_OK;
}

int
lbvh_server_destroy(lbvh_server* s)
{
  if (!s)
    return LBVH_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->dirty = true;
    s->cv_dispatch.notify_one();
  }
  if (s->dispatcher.joinable())
    s->dispatcher.join(); // finishes every queued request, then stops the workers
  destroy_all(s);
  return LBVH_OK;
}

} // extern "C"
