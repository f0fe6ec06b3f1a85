// server.cpp -- request serving over a scene pool with continuous batching.
//
// Requests are ray queries (scene id + host ray buffer) and scene uploads.
// Three host threads:
//   dispatcher  forms a batch from the pending ray queries in arrival order as
//               staging memory allows, uploads their rays, traces the batch in
//               one pool launch and downloads the hits, all on one of
//               `max_inflight` streams, so a new batch is formed and launched
//               while earlier ones still run on the device;
//   completer   retires batches in launch order when their event fires, frees
//               their staging and wakes the requests' waiters;
//   uploader    builds and admits new scenes against the pool's byte budget,
//               evicting least-recently-used idle scenes when needed.
// No thread ever waits on the GPU without a deadline it can give up on except
// the completer's event waits, which end when the device work ends.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "rt_internal.h"

namespace rtgb {
void set_error(const std::string& msg);
}

using Clock = std::chrono::steady_clock;

namespace {

enum Kind { kRays = 0, kUpload = 1 };
enum State { kPending = 0, kRunning = 1, kDone = 2 };

struct Request {
  uint64_t id = 0;
  Kind kind = kRays;
  uint32_t scene = 0;
  const RtRay* h_rays = nullptr;
  RtHit* h_hits = nullptr;
  uint32_t n = 0;
  uint32_t flags = 0;
  RtSceneDesc desc{};
  Clock::time_point submit, start, done;
  State state = kPending;
  rt_status status = RT_OK;
  uint32_t result_scene = 0;
  uint64_t stage_off = 0;
  uint32_t batch_jobs = 0;
};

struct Batch {
  std::vector<Request*> reqs;
  int stream = 0;
  cudaEvent_t done = nullptr;
};

// Server scene ids are never reused (an evicted scene's id stays dead), and
// map to the pool's ids, which are.
struct SceneRec {
  bool live = false;
  uint32_t pool_id = 0;
  uint32_t refs = 0;  // pending + running ray requests
  uint64_t last_use = 0;
  uint32_t triangles = 0;
};

// First-fit ranges of staging rays.
struct StageAlloc {
  std::map<uint64_t, uint64_t> free_;
  explicit StageAlloc(uint64_t cap = 0) {
    if (cap) free_[0] = cap;
  }
  bool alloc(uint64_t n, uint64_t* off) {
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= n) {
        *off = it->first;
        const uint64_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    return false;
  }
  void release(uint64_t off, uint64_t n) {
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

}  // namespace

struct rt_server {
  RtServerOptions opt{};
  rt_pool* pool = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_upload, cv_inflight;
  bool stop = false;
  uint64_t next_id = 1;
  uint64_t use_clock = 0;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::deque<Request*> pending;  // ray queries, arrival order
  std::deque<Request*> uploads;
  std::deque<Batch*> inflight;  // launched batches, in launch order
  uint32_t launched = 0;         // batches launched and not yet retired
  uint64_t stage_gen = 0;        // bumps whenever staging is released
  std::vector<SceneRec> scenes;
  // staging: rays then hits, capacity `stage_rays`
  RtRay* d_rays = nullptr;
  RtHit* d_hits = nullptr;
  StageAlloc stage;
  std::vector<cudaStream_t> streams;
  int next_stream = 0;
  std::thread dispatcher, completer, uploader;
  int device = 0;
  RtServerStats stats{};
};

namespace {

void finish_locked(rt_server* S, Request* r, rt_status st) {
  r->status = st;
  r->state = kDone;
  r->done = Clock::now();
  if (r->kind == kRays) {
    if (r->scene < S->scenes.size() && S->scenes[r->scene].refs) S->scenes[r->scene].refs--;
    S->stats.requests_done++;
    if (st == RT_OK) S->stats.rays_done += r->n;
  } else {
    S->stats.uploads_done++;
  }
}

void dispatch_loop(rt_server* S) {
  cudaSetDevice(S->device);
  std::vector<RtJob> jobs;
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_work.wait(lk, [&] {
      return S->stop || (!S->pending.empty() && S->launched < S->opt.max_inflight);
    });
    if (S->stop) return;
    // Take queries in arrival order while staging and the batch limits allow.
    std::unique_ptr<Batch> b(new Batch());
    uint64_t rays = 0;
    const uint32_t flags = S->pending.front()->flags;
    while (!S->pending.empty()) {
      Request* r = S->pending.front();
      if (r->flags != flags) break;
      if (!b->reqs.empty() && (rays + r->n > S->opt.max_batch_rays || b->reqs.size() >= S->opt.max_batch_jobs)) break;
      uint64_t off = 0;
      if (!S->stage.alloc(r->n ? r->n : 1, &off)) break;
      r->stage_off = off;
      r->state = kRunning;
      r->start = Clock::now();
      S->pending.pop_front();
      b->reqs.push_back(r);
      rays += r->n;
    }
    if (b->reqs.empty()) {  // staging full: wait until a retired batch frees some
      const uint64_t gen = S->stage_gen;
      S->cv_work.wait(lk, [&] { return S->stop || S->stage_gen != gen; });
      continue;
    }
    b->stream = S->next_stream;
    S->next_stream = (S->next_stream + 1) % (int)S->streams.size();
    cudaStream_t st = S->streams[b->stream];
    jobs.clear();
    for (Request* r : b->reqs) {
      r->batch_jobs = (uint32_t)b->reqs.size();
      jobs.push_back(RtJob{S->scenes[r->scene].pool_id, r->n, S->d_rays + r->stage_off, S->d_hits + r->stage_off});
      S->scenes[r->scene].last_use = ++S->use_clock;
    }
    S->launched++;
    S->stats.batches++;
    lk.unlock();
    rtgb::NvtxRange nvtx_range("rt_server batch");
    cudaError_t e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    for (Request* r : b->reqs)
      if (r->n && e == cudaSuccess)
        e = cudaMemcpyAsync(S->d_rays + r->stage_off, r->h_rays, (size_t)r->n * sizeof(RtRay),
                            cudaMemcpyHostToDevice, st);
    rt_status ts = e == cudaSuccess ? rt_pool_trace(S->pool, jobs.data(), (uint32_t)jobs.size(), flags, st) : RT_ECUDA;
    for (Request* r : b->reqs)
      if (r->n && e == cudaSuccess)
        e = cudaMemcpyAsync(r->h_hits, S->d_hits + r->stage_off, (size_t)r->n * sizeof(RtHit),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->done, st);
    lk.lock();
    if (e != cudaSuccess || ts != RT_OK)
      for (Request* r : b->reqs) r->status = ts != RT_OK ? ts : RT_ECUDA;
    S->inflight.push_back(b.release());  // its event is recorded: the completer may wait on it
    S->cv_inflight.notify_all();
  }
}

void complete_loop(rt_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_inflight.wait(lk, [&] { return !S->inflight.empty() || (S->stop && S->inflight.empty()); });
    if (S->inflight.empty()) {
      if (S->stop) return;
      continue;
    }
    Batch* b = S->inflight.front();
    lk.unlock();
    cudaError_t e = b->done ? cudaEventSynchronize(b->done) : cudaErrorInvalidResourceHandle;
    lk.lock();
    S->inflight.pop_front();
    S->launched--;
    S->stage_gen++;
    for (Request* r : b->reqs) {
      S->stage.release(r->stage_off, r->n ? r->n : 1);
      rt_status st = r->status;
      if (st == RT_OK && e != cudaSuccess) st = RT_ECUDA;
      finish_locked(S, r, st);
    }
    if (b->done) cudaEventDestroy(b->done);
    delete b;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

void upload_loop(rt_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_upload.wait(lk, [&] { return S->stop || !S->uploads.empty(); });
    if (S->stop) return;
    Request* r = S->uploads.front();
    S->uploads.pop_front();
    r->state = kRunning;
    r->start = Clock::now();
    for (;;) {
      lk.unlock();
      uint32_t id = 0;
      rt_status st = rt_pool_add_scene(S->pool, &r->desc, &id);
      lk.lock();
      if (st == RT_OK) {
        r->result_scene = (uint32_t)S->scenes.size();
        S->scenes.push_back(SceneRec{true, id, 0, ++S->use_clock, r->desc.num_triangles});
        finish_locked(S, r, RT_OK);
        break;
      }
      if (st != RT_ENOMEM) {
        finish_locked(S, r, st);
        break;
      }
      // evict the least recently used idle scene and retry
      int victim = -1;
      for (size_t i = 0; i < S->scenes.size(); ++i)
        if (S->scenes[i].live && S->scenes[i].refs == 0 &&
            (victim < 0 || S->scenes[i].last_use < S->scenes[(size_t)victim].last_use))
          victim = (int)i;
      if (victim < 0 || rt_pool_remove_scene(S->pool, S->scenes[(size_t)victim].pool_id) != RT_OK) {
        finish_locked(S, r, RT_ENOMEM);
        break;
      }
      S->scenes[(size_t)victim].live = false;
      S->stats.evictions++;
    }
    S->cv_done.notify_all();
  }
}

}  // namespace

using namespace rtgb;

extern "C" {

rt_status rt_server_create(const RtServerOptions* opt, rt_server** out) {
  if (!out) return RT_EINVAL;
  *out = nullptr;
  std::unique_ptr<rt_server> S(new rt_server());
  if (opt) S->opt = *opt;
  if (!S->opt.stage_rays) S->opt.stage_rays = 1u << 25;
  if (!S->opt.max_batch_rays) S->opt.max_batch_rays = 1u << 23;
  if (!S->opt.max_batch_jobs) S->opt.max_batch_jobs = 1024;
  if (!S->opt.max_inflight) S->opt.max_inflight = 3;
  if (S->opt.max_batch_jobs > 8192) S->opt.max_batch_jobs = 8192;
  if (S->opt.max_inflight > 16) S->opt.max_inflight = 16;
  RtPoolOptions po{};
  po.budget_bytes = S->opt.budget_bytes;
  po.max_scenes = S->opt.max_scenes;
  rt_status st = rt_pool_create(&po, &S->pool);
  if (st != RT_OK) return st;
  cudaGetDevice(&S->device);
  cudaError_t e = cudaMalloc(&S->d_rays, (size_t)S->opt.stage_rays * sizeof(RtRay));
  if (e == cudaSuccess) e = cudaMalloc(&S->d_hits, (size_t)S->opt.stage_rays * sizeof(RtHit));
  for (uint32_t i = 0; i < S->opt.max_inflight && e == cudaSuccess; ++i) {
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) S->streams.push_back(s);
  }
  if (e != cudaSuccess) {
    set_error(std::string("rt_server_create: ") + cudaGetErrorString(e));
    if (S->d_rays) cudaFree(S->d_rays);
    if (S->d_hits) cudaFree(S->d_hits);
    for (auto s : S->streams) cudaStreamDestroy(s);
    rt_pool_destroy(S->pool);
    return RT_ENOMEM;
  }
  S->stage = StageAlloc(S->opt.stage_rays);
  rt_server* raw = S.release();
  raw->dispatcher = std::thread(dispatch_loop, raw);
  raw->completer = std::thread(complete_loop, raw);
  raw->uploader = std::thread(upload_loop, raw);
  *out = raw;
  return RT_OK;
}

rt_status rt_server_destroy(rt_server* S) {
  if (!S) return RT_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    for (Request* r : S->pending) finish_locked(S, r, RT_ECANCELED);
    S->pending.clear();
    for (Request* r : S->uploads) finish_locked(S, r, RT_ECANCELED);
    S->uploads.clear();
  }
  S->cv_work.notify_all();
  S->cv_upload.notify_all();
  S->cv_inflight.notify_all();
  S->dispatcher.join();
  S->uploader.join();
  S->cv_inflight.notify_all();
  S->completer.join();
  cudaDeviceSynchronize();
  for (auto s : S->streams) cudaStreamDestroy(s);
  cudaFree(S->d_rays);
  cudaFree(S->d_hits);
  rt_pool_destroy(S->pool);
  delete S;
  return RT_OK;
}

rt_status rt_server_upload(rt_server* S, const RtSceneDesc* desc, uint64_t* out_id) {
  if (!S || !desc || !out_id) {
    set_error("rt_server_upload: null argument");
    return RT_EINVAL;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) return RT_ECANCELED;
  std::unique_ptr<Request> r(new Request());
  r->id = S->next_id++;
  r->kind = kUpload;
  r->desc = *desc;
  r->submit = Clock::now();
  *out_id = r->id;
  S->uploads.push_back(r.get());
  S->reqs[r->id] = std::move(r);
  S->cv_upload.notify_one();
  return RT_OK;
}

rt_status rt_server_submit(rt_server* S, uint32_t scene_id, const RtRay* h_rays, uint32_t n, RtHit* h_hits,
                           uint32_t flags, uint64_t* out_id) {
  if (!S || !out_id || (n && (!h_rays || !h_hits)) || flags > RT_TRACE_ANY) {
    set_error("rt_server_submit: bad argument");
    return RT_EINVAL;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) return RT_ECANCELED;
  if (n > S->opt.stage_rays) {
    set_error("rt_server_submit: more rays than the staging capacity");
    return RT_EINVAL;
  }
  if (scene_id >= S->scenes.size() || !S->scenes[scene_id].live) {
    set_error("rt_server_submit: unknown scene");
    return RT_ENOTFOUND;
  }
  std::unique_ptr<Request> r(new Request());
  r->id = S->next_id++;
  r->kind = kRays;
  r->scene = scene_id;
  r->h_rays = h_rays;
  r->h_hits = h_hits;
  r->n = n;
  r->flags = flags;
  r->submit = Clock::now();
  *out_id = r->id;
  S->scenes[scene_id].refs++;
  S->pending.push_back(r.get());
  S->reqs[r->id] = std::move(r);
  S->cv_work.notify_one();
  return RT_OK;
}

rt_status rt_server_cancel(rt_server* S, uint64_t id) {
  if (!S) return RT_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return RT_ENOTFOUND;
  Request* r = it->second.get();
  if (r->state != kPending) {
    set_error("rt_server_cancel: the request is already running or done");
    return RT_EBUSY;
  }
  auto& q = r->kind == kRays ? S->pending : S->uploads;
  q.erase(std::remove(q.begin(), q.end(), r), q.end());
  finish_locked(S, r, RT_ECANCELED);
  S->cv_done.notify_all();
  return RT_OK;
}

rt_status rt_server_wait(rt_server* S, uint64_t id, double timeout_seconds, RtRequestResult* out) {
  if (!S) return RT_EINVAL;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) {
    set_error("rt_server_wait: unknown request");
    return RT_ENOTFOUND;
  }
  Request* r = it->second.get();
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(
                                           timeout_seconds < 0 ? 0.0 : timeout_seconds));
  if (!S->cv_done.wait_until(lk, deadline, [&] { return r->state == kDone; })) {
    set_error("rt_server_wait: deadline passed");
    return RT_ETIMEOUT;
  }
  if (out) {
    out->status = r->status;
    out->scene_id = r->kind == kUpload ? r->result_scene : r->scene;
    out->num_rays = r->n;
    out->batch_jobs = r->batch_jobs;
    out->latency_seconds = std::chrono::duration<double>(r->done - r->submit).count();
    out->queue_seconds = std::chrono::duration<double>(r->start - r->submit).count();
  }
  const rt_status st = r->status;
  S->reqs.erase(it);
  return st;
}

rt_status rt_server_remove_scene(rt_server* S, uint32_t scene_id) {
  if (!S) return RT_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  if (scene_id >= S->scenes.size() || !S->scenes[scene_id].live) return RT_ENOTFOUND;
  if (S->scenes[scene_id].refs) {
    set_error("rt_server_remove_scene: the scene has queued or running ray requests");
    return RT_EBUSY;
  }
  rt_status st = rt_pool_remove_scene(S->pool, S->scenes[scene_id].pool_id);
  if (st == RT_OK) S->scenes[scene_id].live = false;
  return st;
}

rt_status rt_server_get_stats(rt_server* S, RtServerStats* out) {
  if (!S || !out) return RT_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  out->pending = (uint32_t)S->pending.size();
  out->inflight_batches = (uint32_t)S->inflight.size();
  uint32_t live = 0;
  for (auto& s : S->scenes) live += s.live ? 1u : 0u;
  out->resident_scenes = live;
  RtPoolInfo pi{};
  rt_pool_get_info(S->pool, &pi);
  out->resident_bytes = pi.used_bytes;
  return RT_OK;
}

rt_status rt_server_set_batching(rt_server* S, uint32_t max_batch_jobs, uint32_t max_inflight) {
  if (!S || max_batch_jobs == 0 || max_batch_jobs > 8192 || max_inflight == 0 || max_inflight > S->streams.size()) {
    set_error("rt_server_set_batching: 1 <= max_batch_jobs <= 8192, 1 <= max_inflight <= streams");
    return RT_EINVAL;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->opt.max_batch_jobs = max_batch_jobs;
  S->opt.max_inflight = max_inflight;
  S->cv_work.notify_all();
  return RT_OK;
}

rt_status rt_server_autotune(rt_server* S, uint32_t scene_id, const RtRay* d_rays, uint32_t n, RtHit* d_hits) {
  if (!S) return RT_EINVAL;
  RtJob j{scene_id, n, d_rays, d_hits};
  std::lock_guard<std::mutex> lk(S->mu);
  if (scene_id >= S->scenes.size() || !S->scenes[scene_id].live) return RT_ENOTFOUND;
  j.scene_id = S->scenes[scene_id].pool_id;
  return rt_pool_autotune(S->pool, &j, 1, RT_TRACE_CLOSEST, S->streams[0], 2);
}

}  // extern "C"
