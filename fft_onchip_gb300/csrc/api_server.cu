// fftoc — serving loop: continuous batching of FFT requests of mixed sizes.
//
// No counterpart in the reference (its harness transforms one resident batch
// per call, includes/testing.cuh:94-175).  A request is `count` transforms of
// one size n in host memory, tagged with an engine.  One scheduler thread:
//   - admits requests in arrival order into a fixed device pool (allocated
//     once at creation) by bytes: a request enters a batch only when a free
//     range of the pool holds it (pool.h);
//   - packs admitted requests of one engine (the oldest pending request's;
//     requests of other engines keep their place) into a device batch (up to
//     max_batch_bytes; the decision is batching.h's) and runs it on one of
//     `slots` streams: H2D copy of each request into the pool, then the
//     plain form's one uneven-batch graph (fftoc_uneven_execute) over all the
//     batch's transforms, or the split form's one launch per size group (the
//     requests of one size placed back to back), D2H copy of each request,
//     and a host callback that timestamps completion;
//   - keeps forming and launching batches while others are on the GPU, as
//     stream slots and pool memory free up (continuous batching).
// Every transform's arithmetic depends only on its own points and its size's
// plan, so a request's result is bit-identical alone and in any mix.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/fftoc.h"
#include "internal.h"
#include "pool.h"
#include "batching.h"

namespace fftoc {
namespace {

using Clock = std::chrono::steady_clock;

double now_us(Clock::time_point t0) {
  return std::chrono::duration<double, std::micro>(Clock::now() - t0).count();
}

struct Request {
  int64_t id = 0;
  int n = 0;
  int64_t count = 0;
  int engine = 0;
  const double* h_in = nullptr;
  double* h_out = nullptr;
  int64_t bytes = 0;
  int64_t pool_off = -1;   // where the request's data sit in the pool
  int64_t range_off = -1;  // the pool range it releases (-1: none; a split size group's other requests)
  double submit_us = 0, launch_us = 0, done_us = 0;
  int state = 0;  // 0 pending, 1 in flight, 2 done
  fftoc_status status = FFTOC_OK;
};

struct Slot {
  cudaStream_t stream = nullptr;
  fftoc_uneven_plan plan[2] = {nullptr, nullptr};  // [0] binary64, [1] fixed point
  int64_t* h_off = nullptr;  // pinned offset / size tables of the batch in flight
  int32_t* h_ns = nullptr;
  int64_t* d_off = nullptr;
  int32_t* d_ns = nullptr;
  bool busy = false;
  std::vector<int64_t> reqs;  // request ids of the batch in flight
  double done_us = 0;
};

}  // namespace
}  // namespace fftoc

struct fftoc_server_s {
  fftoc_server_config cfg{};
  int device = 0;
  unsigned char* pool_base = nullptr;
  fftoc::RangePool* pool = nullptr;
  std::vector<fftoc::Slot> slots;
  int64_t max_count = 0;  // transforms per batch (uneven plan capacity)

  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-up
  std::condition_variable cv_done;  // request completion
  std::deque<int64_t> pending;
  std::unordered_map<int64_t, fftoc::Request> reqs;
  std::unordered_map<int64_t, fftoc::SchedReq> sreqs;  // pending requests, as the batching decision sees them
  std::vector<int> completed_slots;
  int64_t next_id = 1;
  bool stop = false;
  std::thread sched;
  fftoc::Clock::time_point t0;
  // statistics
  int64_t batches = 0, requests_done = 0, transforms_done = 0, bytes_done = 0;
  int max_inflight = 0;
};

namespace fftoc {
namespace {

fftoc_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  return set_error(e == cudaErrorMemoryAllocation ? FFTOC_ERR_NO_MEMORY : FFTOC_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

struct CallbackData {
  fftoc_server_s* s;
  int slot;
};

void CUDART_CB batch_done(void* p) {
  // runs on a CUDA callback thread: no CUDA calls here
  CallbackData* cd = static_cast<CallbackData*>(p);
  fftoc_server_s* s = cd->s;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->slots[cd->slot].done_us = now_us(s->t0);
    s->completed_slots.push_back(cd->slot);
  }
  s->cv.notify_one();
  delete cd;
}

// Enqueue one batch on its slot (scheduler thread, lock NOT held).  Plain
// form: one uneven-batch graph over all the batch's transforms.  Split form:
// one launch per size group (its requests back to back in one pool range).
fftoc_status enqueue_batch(fftoc_server_s* s, int si, const Batch& b, const std::vector<Request*>& rs) {
  Slot& sl = s->slots[si];
  cudaError_t e;
  for (const Request* r : rs)
    if ((e = cudaMemcpyAsync(s->pool_base + r->pool_off, r->h_in, (size_t)r->bytes, cudaMemcpyHostToDevice,
                             sl.stream)) != cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync(request in)");
  if (is_split_engine(b.engine)) {
    for (const SizeGroup& g : b.groups) {
      double* buf = reinterpret_cast<double*>(s->pool_base + g.pool_off);
      const fftoc_status st = launch_split(g.n, buf, buf, g.count, split_kind_of(b.engine), sl.stream);
      if (st != FFTOC_OK) return st;
    }
  } else {
    const int engine_slot = b.engine == FFTOC_ENGINE_F64 ? 0 : 1;
    int64_t k = 0;
    for (const Request* r : rs) {
      const int64_t base = r->pool_off / 16;  // complex elements from the pool base
      for (int64_t t = 0; t < r->count; ++t, ++k) {
        sl.h_off[k] = base + t * r->n;
        sl.h_ns[k] = r->n;
      }
    }
    double* pool = reinterpret_cast<double*>(s->pool_base);
    if ((e = cudaMemcpyAsync(sl.d_off, sl.h_off, (size_t)b.transforms * 8, cudaMemcpyHostToDevice, sl.stream)) !=
        cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync(offsets)");
    if ((e = cudaMemcpyAsync(sl.d_ns, sl.h_ns, (size_t)b.transforms * 4, cudaMemcpyHostToDevice, sl.stream)) !=
        cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync(sizes)");
    const fftoc_status st = fftoc_uneven_execute(sl.plan[engine_slot], pool, pool, sl.d_off, sl.d_ns, b.transforms,
                                                 (fftoc_stream)sl.stream);
    if (st != FFTOC_OK) return st;
  }
  for (const Request* r : rs)
    if ((e = cudaMemcpyAsync(r->h_out, s->pool_base + r->pool_off, (size_t)r->bytes, cudaMemcpyDeviceToHost,
                             sl.stream)) != cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync(request out)");
  CallbackData* cd = new CallbackData{s, si};
  if ((e = cudaLaunchHostFunc(sl.stream, batch_done, cd)) != cudaSuccess) {
    delete cd;
    return cuda_fail(e, "cudaLaunchHostFunc");
  }
  return FFTOC_OK;
}

void retire(fftoc_server_s* s, int si) {  // lock held
  Slot& sl = s->slots[si];
  for (int64_t id : sl.reqs) {
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) continue;
    Request& r = it->second;
    if (r.range_off >= 0) s->pool->release(r.range_off);
    r.pool_off = r.range_off = -1;
    r.done_us = sl.done_us;
    r.state = 2;
    s->requests_done += 1;
    s->transforms_done += r.count;
    s->bytes_done += r.bytes;
  }
  sl.reqs.clear();
  sl.busy = false;
  s->cv_done.notify_all();
}

void fail_requests(fftoc_server_s* s, const std::vector<Request*>& rs, fftoc_status st) {  // lock held
  for (Request* r : rs) {
    if (r->range_off >= 0) s->pool->release(r->range_off);
    r->pool_off = r->range_off = -1;
    r->state = 2;
    r->status = st;
    r->done_us = now_us(s->t0);
  }
  s->cv_done.notify_all();
}

void scheduler(fftoc_server_s* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    for (int si : s->completed_slots) retire(s, si);
    s->completed_slots.clear();
    if (s->stop) {
      // shutting down: requests not yet on the GPU fail, batches in flight finish
      std::vector<Request*> left;
      for (int64_t id : s->pending) {
        left.push_back(&s->reqs[id]);
        s->sreqs.erase(id);
      }
      s->pending.clear();
      fail_requests(s, left, FFTOC_ERR_INVALID_VALUE);
      bool any = false;
      for (const Slot& sl : s->slots) any = any || sl.busy;
      if (!any) break;
      s->cv.wait(lk);
      continue;
    }
    bool waiting_window = false;
    const SchedConfig cfg{s->cfg.max_batch_bytes, s->cfg.max_wait_us, s->max_count};
    auto lookup = [s](int64_t id) -> const SchedReq& { return s->sreqs[id]; };
    while (!s->stop && !s->pending.empty()) {
      int si = -1, inflight = 0;
      for (int i = 0; i < (int)s->slots.size(); ++i) {
        if (s->slots[i].busy) ++inflight;
        else if (si < 0) si = i;
      }
      const double now = now_us(s->t0);
      Batch b;
      nvtxRangePushA("fftoc.serve.form_batch");
      const SchedStep step = form_batch(s->pending, lookup, is_split_engine, si >= 0, inflight, now, cfg, *s->pool, &b);
      nvtxRangePop();
      if (step == SchedStep::kWaitWindow) waiting_window = true;
      if (step != SchedStep::kLaunch) break;
      std::vector<Request*> batch;
      for (const Placement& p : b.reqs) {
        Request& r = s->reqs[p.id];
        r.pool_off = p.pool_off;
        r.range_off = p.range_off;
        r.state = 1;
        r.launch_us = now;
        s->sreqs.erase(p.id);
        batch.push_back(&r);
      }
      Slot& sl = s->slots[si];
      sl.busy = true;
      sl.reqs.clear();
      for (Request* r : batch) sl.reqs.push_back(r->id);
      s->batches += 1;
      if (inflight + 1 > s->max_inflight) s->max_inflight = inflight + 1;
      lk.unlock();
      nvtxRangePushA(is_split_engine(b.engine) ? "fftoc.serve.enqueue_split" : "fftoc.serve.enqueue_plain");
      const fftoc_status st = enqueue_batch(s, si, b, batch);
      nvtxRangePop();
      lk.lock();
      if (st != FFTOC_OK) {
        // the stream may hold part of the batch: drain it before reusing the ranges
        lk.unlock();
        cudaStreamSynchronize(s->slots[si].stream);
        cudaGetLastError();
        lk.lock();
        s->slots[si].reqs.clear();
        s->slots[si].busy = false;
        fail_requests(s, batch, st);
      }
    }
    if (s->stop) continue;
    if (waiting_window && s->completed_slots.empty()) {
      const Request& head = s->reqs[s->pending.front()];
      const double wait = head.submit_us + s->cfg.max_wait_us - now_us(s->t0);
      s->cv.wait_for(lk, std::chrono::microseconds((int64_t)(wait > 1 ? wait : 1)));
    } else if (s->completed_slots.empty()) {
      s->cv.wait(lk);
    }
  }
}

void destroy(fftoc_server_s* s) {
  if (s->sched.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv.notify_one();
    s->sched.join();
  }
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (auto& p : sl.plan)
      if (p) fftoc_uneven_plan_destroy(p);
    if (sl.h_off) cudaFreeHost(sl.h_off);
    if (sl.h_ns) cudaFreeHost(sl.h_ns);
    if (sl.d_off) cudaFree(sl.d_off);
    if (sl.d_ns) cudaFree(sl.d_ns);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  if (s->pool_base) cudaFree(s->pool_base);
  delete s->pool;
  delete s;
}

fftoc_status create(fftoc_server* out, const fftoc_server_config* cfg_in) {
  if (!out) return set_error(FFTOC_ERR_INVALID_VALUE, "null server pointer");
  *out = nullptr;
  fftoc_server_config cfg;
  fftoc_server_config_default(&cfg);
  if (cfg_in) cfg = *cfg_in;
  if (cfg.pool_bytes < (1 << 20) || cfg.slots < 1 || cfg.slots > 64 || cfg.max_batch_bytes < 4096 ||
      cfg.max_batch_bytes > cfg.pool_bytes || cfg.max_wait_us < 0)
    return set_error(FFTOC_ERR_INVALID_VALUE, "invalid server configuration");
  fftoc_server_s* s = new fftoc_server_s;
  s->cfg = cfg;
  s->t0 = Clock::now();
  cudaError_t e = cudaGetDevice(&s->device);
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "cudaGetDevice");
  }
  auto bad = [&](fftoc_status st) {
    destroy(s);
    return st;
  };
  if ((e = cudaMalloc(&s->pool_base, (size_t)cfg.pool_bytes)) != cudaSuccess)
    return bad(cuda_fail(e, "cudaMalloc(server pool)"));
  s->pool = new RangePool(cfg.pool_bytes, 256);
  // transforms per batch: max_batch_bytes of 8-point transforms (a single
  // request may exceed max_batch_bytes, up to the pool, within this count)
  s->max_count = cfg.max_batch_bytes / 128;
  if (s->max_count > 0x7FFFFFFFLL) s->max_count = 0x7FFFFFFFLL;
  s->slots.resize(cfg.slots);
  for (Slot& sl : s->slots) {
    if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess)
      return bad(cuda_fail(e, "cudaStreamCreate"));
    if ((e = cudaMallocHost(&sl.h_off, (size_t)s->max_count * 8)) != cudaSuccess)
      return bad(cuda_fail(e, "cudaMallocHost(offsets)"));
    if ((e = cudaMallocHost(&sl.h_ns, (size_t)s->max_count * 4)) != cudaSuccess)
      return bad(cuda_fail(e, "cudaMallocHost(sizes)"));
    if ((e = cudaMalloc(&sl.d_off, (size_t)s->max_count * 8)) != cudaSuccess)
      return bad(cuda_fail(e, "cudaMalloc(offsets)"));
    if ((e = cudaMalloc(&sl.d_ns, (size_t)s->max_count * 4)) != cudaSuccess)
      return bad(cuda_fail(e, "cudaMalloc(sizes)"));
    fftoc_status st = fftoc_uneven_plan_create(&sl.plan[0], s->max_count, FFTOC_ENGINE_F64);
    if (st == FFTOC_OK) st = fftoc_uneven_plan_create(&sl.plan[1], s->max_count, FFTOC_ENGINE_FX);
    if (st != FFTOC_OK) return bad(st);
  }
  s->sched = std::thread(scheduler, s);
  *out = s;
  return FFTOC_OK;
}

fftoc_status submit(fftoc_server_s* s, int n, int64_t count, int engine, const double* h_in, double* h_out,
                    int64_t* id) {
  if (!s || !id) return set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  if (size_index(n) < 0) return set_error(FFTOC_ERR_INVALID_SIZE, "n=" + std::to_string(n) + " is not one of 8,16,...,4096");
  if (count < 1) return set_error(FFTOC_ERR_INVALID_VALUE, "count must be >= 1");
  if (engine < FFTOC_ENGINE_AUTO || engine > kLastEngine) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown engine");
  const int eng = resolved_engine(n, engine);
  if (eng != FFTOC_ENGINE_F64 && eng != FFTOC_ENGINE_FX && !is_split_engine(eng))
    return set_error(FFTOC_ERR_UNSUPPORTED, "engine not available in the serving loop");
  if (is_split_engine(eng) && !split_supported(n, split_kind_of(eng)))
    return set_error(FFTOC_ERR_UNSUPPORTED, "no split-precision plan for n=" + std::to_string(n));
  if (!h_in || !h_out) return set_error(FFTOC_ERR_INVALID_VALUE, "null buffer");
  if (((uintptr_t)h_in & 15) || ((uintptr_t)h_out & 15)) return set_error(FFTOC_ERR_MISALIGNED, "buffers must be 16-byte aligned");
  const int64_t bytes = count * (int64_t)n * 16;
  if (bytes > s->cfg.pool_bytes || count > s->max_count)
    return set_error(FFTOC_ERR_INVALID_VALUE, "request larger than the server pool or than max_batch_bytes/128 transforms");
  Request r;
  r.n = n;
  r.count = count;
  r.engine = eng;
  r.h_in = h_in;
  r.h_out = h_out;
  r.bytes = bytes;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_error(FFTOC_ERR_INVALID_VALUE, "server is shutting down");
    r.id = s->next_id++;
    r.submit_us = now_us(s->t0);
    s->reqs[r.id] = r;
    fftoc::SchedReq q;
    q.id = r.id;
    q.n = r.n;
    q.count = r.count;
    q.engine = r.engine;
    q.bytes = r.bytes;
    q.submit_us = r.submit_us;
    s->sreqs[r.id] = q;
    s->pending.push_back(r.id);
    *id = r.id;
  }
  s->cv.notify_one();
  return FFTOC_OK;
}

void fill_timing(const Request& r, fftoc_request_timing* t) {
  if (!t) return;
  t->submit_us = r.submit_us;
  t->launch_us = r.launch_us;
  t->done_us = r.done_us;
  t->status = r.status;
}

// done: 1 and the record released when the request finished
fftoc_status poll(fftoc_server_s* s, int64_t id, int* done, fftoc_request_timing* t) {
  if (!s || !done) return set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown request id");
  *done = it->second.state == 2;
  if (*done) {
    fill_timing(it->second, t);
    const fftoc_status st = it->second.status;
    s->reqs.erase(it);
    if (st != FFTOC_OK) return set_error(st, "request failed");
  }
  return FFTOC_OK;
}

fftoc_status wait(fftoc_server_s* s, int64_t id, double timeout_s, fftoc_request_timing* t) {
  if (!s) return set_error(FFTOC_ERR_INVALID_VALUE, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto done = [&] {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() || it->second.state == 2;
  };
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9), done);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown request id");
  if (!ok) return set_error(FFTOC_ERR_TIMEOUT, "request not finished within the timeout");
  fill_timing(it->second, t);
  const fftoc_status st = it->second.status;
  s->reqs.erase(it);
  return st == FFTOC_OK ? FFTOC_OK : set_error(st, "request failed");
}

}  // namespace
}  // namespace fftoc

extern "C" {

void fftoc_server_config_default(fftoc_server_config* cfg) {
  if (!cfg) return;
  cfg->pool_bytes = (int64_t)8 << 30;
  cfg->slots = 4;
  cfg->max_batch_bytes = (int64_t)256 << 20;
  cfg->max_wait_us = 50.0;
}

fftoc_status fftoc_server_create(fftoc_server* server, const fftoc_server_config* cfg) {
  return fftoc::create(server, cfg);
}

fftoc_status fftoc_server_submit(fftoc_server server, int n, int64_t count, int engine, const double* h_in,
                                 double* h_out, int64_t* request_id) {
  return fftoc::submit(server, n, count, engine, h_in, h_out, request_id);
}

fftoc_status fftoc_server_poll(fftoc_server server, int64_t request_id, int* done, fftoc_request_timing* timing) {
  return fftoc::poll(server, request_id, done, timing);
}

fftoc_status fftoc_server_wait(fftoc_server server, int64_t request_id, double timeout_s,
                               fftoc_request_timing* timing) {
  return fftoc::wait(server, request_id, timeout_s, timing);
}

fftoc_status fftoc_server_stats(fftoc_server server, fftoc_server_stats_t* st) {
  if (!server || !st) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  std::lock_guard<std::mutex> lk(server->mu);
  st->batches = server->batches;
  st->requests_done = server->requests_done;
  st->transforms_done = server->transforms_done;
  st->bytes_done = server->bytes_done;
  st->pool_bytes_in_use = server->pool->used();
  st->pending = (int64_t)server->pending.size();
  st->max_inflight_batches = server->max_inflight;
  return FFTOC_OK;
}

fftoc_status fftoc_server_replay(fftoc_server server, const fftoc_replay_item* items, int64_t m,
                                 const double* h_in_arena, double* h_out_arena, double* latency_us, double* wall_s) {
  if (!server || (m > 0 && (!items || !h_in_arena || !h_out_arena || !latency_us)))
    return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  std::vector<int64_t> ids((size_t)m, 0);
  const auto start = fftoc::Clock::now();
  const double start_us = fftoc::now_us(server->t0);
  for (int64_t i = 0; i < m; ++i) {
    const fftoc_replay_item& it = items[i];
    while (std::chrono::duration<double, std::micro>(fftoc::Clock::now() - start).count() < it.arrival_us) {
    }
    fftoc_status st = fftoc::submit(server, it.n, it.count, it.engine, h_in_arena + 2 * it.in_offset,
                                    h_out_arena + 2 * it.out_offset, &ids[i]);
    if (st != FFTOC_OK) return st;
  }
  fftoc_status first = FFTOC_OK;
  for (int64_t i = 0; i < m; ++i) {
    fftoc_request_timing t{};
    fftoc_status st = fftoc::wait(server, ids[i], 600.0, &t);
    if (st != FFTOC_OK && first == FFTOC_OK) first = st;
    latency_us[i] = t.done_us - (start_us + items[i].arrival_us);
  }
  if (wall_s) *wall_s = std::chrono::duration<double>(fftoc::Clock::now() - start).count();
  return first;
}

fftoc_status fftoc_server_destroy(fftoc_server server) {
  if (!server) return FFTOC_OK;
  fftoc::destroy(server);
  return FFTOC_OK;
}

}  // extern "C"
