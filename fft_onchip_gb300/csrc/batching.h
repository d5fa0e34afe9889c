// fftoc — the serving loop's batching decision, free of CUDA so that the host
// tests drive it with a CPU executor (tests/host/sched_check.cpp).
//
// Given the pending requests in arrival order, the decision is:
//   - wait while every stream slot is busy;
//   - wait for the batching window while something is in flight, the queued
//     bytes do not fill a batch and the oldest request is younger than the
//     window;
//   - otherwise form a batch from the oldest request's engine: its requests in
//     arrival order (requests of other engines keep their place), up to the
//     batch's byte and transform limits (a single request may exceed the byte
//     limit), each admitted only into free pool memory, stopping at the first
//     that does not fit.
// Plain-form batches give every request its own pool range (the uneven-batch
// graph reads any offsets).  Split-form batches place the requests of one
// size back to back in one range per size, so each size group is one launch
// of the split kernel; if the groups of the selected requests do not all fit,
// the newest selected request is dropped and the groups are formed again.
#pragma once
#include <cstdint>
#include <deque>
#include <utility>
#include <vector>

#include "pool.h"

namespace fftoc {

struct SchedConfig {
  int64_t max_batch_bytes = 0;  // bytes per batch (one larger request still forms a batch)
  double max_wait_us = 0;       // batching window of the oldest pending request
  int64_t max_count = 0;        // transforms per batch
};

// What the decision needs of a pending request.
struct SchedReq {
  int64_t id = 0;
  int n = 0;
  int64_t count = 0;
  int engine = 0;
  int64_t bytes = 0;
  double submit_us = 0;
};

// A request of a formed batch: where its data go in the pool, and the pool
// range it releases on completion (-1: it shares a range another request of
// its size group releases).
struct Placement {
  int64_t id = 0;
  int n = 0;
  int64_t count = 0;
  int64_t bytes = 0;
  int64_t pool_off = 0;
  int64_t range_off = -1;
};

// Split-form batches: the requests of one size, back to back from pool_off.
struct SizeGroup {
  int n = 0;
  int64_t pool_off = 0;
  int64_t count = 0;
  int64_t bytes = 0;
};

struct Batch {
  int engine = 0;
  int64_t bytes = 0, transforms = 0;
  std::vector<Placement> reqs;  // arrival order
  std::vector<SizeGroup> groups;  // split form only, in order of first appearance
};

enum class SchedStep { kLaunch, kWaitWindow, kWaitSlot, kWaitMemory, kIdle };

// The next step for `pending` (ids in arrival order; lookup(id) -> const
// SchedReq&).  kLaunch: *out holds the batch, its ids are removed from
// `pending` and its ranges are allocated from `pool`.  `grouped(engine)`
// says whether the engine's batches use size groups.
template <class Lookup, class Grouped>
SchedStep form_batch(std::deque<int64_t>& pending, const Lookup& lookup, const Grouped& grouped, bool slot_free,
                     int inflight, double now, const SchedConfig& cfg, RangePool& pool, Batch* out) {
  if (pending.empty()) return SchedStep::kIdle;
  if (!slot_free) return SchedStep::kWaitSlot;
  const SchedReq& head = lookup(pending.front());
  int64_t queued = 0;
  for (int64_t id : pending) {
    queued += lookup(id).bytes;
    if (queued >= cfg.max_batch_bytes) break;
  }
  if (inflight > 0 && queued < cfg.max_batch_bytes && now - head.submit_us < cfg.max_wait_us)
    return SchedStep::kWaitWindow;

  Batch b;
  b.engine = head.engine;
  std::vector<size_t> taken;  // positions in `pending`
  if (!grouped(b.engine)) {
    for (size_t i = 0; i < pending.size(); ++i) {
      const SchedReq& r = lookup(pending[i]);
      if (r.engine != b.engine) continue;
      if (!b.reqs.empty() && (b.bytes + r.bytes > cfg.max_batch_bytes || b.transforms + r.count > cfg.max_count))
        break;
      const int64_t off = pool.alloc(r.bytes);
      if (off < 0) break;  // wait for memory to free up
      Placement p;
      p.id = r.id;
      p.n = r.n;
      p.count = r.count;
      p.bytes = r.bytes;
      p.pool_off = off;
      p.range_off = off;
      b.reqs.push_back(p);
      b.bytes += r.bytes;
      b.transforms += r.count;
      taken.push_back(i);
    }
  } else {
    // the candidates the limits allow, in arrival order
    std::vector<size_t> cand;
    int64_t bytes = 0, transforms = 0;
    for (size_t i = 0; i < pending.size(); ++i) {
      const SchedReq& r = lookup(pending[i]);
      if (r.engine != b.engine) continue;
      if (!cand.empty() && (bytes + r.bytes > cfg.max_batch_bytes || transforms + r.count > cfg.max_count)) break;
      cand.push_back(i);
      bytes += r.bytes;
      transforms += r.count;
    }
    // one range per size; drop the newest candidate until every group fits
    while (!cand.empty()) {
      std::vector<SizeGroup> groups;
      for (size_t i : cand) {
        const SchedReq& r = lookup(pending[i]);
        size_t g = 0;
        while (g < groups.size() && groups[g].n != r.n) ++g;
        if (g == groups.size()) {
          SizeGroup sg;
          sg.n = r.n;
          groups.push_back(sg);
        }
        groups[g].bytes += r.bytes;
        groups[g].count += r.count;
      }
      size_t ok = 0;
      for (; ok < groups.size(); ++ok) {
        const int64_t off = pool.alloc(groups[ok].bytes);
        if (off < 0) break;
        groups[ok].pool_off = off;
      }
      if (ok < groups.size()) {
        for (size_t g = 0; g < ok; ++g) pool.release(groups[g].pool_off);
        cand.pop_back();
        continue;
      }
      std::vector<int64_t> fill(groups.size(), 0);
      for (size_t i : cand) {
        const SchedReq& r = lookup(pending[i]);
        size_t g = 0;
        while (groups[g].n != r.n) ++g;
        Placement p;
        p.id = r.id;
        p.n = r.n;
        p.count = r.count;
        p.bytes = r.bytes;
        p.pool_off = groups[g].pool_off + fill[g];
        p.range_off = fill[g] == 0 ? groups[g].pool_off : -1;
        fill[g] += r.bytes;
        b.reqs.push_back(p);
        b.bytes += r.bytes;
        b.transforms += r.count;
        taken.push_back(i);
      }
      b.groups = groups;
      break;
    }
  }
  if (b.reqs.empty()) return SchedStep::kWaitMemory;
  for (size_t k = taken.size(); k-- > 0;) pending.erase(pending.begin() + (std::ptrdiff_t)taken[k]);
  *out = std::move(b);
  return SchedStep::kLaunch;
}

}  // namespace fftoc
