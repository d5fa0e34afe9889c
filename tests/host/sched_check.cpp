// Host-only test of the serving loop's batching decision (batching.h) with a CPU
// executor in place of the GPU: simulated arrivals on a simulated clock, a
// byte array standing in for the device pool, stream slots that complete a
// batch after a simulated duration, and an "executor" that copies each
// request in, transforms it in place (every value v -> 2v + 1) and copies it
// out, as the device path does with its pool ranges.  Checks:
//   - every request completes once, with the right result (so no two live
//     requests ever shared pool bytes);
//   - a batch holds one engine, stays within the byte limit (unless it is a
//     single request) and the transform limit;
//   - requests of one engine launch in arrival order;
//   - with work in flight, a batch launches only when full or when its oldest
//     request has waited the window;
//   - split-form batches: one range per size, its requests back to back, one
//     owner per range;
//   - the pool is empty at the end.
// Prints "ok" on success.
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <deque>
#include <map>
#include <random>
#include <unordered_map>
#include <vector>

#include "batching.h"

using namespace fftoc;

#define CHECK(c)                                                      \
  do {                                                                \
    if (!(c)) {                                                       \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);                \
      std::exit(1);                                                   \
    }                                                                 \
  } while (0)

struct Req {
  SchedReq q;
  std::vector<double> in, out;
  int64_t pool_off = -1, range_off = -1;
  int64_t launch_seq = -1;
  bool done = false;
};

struct SlotSim {
  bool busy = false;
  double done_at = 0;
  Batch b;
};

static bool split_engine(int e) { return e >= 4; }

static void run(unsigned seed, int slots, int64_t pool_bytes, int64_t max_batch, double window, double rate_per_us) {
  std::mt19937_64 g(seed);
  const int sizes[] = {8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096};
  const int nreq = 600;
  std::vector<Req> reqs(nreq);
  std::vector<double> arrival(nreq);
  double t = 0;
  std::exponential_distribution<double> gap(rate_per_us);
  for (int i = 0; i < nreq; ++i) {
    Req& r = reqs[i];
    r.q.id = i;
    r.q.n = sizes[g() % 10];
    const int64_t max_count = std::max<int64_t>(1, (pool_bytes / 4) / (16 * r.q.n));
    r.q.count = 1 + (int64_t)(g() % (unsigned long long)std::min<int64_t>(max_count, 64));
    r.q.engine = (g() & 1) ? 2 : 5;  // plain fixed point or a split engine
    r.q.bytes = r.q.count * r.q.n * 16;
    r.in.resize((size_t)r.q.count * r.q.n * 2);
    for (double& v : r.in) v = (double)(g() % 1000) - 500.0;
    t += gap(g);
    arrival[i] = t;
    r.q.submit_us = t;
  }
  SchedConfig cfg;
  cfg.max_batch_bytes = max_batch;
  cfg.max_wait_us = window;
  cfg.max_count = max_batch / 128;
  RangePool pool(pool_bytes, 256);
  std::vector<double> device(pool_bytes / 8, 0.0);  // the pool's bytes, as doubles
  std::vector<SlotSim> sl(slots);
  std::deque<int64_t> pending;
  int next = 0, done = 0;
  int64_t seq = 0;
  double now = 0;
  std::map<int, int64_t> last_seq;  // per engine: arrival id of the last launched request
  auto lookup = [&](int64_t id) -> const SchedReq& { return reqs[id].q; };
  for (int iter = 0; iter < 200000 && done < nreq; ++iter) {
    // arrivals up to now
    while (next < nreq && arrival[next] <= now) pending.push_back(next++);
    // completions up to now: copy out, release
    for (SlotSim& s : sl)
      if (s.busy && s.done_at <= now) {
        for (const Placement& p : s.b.reqs) {
          Req& r = reqs[p.id];
          const double* src = &device[(size_t)p.pool_off / 8];
          r.out.assign(src, src + r.in.size());
          if (p.range_off >= 0) CHECK(pool.release(p.range_off));
          r.done = true;
          ++done;
        }
        s.busy = false;
      }
    // launch as long as the decision says so
    while (true) {
      int si = -1, inflight = 0;
      for (int i = 0; i < slots; ++i) {
        if (sl[i].busy) ++inflight;
        else if (si < 0) si = i;
      }
      const double head_wait = pending.empty() ? 0 : now - reqs[pending.front()].q.submit_us;
      int64_t queued = 0;
      for (int64_t id : pending) queued += reqs[id].q.bytes;
      Batch b;
      const SchedStep st = form_batch(pending, lookup, split_engine, si >= 0, inflight, now, cfg, pool, &b);
      if (st != SchedStep::kLaunch) break;
      CHECK(inflight == 0 || queued >= cfg.max_batch_bytes || head_wait >= cfg.max_wait_us);
      CHECK(!b.reqs.empty());
      CHECK(b.reqs.size() == 1 || b.bytes <= cfg.max_batch_bytes);
      CHECK(b.transforms <= cfg.max_count);
      int64_t owners = 0;
      for (const Placement& p : b.reqs) {
        Req& r = reqs[p.id];
        CHECK(r.q.engine == b.engine && !r.done && r.launch_seq < 0);
        auto it = last_seq.find(r.q.engine);
        CHECK(it == last_seq.end() || it->second < p.id);  // arrival order per engine
        last_seq[r.q.engine] = p.id;
        r.launch_seq = seq++;
        r.pool_off = p.pool_off;
        r.range_off = p.range_off;
        owners += p.range_off >= 0;
        CHECK(p.pool_off % 16 == 0 && p.pool_off + p.bytes <= pool_bytes);
        std::copy(r.in.begin(), r.in.end(), device.begin() + (size_t)p.pool_off / 8);
      }
      if (split_engine(b.engine)) {
        CHECK((int64_t)b.groups.size() == owners);
        for (const SizeGroup& gr : b.groups) {
          int64_t off = gr.pool_off, cnt = 0;
          for (const Placement& p : b.reqs)
            if (p.n == gr.n) {
              CHECK(p.pool_off == off);  // back to back in arrival order
              off += p.bytes;
              cnt += p.count;
            }
          CHECK(off == gr.pool_off + gr.bytes && cnt == gr.count);
          // the executor: one in-place "launch" over the whole group
          for (int64_t k = gr.pool_off / 8; k < (gr.pool_off + gr.bytes) / 8; ++k) device[(size_t)k] = 2 * device[(size_t)k] + 1;
        }
      } else {
        CHECK(b.groups.empty() && owners == (int64_t)b.reqs.size());
        for (const Placement& p : b.reqs)
          for (int64_t k = p.pool_off / 8; k < (p.pool_off + p.bytes) / 8; ++k) device[(size_t)k] = 2 * device[(size_t)k] + 1;
      }
      sl[si].busy = true;
      sl[si].b = b;
      sl[si].done_at = now + 5.0 + (double)b.bytes / 2e5;  // simulated batch time (us)
    }
    // advance the clock to the next event
    double nxt = 1e300;
    if (next < nreq) nxt = std::min(nxt, arrival[next]);
    for (const SlotSim& s : sl)
      if (s.busy) nxt = std::min(nxt, s.done_at);
    if (!pending.empty() && reqs[pending.front()].q.submit_us + cfg.max_wait_us > now)
      nxt = std::min(nxt, reqs[pending.front()].q.submit_us + cfg.max_wait_us);
    if (nxt == 1e300) break;  // nothing can happen any more
    CHECK(nxt > now);
    now = nxt;
  }
  CHECK(done == nreq);
  for (const Req& r : reqs) {
    CHECK(r.done && r.out.size() == r.in.size());
    for (size_t k = 0; k < r.in.size(); ++k) CHECK(r.out[k] == 2 * r.in[k] + 1);
  }
  CHECK(pool.used() == 0);
}

int main() {
  run(1, 4, 64 << 20, 8 << 20, 50.0, 0.05);    // light load
  run(2, 4, 64 << 20, 8 << 20, 50.0, 5.0);     // saturated: batches fill
  run(3, 2, 16 << 20, 8 << 20, 20.0, 5.0);     // pool holds two batches
  run(4, 1, 8 << 20, 8 << 20, 0.0, 1.0);       // one slot, no window, pool = one batch
  std::printf("ok\n");
  return 0;
}
