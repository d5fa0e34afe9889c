// Host check of the serving pool's range allocator (fft_onchip_gb300/csrc/pool.h)
// against a unit-by-unit model: random allocations and frees in any order,
// no two live ranges overlap, every live range lies inside the pool, frees
// coalesce (an empty pool is one free range), and allocation fails only when
// no single free range is large enough.  Prints "ok <ops>" or the failure.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "pool.h"

int main() {
  const int64_t align = 256, units = 4096, cap = units * align;
  fftoc::RangePool pool(cap, align);
  std::vector<int> owner(units, -1);  // live range id per unit, -1 free
  struct Live { int64_t off, len; };
  std::vector<Live> live;
  std::mt19937_64 rng(12345);
  long ops = 0;
  for (int round = 0; round < 200000; ++round) {
    const bool do_alloc = live.empty() || (rng() % 100) < 55;
    if (do_alloc) {
      const int64_t bytes = 1 + (int64_t)(rng() % (64 * align));
      const int64_t need = (bytes + align - 1) / align;
      // largest free run in the model
      int64_t best = 0, run = 0;
      for (int64_t u = 0; u < units; ++u) {
        run = owner[u] < 0 ? run + 1 : 0;
        if (run > best) best = run;
      }
      const int64_t off = pool.alloc(bytes);
      if (off < 0) {
        if (best >= need) { printf("FAIL alloc refused: need %lld units, largest free %lld\n", (long long)need, (long long)best); return 1; }
        continue;
      }
      if (off % align || off < 0 || off + need * align > cap) { printf("FAIL range out of pool\n"); return 1; }
      for (int64_t u = off / align; u < off / align + need; ++u) {
        if (owner[u] >= 0) { printf("FAIL overlap at unit %lld\n", (long long)u); return 1; }
        owner[u] = (int)live.size();
      }
      live.push_back({off, need});
    } else {
      const size_t k = rng() % live.size();
      const Live l = live[k];
      if (!pool.release(l.off)) { printf("FAIL release of live range\n"); return 1; }
      for (int64_t u = l.off / align; u < l.off / align + l.len; ++u) owner[u] = -1;
      live[k] = live.back();
      live.pop_back();
      for (size_t i = 0; i < live.size(); ++i)
        for (int64_t u = live[i].off / align; u < live[i].off / align + live[i].len; ++u) owner[u] = (int)i;
    }
    int64_t used = 0;
    for (const Live& l : live) used += l.len * align;
    if (used != pool.used()) { printf("FAIL used bytes %lld vs %lld\n", (long long)pool.used(), (long long)used); return 1; }
    ++ops;
  }
  if (pool.release(12345)) { printf("FAIL released a range that is not live\n"); return 1; }
  for (const Live& l : live) pool.release(l.off);
  if (pool.used() != 0 || pool.free_ranges() != 1 || pool.largest_free() != cap) {
    printf("FAIL empty pool not coalesced: %zu ranges\n", pool.free_ranges());
    return 1;
  }
  if (pool.alloc(cap + 1) != -1 || pool.alloc(0) != -1) { printf("FAIL oversize/zero allocation accepted\n"); return 1; }
  printf("ok %ld\n", ops);
  return 0;
}
