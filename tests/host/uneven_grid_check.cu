// Host-side check of the uneven graph's grid rule (uneven_grid in
// fft_uneven.cuh): one CTA per tile for a size with at least 40 % of the
// batch's bytes or with fewer tiles than one wave, else one wave of
// persistent CTAs; never 0.  Prints "ok" on success.
#include <cstdio>
#include <cstdlib>

#include "fft_uneven.cuh"

using namespace fftoc;

#define CHECK(c)                                             \
  do {                                                       \
    if (!(c)) {                                              \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);       \
      std::exit(1);                                          \
    }                                                        \
  } while (0)

int main() {
  int c[kUnevenBins] = {};
  // one size alone: one CTA per tile
  c[9] = 41856;  // N = 4096
  CHECK(uneven_grid(c, 9, 1, 304) == 41856);
  // the mixed batch of 200,000 transforms: N = 4096 (45 % of the bytes) one
  // CTA per tile, every other size persistent (or its few tiles)
  const int mix[10] = {41319, 31169, 24991, 20607, 17961, 15674, 13979, 12656, 11180, 10464};
  for (int i = 0; i < 10; ++i) c[i] = mix[i];
  CHECK(uneven_grid(c, 9, 1, 304) == 10464);
  CHECK(uneven_grid(c, 8, 1, 456) == 456);        // 24 % of the bytes
  CHECK(uneven_grid(c, 7, 2, 1216) == 1216);
  CHECK(uneven_grid(c, 0, 256, 304) == 162);      // N = 8: 162 tiles, fewer than a wave
  // a dominant size next to a few small ones
  for (int i = 0; i < 10; ++i) c[i] = 0;
  c[9] = 10000;  // 655 MB
  c[0] = 50000;  // 12.8 MB
  CHECK(uneven_grid(c, 9, 1, 304) == 10000);
  CHECK(uneven_grid(c, 0, 256, 304) == 196);
  // 4096 holds 74 % of the bytes: one CTA per tile
  c[9] = 1000;
  c[6] = 2000;
  CHECK(uneven_grid(c, 9, 1, 304) == 1000);
  c[6] = 2000 * 8;   // 512 now holds 65 % of the bytes and 4096 32 %
  CHECK(uneven_grid(c, 9, 1, 304) == 304);
  CHECK(uneven_grid(c, 6, 1, 2128) == 16000);
  c[6] = 2000;
  // empty bucket and empty batch: one CTA, which returns at once
  CHECK(uneven_grid(c, 3, 32, 608) == 1);
  for (int i = 0; i < 10; ++i) c[i] = 0;
  CHECK(uneven_grid(c, 5, 8, 1216) == 1);
  std::printf("ok\n");
  return 0;
}
