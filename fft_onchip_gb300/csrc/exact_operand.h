// fftoc — the exact-slice split form's B operand (host code): the 16-point
// DFT matrix cut into 8-bit digits, in the layout fft_exact.cuh reads.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace fftoc {

// FP16 bit pattern of an integer |v| < 2048 (exact).
inline uint16_t f16_int(int v) {
  if (v == 0) return 0;
  const unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((a >> (e + 1)) != 0) ++e;
  const unsigned mant = ((a << (10 - e)) & 0x3FFu);
  return (uint16_t)((v < 0 ? 0x8000u : 0u) | ((unsigned)(e + 15) << 10) | mant);
}

// The DFT matrix for the exact-slice form: entries scaled by 2^46 (rounded
// from long double) and cut into six balanced 8-bit digits f_0..f_5, most
// significant first (|f_j| <= 128, |f_0| <= 64).  192 rows of 64 FP16 K elements, K-major
// core matrices of 8 rows x 16 bytes: row 32j + c, K element 2v + e holds
// digit j - e (zero for j - e < 0) of the entry for accumulator column c
// (c = 2m: real part of output m, c = 2m + 1: imaginary part) and input value
// v (v < 16: real part of input v, else imaginary part of input v - 16).
inline std::vector<unsigned char> dft16_exact_operand() {
  const int kc = 8;
  std::vector<unsigned char> out((size_t)192 * kc * 16, 0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int c = 0; c < 32; ++c)
    for (int v = 0; v < 32; ++v) {
      const int m = c >> 1, mi = v & 15;
      const long double ang = -2.0L * pi * (long double)((m * mi) % 16) / 16.0L;
      const long double fr = cosl(ang), fi = sinl(ang);  // F = fr + i fi
      long double x;
      if ((c & 1) == 0) x = v < 16 ? fr : -fi;  // real part of the output
      else x = v < 16 ? fi : fr;                // imaginary part
      long long t = llroundl(x * 70368744177664.0L);  // 2^46
      int dig[6];
      for (int q = 5; q >= 1; --q) {
        const int d = (int)(signed char)(t & 0xFF);
        dig[q] = d;
        t = (t - d) >> 8;
      }
      dig[0] = (int)t;  // |t| <= 64
      for (int j = 0; j < 6; ++j)
        for (int e = 0; e < 2; ++e) {
          if (j - e < 0) continue;
          const int r = 32 * j + c, k = 2 * v + e;
          const size_t off = (size_t)(((r >> 3) * kc + k / 8) * 128 + (r & 7) * 16 + (k % 8) * 2);
          const uint16_t h = f16_int(dig[j - e]);
          memcpy(&out[off], &h, 2);
        }
    }
  return out;
}

}  // namespace fftoc
