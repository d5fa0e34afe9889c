// Host-side check of the exact-slice split form's arithmetic (fft_exact.cuh,
// exact_operand.h), compiled as host code: the 49-bit offset-binary digit
// cut, the library's B operand in its FP16 core-matrix layout, the twelve
// MMAs of a radix-16 pass emulated on the kernel's A layout (digit-pair K
// blocks, N = 192 / 128 / 64 into columns 64q..191), the exactness bound of
// every FP32 accumulator and the integer recombination, against the 16-point
// DFT in long double.  Prints "name value" lines.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <random>

#include "exact_operand.h"
#include "fft_exact.cuh"

using namespace fftoc;

static double f16_value(uint16_t h) {
  const int e = (h >> 10) & 31, m = h & 0x3FF;
  const double v = e == 0 ? std::ldexp((double)m, -24) : std::ldexp((double)(m | 0x400), e - 25);
  return (h & 0x8000) ? -v : v;
}

static double g_digit_bad = 0, g_acc_max = 0, g_pass_err = 0, g_cut_bad = 0, g_acc_inexact = 0, g_out_max = 0;

// digits of the kernel's cut: d_i = byte (5 - i) of the offset word - 128
// for i >= 1, d_0 = bits 40..49 - 256
template <int BS>
static void digits(long long x, int (&d)[6]) {
  const unsigned long long u = exact_offset_bits<BS>(x);
  d[0] = (int)((u >> 40) & 0x3FF) - 256;
  for (int i = 1; i < 6; ++i) d[i] = (int)((u >> (8 * (5 - i))) & 0xFF) - 128;
  // t = floor(x / 2^(BS - 48)) = sum d_i 256^(5-i), |d_0| <= 256
  const long long t = x >> (BS - 48);
  long long s = 0;
  for (int i = 0; i < 6; ++i) s = s * 256 + d[i];
  if (s != t || d[0] < -256 || d[0] > 256 || (u >> 50) != 0) g_cut_bad += 1;
  // the device's FP16 route, emulated: byte permutes of the offset word's
  // halves with 0x64 bytes (bit 48 into the top digit's exponent byte) give
  // FP16 pairs (1024 + byte, ...), and subtracting 1152 is exact
  auto prmt = [](unsigned a, unsigned b, unsigned sel) {
    const unsigned long long v = ((unsigned long long)b << 32) | a;
    unsigned r = 0;
    for (int i = 0; i < 4; ++i) r |= (unsigned)((v >> (8 * ((sel >> (4 * i)) & 7))) & 0xFF) << (8 * i);
    return r;
  };
  const unsigned lo = (unsigned)u, hi = (unsigned)(u >> 32);
  const unsigned w[3] = {prmt(hi | 0x00640000u, 0x64646464u, 0x4021), prmt(lo, 0x64646464u, 0x4243),
                         prmt(lo, 0x64646464u, 0x4041)};
  for (int q = 0; q < 3; ++q)
    for (int e = 0; e < 2; ++e) {
      const double biased = f16_value((uint16_t)(w[q] >> (16 * e)));
      const double bias = (q == 0 && e == 0) ? 1280.0 : 1152.0;
      if (biased - bias != (double)d[2 * q + e]) g_digit_bad += 1;
    }
}

template <int BS>
static void check_pass(std::mt19937_64& g, const std::vector<unsigned char>& bop, int trials) {
  const long long lim = (1LL << BS) - 1;
  std::uniform_int_distribution<long long> any(-lim, lim);
  std::uniform_int_distribution<int> pick(0, 5);
  auto bval = [&](int r, int k) {
    uint16_t h;
    memcpy(&h, &bop[(size_t)(((r >> 3) * 8 + k / 8) * 128 + (r & 7) * 16 + (k % 8) * 2)], 2);
    return f16_value(h);
  };
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int tr = 0; tr < trials; ++tr) {
    long long xr[16], xi[16];
    const int kind = pick(g);
    for (int i = 0; i < 16; ++i) {
      if (kind == 0) { xr[i] = lim; xi[i] = -lim; }  // extremes
      else if (kind == 1) { xr[i] = (i & 1) ? lim : -lim; xi[i] = (i & 2) ? -lim : lim; }
      else if (kind == 2) { xr[i] = any(g) >> 20; xi[i] = any(g) >> 20; }  // small values
      else { xr[i] = any(g); xi[i] = any(g); }
    }
    // A row: block q, K element 2v + e = digit 2q + e of value v
    double A[3][64];
    for (int v = 0; v < 32; ++v) {
      int d[6];
      digits<BS>(v < 16 ? xr[v] : xi[v - 16], d);
      for (int q = 0; q < 3; ++q)
        for (int e = 0; e < 2; ++e) A[q][2 * v + e] = (double)d[2 * q + e];
    }
    // the twelve MMAs: block q adds A_q . B[rows 0 .. 192 - 64q) to columns 64q..191
    double D[192] = {0};
    for (int q = 0; q < 3; ++q)
      for (int col = 64 * q; col < 192; ++col) {
        double s = 0;
        for (int k = 0; k < 64; ++k) s += A[q][k] * bval(col - 64 * q, k);
        D[col] += s;
      }
    for (int col = 0; col < 192; ++col) {
      if (std::fabs(D[col]) > g_acc_max) g_acc_max = std::fabs(D[col]);
    }
    // recombination per output (accumulators seeded with 1.5 * 2^23, read as
    // FP32 bit patterns) and comparison with the exact DFT of x, scaled by
    // 2^(54 - BS)
    auto bits = [](double acc) {
      const float f = (float)(acc + 12582912.0);
      if ((double)f != acc + 12582912.0) g_acc_inexact += 1;
      unsigned u;
      memcpy(&u, &f, 4);
      return u;
    };
    for (int m = 0; m < 16; ++m) {
      const long long yr = exact_combine(bits(D[2 * m]), bits(D[32 + 2 * m]), bits(D[64 + 2 * m]),
                                         bits(D[96 + 2 * m]), bits(D[128 + 2 * m]), bits(D[160 + 2 * m]));
      const long long yi = exact_combine(bits(D[2 * m + 1]), bits(D[33 + 2 * m]), bits(D[65 + 2 * m]),
                                         bits(D[97 + 2 * m]), bits(D[129 + 2 * m]), bits(D[161 + 2 * m]));
      long double er = 0, ei = 0;
      for (int k = 0; k < 16; ++k) {
        const long double ang = -2.0L * pi * (long double)((m * k) % 16) / 16.0L;
        const long double c = cosl(ang), s = sinl(ang);
        er += c * xr[k] - s * xi[k];
        ei += s * xr[k] + c * xi[k];
      }
      // error relative to the output bound 2^58.5 (modulus)
      const long double sc = ldexpl(1.0L, 54 - BS), bound = ldexpl(1.0L, 58) * sqrtl(2.0L);
      const double e = (double)(fabsl((long double)yr - er * sc) / bound + fabsl((long double)yi - ei * sc) / bound);
      if (e > g_pass_err) g_pass_err = e;
      const double mag = (double)std::max(std::llabs(yr), std::llabs(yi));
      if (mag > g_out_max) g_out_max = mag;
    }
  }
}

int main() {
  std::mt19937_64 g(11);
  const std::vector<unsigned char> bop = dft16_exact_operand();
  // every B entry is an integer digit |f| <= 128
  double bmax = 0;
  for (size_t i = 0; i < bop.size(); i += 2) {
    uint16_t h;
    memcpy(&h, &bop[i], 2);
    const double v = f16_value(h);
    if (v != std::floor(v)) bmax = 1e9;
    bmax = std::fmax(bmax, std::fabs(v));
  }
  check_pass<48>(g, bop, 400);  // first pass (inputs converted below 2^48)
  check_pass<59>(g, bop, 400);  // later passes
  std::printf("exact_cut_bad %g\n", g_cut_bad);
  std::printf("exact_digit_bad %g\n", g_digit_bad);
  std::printf("exact_b_max %g\n", bmax);
  std::printf("exact_acc_max %g\n", g_acc_max);
  std::printf("exact_pass_err %g\n", g_pass_err);
  std::printf("exact_acc_inexact %g\n", g_acc_inexact);
  std::printf("exact_out_log2 %g\n", std::log2(g_out_max));
  return 0;
}
