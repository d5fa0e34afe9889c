// Host-side check of the engine arithmetic in fft_core.cuh / fft_kernel.cuh:
// the radix-2/4/8/16 DFT kernels, complex twiddle products and the
// binary64 <-> block fixed-point conversions, compiled as host code and
// compared with long-double references.  Prints "name max_rel_err" lines.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "fft_kernel.cuh"

using namespace fftoc;

static long double cosl2pi(long long k, long long n) { return cosl(2.0L * 3.141592653589793238462643383279502884L * k / n); }
static long double sinl2pi(long long k, long long n) { return sinl(2.0L * 3.141592653589793238462643383279502884L * k / n); }

template <class E, int R>
static double check_dft(std::mt19937_64& g, double scale) {
  std::normal_distribution<double> nd(0.0, 1.0);
  double worst = 0;
  for (int trial = 0; trial < 200; ++trial) {
    typename E::S re[R], im[R];
    long double xr[R], xi[R];
    for (int i = 0; i < R; ++i) {
      const double a = nd(g) * scale, b = nd(g) * scale;
      re[i] = (typename E::S)a;
      im[i] = (typename E::S)b;
      xr[i] = (long double)re[i];
      xi[i] = (long double)im[i];
    }
    dft<E, R, 0, 1, R>(re, im);
    long double num = 0, den = 0;
    for (int k = 0; k < R; ++k) {
      long double sr = 0, si = 0;
      for (int j = 0; j < R; ++j) {
        const long double c = cosl2pi((long long)j * k % R, R), s = -sinl2pi((long long)j * k % R, R);
        sr += xr[j] * c - xi[j] * s;
        si += xr[j] * s + xi[j] * c;
      }
      num += (sr - (long double)re[k]) * (sr - (long double)re[k]) + (si - (long double)im[k]) * (si - (long double)im[k]);
      den += sr * sr + si * si;
    }
    const double e = (double)sqrtl(num / den);
    if (e > worst) worst = e;
  }
  return worst;
}

static void fx_tw(long double v, int* h, int* l) {
  const long long q = llroundl(v * 1152921504606846976.0L);
  *h = (int)(q >> 30);
  *l = (int)(q & ((1LL << 30) - 1));
}

static double check_fx_cmul(std::mt19937_64& g) {
  std::uniform_int_distribution<long long> ud(-(1LL << 60) + 1, (1LL << 60) - 1);
  double worst = 0;
  for (int trial = 0; trial < 20000; ++trial) {
    const int n = 4096, k = (int)(g() % n);
    const long double c = cosl2pi(k, n), s = -sinl2pi(k, n);
    int4 w;
    fx_tw(c, &w.x, &w.y);
    fx_tw(s, &w.z, &w.w);
    long long xr = ud(g), xi = ud(g);
    if (trial < 8) { xr = (trial & 1) ? (1LL << 61) - 1 : -(1LL << 61) + 1; xi = (trial & 2) ? (1LL << 61) - 1 : -(1LL << 61) + 1; }
    const long double er = (long double)xr * c - (long double)xi * s;
    const long double ei = (long double)xr * s + (long double)xi * c;
    EngFx::cmul(xr, xi, w);
    const long double d = sqrtl((er - xr) * (er - xr) + (ei - xi) * (ei - xi));
    // absolute error in units of the fixed-point LSB
    if ((double)d > worst) worst = (double)d;
  }
  return worst;
}

static double check_fx_mulc(std::mt19937_64& g) {
  std::uniform_int_distribution<long long> ud(-(1LL << 61) + 1, (1LL << 61) - 1);
  double worst = 0;
  const long double h = sqrtl(0.5L);
  for (int trial = 0; trial < 20000; ++trial) {
    long long x = ud(g);
    const long double e = (long double)x * h;
    const long long y = EngFx::mulc(x, Konst<EngFx>::h());
    const double d = (double)fabsl(e - (long double)y);
    if (d > worst) worst = d;
  }
  return worst;
}

// conversion round trip: x -> fixed -> binary64 must reproduce x to within
// the fixed-point LSB of the transform (relative to its largest element).
template <int NB>
static double check_conversions(std::mt19937_64& g) {
  std::normal_distribution<double> nd(0.0, 1.0);
  double worst = 0;
  const double scales[] = {1.0, 1e-300, 1e300, 3e-310, 1e-30, 1e30, 2.0};
  for (double sc : scales) {
    double x[64];
    int em = 0;
    for (int i = 0; i < 64; ++i) {
      x[i] = nd(g) * sc * (i == 5 ? 1e-12 : 1.0);
      if (i == 7) x[i] = 0.0;
      em = em > expo_of(hi_word(x[i])) ? em : expo_of(hi_word(x[i]));
    }
    constexpr int B = FxBits<NB>::B;
    const FxScale s = fx_scale<B>(em);
    double mx = 0;
    for (int i = 0; i < 64; ++i) mx = fmax(mx, fabs(x[i]));
    for (int i = 0; i < 64; ++i) {
      const long long f = fx_in(hi_word(x[i]), lo_word(x[i]), s.eref);
      const double y = s.slow ? fx_out_slow(f, s.K) : fx_out(f, s.kshift);
      const double e = fabs(y - x[i]) / mx;
      if (e > worst) worst = e;
    }
  }
  return worst;
}

// The fast input conversions (floor and truncating) against the general one
// of the same rounding over the fast path's domain: normal values whose exponent lies within 31 of eref (every size's
// B, random signs, mantissas and exponents).  Returns the mismatch count.
template <int NB>
static double check_fx_in_near(std::mt19937_64& g) {
  constexpr int B = FxBits<NB>::B;
  long long bad = 0;
  for (int trial = 0; trial < 200000; ++trial) {
    const int em = 1 + (int)(g() % 2046);
    const FxScale s = fx_scale<B>(em);
    const int lo_e = s.eref - 31 > 1 ? s.eref - 31 : 1;
    const int span = em - lo_e + 1;
    if (span <= 0) continue;
    const int e = lo_e + (int)(g() % (unsigned)span);
    const unsigned long long bits = g();
    const unsigned hw = (unsigned)(bits >> 32 & 0x800FFFFFu) | ((unsigned)e << 20);
    const unsigned lw = (unsigned)bits;
    if (fx_in_near(hw, lw, s.eref) != fx_in<false>(hw, lw, s.eref)) ++bad;
    if (fx_in_near_trunc(hw, lw, s.eref) != fx_in<true>(hw, lw, s.eref)) ++bad;
  }
  return (double)bad;
}

// The fast output conversion (exponent-field add, both zero tests) against
// ldexp over values whose results stay normal, including zero.  Returns the
// mismatch count.
static double check_fx_out(std::mt19937_64& g) {
  long long bad = 0;
  for (int trial = 0; trial < 300000; ++trial) {
    const int sh = (int)(g() % 62);
    long long x = (long long)(g() >> (2 + sh));  // magnitudes 2^0 .. 2^62
    if (g() & 1) x = -x;
    if (trial % 1000 == 0) x = 0;
    const int K = -1000 + (int)(g() % 1900);     // |x| 2^K within the normal range
    const int kshift = (int)((unsigned)K << 20);
    const double want = ldexp((double)x, K);
    const double a = fx_out<false>(x, kshift), b = fx_out<true>(x, kshift);
    if (memcmp(&a, &want, 8) != 0 || memcmp(&b, &want, 8) != 0) ++bad;
  }
  return (double)bad;
}

// The fixed-point constants of the DFT kernels: h*2^30 + l must be the
// nearest integer to v*2^60, with 0 <= l < 2^30.  Returns the largest
// distance from v*2^60 in units of the last place (at most 0.5), or 99 for a
// low limb out of range.
static double check_fx_konst() {
  using K = Konst<EngFx>;
  const long double pi = 3.141592653589793238462643383279502884L;
  const long double r2 = sqrtl(0.5L), c8 = cosl(pi / 8), s8 = sinl(pi / 8);
  const FxKC kc[] = {K::h(), K::nh(), K::c8(), K::s8(), K::nc8(), K::ns8()};
  const long double v[] = {r2, -r2, c8, s8, -c8, -s8};
  double worst = 0;
  for (int i = 0; i < 6; ++i) {
    if (kc[i].l < 0 || kc[i].l >= (1 << 30)) return 99;
    const long double q = (long double)kc[i].h * 1073741824.0L + (long double)kc[i].l;
    const double d = (double)fabsl(q - v[i] * 1152921504606846976.0L);
    if (d > worst) worst = d;
  }
  return worst;
}

int main() {
  std::mt19937_64 g(12345);
  printf("f64_dft2 %.3e\n", check_dft<EngF64, 2>(g, 1.0));
  printf("f64_dft4 %.3e\n", check_dft<EngF64, 4>(g, 1.0));
  printf("f64_dft8 %.3e\n", check_dft<EngF64, 8>(g, 1.0));
  printf("f64_dft16 %.3e\n", check_dft<EngF64, 16>(g, 1.0));
  const double fxs = 1e15;  // ~2^50 fixed-point magnitudes
  printf("fx_dft2 %.3e\n", check_dft<EngFx, 2>(g, fxs));
  printf("fx_dft4 %.3e\n", check_dft<EngFx, 4>(g, fxs));
  printf("fx_dft8 %.3e\n", check_dft<EngFx, 8>(g, fxs));
  printf("fx_dft16 %.3e\n", check_dft<EngFx, 16>(g, fxs));
  printf("fx_cmul_lsb %.3e\n", check_fx_cmul(g));
  printf("fx_mulc_lsb %.3e\n", check_fx_mulc(g));
  const double r1 = check_conversions<4096>(g), r2 = check_conversions<16>(g);
  printf("fx_roundtrip %.3e\n", r1 > r2 ? r1 : r2);
  printf("fx_in_near_mismatch %.0f\n", check_fx_in_near<8>(g) + check_fx_in_near<512>(g) + check_fx_in_near<4096>(g));
  printf("fx_out_mismatch %.0f\n", check_fx_out(g));
  printf("fx_konst_ulp %.3f\n", check_fx_konst());
  return 0;
}
