/*
 * fftoc oracle — CPU restatement of gprabowski/fft_onchip's batched forward
 * complex FFT path.  TEST INFRASTRUCTURE ONLY: the product library never links,
 * loads or calls anything in this file; tests, smoke() and the CPU-baseline leg
 * of bench.py use it to check and time results.
 *
 * Convention (reference includes/reference.cuh:10-12 — cuFFTDx C2C, forward,
 * double, no scaling; and every executor's pow_theta, e.g.
 * includes/tensor_fft_64.cuh:33-39 with angle p*(-2/N)*pi):
 *     X[k] = sum_n x[n] * exp(-2*pi*i*n*k/N),  natural order in and out.
 * Data layout (includes/config.hpp:6, thrust::complex<double>): interleaved
 * (re, im) doubles, transform b occupies complex elements [b*N, (b+1)*N).
 *
 * Contents
 *   - twiddles from exact rational angles in long double (octant reduction);
 *   - orc_dft_naive_ld: O(N^2) long-double DFT (checks everything else);
 *   - orc_fft_ld: radix-2 long-double FFT (ground truth at any batch);
 *   - orc_fft_f64: mixed radix-8/4/2 Stockham in double, OpenMP over the batch
 *     (the timed CPU baseline; same pass structure as includes/legacy8_fft.cuh);
 *   - orc_ref_tensor: lane-exact restatement of the reference's DMMA executors
 *     (tensor_fft_{8,64,128,256,512,4096}.cuh) on an emulated warp, using the
 *     m8n8k4.f64 fragment layout of includes/common.cuh:21-33;
 *   - orc_ref_legacy8 / orc_ref_legacy16: restatements of the radix-8 / radix-16
 *     Stockham executors (includes/legacy8_fft.cuh, includes/legacy16_fft.cuh).
 *   Each restatement runs with exact twiddles (mode 0) or with the reference's own
 *   twiddle sources (mode 1: FP32 sincospif, the 6-significant-digit table of
 *   includes/constants.cuh:7, the 12-digit constants of legacy8/16).
 *
 * Parity status: the reference ships no golden vectors, no fixtures and no
 * known-answer tests (its only check, src/gpu_fft.cu:41-66, prints an MSE
 * against cuFFTDx, which is absent here).  These restatements are checked
 * against the mathematics (naive DFT, analytic known answers), against
 * numpy.fft, and against the reference's own executors run on a GPU:
 * oracle/ref_runner.py launches them (compiled unmodified from the
 * reference's headers by oracle/build_ref.py) and recorded their outputs in
 * tests/golden/ref_out_*.npz, which tests/test_reference_pinning.py compares
 * with orc_ref_tensor / orc_ref_legacy8 / orc_ref_legacy16.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cd;
typedef struct { long double re, im; } cld;

#define ORC_PI_L 3.141592653589793238462643383279502884L

/* ------------------------------------------------------------------------- */
/* Twiddles: exp(-2*pi*i*k/n) from the exact rational angle k/n.              */
/* ------------------------------------------------------------------------- */

/* cos and sin of 2*pi*k/n in long double, reduced to |angle| <= pi/4. */
static void cs_ld(long long n, long long k, long double *c, long double *s) {
  k %= n;
  if (k < 0) k += n;
  /* angle = 2*pi*k/n = (pi/4) * (8k/n); octant o = floor(8k/n), remainder r/n */
  long long k8 = 8 * k;
  long long o = k8 / n;
  long long r = k8 - o * n; /* angle = (pi/4)*(o + r/n), 0 <= r < n */
  long double phi;
  int oct = (int)o;
  /* map to base angle in [0, pi/4] plus symmetry */
  long double cb, sb;
  if (oct & 1) {
    /* (pi/4)*(o+1) - (pi/4)*((n-r)/n) */
    phi = (ORC_PI_L / 4.0L) * ((long double)(n - r) / (long double)n);
    cb = cosl(phi);
    sb = sinl(phi);
    /* angle = (o+1)*pi/4 - phi, with o+1 even: quadrant q = (o+1)/2 */
    int q = ((oct + 1) / 2) & 3;
    /* cos(q*pi/2 - phi), sin(q*pi/2 - phi) */
    switch (q) {
      case 0: *c = cb; *s = -sb; break;
      case 1: *c = sb; *s = cb; break;
      case 2: *c = -cb; *s = sb; break;
      default: *c = -sb; *s = -cb; break;
    }
  } else {
    phi = (ORC_PI_L / 4.0L) * ((long double)r / (long double)n);
    cb = cosl(phi);
    sb = sinl(phi);
    int q = (oct / 2) & 3; /* angle = q*pi/2 + phi */
    switch (q) {
      case 0: *c = cb; *s = sb; break;
      case 1: *c = -sb; *s = cb; break;
      case 2: *c = -cb; *s = -sb; break;
      default: *c = sb; *s = -cb; break;
    }
  }
}

/* forward twiddle W_n^k = exp(-2*pi*i*k/n) */
static cld tw_ld(long long n, long long k) {
  long double c, s;
  cs_ld(n, k, &c, &s);
  cld w = {c, -s};
  return w;
}
static cd tw_d(long long n, long long k) {
  cld w = tw_ld(n, k);
  cd r = {(double)w.re, (double)w.im};
  return r;
}

void orc_twiddle(long long n, long long k, double *re, double *im) {
  cd w = tw_d(n, k);
  *re = w.re;
  *im = w.im;
}

/* ------------------------------------------------------------------------- */
/* Ground truth                                                               */
/* ------------------------------------------------------------------------- */

/* O(N^2) DFT of `batch` transforms in long double; output rounded to double. */
void orc_dft_naive_ld(int n, long long batch, const double *in, double *out) {
  cld *w = (cld *)malloc(sizeof(cld) * (size_t)n);
  for (int k = 0; k < n; ++k) w[k] = tw_ld(n, k);
  for (long long b = 0; b < batch; ++b) {
    const double *x = in + 2 * (size_t)n * b;
    double *y = out + 2 * (size_t)n * b;
    for (int k = 0; k < n; ++k) {
      long double sr = 0, si = 0;
      for (int j = 0; j < n; ++j) {
        cld t = w[((long long)j * k) % n];
        long double xr = x[2 * j], xi = x[2 * j + 1];
        sr += xr * t.re - xi * t.im;
        si += xr * t.im + xi * t.re;
      }
      y[2 * k] = (double)sr;
      y[2 * k + 1] = (double)si;
    }
  }
  free(w);
}

static int ilog2(long long n) {
  int l = 0;
  while ((1LL << l) < n) ++l;
  return l;
}

/* Iterative radix-2 DIT FFT in long double (bit-reversed load). */
void orc_fft_ld(int n, long long batch, const double *in, double *out) {
  int lg = ilog2(n);
  cld *w = (cld *)malloc(sizeof(cld) * (size_t)(n / 2 > 0 ? n / 2 : 1));
  for (int k = 0; k < n / 2; ++k) w[k] = tw_ld(n, k);
  cld *a = (cld *)malloc(sizeof(cld) * (size_t)n);
  for (long long b = 0; b < batch; ++b) {
    const double *x = in + 2 * (size_t)n * b;
    for (int i = 0; i < n; ++i) {
      int r = 0;
      for (int bit = 0; bit < lg; ++bit) r |= ((i >> bit) & 1) << (lg - 1 - bit);
      a[r].re = x[2 * i];
      a[r].im = x[2 * i + 1];
    }
    for (int len = 2; len <= n; len <<= 1) {
      int half = len / 2, step = n / len;
      for (int s = 0; s < n; s += len) {
        for (int j = 0; j < half; ++j) {
          cld t = w[j * step];
          cld u = a[s + j], v = a[s + j + half];
          cld vt = {v.re * t.re - v.im * t.im, v.re * t.im + v.im * t.re};
          a[s + j].re = u.re + vt.re;
          a[s + j].im = u.im + vt.im;
          a[s + j + half].re = u.re - vt.re;
          a[s + j + half].im = u.im - vt.im;
        }
      }
    }
    double *y = out + 2 * (size_t)n * b;
    for (int i = 0; i < n; ++i) {
      y[2 * i] = (double)a[i].re;
      y[2 * i + 1] = (double)a[i].im;
    }
  }
  free(a);
  free(w);
}

/* ------------------------------------------------------------------------- */
/* FP64 Stockham (timed CPU baseline).  Pass structure follows the reference's */
/* radix-8 Stockham executor (includes/legacy8_fft.cuh:57-119): for pass with  */
/* span p, element j = t + m*(N/R) is twiddled by W_{R p}^{k m} with           */
/* k = t mod p and written to ((t - k) * R) + k + m*p.  Radix 4 and 2 finish   */
/* sizes that are not powers of 8.                                             */
/* ------------------------------------------------------------------------- */

typedef struct {
  int n;
  int npass;
  int radix[16];
  cd *tw[16]; /* per pass: twiddle W_{R p}^{k m}, index [k*R + m] */
} stock_plan;

static void stock_plan_make(stock_plan *pl, int n) {
  memset(pl, 0, sizeof(*pl));
  pl->n = n;
  int rem = n, p = 1;
  while (rem > 1) {
    int r = (rem % 8 == 0) ? 8 : (rem % 4 == 0 ? 4 : 2);
    int i = pl->npass++;
    pl->radix[i] = r;
    pl->tw[i] = (cd *)malloc(sizeof(cd) * (size_t)p * r);
    for (int k = 0; k < p; ++k)
      for (int m = 0; m < r; ++m) pl->tw[i][k * r + m] = tw_d((long long)r * p, (long long)k * m);
    p *= r;
    rem /= r;
  }
}
static void stock_plan_free(stock_plan *pl) {
  for (int i = 0; i < pl->npass; ++i) free(pl->tw[i]);
}

static inline cd cmul(cd a, cd b) {
  cd r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}

/* small in-register DFT of size r (2,4,8), forward */
static void dft_small(int r, cd *u) {
  static const double h = 0.70710678118654752440;
  if (r == 2) {
    cd a = u[0], b = u[1];
    u[0].re = a.re + b.re; u[0].im = a.im + b.im;
    u[1].re = a.re - b.re; u[1].im = a.im - b.im;
    return;
  }
  if (r == 4) {
    cd a0 = {u[0].re + u[2].re, u[0].im + u[2].im};
    cd a1 = {u[0].re - u[2].re, u[0].im - u[2].im};
    cd b0 = {u[1].re + u[3].re, u[1].im + u[3].im};
    cd b1 = {u[1].re - u[3].re, u[1].im - u[3].im};
    /* -i * b1 */
    cd mb1 = {b1.im, -b1.re};
    u[0].re = a0.re + b0.re; u[0].im = a0.im + b0.im;
    u[2].re = a0.re - b0.re; u[2].im = a0.im - b0.im;
    u[1].re = a1.re + mb1.re; u[1].im = a1.im + mb1.im;
    u[3].re = a1.re - mb1.re; u[3].im = a1.im - mb1.im;
    return;
  }
  /* r == 8: radix-2 then two radix-4 */
  cd e[4] = {u[0], u[2], u[4], u[6]}, o[4] = {u[1], u[3], u[5], u[7]};
  dft_small(4, e);
  dft_small(4, o);
  cd w1 = {h, -h}, w3 = {-h, -h};
  cd t0 = o[0], t1 = cmul(o[1], w1), t2 = {o[2].im, -o[2].re}, t3 = cmul(o[3], w3);
  cd t[4] = {t0, t1, t2, t3};
  for (int k = 0; k < 4; ++k) {
    u[k].re = e[k].re + t[k].re; u[k].im = e[k].im + t[k].im;
    u[k + 4].re = e[k].re - t[k].re; u[k + 4].im = e[k].im - t[k].im;
  }
}

static void stock_run(const stock_plan *pl, const cd *x, cd *y, cd *scratch) {
  int n = pl->n;
  if (n == 1) { y[0] = x[0]; return; }
  const cd *src = x;
  cd *bufs[2];
  /* final pass must land in y */
  bufs[(pl->npass - 1) & 1] = y;
  bufs[pl->npass & 1] = scratch;
  int p = 1;
  for (int i = 0; i < pl->npass; ++i) {
    int r = pl->radix[i];
    int B = n / r;
    cd *dst = bufs[i & 1];
    const cd *tw = pl->tw[i];
    for (int t = 0; t < B; ++t) {
      int k = t & (p - 1); /* p is a power of two */
      cd u[8];
      for (int m = 0; m < r; ++m) {
        cd v = src[t + m * B];
        u[m] = (k == 0) ? v : cmul(v, tw[k * r + m]);
      }
      dft_small(r, u);
      int base = (t - k) * r + k;
      for (int m = 0; m < r; ++m) dst[base + m * p] = u[m];
    }
    src = dst;
    p *= r;
  }
}

/* Batched FP64 forward FFT on `threads` host threads (<=0: all). */
void orc_fft_f64(int n, long long batch, const double *in, double *out, int threads) {
  stock_plan pl;
  stock_plan_make(&pl, n);
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
  {
    cd *scratch = (cd *)malloc(sizeof(cd) * (size_t)n);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long long b = 0; b < batch; ++b)
      stock_run(&pl, (const cd *)(in + 2 * (size_t)n * b), (cd *)(out + 2 * (size_t)n * b), scratch);
    free(scratch);
  }
  stock_plan_free(&pl);
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Lane-exact restatement of the reference's DMMA executors.                  */
/* ------------------------------------------------------------------------- */

/* Twiddle source of the reference executors. */
enum { TW_EXACT = 0, TW_REFERENCE = 1 };

/* pow_theta<N>(p) with FP32 sincospif: includes/tensor_fft_64.cuh:33-39.
 * sincospif is modelled by the correctly rounded sin/cos of pi*ang. */
static cd pt_f32(int N, int p) {
  p = p % N;
  float ang = (float)p * (-2.f / (float)N);
  float s = (float)sin(M_PI * (double)ang), c = (float)cos(M_PI * (double)ang);
  cd r = {c, s};
  return r;
}
/* pow_theta<N>(p) through constants::twiddles (includes/tensor_fft_256.cuh:25-28):
 * a table of W_256^k printed at 6 significant digits (includes/constants.cuh:7). */
static double six_digits(double v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.6g", v);
  return strtod(buf, NULL);
}
static cd pt_table6(int N, int p) {
  int idx = (p & (N - 1)) * 256 / N;
  cd w = tw_d(256, idx);
  cd r = {six_digits(w.re), six_digits(w.im)};
  return r;
}
static cd pt_exact(int N, int p) { return tw_d(N, p); }

typedef cd (*pt_fn)(int, int);

/* mma.sync.aligned.m8n8k4.row.col.f64 on an emulated warp.
 * Fragment layout (includes/common.cuh:21-33 and the PTX ISA):
 *   A 8x4 row-major: lane l holds A[l>>2][l&3]
 *   B 4x8 col-major: lane l holds B[l&3][l>>2]
 *   C/D 8x8:         lane l holds D[l>>2][2(l&3)] and D[l>>2][2(l&3)+1]      */
static void mma884(const double a[32], const double b[32], double c0[32], double c1[32]) {
  double A[8][4], B[4][8];
  for (int l = 0; l < 32; ++l) {
    A[l >> 2][l & 3] = a[l];
    B[l & 3][l >> 2] = b[l];
  }
  for (int l = 0; l < 32; ++l) {
    int row = l >> 2, col = 2 * (l & 3);
    double s0 = c0[l], s1 = c1[l];
    for (int k = 0; k < 4; ++k) {
      s0 = fma(A[row][k], B[k][col], s0);
      s1 = fma(A[row][k], B[k][col + 1], s1);
    }
    c0[l] = s0;
    c1[l] = s1;
  }
}

/* mma8x8x8 = two k4 MMAs (includes/tensor_utils.cuh:13-15). */
static void mma888(const double a1[32], const double a2[32], const double b1[32], const double b2[32],
                   double c1[32], double c2[32]) {
  mma884(a1, b1, c1, c2);
  mma884(a2, b2, c1, c2);
}

/* Karatsuba complex 8x8x8 GEMM, 3 real GEMMs (includes/tensor_utils.cuh:32-36):
 * s1 = Ar Br, s2 = Ai Bi, s3 = (Ar+Ai)(Br+Bi); then (re, im) = (s1-s2, s3-s2-s1).
 * Results are written back into b1/b2 (the caller's register reuse). */
static void kara(const cd a1[32], const cd a2[32], cd b1[32], cd b2[32]) {
  double ar1[32], ar2[32], ai1[32], ai2[32], as1[32], as2[32];
  double br1[32], br2[32], bi1[32], bi2[32], bs1[32], bs2[32];
  double s11[32] = {0}, s12[32] = {0}, s21[32] = {0}, s22[32] = {0}, s31[32] = {0}, s32[32] = {0};
  for (int l = 0; l < 32; ++l) {
    ar1[l] = a1[l].re; ar2[l] = a2[l].re; ai1[l] = a1[l].im; ai2[l] = a2[l].im;
    as1[l] = a1[l].re + a1[l].im; as2[l] = a2[l].re + a2[l].im;
    br1[l] = b1[l].re; br2[l] = b2[l].re; bi1[l] = b1[l].im; bi2[l] = b2[l].im;
    bs1[l] = b1[l].re + b1[l].im; bs2[l] = b2[l].re + b2[l].im;
  }
  mma888(ar1, ar2, br1, br2, s11, s12);
  mma888(ai1, ai2, bi1, bi2, s21, s22);
  mma888(as1, as2, bs1, bs2, s31, s32);
  for (int l = 0; l < 32; ++l) {
    b1[l].re = s11[l] - s21[l];
    b1[l].im = s31[l] - s21[l] - s11[l];
    b2[l].re = s12[l] - s22[l];
    b2[l].im = s32[l] - s22[l] - s12[l];
  }
}

/* c64_fft64 (includes/c64_fft64.cuh:8-27): GEMM, twiddle, GEMM on the same
 * fragments; the C fragment is reused as the next B fragment. */
static void c64(const cd a1[32], const cd a2[32], cd b1[32], cd b2[32], const cd t1[32], const cd t2[32]) {
  kara(a1, a2, b1, b2);
  for (int l = 0; l < 32; ++l) {
    b1[l] = cmul(t1[l], b1[l]);
    b2[l] = cmul(t2[l], b2[l]);
  }
  kara(a1, a2, b1, b2);
}

#define AROW(l) ((l) >> 2)
#define ACOL(l) ((l) & 3)
#define BROW(l) ((l) & 3)
#define BCOL(l) ((l) >> 2)
#define CROW(l) ((l) >> 2)
#define CCOL(l) (2 * ((l) & 3))

/* tensor_fft_8 (includes/tensor_fft_8.cuh:37-65): 8 transforms per GEMM,
 * B column = transform.  d holds 8 consecutive transforms. */
static void ref_t8(cd *d, pt_fn pt) {
  cd a1[32], a2[32], b1[32], b2[32];
  for (int l = 0; l < 32; ++l) {
    a1[l] = pt(8, AROW(l) * ACOL(l));
    a2[l] = pt(8, AROW(l) * (ACOL(l) + 4));
    b1[l] = d[BROW(l) + BCOL(l) * 8];
    b2[l] = d[(BROW(l) + 4) + BCOL(l) * 8];
  }
  kara(a1, a2, b1, b2);
  for (int l = 0; l < 32; ++l) {
    d[CROW(l) + CCOL(l) * 8] = b1[l];
    d[CROW(l) + (CCOL(l) + 1) * 8] = b2[l];
  }
}

static void f64_frags(cd a1[32], cd a2[32], cd t1[32], cd t2[32], pt_fn pt) {
  for (int l = 0; l < 32; ++l) {
    t1[l] = pt(64, CROW(l) * CCOL(l));
    t2[l] = pt(64, CROW(l) * (CCOL(l) + 1));
    a1[l] = pt(8, AROW(l) * (2 * ACOL(l)));
    a2[l] = pt(8, AROW(l) * (2 * ACOL(l) + 1));
  }
}

/* tensor_fft_64 (includes/tensor_fft_64.cuh:43-76), FPU = 1. */
static void ref_t64(cd *d, pt_fn pt) {
  cd a1[32], a2[32], t1[32], t2[32], b1[32], b2[32];
  f64_frags(a1, a2, t1, t2, pt);
  for (int l = 0; l < 32; ++l) {
    b1[l] = d[(BROW(l) * 2) * 8 + BCOL(l)];
    b2[l] = d[(BROW(l) * 2 + 1) * 8 + BCOL(l)];
  }
  c64(a1, a2, b1, b2, t1, t2);
  for (int l = 0; l < 32; ++l) {
    d[CROW(l) * 8 + CCOL(l)] = b1[l];
    d[CROW(l) * 8 + CCOL(l) + 1] = b2[l];
  }
}

/* tensor_fft_128 (includes/tensor_fft_128.cuh:43-98), FPU = 1: two c64 on the
 * even/odd samples, then a radix-2 combine with W_128. */
static void ref_t128(cd *d, pt_fn pt) {
  cd a1[32], a2[32], t1[32], t2[32], b0[32], b1[32], b2[32], b3[32];
  f64_frags(a1, a2, t1, t2, pt);
  for (int l = 0; l < 32; ++l) {
    int bpos = (BROW(l) * 2) * 32 + BCOL(l) * 4;
    b0[l] = d[bpos / 2];
    b1[l] = d[bpos / 2 + 16];
    b2[l] = d[1 + bpos / 2];
    b3[l] = d[1 + bpos / 2 + 16];
  }
  c64(a1, a2, b0, b1, t1, t2);
  c64(a1, a2, b2, b3, t1, t2);
  for (int l = 0; l < 32; ++l) {
    int o = CROW(l) * 8 + CCOL(l);
    cd w4 = pt(128, o), w5 = pt(128, o + 1);
    cd tmp = cmul(b2[l], w4);
    cd x2 = {b0[l].re - tmp.re, b0[l].im - tmp.im};
    cd x0 = {b0[l].re + tmp.re, b0[l].im + tmp.im};
    d[o] = x0;
    d[o + 64] = x2;
    tmp = cmul(b3[l], w5);
    cd x3 = {b1[l].re - tmp.re, b1[l].im - tmp.im};
    cd x1 = {b1[l].re + tmp.re, b1[l].im + tmp.im};
    d[o + 1] = x1;
    d[o + 65] = x3;
  }
}

/* tensor_fft_256 (includes/tensor_fft_256.cuh:34-122), FPU = 1: radix-8 GEMM,
 * W_32 twiddle, register radix-4, W_256 twiddle, radix-8 GEMM. */
static void ref_t256(cd *d, pt_fn pt) {
  cd a1[32], a2[32], b[8][32];
  for (int l = 0; l < 32; ++l) {
    a1[l] = pt(8, AROW(l) * (2 * ACOL(l)));
    a2[l] = pt(8, AROW(l) * (2 * ACOL(l) + 1));
  }
  for (int j = 0; j < 4; ++j) {
    for (int l = 0; l < 32; ++l) {
      b[2 * j][l] = d[8 * j + BROW(l) * 2 * 32 + BCOL(l)];
      b[2 * j + 1][l] = d[8 * j + (BROW(l) * 2 + 1) * 32 + BCOL(l)];
    }
    kara(a1, a2, b[2 * j], b[2 * j + 1]);
  }
  for (int l = 0; l < 32; ++l) {
    int r = CROW(l);
    b[2][l] = cmul(b[2][l], pt(32, r));
    b[4][l] = cmul(b[4][l], pt(32, 2 * r));
    b[6][l] = cmul(b[6][l], pt(32, 3 * r));
    b[3][l] = cmul(b[3][l], pt(32, r));
    b[5][l] = cmul(b[5][l], pt(32, 2 * r));
    b[7][l] = cmul(b[7][l], pt(32, 3 * r));
    cd v[8];
    for (int q = 0; q < 8; ++q) v[q] = b[q][l];
    cd t1 = {v[0].re + v[4].re, v[0].im + v[4].im}, t2 = {v[0].re - v[4].re, v[0].im - v[4].im};
    cd t3 = {v[1].re + v[5].re, v[1].im + v[5].im}, t4 = {v[1].re - v[5].re, v[1].im - v[5].im};
    cd t5 = {v[2].re + v[6].re, v[2].im + v[6].im}, t6 = {v[2].re - v[6].re, v[2].im - v[6].im};
    cd t7 = {v[3].re + v[7].re, v[3].im + v[7].im}, t8 = {v[3].re - v[7].re, v[3].im - v[7].im};
    cd t9 = {-t6.im, t6.re}, t10 = {-t8.im, t8.re};
    b[0][l] = (cd){t1.re + t5.re, t1.im + t5.im};
    b[1][l] = (cd){t3.re + t7.re, t3.im + t7.im};
    b[2][l] = (cd){t2.re - t9.re, t2.im - t9.im};
    b[3][l] = (cd){t4.re - t10.re, t4.im - t10.im};
    b[4][l] = (cd){t1.re - t5.re, t1.im - t5.im};
    b[5][l] = (cd){t3.re - t7.re, t3.im - t7.im};
    b[6][l] = (cd){t2.re + t9.re, t2.im + t9.im};
    b[7][l] = (cd){t4.re + t10.re, t4.im + t10.im};
  }
  for (int j = 0; j < 4; ++j) {
    for (int l = 0; l < 32; ++l) {
      b[2 * j][l] = cmul(b[2 * j][l], pt(256, BROW(l) * 2 * (BCOL(l) + j * 8)));
      b[2 * j + 1][l] = cmul(b[2 * j + 1][l], pt(256, (BROW(l) * 2 + 1) * (BCOL(l) + j * 8)));
    }
    kara(a1, a2, b[2 * j], b[2 * j + 1]);
    for (int l = 0; l < 32; ++l) {
      d[(CCOL(l) + j * 8) + CROW(l) * 32] = b[2 * j][l];
      d[(CCOL(l) + 1 + j * 8) + CROW(l) * 32] = b[2 * j + 1][l];
    }
  }
}

/* tensor_fft_512 (includes/tensor_fft_512.cuh:45-118), FPU = 1, two warps. */
static void ref_t512(cd *d, pt_fn pt) {
  cd a1[32], a2[32], t1[32], t2[32];
  f64_frags(a1, a2, t1, t2, pt);
  cd lb[2][8][32];
  for (int w = 0; w < 2; ++w) {
    for (int i = 0; i < 4; ++i) {
      cd *x = lb[w][2 * i], *y = lb[w][2 * i + 1];
      for (int l = 0; l < 32; ++l) {
        int bpos = (BROW(l) * 2) * 32 + BCOL(l) * 4;
        x[l] = d[2 * i + w + bpos * 2];
        y[l] = d[2 * i + w + bpos * 2 + 64];
      }
      c64(a1, a2, x, y, t1, t2);
      for (int l = 0; l < 32; ++l) {
        d[2 * i + w + CROW(l) * 64 + CCOL(l) * 8] = x[l];
        d[2 * i + w + CROW(l) * 64 + (CCOL(l) + 1) * 8] = y[l];
      }
    }
  }
  /* fft_group.sync() */
  for (int w = 0; w < 2; ++w) {
    for (int i = 0; i < 4; ++i) {
      cd *x = lb[w][2 * i], *y = lb[w][2 * i + 1];
      for (int l = 0; l < 32; ++l) {
        int load_col = BCOL(l) + (w + 2 * i) * 8;
        cd tw3 = pt(512, load_col * 2 * BROW(l));
        cd tw4 = pt(512, load_col * (2 * BROW(l) + 1));
        const cd *ld = d + (w + 2 * i) * 64;
        x[l] = cmul(tw3, ld[BROW(l) * 2 + BCOL(l) * 8]);
        y[l] = cmul(tw4, ld[BROW(l) * 2 + 1 + BCOL(l) * 8]);
      }
      kara(a1, a2, x, y);
    }
  }
  /* fft_group.sync() */
  for (int w = 0; w < 2; ++w) {
    for (int i = 0; i < 4; ++i) {
      for (int l = 0; l < 32; ++l) {
        int e = CCOL(l) + (w + 2 * i) * 8;
        d[e + CROW(l) * 64] = lb[w][2 * i][l];
        d[e + 1 + CROW(l) * 64] = lb[w][2 * i + 1][l];
      }
    }
  }
}

/* tensor_fft_4096 (includes/tensor_fft_4096.cuh:54-96), 16 warps.  Note that
 * its A fragments split K as {0..3},{4..7} (:31-32) while c64_fft64 reuses the
 * C fragment as B with an even/odd K split; the restatement keeps that as is. */
static void ref_t4096(cd *sh, pt_fn pt) {
  cd a1[32], a2[32], t1[32], t2[32];
  for (int l = 0; l < 32; ++l) {
    t1[l] = pt(64, CROW(l) * CCOL(l));
    t2[l] = pt(64, CROW(l) * (CCOL(l) + 1));
    a1[l] = pt(8, AROW(l) * ACOL(l));
    a2[l] = pt(8, AROW(l) * (ACOL(l) + 4));
  }
  static cd lb[16][8][32];
  for (int w = 0; w < 16; ++w) {
    for (int i = w; i < 64; i += 16) {
      cd b1[32], b2[32];
      for (int l = 0; l < 32; ++l) {
        int bri = BROW(l) * 8 + BCOL(l);
        b1[l] = sh[i + bri * 64];
        b2[l] = sh[i + (bri + 32) * 64];
      }
      c64(a1, a2, b1, b2, t1, t2);
      for (int l = 0; l < 32; ++l) {
        int cri = CROW(l) * 8 + CCOL(l);
        sh[i + cri * 64] = b1[l];
        sh[i + (cri + 1) * 64] = b2[l];
      }
    }
  }
  for (int w = 0; w < 16; ++w) {
    for (int i = w; i < 64; i += 16) {
      int reg = 2 * (i / 16);
      for (int l = 0; l < 32; ++l) {
        int bri = BROW(l) * 8 + BCOL(l);
        cd tw3 = pt(4096, i * bri), tw4 = pt(4096, i * (bri + 32));
        lb[w][reg][l] = cmul(tw3, sh[i * 64 + bri]);
        lb[w][reg + 1][l] = cmul(tw4, sh[i * 64 + (bri + 32)]);
      }
      c64(a1, a2, lb[w][reg], lb[w][reg + 1], t1, t2);
    }
  }
  for (int w = 0; w < 16; ++w) {
    for (int i = w; i < 64; i += 16) {
      int reg = 2 * (i / 16);
      for (int l = 0; l < 32; ++l) {
        int cri = CROW(l) * 8 + CCOL(l);
        sh[i + cri * 64] = lb[w][reg][l];
        sh[i + (cri + 1) * 64] = lb[w][reg + 1][l];
      }
    }
  }
}

/* Run one of the reference's DMMA executors over a batch.
 * n in {8, 64, 128, 256, 512, 4096}; tw_mode: 0 exact twiddles, 1 the
 * reference's own.  Returns 0, or -1 for an unsupported n. */
int orc_ref_tensor(int n, long long batch, const double *in, double *out, int tw_mode) {
  pt_fn pt = pt_exact;
  if (tw_mode == TW_REFERENCE) pt = (n == 256) ? pt_table6 : pt_f32;
  if (n == 8) {
    cd tile[64];
    for (long long b0 = 0; b0 < batch; b0 += 8) {
      long long cnt = batch - b0 < 8 ? batch - b0 : 8;
      memset(tile, 0, sizeof tile);
      memcpy(tile, in + 16 * b0, sizeof(cd) * 8 * (size_t)cnt);
      ref_t8(tile, pt);
      memcpy(out + 16 * b0, tile, sizeof(cd) * 8 * (size_t)cnt);
    }
    return 0;
  }
  void (*fn)(cd *, pt_fn) = NULL;
  switch (n) {
    case 64: fn = ref_t64; break;
    case 128: fn = ref_t128; break;
    case 256: fn = ref_t256; break;
    case 512: fn = ref_t512; break;
    case 4096: fn = ref_t4096; break;
    default: return -1;
  }
  cd *tile = (cd *)malloc(sizeof(cd) * (size_t)n);
  for (long long b = 0; b < batch; ++b) {
    memcpy(tile, in + 2 * (size_t)n * b, sizeof(cd) * (size_t)n);
    fn(tile, pt);
    memcpy(out + 2 * (size_t)n * b, tile, sizeof(cd) * (size_t)n);
  }
  free(tile);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Legacy CUDA-core executors.                                                */
/* ------------------------------------------------------------------------- */

/* pow_theta(p, N) with double sincospi (includes/legacy8_fft.cuh:25-30). */
static cd pt_sincospi(int p, int N) {
  p = p & (N - 1);
  double ang = p * (-2.0 / N);
  cd r = {cos(M_PI * ang), sin(M_PI * ang)};
  return r;
}

/* sqr_1 (includes/legacy8_fft.cuh:37-40): a^2 */
static cd sqr1(cd a) {
  cd r = {a.re * a.re - a.im * a.im, 2.0 * a.re * a.im};
  return r;
}

/* includes/legacy8_fft.cuh:57-119 — radix-8 Stockham, N/8 threads, log8 N
 * passes; twiddle powers by repeated squaring.  Valid for N a power of 8. */
static void ref_legacy8_one(cd *sh, int N, int exact) {
  const int BS = N / 8;
  const double S = exact ? 0.70710678118654752440 : 0.707106781188; /* :44 */
  cd *u = (cd *)malloc(sizeof(cd) * 8 * (size_t)BS);
  int p = 1;
  for (int depth = 0; p < N; ++depth) {
    for (int tid = 0; tid < BS; ++tid) { /* loads of every thread (before the 2nd __syncthreads) */
      int k = tid & (p - 1);
      cd tw = exact ? tw_d(8 * p, k) : pt_sincospi(k, 8 * p);
      cd *v = u + 8 * tid;
      for (int m = 0; m < 8; ++m) v[m] = sh[tid + m * BS];
      v[1] = cmul(tw, v[1]); v[3] = cmul(tw, v[3]); v[5] = cmul(tw, v[5]); v[7] = cmul(tw, v[7]);
      tw = sqr1(tw);
      v[2] = cmul(tw, v[2]); v[3] = cmul(tw, v[3]); v[6] = cmul(tw, v[6]); v[7] = cmul(tw, v[7]);
      tw = sqr1(tw);
      v[4] = cmul(tw, v[4]); v[5] = cmul(tw, v[5]); v[6] = cmul(tw, v[6]); v[7] = cmul(tw, v[7]);
    }
    for (int tid = 0; tid < BS; ++tid) {
      int k = tid & (p - 1);
      cd *v = u + 8 * tid;
      cd *o = sh + ((tid - k) << 3) + k;
#define ADD(a, b) ((cd){(a).re + (b).re, (a).im + (b).im})
#define SUB(a, b) ((cd){(a).re - (b).re, (a).im - (b).im})
      cd v0 = ADD(v[0], v[4]), v4 = SUB(v[0], v[4]);
      cd v1 = ADD(v[1], v[5]), d5 = SUB(v[1], v[5]);
      cd v5 = {S * (d5.re + d5.im), S * (-d5.re + d5.im)}; /* b14 */
      cd v2 = ADD(v[2], v[6]), d6 = SUB(v[2], v[6]);
      cd v6 = {d6.im, -d6.re}; /* b24 */
      cd v3 = ADD(v[3], v[7]), d7 = SUB(v[3], v[7]);
      cd v7 = {S * (-d7.re + d7.im), S * (-d7.re - d7.im)}; /* b34 */
      cd u0 = ADD(v0, v2), u2 = SUB(v0, v2);
      cd u1 = ADD(v1, v3), d13 = SUB(v1, v3);
      cd u3 = {d13.im, -d13.re}; /* b12 */
      cd u4 = ADD(v4, v6), u6 = SUB(v4, v6);
      cd u5 = ADD(v5, v7), d57 = SUB(v5, v7);
      cd u7 = {d57.im, -d57.re};
      o[0] = ADD(u0, u1); o[p] = ADD(u4, u5); o[2 * p] = ADD(u2, u3); o[3 * p] = ADD(u6, u7);
      o[4 * p] = SUB(u0, u1); o[5 * p] = SUB(u4, u5); o[6 * p] = SUB(u2, u3); o[7 * p] = SUB(u6, u7);
    }
    p *= 8;
  }
  free(u);
}

int orc_ref_legacy8(int n, long long batch, const double *in, double *out, int tw_mode) {
  if (n != 8 && n != 64 && n != 512 && n != 4096) return -1;
  cd *t = (cd *)malloc(sizeof(cd) * (size_t)n);
  for (long long b = 0; b < batch; ++b) {
    memcpy(t, in + 2 * (size_t)n * b, sizeof(cd) * (size_t)n);
    ref_legacy8_one(t, n, tw_mode == TW_EXACT);
    memcpy(out + 2 * (size_t)n * b, t, sizeof(cd) * (size_t)n);
  }
  free(t);
  return 0;
}

/* includes/legacy16_fft.cuh:220-292 — radix-16 Stockham, 4 layers of dft2
 * with constant twiddles (:169-210).  Valid for N a power of 16. */
typedef struct { double c8, s8, h; } l16c;

static cd l16_mul(int code, cd a, const l16c *K) {
  /* code = rotation by W_16^code (forward), code in 0..7 */
  switch (code) {
    case 0: return a;
    case 1: return cmul((cd){K->c8, -K->s8}, a);
    case 2: return (cd){K->h * (a.re + a.im), K->h * (-a.re + a.im)};
    case 3: return cmul((cd){K->s8, -K->c8}, a);
    case 4: return (cd){a.im, -a.re};
    case 5: return cmul((cd){-K->s8, -K->c8}, a);
    case 6: return (cd){K->h * (-a.re + a.im), K->h * (-a.re - a.im)};
    default: return cmul((cd){-K->c8, -K->s8}, a);
  }
}
static void dft2t(cd *a, cd *b, int code, const l16c *K) {
  cd t = l16_mul(code, SUB(*a, *b), K);
  *a = ADD(*a, *b);
  *b = t;
}

static void ref_legacy16_one(cd *sh, int N, int exact) {
  const int BS = N / 16;
  l16c K;
  if (exact) {
    K.h = 0.70710678118654752440; K.c8 = 0.92387953251128675613; K.s8 = 0.38268343236508977173;
  } else { /* includes/legacy16_fft.cuh:13-15 */
    K.h = 0.707106781188; K.c8 = 0.923879532511; K.s8 = 0.382683432365;
  }
  cd *U = (cd *)malloc(sizeof(cd) * 16 * (size_t)BS);
  int p = 1;
  while (p < N) {
    for (int tid = 0; tid < BS; ++tid) {
      int k = tid & (p - 1);
      cd *u = U + 16 * tid;
      for (int m = 0; m < 16; ++m) u[m] = sh[tid + m * BS];
      for (int m = 1; m < 16; ++m) u[m] = cmul(exact ? tw_d(16 * p, (long long)m * k) : pt_sincospi(m * k, 16 * p), u[m]);
    }
    for (int tid = 0; tid < BS; ++tid) {
      int k = tid & (p - 1);
      cd *u = U + 16 * tid;
      for (int m = 0; m < 8; ++m) dft2t(&u[m], &u[m + 8], m, &K);
      static const int c4[4] = {0, 2, 4, 6};
      for (int m = 0; m < 4; ++m) { dft2t(&u[m], &u[m + 4], c4[m], &K); dft2t(&u[m + 8], &u[m + 12], c4[m], &K); }
      static const int c2[2] = {0, 4};
      for (int g = 0; g < 16; g += 4)
        for (int m = 0; m < 2; ++m) dft2t(&u[g + m], &u[g + m + 2], c2[m], &K);
      cd *o = sh + ((tid - k) << 4) + k;
      static const int order[8] = {0, 8, 4, 12, 2, 10, 6, 14};
      for (int q = 0; q < 8; ++q) {
        o[q * p] = ADD(u[order[q]], u[order[q] + 1]);
        o[(q + 8) * p] = SUB(u[order[q]], u[order[q] + 1]);
      }
    }
    p *= 16;
  }
  free(U);
}

int orc_ref_legacy16(int n, long long batch, const double *in, double *out, int tw_mode) {
  if (n != 16 && n != 256 && n != 4096) return -1;
  cd *t = (cd *)malloc(sizeof(cd) * (size_t)n);
  for (long long b = 0; b < batch; ++b) {
    memcpy(t, in + 2 * (size_t)n * b, sizeof(cd) * (size_t)n);
    ref_legacy16_one(t, n, tw_mode == TW_EXACT);
    memcpy(out + 2 * (size_t)n * b, t, sizeof(cd) * (size_t)n);
  }
  free(t);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Seeded inputs: counter-based SplitMix64, identical to the host generator   */
/* of the library's test/bench helpers.                                       */
/* ------------------------------------------------------------------------- */

static inline uint64_t smix(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* count doubles uniform in [-1, 1): (z >> 11) * 2^-52 - 1, exact in double */
void orc_gen_uniform(uint64_t seed, long long count, double *out) {
  for (long long i = 0; i < count; ++i) out[i] = (double)(smix(seed, (uint64_t)i) >> 11) * 0x1p-52 - 1.0;
}
