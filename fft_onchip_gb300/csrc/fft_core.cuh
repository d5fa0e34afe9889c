// fftoc — batched forward complex FFTs (N = 8..4096) for GB300 (sm_103a).
//
// Device core shared by every engine.  A transform of N points is computed by
// T = N / P threads, each holding P points in registers.  Each pass of radix R
// is one Stockham step (the structure of the reference's radix-8 executor,
// includes/legacy8_fft.cuh:57-119): butterfly t' reads x[t' + m*N/R],
// multiplies input m by W_{R*p}^{k*m} (k = t' mod p, p = product of earlier
// radices), runs an R-point DFT and writes y[(t'-k)*R + k + m*p].  Passes are
// joined through shared memory; the first pass reads HBM and the last writes
// HBM, both coalesced (consecutive threads touch consecutive 16-byte points).
//
// Engines (arithmetic used inside the transform; input/output are always
// interleaved binary64 complex values):
//   EngF64 — IEEE binary64 (DFMA/DADD).
//   EngFx  — 64-bit block fixed point.  Each transform is scaled by a power of
//            two taken from its largest exponent so that no value can overflow
//            (headroom for the worst-case growth of N), adds are exact 64-bit
//            integer adds, and products use 30-bit limbs on IMAD.WIDE.  The
//            conversion back to binary64 rounds once (cvt.rn.f64.s64).
#pragma once
#include <type_traits>
#include <cstdint>
#include <cuda_runtime.h>

#define FFTOC_HD __host__ __device__ __forceinline__

namespace fftoc {

// ---------------------------------------------------------------------------
// Plans: a transform of N points is split over T = N/P threads holding P
// points each, and computed in passes of radix R[0], R[1], ... (product N,
// every R dividing P).  T threads per transform, TPB transforms per CTA.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N_, int P_, int TPB_, int R0, int R1 = 1, int R2 = 1, int R3 = 1, int MINB_ = 1>
struct PlanT {
  static constexpr int N = N_;
  static constexpr int P = P_;
  static constexpr int TPB = TPB_;
  static constexpr int MINB = MINB_;  // minimum resident CTAs per SM (register budget)
  static constexpr bool PREFETCH = false;  // batched kernel: L2 prefetch one wave ahead (Prefetched<>)
  static constexpr long long PREFETCH_MIN_BYTES = 0;  // ... for batches of at least this much input
  static constexpr bool OUTLINE_SLOW_IN = false;  // batched kernel: rare input path out of line (OutlinedSlowIn<>)
  static constexpr bool IMAD_SPLIT = false;  // fixed point: low limbs by integer multiply-add (ImadSplit<>)
  static constexpr bool OUT_HI_ZERO = false;  // fixed point: zero test on the converted word (OutHiZero<>)
  static constexpr bool NO_STAGE = false;  // fewer than 8 threads per transform: direct HBM access (NoStage<>)
  static constexpr bool UNEVEN_DEFAULT = false;  // the uneven path's default plan for its size (UnevenDefault<>)
  static constexpr int R[4] = {R0, R1, R2, R3};
  static constexpr int S = (R0 > 1) + (R1 > 1) + (R2 > 1) + (R3 > 1);
  static constexpr int T = N / P;
  static_assert(R0 * R1 * R2 * R3 == N, "radices must multiply to N");
  static_assert(P % R0 == 0 && P % R1 == 0 && P % R2 == 0 && P % R3 == 0, "every radix divides P");
  // span p of pass s (product of the radices before it)
  __host__ __device__ static constexpr int span(int s) {
    int p = 1;
    for (int i = 0; i < s; ++i) p *= R[i];
    return p;
  }
  // offset (in twiddle entries) of pass s's table; pass s holds (R-1)*p
  // entries, entry (m-1)*p + k = W_{R p}^{k m}.  Pass 0 has no twiddles.
  __host__ __device__ static constexpr int tw_offset(int s) {
    int off = 0;
    for (int i = 1; i < s; ++i) off += (R[i] - 1) * span(i);
    return off;
  }
  static constexpr int TW_COUNT = tw_offset(S);
};

// ---------------------------------------------------------------------------
// Engines
// ---------------------------------------------------------------------------
struct EngF64 {
  using S = double;
  using TW = double2;   // (cos, -sin) of the twiddle
  struct KC { double c; };
  static constexpr int kId = 1;
  FFTOC_HD static S add(S a, S b) { return a + b; }
  FFTOC_HD static S sub(S a, S b) { return a - b; }
  FFTOC_HD static S add3(S a, S b, S c) { return (a + b) + c; }
  FFTOC_HD static S addsub(S a, S b, S c) { return (a + b) - c; }
  FFTOC_HD static S subadd(S a, S b, S c) { return (a - b) + c; }
  FFTOC_HD static S sub3(S a, S b, S c) { return (a - b) - c; }
  FFTOC_HD static S mulc(S x, KC k) { return x * k.c; }
  FFTOC_HD static void cmul(S& xr, S& xi, const TW w) {
    const double r = fma(xr, w.x, -xi * w.y);
    const double i = fma(xr, w.y, xi * w.x);
    xr = r;
    xi = i;
  }
  // complex multiply by a compile-time constant (c, s)
  FFTOC_HD static void cmulk(S& xr, S& xi, KC c, KC s) {
    const double r = fma(xr, c.c, -xi * s.c);
    const double i = fma(xr, s.c, xi * c.c);
    xr = r;
    xi = i;
  }
};

// Limbs of a fixed-point constant: v*2^60 = h*2^30 + l, 0 <= l < 2^30.
struct FxKC {
  int h, l;
};

// IMAD_SPLIT selects how the low limb of a split is formed (a logic op or an
// integer multiply-add: same value, different pipe); the plans choose the form
// that measured faster.
template <bool IMAD_SPLIT = false>
struct EngFxT {
  using S = long long;
  using TW = int4;      // (wr.h, wr.l, wi.h, wi.l): w*2^60 = h*2^30 + l, 0 <= l < 2^30
  using KC = FxKC;
  static constexpr int kId = 2;
  FFTOC_HD static S add(S a, S b) { return a + b; }
  FFTOC_HD static S sub(S a, S b) { return a - b; }
  // Three-operand sums as one PTX sequence each: the front end cannot share
  // partial sums between outputs, so ptxas can emit a fused 3-input add pair.
#ifdef __CUDA_ARCH__
  FFTOC_HD static S add3(S a, S b, S c) {
    S r;
    asm("add.s64 %0, %1, %2;\n\tadd.s64 %0, %0, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
  }
  FFTOC_HD static S addsub(S a, S b, S c) {
    S r;
    asm("add.s64 %0, %1, %2;\n\tsub.s64 %0, %0, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
  }
  FFTOC_HD static S subadd(S a, S b, S c) {
    S r;
    asm("sub.s64 %0, %1, %2;\n\tadd.s64 %0, %0, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
  }
  FFTOC_HD static S sub3(S a, S b, S c) {
    S r;
    asm("sub.s64 %0, %1, %2;\n\tsub.s64 %0, %0, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
  }
#else
  static S add3(S a, S b, S c) { return a + b + c; }
  static S addsub(S a, S b, S c) { return a + b - c; }
  static S subadd(S a, S b, S c) { return a - b + c; }
  static S sub3(S a, S b, S c) { return a - b - c; }
#endif
  // Limbs of a value, |x| < 2^61: x = xh*2^30 + xl, |xh| < 2^31, 0 <= xl < 2^30.
  FFTOC_HD static void split(S x, int& xh, int& xl) {
    xh = (int)(x >> 30);
#ifdef __CUDA_ARCH__
    if constexpr (IMAD_SPLIT) {  // lo32(x) - xh * 2^30 (mod 2^32)
      asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(xl) : "r"(xh), "r"(0xC0000000u), "r"((unsigned)x));
      return;
    }
#endif
    xl = (int)((unsigned)x & 0x3FFFFFFFu);
  }
  // a*b + c with a, b 32-bit and c 64-bit: one IMAD.WIDE (spelled out in PTX;
  // written as (long long)a * b + c the front end may emit a 64x64 multiply)
  FFTOC_HD static S madw(int a, int b, S c) {
#ifdef __CUDA_ARCH__
    S d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
#else
    return (S)a * (S)b + c;
#endif
  }
  // a*b with a, b 32-bit: one IMAD.WIDE without an addend
  FFTOC_HD static S mulw(int a, int b) {
#ifdef __CUDA_ARCH__
    S d;
    asm("mul.wide.s32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
    return d;
#else
    return (S)a * (S)b;
#endif
  }
  // x * c for a real constant, |c| <= 1:
  //   x*c = xh*ch + (xh*cl + xl*ch) / 2^30 + xl*cl/2^60   (last term < 1, dropped)
  // |xh*cl| < 2^61, |xl*ch| <= 2^60, so the middle sum cannot overflow.  The
  // middle sum is shifted without a rounding constant (floor): the product is
  // within 2 units of the exact value, and a chain that opens with a plain
  // multiply measured 2-4 % faster than one that opens with a 64-bit addend.
  FFTOC_HD static S mulc(S x, KC k) {
    int xh, xl;
    split(x, xh, xl);
    const long long m = madw(xl, k.h, mulw(xh, k.l));
    return madw(xh, k.h, m >> 30);
  }
  // (xr + i xi) * (wr + i wi); each middle sum has four terms of magnitude
  // < 2^61 or <= 2^60, so |m| < 1.5 * 2^62.
  FFTOC_HD static void cmul_limbs(S& xr, S& xi, int wrh, int wrl, int wih, int wil) {
    int rh, rl, ih, il;
    split(xr, rh, rl);
    split(xi, ih, il);
    // negate the twiddle limbs (|wih| <= 2^30, 0 <= wil < 2^30), never the
    // data limbs (ih may be -2^31)
    const int nwih = -wih, nwil = -wil;
    const long long mr = madw(il, nwih, madw(ih, nwil, madw(rl, wrh, mulw(rh, wrl))));
    const long long mi = madw(il, wrh, madw(ih, wrl, madw(rl, wih, mulw(rh, wil))));
    xr = madw(ih, nwih, madw(rh, wrh, mr >> 30));
    xi = madw(ih, wrh, madw(rh, wih, mi >> 30));
  }
  FFTOC_HD static void cmul(S& xr, S& xi, const int4 w) { cmul_limbs(xr, xi, w.x, w.y, w.z, w.w); }
  FFTOC_HD static void cmulk(S& xr, S& xi, KC c, KC s) { cmul_limbs(xr, xi, c.h, c.l, s.h, s.l); }
};
using EngFx = EngFxT<false>;

// constants of the DFT kernels, per engine
template <class E> struct Konst;
template <> struct Konst<EngF64> {
  // sqrt(1/2), cos(pi/8), sin(pi/8)
  FFTOC_HD static EngF64::KC h() { return {0.70710678118654752440}; }
  FFTOC_HD static EngF64::KC nh() { return {-0.70710678118654752440}; }
  FFTOC_HD static EngF64::KC c8() { return {0.92387953251128675613}; }
  FFTOC_HD static EngF64::KC s8() { return {0.38268343236508977173}; }
  FFTOC_HD static EngF64::KC nc8() { return {-0.92387953251128675613}; }
  FFTOC_HD static EngF64::KC ns8() { return {-0.38268343236508977173}; }
};
// Fixed-point limbs of the same constants: v*2^60 = h*2^30 + l, 0 <= l < 2^30.
template <bool B> struct Konst<EngFxT<B>> {
  FFTOC_HD static FxKC h() { return {759250124, 1067312712}; }
  FFTOC_HD static FxKC nh() { return {-759250125, 6429112}; }
  FFTOC_HD static FxKC c8() { return {992008094, 424059668}; }
  FFTOC_HD static FxKC s8() { return {410903206, 732584116}; }
  FFTOC_HD static FxKC nc8() { return {-992008095, 649682156}; }
  FFTOC_HD static FxKC ns8() { return {-410903207, 341157708}; }
};

// A plan whose batched kernel also prefetches, into L2, the tile of the CTA
// that starts one full wave (SMs x MINB CTAs) later, for batches of at least
// MIN_MIB MiB of input (below that the prefetch measured slower at some sizes:
// N = 64 by 16 % at 64 MiB, N = 4096 by 1-2 % up to 256 MiB).
template <class PL, int MIN_MIB = 0>
struct Prefetched : PL {
  static constexpr bool PREFETCH = true;
  static constexpr long long PREFETCH_MIN_BYTES = (long long)MIN_MIB << 20;
};

// A plan whose batched kernel converts the rare transforms that leave the
// fast binary64 -> fixed-point input path through an out-of-line function
// (otherwise the compiler may if-convert that path into the fast one).
template <class PL>
struct OutlinedSlowIn : PL {
  static constexpr bool OUTLINE_SLOW_IN = true;
};

// A plan whose fixed-point splits form the low limb with an integer
// multiply-add instead of a mask (moves work from the ALU pipe to the FMA pipe).
template <class PL>
struct ImadSplit : PL {
  static constexpr bool IMAD_SPLIT = true;
};

// A plan whose output conversion tests the converted value's high word for
// zero instead of the 64-bit integer (one compare less per value).
template <class PL>
struct OutHiZero : PL {
  static constexpr bool OUT_HI_ZERO = true;
};

// A plan with fewer than 8 threads per transform that loads and stores HBM
// directly instead of staging its tile through shared memory.  With T
// threads per transform each warp access still covers whole 32-byte sectors
// for T >= 2; it pays off where the staging round trip costs more than the
// spread of the access (measured: T = 4).
template <class PL>
struct NoStage : PL {
  static constexpr bool NO_STAGE = true;
};

// The plan the uneven-batch path uses for its size while the size's plan
// choice is the library default (its persistent kernels measured faster
// with it than with the batched default).
template <class PL>
struct UnevenDefault : PL {
  static constexpr bool UNEVEN_DEFAULT = true;
};

// The engine a plan's kernels compute with: the fixed-point engine in the
// plan's split form, or E unchanged.
template <class E, class PL>
using PlanEngine = typename std::conditional<E::kId == EngFx::kId && PL::IMAD_SPLIT, EngFxT<true>, E>::type;

// ---------------------------------------------------------------------------
// Small forward DFTs on registers.  re[i], im[i] at compile-time indices
// base + stride*m, in place, natural order.
// ---------------------------------------------------------------------------
template <class E, int B, int ST, int PP>
FFTOC_HD void dft2(typename E::S (&re)[PP], typename E::S (&im)[PP]) {
  using S = typename E::S;
  const S ar = re[B], ai = im[B], br = re[B + ST], bi = im[B + ST];
  re[B] = E::add(ar, br); im[B] = E::add(ai, bi);
  re[B + ST] = E::sub(ar, br); im[B + ST] = E::sub(ai, bi);
}

// 4-point DFT of (x0, x1, x2, x3): with t = x1 + x3 and u = x1 - x3,
//   y0 = x0 + x2 + t, y2 = x0 + x2 - t, y1 = x0 - x2 - i*u, y3 = x0 - x2 + i*u,
// every output one three-operand sum.
template <class E>
FFTOC_HD void dft4_core(typename E::S x0r, typename E::S x0i, typename E::S x1r, typename E::S x1i,
                        typename E::S x2r, typename E::S x2i, typename E::S x3r, typename E::S x3i,
                        typename E::S& y0r, typename E::S& y0i, typename E::S& y1r, typename E::S& y1i,
                        typename E::S& y2r, typename E::S& y2i, typename E::S& y3r, typename E::S& y3i) {
  using S = typename E::S;
  const S tr = E::add(x1r, x3r), ti = E::add(x1i, x3i);
  const S ur = E::sub(x1r, x3r), ui = E::sub(x1i, x3i);
  y0r = E::add3(x0r, x2r, tr);
  y0i = E::add3(x0i, x2i, ti);
  y2r = E::addsub(x0r, x2r, tr);
  y2i = E::addsub(x0i, x2i, ti);
  y1r = E::subadd(x0r, x2r, ui);
  y1i = E::sub3(x0i, x2i, ur);
  y3r = E::sub3(x0r, x2r, ui);
  y3i = E::subadd(x0i, x2i, ur);
}

template <class E, int B, int ST, int PP>
FFTOC_HD void dft4(typename E::S (&re)[PP], typename E::S (&im)[PP]) {
  dft4_core<E>(re[B], im[B], re[B + ST], im[B + ST], re[B + 2 * ST], im[B + 2 * ST], re[B + 3 * ST], im[B + 3 * ST],
               re[B], im[B], re[B + ST], im[B + ST], re[B + 2 * ST], im[B + 2 * ST], re[B + 3 * ST], im[B + 3 * ST]);
}

// 8-point DFT: a_m = x_m + x_{m+4}, b_m = (x_m - x_{m+4}) W8^m; even outputs
// are DFT4(a), odd outputs DFT4(b).  W8^1 and W8^3 are real-constant
// products (sqrt(1/2)); W8^2 = -i is folded into the odd DFT4's signs.
template <class E, int B, int ST, int PP>
FFTOC_HD void dft8(typename E::S (&re)[PP], typename E::S (&im)[PP]) {
  using S = typename E::S;
  using K = Konst<E>;
  S ar[4], ai[4], br[4], bi[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    ar[m] = E::add(re[B + m * ST], re[B + (m + 4) * ST]);
    ai[m] = E::add(im[B + m * ST], im[B + (m + 4) * ST]);
    br[m] = E::sub(re[B + m * ST], re[B + (m + 4) * ST]);
    bi[m] = E::sub(im[B + m * ST], im[B + (m + 4) * ST]);
  }
  // b1 *= (1 - i)/sqrt2 ; b3 *= (-1 - i)/sqrt2
  const S b1r = E::mulc(E::add(br[1], bi[1]), K::h());
  const S b1i = E::mulc(E::sub(bi[1], br[1]), K::h());
  const S b3r = E::mulc(E::sub(bi[3], br[3]), K::h());
  const S b3i = E::mulc(E::add(br[3], bi[3]), K::nh());
  // even outputs X0, X2, X4, X6
  dft4_core<E>(ar[0], ai[0], ar[1], ai[1], ar[2], ai[2], ar[3], ai[3], re[B], im[B], re[B + 2 * ST], im[B + 2 * ST],
               re[B + 4 * ST], im[B + 4 * ST], re[B + 6 * ST], im[B + 6 * ST]);
  // odd outputs X1, X3, X5, X7: DFT4(b0, b1', b2', b3') with b2' = -i*b2 = (b2i, -b2r)
  {
    const S tr = E::add(b1r, b3r), ti = E::add(b1i, b3i);
    const S ur = E::sub(b1r, b3r), ui = E::sub(b1i, b3i);
    re[B + ST] = E::add3(br[0], bi[2], tr);
    im[B + ST] = E::subadd(bi[0], br[2], ti);
    re[B + 5 * ST] = E::addsub(br[0], bi[2], tr);
    im[B + 5 * ST] = E::sub3(bi[0], br[2], ti);
    re[B + 3 * ST] = E::subadd(br[0], bi[2], ui);
    im[B + 3 * ST] = E::addsub(bi[0], br[2], ur);
    re[B + 7 * ST] = E::sub3(br[0], bi[2], ui);
    im[B + 7 * ST] = E::add3(bi[0], br[2], ur);
  }
}

// 16-point DFT as 4 x 4: with n = 4*n1 + n2 and k = k1 + 4*k2,
//   X[k1 + 4 k2] = sum_n2 W4^(n2 k2) * (W16^(n2 k1) * sum_n1 x[4 n1 + n2] W4^(n1 k1)):
// four DFT4s over n1, the nine non-trivial W16^(n2 k1), four DFT4s over n2,
// and a transposition of the outputs (register renaming).
template <class E, int B, int ST, int PP>
FFTOC_HD void dft16(typename E::S (&re)[PP], typename E::S (&im)[PP]) {
  using S = typename E::S;
  using K = Konst<E>;
  // y[n2][k1] at B + (n2 + 4 k1) ST
  dft4<E, B, 4 * ST, PP>(re, im);
  dft4<E, B + ST, 4 * ST, PP>(re, im);
  dft4<E, B + 2 * ST, 4 * ST, PP>(re, im);
  dft4<E, B + 3 * ST, 4 * ST, PP>(re, im);
  auto at = [](int n2, int k1) { return B + (n2 + 4 * k1) * ST; };
  S r, i;
  // W16^1 = (c8, -s8)
  r = re[at(1, 1)]; i = im[at(1, 1)]; E::cmulk(r, i, K::c8(), K::ns8()); re[at(1, 1)] = r; im[at(1, 1)] = i;
  // W16^2 = (1 - i)/sqrt2, at (1, 2) and (2, 1)
  r = re[at(1, 2)]; i = im[at(1, 2)];
  re[at(1, 2)] = E::mulc(E::add(r, i), K::h()); im[at(1, 2)] = E::mulc(E::sub(i, r), K::h());
  r = re[at(2, 1)]; i = im[at(2, 1)];
  re[at(2, 1)] = E::mulc(E::add(r, i), K::h()); im[at(2, 1)] = E::mulc(E::sub(i, r), K::h());
  // W16^3 = (s8, -c8), at (1, 3) and (3, 1)
  r = re[at(1, 3)]; i = im[at(1, 3)]; E::cmulk(r, i, K::s8(), K::nc8()); re[at(1, 3)] = r; im[at(1, 3)] = i;
  r = re[at(3, 1)]; i = im[at(3, 1)]; E::cmulk(r, i, K::s8(), K::nc8()); re[at(3, 1)] = r; im[at(3, 1)] = i;
  // W16^4 = -i, at (2, 2)
  r = re[at(2, 2)]; i = im[at(2, 2)]; re[at(2, 2)] = i; im[at(2, 2)] = E::sub(S(0), r);
  // W16^6 = (-1 - i)/sqrt2, at (2, 3) and (3, 2)
  r = re[at(2, 3)]; i = im[at(2, 3)];
  re[at(2, 3)] = E::mulc(E::sub(i, r), K::h()); im[at(2, 3)] = E::mulc(E::add(r, i), K::nh());
  r = re[at(3, 2)]; i = im[at(3, 2)];
  re[at(3, 2)] = E::mulc(E::sub(i, r), K::h()); im[at(3, 2)] = E::mulc(E::add(r, i), K::nh());
  // W16^9 = (-c8, s8), at (3, 3)
  r = re[at(3, 3)]; i = im[at(3, 3)]; E::cmulk(r, i, K::nc8(), K::s8()); re[at(3, 3)] = r; im[at(3, 3)] = i;
  // DFT4 over n2 for each k1: inputs at B + (4 k1 + n2) ST, outputs X[k1 + 4 k2] at B + (4 k1 + k2) ST
  dft4<E, B, ST, PP>(re, im);
  dft4<E, B + 4 * ST, ST, PP>(re, im);
  dft4<E, B + 8 * ST, ST, PP>(re, im);
  dft4<E, B + 12 * ST, ST, PP>(re, im);
  S xr[16], xi[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      xr[k1 + 4 * k2] = re[B + (4 * k1 + k2) * ST];
      xi[k1 + 4 * k2] = im[B + (4 * k1 + k2) * ST];
    }
#pragma unroll
  for (int k = 0; k < 16; ++k) { re[B + k * ST] = xr[k]; im[B + k * ST] = xi[k]; }
}

template <class E, int R, int B, int ST, int PP>
FFTOC_HD void dft(typename E::S (&re)[PP], typename E::S (&im)[PP]) {
  if constexpr (R == 2) dft2<E, B, ST, PP>(re, im);
  else if constexpr (R == 4) dft4<E, B, ST, PP>(re, im);
  else if constexpr (R == 8) dft8<E, B, ST, PP>(re, im);
  else if constexpr (R == 16) dft16<E, B, ST, PP>(re, im);
}

// ---------------------------------------------------------------------------
// Shared-memory layout: element e of a transform lives at 16-byte slot
// e ^ ((e >> SW) & 7).  Writes of the first pass go at stride R (=2^SW) points
// per thread; the XOR keeps 8 consecutive threads on 8 distinct bank groups.
// ---------------------------------------------------------------------------
template <int SW> FFTOC_HD int swz(int e) { return e ^ ((e >> SW) & 7); }

}  // namespace fftoc
