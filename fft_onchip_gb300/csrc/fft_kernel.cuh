// fftoc — the batched forward-FFT kernel template (one launch = `batch`
// transforms of size N, TPB transforms per CTA).
#pragma once
#include <cstring>
#include <utility>
#include "fft_core.cuh"

namespace fftoc {

// Fixed-point scale: input magnitudes are mapped below 2^FxBits<N>, leaving
// log2(N) + 2 bits of headroom under 2^63 (worst-case growth N, plus the
// sqrt(2)-scaled sums inside the radix-8/16 kernels and the 2^61 limit of the
// limb products).
template <int N> struct FxBits {
  static constexpr int B = (61 - ilog2c(N)) < 53 ? (61 - ilog2c(N)) : 53;
};

// Rounding of the binary64 -> fixed-point input conversion of a size N.
// Small transforms (N <= 32) stream at the HBM limit with every resident CTA
// slot in use; there the truncating sequence (round toward zero, a negation
// after the shift) fits 64 registers and measured fastest (+9% at N = 8 on
// GB300).  From N = 64 up the kernels are bound by the integer pipes, and the
// floor sequence (the sign complemented before the shift, fewer instructions)
// measured 1-5% faster.  Every path of one size (batched, uneven, on-chip,
// device executors) uses its size's rounding, so their results agree bit for
// bit.
template <int N> struct FxTrunc {
  static constexpr bool value = N <= 32;
};

// --- binary64 <-> block fixed point -------------------------------------------
FFTOC_HD unsigned hi_word(double v) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(v);
#else
  unsigned long long b;
  memcpy(&b, &v, 8);
  return (unsigned)(b >> 32);
#endif
}
FFTOC_HD unsigned lo_word(double v) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(v);
#else
  unsigned long long b;
  memcpy(&b, &v, 8);
  return (unsigned)b;
#endif
}
FFTOC_HD double from_words(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const unsigned long long b = ((unsigned long long)hi << 32) | lo;
  double v;
  memcpy(&v, &b, 8);
  return v;
#endif
}

FFTOC_HD int expo_of(unsigned hw) { return (int)((hw >> 20) & 0x7FFu); }

// value * 2^(1022 + B - Emax), eref = Emax + 53 - B, with M the 53-bit
// significand and d = eref - e: M >> d for a positive value.  A negative one
// gives -(M >> d) (TRUNC: toward zero) or ~(M >> d) = floor(-M / 2^d) -
// [2^d divides M] (floor: the complement of the shifted magnitude, which the
// fast path below forms by complementing before the shift).  Zeros of either
// sign give 0.
template <bool TRUNC = false>
FFTOC_HD long long fx_in(unsigned hw, unsigned lw, int eref) {
  const int e = expo_of(hw);
  const unsigned mh = (hw & 0xFFFFFu) | (e ? 0x100000u : 0u);
  if ((mh | lw) == 0u) return 0;
  const int ee = e > 1 ? e : 1;
  const int d0 = eref - ee;
  const int d = d0 < 63 ? d0 : 63;
  const unsigned long long m = ((((unsigned long long)mh) << 32) | lw) >> d;
  const long long r = (long long)m;
  return ((int)hw < 0) ? (TRUNC ? -r : ~r) : r;
}

// x * 2^K, K = Emax - 1022 - B: the correctly rounded conversion with K added
// to its exponent field (exact).  Valid while every result exponent stays in
// the normal range (fx_scale's `slow` is false); one FP64-pipe instruction.
// HI_ZERO: test the converted high word for zero (a nonzero integer converts
// to a normal number, so the two tests agree).
template <bool HI_ZERO = false>
FFTOC_HD double fx_out(long long x, int kshift) {
  const double d = (double)x;
  const unsigned hi = hi_word(d);
  const bool nonzero = HI_ZERO ? hi != 0u : x != 0;
  return from_words(nonzero ? hi + (unsigned)kshift : hi, lo_word(d));
}

// Transforms whose outputs may be subnormal or overflow: ldexp.  Kept out of
// line so the compiler cannot if-convert it into the fast path (predicated-off
// FP64 instructions would still occupy the FP64 pipe).
#ifdef __CUDA_ARCH__
__device__ __noinline__ double fx_out_slow(long long x, int K) { return ldexp((double)x, K); }
#else
inline double fx_out_slow(long long x, int K) { return ldexp((double)x, K); }
#endif

// fx_in out of line, for the rare transforms that leave the fast input path.
#ifdef __CUDA_ARCH__
template <bool TRUNC>
__device__ __noinline__ long long fx_in_slow(unsigned hw, unsigned lw, int eref) { return fx_in<TRUNC>(hw, lw, eref); }
#else
template <bool TRUNC>
inline long long fx_in_slow(unsigned hw, unsigned lw, int eref) { return fx_in<TRUNC>(hw, lw, eref); }
#endif

// Scale parameters of a transform from its largest biased exponent.
struct FxScale {
  int eref, K, kshift;
  bool slow, special;
};
template <int B>
FFTOC_HD FxScale fx_scale(int em) {
  FxScale s;
  s.special = (em == 0x7FF);
  // subnormals (exponent field 0) are scaled like exponent field 1
  if (em < 1) em = 1;
  s.K = em - 1022 - B;
  s.kshift = (int)((unsigned)s.K << 20);
  s.slow = (em < B) || (em > 1983 + B);
  s.eref = em + 53 - B;
  return s;
}

// Fast conversion for values within 2^31 of the transform's largest exponent
// (all normal), bit-identical to fx_in there.  With S the sign mask
// (0 or ~0), the 96-bit word S:(M ^ S) is shifted right by d with two
// wrap-mode funnel shifts, which use d mod 32: d is taken as
// eref - (hw >> 20), whose sign bit at position 11 is a multiple of 32.
FFTOC_HD long long fx_in_near(unsigned hw, unsigned lw, int eref) {
  const unsigned S = (unsigned)((int)hw >> 31);
  const unsigned mh = (hw & 0xFFFFFu) ^ (S ^ 0x100000u);  // ((hw & 0xFFFFF) | 0x100000) ^ S
  const unsigned l = lw ^ S;
  const unsigned d = (unsigned)eref - (hw >> 20);
#ifdef __CUDA_ARCH__
  unsigned lo, hi;
  asm("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(lo) : "r"(l), "r"(mh), "r"(d));
  asm("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(hi) : "r"(mh), "r"(S), "r"(d));
#else
  const unsigned sh = d & 31u;
  const unsigned lo = (unsigned)((((unsigned long long)mh << 32) | l) >> sh);
  const unsigned hi = (unsigned)((((unsigned long long)S << 32) | mh) >> sh);
#endif
  return (long long)(((unsigned long long)hi << 32) | lo);
}

// The truncating fast conversion (bit-identical to fx_in<true> on the same
// domain): the shifted magnitude, negated for a negative value.
FFTOC_HD long long fx_in_near_trunc(unsigned hw, unsigned lw, int eref) {
  const int d = eref - expo_of(hw);
  const unsigned mh = (hw & 0xFFFFFu) | 0x100000u;
#ifdef __CUDA_ARCH__
  const unsigned lo = __funnelshift_r(lw, mh, d);
#else
  const unsigned lo = (unsigned)((((unsigned long long)mh << 32) | lw) >> d);
#endif
  const unsigned hi = mh >> d;
  const long long m = (long long)(((unsigned long long)hi << 32) | lo);
  return ((int)hw < 0) ? -m : m;
}

// Largest and smallest biased exponents of a thread's raw points: from the
// sign-cleared high words (floor sizes), or the exponent fields in two loops
// (the sequence that fits the small sizes' register budget).
template <int P, bool TRUNC = false>
FFTOC_HD void fx_exponent_range(const double2 (&raw)[P], int& emax, int& emin) {
  if constexpr (TRUNC) {
    int em = 0, en = 0x7FF;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const int a = expo_of(hi_word(raw[i].x)), b = expo_of(hi_word(raw[i].y));
      const int hi = a > b ? a : b;
      em = em > hi ? em : hi;
    }
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const int a = expo_of(hi_word(raw[i].x)), b = expo_of(hi_word(raw[i].y));
      en = en < a ? en : a;
      en = en < b ? en : b;
    }
    emax = em;
    emin = en;
  } else {
    unsigned amax = 0u, amin = 0x7FFFFFFFu;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const unsigned a = hi_word(raw[i].x) & 0x7FFFFFFFu, b = hi_word(raw[i].y) & 0x7FFFFFFFu;
      const unsigned hi = a > b ? a : b, lo = a < b ? a : b;
      amax = amax > hi ? amax : hi;
      amin = amin < lo ? amin : lo;
    }
    emax = (int)(amax >> 20);
    emin = (int)(amin >> 20);
  }
}

// Convert a thread's P raw points; the fast path is taken when every value is
// normal and within 2^31 of the transform maximum (the usual case).  emin is
// the thread's smallest biased exponent (fx_exponent_range).
// OUTLINE: the other path calls the out-of-line fx_in_slow.  TRUNC: the
// size's rounding (FxTrunc).
template <int P, bool OUTLINE = false, bool TRUNC = false>
FFTOC_HD void fx_convert_in(const double2 (&raw)[P], long long (&re)[P], long long (&im)[P], int eref, int emin) {
  if (emin >= 1 && eref - emin < 32) {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      if constexpr (TRUNC) {
        re[i] = fx_in_near_trunc(hi_word(raw[i].x), lo_word(raw[i].x), eref);
        im[i] = fx_in_near_trunc(hi_word(raw[i].y), lo_word(raw[i].y), eref);
      } else {
        re[i] = fx_in_near(hi_word(raw[i].x), lo_word(raw[i].x), eref);
        im[i] = fx_in_near(hi_word(raw[i].y), lo_word(raw[i].y), eref);
      }
    }
  } else if constexpr (OUTLINE) {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      re[i] = fx_in_slow<TRUNC>(hi_word(raw[i].x), lo_word(raw[i].x), eref);
      im[i] = fx_in_slow<TRUNC>(hi_word(raw[i].y), lo_word(raw[i].y), eref);
    }
  } else {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      re[i] = fx_in<TRUNC>(hi_word(raw[i].x), lo_word(raw[i].x), eref);
      im[i] = fx_in<TRUNC>(hi_word(raw[i].y), lo_word(raw[i].y), eref);
    }
  }
}
template <int P, bool OUTLINE = false, bool TRUNC = false>
FFTOC_HD void fx_convert_in(const double2 (&raw)[P], long long (&re)[P], long long (&im)[P], int eref) {
  int emax, emin;
  fx_exponent_range<P, TRUNC>(raw, emax, emin);
  fx_convert_in<P, OUTLINE, TRUNC>(raw, re, im, eref, emin);
}

// Largest value of em over the T consecutive threads of each transform (TPB
// transforms per CTA, thread tid, transform j = tid / T).  T <= 32: within the
// warp (a warp reduction for T = 32, shuffles over the T lanes otherwise).
// T > 32 (whole warps per transform): a warp reduction, one word per warp in
// `red` (TPB * T / 32 ints of shared memory) and one __syncthreads().
template <int T, int TPB>
__device__ __forceinline__ int fx_transform_max(int em, int tid, int j, int* red) {
  if constexpr (T == 32) {
    em = __reduce_max_sync(0xffffffffu, em);
  } else if constexpr (T > 1 && T < 32) {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o, T));
  } else if constexpr (T > 32) {
    constexpr int W = T / 32;
    em = __reduce_max_sync(0xffffffffu, em);
    if ((tid & 31) == 0) red[tid >> 5] = em;
    __syncthreads();
    em = red[j * W];
#pragma unroll
    for (int w = 1; w < W; ++w) em = max(em, red[j * W + w]);
  }
  return em;
}

// --- the kernel ---------------------------------------------------------------
template <class E, class PL>
struct Fft {
  using S = typename E::S;
  using TW = typename E::TW;
  static constexpr int N = PL::N;
  static constexpr int TPB = PL::TPB;
  static constexpr int P = PL::P;
  static constexpr int T = PL::T;
  static constexpr int NS = PL::S;
  // padded shared layout: one 16-byte pad slot after every 2^SH points, so
  // the first pass's stride-R writes and every stride-1 read hit distinct
  // bank groups, and all addresses are a per-thread base plus a constant
  static constexpr int SH = PL::R[0] >= 16 ? 4 : 3;
  static constexpr int NP = N + (N >> SH);
  static constexpr int THREADS = T * TPB;
  static constexpr bool STAGED = T < 8 && !PL::NO_STAGE;  // small N: stage HBM tiles through smem
  static constexpr int SMEM = TPB * NP * 16 + 64;  // + 16 words of exponent scratch
  static_assert(T <= 32 || TPB * (T / 32) <= 16, "exponent scratch holds one word per warp, 16 words");

  // 16-byte slot of element e of block-local transform j
  __device__ __forceinline__ static int slot(int j, int e) { return j * NP + e + (e >> SH); }

  template <int s, int b>
  __device__ __forceinline__ static void butterfly(S (&re)[P], S (&im)[P], int t, const TW* __restrict__ tw) {
    constexpr int R = PL::R[s];
    constexpr int B = P / R;
    constexpr int p = PL::span(s);
    if constexpr (s > 0) {
      const int tp = t + T * b;
      const int k = tp & (p - 1);
      const TW* base = tw + PL::tw_offset(s) + k;
#pragma unroll
      for (int m = 1; m < R; ++m) {
        const TW w = __ldg(base + (m - 1) * p);
        E::cmul(re[b + B * m], im[b + B * m], w);
      }
    }
    dft<E, R, b, B, P>(re, im);
  }

  template <int s, int... bs>
  __device__ __forceinline__ static void pass(S (&re)[P], S (&im)[P], int t, const TW* __restrict__ tw,
                                              std::integer_sequence<int, bs...>) {
    (butterfly<s, bs>(re, im, t, tw), ...);
  }

  // destination index of output m of butterfly b in pass s
  template <int s>
  __device__ __forceinline__ static int dest(int t, int b, int m) {
    constexpr int R = PL::R[s];
    constexpr int p = PL::span(s);
    const int tp = t + T * b;
    const int k = tp & (p - 1);
    return (tp - k) * R + k + m * p;
  }

  template <int s>
  __device__ __forceinline__ static void write_smem(S (&re)[P], S (&im)[P], int j, int t, longlong2* sm) {
    constexpr int R = PL::R[s];
    constexpr int B = P / R;
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        longlong2 v;
        v.x = to_bits(re[b + B * m]);
        v.y = to_bits(im[b + B * m]);
        sm[slot(j, dest<s>(t, b, m))] = v;
      }
  }

  __device__ __forceinline__ static void read_smem(S (&re)[P], S (&im)[P], int j, int t, const longlong2* sm) {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const longlong2 v = sm[slot(j, t + T * i)];
      re[i] = from_bits(v.x);
      im[i] = from_bits(v.y);
    }
  }
  __device__ __forceinline__ static long long to_bits(S v) {
    if constexpr (E::kId == EngF64::kId) return __double_as_longlong(v);
    else return (long long)v;
  }
  __device__ __forceinline__ static S from_bits(long long b) {
    if constexpr (E::kId == EngF64::kId) return __longlong_as_double(b);
    else return (S)b;
  }

  template <int s>
  __device__ __forceinline__ static void run_passes(S (&re)[P], S (&im)[P], int j, int t, const TW* __restrict__ tw,
                                                    longlong2* sm) {
    constexpr int R = PL::R[s];
    pass<s>(re, im, t, tw, std::make_integer_sequence<int, P / R>{});
    if constexpr (s + 1 < NS) {
      if constexpr (s > 0) __syncthreads();  // previous readers of the buffer are done
      write_smem<s>(re, im, j, t, sm);
      __syncthreads();
      read_smem(re, im, j, t, sm);
      run_passes<s + 1>(re, im, j, t, tw, sm);
    }
  }
};

// Where the transforms of one CTA tile live.  ContigTile: the batched entry
// points, transform tile0 + j at element (tile0 + j) * N.  IndexedTile (the
// uneven-batch kernel): transform j of the tile at element base[j], with the
// bases staged in shared memory by the caller.
template <int N>
struct ContigTile {
  const double2* __restrict__ in;
  double2* __restrict__ out;
  long long tile0, count;
  __device__ __forceinline__ const double2* in_of(int j) const { return in + (tile0 + j) * N; }
  __device__ __forceinline__ double2* out_of(int j) const { return out + (tile0 + j) * N; }
  // element e of transform jj, idx = jj * N + e
  __device__ __forceinline__ const double2* in_elem(int idx, int, int) const { return in + tile0 * N + idx; }
  __device__ __forceinline__ double2* out_elem(int idx, int, int) const { return out + tile0 * N + idx; }
  __device__ __forceinline__ static double2 load(const double2* p) { return __ldg(p); }
};

struct IndexedTile {
  const double2* __restrict__ in;
  double2* __restrict__ out;
  const long long* base;  // shared memory, one entry per transform of the tile
  long long tile0, count;
  __device__ __forceinline__ const double2* in_of(int j) const { return in + base[j]; }
  __device__ __forceinline__ double2* out_of(int j) const { return out + base[j]; }
  __device__ __forceinline__ const double2* in_elem(int, int jj, int e) const { return in + base[jj] + e; }
  __device__ __forceinline__ double2* out_elem(int, int jj, int e) const { return out + base[jj] + e; }
  __device__ __forceinline__ static double2 load(const double2* p) { return __ldg(p); }
};

// Tiles of an uneven batch for plans that do not stage their tile (each
// thread touches only its own transform): the thread's transform offset in a
// register, loaded ahead by the caller.
struct RegTile {
  const double2* __restrict__ in;
  double2* __restrict__ out;
  long long off;  // this thread's transform
  long long tile0, count;
  __device__ __forceinline__ const double2* in_of(int) const { return in + off; }
  __device__ __forceinline__ double2* out_of(int) const { return out + off; }
  __device__ __forceinline__ const double2* in_elem(int, int, int e) const { return in + off + e; }
  __device__ __forceinline__ double2* out_elem(int, int, int e) const { return out + off + e; }
  __device__ __forceinline__ static double2 load(const double2* p) { return __ldg(p); }
};

// The on-chip repeat harness: the tile's transforms resident in shared
// memory (`buf`, TPB * N points, transformed in place), loaded with plain
// shared loads.
template <int N>
struct SmemTile {
  double2* buf;
  long long tile0, count;  // tile0 = 0, count = TPB
  __device__ __forceinline__ const double2* in_of(int j) const { return buf + j * N; }
  __device__ __forceinline__ double2* out_of(int j) const { return buf + j * N; }
  __device__ __forceinline__ const double2* in_elem(int idx, int, int) const { return buf + idx; }
  __device__ __forceinline__ double2* out_elem(int idx, int, int) const { return buf + idx; }
  __device__ __forceinline__ static double2 load(const double2* p) { return *p; }
};

// One CTA tile: load raw points (binary64), convert, run the passes, convert
// back and store.  Engine-specific entry/exit.  Used by the uneven-batch
// kernel; the batched kernel below carries the same body.
template <class E, class PL, class Tile>
__device__ __forceinline__ void fft_tile(const Tile& tl, const typename E::TW* __restrict__ tw,
                                         unsigned char* smem_raw) {
  using EK = PlanEngine<E, PL>;
  using F = Fft<EK, PL>;
  using S = typename EK::S;
  constexpr int N = PL::N, TPB = PL::TPB;
  constexpr int P = F::P, T = F::T, NS = F::NS;
  longlong2* sm = reinterpret_cast<longlong2*>(smem_raw);

  const int tid = threadIdx.x;
  const int j = tid / T;
  const int t = tid - j * T;
  const long long tile0 = tl.tile0;
  const bool active = tile0 + j < tl.count;
  const long long tile_elems = (min((long long)TPB, tl.count - tile0)) * N;

  // ---- load raw binary64 points: point i of this thread is element t + T*i
  double2 raw[P];
  if constexpr (F::STAGED) {
    for (int idx = tid; idx < tile_elems; idx += F::THREADS) {
      const int jj = idx / N, e = idx - jj * N;
      const double2 v = Tile::load(tl.in_elem(idx, jj, e));
      sm[F::slot(jj, e)] = make_longlong2(__double_as_longlong(v.x), __double_as_longlong(v.y));
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const longlong2 v = sm[F::slot(j, t + T * i)];
      raw[i] = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
    }
  } else {
    const double2* src = tl.in_of(j) + t;  // in range or unused: loads are guarded
#pragma unroll
    for (int i = 0; i < P; ++i) raw[i] = active ? Tile::load(src + T * i) : make_double2(0.0, 0.0);
  }

  S re[P], im[P];
  int K = 0, kshift = 0;
  bool slow = false, special = false;
  if constexpr (E::kId == EngF64::kId) {
#pragma unroll
    for (int i = 0; i < P; ++i) { re[i] = raw[i].x; im[i] = raw[i].y; }
  } else {
    // largest biased exponent of the transform, smallest of this thread
    constexpr bool TR = FxTrunc<N>::value;
    int em, emin;
    fx_exponent_range<P, TR>(raw, em, emin);
    em = fx_transform_max<T, TPB>(em, tid, j, reinterpret_cast<int*>(smem_raw + TPB * F::NP * 16));
    const FxScale sc = fx_scale<FxBits<N>::B>(em);
    special = sc.special;
    K = sc.K;
    kshift = sc.kshift;
    slow = sc.slow;
    fx_convert_in<P, false, TR>(raw, re, im, sc.eref, emin);
  }

  if constexpr (F::STAGED) __syncthreads();  // staging buffer is reused by the passes
  F::template run_passes<0>(re, im, j, t, tw, sm);

  // ---- store: output m of butterfly b of the last pass is element dest(...)
  constexpr int RL = PL::R[NS - 1];
  constexpr int BL = P / RL;
  // Fixed point: the rare transforms whose outputs leave the normal range, or
  // whose inputs were not finite, take the slow conversion: a per-value select
  // where the output is staged or the size is small (FxTrunc; both measured
  // faster so), else one branch per thread between two store loops.
  auto value = [&](int i) -> double2 {
    if constexpr (E::kId == EngF64::kId) {
      return make_double2(re[i], im[i]);
    } else {
      return make_double2(fx_out<PL::OUT_HI_ZERO>((long long)re[i], kshift),
                          fx_out<PL::OUT_HI_ZERO>((long long)im[i], kshift));
    }
  };
  auto slow_value = [&](int i) -> double2 {
    if constexpr (E::kId == EngF64::kId) {
      return make_double2(re[i], im[i]);
    } else {
      const double qnan = __longlong_as_double(0x7FF8000000000000LL);
      return special ? make_double2(qnan, qnan)
                     : make_double2(fx_out_slow((long long)re[i], K), fx_out_slow((long long)im[i], K));
    }
  };
  const bool redo = E::kId != EngF64::kId && (slow || special);
  // Small sizes with at most 4 points per thread: the slow values replace the
  // fixed-point words in place (one branch; the words are few, so this costs
  // no registers), and the stores select the words or the fast conversion.
  constexpr bool IN_PLACE = E::kId != EngF64::kId && FxTrunc<N>::value && P <= 4;
  if constexpr (IN_PLACE) {
    if (redo) {
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const double2 v = slow_value(i);
        re[i] = __double_as_longlong(v.x);
        im[i] = __double_as_longlong(v.y);
      }
    }
  }
  auto stored = [&](int i) -> double2 {
    if constexpr (IN_PLACE) {
      return redo ? make_double2(__longlong_as_double(re[i]), __longlong_as_double(im[i])) : value(i);
    } else {
      return redo ? slow_value(i) : value(i);
    }
  };
  if constexpr (F::STAGED) {
    if constexpr (NS > 1) __syncthreads();
#pragma unroll
    for (int b = 0; b < BL; ++b)
#pragma unroll
      for (int m = 0; m < RL; ++m) {
        const double2 v = stored(b + BL * m);
        sm[F::slot(j, F::template dest<NS - 1>(t, b, m))] =
            make_longlong2(__double_as_longlong(v.x), __double_as_longlong(v.y));
      }
    __syncthreads();
    for (int idx = tid; idx < tile_elems; idx += F::THREADS) {
      const int jj = idx / N, e = idx - jj * N;
      const longlong2 v = sm[F::slot(jj, e)];
      *tl.out_elem(idx, jj, e) = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
    }
  } else {
    if (active) {
      double2* dst = tl.out_of(j);
      if constexpr (FxTrunc<N>::value) {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m)
            dst[F::template dest<NS - 1>(t, b, m)] = stored(b + BL * m);
      } else if (!redo) {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) dst[F::template dest<NS - 1>(t, b, m)] = value(b + BL * m);
      } else {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) dst[F::template dest<NS - 1>(t, b, m)] = slow_value(b + BL * m);
      }
    }
  }
}


// The batched kernel: CTA b transforms transforms [b*TPB, b*TPB + TPB).
// in and out may be the same buffer (in place): a CTA reads only the tile it
// writes, and every load of that tile (registers, or the shared staging
// buffer) happens before its first store, which is what the __restrict__
// qualifiers and the read-only loads rely on; the tests run every plan in
// place.
// Its body is fft_tile's with contiguous addressing written out: routing it
// through fft_tile<ContigTile> computes the same results but compiled to
// code measured 2.5-4% slower at N=64 and N=512, so the two are kept
// separate and the tests check them against each other bit for bit.
template <class E, class PL>
__global__ void __launch_bounds__(Fft<E, PL>::THREADS, PL::MINB)
fft_fwd_kernel(const double2* __restrict__ in, double2* __restrict__ out, long long batch,
               const typename E::TW* __restrict__ tw, int* __restrict__ err) {
  (void)err;  // no waits in this kernel; the argument keeps one launch signature
  using EK = PlanEngine<E, PL>;
  using F = Fft<EK, PL>;
  using S = typename EK::S;
  constexpr int N = PL::N, TPB = PL::TPB;
  constexpr int P = F::P, T = F::T, NS = F::NS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  longlong2* sm = reinterpret_cast<longlong2*>(smem_raw);

  if constexpr (PL::PREFETCH) {
    if (threadIdx.x == 0 && batch * (PL::N * 16) >= PL::PREFETCH_MIN_BYTES) {
      // the tile of the CTA that starts one full wave later, into L2
      unsigned nsm;
      asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
      const long long first = ((long long)blockIdx.x + (long long)nsm * PL::MINB) * TPB;
      if (first < batch) {
        const long long cnt = batch - first < TPB ? batch - first : TPB;
        const char* p = reinterpret_cast<const char*>(in + first * N);
        long long bytes = cnt * N * 16;
        while (bytes > 0) {  // pieces of at most 64 KiB; 16-byte aligned multiples of 16
          const unsigned b = bytes > 65536 ? 65536u : (unsigned)bytes;
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(b) : "memory");
          p += b;
          bytes -= b;
        }
      }
    }
  }

  const int tid = threadIdx.x;
  const int j = tid / T;
  const int t = tid - j * T;
  const long long tile0 = (long long)blockIdx.x * TPB;
  const long long tr = tile0 + j;
  const bool active = tr < batch;
  const long long tile_elems = (min((long long)TPB, batch - tile0)) * N;

  // ---- load raw binary64 points: point i of this thread is element t + T*i
  double2 raw[P];
  if constexpr (F::STAGED) {
    const double2* src = in + tile0 * N;
    for (int idx = tid; idx < tile_elems; idx += F::THREADS) {
      const int jj = idx / N, e = idx - jj * N;
      const double2 v = __ldg(src + idx);
      sm[F::slot(jj, e)] = make_longlong2(__double_as_longlong(v.x), __double_as_longlong(v.y));
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const longlong2 v = sm[F::slot(j, t + T * i)];
      raw[i] = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
    }
  } else {
    const double2* src = in + tr * N + t;
#pragma unroll
    for (int i = 0; i < P; ++i) raw[i] = active ? __ldg(src + T * i) : make_double2(0.0, 0.0);
  }

  S re[P], im[P];
  int K = 0, kshift = 0;
  bool slow = false, special = false;
  if constexpr (E::kId == EngF64::kId) {
#pragma unroll
    for (int i = 0; i < P; ++i) { re[i] = raw[i].x; im[i] = raw[i].y; }
  } else {
    // largest biased exponent of the transform, smallest of this thread
    constexpr bool TR = FxTrunc<N>::value;
    int em, emin;
    fx_exponent_range<P, TR>(raw, em, emin);
    em = fx_transform_max<T, TPB>(em, tid, j, reinterpret_cast<int*>(smem_raw + TPB * F::NP * 16));
    const FxScale sc = fx_scale<FxBits<N>::B>(em);
    special = sc.special;
    K = sc.K;
    kshift = sc.kshift;
    slow = sc.slow;
    fx_convert_in<P, PL::OUTLINE_SLOW_IN, TR>(raw, re, im, sc.eref, emin);
  }

  if constexpr (F::STAGED) __syncthreads();  // staging buffer is reused by the passes
  F::template run_passes<0>(re, im, j, t, tw, sm);

  // ---- store: output m of butterfly b of the last pass is element dest(...)
  constexpr int RL = PL::R[NS - 1];
  constexpr int BL = P / RL;
  // Fixed point: the rare transforms whose outputs leave the normal range, or
  // whose inputs were not finite, take the slow conversion: a per-value select
  // where the output is staged or the size is small (FxTrunc; both measured
  // faster so), else one branch per thread between two store loops.
  auto value = [&](int i) -> double2 {
    if constexpr (E::kId == EngF64::kId) {
      return make_double2(re[i], im[i]);
    } else {
      return make_double2(fx_out<PL::OUT_HI_ZERO>((long long)re[i], kshift),
                          fx_out<PL::OUT_HI_ZERO>((long long)im[i], kshift));
    }
  };
  auto slow_value = [&](int i) -> double2 {
    if constexpr (E::kId == EngF64::kId) {
      return make_double2(re[i], im[i]);
    } else {
      const double qnan = __longlong_as_double(0x7FF8000000000000LL);
      return special ? make_double2(qnan, qnan)
                     : make_double2(fx_out_slow((long long)re[i], K), fx_out_slow((long long)im[i], K));
    }
  };
  const bool redo = E::kId != EngF64::kId && (slow || special);
  // Small sizes with at most 4 points per thread: the slow values replace the
  // fixed-point words in place (one branch; the words are few, so this costs
  // no registers), and the stores select the words or the fast conversion.
  constexpr bool IN_PLACE = E::kId != EngF64::kId && FxTrunc<N>::value && P <= 4;
  if constexpr (IN_PLACE) {
    if (redo) {
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const double2 v = slow_value(i);
        re[i] = __double_as_longlong(v.x);
        im[i] = __double_as_longlong(v.y);
      }
    }
  }
  auto stored = [&](int i) -> double2 {
    if constexpr (IN_PLACE) {
      return redo ? make_double2(__longlong_as_double(re[i]), __longlong_as_double(im[i])) : value(i);
    } else {
      return redo ? slow_value(i) : value(i);
    }
  };
  if constexpr (F::STAGED) {
    if constexpr (NS > 1) __syncthreads();
#pragma unroll
    for (int b = 0; b < BL; ++b)
#pragma unroll
      for (int m = 0; m < RL; ++m) {
        const double2 v = stored(b + BL * m);
        sm[F::slot(j, F::template dest<NS - 1>(t, b, m))] =
            make_longlong2(__double_as_longlong(v.x), __double_as_longlong(v.y));
      }
    __syncthreads();
    double2* dst = out + tile0 * N;
    for (int idx = tid; idx < tile_elems; idx += F::THREADS) {
      const int jj = idx / N, e = idx - jj * N;
      const longlong2 v = sm[F::slot(jj, e)];
      dst[idx] = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
    }
  } else {
    if (active) {
      double2* dst = out + tr * N;
      if constexpr (FxTrunc<N>::value) {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m)
            dst[F::template dest<NS - 1>(t, b, m)] = stored(b + BL * m);
      } else if (!redo) {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) dst[F::template dest<NS - 1>(t, b, m)] = value(b + BL * m);
      } else {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) dst[F::template dest<NS - 1>(t, b, m)] = slow_value(b + BL * m);
      }
    }
  }
}

}  // namespace fftoc
