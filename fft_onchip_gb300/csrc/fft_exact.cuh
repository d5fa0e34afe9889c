// fftoc — exact-slice split form: radix-16 passes on the BF16 tensor cores
// with products that are exact in FP32, for relative errors ~1e-14.
//
// Data stay in the block fixed point of the fixed-point engine (64-bit
// integers below 2^B, per-transform power-of-two scale, 60-bit limb twiddles
// on the CUDA cores).  For a radix-16 pass each butterfly input x is cut to
// its top 48 bits, t = x >> (B - 47), and written as six balanced 8-bit
// digits, t = sum_i d_i 2^(8(5-i)), d_i in [-128, 128] (exact in BF16), where
// B is the bound of the pass's inputs (the block bound grown by the span of
// the earlier passes).  The
// 16-point DFT matrix, real-stacked as in the split form and scaled by 2^47,
// is cut the same way into f_j.  Every digit product |d_i f_j| <= 2^14 is
// exact in FP32, and so is every sum over one slice order s = i + j (at most
// 6 pairs x 32 terms < 2^22): the GEMMs of order s accumulate exactly in
// their own FP32 accumulator.  The 21 products with s <= 5 are kept (the rest
// are below 2^-47 of the result), and
//   sum_k x_k F_k = 2^(B-54) * C,  C = sum_s acc_s 2^(8(5-s)),  |C| < 2^58,
// recombined in 64-bit integers.  Error sources: the 48-bit cut of x, the
// dropped orders, the twiddle products and the final binary64 rounding.
#pragma once
#include <cuda_bf16.h>

#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "fft_split.cuh"
#include "internal.h"

namespace fftoc {

constexpr int kSplitExact = 3;
constexpr int kExactDigits = 6;  // 8-bit digits per operand
constexpr int kExactOrders = 6;  // slice orders s = 0..5 kept
constexpr int kExactPairs = 21;  // (i, j) with i + j <= 5

// Pair q in order of s = i + j: (0,0) | (0,1) (1,0) | (0,2) (1,1) (2,0) | ...
FFTOC_HD constexpr int exact_pair_i(int q) {
  int s = 0;
  while (q > s) { q -= s + 1; ++s; }
  return q;
}
FFTOC_HD constexpr int exact_pair_s(int q) {
  int s = 0;
  while (q > s) { q -= s + 1; ++s; }
  return s;
}

template <class PL, int G>
struct ExactPlan {
  using L = OpLayout<2>;  // BF16 operands
  static constexpr int N = PL::N, TPB = PL::TPB, P = PL::P, T = PL::T, NS = PL::S;
  static constexpr int THREADS = 128 * G;
  static_assert(P == 16 && PL::R[0] == 16, "radix-16 first pass, 16 points per thread");
  static_assert(T * TPB == THREADS, "one thread per radix-16 butterfly");
  static constexpr int B = FxBits<N>::B;  // bound of the first pass's inputs
  static_assert(B >= 49, "the 48-bit cut needs B >= 49");
  static constexpr int A_SLICE = 128 * L::ROW_BYTES;                // 8 KB
  static constexpr int A_BYTES = G * kExactDigits * A_SLICE;
  static constexpr int B_SLICE = 32 * L::ROW_BYTES;                 // 2 KB
  static constexpr int B_BYTES = kExactDigits * B_SLICE;
  static constexpr int SH = 4;
  static constexpr int NP = N + (N >> SH);
  static constexpr int DATA_OFF = A_BYTES + B_BYTES;
  static constexpr int DATA_BYTES = TPB * NP * 16;                  // longlong2 exchange
  static constexpr int RED_OFF = DATA_OFF + DATA_BYTES;
  static constexpr int BAR_OFF = RED_OFF + ((TPB * 4 + 15) / 16) * 16;
  static constexpr int SMEM = BAR_OFF + 8 * G + 8;
  // 6 orders x 32 columns per group, rounded up to a power of two: one group
  // takes 256 columns, so two one-group CTAs share an SM's TMEM
  static constexpr int TMEM_COLS = G == 1 ? 256 : 512;
  static_assert(32 * kExactOrders * G <= TMEM_COLS, "accumulators fit in TMEM");
  static_assert(G <= 2, "named barriers 1 and 2 serve the two groups");
  static constexpr bool GROUP_LOCAL = T <= 128;
  __device__ __forceinline__ static int slot(int j, int e) { return j * NP + e + (e >> SH); }
};

// Six balanced 8-bit digits (most significant first) of the top 48 bits of x
// (|x| < 2^B, B >= 49), as exact floats.
template <int B>
__device__ __forceinline__ void exact_digits(long long x, float (&d)[kExactDigits]) {
  const long long t = x >> (B - 47);  // |t| < 2^47
  int lo = (int)((unsigned)t & 0xFFFFFFu);  // low 24 bits, unsigned
  int hi = (int)(t >> 24);                  // |hi| < 2^23
#pragma unroll
  for (int q = 5; q >= 3; --q) {
    int v;
    asm("bfe.s32 %0, %1, 0, 8;" : "=r"(v) : "r"(lo));  // sign-extended low byte
    d[q] = __int_as_float(0x4B400000 + v) - 12582912.0f;
    lo = (lo - v) >> 8;
  }
  hi += lo;  // carry out of the low 24 bits (0 or 1)
#pragma unroll
  for (int q = 2; q >= 1; --q) {
    int v;
    asm("bfe.s32 %0, %1, 0, 8;" : "=r"(v) : "r"(hi));
    d[q] = __int_as_float(0x4B400000 + v) - 12582912.0f;
    hi = (hi - v) >> 8;
  }
  d[0] = __int_as_float(0x4B400000 + hi) - 12582912.0f;  // |hi| <= 128
}

// The thread's A rows: 32 real-stacked values (re 0..15, im 0..15) as six
// digit slices.
template <int B, int A_SLICE>
__device__ __forceinline__ void store_exact_slices(unsigned char* a_group, int row, const long long (&re)[16],
                                                   const long long (&im)[16]) {
  using L = OpLayout<2>;
#pragma unroll
  for (int c = 0; c < 4; ++c) {  // chunk c: K elements 8c..8c+7
    unsigned w[kExactDigits][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = (c & 1) * 8 + 2 * q;
      float da[kExactDigits], db[kExactDigits];
      exact_digits<B>(c < 2 ? re[e] : im[e], da);
      exact_digits<B>(c < 2 ? re[e + 1] : im[e + 1], db);
#pragma unroll
      for (int s = 0; s < kExactDigits; ++s) w[s][q] = bf16x2_bits(__floats2bfloat162_rn(da[s], db[s]));
    }
    const int off = L::chunk_off(row, c);
#pragma unroll
    for (int s = 0; s < kExactDigits; ++s)
      *reinterpret_cast<uint4*>(a_group + s * A_SLICE + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
  }
}

// FP32 accumulator (an exact integer, |v| < 2^22) to int.
__device__ __forceinline__ int exact_int(float v) { return __float_as_int(v + 12582912.0f) - 0x4B400000; }

template <int R, int Bq, int... bs>
__device__ __forceinline__ void exact_small_dfts(long long (&re)[16], long long (&im)[16],
                                                 std::integer_sequence<int, bs...>) {
  (dft<EngFx, R, bs, Bq, 16>(re, im), ...);
}

// Where and how the last pass stores: binary64 conversion of the block fixed
// point (the fixed-point engine's fast, slow and non-finite paths).
struct ExactOut {
  double2* dst;
  bool active, slow, special;
  int kshift, K;
};

struct ExactCtx {
  unsigned char* sA;
  unsigned char* sB;
  longlong2* data;
  unsigned long long* bar;
  const int4* tw;
  unsigned tmem, idesc, phase;
  int tid, g, row, lane_block, j, t;
  bool failed;
};

template <class PL, int G, int s>
__device__ __forceinline__ void exact_pass(ExactCtx& c, long long (&re)[16], long long (&im)[16], const ExactOut& o) {
  using XP = ExactPlan<PL, G>;
  using L = OpLayout<2>;
  constexpr int T = PL::T, NS = PL::S;
  constexpr int R = PL::R[s];
  constexpr int p = PL::span(s);
  constexpr int Bq = 16 / R;
  static_assert(R == 16 || s == NS - 1, "radix 2/4/8 only in the last pass");
  // inputs of pass s are sums of p inputs of the transform: |x| < 2^BS
  constexpr int BS = XP::B + ilog2c(p);
  static_assert(BS + ilog2c(R) <= 61, "outputs stay below 2^61");
  if constexpr (s > 0) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const longlong2 v = c.data[XP::slot(c.j, c.t + T * i)];
      re[i] = v.x;
      im[i] = v.y;
    }
  }
  if constexpr (R == 16) {
    if constexpr (s > 0) {
      const int k = c.t & (p - 1);
      const int4* base = c.tw + PL::tw_offset(s) + k;
#pragma unroll
      for (int m = 1; m < 16; ++m) EngFx::cmul(re[m], im[m], __ldg(base + (m - 1) * p));
    }
    store_exact_slices<BS, XP::A_SLICE>(c.sA + c.g * kExactDigits * XP::A_SLICE, c.row, re, im);
    fence_proxy_async_smem();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    tile_sync<XP::GROUP_LOCAL>(c.g);
    if (c.row == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned a0 = smem_u32(c.sA + c.g * kExactDigits * XP::A_SLICE), b0 = smem_u32(c.sB);
#pragma unroll
      for (int q = 0; q < kExactPairs; ++q)
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
          const int i = exact_pair_i(q), so = exact_pair_s(q), jj = so - i;
          const unsigned aa = a0 + i * XP::A_SLICE + kk * 256;
          const unsigned bb = b0 + jj * XP::B_SLICE + kk * 256;
          // the first product of each order starts its accumulator
          const bool first = (i == 0) && (kk == 0);
          umma<kSplitBF16x3>(c.tmem + 32 * (kExactOrders * c.g + so), umma_desc(aa, 128, L::KC * 128),
                             umma_desc(bb, 128, L::KC * 128), c.idesc, first ? 0u : 1u);
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(c.bar + c.g))
                   : "memory");
    }
    if (!c.failed && !mbar_wait_bounded(c.bar + c.g, c.phase, kWaitLimitNs)) c.failed = true;
    c.phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // C = sum_s acc_s 2^(8(5-s)); outputs = C * 2^(B-54), rounded
    long long cr[16], ci[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) cr[m] = ci[m] = 0;
#pragma unroll
    for (int so = 0; so < kExactOrders; ++so) {
      float d[32];
      tmem_ld32(c.tmem + ((unsigned)(c.lane_block * 32) << 16) + 32 * (kExactOrders * c.g + so), d);
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        cr[m] += (long long)exact_int(d[m]) << (8 * (5 - so));
        ci[m] += (long long)exact_int(d[16 + m]) << (8 * (5 - so));
      }
    }
    constexpr int SHR = 54 - BS;  // outputs = C * 2^-SHR: rounded right shift, or exact left shift
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      if constexpr (SHR > 0) {
        re[m] = (cr[m] + (1LL << (SHR - 1))) >> SHR;
        im[m] = (ci[m] + (1LL << (SHR - 1))) >> SHR;
      } else {
        re[m] = cr[m] << (-SHR);
        im[m] = ci[m] << (-SHR);
      }
    }
  } else {
    // last pass of radix 2/4/8 on the CUDA cores, fixed point
#pragma unroll
    for (int b = 0; b < Bq; ++b) {
      const int tp = c.t + T * b;
      const int k = tp & (p - 1);
      const int4* base = c.tw + PL::tw_offset(s) + k;
#pragma unroll
      for (int m = 1; m < R; ++m) EngFx::cmul(re[b + Bq * m], im[b + Bq * m], __ldg(base + (m - 1) * p));
    }
    exact_small_dfts<R, Bq>(re, im, std::make_integer_sequence<int, Bq>{});
  }
  if constexpr (s + 1 < NS) {
#pragma unroll
    for (int b = 0; b < Bq; ++b)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        const int tp = c.t + T * b;
        const int k = tp & (p - 1);
        c.data[XP::slot(c.j, (tp - k) * R + k + m * p)] = make_longlong2(re[b + Bq * m], im[b + Bq * m]);
      }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    tile_sync<XP::GROUP_LOCAL>(c.g);
    exact_pass<PL, G, s + 1>(c, re, im, o);
  } else if (o.active) {
    const double qnan = __longlong_as_double(0x7FF8000000000000LL);
#pragma unroll
    for (int b = 0; b < Bq; ++b)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        const int tp = c.t + T * b;
        const int k = tp & (p - 1);
        const long long xr = re[b + Bq * m], xi = im[b + Bq * m];
        double2 v;
        if (o.special) v = make_double2(qnan, qnan);
        else if (o.slow) v = make_double2(fx_out_slow(xr, o.K), fx_out_slow(xi, o.K));
        else v = make_double2(fx_out(xr, o.kshift), fx_out(xi, o.kshift));
        o.dst[(tp - k) * R + k + m * p] = v;
      }
  }
}

template <class PL, int G>
__global__ void __launch_bounds__(128 * G, 1)
fft_exact_kernel(const double2* __restrict__ in, double2* __restrict__ out, long long batch,
                 const int4* __restrict__ tw, const uint4* __restrict__ bmat, int* __restrict__ err) {
  using XP = ExactPlan<PL, G>;
  constexpr int N = PL::N, TPB = PL::TPB, T = PL::T;
  extern __shared__ __align__(1024) unsigned char smem_exact[];
  int* red = reinterpret_cast<int*>(smem_exact + XP::RED_OFF);
  unsigned* tslot = reinterpret_cast<unsigned*>(smem_exact + XP::BAR_OFF + 8 * G);

  ExactCtx c;
  c.sA = smem_exact;
  c.sB = smem_exact + XP::A_BYTES;
  c.data = reinterpret_cast<longlong2*>(smem_exact + XP::DATA_OFF);
  c.bar = reinterpret_cast<unsigned long long*>(smem_exact + XP::BAR_OFF);
  c.tw = tw;
  c.tid = threadIdx.x;
  c.g = c.tid >> 7;
  c.row = c.tid & 127;
  c.lane_block = (c.tid >> 5) & 3;
  c.j = c.tid / T;
  c.t = c.tid - c.j * T;
  c.failed = false;
  const int warp = c.tid >> 5;

  for (int i = c.tid; i < XP::B_BYTES / 16; i += XP::THREADS) reinterpret_cast<uint4*>(c.sB)[i] = __ldg(bmat + i);
  if (c.tid == 0) {
    for (int gg = 0; gg < G; ++gg) mbar_init(c.bar + gg, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(XP::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_proxy_async_smem();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  c.tmem = *tslot;
  c.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);  // BF16 -> FP32
  c.phase = 0;

  const long long ntiles = (batch + TPB - 1) / TPB;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (c.tid == 0) prefetch_next_tile<N, TPB>(in, tile, batch);
    const long long tr = tile * TPB + c.j;
    const bool active = tr < batch;
    double2 raw[16];
    const double2* src = in + tr * N + c.t;
#pragma unroll
    for (int i = 0; i < 16; ++i) raw[i] = active ? __ldg(src + T * i) : make_double2(0.0, 0.0);
    int em = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) em = max(em, max(expo_of(hi_word(raw[i].x)), expo_of(hi_word(raw[i].y))));
    if constexpr (T > 1 && T <= 32) {
#pragma unroll
      for (int o = T / 2; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o, T));
    } else if constexpr (T > 32) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
      if (c.tid < TPB) red[c.tid] = 0;
      __syncthreads();
      if ((c.tid & 31) == 0) atomicMax(&red[c.j], em);
      __syncthreads();
      em = red[c.j];
    }
    const FxScale sc = fx_scale<XP::B>(em);
    long long re[16], im[16];
    fx_convert_in<16>(raw, re, im, sc.eref);
    const ExactOut o{out + tr * N, active, sc.slow, sc.special, sc.kshift, sc.K};
    exact_pass<PL, G, 0>(c, re, im, o);
    if (__syncthreads_or(c.failed)) {
      if (c.tid == 0) atomicOr(err, kErrTimeout);
      mbar_wait_bounded(c.bar + c.g, c.phase ^ 1, kWaitLimitNs);  // bounded drain of the MMAs in flight
      break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(XP::TMEM_COLS));
}

}  // namespace fftoc
