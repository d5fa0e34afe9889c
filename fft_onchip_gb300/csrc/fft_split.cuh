// fftoc — split-precision form: the radix-16 DFT stages as BF16 / TF32
// tensor-core GEMMs (tcgen05.mma, accumulators in TMEM), operands split into
// 3 BF16 or 2 TF32 terms, FP32 accumulation, FP32 data between stages.
//
// The reference's tensor path multiplies complex matrices on the FP64 tensor
// core with the Karatsuba scheme (tensor_utils.cuh:3-36, tensor_fft_64.cuh
// :12-77).  Here each radix-16 pass of the Stockham plan is one GEMM per 128
// butterflies:
//   D[b][c] = sum_k A[b][k] * B[c][k],  k, c in [0, 32)
// A row b = butterfly b's 16 twiddled inputs, real-stacked (re 0..15, im
// 0..15); B = the 16-point DFT matrix real-stacked ([[Fr, -Fi], [Fi, Fr]]),
// so D row b = the butterfly's 16 outputs (re 0..15, im 0..15).  With
// x = x0 + x1 + x2 (BF16 terms of the FP32 value) and F = F0 + F1 + F2, the
// six products x_i F_j with i + j <= 2 accumulate into the same FP32
// accumulator (BF16x3); with two TF32 terms, the three products with
// i + j <= 1 (TF32x2).  Twiddles (FP32 table from long-double values) and
// the short last pass of radix 2/4/8 run on the CUDA cores in FP32.
//
// CTA: 128*G threads = G groups of 128 butterflies (one thread per butterfly
// row); thread 0 issues the G*12 MMAs of a pass and commits them to an
// mbarrier that every thread waits on (bounded); each warp reads its 32 TMEM
// lanes.  Persistent CTAs stride over tiles of TPB transforms.
#pragma once
#include <cuda_bf16.h>

#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "internal.h"

namespace fftoc {

constexpr int kSplitBF16x3 = 1;
constexpr int kSplitTF32x2 = 2;

template <int KIND> struct SplitT;
template <> struct SplitT<kSplitBF16x3> {
  static constexpr int ESIZE = 2;     // bytes per operand element
  static constexpr int SLICES = 3;
  static constexpr int NPAIRS = 6;
  static constexpr int KMMA = 16;     // K of one MMA
  static constexpr unsigned FMT = 1;  // BF16 in kind::f16
  __host__ __device__ static constexpr int pair_x(int q) { return q == 0 ? 0 : q == 1 ? 1 : q == 2 ? 0 : q == 3 ? 2 : q == 4 ? 1 : 0; }
  __host__ __device__ static constexpr int pair_f(int q) { return q == 0 ? 0 : q == 1 ? 0 : q == 2 ? 1 : q == 3 ? 0 : q == 4 ? 1 : 2; }
};
template <> struct SplitT<kSplitTF32x2> {
  static constexpr int ESIZE = 4;
  static constexpr int SLICES = 2;
  static constexpr int NPAIRS = 3;
  static constexpr int KMMA = 8;
  static constexpr unsigned FMT = 2;  // TF32 in kind::tf32
  __host__ __device__ static constexpr int pair_x(int q) { return q == 1 ? 1 : 0; }
  __host__ __device__ static constexpr int pair_f(int q) { return q == 2 ? 1 : 0; }
};

// Operand tile of R rows x 32 K-elements in the no-swizzle K-major layout:
// core matrix (8 rows x 16 bytes) (i, j) at (i * KC + j) * 128 bytes, so the
// descriptor's leading (K) byte offset is 128 and its stride (row-group)
// byte offset KC * 128.
template <int ESIZE>
struct OpLayout {
  static constexpr int ROW_BYTES = 32 * ESIZE;
  static constexpr int KC = ROW_BYTES / 16;  // 16-byte K chunks per row
  static constexpr int PER_CHUNK = 16 / ESIZE;
  FFTOC_HD static int chunk_off(int row, int chunk) { return ((row >> 3) * KC + chunk) * 128 + (row & 7) * 16; }
};

template <int KIND, class PL, int G>
struct SplitPlan {
  using K = SplitT<KIND>;
  using L = OpLayout<K::ESIZE>;
  static constexpr int N = PL::N, TPB = PL::TPB, P = PL::P, T = PL::T, NS = PL::S;
  static constexpr int THREADS = 128 * G;
  static_assert(P == 16 && PL::R[0] == 16, "radix-16 first pass, 16 points per thread");
  static_assert(T * TPB == THREADS, "one thread per radix-16 butterfly");
  static constexpr int A_SLICE = 128 * L::ROW_BYTES;
  static constexpr int A_BYTES = G * K::SLICES * A_SLICE;
  static constexpr int B_SLICE = 32 * L::ROW_BYTES;
  static constexpr int B_BYTES = K::SLICES * B_SLICE;
  static constexpr int SH = 4;
  static constexpr int NP = N + (N >> SH);
  static constexpr int DATA_OFF = A_BYTES + B_BYTES;
  static constexpr int DATA_BYTES = TPB * NP * 8;
  static constexpr int RED_OFF = DATA_OFF + DATA_BYTES;  // per-transform exponent scratch
  static constexpr int BAR_OFF = RED_OFF + ((TPB * 4 + 15) / 16) * 16;
  static constexpr int SMEM = BAR_OFF + 8 * G + 8;  // one mbarrier per group + TMEM address slot
  // a transform's threads lie inside one 128-row group: the groups need no
  // CTA-wide barrier inside a tile
  static constexpr bool GROUP_LOCAL = T <= 128;
  static_assert(G <= 2, "named barriers 1 and 2 serve the two groups");
  static constexpr int TMEM_COLS = 32 * G < 32 ? 32 : 32 * G;
  static constexpr int MMAS = K::NPAIRS * (32 / K::KMMA);
  static_assert((TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM allocation is a power of two");
  __device__ __forceinline__ static int slot(int j, int e) { return j * NP + e + (e >> SH); }
};

__device__ __forceinline__ unsigned long long umma_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFF) | ((unsigned long long)((lbo >> 4) & 0x3FFF) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

template <int KIND>
__device__ __forceinline__ void umma(unsigned d_tmem, unsigned long long a, unsigned long long b, unsigned idesc,
                                     unsigned acc) {
  if constexpr (KIND == kSplitTF32x2)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Bulk prefetch of [p, p + bytes) into L2 (no shared memory involved);
// p 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// The next tile of a persistent CTA into L2 while it works on this one.
template <int N, int TPB>
__device__ __forceinline__ void prefetch_next_tile(const double2* in, long long tile, long long batch) {
  const long long next = tile + gridDim.x;
  const long long first = next * TPB;
  if (first >= batch) return;
  const long long count = batch - first < TPB ? batch - first : TPB;
  const char* p = reinterpret_cast<const char*>(in + first * N);
  long long bytes = count * N * 16;
  while (bytes > 0) {  // in pieces of at most 64 KiB
    const unsigned b = bytes > 65536 ? 65536u : (unsigned)bytes;
    prefetch_l2(p, b);
    p += b;
    bytes -= b;
  }
}

__device__ __forceinline__ unsigned tf32_rna(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ unsigned bf16x2_bits(__nv_bfloat162 h) {
  unsigned u;
  memcpy(&u, &h, 4);
  return u;
}

// Write the A row of this thread (32 real-stacked values) as operand slices.
template <int KIND, int A_SLICE>
__device__ __forceinline__ void store_slices(unsigned char* a_group, int row, const float (&re)[16],
                                             const float (&im)[16]) {
  using L = OpLayout<SplitT<KIND>::ESIZE>;
  if constexpr (KIND == kSplitBF16x3) {
    // chunk c holds K elements 8c..8c+7: chunks 0,1 = re 0..15, chunks 2,3 = im 0..15
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      unsigned w[3][4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = (c & 1) * 8 + 2 * q;
        const float a = c < 2 ? re[e] : im[e];
        const float b = c < 2 ? re[e + 1] : im[e + 1];
        const __nv_bfloat162 h0 = __floats2bfloat162_rn(a, b);
        const float a1 = a - __low2float(h0), b1 = b - __high2float(h0);
        const __nv_bfloat162 h1 = __floats2bfloat162_rn(a1, b1);
        const float a2 = a1 - __low2float(h1), b2 = b1 - __high2float(h1);
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(a2, b2);
        w[0][q] = bf16x2_bits(h0);
        w[1][q] = bf16x2_bits(h1);
        w[2][q] = bf16x2_bits(h2);
      }
      const int off = L::chunk_off(row, c);
#pragma unroll
      for (int s = 0; s < 3; ++s)
        *reinterpret_cast<uint4*>(a_group + s * A_SLICE + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
  } else {
    // chunk c holds K elements 4c..4c+3: chunks 0..3 = re 0..15, chunks 4..7 = im 0..15
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      unsigned w0[4], w1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = (c & 3) * 4 + q;
        const float x = c < 4 ? re[e] : im[e];
        const unsigned t0 = tf32_rna(x);
        w0[q] = t0;
        w1[q] = tf32_rna(x - __uint_as_float(t0));
      }
      const int off = L::chunk_off(row, c);
      *reinterpret_cast<uint4*>(a_group + off) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
      *reinterpret_cast<uint4*>(a_group + A_SLICE + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    }
  }
}

// binary64 -> FP32 on the integer pipes (the FP64 pipe of this part is the
// scarcest unit): exponent rebias, 23 mantissa bits rounded half up on the
// magnitude; below the FP32 normal range -> 0, non-finite -> NaN.  Callers
// keep finite magnitudes below 2^64 (per-transform scaling).
__device__ __forceinline__ float f64_to_f32_int(double v) {
  const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
  const int e = (int)((hi >> 20) & 0x7FFu) - (1023 - 127);
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  unsigned bits = ((unsigned)e << 23) + m + ((lo >> 28) & 1u);
  bits = e > 0 ? bits : 0u;
  bits = e >= 255 ? 0x7FC00000u : bits;
  return __uint_as_float(bits | (hi & 0x80000000u));
}

// FP32 -> binary64 (exact) on the integer pipes; FP32 subnormals -> 0.
__device__ __forceinline__ double f32_to_f64_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu, sgn = u & 0x80000000u;
  unsigned hi = sgn | ((e + (1023u - 127u)) << 20) | ((u & 0x7FFFFFu) >> 3);
  unsigned lo = u << 29;
  if (e == 0) { hi = sgn; lo = 0; }
  if (e == 255) hi = sgn | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

// Small DFT of radix R (2, 4 or 8) on points b + B*m, FP32, natural-order output.
template <int R, int B>
__device__ __forceinline__ void dft_small(float (&re)[16], float (&im)[16], int b) {
  float xr[R], xi[R];
#pragma unroll
  for (int m = 0; m < R; ++m) { xr[m] = re[b + B * m]; xi[m] = im[b + B * m]; }
#pragma unroll
  for (int c = 0; c < R; ++c) {
    float sr = 0.f, si = 0.f;
#pragma unroll
    for (int m = 0; m < R; ++m) {
      // exp(-2 pi i c m / R)
      const int q = (c * m) % R;
      float wr, wi;
      if constexpr (R == 2) { wr = q ? -1.f : 1.f; wi = 0.f; }
      else if constexpr (R == 4) {
        wr = q == 0 ? 1.f : q == 2 ? -1.f : 0.f;
        wi = q == 1 ? -1.f : q == 3 ? 1.f : 0.f;
      } else {
        constexpr float h = 0.70710678118654752440f;
        const float cr[8] = {1.f, h, 0.f, -h, -1.f, -h, 0.f, h};
        const float ci[8] = {0.f, -h, -1.f, -h, 0.f, h, 1.f, h};
        wr = cr[q];
        wi = ci[q];
      }
      sr += xr[m] * wr - xi[m] * wi;
      si += xr[m] * wi + xi[m] * wr;
    }
    re[b + B * c] = sr;
    im[b + B * c] = si;
  }
}

// Multiply this thread's stored outputs by 2^unshift (exact, binary64).
template <int T, int R, int Bq, int p>
__device__ __noinline__ void split_unscale_outputs(double2* dst, int t, int unshift) {
  for (int b = 0; b < Bq; ++b)
    for (int m = 0; m < R; ++m) {
      const int tp = t + T * b;
      const int k = tp & (p - 1);
      double2* q = dst + (tp - k) * R + k + m * p;
      const double2 v = *q;
      *q = make_double2(ldexp(v.x, unshift), ldexp(v.y, unshift));
    }
}

// Per-CTA state shared by the passes.
struct SplitCtx {
  unsigned char* sA;
  unsigned char* sB;
  float2* data;
  unsigned long long* bar;  // one per group
  const float2* tw;
  unsigned tmem, idesc, phase;
  int tid, g, row, lane_block, j, t;
  bool failed;  // a bounded wait gave up (the tile loop ends after the tile)
};

// Barrier over the threads that share data inside a tile: the thread's
// 128-row group when transforms do not span groups, else the CTA.
template <bool GROUP_LOCAL>
__device__ __forceinline__ void tile_sync(int g) {
  if constexpr (GROUP_LOCAL) {
    // immediate barrier ids (a register id would reserve all 16 named barriers)
    if (g == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
    else asm volatile("bar.sync 2, 128;" ::: "memory");
  } else {
    __syncthreads();
  }
}

// Pass s of the plan on the thread's 16 points; the last pass stores to
// `dst` (transform base, binary64).  A bounded wait that gives up sets
// c.failed; the passes still run their barriers so every thread reaches the
// end of the tile.
template <int KIND, class PL, int G, int s>
__device__ __forceinline__ void split_pass(SplitCtx& c, float (&re)[16], float (&im)[16], double2* dst, bool active,
                                           int unshift, bool scaled) {
  using SP = SplitPlan<KIND, PL, G>;
  using K = SplitT<KIND>;
  using L = OpLayout<K::ESIZE>;
  constexpr int T = PL::T, NS = PL::S;
  constexpr int R = PL::R[s];
  constexpr int p = PL::span(s);
  constexpr int Bq = 16 / R;
  static_assert(R == 16 || s == NS - 1, "radix 2/4/8 only in the last pass");
  if constexpr (s > 0) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const float2 v = c.data[SP::slot(c.j, c.t + T * i)];
      re[i] = v.x;
      im[i] = v.y;
    }
  }
  if constexpr (R == 16) {
    if constexpr (s > 0) {
      const int k = c.t & (p - 1);
      const float2* base = c.tw + PL::tw_offset(s) + k;
#pragma unroll
      for (int m = 1; m < 16; ++m) {
        const float2 w = __ldg(base + (m - 1) * p);
        const float xr = re[m], xi = im[m];
        re[m] = xr * w.x - xi * w.y;
        im[m] = xr * w.y + xi * w.x;
      }
    }
    store_slices<KIND, SP::A_SLICE>(c.sA + c.g * K::SLICES * SP::A_SLICE, c.row, re, im);
    fence_proxy_async_smem();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    tile_sync<SP::GROUP_LOCAL>(c.g);
    if (c.row == 0) {
      // row 0 of each group issues that group's MMAs and commits them to its mbarrier
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned a0 = smem_u32(c.sA + c.g * K::SLICES * SP::A_SLICE), b0 = smem_u32(c.sB);
#pragma unroll
      for (int q = 0; q < K::NPAIRS; ++q)
#pragma unroll
        for (int kk = 0; kk < 32 / K::KMMA; ++kk) {
          // K elements [kk*KMMA, kk*KMMA + KMMA) = 16-byte chunks 2kk, 2kk+1
          const unsigned aa = a0 + K::pair_x(q) * SP::A_SLICE + kk * 256;
          const unsigned bb = b0 + K::pair_f(q) * SP::B_SLICE + kk * 256;
          umma<KIND>(c.tmem + 32 * c.g, umma_desc(aa, 128, L::KC * 128), umma_desc(bb, 128, L::KC * 128), c.idesc,
                     (q | kk) != 0);
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(c.bar + c.g))
                   : "memory");
    }
    if (!c.failed && !mbar_wait_bounded(c.bar + c.g, c.phase, kWaitLimitNs)) c.failed = true;
    c.phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    float d[32];
    tmem_ld32(c.tmem + ((unsigned)(c.lane_block * 32) << 16) + 32 * c.g, d);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      re[m] = d[m];
      im[m] = d[16 + m];
    }
  } else {
    // last pass of radix 2/4/8 on the CUDA cores: 16/R butterflies per thread
#pragma unroll
    for (int b = 0; b < Bq; ++b) {
      const int tp = c.t + T * b;
      const int k = tp & (p - 1);
      const float2* base = c.tw + PL::tw_offset(s) + k;
#pragma unroll
      for (int m = 1; m < R; ++m) {
        const float2 w = __ldg(base + (m - 1) * p);
        const float xr = re[b + Bq * m], xi = im[b + Bq * m];
        re[b + Bq * m] = xr * w.x - xi * w.y;
        im[b + Bq * m] = xr * w.y + xi * w.x;
      }
      dft_small<R, Bq>(re, im, b);
    }
  }
  // output m of butterfly b is element dest = (tp - k) * R + k + m * p
  if constexpr (s + 1 < NS) {
#pragma unroll
    for (int b = 0; b < Bq; ++b)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        const int tp = c.t + T * b;
        const int k = tp & (p - 1);
        c.data[SP::slot(c.j, (tp - k) * R + k + m * p)] = make_float2(re[b + Bq * m], im[b + Bq * m]);
      }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");  // this pass's TMEM reads precede the next MMAs
    tile_sync<SP::GROUP_LOCAL>(c.g);
    split_pass<KIND, PL, G, s + 1>(c, re, im, dst, active, unshift, scaled);
  } else {
    if (active) {
#pragma unroll
      for (int b = 0; b < Bq; ++b)
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const int tp = c.t + T * b;
          const int k = tp & (p - 1);
          const double xr = f32_to_f64_int(re[b + Bq * m]), xi = f32_to_f64_int(im[b + Bq * m]);
          dst[(tp - k) * R + k + m * p] = make_double2(xr, xi);
        }
      // rare transforms scaled at the input: undo the scale in place, out of
      // line (an if-converted ldexp would occupy the FP64 pipe for every value)
      if (scaled) split_unscale_outputs<T, R, Bq, p>(dst, c.t, unshift);
    }
  }
}

template <int KIND, class PL, int G>
__global__ void __launch_bounds__(128 * G, PL::MINB)
fft_split_kernel(const double2* __restrict__ in, double2* __restrict__ out, long long batch,
                 const float2* __restrict__ tw, const uint4* __restrict__ bmat, int* __restrict__ err) {
  using SP = SplitPlan<KIND, PL, G>;
  using K = SplitT<KIND>;
  constexpr int N = PL::N, TPB = PL::TPB, T = PL::T;
  extern __shared__ __align__(1024) unsigned char smem_split[];
  int* red = reinterpret_cast<int*>(smem_split + SP::RED_OFF);
  unsigned* tslot = reinterpret_cast<unsigned*>(smem_split + SP::BAR_OFF + 8 * G);

  SplitCtx c;
  c.sA = smem_split;
  c.sB = smem_split + SP::A_BYTES;
  c.data = reinterpret_cast<float2*>(smem_split + SP::DATA_OFF);
  c.bar = reinterpret_cast<unsigned long long*>(smem_split + SP::BAR_OFF);
  c.tw = tw;
  c.tid = threadIdx.x;
  c.g = c.tid >> 7;
  c.row = c.tid & 127;
  c.lane_block = (c.tid >> 5) & 3;
  c.j = c.tid / T;
  c.t = c.tid - c.j * T;
  const int warp = c.tid >> 5;

  // constant DFT-matrix slices, TMEM, mbarrier
  for (int i = c.tid; i < SP::B_BYTES / 16; i += SP::THREADS) reinterpret_cast<uint4*>(c.sB)[i] = __ldg(bmat + i);
  if (c.tid == 0) {
    for (int gg = 0; gg < G; ++gg) mbar_init(c.bar + gg, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(SP::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_proxy_async_smem();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  c.tmem = *tslot;
  c.idesc = (1u << 4) | (K::FMT << 7) | (K::FMT << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
  c.phase = 0;
  c.failed = false;

  const long long ntiles = (batch + TPB - 1) / TPB;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (c.tid == 0) prefetch_next_tile<N, TPB>(in, tile, batch);
    const long long tr = tile * TPB + c.j;
    const bool active = tr < batch;
    // ---- load: point i of this thread is element t + T*i; per-transform
    // power-of-two scale when the largest magnitude is outside [2^-60, 2^60]
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
    // largest magnitude in [2^(em-1023), 2^(em-1022)); outside [2^-60, 2^60]
    // (or all subnormal, em = 0) scale it to ~1 by an exact power of two
    const bool scaled = em < 2047 && (em > 1023 + 60 || em < 1023 - 60);
    const int shift = scaled ? (em == 0 ? 1023 + 52 : 1023 - em) : 0;
    if (scaled) {  // rare: exact binary64 scaling by 2^shift
#pragma unroll
      for (int i = 0; i < 16; ++i) raw[i] = make_double2(ldexp(raw[i].x, shift), ldexp(raw[i].y, shift));
    }
    float re[16], im[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      re[i] = f64_to_f32_int(raw[i].x);
      im[i] = f64_to_f32_int(raw[i].y);
    }
    split_pass<KIND, PL, G, 0>(c, re, im, out + tr * N, active, -shift, scaled);
    // exchange buffer and exponent scratch free for the next tile; stop after
    // a bounded wait gave up anywhere in the CTA
    if (__syncthreads_or(c.failed)) {
      if (c.tid == 0) atomicOr(err, kErrTimeout);
      mbar_wait_bounded(c.bar + c.g, c.phase ^ 1, kWaitLimitNs);  // bounded drain of the MMAs in flight
      break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(SP::TMEM_COLS));
}

}  // namespace fftoc
