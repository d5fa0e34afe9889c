// fftoc — exact-slice split form: radix-16 passes on the FP16 tensor cores
// with products that are exact in FP32, for relative errors ~1e-14.
//
// Data stay in 64-bit block fixed point (per-transform power-of-two scale,
// 60-bit limb twiddles on the CUDA cores).  A radix-16 pass's inputs are
// below 2^BS: BS = B (the fixed-point engine's block bound) for the first
// pass, 59 for later ones.  Each butterfly input x is cut to its top 49 bits,
// t = x >> (BS - 48), and written as six balanced digits,
// t = sum_i d_i 2^(8(5-i)), d_i in [-128, 127] for i >= 1 and d_0 in
// [-256, 256]: the offset-binary digits of u = t + 0x1008080808080 (bytes
// 0..4 offset by 128, bits 40..49 by 256), each turned into the FP16 value
// 1024 + digit by a byte permute and brought to its signed value by one FP16
// subtraction (all exact).  The 16-point DFT matrix, real-stacked and scaled
// by 2^46, is cut into balanced 8-bit digits f_j, |f_j| <= 128, |f_0| <= 64.
// Every digit product is exact, and so is every sum over one slice order
// s = i + j: at most 2^20 from the pair (0, s) and 2^19 from each other pair
// (32 terms), 3.5 2^20 < 2^22 for s = 5.  Each order accumulates exactly in
// its own FP32 accumulator, which starts at 1.5 * 2^23 so that its bit pattern
// is 0x4B400000 plus the integer.  The 21 digit pairs with s <= 5 are kept
// (the rest are below 2^-46 of the result), and
//   C = sum_s acc_s 2^(8(5-s)) = 2^-40 sum_k t_k F_k = 2^(54-BS) sum_k x_k F_k,
// recombined in integers (two orders per 32-bit word, one 64-bit sum) and
// kept as the next pass's input: each pass rescales the transform by a power
// of two, accounted for in the output conversion.  Bounds by modulus: inputs
// of modulus below sqrt2 2^BS give |C| <= 2^(54-BS) 16 sqrt2 2^BS = 2^58.5;
// twiddles keep the modulus, so later passes cut at BS = 59 and give
// |C| <= 2^-5 16 2^58.5 = 2^57.5, and a radix-2/4/8 last pass ends below
// 2^61.5 (inside int64; its constant products see at most 2^59.5).
//
// Operand layout (FP16, K-major core matrices of 8 rows x 16 bytes).  The A
// operand of a 128-row group is three K blocks, one per digit pair
// (d_0, d_1), (d_2, d_3), (d_4, d_5); in block q, K element 2v + e is digit
// 2q + e of input value v (v < 16: real part of input v, else imaginary
// part of input v - 16), so one 32-bit word holds two digits of one value.
// The B operand stacks six 32-row matrices: rows 32j..32j+31 hold, at K
// element 2v + e, digit j - e of the DFT matrix (zero for j - e < 0).  Block q
// times B rows 0..32(6-2q)-1 adds the pairs (2q, j) and (2q+1, j-1) to the
// orders 2q..5, so a pass is 3 blocks x 4 K steps = 12 MMAs of N = 192, 128
// and 64 into the accumulators (columns 64q..191).  Accumulator columns are
// 2m (real part of output m) and 2m+1 (imaginary part).
//
// Two threads serve each butterfly row: half h holds inputs and outputs
// 8h..8h+7, writes their A digits and reads its 16 accumulator columns of
// each order.
#pragma once
#include <cuda_fp16.h>

#include <cstring>

#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "fft_split.cuh"
#include "internal.h"

namespace fftoc {

constexpr int kSplitExact = 3;
constexpr int kExactDigits = 6;  // 8-bit digits per operand
constexpr int kExactOrders = 6;  // slice orders s = 0..5 kept (21 digit pairs)
constexpr int kExactBlocks = 3;  // digit pairs per operand row
constexpr int kExactBound = 59;  // components of radix-16 pass outputs are below 2^59

template <class PL, int G>
struct ExactPlan {
  static constexpr int N = PL::N, TPB = PL::TPB, P = PL::P, T = PL::T, NS = PL::S;
  static constexpr int ROWS = 128 * G;      // butterfly rows (TMEM lanes) per CTA
  static constexpr int THREADS = 2 * ROWS;  // two threads per row
  static_assert(P == 16 && PL::R[0] == 16, "radix-16 first pass, 16 points per butterfly row");
  static_assert(T * TPB == ROWS, "one row per radix-16 butterfly");
  // inputs are converted to block fixed point below 2^48: the first pass's
  // 49-bit cut is then the converted value itself (floor of a floor)
  static constexpr int B = 48;
  static constexpr int KC = 8;                        // 16-byte K chunks per operand row (64 FP16)
  static constexpr int A_BLOCK = 128 * KC * 16;       // 16 KB: one digit pair of 128 rows
  static constexpr int A_BYTES = G * kExactBlocks * A_BLOCK;
  static constexpr int B_ROWS = 32 * kExactOrders;    // 192
  static constexpr int B_BYTES = B_ROWS * KC * 16;    // 24 KB
  static constexpr int SH = 4;
  static constexpr int NP = N + (N >> SH);
  static constexpr int DATA_OFF = A_BYTES + B_BYTES;
  static constexpr int DATA_BYTES = TPB * NP * 16;    // longlong2 exchange
  static constexpr int W = T > 32 ? T / 32 : 1;       // exponent words per transform and half
  static constexpr int RED_OFF = DATA_OFF + DATA_BYTES;
  static constexpr int BAR_OFF = RED_OFF + ((2 * TPB * W * 4 + 15) / 16) * 16;
  static constexpr int SMEM = BAR_OFF + 8 * G + 8;
  // 6 orders x 32 columns per group; a group's accumulators start at column
  // 256 g (one-group CTAs allocate 256 columns, so two share an SM's TMEM)
  static constexpr int TMEM_COLS = G == 1 ? 256 : 512;
  static_assert(G <= 2, "at most two 128-row groups");
  // radix-16 passes; the first scales the transform by 2^(54 - B), each
  // later one by 2^(54 - 59), so outputs are y 2^(K + OUT_SHIFT) for the input
  // scale 2^K
  static constexpr int NR16 = PL::R[NS - 1] == 16 ? NS : NS - 1;
  static constexpr int OUT_SHIFT = (B - 54) + (kExactBound - 54) * (NR16 - 1);
  __device__ __forceinline__ static int slot(int j, int e) { return j * NP + e + (e >> SH); }
};

FFTOC_HD int exact_float_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_int(f);
#else
  int i;
  memcpy(&i, &f, 4);
  return i;
#endif
}

// Offset-binary form of the top 49 bits of x (|x| < 2^BS): the word
// (x >> (BS - 48)) + 0x1008080808080 < 2^50, whose byte 5 - i is digit
// i + 128 for i >= 1 and whose bits 40..49 are digit 0 + 256.
template <int BS>
FFTOC_HD unsigned long long exact_offset_bits(long long x) {
  constexpr int n = BS - 48;
  static_assert(n >= 0 && BS <= 60, "cut of a value below 2^BS");
  return (unsigned long long)(x + (0x1008080808080LL << n)) >> n;
}

// FP16 pair of signed digits from two offset digits a, b < 1024: the byte
// permute `sel` of `word` and 0x64 bytes makes the FP16 pair (1024 + a,
// 1024 + b) (low mantissa byte from the data, exponent byte 0x64 or, for the
// 10-bit top digit, 0x64 | bits 8..9), and subtracting `bias` (the FP16 pair
// 1024 + the offsets) is exact.
template <unsigned BIAS>
__device__ __forceinline__ unsigned exact_f16_pair(unsigned word, unsigned sel) {
  const unsigned biased = __byte_perm(word, 0x64646464u, sel);
  unsigned r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(biased), "r"(BIAS));
  return r;
}

// The three digit-pair words of x: (d_0, d_1), (d_2, d_3), (d_4, d_5).
template <int BS>
__device__ __forceinline__ void exact_digit_words(long long x, unsigned& w0, unsigned& w1, unsigned& w2) {
  const unsigned long long u = exact_offset_bits<BS>(x);
  const unsigned lo = (unsigned)u, hi = (unsigned)(u >> 32);
  // digit 0 is 10 bits: bits 48..49 (byte 2 of hi) go into its FP16
  // exponent byte 0x64 | bits; its offset is 256 (FP16 1280 = 0x6500)
  w0 = exact_f16_pair<0x64806500u>(hi | 0x00640000u, 0x4021);  // bits 40..49, byte 4
  w1 = exact_f16_pair<0x64806480u>(lo, 0x4243);                // bytes 3, 2
  w2 = exact_f16_pair<0x64806480u>(lo, 0x4041);                // bytes 1, 0
}

// One output from the bit patterns x[s] of its six order accumulators.  The
// accumulators start at 1.5 * 2^23 (exact_tmem_fill) and gather exact
// integers a[s], |a[s]| < 2^22, so each stays in [2^23, 2^24) and
// x[s] = 0x4B400000 + a[s].  Returns C = sum_s a[s] 2^(8(5-s)): pairs of
// orders are combined in 32 bits, (x[2i] - M) 2^8 + x[2i+1] = a[2i] 2^8 +
// a[2i+1] + M, which lies in [0, 2^31) for i = 1, 2, the three pairs in 64
// bits with one constant for the M terms.
FFTOC_HD long long exact_combine(unsigned x0, unsigned x1, unsigned x2, unsigned x3, unsigned x4, unsigned x5) {
  constexpr unsigned M = 0x4B400000u;
  constexpr unsigned long long KC = ((unsigned long long)(257u * M) << 32) + ((unsigned long long)M << 16) + M;
  const unsigned pa = x0 * 256u + x1;        // a0 2^8 + a1 + 257 M (mod 2^32)
  const unsigned pb = (x2 - M) * 256u + x3;  // a2 2^8 + a3 + M
  const unsigned pc = (x4 - M) * 256u + x5;  // a4 2^8 + a5 + M
  return (long long)(((unsigned long long)pb << 16) + pc + ((unsigned long long)pa << 32) - KC);
}

// Six 4-column TMEM loads (one per order, 32 columns apart) and the wait
// for them, in one statement so that no use of the values can be scheduled
// before the wait.
__device__ __forceinline__ void exact_tmem_ld6x4(unsigned taddr, unsigned (&v)[kExactOrders][4]) {
  unsigned r[24];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%24];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4,%5,%6,%7}, [%25];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8,%9,%10,%11}, [%26];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%12,%13,%14,%15}, [%27];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%28];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20,%21,%22,%23}, [%29];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
      : "r"(taddr), "r"(taddr + 32), "r"(taddr + 64), "r"(taddr + 96), "r"(taddr + 128), "r"(taddr + 160)
      : "memory");
#pragma unroll
  for (int s = 0; s < kExactOrders; ++s)
#pragma unroll
    for (int i = 0; i < 4; ++i) v[s][i] = r[4 * s + i];
}

// The same with 8 columns per order.
__device__ __forceinline__ void exact_tmem_ld6x8(unsigned taddr, unsigned (&v)[kExactOrders][8]) {
  unsigned r[48];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%48];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%49];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%50];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%51];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%32,%33,%34,%35,%36,%37,%38,%39}, [%52];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%40,%41,%42,%43,%44,%45,%46,%47}, [%53];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
      : "r"(taddr), "r"(taddr + 32), "r"(taddr + 64), "r"(taddr + 96), "r"(taddr + 128), "r"(taddr + 160)
      : "memory");
#pragma unroll
  for (int s = 0; s < kExactOrders; ++s)
#pragma unroll
    for (int i = 0; i < 8; ++i) v[s][i] = r[8 * s + i];
}

// The accumulator start value 1.5 * 2^23 into this thread's 16 columns of
// each order (`taddr`: its lanes, column 16h), and the wait for the stores.
__device__ __forceinline__ void exact_tmem_fill(unsigned taddr) {
  const unsigned m = 0x4B400000u;
#pragma unroll
  for (int s = 0; s < kExactOrders; ++s)
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(
            taddr + 32 * s),
        "r"(m)
        : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Where and how the last pass stores: binary64 conversion of the block fixed
// point (the fixed-point engine's fast, slow and non-finite paths).
struct ExactOut {
  double2* dst;
  bool active, slow, special;
  int kshift, K;
};

__device__ __forceinline__ double2 exact_out_value(const ExactOut& o, long long xr, long long xi) {
  if (o.special) {
    const double qnan = __longlong_as_double(0x7FF8000000000000LL);
    return make_double2(qnan, qnan);
  }
  if (o.slow) return make_double2(fx_out_slow(xr, o.K), fx_out_slow(xi, o.K));
  return make_double2(fx_out(xr, o.kshift), fx_out(xi, o.kshift));
}

struct ExactCtx {
  unsigned char* sA;  // this group's three A blocks
  unsigned char* sB;
  longlong2* data;
  unsigned long long* bar;  // this group's MMA barrier
  const int4* tw;
  unsigned tmem;            // this group's accumulators, lane 0
  unsigned tmem_rd;         // this thread's lanes and columns
  unsigned phase;
  int tid, g, h, row, j, t;
  bool issuer, failed;
  const double2* nsrc;  // this thread's first input of the next tile
  bool nactive;         // the next tile holds this thread's transform
};

// A thread's 8 inputs of a tile (zeros past the batch).
template <int T>
__device__ __forceinline__ void exact_load_inputs(double2 (&raw)[8], const double2* src, bool active) {
#pragma unroll
  for (int i = 0; i < 8; ++i) raw[i] = active ? __ldg(src + T * i) : make_double2(0.0, 0.0);
}

// Passes whose twiddles are loaded into registers before the barrier that
// precedes them: a radix-16 last pass after another radix-16 pass (measured
// 4 % faster at N = 256; loading the twiddles of earlier passes ahead, or
// into an array at all, measured 2-3 % slower at N = 512 and 4096 than
// loading each at its product).
template <class PL, int s>
constexpr bool EARLY_TW = s > 0 && s == PL::S - 1 && PL::R[s] == 16;

// The twiddles of radix-16 pass s (s >= 1) for this thread's inputs
// m = 8h + i: entry (m - 1) p + k (none for m = 0).
template <class PL, int s>
__device__ __forceinline__ void exact_load_twiddles(const ExactCtx& c, int4 (&w)[8]) {
  constexpr int p = PL::span(s);
  const int k = c.t & (p - 1);
  const int4* base = c.tw + PL::tw_offset(s) + k + 8 * c.h * p;
#pragma unroll
  for (int i = 1; i < 8; ++i) w[i] = __ldg(base + (i - 1) * p);
  w[0] = c.h ? __ldg(base - p) : w[1];
}

template <int R, int Bq, int... bs>
__device__ __forceinline__ void exact_small_dfts(long long (&re)[8], long long (&im)[8],
                                                 std::integer_sequence<int, bs...>) {
  (dft<EngFx, R, bs, Bq, 8>(re, im), ...);
}

// Pass s of the plan.  Radix-16 passes: the half's 8 inputs (already in re/im
// for s = 0) are twiddled, cut into digit words, multiplied on the tensor
// cores, recombined and stored to the exchange buffer (or, in the last pass,
// converted and stored to `o.dst`).  A radix 2/4/8 last pass runs on the CUDA
// cores: half h takes butterflies h Bq/2 .. (h+1) Bq/2 - 1 of its row.  The
// last pass loads the next tile's inputs into `raw` (at its start, or for a
// radix-16 last pass once its digits are stored) so that their latency
// overlaps the pass.
template <class PL, int G, int s>
__device__ __forceinline__ void exact_pass(ExactCtx& c, long long (&re)[8], long long (&im)[8], const ExactOut& o,
                                           double2 (&raw)[8], const int4 (&w)[8]) {
  using XP = ExactPlan<PL, G>;
  constexpr int T = PL::T, NS = PL::S;
  constexpr int R = PL::R[s];
  constexpr int p = PL::span(s);
  static_assert(R == 16 || s == NS - 1, "radix 2/4/8 only in the last pass");
  static_assert(R == 16 || s > 0, "radix-16 first pass");
  // input components of pass s: below 2^B (s = 0) or 2^59 (C of the
  // previous pass, modulus <= 2^58.5, kept by the twiddle products)
  constexpr int BS = s == 0 ? XP::B : kExactBound;
  static_assert(R <= 8 || R == 16, "radix 2/4/8 last pass: outputs below 2^61.5");
  if constexpr (R == 16) {
    if constexpr (s > 0) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const longlong2 v = c.data[XP::slot(c.j, c.t + T * (8 * c.h + i))];
        re[i] = v.x;
        im[i] = v.y;
      }
      if constexpr (EARLY_TW<PL, s>) {
#pragma unroll
        for (int i = 1; i < 8; ++i) EngFx::cmul(re[i], im[i], w[i]);
        if (c.h) EngFx::cmul(re[0], im[0], w[0]);
      } else {
        const int k = c.t & (p - 1);
        const int4* base = c.tw + PL::tw_offset(s) + k + (8 * c.h - 1) * p;  // input m = 8h + i: (m - 1) p
#pragma unroll
        for (int i = 1; i < 8; ++i) EngFx::cmul(re[i], im[i], __ldg(base + i * p));
        if (c.h) EngFx::cmul(re[0], im[0], __ldg(base));
      }
    }
    // A digits: values 8h..8h+7 (real) are chunks 2h, 2h+1 of each block,
    // values 16+8h..23+8h (imaginary) chunks 4+2h, 5+2h
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      unsigned w[kExactBlocks][4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = (ch & 1) * 4 + q;
        exact_digit_words<BS>(ch < 2 ? re[i] : im[i], w[0][q], w[1][q], w[2][q]);
      }
      const int chunk = (ch < 2 ? 2 * c.h : 4 + 2 * c.h) + (ch & 1);
      const int off = ((c.row >> 3) * XP::KC + chunk) * 128 + (c.row & 7) * 16;
#pragma unroll
      for (int b = 0; b < kExactBlocks; ++b)
        *reinterpret_cast<uint4*>(c.sA + b * XP::A_BLOCK + off) = make_uint4(w[b][0], w[b][1], w[b][2], w[b][3]);
    }
    if constexpr (s == NS - 1) exact_load_inputs<T>(raw, c.nsrc, c.nactive);
    exact_tmem_fill(c.tmem_rd);
    fence_proxy_async_smem();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // the group's MMAs read only its own rows: a barrier over the group
    if constexpr (G == 1) __syncthreads();
    else if (c.g == 0) asm volatile("bar.sync 1, 256;" ::: "memory");
    else asm volatile("bar.sync 2, 256;" ::: "memory");
    if (c.issuer) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned a0 = smem_u32(c.sA), b0 = smem_u32(c.sB);
#pragma unroll
      for (int q = 0; q < kExactBlocks; ++q) {
        const unsigned n = 32 * (kExactOrders - 2 * q);
        const unsigned idesc = (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24);  // FP16 x FP16 -> FP32
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          umma<kSplitBF16x3>(c.tmem + 64 * q, umma_desc(a0 + q * XP::A_BLOCK + kk * 256, 128, XP::KC * 128),
                             umma_desc(b0 + kk * 256, 128, XP::KC * 128), idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(c.bar))
                   : "memory");
    }
    if (!c.failed && !mbar_wait_bounded(c.bar, c.phase, kWaitLimitNs)) c.failed = true;
    c.phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // outputs C = (sum_k x_k F_k) 2^(54 - BS), modulus <= 2^58.5
    const int k = c.t & (p - 1);
    // rounds of WC columns (WC / 2 outputs) per order: 8 with one group, 4
    // with two (the register budget of 512 threads)
    constexpr int WC = G == 1 ? 8 : 4;
#pragma unroll
    for (int r = 0; r < 16 / WC; ++r) {
      unsigned v[kExactOrders][WC];
      if constexpr (WC == 8) exact_tmem_ld6x8(c.tmem_rd + WC * r, v);
      else exact_tmem_ld6x4(c.tmem_rd + WC * r, v);
#pragma unroll
      for (int q = 0; q < WC / 2; ++q) {
        const long long yr = exact_combine(v[0][2 * q], v[1][2 * q], v[2][2 * q], v[3][2 * q], v[4][2 * q],
                                           v[5][2 * q]);
        const long long yi = exact_combine(v[0][2 * q + 1], v[1][2 * q + 1], v[2][2 * q + 1], v[3][2 * q + 1],
                                           v[4][2 * q + 1], v[5][2 * q + 1]);
        const int m = 8 * c.h + (WC / 2) * r + q;
        const int e = (c.t - k) * 16 + k + m * p;
        if constexpr (s + 1 < NS) c.data[XP::slot(c.j, e)] = make_longlong2(yr, yi);
        else if (o.active) o.dst[e] = exact_out_value(o, yr, yi);
      }
    }
  } else {
    // last pass of radix 2/4/8 on the CUDA cores, fixed point
    exact_load_inputs<T>(raw, c.nsrc, c.nactive);
    constexpr int Bq = 16 / R, Bh = Bq / 2;
#pragma unroll
    for (int b = 0; b < Bh; ++b)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        const longlong2 v = c.data[XP::slot(c.j, c.t + T * (c.h * Bh + b + Bq * m))];
        re[b + Bh * m] = v.x;
        im[b + Bh * m] = v.y;
      }
#pragma unroll
    for (int b = 0; b < Bh; ++b) {
      const int tp = c.t + T * (c.h * Bh + b);
      const int4* base = c.tw + PL::tw_offset(s) + (tp & (p - 1));
#pragma unroll
      for (int m = 1; m < R; ++m) EngFx::cmul(re[b + Bh * m], im[b + Bh * m], __ldg(base + (m - 1) * p));
    }
    exact_small_dfts<R, Bh>(re, im, std::make_integer_sequence<int, Bh>{});
    if (o.active) {
#pragma unroll
      for (int b = 0; b < Bh; ++b)
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const int tp = c.t + T * (c.h * Bh + b);
          const int k = tp & (p - 1);
          o.dst[(tp - k) * R + k + m * p] = exact_out_value(o, re[b + Bh * m], im[b + Bh * m]);
        }
    }
  }
  if constexpr (s + 1 < NS) {
    int4 wn[8];
    if constexpr (EARLY_TW<PL, s + 1>) exact_load_twiddles<PL, s + 1>(c, wn);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    exact_pass<PL, G, s + 1>(c, re, im, o, raw, wn);
  }
}

// Largest sign-cleared high word of a thread's inputs: the exponent field
// of its largest value, or for subnormals the position of the leading bit.
__device__ __forceinline__ unsigned exact_high_max(const double2 (&raw)[8]) {
  unsigned a = 0u;
#pragma unroll
  for (int i = 0; i < 8; ++i) a = max(a, max(hi_word(raw[i].x) & 0x7FFFFFFFu, hi_word(raw[i].y) & 0x7FFFFFFFu));
  return a;
}

// Largest value of a over a transform's rows and both halves, in two steps
// around a barrier: shuffles within the warp and one word per (transform,
// half, warp) in `red`; after the barrier, the maximum of the transform's words.
template <int T, int TPB, int W>
__device__ __forceinline__ void exact_transform_put(unsigned a, int h, int j, int t, unsigned* red) {
  if constexpr (T >= 32) {
    a = __reduce_max_sync(0xffffffffu, a);
  } else if constexpr (T > 1) {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) a = max(a, __shfl_xor_sync(0xffffffffu, a, o, T));
  }
  if ((t & 31) == 0) red[(h * TPB + j) * W + (t >> 5)] = a;
}
template <int TPB, int W>
__device__ __forceinline__ unsigned exact_transform_get(int j, const unsigned* red) {
  unsigned a = red[j * W];
#pragma unroll
  for (int w = 1; w < 2 * W; ++w) a = max(a, red[((w / W) * TPB + j) * W + (w % W)]);
  return a;
}

template <class PL, int G>
__global__ void __launch_bounds__(256 * G, G == 1 ? 2 : 1)
fft_exact_kernel(const double2* __restrict__ in, double2* __restrict__ out, long long batch,
                 const int4* __restrict__ tw, const uint4* __restrict__ bmat, int* __restrict__ err) {
  using XP = ExactPlan<PL, G>;
  constexpr int N = PL::N, TPB = PL::TPB, T = PL::T;
  extern __shared__ __align__(1024) unsigned char smem_exact[];
  unsigned* red = reinterpret_cast<unsigned*>(smem_exact + XP::RED_OFF);
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem_exact + XP::BAR_OFF);
  unsigned* tslot = reinterpret_cast<unsigned*>(smem_exact + XP::BAR_OFF + 8 * G);

  const int tid = threadIdx.x;
  const int g = tid >> 8;            // 128-row group
  const int h = (tid >> 7) & 1;      // half of the row
  const int row = tid & 127;         // TMEM lane
  const int grow = g * 128 + row;    // row in the CTA
  ExactCtx c;
  c.sA = smem_exact + g * kExactBlocks * XP::A_BLOCK;
  c.sB = smem_exact + XP::A_BYTES;
  c.data = reinterpret_cast<longlong2*>(smem_exact + XP::DATA_OFF);
  c.bar = bars + g;
  c.tw = tw;
  c.tid = tid;
  c.g = g;
  c.h = h;
  c.row = row;
  c.j = grow / T;
  c.t = grow - c.j * T;
  c.issuer = (tid & 255) == 0;
  c.failed = false;
  const int warp = tid >> 5;

  for (int i = tid; i < XP::B_BYTES / 16; i += XP::THREADS) reinterpret_cast<uint4*>(c.sB)[i] = __ldg(bmat + i);
  if (tid == 0) {
    for (int gg = 0; gg < G; ++gg) mbar_init(bars + gg, 1);
    mbar_fence_init();
  }
  // the first tile's inputs and maximum (read after the set-up barrier)
  const long long ntiles = (batch + TPB - 1) / TPB;
  double2 raw[8];  // the current tile's inputs, loaded during the previous tile
  {
    const long long tr = (long long)blockIdx.x * TPB + c.j;
    exact_load_inputs<T>(raw, in + (tr < batch ? tr : 0) * N + c.t + T * 8 * h, tr < batch);
    exact_transform_put<T, TPB, XP::W>(exact_high_max(raw), h, c.j, c.t, red);
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
  const unsigned tbase = *tslot;
  c.tmem = tbase + 256 * g;
  // lanes 32 (warp % 4) .. +31, columns 16h.. of each order
  c.tmem_rd = c.tmem + ((unsigned)((warp & 3) * 32) << 16) + 16 * h;
  c.phase = 0;

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (tid == 0) prefetch_next_tile<N, TPB>(in, tile, batch);
    const long long tr = tile * TPB + c.j;
    const bool active = tr < batch;
    const long long ntr = tr + (long long)gridDim.x * TPB;
    c.nactive = ntr < batch;
    c.nsrc = in + (c.nactive ? ntr : 0) * N + c.t + T * 8 * h;
    // the transform's largest sign-cleared high word (put before the previous
    // barrier): its exponent field, or for a transform of subnormals (field
    // 0) the position of its leading bit
    const unsigned at = exact_transform_get<TPB, XP::W>(c.j, red);
    int em = (int)(at >> 20), kadj = 0;
    if (em == 0 && at != 0u) {
      // subnormal transform (largest value in [2^-1074 2^32, 2^-1022)): scale
      // by 2^64 (exact) so it keeps all its bits in the block fixed point;
      // its largest exponent field is then bitlen(at) + 44
#pragma unroll
      for (int i = 0; i < 8; ++i) raw[i] = make_double2(raw[i].x * 0x1p64, raw[i].y * 0x1p64);
      em = (32 - __clz(at)) + 44;
      kadj = -64;
    }
    int em_thread, emin;
    fx_exponent_range<8>(raw, em_thread, emin);
    const FxScale sc = fx_scale<XP::B>(em);
    long long re[8], im[8];
    fx_convert_in<8>(raw, re, im, sc.eref, emin);
    // the passes scale the transform by 2^-OUT_SHIFT: outputs are y 2^(K + OUT_SHIFT)
    const int e_out = (em < 1 ? 1 : em) + XP::OUT_SHIFT + kadj, k_out = sc.K + XP::OUT_SHIFT + kadj;
    const ExactOut o{out + tr * N, active, e_out < XP::B || e_out > 1983 + XP::B, sc.special,
                     (int)((unsigned)k_out << 20), k_out};
    const int4 w0[8] = {};
    exact_pass<PL, G, 0>(c, re, im, o, raw, w0);
    // the next tile's maximum, read after the barrier
    exact_transform_put<T, TPB, XP::W>(exact_high_max(raw), h, c.j, c.t, red);
    if (__syncthreads_or(c.failed)) {
      if (tid == 0) atomicOr(err, kErrTimeout);
      mbar_wait_bounded(c.bar, c.phase ^ 1, kWaitLimitNs);  // bounded drain of the MMAs in flight
      break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(XP::TMEM_COLS));
}

}  // namespace fftoc
