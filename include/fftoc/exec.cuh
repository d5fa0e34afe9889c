// fftoc/exec.cuh — device-side executors in the shape of gprabowski/fft_onchip's
// FFTExec concept (includes/tensor_fft_64.cuh:12-45, includes/reference.cuh:9-24),
// so a harness with testing::fft_tester semantics (includes/testing.cuh:16-57)
// drives this library's transforms on-chip:
//
//   using Exec = fftoc::exec::fft<thrust::complex<double>, 64>;  // fixed-point engine
//   fftoc::exec::bind();                  // once per device, before the first launch
//   testing::run_perf_tests<config::CT, 64, Exec>(data);
//
// Contract (the concept's members):
//   threads                lanes of one unit (blockDim.x)
//   units_per_block        units per CTA (blockDim.y)
//   ffts_per_unit          transforms per unit
//   max_threads_per_block  threads * units_per_block (for __launch_bounds__)
//   print_type             name printed by the harness
//   fft(CT* smem)          construct on the CTA's tile: units_per_block *
//                          ffts_per_unit transforms of Size points, back to back,
//                          interleaved (re, im) doubles in shared memory
//   operator()()           forward, unscaled, natural-order DFT of every
//                          transform of the tile, in place; called by every
//                          thread of the CTA (it synchronises the CTA)
//
// The tile is the only shared memory the executor needs (plus a few static
// shared words for N >= 512): once each thread holds its points in registers
// the tile doubles as the exchange area between passes.  Arithmetic, plans
// and error bounds are the library's (relative L2 error ~1e-15 for the
// fixed-point engine).  Twiddle tables live in device memory owned by
// libfftoc (fftoc_exec_twiddles); bind() copies their addresses into this
// translation unit.  An executor whose table is not bound writes quiet NaNs
// instead of transforming (sizes with one pass need no table).
#pragma once
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "../fftoc.h"
#include "../../fft_onchip_gb300/csrc/fft_kernel.cuh"

namespace fftoc {
namespace exec {

// Per-size plan of the executors: points per thread and radices.  The
// twiddle table of a plan depends only on its radices.
template <int N, int TPB> struct plan_of;
template <int TPB> struct plan_of<8, TPB> { using type = PlanT<8, 8, TPB, 8>; };
template <int TPB> struct plan_of<16, TPB> { using type = PlanT<16, 8, TPB, 8, 2>; };
template <int TPB> struct plan_of<32, TPB> { using type = PlanT<32, 8, TPB, 8, 4>; };
template <int TPB> struct plan_of<64, TPB> { using type = PlanT<64, 8, TPB, 8, 8>; };
template <int TPB> struct plan_of<128, TPB> { using type = PlanT<128, 16, TPB, 16, 8>; };
template <int TPB> struct plan_of<256, TPB> { using type = PlanT<256, 16, TPB, 16, 16>; };
template <int TPB> struct plan_of<512, TPB> { using type = PlanT<512, 8, TPB, 8, 8, 8>; };
template <int TPB> struct plan_of<1024, TPB> { using type = PlanT<1024, 16, TPB, 16, 16, 4>; };
template <int TPB> struct plan_of<2048, TPB> { using type = PlanT<2048, 8, TPB, 8, 8, 8, 4>; };
template <int TPB> struct plan_of<4096, TPB> { using type = PlanT<4096, 16, TPB, 16, 16, 16>; };

constexpr int kSizes = 10;
// 8 -> 0, 16 -> 1, ..., 4096 -> 9
__host__ __device__ constexpr int size_slot(int n) { return n <= 8 ? 0 : 1 + size_slot(n / 2); }

// Twiddle tables of this translation unit, [0 binary64 | 1 fixed point][size slot];
// written by bind().
static __device__ const void* g_tables[2][kSizes];

template <int Engine> struct engine_of { using type = EngFx; };
template <> struct engine_of<FFTOC_ENGINE_F64> { using type = EngF64; };

template <class CT, int Size, int UPB = 0, int Engine = FFTOC_ENGINE_FX>
struct fft {
  static_assert(sizeof(CT) == 16, "CT must be an interleaved complex double (16 bytes)");
  static_assert(Engine == FFTOC_ENGINE_FX || Engine == FFTOC_ENGINE_F64,
                "executors exist for the fixed-point and binary64 engines");
  using E = typename engine_of<Engine>::type;
  using S = typename E::S;
  using TW = typename E::TW;

  static constexpr int P = plan_of<Size, 1>::type::P;  // points per thread
  static constexpr int T = Size / P;                   // threads per transform
  static constexpr int threads = T < 32 ? 32 : T;
  static constexpr int ffts_per_unit = T < 32 ? 32 / T : 1;
  static constexpr int units_per_block = UPB > 0 ? UPB : (256 / threads > 0 ? 256 / threads : 1);
  static constexpr int max_threads_per_block = threads * units_per_block;
  static constexpr int transforms_per_block = units_per_block * ffts_per_unit;
  static constexpr const char* print_type = Engine == FFTOC_ENGINE_F64 ? "fftoc_f64" : "fftoc_fx";

  using PL = typename plan_of<Size, transforms_per_block>::type;
  using F = Fft<E, PL>;
  static constexpr int NS = PL::S;
  static constexpr int kSlot = size_slot(Size);
  static_assert(T * transforms_per_block == max_threads_per_block, "every thread owns P points of one transform");

  CT* sh_d;
  __device__ explicit fft(CT* d) : sh_d(d) {}

  __device__ void operator()() {
    longlong2* sm = reinterpret_cast<longlong2*>(sh_d);
    const int tid = threadIdx.y * threads + threadIdx.x;
    const int j = tid / T;
    const int t = tid - j * T;
    const TW* tw = static_cast<const TW*>(g_tables[E::kId == EngF64::kId ? 0 : 1][kSlot]);

    // point i of this thread is element t + T*i of transform j
    double2 raw[P];
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const longlong2 v = sm[j * Size + t + T * i];
      raw[i] = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
    }

    S re[P], im[P];
    int K = 0, kshift = 0;
    bool slow = false, special = false;
    if constexpr (E::kId == EngF64::kId) {
#pragma unroll
      for (int i = 0; i < P; ++i) { re[i] = raw[i].x; im[i] = raw[i].y; }
    } else {
      // largest biased exponent of the transform, smallest of this thread
      __shared__ int red[transforms_per_block * (T > 32 ? T / 32 : 1)];
      constexpr bool TR = FxTrunc<Size>::value;
      int em, emin;
      fx_exponent_range<P, TR>(raw, em, emin);
      em = fx_transform_max<T, transforms_per_block>(em, tid, j, red);
      const FxScale sc = fx_scale<FxBits<Size>::B>(em);
      special = sc.special;
      K = sc.K;
      kshift = sc.kshift;
      slow = sc.slow;
      fx_convert_in<P, false, TR>(raw, re, im, sc.eref, emin);
    }
    __syncthreads();  // the whole tile is in registers: it is the exchange area from here on

    constexpr int RL = PL::R[NS - 1];
    constexpr int BL = P / RL;
    if (PL::TW_COUNT > 0 && tw == nullptr) {  // not bound: visible failure, no access
      const long long qnan = 0x7FF8000000000000LL;
#pragma unroll
      for (int i = 0; i < P; ++i) sm[j * Size + t + T * i] = make_longlong2(qnan, qnan);
      __syncthreads();
      return;
    }
    run<0>(re, im, j, t, tw, sm);
    if constexpr (NS > 1) __syncthreads();  // every thread has read its last exchange

    if constexpr (E::kId == EngF64::kId) {
#pragma unroll
      for (int b = 0; b < BL; ++b)
#pragma unroll
        for (int m = 0; m < RL; ++m)
          sm[j * Size + F::template dest<NS - 1>(t, b, m)] =
              make_longlong2(__double_as_longlong(re[b + BL * m]), __double_as_longlong(im[b + BL * m]));
    } else if (slow || special) {  // outputs outside the normal range, or non-finite inputs
      const double qnan = __longlong_as_double(0x7FF8000000000000LL);
#pragma unroll
      for (int b = 0; b < BL; ++b)
#pragma unroll
        for (int m = 0; m < RL; ++m) {
          const int i = b + BL * m;
          const double r = special ? qnan : fx_out_slow((long long)re[i], K);
          const double q = special ? qnan : fx_out_slow((long long)im[i], K);
          sm[j * Size + F::template dest<NS - 1>(t, b, m)] = make_longlong2(__double_as_longlong(r), __double_as_longlong(q));
        }
    } else {
#pragma unroll
      for (int b = 0; b < BL; ++b)
#pragma unroll
        for (int m = 0; m < RL; ++m) {
          const int i = b + BL * m;
          sm[j * Size + F::template dest<NS - 1>(t, b, m)] =
              make_longlong2(__double_as_longlong(fx_out((long long)re[i], kshift)),
                             __double_as_longlong(fx_out((long long)im[i], kshift)));
        }
    }
    __syncthreads();  // the next call (or the harness) reads the tile
  }

 private:
  // pass s, then the in-place exchange to pass s+1 (unpadded: transform j at
  // elements [j*Size, (j+1)*Size) of the tile)
  template <int s>
  __device__ __forceinline__ static void run(S (&re)[P], S (&im)[P], int j, int t, const TW* __restrict__ tw,
                                             longlong2* sm) {
    constexpr int R = PL::R[s];
    constexpr int B = P / R;
    F::template pass<s>(re, im, t, tw, std::make_integer_sequence<int, P / R>{});
    if constexpr (s + 1 < NS) {
      if constexpr (s > 0) __syncthreads();  // previous readers of the tile are done
#pragma unroll
      for (int b = 0; b < B; ++b)
#pragma unroll
        for (int m = 0; m < R; ++m)
          sm[j * Size + F::template dest<s>(t, b, m)] =
              make_longlong2(F::to_bits(re[b + B * m]), F::to_bits(im[b + B * m]));
      __syncthreads();
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const longlong2 v = sm[j * Size + t + T * i];
        re[i] = F::from_bits(v.x);
        im[i] = F::from_bits(v.y);
      }
      run<s + 1>(re, im, j, t, tw, sm);
    }
  }
};

namespace detail {
template <int N>
inline fftoc_status bind_size(const void* (&h)[2][kSizes]) {
  using PL = typename plan_of<N, 1>::type;
  const int radix[4] = {PL::R[0], PL::R[1], PL::R[2], PL::R[3]};
  fftoc_status st = fftoc_exec_twiddles(N, FFTOC_ENGINE_F64, radix, &h[0][size_slot(N)]);
  if (st == FFTOC_OK) st = fftoc_exec_twiddles(N, FFTOC_ENGINE_FX, radix, &h[1][size_slot(N)]);
  return st;
}
template <int... Ns>
inline fftoc_status bind_sizes(const void* (&h)[2][kSizes], std::integer_sequence<int, Ns...>) {
  fftoc_status st = FFTOC_OK;
  ((st = st == FFTOC_OK ? bind_size<Ns>(h) : st), ...);
  return st;
}
}  // namespace detail

// Bind the executors of this translation unit to the library's twiddle tables
// on the current device.  Call once per device before the first launch.
inline fftoc_status bind() {
  const void* h[2][kSizes] = {};
  fftoc_status st =
      detail::bind_sizes(h, std::integer_sequence<int, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096>{});
  if (st != FFTOC_OK) return st;
  return cudaMemcpyToSymbol(g_tables, h, sizeof(h)) == cudaSuccess ? FFTOC_OK : FFTOC_ERR_CUDA;
}

// Clear this translation unit's bindings (executors then write quiet NaNs).
inline fftoc_status unbind() {
  const void* h[2][kSizes] = {};
  return cudaMemcpyToSymbol(g_tables, h, sizeof(h)) == cudaSuccess ? FFTOC_OK : FFTOC_ERR_CUDA;
}

}  // namespace exec
}  // namespace fftoc
