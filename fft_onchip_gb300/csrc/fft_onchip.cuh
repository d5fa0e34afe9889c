// fftoc — on-chip repeat kernel: the reference harness's timing mode
// (testing::fft_tester, includes/testing.cuh:16-57) for this library's plans.
//
// Each CTA copies its TPB transforms from global memory into shared memory
// once, transforms them in place `repeats` times (the whole per-transform
// computation of the plan, binary64 conversion included), and copies them
// back.  Timing two repeat counts and differencing
// (includes/testing.cuh:94-127) leaves the on-chip cost of one pass.
#pragma once
#include "fft_kernel.cuh"

namespace fftoc {

template <class E, class PL>
__global__ void __launch_bounds__(Fft<E, PL>::THREADS, PL::MINB)
fft_onchip_kernel(double2* __restrict__ data, int repeats, const typename E::TW* __restrict__ tw) {
  using F = Fft<E, PL>;
  constexpr int N = PL::N, TPB = PL::TPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* buf = reinterpret_cast<double2*>(smem_raw + F::SMEM);  // after the exchange area
  double2* g = data + (long long)blockIdx.x * TPB * N;
  for (int i = threadIdx.x; i < TPB * N; i += F::THREADS) buf[i] = g[i];
  __syncthreads();
  const SmemTile<N> tl{buf, 0, TPB};
#pragma unroll 1
  for (int r = 0; r < repeats; ++r) {
    fft_tile<E, PL>(tl, tw, smem_raw);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < TPB * N; i += F::THREADS) g[i] = buf[i];
}

}  // namespace fftoc
