// fftoc — binary64 engine instantiations.
#include "fft_kernel.cuh"
#include "internal.h"

namespace fftoc {

template <class E, int N>
static void describe_one(KernelDesc& d) {
  constexpr int TPB = tpb_of(N);
  using F = Fft<E, N, TPB>;
  d.fn = (const void*)&fft_fwd_kernel<E, N, TPB>;
  d.threads = F::THREADS;
  d.tpb = TPB;
  d.smem = F::SMEM;
  d.tpt = F::T;
  d.passes = F::NS;
  for (int i = 0; i < 4; ++i) d.radix[i] = Plan<N>::R[i];
  d.tw_entries = tw_count<N>();
}

template <class E>
static void describe_all(KernelDesc* d) {
  describe_one<E, 8>(d[0]);
  describe_one<E, 16>(d[1]);
  describe_one<E, 32>(d[2]);
  describe_one<E, 64>(d[3]);
  describe_one<E, 128>(d[4]);
  describe_one<E, 256>(d[5]);
  describe_one<E, 512>(d[6]);
  describe_one<E, 1024>(d[7]);
  describe_one<E, 2048>(d[8]);
  describe_one<E, 4096>(d[9]);
}

void describe_f64(KernelDesc* d) { describe_all<EngF64>(d); }

}  // namespace fftoc
