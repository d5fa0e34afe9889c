// fftoc — split-precision form instantiations: one plan per size (radix-16
// GEMM passes, a radix 2/4/8 last pass where N is not a power of 16), for
// the BF16x3 and TF32x2 operand splits (one group of 128 butterfly rows per
// CTA and four CTAs per SM from N = 32 to 2048, two groups and two CTAs per
// SM at N = 16 and 4096) and the exact-slice form
// (fft_exact.cuh: one group per CTA and two CTAs per SM up to N = 2048, whose
// accumulators then share TMEM; two groups and one CTA per SM at N = 4096).
#include "fft_exact.cuh"
#include "fft_split.cuh"
#include "internal.h"

namespace fftoc {
namespace {

template <int KIND, class PL, int G>
void add_split(SplitDesc& d) {
  using SP = SplitPlan<KIND, PL, G>;
  d.fn = (const void*)&fft_split_kernel<KIND, PL, G>;
  d.threads = SP::THREADS;
  d.tpb = PL::TPB;
  d.smem = SP::SMEM;
  d.passes = PL::S;
  for (int i = 0; i < 4; ++i) d.radix[i] = PL::R[i];
  d.tw_entries = PL::TW_COUNT;
  d.b_bytes = SP::B_BYTES;
  d.esize = SplitT<KIND>::ESIZE;
  d.slices = SplitT<KIND>::SLICES;
}

template <int KIND>
void describe(SplitDesc* d) {
  // index = size index (8 has no radix-16 pass: left empty)
  // one 128-thread group per CTA, four CTAs per SM, from N = 32 to 2048
  // (measured 1.06-1.16x the two-group CTA); two groups at N = 16 and 4096
  add_split<KIND, PlanT<16, 16, 256, 16, 1, 1, 1, 2>, 2>(d[1]);
  add_split<KIND, PlanT<32, 16, 64, 16, 2, 1, 1, 4>, 1>(d[2]);
  add_split<KIND, PlanT<64, 16, 32, 16, 4, 1, 1, 4>, 1>(d[3]);
  add_split<KIND, PlanT<128, 16, 16, 16, 8, 1, 1, 4>, 1>(d[4]);
  add_split<KIND, PlanT<256, 16, 8, 16, 16, 1, 1, 4>, 1>(d[5]);
  add_split<KIND, PlanT<512, 16, 4, 16, 16, 2, 1, 4>, 1>(d[6]);
  add_split<KIND, PlanT<1024, 16, 2, 16, 16, 4, 1, 4>, 1>(d[7]);
  add_split<KIND, PlanT<2048, 16, 1, 16, 16, 8, 1, 4>, 1>(d[8]);
  add_split<KIND, PlanT<4096, 16, 1, 16, 16, 16, 1, 2>, 2>(d[9]);
}

template <class PL, int G>
void add_exact(SplitDesc& d) {
  using XP = ExactPlan<PL, G>;
  d.fn = (const void*)&fft_exact_kernel<PL, G>;
  d.threads = XP::THREADS;
  d.tpb = PL::TPB;
  d.smem = XP::SMEM;
  d.passes = PL::S;
  for (int i = 0; i < 4; ++i) d.radix[i] = PL::R[i];
  d.tw_entries = PL::TW_COUNT;
  d.b_bytes = XP::B_BYTES;
  d.esize = 2;
  d.slices = kExactDigits;
}

void describe_exact(SplitDesc* d) {
  // one 128-thread group per CTA (two CTAs per SM) where a transform fits in
  // 128 threads: measured 1.1-1.33x the two-group CTA; N=4096 needs both groups
  add_exact<PlanT<16, 16, 128, 16>, 1>(d[1]);
  add_exact<PlanT<32, 16, 64, 16, 2>, 1>(d[2]);
  add_exact<PlanT<64, 16, 32, 16, 4>, 1>(d[3]);
  add_exact<PlanT<128, 16, 16, 16, 8>, 1>(d[4]);
  add_exact<PlanT<256, 16, 8, 16, 16>, 1>(d[5]);
  add_exact<PlanT<512, 16, 4, 16, 16, 2>, 1>(d[6]);
  add_exact<PlanT<1024, 16, 2, 16, 16, 4>, 1>(d[7]);
  add_exact<PlanT<2048, 16, 1, 16, 16, 8>, 1>(d[8]);
  add_exact<PlanT<4096, 16, 1, 16, 16, 16>, 2>(d[9]);
}

}  // namespace

void describe_split(int kind, SplitDesc* per_size) {
  if (kind == kSplitBF16x3) describe<kSplitBF16x3>(per_size);
  else if (kind == kSplitTF32x2) describe<kSplitTF32x2>(per_size);
  else describe_exact(per_size);
}

}  // namespace fftoc
