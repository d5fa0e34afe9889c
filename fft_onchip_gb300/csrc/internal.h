// fftoc — declarations shared by the host translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace fftoc {

constexpr int kNumSizes = 10;
constexpr int kSizes[kNumSizes] = {8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096};

inline int size_index(int n) {
  for (int i = 0; i < kNumSizes; ++i)
    if (kSizes[i] == n) return i;
  return -1;
}

// Transforms per CTA for the register/shared-memory kernels (about 256 threads
// per CTA, at most 64 KiB of shared memory).
constexpr int tpb_of(int n) {
  return n == 8 ? 256 : n == 16 ? 256 : n == 32 ? 64 : n == 64 ? 32 : n == 128 ? 32 : n == 256 ? 16
       : n == 512 ? 4 : n == 1024 ? 4 : n == 2048 ? 2 : 1;
}

// Per-size launch description filled by the engine translation units.
struct KernelDesc {
  const void* fn = nullptr;     // __global__ function
  int threads = 0;              // threads per CTA
  int tpb = 0;                  // transforms per CTA
  int smem = 0;                 // dynamic shared memory bytes
  int tpt = 0;                  // threads per transform
  int passes = 0;
  int radix[4] = {1, 1, 1, 1};
  int tw_entries = 0;           // twiddle table entries (16 bytes each)
};

// Fill `desc[kNumSizes]` for an engine (implemented in kernels_<engine>.cu).
void describe_f64(KernelDesc* desc);
void describe_fx(KernelDesc* desc);

// Twiddle tables (api.cu): entry (m-1)*p + k of pass s = W_{R p}^{k m}.
struct TwiddleSet {
  void* dev[kNumSizes] = {};  // device pointer per size
};

}  // namespace fftoc
