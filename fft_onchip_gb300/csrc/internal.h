// fftoc — declarations shared by the host translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fftoc.h"

namespace fftoc {

constexpr int kNumSizes = 10;
constexpr int kSizes[kNumSizes] = {8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096};

inline int size_index(int n) {
  for (int i = 0; i < kNumSizes; ++i)
    if (kSizes[i] == n) return i;
  return -1;
}

// One compiled kernel (an engine x plan instantiation).
struct KernelDesc {
  const void* fn = nullptr;  // __global__ function
  int threads = 0;           // threads per CTA
  int tpb = 0;               // transforms per CTA
  int smem = 0;              // dynamic shared memory bytes
  int tpt = 0;               // threads per transform
  int ppt = 0;               // points per thread
  int passes = 0;
  int radix[4] = {1, 1, 1, 1};
  int tw_entries = 0;        // twiddle table entries (16 bytes each)
  int persistent = 0;        // 1: grid-stride persistent CTAs with TMA prefetch (extra error-flag argument)
  int stages = 0;            // shared-memory stages of the persistent kernel
  int blocks_per_sm = 0;     // resident CTAs per SM (filled at device set-up)
  // uneven-batch kernel of the same plan (nullptr for TMA-prefetching plans)
  const void* fn_uneven = nullptr;
  int smem_uneven = 0;
  int blocks_per_sm_uneven = 0;
};

constexpr int kMaxVariants = 8;
struct SizeVariants {
  int count = 0;
  KernelDesc v[kMaxVariants];
};

// Fill `per_size[kNumSizes]` with the compiled plans of an engine
// (kernels_<engine>.cu); variant 0 is the default choice.
void describe_f64(SizeVariants* per_size);
void describe_fx(SizeVariants* per_size);
// Same walk over the plan list, filling only fn_uneven / smem_uneven
// (kernels_uneven_<engine>.cu).
void describe_uneven_f64(SizeVariants* per_size);
void describe_uneven_fx(SizeVariants* per_size);

// Device error-flag bits (the flag is returned by fftoc_device_error_check).
constexpr int kErrTimeout = 1;        // a bounded wait for a prefetched tile gave up
constexpr int kErrUnevenSkipped = 2;  // uneven-batch entries with a bad size or offset were skipped

// api.cu accessors: compiled plans per engine slot (0 F64, 1 FX), twiddle
// tables of a plan (16 bytes per entry: double2 / 4 x int32 limbs), the plan
// currently chosen for (slot, size index), AUTO resolution, and the
// per-thread error message.
const SizeVariants* compiled_variants(int eng_slot);
void twiddle_tables(const KernelDesc& d, std::vector<double>& f64, std::vector<int>& fx);
int chosen_variant(int eng_slot, int idx);
int resolved_engine(int n, int engine);
// The current device's twiddle table of plan (slot, size index, variant), its
// error flag and SM count (device set-up on first use).
fftoc_status device_plan_resources(int slot, int idx, int var, const void** tw, int** err, int* sms);
fftoc_status set_error(fftoc_status st, const std::string& msg);

}  // namespace fftoc
