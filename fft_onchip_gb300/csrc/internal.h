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
  int prefetch = 0;          // 1: L2 prefetch one wave ahead (Prefetched<> plans)
  int code_flags = 0;        // FFTOC_CODE_* bits of the plan
  int uneven_default = 0;    // 1: the uneven path's default plan for this size (UnevenDefault<>)
  // uneven-batch kernel of the same plan (nullptr for TMA-prefetching plans)
  const void* fn_uneven = nullptr;
  int smem_uneven = 0;
  int blocks_per_sm_uneven = 0;
  // on-chip repeat kernel of the same plan (nullptr for TMA-prefetching plans)
  const void* fn_onchip = nullptr;
  int smem_onchip = 0;
};

constexpr int kMaxVariants = 12;
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
void describe_onchip_f64(SizeVariants* per_size);
void describe_onchip_fx(SizeVariants* per_size);

// Split-precision form: one compiled plan per size (fn == nullptr: none).
struct SplitDesc {
  const void* fn = nullptr;
  int threads = 0, tpb = 0, smem = 0, passes = 0;
  int radix[4] = {1, 1, 1, 1};
  int tw_entries = 0;  // FP32 twiddles (8 bytes each)
  int b_bytes = 0;     // DFT-matrix operand slices
  int esize = 0, slices = 0;
  int blocks_per_sm = 0;
};
// kernels_split.cu; kind 1 = BF16x3, 2 = TF32x2, 3 = exact slices
void describe_split(int kind, SplitDesc* per_size);
// api_split.cu; kind = fftoc_split_kind
bool split_supported(int n, int kind);
fftoc_status split_plan_info(int n, int kind, fftoc_plan_info* info);
fftoc_status launch_split(int n, const double* in, double* out, int64_t batch, int kind, cudaStream_t stream);
inline bool is_split_engine(int engine) {
  return engine == FFTOC_ENGINE_SPLIT_BF16X3 || engine == FFTOC_ENGINE_SPLIT_TF32X2 ||
         engine == FFTOC_ENGINE_SPLIT_EXACT;
}
inline int split_kind_of(int engine) {
  return engine == FFTOC_ENGINE_SPLIT_BF16X3   ? FFTOC_SPLIT_BF16X3
         : engine == FFTOC_ENGINE_SPLIT_TF32X2 ? FFTOC_SPLIT_TF32X2
                                               : FFTOC_SPLIT_EXACT;
}
constexpr int kLastEngine = FFTOC_ENGINE_SPLIT_EXACT;

// Resident CTAs per SM of a persistent kernel, and the shared-memory carveout
// that holds exactly that many (the rest of the SM's memory stays L1).  The
// occupancy query applies neither a function's carveout preference nor, for
// kernels that use tcgen05 (it returns 1 for them at any size), the actual
// limits, so the CTAs are computed here: the smallest of the register-file
// limit (registers per thread rounded to the 256-register warp allocation
// unit, 64K registers per SM), the thread limit (2048 per SM) and the
// shared-memory limit of the largest carveout.  The carveout is then set to
// the smallest percentage of the SM's shared memory that holds them.
inline cudaError_t fit_carveout(const void* fn, int threads, int smem, int* blocks_per_sm) {
  int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
  cudaFuncAttributes fa;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  const int warps = (threads + 31) / 32;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
  int by_regs = regs_warp > 0 ? regs_sm / (regs_warp * warps) : 32;
  const int by_threads = threads_sm / (warps * 32);
  if (by_threads < by_regs) by_regs = by_threads;
  const int by_smem = smem_sm / (smem + reserved);
  int b = by_regs < by_smem ? by_regs : by_smem;
  if (b < 1) b = 1;
  *blocks_per_sm = b;
  const long long need = (long long)b * (smem + reserved);
  int pct = (int)((100 * need + smem_sm - 1) / smem_sm);
  if (pct > 100) pct = 100;
  return cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

// Device error-flag bits (the flag is returned by fftoc_device_error_check).
constexpr int kErrTimeout = 1;        // a bounded wait for a prefetched tile gave up
constexpr int kErrUnevenSkipped = 2;  // uneven-batch entries with a bad size or offset were skipped

// api_dmma.cu: FFTOC_ENGINE_DMMA (n = 8)
bool dmma_supported(int n);
fftoc_status dmma_plan_info(int n, fftoc_plan_info* info);
fftoc_status launch_dmma(int n, const double* in, double* out, int64_t batch, cudaStream_t stream);

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
// api_noalloc.cu: read (into *flags) and clear the allocation-free entry
// point's device error flag of device `dev`; *flags = 0 if that path has not
// been set up there.  Allocates nothing.
fftoc_status noalloc_take_error(int dev, int* flags);
// Plan variant the uneven-batch path uses for (engine slot, size index), or -1.
int uneven_variant(int slot, int idx);

}  // namespace fftoc
