// Reference executors of gprabowski/fft_onchip, compiled unmodified from the
// reference's own headers (include path = the reference checkout's includes/)
// into a cubin under oracle/_ref/.  TEST INFRASTRUCTURE ONLY: used to produce
// the reference's actual outputs for the golden fixtures and its on-chip
// timings; nothing in the product links or loads it.
//
// Each wrapper does what the reference harness's fft_tester does per block
// (includes/testing.cuh:16-57): stage UPB*FPU*N points of this block's slice
// from global to shared memory, construct the executor on the shared buffer,
// run it `repeats` times, and write the slice back.  Block shape is
// (Exec::threads, Exec::units_per_block) as in includes/testing.cuh:70.
// tensor_fft_16 (does not compile upstream) and reference_fft (needs
// cuFFTDx) are not built.
#include <config.hpp>
#include <common.cuh>
#include <tensor_fft_8.cuh>
#include <tensor_fft_64.cuh>
#include <tensor_fft_128.cuh>
#include <tensor_fft_256.cuh>
#include <tensor_fft_512.cuh>
#include <tensor_fft_4096.cuh>
#include <legacy8_fft.cuh>
#include <legacy16_fft.cuh>

using CT = config::CT;

template <class Exec, int N>
__device__ __forceinline__ void run_exec(CT* data, int repeats) {
  extern __shared__ __align__(16) unsigned char sh_raw[];
  CT* sh = reinterpret_cast<CT*>(sh_raw);
  constexpr int E = N * Exec::units_per_block * Exec::ffts_per_unit;
  CT* base = data + (size_t)E * blockIdx.x;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nt = blockDim.x * blockDim.y;
  for (int i = tid; i < E; i += nt) sh[i] = base[i];
  __syncthreads();
  Exec fft(sh);
#pragma unroll 1
  for (int r = 0; r < repeats; ++r) fft();
  __syncthreads();
  for (int i = tid; i < E; i += nt) base[i] = sh[i];
}

#define REF_KERNEL(NAME, EXEC, N)                                                        \
  extern "C" __global__ void __launch_bounds__(EXEC::max_threads_per_block)            \
      NAME(CT* data, int repeats) {                                                      \
    run_exec<EXEC, N>(data, repeats);                                                    \
  }

// Executor configurations: the header defaults with FPU = 1 (the FPU > 1
// variants of tensor_fft_64/128/256 index the wrong transforms), UPB = 1;
// tensor_fft_8 needs FPU a multiple of 8.
using T8 = fft::tensor_fft_8<CT, 8, 1, 8>;
using T64 = fft::tensor_fft_64<CT, 64, 1, 1>;
using T128 = fft::tensor_fft_128<CT, 128, 1, 1>;
using T256 = fft::tensor_fft_256<CT, 256, 1, 1>;
using T512 = fft::tensor_fft_512<CT, 512, 1, 1>;
using T4096 = fft::tensor_fft_4096<CT, 4096, 1, 1>;
using L8_8 = fft::legacy_fft<CT, 8>;
using L8_64 = fft::legacy_fft<CT, 64>;
using L8_512 = fft::legacy_fft<CT, 512>;
using L8_4096 = fft::legacy_fft<CT, 4096>;
using L16_16 = fft::legacy16_fft<CT, 16>;
using L16_256 = fft::legacy16_fft<CT, 256>;
using L16_4096 = fft::legacy16_fft<CT, 4096>;

REF_KERNEL(ref_tensor_fft_8, T8, 8)
REF_KERNEL(ref_tensor_fft_64, T64, 64)
REF_KERNEL(ref_tensor_fft_128, T128, 128)
REF_KERNEL(ref_tensor_fft_256, T256, 256)
REF_KERNEL(ref_tensor_fft_512, T512, 512)
REF_KERNEL(ref_tensor_fft_4096, T4096, 4096)
REF_KERNEL(ref_legacy8_fft_8, L8_8, 8)
REF_KERNEL(ref_legacy8_fft_64, L8_64, 64)
REF_KERNEL(ref_legacy8_fft_512, L8_512, 512)
REF_KERNEL(ref_legacy8_fft_4096, L8_4096, 4096)
REF_KERNEL(ref_legacy16_fft_16, L16_16, 16)
REF_KERNEL(ref_legacy16_fft_256, L16_256, 256)
REF_KERNEL(ref_legacy16_fft_4096, L16_4096, 4096)
