// The reference's harness kernel, testing::fft_tester (includes/testing.cuh:16-57
// of gprabowski/fft_onchip), compiled unmodified from the reference checkout
// and instantiated with this library's executors under the reference's
// executor names (include/fftoc/compat.cuh), into a device-only cubin under
// oracle/_ref/.  TEST INFRASTRUCTURE ONLY: tests/test_exec_reference_harness.py
// launches it through the driver API (oracle/harness_runner.py) with the
// geometry of the reference's host driver (includes/testing.cuh:59-92) and
// checks it against the library's batched kernels.  Nothing in the product
// links or loads it.
#include <testing.cuh>
#include <fftoc/compat.cuh>

namespace fft = fftoc::compat;
using CT = config::CT;

// fft_tester<CT, FFTExec, Size, FFTExec::units_per_block>, as run_fft_kernel
// instantiates it (includes/testing.cuh:76-84)
using X8 = fft::tensor_fft_8<CT, 8>;
using X16 = fft::tensor_fft_16<CT, 16>;
using X32 = fftoc::exec::fft<CT, 32>;
using X64 = fft::tensor_fft_64<CT, 64>;
using X128 = fft::tensor_fft_128<CT, 128>;
using X256 = fft::tensor_fft_256<CT, 256>;
using X512 = fft::tensor_fft_512<CT, 512>;
using X1024 = fftoc::exec::fft<CT, 1024>;
using X2048 = fftoc::exec::fft<CT, 2048>;
using X4096 = fft::tensor_fft_4096<CT, 4096>;
using L512 = fft::legacy_fft<CT, 512>;
using L256 = fft::legacy16_fft<CT, 256>;

template __global__ void testing::fft_tester<CT, X8, 8, X8::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X16, 16, X16::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X32, 32, X32::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X64, 64, X64::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X128, 128, X128::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X256, 256, X256::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X512, 512, X512::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X1024, 1024, X1024::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X2048, 2048, X2048::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, X4096, 4096, X4096::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, L512, 512, L512::units_per_block>(int, CT*, bool);
template __global__ void testing::fft_tester<CT, L256, 256, L256::units_per_block>(int, CT*, bool);

// What fftoc::exec::bind() does from host code of an executor's own
// translation unit: store the twiddle-table addresses (from
// fftoc_exec_twiddles) in this module's table, [engine][size slot].
extern "C" __global__ void fftoc_harness_bind(const void* const* tables) {
  const int i = threadIdx.x;
  if (i < 2 * fftoc::exec::kSizes) fftoc::exec::g_tables[i / fftoc::exec::kSizes][i % fftoc::exec::kSizes] = tables[i];
}

// Executor shape for the runner: threads, units_per_block, ffts_per_unit per
// instantiation above, in order.
struct Shape {
  int n, threads, upb, fpu;
};
extern "C" __global__ void fftoc_harness_shapes(Shape* out) {
  const Shape s[] = {{8, X8::threads, X8::units_per_block, X8::ffts_per_unit},
                     {16, X16::threads, X16::units_per_block, X16::ffts_per_unit},
                     {32, X32::threads, X32::units_per_block, X32::ffts_per_unit},
                     {64, X64::threads, X64::units_per_block, X64::ffts_per_unit},
                     {128, X128::threads, X128::units_per_block, X128::ffts_per_unit},
                     {256, X256::threads, X256::units_per_block, X256::ffts_per_unit},
                     {512, X512::threads, X512::units_per_block, X512::ffts_per_unit},
                     {1024, X1024::threads, X1024::units_per_block, X1024::ffts_per_unit},
                     {2048, X2048::threads, X2048::units_per_block, X2048::ffts_per_unit},
                     {4096, X4096::threads, X4096::units_per_block, X4096::ffts_per_unit},
                     {512, L512::threads, L512::units_per_block, L512::ffts_per_unit},
                     {256, L256::threads, L256::units_per_block, L256::ffts_per_unit}};
  if (threadIdx.x < 12) out[threadIdx.x] = s[threadIdx.x];
}
