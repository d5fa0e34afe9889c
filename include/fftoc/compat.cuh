// fftoc/compat.cuh — this library's device executors under the executor names
// and template parameter lists of gprabowski/fft_onchip
// (includes/tensor_fft_{8,16,64,128,256,512,4096}.cuh, includes/legacy8_fft.cuh:11,
// includes/legacy16_fft.cuh:17), so code written against those headers — the
// instantiations scripts/generate_bench.py emits, or testing::fft_tester —
// switches over with one line and no edit to its type names:
//
//   #include <fftoc/compat.cuh>
//   namespace fft = fftoc::compat;   // instead of the reference's executor headers
//   ...
//   fftoc::exec::bind();             // once per device, before the first launch
//
// tensor_fft_N<CT, Size, UPB, FPU>: UPB units per CTA (blockDim.y), as in the
// reference, with the reference's defaults.  FPU is accepted for source
// compatibility; the transforms per unit follow this library's plan for Size
// and are reported by ffts_per_unit, which the harness reads for its grid and
// tile (includes/testing.cuh:68-74).  legacy_fft<CT, Size> and
// legacy16_fft<CT, Size>: one unit per CTA, as there.  Every alias computes
// the forward, unscaled, natural-order DFT in place with the fixed-point
// engine (relative L2 error ~1e-15), whatever the reference executor's
// arithmetic was.
#pragma once
#include "exec.cuh"

namespace fftoc {
namespace compat {

template <class CT, int Size, int UPB = 1, int FPU = 32> using tensor_fft_8 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 2, int FPU = 2> using tensor_fft_16 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 2, int FPU = 1> using tensor_fft_64 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 2, int FPU = 1> using tensor_fft_128 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 2, int FPU = 1> using tensor_fft_256 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 2, int FPU = 1> using tensor_fft_512 = exec::fft<CT, Size, UPB>;
template <class CT, int Size, int UPB = 1, int FPU = 1> using tensor_fft_4096 = exec::fft<CT, Size, UPB>;
template <class CT, int Size> using legacy_fft = exec::fft<CT, Size, 1>;
template <class CT, int Size> using legacy16_fft = exec::fft<CT, Size, 1>;

}  // namespace compat
}  // namespace fftoc
