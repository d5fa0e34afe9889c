// fftoc — binary64 engine instantiations (every candidate plan per size).
#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_f64(SizeVariants* d) { describe_all<EngF64>(d); }
}  // namespace fftoc
