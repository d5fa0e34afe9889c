// fftoc — IEEE binary64 engine instantiations (every candidate plan per size).
#define FFTOC_DESCRIBE_KERNELS
#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_f64(SizeVariants* d) { describe_all<EngF64, DescribeKernels>(d); }
}  // namespace fftoc
