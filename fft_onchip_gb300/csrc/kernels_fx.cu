// fftoc — block fixed-point engine instantiations (every candidate plan per size).
#define FFTOC_DESCRIBE_KERNELS
#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_fx(SizeVariants* d) { describe_all<EngFx, DescribeKernels>(d); }
}  // namespace fftoc
