// fftoc — block fixed-point engine instantiations (every candidate plan per size).
#include "fft_kernel.cuh"
#include "fft_persistent.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_fx(SizeVariants* d) { describe_all<EngFx>(d); }
}  // namespace fftoc
