// fftoc — on-chip repeat kernels of the block fixed-point engine (same plan list as
// kernels_fx.cu; TMA-prefetching plans have none).
#define FFTOC_DESCRIBE_ONCHIP
#include "fft_onchip.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_onchip_fx(SizeVariants* d) { describe_all<EngFx, DescribeOnchip>(d); }
}  // namespace fftoc
