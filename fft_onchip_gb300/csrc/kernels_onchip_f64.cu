// fftoc — on-chip repeat kernels of the IEEE binary64 engine (same plan list as
// kernels_f64.cu; TMA-prefetching plans have none).
#define FFTOC_DESCRIBE_ONCHIP
#include "fft_onchip.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_onchip_f64(SizeVariants* d) { describe_all<EngF64, DescribeOnchip>(d); }
}  // namespace fftoc
