// fftoc — uneven-batch kernels of the block fixed-point engine (same plan list as
// kernels_fx.cu; TMA-prefetching plans have none).
#define FFTOC_DESCRIBE_UNEVEN
#include "fft_uneven.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_uneven_fx(SizeVariants* d) { describe_all<EngFx, DescribeUneven>(d); }
}  // namespace fftoc
