// fftoc — uneven-batch kernels of the IEEE binary64 engine (same plan list as
// kernels_f64.cu; TMA-prefetching plans have none).
#define FFTOC_DESCRIBE_UNEVEN
#include "fft_uneven.cuh"
#include "internal.h"
#include "plans.inc"

namespace fftoc {
void describe_uneven_f64(SizeVariants* d) { describe_all<EngF64, DescribeUneven>(d); }
}  // namespace fftoc
