// fftoc — FFTOC_ENGINE_DMMA launches (fft_dmma.cuh): n = 8 only.  Larger
// sizes return FFTOC_ERR_UNSUPPORTED: there the Karatsuba scheme needs more
// FP64 tensor work per point than the binary64 engine's FMA butterflies
// (12 m8n8k4 steps per 64-point transform, the reference's tensor_fft_64),
// and the FP64 tensor rate of this part is no higher than its FMA rate.
#include <string>

#include "../../include/fftoc.h"
#include "fft_dmma.cuh"
#include "internal.h"

namespace fftoc {

bool dmma_supported(int n) { return n == 8; }

fftoc_status dmma_plan_info(int n, fftoc_plan_info* info) {
  if (!dmma_supported(n)) return set_error(FFTOC_ERR_UNSUPPORTED, "DMMA engine not available for n=" + std::to_string(n));
  *info = fftoc_plan_info{};
  info->n = n;
  info->engine = FFTOC_ENGINE_DMMA;
  info->threads_per_transform = 4;  // a transform's points sit on 4 lanes of its warp
  info->transforms_per_block = 8 * kDmmaWarps;
  info->threads_per_block = 32 * kDmmaWarps;
  info->smem_bytes = 0;
  info->passes = 1;
  info->radix[0] = 8;
  info->radix[1] = info->radix[2] = info->radix[3] = 1;
  info->points_per_thread = 2;
  info->variant = 0;
  info->variants = 1;
  info->uneven_variant = -1;
  return FFTOC_OK;
}

fftoc_status launch_dmma(int n, const double* in, double* out, int64_t batch, cudaStream_t stream) {
  if (!dmma_supported(n)) return set_error(FFTOC_ERR_UNSUPPORTED, "DMMA engine not available for n=" + std::to_string(n));
  const long long tiles = (batch + 7) / 8;
  long long blocks = (tiles + kDmmaWarps - 1) / kDmmaWarps;
  if (blocks > 0x7FFFFFFFLL) blocks = 0x7FFFFFFFLL;  // the kernel strides over the rest
  fft8_dmma_kernel<<<(unsigned)blocks, 32 * kDmmaWarps, 0, stream>>>(reinterpret_cast<const double2*>(in),
                                                                    reinterpret_cast<double2*>(out), (long long)batch);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FFTOC_ERR_CUDA, std::string("fft8_dmma_kernel: ") + cudaGetErrorString(e));
  return FFTOC_OK;
}

}  // namespace fftoc
