// fftoc — self-test of the failure path of the bounded device waits.
//
// The persistent, split and exact kernels wait on mbarriers with a time limit
// (mbar_wait_bounded) and, when it expires, raise the device error flag and
// return instead of hanging.  This entry point exercises that path on purpose
// and safely: one CTA initialises an mbarrier that nothing ever arrives on,
// waits on it with a short limit, and raises the flag when the wait gives up.
// The host then reads FFTOC_ERR_TIMEOUT from fftoc_device_error_check().
#include <string>

#include "../../include/fftoc.h"
#include "fft_persistent.cuh"
#include "internal.h"

namespace fftoc {
namespace {

__global__ void selftest_wait_kernel(unsigned long long limit_ns, int* err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // expects one arrival, which never comes
    mbar_fence_init();
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
  if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicOr(err, kErrTimeout);
}

}  // namespace
}  // namespace fftoc

extern "C" fftoc_status fftoc_selftest_bounded_wait(double limit_ms, fftoc_stream stream) {
  if (!(limit_ms > 0.0) || limit_ms > 1000.0)
    return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "limit_ms must be in (0, 1000]");
  const void* tw = nullptr;
  int* err = nullptr;
  int sms = 0;
  fftoc_status st = fftoc::device_plan_resources(1, 0, 0, &tw, &err, &sms);  // the device's error flag
  if (st != FFTOC_OK) return st;
  fftoc::selftest_wait_kernel<<<1, 64, 0, (cudaStream_t)stream>>>((unsigned long long)(limit_ms * 1e6), err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fftoc::set_error(FFTOC_ERR_CUDA, std::string("selftest launch: ") + cudaGetErrorString(e));
  return FFTOC_OK;
}
