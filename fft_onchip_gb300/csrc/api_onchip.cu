// fftoc — on-chip repeat harness (the reference's timing mode): launch of the
// on-chip repeat kernels (fft_onchip.cuh) over a device buffer of blocks x TPB
// transforms, for the plan the library uses for (n, engine).
//
// The reference's run_fft_kernel (includes/testing.cuh:59-92) launches
// (sm_multiplier * SMs) / (UPB * FPU) blocks, each transforming its
// UPB * FPU transforms in shared memory `inner_repeats` times; run_perf_tests
// (:94-127) times 100 and 1100 repeats and reports the difference / 1000 as
// microseconds per pass.  fftoc_onchip_run is the launch; the timing loop is
// fft_onchip_gb300/onchip.py.
#include <mutex>
#include <string>

#include "../../include/fftoc.h"
#include "internal.h"

namespace fftoc {
namespace {

struct OnchipDevice {
  std::once_flag once;
  fftoc_status status = FFTOC_OK;
  std::string error;
  SizeVariants var[2][kNumSizes];
};
constexpr int kMaxDevices = 64;
OnchipDevice g_odev[kMaxDevices];

fftoc_status onchip_device(OnchipDevice** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(FFTOC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return set_error(FFTOC_ERR_INVALID_VALUE, "device ordinal out of range");
  OnchipDevice& o = g_odev[dev];
  std::call_once(o.once, [&] {
    SizeVariants tmp[2][kNumSizes];
    describe_onchip_f64(tmp[0]);
    describe_onchip_fx(tmp[1]);
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < kNumSizes; ++i) {
        o.var[s][i] = compiled_variants(s)[i];
        for (int v = 0; v < o.var[s][i].count; ++v) {
          KernelDesc& d = o.var[s][i].v[v];
          d.fn_onchip = tmp[s][i].v[v].fn_onchip;
          d.smem_onchip = tmp[s][i].v[v].smem_onchip;
          if (!d.fn_onchip) continue;
          e = cudaFuncSetAttribute(d.fn_onchip, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem_onchip);
          if (e != cudaSuccess) {
            cudaGetLastError();
            o.status = FFTOC_ERR_CUDA;
            o.error = std::string("on-chip kernel set-up: ") + cudaGetErrorString(e);
            return;
          }
        }
      }
  });
  if (o.status != FFTOC_OK) return set_error(o.status, o.error);
  *out = &o;
  return FFTOC_OK;
}

// the size's chosen plan if it has an on-chip kernel, else its first plan that has one
int onchip_variant(const OnchipDevice& o, int slot, int idx) {
  const int c = chosen_variant(slot, idx);
  if (c < o.var[slot][idx].count && o.var[slot][idx].v[c].fn_onchip) return c;
  for (int v = 0; v < o.var[slot][idx].count; ++v)
    if (o.var[slot][idx].v[v].fn_onchip) return v;
  return -1;
}

fftoc_status resolve(int n, int engine, OnchipDevice** o, int* slot, int* var) {
  const int idx = size_index(n);
  if (idx < 0) return set_error(FFTOC_ERR_INVALID_SIZE, "n=" + std::to_string(n) + " is not one of 8,16,...,4096");
  if (engine < FFTOC_ENGINE_AUTO || engine > kLastEngine) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown engine");
  const int eng = resolved_engine(n, engine);
  if (eng != FFTOC_ENGINE_F64 && eng != FFTOC_ENGINE_FX)
    return set_error(FFTOC_ERR_UNSUPPORTED, "the on-chip harness covers the binary64 and fixed-point engines");
  fftoc_status st = onchip_device(o);
  if (st != FFTOC_OK) return st;
  *slot = eng == FFTOC_ENGINE_FX ? 1 : 0;
  *var = onchip_variant(**o, *slot, idx);
  if (*var < 0) return set_error(FFTOC_ERR_UNSUPPORTED, "no on-chip kernel for this size");
  return FFTOC_OK;
}

}  // namespace
}  // namespace fftoc

extern "C" {

fftoc_status fftoc_onchip_plan(int n, int engine, int* transforms_per_block, int* variant) {
  fftoc::OnchipDevice* o = nullptr;
  int slot = 0, var = 0;
  fftoc_status st = fftoc::resolve(n, engine, &o, &slot, &var);
  if (st != FFTOC_OK) return st;
  if (transforms_per_block) *transforms_per_block = o->var[slot][fftoc::size_index(n)].v[var].tpb;
  if (variant) *variant = var;
  return FFTOC_OK;
}

fftoc_status fftoc_onchip_run(int n, int engine, double* data, int64_t blocks, int repeats, fftoc_stream stream) {
  fftoc::OnchipDevice* o = nullptr;
  int slot = 0, var = 0;
  fftoc_status st = fftoc::resolve(n, engine, &o, &slot, &var);
  if (st != FFTOC_OK) return st;
  if (blocks < 0 || blocks > 0x7FFFFFFFLL || repeats < 0)
    return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "blocks in [0, 2^31) and repeats >= 0");
  if (blocks == 0) return FFTOC_OK;
  if (!data) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "null buffer");
  if ((uintptr_t)data & 15) return fftoc::set_error(FFTOC_ERR_MISALIGNED, "buffer must be 16-byte aligned");
  const int idx = fftoc::size_index(n);
  const fftoc::KernelDesc& d = o->var[slot][idx].v[var];
  const void* tw = nullptr;
  int* err = nullptr;
  int sms = 0;
  if ((st = fftoc::device_plan_resources(slot, idx, var, &tw, &err, &sms)) != FFTOC_OK) return st;
  double2* p = reinterpret_cast<double2*>(data);
  int r = repeats;
  void* args[] = {(void*)&p, (void*)&r, (void*)&tw};
  cudaError_t e = cudaLaunchKernel(d.fn_onchip, dim3((unsigned)blocks), dim3(d.threads), args, (size_t)d.smem_onchip,
                                   (cudaStream_t)stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fftoc::set_error(FFTOC_ERR_CUDA, std::string("cudaLaunchKernel(on-chip): ") + cudaGetErrorString(e));
  }
  return FFTOC_OK;
}

}  // extern "C"
