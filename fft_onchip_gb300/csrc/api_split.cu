// fftoc — split-precision form: device set-up (FP32 twiddles, DFT-matrix
// operand slices, kernel attributes) and launch.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fftoc.h"
#include "internal.h"
#include "exact_operand.h"

namespace fftoc {
namespace {

constexpr int kKinds = 3;  // [0] BF16x3, [1] TF32x2, [2] exact slices
int kind_index(int kind) { return kind - 1; }

struct SplitDevice {
  std::once_flag once;
  fftoc_status status = FFTOC_OK;
  std::string error;
  SplitDesc d[kKinds][kNumSizes];
  void* tw[kKinds][kNumSizes] = {};
  void* bmat[kKinds] = {};
  int* err = nullptr;
  int sms = 0;
};
constexpr int kMaxDevices = 64;
SplitDevice g_sdev[kMaxDevices];

const SplitDesc* host_split(int k) {
  static SplitDesc table[kKinds][kNumSizes];
  static std::once_flag once;
  std::call_once(once, [] {
    describe_split(1, table[0]);
    describe_split(2, table[1]);
    describe_split(3, table[2]);
  });
  return table[k];
}

uint16_t bf16_rn(float f) {  // finite values
  uint32_t u;
  memcpy(&u, &f, 4);
  return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}
float bf16_f(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
uint32_t tf32_rna(float f) {  // round to 10 mantissa bits, ties away from zero
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u + 0x1000u) & 0xFFFFE000u;
}
float u32_f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// DFT-16 matrix, real-stacked as the GEMM's B operand (row c = output, column
// k = input; rows 0..15 real parts, 16..31 imaginary), each entry split into
// `slices` terms, laid out as core matrices of 8 rows x 16 bytes.
std::vector<unsigned char> dft16_operand(int esize, int slices) {
  const int row_bytes = 32 * esize, kc = row_bytes / 16, per_chunk = 16 / esize;
  std::vector<unsigned char> out((size_t)slices * 32 * row_bytes, 0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int c = 0; c < 32; ++c)
    for (int k = 0; k < 32; ++k) {
      const int cc = c & 15, kk = k & 15;
      const long double ang = -2.0L * pi * (long double)((cc * kk) % 16) / 16.0L;
      const double fr = (double)cosl(ang), fi = (double)sinl(ang);  // F = fr + i fi
      double v;
      if (c < 16) v = k < 16 ? fr : -fi;
      else v = k < 16 ? fi : fr;
      double rest = v;
      for (int q = 0; q < slices; ++q) {
        const size_t off = (size_t)q * 32 * row_bytes + (size_t)(((c >> 3) * kc + k / per_chunk) * 128 + (c & 7) * 16 +
                                                                 (k % per_chunk) * esize);
        if (esize == 2) {
          const uint16_t h = bf16_rn((float)rest);
          memcpy(&out[off], &h, 2);
          rest -= (double)bf16_f(h);
        } else {
          const uint32_t t = tf32_rna((float)rest);
          memcpy(&out[off], &t, 4);
          rest -= (double)u32_f(t);
        }
      }
    }
  return out;
}

void setup(SplitDevice& sd, int dev) {
  auto bad = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    sd.status = e == cudaErrorMemoryAllocation ? FFTOC_ERR_NO_MEMORY : FFTOC_ERR_CUDA;
    sd.error = std::string(what) + ": " + cudaGetErrorString(e);
  };
  cudaError_t e;
  if ((e = cudaDeviceGetAttribute(&sd.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return bad(e, "cudaDeviceGetAttribute");
  const void* tw0 = nullptr;
  int* err = nullptr;
  int sms = 0;
  // the library's device error flag (set-up of the batched path on first use)
  fftoc_status st = device_plan_resources(1, 0, 0, &tw0, &err, &sms);
  if (st != FFTOC_OK) {
    sd.status = st;
    sd.error = "device set-up failed";
    return;
  }
  sd.err = err;
  for (int k = 0; k < kKinds; ++k) {
    const SplitDesc* h = host_split(k);
    const std::vector<unsigned char> b = k == 2 ? dft16_exact_operand() : dft16_operand(k == 0 ? 2 : 4, k == 0 ? 3 : 2);
    if ((e = cudaMalloc(&sd.bmat[k], b.size())) != cudaSuccess) return bad(e, "cudaMalloc(split matrix)");
    if ((e = cudaMemcpy(sd.bmat[k], b.data(), b.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
      return bad(e, "cudaMemcpy(split matrix)");
    for (int i = 0; i < kNumSizes; ++i) {
      sd.d[k][i] = h[i];
      SplitDesc& d = sd.d[k][i];
      if (!d.fn) continue;
      if ((int)b.size() != d.b_bytes) {
        sd.status = FFTOC_ERR_INVALID_VALUE;
        sd.error = "split matrix size mismatch";
        return;
      }
      if ((e = cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem)) != cudaSuccess)
        return bad(e, "cudaFuncSetAttribute(split)");
      if ((e = fit_carveout(d.fn, d.threads, d.smem, &d.blocks_per_sm)) != cudaSuccess)
        return bad(e, "occupancy / carveout (split)");
      KernelDesc kd;
      kd.passes = d.passes;
      for (int r = 0; r < 4; ++r) kd.radix[r] = d.radix[r];
      kd.tw_entries = d.tw_entries;
      std::vector<double> f64;
      std::vector<int> fx;
      twiddle_tables(kd, f64, fx);
      const void* src;
      size_t bytes;
      std::vector<float> f32(f64.size() > 0 ? f64.size() : 2, 0.f);
      if (k == 2) {  // exact slices: the fixed-point engine's 60-bit limb twiddles
        if (fx.empty()) fx.assign(4, 0);
        src = fx.data();
        bytes = fx.size() * 4;
      } else {
        for (size_t q = 0; q < f64.size(); ++q) f32[q] = (float)f64[q];
        src = f32.data();
        bytes = f32.size() * 4;
      }
      if ((e = cudaMalloc(&sd.tw[k][i], bytes)) != cudaSuccess) return bad(e, "cudaMalloc(split twiddles)");
      if ((e = cudaMemcpy(sd.tw[k][i], src, bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bad(e, "cudaMemcpy(split twiddles)");
    }
  }
}

fftoc_status split_device(SplitDevice** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(FFTOC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return set_error(FFTOC_ERR_INVALID_VALUE, "device ordinal out of range");
  SplitDevice& sd = g_sdev[dev];
  std::call_once(sd.once, [&] { setup(sd, dev); });
  if (sd.status != FFTOC_OK) return set_error(sd.status, sd.error);
  *out = &sd;
  return FFTOC_OK;
}

}  // namespace

bool split_supported(int n, int kind) {
  const int idx = size_index(n);
  return idx >= 0 && kind >= FFTOC_SPLIT_BF16X3 && kind <= FFTOC_SPLIT_EXACT &&
         host_split(kind_index(kind))[idx].fn != nullptr;
}

fftoc_status split_plan_info(int n, int kind, fftoc_plan_info* info) {
  if (!split_supported(n, kind)) return set_error(FFTOC_ERR_UNSUPPORTED, "no split-precision plan for this size");
  const SplitDesc& d = host_split(kind_index(kind))[size_index(n)];
  memset(info, 0, sizeof(*info));
  info->n = n;
  info->engine = kind == FFTOC_SPLIT_BF16X3 ? FFTOC_ENGINE_SPLIT_BF16X3
                 : kind == FFTOC_SPLIT_TF32X2 ? FFTOC_ENGINE_SPLIT_TF32X2
                                              : FFTOC_ENGINE_SPLIT_EXACT;
  info->threads_per_transform = n / 16;
  info->transforms_per_block = d.tpb;
  info->threads_per_block = d.threads;
  info->smem_bytes = d.smem;
  info->passes = d.passes;
  for (int r = 0; r < 4; ++r) info->radix[r] = d.radix[r];
  info->points_per_thread = 16;
  info->variant = 0;
  info->variants = 1;
  info->persistent = 1;
  info->stages = 1;
  return FFTOC_OK;
}

fftoc_status launch_split(int n, const double* in, double* out, int64_t batch, int kind, cudaStream_t stream) {
  const int idx = size_index(n);
  if (idx < 0) return set_error(FFTOC_ERR_INVALID_SIZE, "n=" + std::to_string(n) + " is not one of 8,16,...,4096");
  if (kind < FFTOC_SPLIT_BF16X3 || kind > FFTOC_SPLIT_EXACT) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown split kind");
  if (batch < 0) return set_error(FFTOC_ERR_INVALID_VALUE, "batch must be >= 0");
  if (!split_supported(n, kind)) return set_error(FFTOC_ERR_UNSUPPORTED, "no split-precision plan for n=" + std::to_string(n));
  if (batch == 0) return FFTOC_OK;
  if (!in || !out) return set_error(FFTOC_ERR_INVALID_VALUE, "null buffer");
  if (((uintptr_t)in & 15) || ((uintptr_t)out & 15)) return set_error(FFTOC_ERR_MISALIGNED, "buffers must be 16-byte aligned");
  if (batch > INT64_MAX / ((int64_t)n * 16)) return set_error(FFTOC_ERR_INVALID_VALUE, "batch*n overflows");
  const uintptr_t bytes = (uintptr_t)batch * (uintptr_t)n * 16u;
  const uintptr_t a = (uintptr_t)in, b = (uintptr_t)out;
  if (a != b && a < b + bytes && b < a + bytes) return set_error(FFTOC_ERR_INVALID_VALUE, "in and out overlap partially");
  SplitDevice* sd = nullptr;
  fftoc_status st = split_device(&sd);
  if (st != FFTOC_OK) return st;
  const int k = kind_index(kind);
  const SplitDesc& d = sd->d[k][idx];
  const long long tiles = (batch + d.tpb - 1) / d.tpb;
  const long long cap = (long long)sd->sms * d.blocks_per_sm;
  const long long blocks = tiles < cap ? tiles : cap;
  const double2* in2 = reinterpret_cast<const double2*>(in);
  double2* out2 = reinterpret_cast<double2*>(out);
  long long bl = (long long)batch;
  const void* tw = sd->tw[k][idx];
  const void* bm = sd->bmat[k];
  int* err = sd->err;
  void* args[] = {(void*)&in2, (void*)&out2, (void*)&bl, (void*)&tw, (void*)&bm, (void*)&err};
  cudaError_t e = cudaLaunchKernel(d.fn, dim3((unsigned)blocks), dim3(d.threads), args, (size_t)d.smem, stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(FFTOC_ERR_CUDA, std::string("cudaLaunchKernel(split): ") + cudaGetErrorString(e));
  }
  return FFTOC_OK;
}

}  // namespace fftoc

extern "C" fftoc_status fftoc_c2c_fwd_split(int n, const double* in, double* out, int64_t batch, int kind,
                                            fftoc_stream stream) {
  return fftoc::launch_split(n, in, out, batch, kind, (cudaStream_t)stream);
}
