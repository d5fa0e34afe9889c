// fftoc — host-buffer transform that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: processes whose device
// memory is already claimed by another allocator (a framework's caching
// allocator or a pool sized to the whole GPU, where a new cudaMalloc fails or
// competes with it), services that account for every byte of device memory
// and must not grow after start-up, and latency-sensitive code for which
// cudaMalloc's implicit device-wide synchronisation is unacceptable.
// fftoc_c2c_fwd_host allocates 192 MiB of staging (and its device set-up
// allocates twiddle tables) on first use, so it is not usable there.
//
// This entry point stages the batch in a file-scope __device__ array of
// kNoAllocScratchBytes instead, keeps its twiddle tables and error flag in
// file-scope __device__ arrays too, and runs H2D copy, transform and D2H copy
// on the caller's stream.  The arrays are part of the loaded module: every GPU
// that loads the library holds them (~35 MiB) until the process exits.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fftoc.h"
#include "fft_core.cuh"
#include "internal.h"

namespace fftoc {

fftoc_status set_error(fftoc_status st, const std::string& msg);

namespace {

constexpr size_t kNoAllocScratchBytes = 32u << 20;  // largest batch*n*16 accepted
constexpr int kNoAllocTwiddleEntries = 192 * 1024;   // 16-byte entries, every compiled plan of both engines

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
__device__ __align__(256) int4 g_noalloc_twiddles[kNoAllocTwiddleEntries];
__device__ int g_noalloc_err;

// Per-device set-up, done by the first successful call on a device with that
// device current: addresses of the arrays (a host-side name of a __device__
// array is not a device address), twiddle upload, kernel attributes.  No
// allocation.  A set-up that fails is retried by the next call.
struct NoAllocDevice {
  std::mutex mu;
  std::atomic<bool> ready{false};
  fftoc_status status = FFTOC_OK;
  std::string error;
  unsigned char* scratch = nullptr;
  int4* twiddles = nullptr;
  int* err = nullptr;
  int sms = 0;
  SizeVariants var[2][kNumSizes];
  int tw_offset[2][kNumSizes][kMaxVariants] = {};  // entry offset of each plan's table
};

constexpr int kMaxDevices = 64;
NoAllocDevice g_dev[kMaxDevices];

void setup(NoAllocDevice& nd, int dev) {
  auto bad = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    nd.status = FFTOC_ERR_CUDA;
    nd.error = std::string(what) + ": " + cudaGetErrorString(e);
  };
  cudaError_t e;
  if ((e = cudaGetSymbolAddress((void**)&nd.scratch, g_noalloc_scratch)) != cudaSuccess)
    return bad(e, "cudaGetSymbolAddress(scratch)");
  if ((e = cudaGetSymbolAddress((void**)&nd.twiddles, g_noalloc_twiddles)) != cudaSuccess)
    return bad(e, "cudaGetSymbolAddress(twiddles)");
  if ((e = cudaGetSymbolAddress((void**)&nd.err, g_noalloc_err)) != cudaSuccess)
    return bad(e, "cudaGetSymbolAddress(error flag)");
  if ((e = cudaDeviceGetAttribute(&nd.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return bad(e, "cudaDeviceGetAttribute");
  std::vector<int4> host;
  host.reserve(kNoAllocTwiddleEntries);
  for (int slot = 0; slot < 2; ++slot)
    for (int i = 0; i < kNumSizes; ++i) {
      nd.var[slot][i] = compiled_variants(slot)[i];
      for (int v = 0; v < nd.var[slot][i].count; ++v) {
        KernelDesc& d = nd.var[slot][i].v[v];
        if ((e = cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem)) != cudaSuccess)
          return bad(e, "cudaFuncSetAttribute");
        if ((e = d.persistent ? fit_carveout(d.fn, d.threads, d.smem, &d.blocks_per_sm)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.blocks_per_sm, d.fn, d.threads,
                                                                              d.smem)) != cudaSuccess)
          return bad(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        if (d.blocks_per_sm < 1) d.blocks_per_sm = 1;
        std::vector<double> f64;
        std::vector<int> fx;
        twiddle_tables(d, f64, fx);
        nd.tw_offset[slot][i][v] = (int)host.size();
        for (int k = 0; k < d.tw_entries; ++k) {
          int4 w;
          if (slot == 0) {
            const double re = f64[2 * k], im = f64[2 * k + 1];
            memcpy(&w.x, &re, 8);
            memcpy(&w.z, &im, 8);
          } else {
            w = make_int4(fx[4 * k], fx[4 * k + 1], fx[4 * k + 2], fx[4 * k + 3]);
          }
          host.push_back(w);
        }
      }
    }
  if ((int)host.size() > kNoAllocTwiddleEntries) {
    nd.status = FFTOC_ERR_INVALID_VALUE;
    nd.error = "compiled plans need more twiddle entries than the static table holds";
    return;
  }
  if ((e = cudaMemcpy(nd.twiddles, host.data(), host.size() * sizeof(int4), cudaMemcpyHostToDevice)) != cudaSuccess)
    return bad(e, "cudaMemcpy(twiddles)");
  if ((e = cudaMemset(nd.err, 0, sizeof(int))) != cudaSuccess) return bad(e, "cudaMemset(error flag)");
}

}  // namespace

fftoc_status noalloc_take_error(int dev, int* flags) {
  *flags = 0;
  if (dev < 0 || dev >= kMaxDevices) return FFTOC_OK;
  NoAllocDevice& nd = g_dev[dev];
  if (!nd.ready.load(std::memory_order_acquire)) return FFTOC_OK;
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, nd.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_error(FFTOC_ERR_CUDA, std::string("cudaMemcpy(error flag): ") + cudaGetErrorString(e));
  if (h != 0 && (e = cudaMemset(nd.err, 0, sizeof(int))) != cudaSuccess)
    return set_error(FFTOC_ERR_CUDA, std::string("cudaMemset(error flag): ") + cudaGetErrorString(e));
  *flags = h;
  return FFTOC_OK;
}

fftoc_status launch_fwd_host_noalloc(int n, const double* h_in, double* h_out, int64_t batch, int engine,
                                     cudaStream_t stream) {
  const int idx = size_index(n);
  if (idx < 0) return set_error(FFTOC_ERR_INVALID_SIZE, "n=" + std::to_string(n) + " is not one of 8,16,...,4096");
  if (batch < 0) return set_error(FFTOC_ERR_INVALID_VALUE, "batch must be >= 0");
  if (engine < FFTOC_ENGINE_AUTO || engine > kLastEngine)
    return set_error(FFTOC_ERR_INVALID_VALUE, "unknown engine");
  if (batch == 0) return FFTOC_OK;
  if (!h_in || !h_out) return set_error(FFTOC_ERR_INVALID_VALUE, "null buffer");
  if (((uintptr_t)h_in & 15) || ((uintptr_t)h_out & 15))
    return set_error(FFTOC_ERR_MISALIGNED, "buffers must be 16-byte aligned");
  if (batch > (int64_t)(kNoAllocScratchBytes / ((size_t)n * 16)))
    return set_error(FFTOC_ERR_INVALID_VALUE,
                     "batch " + std::to_string(batch) + " x n " + std::to_string(n) + " x 16 bytes exceeds the " +
                         std::to_string(kNoAllocScratchBytes >> 20) + " MiB allocation-free scratch (max batch " +
                         std::to_string(kNoAllocScratchBytes / ((size_t)n * 16)) + " for this n)");
  const size_t bytes = (size_t)batch * (size_t)n * 16;
  const uintptr_t a = (uintptr_t)h_in, b = (uintptr_t)h_out;
  if (a != b && a < b + bytes && b < a + bytes)
    return set_error(FFTOC_ERR_INVALID_VALUE, "in and out overlap partially");
  const int eng = resolved_engine(n, engine);
  if (eng != FFTOC_ENGINE_F64 && eng != FFTOC_ENGINE_FX)
    return set_error(FFTOC_ERR_UNSUPPORTED, "engine not available for n=" + std::to_string(n));

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FFTOC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(FFTOC_ERR_INVALID_VALUE, "device ordinal out of range");
  NoAllocDevice& nd = g_dev[dev];
  if (!nd.ready.load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lock(nd.mu);
    if (!nd.ready.load(std::memory_order_relaxed)) {
      nd.status = FFTOC_OK;
      nd.error.clear();
      setup(nd, dev);
      if (nd.status != FFTOC_OK) return set_error(nd.status, nd.error);
      nd.ready.store(true, std::memory_order_release);
    }
  }

  const int slot = eng == FFTOC_ENGINE_FX ? 1 : 0;
  const int var = chosen_variant(slot, idx);
  const KernelDesc& d = nd.var[slot][idx].v[var];
  const void* tw = nd.twiddles + nd.tw_offset[slot][idx][var];
  const long long tiles = (batch + d.tpb - 1) / d.tpb;
  const long long cap = (long long)nd.sms * d.blocks_per_sm;
  const long long blocks = d.persistent ? (tiles < cap ? tiles : cap) : tiles;

  if ((e = cudaMemcpyAsync(nd.scratch, h_in, bytes, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return set_error(FFTOC_ERR_CUDA, std::string("cudaMemcpyAsync(H2D): ") + cudaGetErrorString(e));
  const double2* x = reinterpret_cast<const double2*>(nd.scratch);
  double2* y = reinterpret_cast<double2*>(nd.scratch);
  long long bl = (long long)batch;
  int* err = nd.err;
  void* args[] = {(void*)&x, (void*)&y, (void*)&bl, (void*)&tw, (void*)&err};
  if ((e = cudaLaunchKernel(d.fn, dim3((unsigned)blocks), dim3(d.threads), args, (size_t)d.smem, stream)) != cudaSuccess)
    return set_error(FFTOC_ERR_CUDA, std::string("cudaLaunchKernel: ") + cudaGetErrorString(e));
  if ((e = cudaMemcpyAsync(h_out, nd.scratch, bytes, cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
    return set_error(FFTOC_ERR_CUDA, std::string("cudaMemcpyAsync(D2H): ") + cudaGetErrorString(e));
  return FFTOC_OK;
}

}  // namespace fftoc

extern "C" fftoc_status fftoc_c2c_fwd_host_noalloc(int n, const double* h_in, double* h_out, int64_t batch, int engine,
                                                   fftoc_stream stream) {
  return fftoc::launch_fwd_host_noalloc(n, h_in, h_out, batch, engine, (cudaStream_t)stream);
}
