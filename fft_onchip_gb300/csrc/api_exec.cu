// fftoc — twiddle tables for the device-side executors of <fftoc/exec.cuh>.
//
// The executors are compiled into the caller's own kernels (the reference's
// harness instantiates testing::fft_tester<CT, FFTExec, ...> itself,
// includes/testing.cuh:16-57), so the library only supplies the tables: one
// per (device, engine, radices), built with the same long-double twiddles as
// the library's own plans and kept until the process exits.
#include <array>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fftoc.h"
#include "internal.h"

namespace fftoc {
namespace {

struct ExecTables {
  std::mutex mu;
  std::map<std::array<int, 6>, void*> table;  // (device, engine slot, radices) -> device table
};
ExecTables g_exec;

bool radix_ok(int r) { return r == 2 || r == 4 || r == 8 || r == 16; }

}  // namespace
}  // namespace fftoc

extern "C" fftoc_status fftoc_exec_twiddles(int n, int engine, const int radix[4], const void** table) {
  using namespace fftoc;
  if (!table || !radix) return set_error(FFTOC_ERR_INVALID_VALUE, "null argument");
  *table = nullptr;
  if (size_index(n) < 0) return set_error(FFTOC_ERR_INVALID_SIZE, "n=" + std::to_string(n) + " is not one of 8,16,...,4096");
  if (engine < FFTOC_ENGINE_AUTO || engine > kLastEngine) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown engine");
  const int eng = engine == FFTOC_ENGINE_AUTO ? FFTOC_ENGINE_FX : engine;
  if (eng != FFTOC_ENGINE_F64 && eng != FFTOC_ENGINE_FX)
    return set_error(FFTOC_ERR_UNSUPPORTED, "executors exist for the binary64 and fixed-point engines");

  KernelDesc d;
  long long prod = 1;
  bool tail = false;  // an unused pass (1) was seen: only 1s may follow
  for (int s = 0; s < 4; ++s) {
    const int r = radix[s];
    if (r == 1) {
      tail = true;
      continue;
    }
    if (!radix_ok(r) || tail) return set_error(FFTOC_ERR_INVALID_VALUE, "radices must be 2, 4, 8 or 16, unused passes 1 at the end");
    d.radix[s] = r;
    d.passes = s + 1;
    prod *= r;
  }
  if (d.passes == 0 || prod != n) return set_error(FFTOC_ERR_INVALID_VALUE, "radices must multiply to n");
  for (int s = 1, p = d.radix[0]; s < d.passes; p *= d.radix[s], ++s) d.tw_entries += (d.radix[s] - 1) * p;
  if (d.tw_entries == 0) return FFTOC_OK;  // one pass: no table

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(FFTOC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  const std::array<int, 6> key = {dev, eng, d.radix[0], d.radix[1], d.radix[2], d.radix[3]};
  std::lock_guard<std::mutex> lock(g_exec.mu);
  auto it = g_exec.table.find(key);
  if (it != g_exec.table.end()) {
    *table = it->second;
    return FFTOC_OK;
  }
  std::vector<double> f64;
  std::vector<int> fx;
  twiddle_tables(d, f64, fx);
  const size_t bytes = (size_t)d.tw_entries * 16;
  void* p = nullptr;
  if ((e = cudaMalloc(&p, bytes)) != cudaSuccess) {
    cudaGetLastError();
    return set_error(FFTOC_ERR_NO_MEMORY, std::string("cudaMalloc(twiddles): ") + cudaGetErrorString(e));
  }
  const void* src = eng == FFTOC_ENGINE_F64 ? (const void*)f64.data() : (const void*)fx.data();
  if ((e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p);
    return set_error(FFTOC_ERR_CUDA, std::string("cudaMemcpy(twiddles): ") + cudaGetErrorString(e));
  }
  g_exec.table[key] = p;
  *table = p;
  return FFTOC_OK;
}
