// Test harness for the device-side executors of <fftoc/exec.cuh>, with the
// semantics of the reference harness testing::fft_tester
// (includes/testing.cuh:16-57): each CTA copies its tile of
// units_per_block * ffts_per_unit transforms into dynamic shared memory of
// exactly that size, constructs the executor on it, calls it `repeats` times
// and copies the tile back.  Block shape (threads, units_per_block).
// CT = thrust::complex<double>, the reference's element type (config.hpp:6).
#include <thrust/complex.h>

#include <cstdint>

#include <fftoc/exec.cuh>

namespace {

using CT = thrust::complex<double>;

template <class Exec, int Size>
__global__ void __launch_bounds__(Exec::max_threads_per_block) tester(CT* data, int repeats) {
  extern __shared__ __align__(16) unsigned char shared[];
  CT* tile = reinterpret_cast<CT*>(shared);
  constexpr int elems = Size * Exec::units_per_block * Exec::ffts_per_unit;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  CT* g = data + (long long)blockIdx.x * elems;
  for (int i = tid; i < elems; i += Exec::max_threads_per_block) tile[i] = g[i];
  __syncthreads();
  Exec fft(tile);
#pragma unroll 1
  for (int r = 0; r < repeats; ++r) fft();
  __syncthreads();
  for (int i = tid; i < elems; i += Exec::max_threads_per_block) g[i] = tile[i];
}

template <int Size, int Engine>
int shape(int* threads, int* upb, int* fpu, int* smem) {
  using Exec = fftoc::exec::fft<CT, Size, 0, Engine>;
  *threads = Exec::threads;
  *upb = Exec::units_per_block;
  *fpu = Exec::ffts_per_unit;
  *smem = (int)(Size * sizeof(CT) * Exec::units_per_block * Exec::ffts_per_unit);
  return 0;
}

template <int Size, int Engine>
int run(double* data, long long blocks, int repeats, cudaStream_t s) {
  using Exec = fftoc::exec::fft<CT, Size, 0, Engine>;
  const int smem = (int)(Size * sizeof(CT) * Exec::units_per_block * Exec::ffts_per_unit);
  auto k = tester<Exec, Size>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return -1;
  k<<<(unsigned)blocks, dim3(Exec::threads, Exec::units_per_block), smem, s>>>(reinterpret_cast<CT*>(data), repeats);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int Engine>
int dispatch_shape(int n, int* a, int* b, int* c, int* d) {
  switch (n) {
    case 8: return shape<8, Engine>(a, b, c, d);
    case 16: return shape<16, Engine>(a, b, c, d);
    case 32: return shape<32, Engine>(a, b, c, d);
    case 64: return shape<64, Engine>(a, b, c, d);
    case 128: return shape<128, Engine>(a, b, c, d);
    case 256: return shape<256, Engine>(a, b, c, d);
    case 512: return shape<512, Engine>(a, b, c, d);
    case 1024: return shape<1024, Engine>(a, b, c, d);
    case 2048: return shape<2048, Engine>(a, b, c, d);
    case 4096: return shape<4096, Engine>(a, b, c, d);
  }
  return -2;
}

template <int Engine>
int dispatch_run(int n, double* data, long long blocks, int repeats, cudaStream_t s) {
  switch (n) {
    case 8: return run<8, Engine>(data, blocks, repeats, s);
    case 16: return run<16, Engine>(data, blocks, repeats, s);
    case 32: return run<32, Engine>(data, blocks, repeats, s);
    case 64: return run<64, Engine>(data, blocks, repeats, s);
    case 128: return run<128, Engine>(data, blocks, repeats, s);
    case 256: return run<256, Engine>(data, blocks, repeats, s);
    case 512: return run<512, Engine>(data, blocks, repeats, s);
    case 1024: return run<1024, Engine>(data, blocks, repeats, s);
    case 2048: return run<2048, Engine>(data, blocks, repeats, s);
    case 4096: return run<4096, Engine>(data, blocks, repeats, s);
  }
  return -2;
}

}  // namespace

extern "C" {

// Executor shape for (n, engine): threads, units_per_block, ffts_per_unit and
// the tile's shared-memory bytes.  0 on success, -2 for a bad size or engine.
int exec_harness_shape(int n, int engine, int* threads, int* upb, int* fpu, int* smem) {
  if (engine == FFTOC_ENGINE_F64) return dispatch_shape<FFTOC_ENGINE_F64>(n, threads, upb, fpu, smem);
  if (engine == FFTOC_ENGINE_FX) return dispatch_shape<FFTOC_ENGINE_FX>(n, threads, upb, fpu, smem);
  return -2;
}

int exec_harness_bind(void) { return (int)fftoc::exec::bind(); }
int exec_harness_unbind(void) { return (int)fftoc::exec::unbind(); }

// `blocks` CTAs over data[blocks * units_per_block * ffts_per_unit * n]
// complex values (device memory), `repeats` executor calls each.
int exec_harness_run(int n, int engine, double* data, long long blocks, int repeats, void* stream) {
  if (blocks <= 0 || blocks > 0x7FFFFFFFLL || repeats < 0 || !data) return -3;
  const cudaStream_t s = (cudaStream_t)stream;
  if (engine == FFTOC_ENGINE_F64) return dispatch_run<FFTOC_ENGINE_F64>(n, data, blocks, repeats, s);
  if (engine == FFTOC_ENGINE_FX) return dispatch_run<FFTOC_ENGINE_FX>(n, data, blocks, repeats, s);
  return -2;
}

}  // extern "C"
