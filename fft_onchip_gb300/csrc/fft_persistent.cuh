// fftoc — persistent, TMA-pipelined variant of the batched FFT kernel.
//
// One CTA per resident slot loops over tiles of TPB transforms.  An elected
// thread prefetches the next tile into the other shared-memory stage with a
// 1-D bulk copy (cp.async.bulk ... mbarrier::complete_tx), so the HBM reads of
// tile i+1 overlap the passes of tile i.  The passes run in the stage buffer
// itself (pass 0 reads the linear layout, later exchanges use the swizzled
// slots) and the last pass stores straight to HBM with coalesced 16-byte
// stores.  Every mbarrier wait is bounded (%globaltimer); on a timeout the
// CTA raises the library's device error flag, waits (bounded) for its own
// copies in flight and returns.
#pragma once
#include "fft_kernel.cuh"
#include "internal.h"

namespace fftoc {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for `phase` of `bar`, giving up after `limit_ns`.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned phase, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, phase)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned it = 1;; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((it & 255u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
}

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

template <class E, class PL, int NSTAGE>
struct Persist {
  using F = Fft<E, PL>;
  static constexpr int N = PL::N, TPB = PL::TPB, P = PL::P, T = PL::T, NS = PL::S;
  static constexpr int TILE_BYTES = TPB * N * 16;                           // bytes loaded per tile
  static constexpr int STAGE_BYTES = ((TPB * F::NP * 16 + 127) / 128) * 128;  // padded exchange layout
  static constexpr int THREADS = F::THREADS;
  // stages, then TPB ints of exponent scratch, then NSTAGE mbarriers
  static constexpr int RED_OFF = NSTAGE * STAGE_BYTES;
  static constexpr int BAR_OFF = RED_OFF + 64;
  static constexpr int SMEM = BAR_OFF + 8 * NSTAGE;
  static_assert(T >= 8, "pass-0 reads of the linear tile need >= 8 threads per transform");
};

template <class E, class PL, int NSTAGE>
__global__ void __launch_bounds__(Fft<E, PL>::THREADS, PL::MINB)
fft_fwd_persistent(const double2* __restrict__ in, double2* __restrict__ out, long long batch,
                   const typename E::TW* __restrict__ tw, int* __restrict__ err) {
  using F = Fft<E, PL>;
  using C = Persist<E, PL, NSTAGE>;
  using S = typename E::S;
  constexpr int N = PL::N, TPB = PL::TPB, P = PL::P, T = PL::T, NS = PL::S;
  extern __shared__ __align__(128) unsigned char smem_persist[];
  unsigned char* smem_raw = smem_persist;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem_raw + C::BAR_OFF);
  int* red = reinterpret_cast<int*>(smem_raw + C::RED_OFF);

  const int tid = threadIdx.x;
  const int j = tid / T;
  const int t = tid - j * T;
  const long long ntiles = (batch + TPB - 1) / TPB;

  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    mbar_fence_init();
  }
  __syncthreads();

  auto issue = [&](long long tile, int s) {
    const long long t0 = tile * TPB;
    const long long cnt = min((long long)TPB, batch - t0);
    const unsigned bytes = (unsigned)(cnt * N * 16);
    mbar_expect_tx(&bars[s], bytes);
    bulk_load(smem_raw + s * C::STAGE_BYTES, in + t0 * N, bytes, &bars[s]);
  };

  // prologue: the first NSTAGE-1 tiles of this CTA
  if (tid == 0) {
    for (int s = 0; s < NSTAGE - 1; ++s) {
      const long long tile = blockIdx.x + (long long)s * gridDim.x;
      if (tile < ntiles) issue(tile, s);
    }
  }

  int it = 0;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = it % NSTAGE;
    const unsigned phase = (unsigned)((it / NSTAGE) & 1);
    // refill the stage freed at the end of the previous iteration
    if (tid == 0) {
      const long long nxt = tile + (long long)(NSTAGE - 1) * gridDim.x;
      if (nxt < ntiles) issue(nxt, (it + NSTAGE - 1) % NSTAGE);
    }
    const bool got = mbar_wait_bounded(&bars[s], phase, kWaitLimitNs);
    if (!__syncthreads_and(got)) {
      if (tid == 0) {
        atomicOr(err, kErrTimeout);
        // bounded drain of this CTA's copies still in flight
        for (int k = 0; k < NSTAGE; ++k) {
          const long long pend = tile + (long long)k * gridDim.x;
          if (pend < ntiles) mbar_wait_bounded(&bars[(it + k) % NSTAGE], (unsigned)(((it + k) / NSTAGE) & 1), kWaitLimitNs);
        }
      }
      __syncthreads();
      return;
    }

    longlong2* sm = reinterpret_cast<longlong2*>(smem_raw + s * C::STAGE_BYTES);
    const long long tr = tile * TPB + j;
    const bool active = tr < batch;

    // pass-0 inputs from the linear tile: point i of this thread is element t + T*i
    S re[P], im[P];
    int K = 0, kshift = 0;
    bool slow = false, special = false;
    if constexpr (E::kId == EngF64::kId) {
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const longlong2 v = active ? sm[j * N + t + T * i] : make_longlong2(0, 0);
        re[i] = __longlong_as_double(v.x);
        im[i] = __longlong_as_double(v.y);
      }
    } else {
      double2 raw[P];
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const longlong2 v = active ? sm[j * N + t + T * i] : make_longlong2(0, 0);
        raw[i] = make_double2(__longlong_as_double(v.x), __longlong_as_double(v.y));
      }
      constexpr bool TR = FxTrunc<N>::value;
      int em, emin;
      fx_exponent_range<P, TR>(raw, em, emin);
      em = fx_transform_max<T, TPB>(em, tid, j, red);
      const FxScale sc = fx_scale<FxBits<N>::B>(em);
      special = sc.special;
      K = sc.K;
      kshift = sc.kshift;
      slow = sc.slow;
      fx_convert_in<P, false, TR>(raw, re, im, sc.eref, emin);
    }
    if constexpr (NS > 1) __syncthreads();  // every linear read is done before pass-0 writes
    F::template run_passes<0>(re, im, j, t, tw, sm);

    // fixed point: one branch per thread between the fast conversion and, for
    // the rare transforms whose outputs leave the normal range (or had
    // non-finite inputs), the slow one
    constexpr int RL = PL::R[NS - 1];
    constexpr int BL = P / RL;
    if (active) {
      double2* dst = out + tr * N;
      if (E::kId == EngF64::kId || !(slow || special)) {
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) {
            const int i = b + BL * m;
            double2 v;
            if constexpr (E::kId == EngF64::kId) {
              v = make_double2(re[i], im[i]);
            } else {
              v = make_double2(fx_out((long long)re[i], kshift), fx_out((long long)im[i], kshift));
            }
            dst[F::template dest<NS - 1>(t, b, m)] = v;
          }
      } else {
        const double qnan = __longlong_as_double(0x7FF8000000000000LL);
#pragma unroll
        for (int b = 0; b < BL; ++b)
#pragma unroll
          for (int m = 0; m < RL; ++m) {
            const int i = b + BL * m;
            dst[F::template dest<NS - 1>(t, b, m)] =
                special ? make_double2(qnan, qnan)
                        : make_double2(fx_out_slow((long long)re[i], K), fx_out_slow((long long)im[i], K));
          }
      }
    }
    // this thread's generic-proxy writes to stage s are ordered before the
    // bulk copy that refills it (async proxy) after the barrier
    fence_proxy_async_smem();
    __syncthreads();  // stage s is free for the next refill
  }
}

}  // namespace fftoc
