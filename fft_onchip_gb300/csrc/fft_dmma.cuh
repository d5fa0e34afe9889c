// fftoc — FFTOC_ENGINE_DMMA: 8-point transforms as a Karatsuba complex product
// on the FP64 tensor cores (mma.m8n8k4.f64), IEEE binary64 throughout.
//
// The reference's tensor path (includes/tensor_fft_8.cuh:37-65 with the
// Karatsuba macros of includes/tensor_utils.cuh:25-36) computes X = F8 x for
// 8 transforms per warp as three real products,
//   P1 = Fr xr,  P2 = Fi xi,  P3 = (Fr + Fi)(xr + xi),
//   Xr = P1 - P2,  Xi = P3 - P1 - P2,
// each 8x8x8 real product being two m8n8k4 steps (K = 4 + 4).  Here the DFT
// matrix is exact (F8[m][k] = W8^(mk) from correctly rounded cos/sin of
// multiples of pi/4; the reference's twiddles are FP32 sincospif), and each
// warp takes tiles of 8 transforms straight from HBM.
//
// Fragment layout of mma.m8n8k4.f64 (lane l): A (8x4, row) holds
// A[l >> 2][l & 3]; B (4x8, col) holds B[l & 3][l >> 2]; C/D (8x8) hold
// C[l >> 2][2 (l & 3) + {0, 1}].  With A = F (bin m x point k), B = x (point
// k x transform n) and C = X (bin m x transform n): lane l loads points
// k = l & 3 and 4 + (l & 3) of transform l >> 2 and stores bin l >> 2 of
// transforms 2 (l & 3) and 2 (l & 3) + 1.
#pragma once
#include <cuda_runtime.h>

namespace fftoc {

constexpr int kDmmaWarps = 8;  // warps per CTA; each takes tiles of 8 transforms

__device__ __forceinline__ void dmma_884(double& d0, double& d1, double a, double b, double c0, double c1) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%4, %5};"
               : "=d"(d0), "=d"(d1)
               : "d"(a), "d"(b), "d"(c0), "d"(c1));
}

// cos(2 pi j / 8) and -sin(2 pi j / 8), j = 0..7, correctly rounded
static __constant__ double kW8Re[8] = {1.0, 0.70710678118654752440, 0.0, -0.70710678118654752440,
                                       -1.0, -0.70710678118654752440, 0.0, 0.70710678118654752440};
static __constant__ double kW8Im[8] = {0.0, -0.70710678118654752440, -1.0, -0.70710678118654752440,
                                       0.0, 0.70710678118654752440, 1.0, 0.70710678118654752440};
__device__ __forceinline__ void w8(int j, double& c, double& s) {
  c = kW8Re[j & 7];
  s = kW8Im[j & 7];
}

__global__ void __launch_bounds__(32 * kDmmaWarps, 4) fft8_dmma_kernel(const double2* in, double2* out, long long batch) {
  const int lane = threadIdx.x & 31;
  const int m = lane >> 2, q = lane & 3;
  // A fragments: F8[m][k] for k = q (first step) and q + 4 (second)
  double fr0, fi0, fr1, fi1;
  w8(m * q, fr0, fi0);
  w8(m * (q + 4), fr1, fi1);
  const double fs0 = fr0 + fi0, fs1 = fr1 + fi1;
  const long long tiles = (batch + 7) / 8;
  const long long stride = (long long)gridDim.x * kDmmaWarps;
  for (long long tile = (long long)blockIdx.x * kDmmaWarps + (threadIdx.x >> 5); tile < tiles; tile += stride) {
    const long long base = tile * 8;
    const long long tn = base + m;  // transform whose points k = q, q + 4 this lane loads
    double2 x0 = make_double2(0.0, 0.0), x1 = make_double2(0.0, 0.0);
    if (tn < batch) {
      x0 = in[tn * 8 + q];
      x1 = in[tn * 8 + q + 4];
    }
    double p10, p11, p20, p21, p30, p31;
    dmma_884(p10, p11, fr0, x0.x, 0.0, 0.0);
    dmma_884(p10, p11, fr1, x1.x, p10, p11);
    dmma_884(p20, p21, fi0, x0.y, 0.0, 0.0);
    dmma_884(p20, p21, fi1, x1.y, p20, p21);
    dmma_884(p30, p31, fs0, x0.x + x0.y, 0.0, 0.0);
    dmma_884(p30, p31, fs1, x1.x + x1.y, p30, p31);
    const long long t0 = base + 2 * q;  // transforms of this lane's outputs: t0, t0 + 1; bin m
    if (t0 < batch) out[t0 * 8 + m] = make_double2(p10 - p20, (p30 - p10) - p20);
    if (t0 + 1 < batch) out[(t0 + 1) * 8 + m] = make_double2(p11 - p21, (p31 - p11) - p21);
  }
}

}  // namespace fftoc
