// fftoc — uneven batches: transforms of mixed sizes packed in one buffer and
// described by an int64 offset table, run as one CUDA graph.
//
// The reference runs one size per launch (its harness stages UPB*FPU
// transforms of a single executor per block, includes/testing.cuh:16-57, and
// its benchmark driver loops over sizes, scripts/generate_bench.py:93-113).
// Here one graph takes the whole mixed batch:
//   1. uneven_hist     per 1024-entry chunk of the table, a histogram by size;
//   2. uneven_scan     bucket starts and per-chunk bases (one CTA);
//   3. uneven_scatter  stable bucketing: transform offsets grouped by size, in
//                      table order within a size;
//   4. fft_uneven_kernel<E, PL>, one per size on parallel graph branches,
//      each CTA loading its transforms from their own offsets.
// Steps 1-3 read the transform count from device memory.  The size kernels
// are device-updatable graph nodes whose grids uneven_scan sets from the
// bucket counts: one CTA per tile (like the batched kernels) for a size that
// holds at least 40 % of the batch's bytes, else persistent grids of the
// size's resident CTAs, the sizes side by side on parallel branches.  Where
// the runtime refuses device-updatable nodes, the graph keeps persistent
// grids (the SM count times the resident CTAs) and the CTAs walk their
// bucket tile by tile.
#pragma once
#include "fft_kernel.cuh"
#include "internal.h"

namespace fftoc {

constexpr int kUnevenChunk = 1024;              // table entries per bucketing CTA
constexpr int kUnevenBins = 16;                 // 10 sizes + 1 "invalid" bin, padded
constexpr int kUnevenInvalid = 10;

// Argument block of one uneven execution (device memory; written by
// uneven_set_args before each graph launch).
struct UnevenArgs {
  const double2* in;
  double2* out;
  const long long* offsets;   // complex-element offset of each transform (in and out)
  const int* ns;              // size of each transform
  long long count;            // transforms in the table
  long long* list;            // bucketed transform offsets [max_count]
  int* chunk_base;            // [chunks][kUnevenBins]
  int bucket_count[kUnevenBins];
  int bucket_start[kUnevenBins];
  // per size, set when the graph is captured: the size kernel's node (null
  // where the graph has persistent grids), its transforms per CTA, and its
  // resident CTAs on the device (the L2 prefetch distance)
  cudaGraphDeviceNode_t nodes[kUnevenBins];
  int tpb[kUnevenBins];
  int wave[kUnevenBins];
};

static __global__ void uneven_set_args(UnevenArgs* a, const double2* in, double2* out, const long long* offsets,
                                const int* ns, long long count) {
  a->in = in;
  a->out = out;
  a->offsets = offsets;
  a->ns = ns;
  a->count = count;
}

__device__ __forceinline__ int uneven_bin(int n) {
  // 8..4096 powers of two -> 0..9; anything else -> kUnevenInvalid
  if (n < 8 || n > 4096 || (n & (n - 1))) return kUnevenInvalid;
  return __ffs(n) - 4;
}

// bin of table entry i (valid size and non-negative offset), or -1 past the end
__device__ __forceinline__ int uneven_entry_bin(const UnevenArgs& a, long long i) {
  if (i >= a.count) return -1;
  const int b = uneven_bin(__ldg(a.ns + i));
  if (b == kUnevenInvalid) return b;
  return __ldg(a.offsets + i) < 0 ? kUnevenInvalid : b;
}

static __global__ void __launch_bounds__(kUnevenChunk) uneven_hist(UnevenArgs* __restrict__ a, int* __restrict__ err) {
  __shared__ int h[kUnevenBins];
  if (threadIdx.x < kUnevenBins) h[threadIdx.x] = 0;
  __syncthreads();
  const long long chunk0 = (long long)blockIdx.x * kUnevenChunk;
  if (chunk0 >= a->count) return;  // uniform per CTA
  const int b = uneven_entry_bin(*a, chunk0 + threadIdx.x);
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  if (b >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&h[b], __popc(peers));
  __syncthreads();
  if (threadIdx.x < kUnevenBins) a->chunk_base[blockIdx.x * kUnevenBins + threadIdx.x] = h[threadIdx.x];
  if (threadIdx.x == kUnevenInvalid && h[kUnevenInvalid] > 0) atomicOr(err, kErrUnevenSkipped);
}

// Grid of size bin b's kernel from the bucket counts (transforms per size,
// sizes 8 << i): one CTA per tile when the size holds at least 40 % of the
// batch's bytes (or its tiles fit in one wave of resident CTAs), else a
// persistent grid of `wave` CTAs.  At least 1.  At most two sizes pass the
// share test.
FFTOC_HD long long uneven_grid(const int* counts, int b, int tpb, int wave) {
  double bytes = 0.0;
  for (int i = 0; i < kUnevenInvalid; ++i) bytes += (double)counts[i] * (double)(8 << i);
  const double share = bytes > 0.0 ? (double)counts[b] * (double)(8 << b) / bytes : 1.0;
  const long long tiles = ((long long)counts[b] + tpb - 1) / tpb;
  const long long grid = share >= 0.4 || tiles < wave ? tiles : wave;
  return grid > 0 ? grid : 1;
}

// One CTA of 32 x kUnevenBins threads: warp b scans bin b over the chunks.
// With `size_nodes` (launched from the graph), the size kernels' grids are
// set from the bucket counts.
static __global__ void __launch_bounds__(32 * kUnevenBins) uneven_scan(UnevenArgs* __restrict__ a, int size_nodes) {
  __shared__ int total[kUnevenBins];
  const int bin = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long count = a->count;
  const int chunks = (int)((count + kUnevenChunk - 1) / kUnevenChunk);
  int run = 0;
  for (int c0 = 0; c0 < chunks; c0 += 32) {
    const int c = c0 + lane;
    const int v = c < chunks ? a->chunk_base[c * kUnevenBins + bin] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (c < chunks) a->chunk_base[c * kUnevenBins + bin] = run + x - v;  // exclusive, within the bin
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) total[bin] = run;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int b = 0; b < kUnevenBins; ++b) {
      a->bucket_start[b] = s;
      a->bucket_count[b] = b < kUnevenInvalid ? total[b] : 0;
      s += total[b];
    }
  }
  if (size_nodes && threadIdx.x < kUnevenInvalid && a->nodes[threadIdx.x] != nullptr) {
    // A size with at least 40 % of the batch's bytes runs one CTA per tile
    // (measured 9-15 % faster alone at N = 512..4096, and 1.8 % faster on a
    // mixed batch whose N = 4096 transforms hold 45 % of the bytes).  The
    // other sizes keep persistent grids of their resident CTAs on the device,
    // so that each can use the whole device as the others finish (measured
    // faster on mixed batches than one CTA per tile for every size, whose
    // grids then run one after another, and than grids in proportion to each
    // size's bytes).
    const int b = threadIdx.x;
    cudaGraphKernelNodeSetGridDim(a->nodes[b], dim3((unsigned)uneven_grid(total, b, a->tpb[b], a->wave[b])));
  }
}

// Stable scatter: the offset of entry i goes to list[start(bin) + chunk base +
// rank of i among the entries of its bin earlier in the chunk], so the size
// kernels find each transform with one load.
static __global__ void __launch_bounds__(kUnevenChunk) uneven_scatter(UnevenArgs* __restrict__ a) {
  __shared__ int wc[kUnevenChunk / 32][kUnevenBins];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long chunk0 = (long long)blockIdx.x * kUnevenChunk;
  if (chunk0 >= a->count) return;
  if (lane < kUnevenBins) wc[warp][lane] = 0;
  __syncwarp();
  const long long i = chunk0 + threadIdx.x;
  const int b = uneven_entry_bin(*a, i);
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  const int rank = __popc(peers & ((1u << lane) - 1u));
  if (b >= 0 && rank == 0) wc[warp][b] = __popc(peers);
  __syncthreads();
  // exclusive scan over the 32 warps, one warp per bin
  if (warp < kUnevenBins) {
    const int v = wc[lane][warp];
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    __syncwarp();
    wc[lane][warp] = x - v;
  }
  __syncthreads();
  if (b >= 0 && b != kUnevenInvalid)
    a->list[a->bucket_start[b] + a->chunk_base[blockIdx.x * kUnevenBins + b] + wc[warp][b] + rank] =
        __ldg(a->offsets + i);
}

// Slots of the per-CTA ring of tile offsets (current, next, the one after).
constexpr int kUnevenRing = 3;

// Per-size kernel: CTAs stride over the tiles of bucket `bin` (one tile each
// when the grid covers the bucket).  The tiles' transform offsets pass
// through a ring of kUnevenRing slots in shared memory, filled with cp.async:
// slot s0 holds the current tile, s1 the tile `ahead` tiles later (this CTA's
// next tile when the grid is persistent, else the tile one wave of resident
// CTAs later), whose transforms are prefetched into L2.  No offset is held in
// a register across a tile (the plans run at their register limit), and one
// barrier per tile makes the slots visible.  Plans that do not stage their
// tile read their own transform's offset once; staged plans index the slot.
template <class E, class PL>
__global__ void __launch_bounds__(Fft<E, PL>::THREADS, PL::MINB)
fft_uneven_kernel(const UnevenArgs* __restrict__ a, int bin, const typename E::TW* __restrict__ tw) {
  using F = Fft<E, PL>;
  using FK = Fft<PlanEngine<E, PL>, PL>;
  constexpr int TPB = PL::TPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long* ring = reinterpret_cast<long long*>(smem_raw + F::SMEM);  // [kUnevenRing][TPB]
  const long long count = a->bucket_count[bin];
  // tiles of the bucket, counted in 32 bits (the loop state stays small: the
  // plans run at their register limit)
  const int ntiles = (int)((count + TPB - 1) / TPB);
  if ((int)blockIdx.x >= ntiles) return;
  const long long* list = a->list + a->bucket_start[bin];
  // a grid that covers the bucket runs one tile per CTA and prefetches one
  // wave of resident CTAs ahead; a smaller (persistent) grid prefetches the
  // CTA's next tile, whose offsets the ring then already holds
  const int wave = a->wave[bin];
  const int ahead = (int)gridDim.x >= ntiles && wave > 0 && wave < (int)gridDim.x ? wave : (int)gridDim.x;
  const int tid = threadIdx.x;
  // offset of the bucket's transform k (0 past the end) into ring slot `slot`
  auto fetch = [&](int slot, long long k) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(ring + slot * TPB + tid);
    const bool in = k < count;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(list + (in ? k : 0)),
                 "r"(in ? 8 : 0)
                 : "memory");
  };
  if (tid < TPB) {
    fetch(0, (long long)blockIdx.x * TPB + tid);
    fetch(1, (long long)(blockIdx.x + ahead) * TPB + tid);
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_all;" ::: "memory");
  }
  __syncthreads();
  int s0 = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long tile0 = (long long)tile * TPB;
    const int s1 = s0 == kUnevenRing - 1 ? 0 : s0 + 1, s2 = s1 == kUnevenRing - 1 ? 0 : s1 + 1;
    if (tid < TPB) {
      if (tile + (int)gridDim.x < ntiles) {  // a next tile of this CTA (persistent grid: ahead = gridDim)
        fetch(s2, (long long)(tile + 2 * ahead) * TPB + tid);
        asm volatile("cp.async.commit_group;" ::: "memory");
      }
      // the transforms `ahead` tiles later, into L2
      if ((long long)(tile + ahead) * TPB + tid < count)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a->in + ring[s1 * TPB + tid]),
                     "r"((unsigned)(PL::N * 16))
                     : "memory");
    }
    if constexpr (!FK::STAGED) {
      const RegTile tl{a->in, a->out, ring[s0 * TPB + tid / FK::T], tile0, count};
      fft_tile<E, PL>(tl, tw, smem_raw);
    } else {
      const IndexedTile tl{a->in, a->out, ring + s0 * TPB, tile0, count};
      fft_tile<E, PL>(tl, tw, smem_raw);
    }
    if (tile + (int)gridDim.x >= ntiles) break;  // the last tile of this CTA
    if (tid < TPB) asm volatile("cp.async.wait_all;" ::: "memory");
    // the ring slot filled above is visible, and this tile's readers of the
    // exchange buffer and of slot s0 are done
    __syncthreads();
    s0 = s1;
  }
}

}  // namespace fftoc
