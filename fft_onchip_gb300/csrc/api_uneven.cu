// fftoc — uneven batches (mixed sizes, int64 offset table) as one CUDA graph.
//
// No counterpart in the reference: its harness launches one executor (one
// size) per kernel, includes/testing.cuh:59-92, and its benchmark driver
// loops over sizes, scripts/generate_bench.py:93-113.  The graph built here
// buckets the table by size on the device (fft_uneven.cuh) and runs one
// persistent kernel per size on parallel branches, so a batch of any size
// mix costs one argument kernel and one graph launch, with no host sync.
#include <atomic>
#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/fftoc.h"
#include "fft_uneven.cuh"
#include "internal.h"

struct fftoc_uneven_plan_s {
  int device = 0;
  int slot = 1;               // 0 binary64, 1 fixed point
  int64_t max_count = 0;
  int chunks = 0;
  fftoc::UnevenArgs* args = nullptr;
  long long* list = nullptr;  // bucketed transform offsets
  int* chunk_base = nullptr;
  int* err = nullptr;
  int sms = 0;
  int variant[fftoc::kNumSizes] = {};   // plan per size in the captured graph
  const fftoc::KernelDesc* kd[fftoc::kNumSizes] = {};
  const void* tw[fftoc::kNumSizes] = {};
  cudaStream_t cap = nullptr;
  cudaStream_t branch[fftoc::kNumSizes] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[fftoc::kNumSizes] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool device_sized = false;  // the graph's size kernels get their grids from uneven_scan
  std::mutex mu;
};

namespace fftoc {
namespace {

// Uneven kernels per engine slot and size, with their attributes set on
// each device that uses them.
const SizeVariants* uneven_variants(int slot) {
  static SizeVariants table[2][kNumSizes];
  static std::once_flag once;
  std::call_once(once, [] {
    describe_uneven_f64(table[0]);
    describe_uneven_fx(table[1]);
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < kNumSizes; ++i) {
        const SizeVariants& full = compiled_variants(s)[i];
        for (int v = 0; v < table[s][i].count; ++v) {
          // everything but the uneven fields from the batched description
          const void* fn = table[s][i].v[v].fn_uneven;
          const int smem = table[s][i].v[v].smem_uneven;
          table[s][i].v[v] = full.v[v];
          table[s][i].v[v].fn_uneven = fn;
          table[s][i].v[v].smem_uneven = smem;
        }
      }
  });
  return table[slot];
}

}  // namespace

// Plan of size index i for the uneven path: while the size's choice is the
// library default (variant 0), its UnevenDefault<> plan if it has one; else
// the chosen plan if it has an uneven kernel; else the first plan that has one.
int uneven_variant(int slot, int i) {
  const SizeVariants& sv = uneven_variants(slot)[i];
  const int c = chosen_variant(slot, i);
  if (c == 0)
    for (int v = 0; v < sv.count; ++v)
      if (sv.v[v].uneven_default && sv.v[v].fn_uneven) return v;
  if (c < sv.count && sv.v[c].fn_uneven) return c;
  for (int v = 0; v < sv.count; ++v)
    if (sv.v[v].fn_uneven) return v;
  return -1;
}

namespace {

struct UnevenDevice {
  std::once_flag once;
  fftoc_status status = FFTOC_OK;
  std::string error;
  SizeVariants var[2][kNumSizes];
};
constexpr int kMaxDevices = 64;
UnevenDevice g_udev[kMaxDevices];

fftoc_status uneven_device(int dev, UnevenDevice** out) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(FFTOC_ERR_INVALID_VALUE, "device ordinal out of range");
  UnevenDevice& u = g_udev[dev];
  std::call_once(u.once, [&] {
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < kNumSizes; ++i) {
        u.var[s][i] = uneven_variants(s)[i];
        for (int v = 0; v < u.var[s][i].count; ++v) {
          KernelDesc& d = u.var[s][i].v[v];
          if (!d.fn_uneven) continue;
          cudaError_t e = cudaFuncSetAttribute(d.fn_uneven, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem_uneven);
          if (e == cudaSuccess) e = fit_carveout(d.fn_uneven, d.threads, d.smem_uneven, &d.blocks_per_sm_uneven);
          if (e != cudaSuccess) {
            cudaGetLastError();
            u.status = FFTOC_ERR_CUDA;
            u.error = std::string("uneven kernel set-up: ") + cudaGetErrorString(e);
            return;
          }
          if (d.blocks_per_sm_uneven < 1) d.blocks_per_sm_uneven = 1;
        }
      }
  });
  if (u.status != FFTOC_OK) return set_error(u.status, u.error);
  *out = &u;
  return FFTOC_OK;
}

fftoc_status cuda_err(cudaError_t e, const char* what) {
  cudaGetLastError();
  return set_error(e == cudaErrorMemoryAllocation ? FFTOC_ERR_NO_MEMORY : FFTOC_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

int uneven_choice(const UnevenDevice&, int slot, int i) { return uneven_variant(slot, i); }

fftoc_status resolve_kernels(fftoc_uneven_plan p, const UnevenDevice& u, bool* changed) {
  *changed = false;
  for (int i = 0; i < kNumSizes; ++i) {
    const int v = uneven_choice(u, p->slot, i);
    if (v < 0) return set_error(FFTOC_ERR_UNSUPPORTED, "no uneven kernel for n=" + std::to_string(kSizes[i]));
    if (p->kd[i] && v == p->variant[i]) continue;
    const void* tw = nullptr;
    int* err = nullptr;
    int sms = 0;
    fftoc_status st = device_plan_resources(p->slot, i, v, &tw, &err, &sms);
    if (st != FFTOC_OK) return st;
    p->variant[i] = v;
    p->kd[i] = &u.var[p->slot][i].v[v];
    p->tw[i] = tw;
    p->err = err;
    p->sms = sms;
    *changed = true;
  }
  return FFTOC_OK;
}

fftoc_status enqueue_bucketing(fftoc_uneven_plan p, cudaStream_t s, bool size_nodes) {
  uneven_hist<<<p->chunks, kUnevenChunk, 0, s>>>(p->args, p->err);
  uneven_scan<<<1, 32 * kUnevenBins, 0, s>>>(p->args, size_nodes ? 1 : 0);
  uneven_scatter<<<p->chunks, kUnevenChunk, 0, s>>>(p->args);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FFTOC_OK : cuda_err(e, "bucketing launch");
}

// Launch of size i's kernel; with `node` (during capture) as a
// device-updatable graph node whose handle is returned there.
fftoc_status launch_size(fftoc_uneven_plan p, int i, long long blocks, cudaStream_t s,
                         cudaGraphDeviceNode_t* node = nullptr) {
  const KernelDesc& d = *p->kd[i];
  UnevenArgs* a = p->args;
  int bin = i;
  const void* tw = p->tw[i];
  void* kargs[] = {(void*)&a, (void*)&bin, (void*)&tw};
  cudaError_t e;
  if (node) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(d.threads);
    cfg.dynamicSmemBytes = (size_t)d.smem_uneven;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeDeviceUpdatableKernelNode;
    attr[0].val.deviceUpdatableKernelNode.deviceUpdatable = 1;
    attr[0].val.deviceUpdatableKernelNode.devNode = nullptr;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelExC(&cfg, d.fn_uneven, kargs);
    *node = attr[0].val.deviceUpdatableKernelNode.devNode;
    if (e == cudaSuccess && *node == nullptr) e = cudaErrorInvalidValue;
  } else {
    e = cudaLaunchKernel(d.fn_uneven, dim3((unsigned)blocks), dim3(d.threads), kargs, (size_t)d.smem_uneven, s);
  }
  return e == cudaSuccess ? FFTOC_OK : cuda_err(e, "cudaLaunchKernel(uneven)");
}

long long wave_blocks(fftoc_uneven_plan p, int i) {
  return (long long)p->sms * p->kd[i]->blocks_per_sm_uneven;
}

long long persistent_blocks(fftoc_uneven_plan p, int i) {
  const KernelDesc& d = *p->kd[i];
  const long long tiles = (p->max_count + d.tpb - 1) / d.tpb;
  const long long cap = (long long)p->sms * d.blocks_per_sm_uneven;
  return tiles < cap ? tiles : cap;
}

// One capture attempt: bucketing, then one kernel per size on its own
// branch.  With `size_nodes` the size kernels are device-updatable nodes whose
// grids uneven_scan sets on every launch; their handles, transforms per CTA
// and wave sizes go to the argument block.
fftoc_status capture_once(fftoc_uneven_plan p, bool size_nodes) {
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  if (p->graph) {
    cudaGraphDestroy(p->graph);
    p->graph = nullptr;
  }
  cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_err(e, "cudaStreamBeginCapture");
  cudaGraphDeviceNode_t nodes[kUnevenBins] = {};
  fftoc_status st = enqueue_bucketing(p, p->cap, size_nodes);
  if (st == FFTOC_OK && (e = cudaEventRecord(p->fork, p->cap)) != cudaSuccess) st = cuda_err(e, "cudaEventRecord");
  // every size on its own branch: the sizes run side by side
  for (int i = 0; i < kNumSizes && st == FFTOC_OK; ++i) {
    if ((e = cudaStreamWaitEvent(p->branch[i], p->fork, 0)) != cudaSuccess) {
      st = cuda_err(e, "cudaStreamWaitEvent");
      break;
    }
    st = launch_size(p, i, persistent_blocks(p, i), p->branch[i], size_nodes ? &nodes[i] : nullptr);
    if (st != FFTOC_OK) break;
    if ((e = cudaEventRecord(p->join[i], p->branch[i])) != cudaSuccess) st = cuda_err(e, "cudaEventRecord");
    else if ((e = cudaStreamWaitEvent(p->cap, p->join[i], 0)) != cudaSuccess) st = cuda_err(e, "cudaStreamWaitEvent");
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(p->cap, &g);
  if (st != FFTOC_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return cuda_err(e, "cudaStreamEndCapture");
  p->graph = g;
  e = cudaGraphInstantiate(&p->exec, g, 0);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphInstantiate");
  // a graph that updates its own nodes from the device is uploaded before
  // its first launch
  if (size_nodes && (e = cudaGraphUpload(p->exec, p->cap)) == cudaSuccess) e = cudaStreamSynchronize(p->cap);
  if (e != cudaSuccess) return cuda_err(e, "cudaGraphUpload");
  int tpb[kUnevenBins] = {}, wave[kUnevenBins] = {};
  for (int i = 0; i < kNumSizes; ++i) {
    tpb[i] = p->kd[i]->tpb;
    wave[i] = (int)wave_blocks(p, i);
  }
  char* a = reinterpret_cast<char*>(p->args);
  if ((e = cudaMemcpy(a + offsetof(UnevenArgs, nodes), nodes, sizeof(nodes), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(a + offsetof(UnevenArgs, tpb), tpb, sizeof(tpb), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(a + offsetof(UnevenArgs, wave), wave, sizeof(wave), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_err(e, "cudaMemcpy(uneven graph nodes)");
  p->device_sized = size_nodes;
  return FFTOC_OK;
}

// Captures the plan's graph with device-sized grids, or with persistent grids
// where the runtime refuses device-updatable nodes.  A re-capture first waits
// for the device: executions of the previous graph read the argument block.
fftoc_status capture(fftoc_uneven_plan p) {
  if (p->exec) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_err(e, "cudaDeviceSynchronize");
  }
  if (capture_once(p, true) == FFTOC_OK) return FFTOC_OK;
  cudaGetLastError();
  return capture_once(p, false);
}

void release(fftoc_uneven_plan p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (int i = 0; i < kNumSizes; ++i) {
    if (p->branch[i]) cudaStreamDestroy(p->branch[i]);
    if (p->join[i]) cudaEventDestroy(p->join[i]);
  }
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->args) cudaFree(p->args);
  if (p->list) cudaFree(p->list);
  if (p->chunk_base) cudaFree(p->chunk_base);
  delete p;
}

fftoc_status plan_create(fftoc_uneven_plan* out, int64_t max_count, int engine) {
  if (!out) return set_error(FFTOC_ERR_INVALID_VALUE, "null plan pointer");
  *out = nullptr;
  if (max_count < 1 || max_count > 0x7FFFFFFFLL)
    return set_error(FFTOC_ERR_INVALID_VALUE, "max_count must be in [1, 2^31 - 1]");
  if (engine < FFTOC_ENGINE_AUTO || engine > kLastEngine) return set_error(FFTOC_ERR_INVALID_VALUE, "unknown engine");
  const int eng = resolved_engine(8, engine);
  if (eng != FFTOC_ENGINE_F64 && eng != FFTOC_ENGINE_FX)
    return set_error(FFTOC_ERR_UNSUPPORTED, "engine not available for uneven batches");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDevice");
  UnevenDevice* u = nullptr;
  fftoc_status st = uneven_device(dev, &u);
  if (st != FFTOC_OK) return st;

  fftoc_uneven_plan p = new fftoc_uneven_plan_s;
  p->device = dev;
  p->slot = eng == FFTOC_ENGINE_FX ? 1 : 0;
  p->max_count = max_count;
  p->chunks = (int)((max_count + kUnevenChunk - 1) / kUnevenChunk);
  auto bad = [&](fftoc_status s) {
    release(p);
    return s;
  };
  if ((e = cudaMalloc(&p->args, sizeof(UnevenArgs))) != cudaSuccess) return bad(cuda_err(e, "cudaMalloc(uneven args)"));
  if ((e = cudaMalloc(&p->list, (size_t)max_count * sizeof(long long))) != cudaSuccess)
    return bad(cuda_err(e, "cudaMalloc(uneven list)"));
  if ((e = cudaMalloc(&p->chunk_base, (size_t)p->chunks * kUnevenBins * sizeof(int))) != cudaSuccess)
    return bad(cuda_err(e, "cudaMalloc(uneven chunk table)"));
  UnevenArgs init{};
  init.list = p->list;
  init.chunk_base = p->chunk_base;
  if ((e = cudaMemcpy(p->args, &init, sizeof(init), cudaMemcpyHostToDevice)) != cudaSuccess)
    return bad(cuda_err(e, "cudaMemcpy(uneven args)"));
  if ((e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking)) != cudaSuccess)
    return bad(cuda_err(e, "cudaStreamCreate"));
  if ((e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) != cudaSuccess)
    return bad(cuda_err(e, "cudaEventCreate"));
  for (int i = 0; i < kNumSizes; ++i) {
    if ((e = cudaStreamCreateWithFlags(&p->branch[i], cudaStreamNonBlocking)) != cudaSuccess)
      return bad(cuda_err(e, "cudaStreamCreate"));
    if ((e = cudaEventCreateWithFlags(&p->join[i], cudaEventDisableTiming)) != cudaSuccess)
      return bad(cuda_err(e, "cudaEventCreate"));
  }
  bool changed = false;
  if ((st = resolve_kernels(p, *u, &changed)) != FFTOC_OK) return bad(st);
  if ((st = capture(p)) != FFTOC_OK) return bad(st);
  *out = p;
  return FFTOC_OK;
}

fftoc_status check_exec_args(fftoc_uneven_plan p, const double* in, double* out, const int64_t* offsets,
                             const int32_t* ns, int64_t count) {
  if (!p) return set_error(FFTOC_ERR_INVALID_VALUE, "null plan");
  if (count < 0) return set_error(FFTOC_ERR_INVALID_VALUE, "count must be >= 0");
  if (count > p->max_count)
    return set_error(FFTOC_ERR_INVALID_VALUE, "count " + std::to_string(count) + " exceeds the plan's max_count " +
                                                  std::to_string(p->max_count));
  if (count == 0) return FFTOC_OK;
  if (!in || !out || !offsets || !ns) return set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  if (((uintptr_t)in & 15) || ((uintptr_t)out & 15)) return set_error(FFTOC_ERR_MISALIGNED, "buffers must be 16-byte aligned");
  if (((uintptr_t)offsets & 7) || ((uintptr_t)ns & 3))
    return set_error(FFTOC_ERR_MISALIGNED, "offsets must be 8-byte and ns 4-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDevice");
  if (dev != p->device) return set_error(FFTOC_ERR_INVALID_VALUE, "plan belongs to another device");
  return FFTOC_OK;
}

fftoc_status set_args(fftoc_uneven_plan p, const double* in, double* out, const int64_t* offsets, const int32_t* ns,
                      int64_t count, cudaStream_t s) {
  uneven_set_args<<<1, 1, 0, s>>>(p->args, reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out),
                                  reinterpret_cast<const long long*>(offsets), reinterpret_cast<const int*>(ns),
                                  (long long)count);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FFTOC_OK : cuda_err(e, "uneven_set_args launch");
}

fftoc_status execute(fftoc_uneven_plan p, const double* in, double* out, const int64_t* offsets, const int32_t* ns,
                     int64_t count, cudaStream_t s) {
  fftoc_status st = check_exec_args(p, in, out, offsets, ns, count);
  if (st != FFTOC_OK || count == 0) return st;
  std::lock_guard<std::mutex> lk(p->mu);
  UnevenDevice* u = nullptr;
  if ((st = uneven_device(p->device, &u)) != FFTOC_OK) return st;
  bool changed = false;
  if ((st = resolve_kernels(p, *u, &changed)) != FFTOC_OK) return st;
  if (changed && (st = capture(p)) != FFTOC_OK) return st;
  if ((st = set_args(p, in, out, offsets, ns, count, s)) != FFTOC_OK) return st;
  cudaError_t e = cudaGraphLaunch(p->exec, s);
  return e == cudaSuccess ? FFTOC_OK : cuda_err(e, "cudaGraphLaunch");
}

const int* device_counts(fftoc_uneven_plan p) {
  return reinterpret_cast<const int*>(reinterpret_cast<const char*>(p->args) + offsetof(UnevenArgs, bucket_count));
}

fftoc_status read_counts(fftoc_uneven_plan p, int* h, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(h, device_counts(p), kNumSizes * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? FFTOC_OK : cuda_err(e, "reading uneven bucket counts");
}

fftoc_status execute_per_size(fftoc_uneven_plan p, const double* in, double* out, const int64_t* offsets,
                              const int32_t* ns, int64_t count, cudaStream_t s) {
  fftoc_status st = check_exec_args(p, in, out, offsets, ns, count);
  if (st != FFTOC_OK || count == 0) return st;
  std::lock_guard<std::mutex> lk(p->mu);
  UnevenDevice* u = nullptr;
  if ((st = uneven_device(p->device, &u)) != FFTOC_OK) return st;
  bool changed = false;
  if ((st = resolve_kernels(p, *u, &changed)) != FFTOC_OK) return st;
  if ((st = set_args(p, in, out, offsets, ns, count, s)) != FFTOC_OK) return st;
  if ((st = enqueue_bucketing(p, s, false)) != FFTOC_OK) return st;
  int h[kNumSizes];
  if ((st = read_counts(p, h, s)) != FFTOC_OK) return st;
  for (int i = 0; i < kNumSizes; ++i) {
    if (h[i] == 0) continue;
    const long long tiles = ((long long)h[i] + p->kd[i]->tpb - 1) / p->kd[i]->tpb;
    if ((st = launch_size(p, i, tiles, s)) != FFTOC_OK) return st;
  }
  return FFTOC_OK;
}

struct OneShot {
  std::mutex mu;
  fftoc_uneven_plan plan = nullptr;
};
OneShot g_oneshot[kMaxDevices];

}  // namespace
}  // namespace fftoc

extern "C" {

fftoc_status fftoc_uneven_plan_create(fftoc_uneven_plan* plan, int64_t max_count, int engine) {
  return fftoc::plan_create(plan, max_count, engine);
}

fftoc_status fftoc_uneven_execute(fftoc_uneven_plan plan, const double* in, double* out, const int64_t* offsets,
                                  const int32_t* ns, int64_t count, fftoc_stream stream) {
  return fftoc::execute(plan, in, out, offsets, ns, count, (cudaStream_t)stream);
}

fftoc_status fftoc_uneven_execute_per_size(fftoc_uneven_plan plan, const double* in, double* out,
                                           const int64_t* offsets, const int32_t* ns, int64_t count,
                                           fftoc_stream stream) {
  return fftoc::execute_per_size(plan, in, out, offsets, ns, count, (cudaStream_t)stream);
}

fftoc_status fftoc_uneven_plan_device_sized(fftoc_uneven_plan plan, int* sized) {
  if (!plan || !sized) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  std::lock_guard<std::mutex> lk(plan->mu);
  *sized = plan->device_sized ? 1 : 0;
  return FFTOC_OK;
}

fftoc_status fftoc_uneven_counts(fftoc_uneven_plan plan, int64_t* counts) {
  if (!plan || !counts) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "null pointer");
  int h[fftoc::kNumSizes];
  std::lock_guard<std::mutex> lk(plan->mu);
  cudaError_t e = cudaMemcpy(h, fftoc::device_counts(plan), sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fftoc::cuda_err(e, "reading uneven bucket counts");
  for (int i = 0; i < fftoc::kNumSizes; ++i) counts[i] = h[i];
  return FFTOC_OK;
}

fftoc_status fftoc_uneven_plan_destroy(fftoc_uneven_plan plan) {
  if (!plan) return FFTOC_OK;
  fftoc::release(plan);
  return FFTOC_OK;
}

fftoc_status fftoc_c2c_fwd_uneven(const double* in, double* out, const int64_t* offsets, const int32_t* ns,
                                  int64_t count, fftoc_stream stream) {
  if (count < 0) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "count must be >= 0");
  if (count == 0) return FFTOC_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fftoc::cuda_err(e, "cudaGetDevice");
  if (dev < 0 || dev >= fftoc::kMaxDevices) return fftoc::set_error(FFTOC_ERR_INVALID_VALUE, "device ordinal out of range");
  fftoc::OneShot& o = fftoc::g_oneshot[dev];
  std::lock_guard<std::mutex> lk(o.mu);
  if (!o.plan || o.plan->max_count < count) {
    if (o.plan) {
      // the previous plan may still be in use by earlier work on `stream`
      e = cudaStreamSynchronize((cudaStream_t)stream);
      if (e != cudaSuccess) return fftoc::cuda_err(e, "cudaStreamSynchronize");
      fftoc::release(o.plan);
      o.plan = nullptr;
    }
    int64_t cap = 1024;
    while (cap < count) cap *= 2;
    fftoc_status st = fftoc::plan_create(&o.plan, cap, FFTOC_ENGINE_AUTO);
    if (st != FFTOC_OK) return st;
  }
  return fftoc::execute(o.plan, in, out, offsets, ns, count, (cudaStream_t)stream);
}

}  // extern "C"
