/*
 * fftoc — batched forward complex FFTs of N = 8..4096 points on one GB300.
 *
 * C ABI of the library (libfftoc.so).  It replaces the per-size executor
 * surface of gprabowski/fft_onchip, where every size N has its own device
 * executor type driven by the test harness:
 *   includes/tensor_fft_8.cuh:12-66      tensor_fft_8<CT,8,UPB,FPU>
 *   includes/tensor_fft_16.cuh:9-63      tensor_fft_16 (does not compile upstream)
 *   includes/tensor_fft_64.cuh:12-77     tensor_fft_64
 *   includes/tensor_fft_128.cuh:12-101   tensor_fft_128
 *   includes/tensor_fft_256.cuh:10-123   tensor_fft_256
 *   includes/tensor_fft_512.cuh:12-122   tensor_fft_512
 *   includes/tensor_fft_4096.cuh:12-98   tensor_fft_4096
 *   includes/legacy8_fft.cuh:11-120      legacy_fft<CT,N>     (N a power of 8)
 *   includes/legacy16_fft.cuh:17-173     legacy16_fft<CT,N>   (N a power of 16)
 * and the harness entry that stages data and launches them,
 *   includes/testing.cuh:16-57 (fft_tester), :59-92 (run_fft_kernel).
 * There, one launch transforms a contiguous batch of N-point transforms of
 * thrust::complex<double> (includes/config.hpp:6), in place, forward
 * (exp(-2*pi*i*n*k/N)), unnormalised, natural order.  The reference has no
 * sizes 32, 1024 or 2048; they are provided here with the same contract.
 *
 * Conventions of every transform entry point:
 *   - in/out are DEVICE pointers to batch*n interleaved (re, im) doubles,
 *     16-byte aligned; transform b occupies doubles [2*n*b, 2*n*(b+1)).
 *   - in == out (in place) is allowed; other overlaps are rejected.
 *   - calls are asynchronous on `stream` (0 = legacy default stream); they
 *     never call exit() and never synchronise.
 *   - errors are returned as fftoc_status; fftoc_last_error_string() gives a
 *     per-thread message for the last failing call.
 *   - the library owns its twiddle tables (built on the host in long double,
 *     uploaded once per device on first use); the caller owns the buffers.
 *   - thread safe across host threads.
 *   - results agree with the exact DFT to relative L2 error <= 1e-13 for
 *     every engine of the FP64 form (see fftoc_engine).
 */
#ifndef FFTOC_H
#define FFTOC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFTOC_VERSION 10000 /* 1.0.0 */

typedef enum {
  FFTOC_OK = 0,
  FFTOC_ERR_INVALID_SIZE = 1,  /* n is not one of 8,16,...,4096            */
  FFTOC_ERR_INVALID_VALUE = 2, /* null pointer, negative batch, bad enum,
                                  partial overlap, batch too large          */
  FFTOC_ERR_MISALIGNED = 3,    /* buffer not 16-byte aligned               */
  FFTOC_ERR_NO_MEMORY = 4,     /* device allocation failed                 */
  FFTOC_ERR_CUDA = 5,          /* CUDA runtime error                       */
  FFTOC_ERR_TIMEOUT = 6,       /* a bounded device wait gave up            */
  FFTOC_ERR_UNSUPPORTED = 7    /* engine not available for this n         */
} fftoc_status;

/* Arithmetic used inside a transform (input/output are always binary64). */
typedef enum {
  FFTOC_ENGINE_AUTO = 0, /* fastest engine of the FP64 form for this n           */
  FFTOC_ENGINE_F64 = 1,  /* IEEE binary64 (DFMA/DADD)                            */
  FFTOC_ENGINE_FX = 2,   /* 64-bit block fixed point: per-transform power-of-two
                            scale, exact integer adds, 60-bit twiddles;
                            relative L2 error ~1e-15                             */
  FFTOC_ENGINE_DMMA = 3, /* IEEE binary64 on the FP64 tensor cores: the
                            Karatsuba complex product (3 real 8x8x8 products,
                            the reference's tensor_utils.cuh:25-36 scheme) of
                            the exact DFT matrix, n = 8 only
                            (FFTOC_ERR_UNSUPPORTED for other n)                 */
  FFTOC_ENGINE_SPLIT_BF16X3 = 4, /* split-precision form, 3 BF16 terms per
                            operand on the tensor cores, FP32 accumulation and
                            data (relative L2 error ~1e-7; n >= 16)              */
  FFTOC_ENGINE_SPLIT_TF32X2 = 5, /* split-precision form, 2 TF32 terms    */
  FFTOC_ENGINE_SPLIT_EXACT = 6   /* exact-slice split form: block fixed point,
                            six 8-bit digits per operand on the BF16 tensor
                            cores, products exact in FP32 (error ~1e-14)    */
} fftoc_engine;

/* Operand splits of the split-precision form (fftoc_c2c_fwd_split). */
typedef enum { FFTOC_SPLIT_BF16X3 = 1, FFTOC_SPLIT_TF32X2 = 2, FFTOC_SPLIT_EXACT = 3 } fftoc_split_kind;

typedef struct CUstream_st *fftoc_stream; /* same type as cudaStream_t */

/* One entry per size (reference: the tensor_fft_N / legacy executors above). */
fftoc_status fftoc_c2c_fwd_n8(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n16(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n32(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n64(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n128(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n256(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n512(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n1024(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n2048(const double *in, double *out, int64_t batch, fftoc_stream stream);
fftoc_status fftoc_c2c_fwd_n4096(const double *in, double *out, int64_t batch, fftoc_stream stream);

/* Size as a runtime argument (reference: run_fft_kernel<CT,Size,FFTExec>,
 * includes/testing.cuh:59-92, with Size a template argument). */
fftoc_status fftoc_c2c_fwd(int n, const double *in, double *out, int64_t batch, fftoc_stream stream);

/* Same, with an explicit engine. */
fftoc_status fftoc_c2c_fwd_ex(int n, const double *in, double *out, int64_t batch, int engine,
                              fftoc_stream stream);

/* Split-precision form (no binary64 counterpart in the reference, whose
 * tensor path is FP64 DMMA with FP32 twiddles, tensor_fft_64.cuh:33-39).
 * Every radix-16 pass of the plan is a GEMM on the tensor cores (tcgen05):
 * butterfly inputs and the 16-point DFT matrix are split into 3 BF16 terms
 * (FFTOC_SPLIT_BF16X3, the six term products with i + j <= 2) or 2 TF32
 * terms (FFTOC_SPLIT_TF32X2, three products), accumulated in FP32; data
 * between passes and the twiddle products are FP32; input and output are
 * binary64, with an exact power-of-two scale per transform when its largest
 * magnitude is outside [2^-60, 2^60].  FFTOC_SPLIT_EXACT keeps the block
 * fixed point of FFTOC_ENGINE_FX between passes and cuts each operand into
 * six balanced 8-bit digits whose products, summed per slice order, are exact
 * in FP32 (the 21 orders-0..5 products are kept), which meets the 1e-11 gate
 * of the split form.  Same arguments and conventions as
 * fftoc_c2c_fwd; n = 16..4096 (FFTOC_ERR_UNSUPPORTED for n = 8).  Also
 * reachable as engines FFTOC_ENGINE_SPLIT_* of fftoc_c2c_fwd_ex. */
fftoc_status fftoc_c2c_fwd_split(int n, const double *in, double *out, int64_t batch, int kind,
                                 fftoc_stream stream);

/* Host buffers in and out (the reference harness's path: cudaMemcpy H2D,
 * launch, cudaMemcpy D2H — includes/testing.cuh:109-113,166-171).
 * h_in/h_out are HOST pointers (pinned memory gives overlapped, full-speed
 * copies; pageable memory works but copies synchronously), 16-byte aligned,
 * batch*n complex values each; h_in == h_out is allowed.  The batch is
 * streamed through the device in chunks of 64 MiB (H2D, transform and D2H
 * of consecutive chunks overlap on three internal streams).  The call is
 * ordered after earlier work on `stream` and `stream` is ordered after its
 * last copy: synchronise `stream` before reading h_out.  The first call on a
 * device allocates 192 MiB of device staging memory and the streams (make it
 * before any stream capture); calls from several host threads serialise
 * their enqueueing. */
fftoc_status fftoc_c2c_fwd_host(int n, const double *h_in, double *h_out, int64_t batch, int engine,
                                fftoc_stream stream);

/* Host buffers in and out, with no device allocation (no counterpart in the
 * reference).  For callers that cannot let a library call cudaMalloc: device
 * memory already claimed by another allocator or a fixed pool, services that
 * must not grow their device footprint after start-up, code that cannot take
 * cudaMalloc's implicit synchronisation.  The batch is staged in a 32 MiB
 * array compiled into the library (file-scope __device__ memory that every
 * GPU loading the library holds until exit): batch*n*16 must be at most
 * 32 MiB, larger batches are rejected with FFTOC_ERR_INVALID_VALUE.  H2D
 * copy, transform (the plan fftoc_plan_query reports) and D2H copy run on
 * `stream`; synchronise it before reading h_out.  All calls share that one
 * array: calls that overlap on the GPU (other streams, other host threads)
 * race and corrupt each other's results — serialise them.  The first call on
 * a device does the set-up (array addresses, twiddle upload into another
 * compiled-in array, kernel attributes): make it before any stream capture;
 * a set-up that fails returns its error and is tried again by the next call.
 * Device-side failures of this path (a bounded wait that gave up) are
 * reported by fftoc_device_error_check(), which allocates nothing. */
fftoc_status fftoc_c2c_fwd_host_noalloc(int n, const double *h_in, double *h_out, int64_t batch, int engine,
                                        fftoc_stream stream);

/* Launch geometry of a size/engine (reference: the FFTExec static members
 * threads / units_per_block / ffts_per_unit, e.g. tensor_fft_64.cuh:16-19). */
typedef struct {
  int n;
  int engine;                 /* resolved engine (never AUTO)               */
  int threads_per_transform;  /* lanes cooperating on one transform         */
  int transforms_per_block;   /* transforms per CTA                          */
  int threads_per_block;
  int smem_bytes;             /* dynamic shared memory per CTA               */
  int passes;                 /* Stockham passes                             */
  int radix[4];               /* radix of each pass                          */
  int points_per_thread;
  int variant;                /* index of this plan among the compiled ones  */
  int variants;               /* number of compiled plans for (n, engine)    */
  int persistent;             /* 1: persistent CTAs, TMA-prefetched tiles    */
  int stages;                 /* shared-memory stages (persistent plans)     */
  int prefetch;               /* 1: each CTA prefetches, into L2, the tile of
                                 the CTA one full wave later                 */
  int code_flags;             /* code and memory-access forms of the plan's
                                 kernels (same results): FFTOC_CODE_* bits   */
  int uneven_variant;         /* plan variant the uneven-batch path and the
                                 serving loop use for this size (equal to the
                                 chosen variant unless the choice is the
                                 default variant 0)                          */
} fftoc_plan_info;
#define FFTOC_CODE_OUTLINED_SLOW_INPUT 1 /* rare input conversions out of line */
#define FFTOC_CODE_IMAD_SPLIT 2          /* limb splits by integer multiply-add */
#define FFTOC_CODE_OUT_HI_ZERO 4         /* output zero test on the high word */
#define FFTOC_CODE_DIRECT_IO 8           /* small n: HBM accessed directly, no
                                            shared-memory staging of the tile */

/* Plan currently used for (n, engine). */
fftoc_status fftoc_plan_query(int n, int engine, fftoc_plan_info *info);

/* Any compiled plan of (n, engine), 0 <= variant < info.variants. */
fftoc_status fftoc_plan_query_variant(int n, int engine, int variant, fftoc_plan_info *info);

/* Use plan `variant` for (n, engine) from now on (process-wide).  The
 * reference picks executor parameters (UPB, FPU) at compile time through the
 * generated sweep, scripts/generate_bench.py:93-113; here the choice is made
 * at run time among the compiled plans. */
fftoc_status fftoc_plan_select(int n, int engine, int variant);

/* Autotuner: time every compiled plan of (n, engine) on a scratch batch of
 * `batch` transforms, select the fastest and return its index and time per
 * launch (ms).  Synchronous on `stream`; allocates and frees 2*batch*n*16
 * bytes of device scratch.  (Reference: the manual sweep of
 * scripts/generate_bench.py:93-113 and src/saturation.cu:36-44.) */
fftoc_status fftoc_autotune(int n, int engine, int64_t batch, fftoc_stream stream, int *best_variant,
                            float *best_ms);

/* Uneven batches: `count` transforms of mixed sizes in one buffer (no
 * counterpart in the reference, whose harness runs one size per launch,
 * includes/testing.cuh:59-92, and whose benchmark loops over sizes,
 * scripts/generate_bench.py:93-113).  Transform i has ns[i] points (8..4096,
 * a power of two) starting at complex element offsets[i] of `in` and of
 * `out`; in/out/offsets/ns are DEVICE pointers, in/out 16-byte aligned,
 * offsets int64 (complex elements), ns int32.  Transforms must not overlap
 * one another in `out` (in == out, in place, is allowed).  Entries with an
 * unsupported size or a negative offset are skipped and raise the device
 * error flag (fftoc_device_error_check -> FFTOC_ERR_INVALID_VALUE); offsets
 * beyond the buffers are the caller's responsibility, as for `batch` in the
 * per-size entry points.
 *
 * A plan owns the bucketing scratch (8 bytes per transform plus 64 bytes per
 * 1024) and one CUDA graph: three bucketing kernels that group the transform
 * offsets by size (stable), then one kernel per size on parallel graph
 * branches, its grid set on the device to the size's tile count (see
 * fftoc_uneven_plan_device_sized), each using the plan currently chosen for its size
 * (fftoc_plan_select / fftoc_autotune; while a size's choice is the default
 * variant 0 the path uses its own default plan for that size, and
 * TMA-prefetching plans fall back to the size's first plan without prefetch;
 * fftoc_plan_info.uneven_variant names the plan used).  fftoc_uneven_execute enqueues a
 * 1-thread argument kernel and the graph on `stream` and is asynchronous; it
 * re-captures the graph when a size's plan choice changed.  One plan runs one
 * batch at a time: executions of one plan must be ordered (same stream, or
 * synchronised); use one plan per concurrent stream.  Create plans before
 * any stream capture (creation allocates and captures). */
typedef struct fftoc_uneven_plan_s *fftoc_uneven_plan;

fftoc_status fftoc_uneven_plan_create(fftoc_uneven_plan *plan, int64_t max_count, int engine);
fftoc_status fftoc_uneven_execute(fftoc_uneven_plan plan, const double *in, double *out, const int64_t *offsets,
                                  const int32_t *ns, int64_t count, fftoc_stream stream);
/* Same transforms without the graph: bucketing kernels, a synchronous read of
 * the per-size counts, then one launch per non-empty size with one CTA per
 * tile, all on `stream` (the comparison path; returns after enqueueing the
 * last launch). */
fftoc_status fftoc_uneven_execute_per_size(fftoc_uneven_plan plan, const double *in, double *out,
                                           const int64_t *offsets, const int32_t *ns, int64_t count,
                                           fftoc_stream stream);
/* Per-size transform counts of the last bucketing (counts[10], sizes 8..4096);
 * synchronous. */
fftoc_status fftoc_uneven_counts(fftoc_uneven_plan plan, int64_t *counts);
/* *sized = 1 when the plan's graph sizes its per-size kernels on the device
 * (device-updatable graph nodes: one CTA per tile), 0 when the runtime refused
 * them and the graph runs persistent per-size kernels. */
fftoc_status fftoc_uneven_plan_device_sized(fftoc_uneven_plan plan, int *sized);
fftoc_status fftoc_uneven_plan_destroy(fftoc_uneven_plan plan);

/* One-shot form: a plan cached per device, grown (re-created) when `count`
 * exceeds its capacity; calls on one device must be ordered. */
fftoc_status fftoc_c2c_fwd_uneven(const double *in, double *out, const int64_t *offsets, const int32_t *ns,
                                  int64_t count, fftoc_stream stream);

/* Serving loop (no counterpart in the reference): continuous batching of FFT
 * requests of mixed sizes from host memory.  A request is `count` transforms
 * of one size n (interleaved complex doubles, 16-byte aligned host buffers,
 * pinned memory for full-speed copies) and an engine.  A scheduler thread
 * admits requests in arrival order into a device pool allocated once at
 * creation (admission by bytes: a request waits until one free range of the
 * pool holds it), packs requests of the oldest pending request's engine
 * into batches of up to max_batch_bytes (requests of other engines keep
 * their place), and runs each batch on one of `slots` streams: H2D copies
 * into the pool, one uneven-batch graph over all its transforms, D2H copies.
 * New batches are formed and launched while others run, as slots and pool
 * memory free up.  A batch launches when it is full, when its oldest request
 * has waited max_wait_us, or when nothing else is in flight.  A request's
 * result is bit-identical whatever it was batched with.  The caller keeps
 * h_in/h_out valid and h_out untouched until the request is done. */
typedef struct {
  int64_t pool_bytes;      /* device pool for request data (default 8 GiB)   */
  int slots;               /* batches in flight, one stream each (default 4) */
  int64_t max_batch_bytes; /* request bytes per batch (default 256 MiB)      */
  double max_wait_us;      /* batching window (default 50 us)                */
} fftoc_server_config;

typedef struct {
  double submit_us, launch_us, done_us; /* server clock (us since creation) */
  fftoc_status status;
} fftoc_request_timing;

typedef struct {
  int64_t batches, requests_done, transforms_done, bytes_done, pool_bytes_in_use, pending;
  int max_inflight_batches;
} fftoc_server_stats_t;

typedef struct fftoc_server_s *fftoc_server;

void fftoc_server_config_default(fftoc_server_config *cfg);
/* Allocates the pool, per-slot streams, offset tables and uneven plans, and
 * starts the scheduler thread (create before any stream capture). */
fftoc_status fftoc_server_create(fftoc_server *server, const fftoc_server_config *cfg);
/* Queue a request; returns at once with its id.  count*n*16 must fit in the
 * pool and count <= max_batch_bytes/128. */
fftoc_status fftoc_server_submit(fftoc_server server, int n, int64_t count, int engine, const double *h_in,
                                 double *h_out, int64_t *request_id);
/* done = 1 once h_out holds the result; the id is then released (poll or
 * wait, once per id). */
fftoc_status fftoc_server_poll(fftoc_server server, int64_t request_id, int *done, fftoc_request_timing *timing);
/* Block until the request is done (FFTOC_ERR_TIMEOUT after timeout_s > 0). */
fftoc_status fftoc_server_wait(fftoc_server server, int64_t request_id, double timeout_s,
                               fftoc_request_timing *timing);
fftoc_status fftoc_server_stats(fftoc_server server, fftoc_server_stats_t *stats);

/* Load replay: submit items[i] at arrival_us after the call starts (a
 * submitting loop on the calling thread), wait for all, and report each
 * request's latency (completion minus scheduled arrival, us) and the wall
 * time.  Requests read h_in_arena + in_offset and write h_out_arena +
 * out_offset (complex elements); requests may share input ranges. */
typedef struct {
  double arrival_us;
  int n;
  int engine;
  int64_t count;
  int64_t in_offset;
  int64_t out_offset;
} fftoc_replay_item;
fftoc_status fftoc_server_replay(fftoc_server server, const fftoc_replay_item *items, int64_t m,
                                 const double *h_in_arena, double *h_out_arena, double *latency_us, double *wall_s);
/* Finish the batches in flight, fail requests not yet started, free everything. */
fftoc_status fftoc_server_destroy(fftoc_server server);

/* On-chip repeat harness (the reference's timing mode: testing::fft_tester
 * and run_perf_tests, includes/testing.cuh:16-127).  Each of `blocks` CTAs
 * copies its transforms_per_block transforms (from data + block * tpb * n)
 * into shared memory, transforms them in place `repeats` times with the plan
 * the library uses for (n, engine) (the whole per-transform computation,
 * binary64 conversion included; TMA-prefetching plans fall back to the
 * size's first plan without prefetch), and copies them back.  Differencing
 * the times of two repeat counts gives the on-chip cost of one pass, as the
 * reference reports it.  `data` holds blocks * tpb * n complex values (device
 * memory).  Binary64 and fixed-point engines. */
fftoc_status fftoc_onchip_plan(int n, int engine, int *transforms_per_block, int *variant);
fftoc_status fftoc_onchip_run(int n, int engine, double *data, int64_t blocks, int repeats, fftoc_stream stream);

/* Twiddle table for the device-side executors of <fftoc/exec.cuh> (the
 * FFTExec shape of includes/tensor_fft_64.cuh:12-45): the table of a plan of
 * size n whose passes have radices radix[0..3] (each 2, 4, 8 or 16, unused
 * passes 1 at the end), in the engine's layout (16 bytes per entry: binary64
 * (cos, -sin), or fixed-point limbs), in device memory of the current device
 * owned by the library until the process exits.  *table is NULL for a
 * one-pass plan (no twiddles).  Engines: binary64, fixed point (AUTO
 * resolves to the latter).  Synchronous on first use of a plan. */
fftoc_status fftoc_exec_twiddles(int n, int engine, const int radix[4], const void **table);

/* Device-side error flags of the current device, those of every entry point
 * including fftoc_c2c_fwd_host_noalloc: FFTOC_ERR_TIMEOUT if a persistent
 * kernel's bounded wait for a prefetched tile gave up since the last check
 * (its outputs are then incomplete), FFTOC_ERR_INVALID_VALUE if an uneven
 * batch skipped entries (bad size or negative offset), FFTOC_OK otherwise.
 * Clears the flags.  Synchronous; allocates nothing (and creates no device
 * state of the library). */
fftoc_status fftoc_device_error_check(void);

/* Self-test of the failure path of the bounded device waits: one CTA waits
 * on an mbarrier that nothing arrives on, gives up after limit_ms (0 < limit_ms
 * <= 1000), raises the device error flag and returns; a following
 * fftoc_device_error_check() reports FFTOC_ERR_TIMEOUT.  Asynchronous on
 * `stream`.  (The persistent, split and exact kernels take the same path when
 * a wait for a copy or an MMA does not complete in 2 s.) */
fftoc_status fftoc_selftest_bounded_wait(double limit_ms, fftoc_stream stream);

/* Engine that FFTOC_ENGINE_AUTO resolves to for size n. */
int fftoc_auto_engine(int n);

/* Messages. */
const char *fftoc_status_string(fftoc_status status);
const char *fftoc_last_error_string(void);
int fftoc_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FFTOC_H */
