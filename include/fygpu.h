/*
 * fygpu.h -- C ABI of the GB300 (sm_103a) 1D complex FFT library (libfygpu.so).
 *
 * Drop-in GPU path for fyFFT's plan/execute API (kjear/fyFFT, foye_FFT.hpp).  Every function
 * returns an int status (FYG_OK == 0); fyg_last_error_string() describes the last failure on
 * the calling thread.  Plain pointers and sizes only: streams are passed as void* holding a
 * cudaStream_t (NULL = the legacy default stream).
 *
 * Data layout: interleaved complex, `dtype` FYG_C32 (re,im float pairs, the reference's
 * `float*` buffers) or FYG_C64 (double pairs).  Forward is exp(-2 pi i kn/N); inverse is
 * exp(+2 pi i kn/N) scaled by 1/N, as in the reference (e.g. src/foye_FFT_radix2.hpp:669-672).
 *
 * Threading: a plan is not thread-safe (it owns mutable scratch, like the reference's
 * mixed-radix, Rader and Bluestein plans); use one plan per host thread or serialize calls.
 */
#ifndef FYGPU_H_
#define FYGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FYG_OK 0
#define FYG_ERR_INVALID_LENGTH 1
#define FYG_ERR_NULL_PTR 2
#define FYG_ERR_MISALIGNED 3
#define FYG_ERR_ALLOC 4
#define FYG_ERR_CUDA 5
#define FYG_ERR_TIMEOUT 6
#define FYG_ERR_INVALID_ARG 7
#define FYG_ERR_UNSUPPORTED 8

/* element types */
#define FYG_C32 0
#define FYG_C64 1

/* directions */
#define FYG_FORWARD 1
#define FYG_INVERSE (-1)

/* execution strategies, numbered like fy::fft::FFT1D_C2C_invoker::FFT_execution_strategy
 * (foye_FFT.hpp:153-160) */
#define FYG_STRATEGY_KERNEL_DIRECT 0
#define FYG_STRATEGY_MIX_RADIX 1
#define FYG_STRATEGY_RADER 2
#define FYG_STRATEGY_BLUESTEIN 3
#define FYG_STRATEGY_DFT 4

/* plan flags */
#define FYG_FLAG_CONV_FP64 0x1   /* Rader/Bluestein convolution in FP64 even for FYG_C32 data */
#define FYG_FLAG_CONV_FP32 0x2   /* force the FP32 convolution (disables the error-budget choice) */
#define FYG_FLAG_NO_L2_CHUNK 0x4 /* process the whole batch per pass (no L2-resident chunking) */
#define FYG_FLAG_SMALL_TILES 0x8 /* single-CTA transforms up to ~100 KB of shared memory, stage radix <= 16 */
#define FYG_FLAG_AUTOTUNED 0x10  /* use the autotuner's cached schedule for this length, if any */
#define FYG_FLAG_GENERIC_KERNELS 0x20 /* only the generic tile kernel (no register-resident
                                       * power-of-two kernels); for comparisons */
#define FYG_FLAG_WIDE_TILES 0x40 /* register-resident passes in 512-thread CTAs with twice the
                                  * columns (wider contiguous row segments); chosen per length by
                                  * the autotuner */
#define FYG_FLAG_TMA_LOADS 0x80  /* every register-resident pass after the first loads its tiles
                                  * with TMA tensor copies (cp.async.bulk.tensor) into shared
                                  * memory; by default only 4-column tiles do (measured faster
                                  * there, slower on wider tiles) */
#define FYG_FLAG_NO_TMA_LOADS 0x100 /* per-thread loads everywhere (comparisons) */
#define FYG_FLAG_BATCH_BRANCHES 0x200 /* uneven batches: one plan per distinct length (register-
                                       * resident kernels where they apply) as parallel chains of
                                       * one CUDA graph instead of the persistent kernel; the batch
                                       * autotuner measures both forms */

typedef struct fyg_plan fyg_plan;
typedef struct fyg_batch fyg_batch;
typedef struct fyg_multi fyg_multi;

/* Creates a plan for `batch` contiguous transforms of length n (n >= 1).
 * Replaces fy::fft::FFT1D_C2C_invoker::FFT1D_C2C_invoker(std::size_t) (foye_FFT.hpp:101-126):
 * the constructor's strategy choice and table/workspace set-up happen here, once. */
int fyg_plan_create(size_t n, int dtype, size_t batch, int flags, fyg_plan** out);

/* fyg_plan_create with schedule overrides (0 = the planner's default): max_pass_radix caps the
 * radix of every multi-pass step; conv_length sets the Rader/Bluestein convolution length
 * (Bluestein: 7-smooth >= 2N-1; Rader: N-1 when 13-smooth, or 7-smooth >= 2N-3).  Used by the
 * autotuner; no counterpart in the reference. */
int fyg_plan_create_ex(size_t n, int dtype, size_t batch, int flags, size_t max_pass_radix,
                       size_t conv_length, fyg_plan** out);

/* Autotuner (no counterpart in the reference): times candidate schedules for one length on the
 * current device -- convolution lengths (Rader/Bluestein), caps on the pass radix (multi-pass),
 * transforms per CTA (single-pass, i.e. threads per transform) -- and stores the fastest in the
 * JSON cache at `cache_path` (NULL: $FYG_AUTOTUNE_CACHE, else ~/.cache/fyfft_gb300/autotune.json),
 * keyed by device name, SM count, compute capability and driver.  `batch` is the batch the
 * candidates are timed with.  Plans created with FYG_FLAG_AUTOTUNED use the cached choice.
 * *best_ms (optional) receives the winner's time per forward batch. */
int fyg_autotune(size_t n, int dtype, size_t batch, const char* cache_path, double* best_ms);

/* The current device's key in autotune caches: "name|SM count|compute capability|driver". */
int fyg_device_signature(char* buf, size_t len);

/* Releases the plan and its device tables and scratch. */
int fyg_plan_destroy(fyg_plan* plan);

/* Process-wide table cache.  Plans share their read-only device tables (twiddles, chirps,
 * Rader index maps, convolution spectra, thread-order tables) through a cache keyed by device
 * and content, so creating a second plan of a length (or the autotuner's candidates) reuses
 * them; each plan keeps only its scratch.  Replaces the reference's process-wide registry of
 * length -> engine with static tables (src/foye_FFT_radix_wrap.hpp:81-85).
 * fyg_plan_cache_stats: entries, device bytes held, lookups that hit and missed.
 * fyg_plan_cache_clear: frees the tables no live plan uses (safe at any time). */
int fyg_plan_cache_stats(size_t* entries, size_t* bytes, uint64_t* hits, uint64_t* misses);
int fyg_plan_cache_clear(void);

/* Runs the batch: direction FYG_FORWARD or FYG_INVERSE (1/N).  `in` and `out` are device
 * pointers, or host pointers (staged through device buffers and synchronized before return).
 * in == out (in place) is allowed.
 * Replaces fy::fft::FFT1D_C2C_invoker::dispatch<bool invert>(const float*, float*)
 * (foye_FFT.hpp:128-151); the reference runs one transform per call. */
int fyg_execute(fyg_plan* plan, const void* in, void* out, int direction, void* stream);

/* As fyg_execute, but host buffers do not block: the call enqueues the staged copies and kernels
 * and returns.  Large host batches copy out on the plan's own copy-out stream: the output is in
 * host memory after fyg_plan_join(plan, s) and a synchronize of s (or a device synchronize);
 * do not read `out` or reuse `in` before.  The host input is read without waiting for earlier
 * work on `stream`, so it must be ready at the call; pinned host memory makes the copies
 * asynchronous.  Consecutive calls of different plans overlap one plan's copies with another's
 * kernels, and the copies of one host thread's calls run in call order.  Device buffers:
 * identical to fyg_execute.  No counterpart in the reference (its dispatch is synchronous). */
int fyg_execute_async(fyg_plan* plan, const void* in, void* out, int direction, void* stream);

/* Makes `stream` wait for the copy-outs of the plan's asynchronous host executions. */
int fyg_plan_join(fyg_plan* plan, void* stream);

/* Adjoint (conjugate transpose) of the forward transform, times `scale`:
 * out = scale * F^H g = scale * N * dispatch<true>(g).  No counterpart in the reference; its
 * backward transform scaled by N is the reference gradient it is checked against. */
int fyg_execute_adjoint(fyg_plan* plan, const void* g, void* out, double scale, void* stream);

/* Strategy the reference would choose for n: fy::fft::FFT1D_C2C_invoker::
 * acquired_execution_strategy(std::size_t) (foye_FFT.hpp:162-184).  Returns -1 for n < 2. */
int fyg_strategy(size_t n);

/* Strategy this library runs for n (never FYG_STRATEGY_DFT). */
int fyg_gpu_strategy(size_t n);

/* Plan introspection: algorithm length (conv length M for Rader/Bluestein, p - 1 for the
 * N = m p split), number of kernel passes per direction, and the GPU strategy (0 single pass,
 * 1 multi-pass, 2 Rader, 3 Bluestein, 4 copy for N = 1, 5 the N = m p split: a pass of
 * length-m DFTs ahead of m Rader transforms of the prime p). */
int fyg_plan_info(const fyg_plan* plan, size_t* conv_length, int* passes, int* strategy);

/* The schedule fyg_plan_create chooses for n with these flags, computed on the host (no GPU
 * needed; FYG_FLAG_AUTOTUNED is ignored): the strategy (numbered as fyg_plan_info reports it),
 * the algorithm length L (n, the convolution length, or p - 1 for the N = m p split), the split
 * factor m (1 when there is none) and the radices of the passes of the length-L transform (up
 * to max_passes written; the pass count in *npasses).  A Rader or Bluestein plan runs 2P - 1
 * kernels for P passes (the last forward and the first inverse pass share one), the split one
 * more.  Any output pointer may be NULL. */
int fyg_plan_schedule(size_t n, int dtype, int flags, int* strategy, size_t* conv_length, int* split_m,
                      int* pass_radices, int max_passes, int* npasses);

/* Device-side error bits the plan's kernels recorded since the last call (synchronizes the
 * stream, then clears them): 1 = a stage radix the kernel was not compiled for, 4 = a TMA tile
 * load that did not complete within its bounded wait.  0 = no error.  Kernels record such
 * conditions instead of trapping, so the context stays usable. */
int fyg_plan_status(fyg_plan* plan, void* stream, int* status);

/* Plan whose user buffers hold the batch's transforms `idist` (input) and `odist` (output)
 * elements apart (0 = n, contiguous; otherwise >= n).  The elements between transforms are
 * neither read nor written, for device and host buffers alike.  In-place execution needs
 * idist == odist.  No counterpart in the reference (one contiguous transform per call). */
int fyg_plan_create_layout(size_t n, int dtype, size_t batch, size_t idist, size_t odist, int flags, fyg_plan** out);

/* Kernel launches one fyg_execute of this plan issues (passes x L2 chunks). */
int fyg_plan_launches(const fyg_plan* plan, int* launches);

/* Plan introspection (no counterpart in the reference): one text line per forward pass with
 * its kernel ("fast" = register-resident power-of-two kernel, "generic" = shared-memory tile
 * kernel), tile length R, columns per tile C, threads, shared memory, Ns, Ns_out and the
 * load/store fusions.  FYG_ERR_INVALID_ARG if `len` is too small. */
int fyg_plan_describe(const fyg_plan* plan, char* buf, size_t len);

/* Instrumentation (no counterpart in the reference): when enabled, every pass launch of
 * fyg_execute is bracketed by CUDA events on the execution stream and its duration is
 * accumulated per pass.  fyg_plan_profile_read synchronizes, then reports for each of up to
 * max_passes passes of the forward pipeline: total milliseconds, launch count and the
 * algorithmic bytes one launch moves (elements read + elements written, times element size). */
int fyg_plan_profile(fyg_plan* plan, int enable);
int fyg_plan_profile_read(fyg_plan* plan, double* total_ms, int64_t* launches, int64_t* bytes_per_launch,
                          int max_passes, int* n_passes);

/* Uneven batch: `count` transforms with the given lengths, packed back to back (element
 * offsets given at execute time).  One persistent kernel runs them all from a device work
 * queue.  No counterpart in the reference (it runs one transform per call). */
int fyg_batch_create(const size_t* lengths, size_t count, int dtype, int flags, fyg_batch** out);

/* Measured schedule of an uneven batch (no counterpart in the reference): times the
 * persistent launch of this length sequence under each group-plan option set (stage-radix cap
 * 16 / 32, single-pass tile cap 48 / 100 / 160 KB of shared memory) on random device data and
 * caches the fastest in the autotune cache (see fyg_autotune) under a key made of the element
 * type and a hash of the lengths.  fyg_batch_create with FYG_FLAG_AUTOTUNED uses it.  FYG_C32
 * only.  *best_ms (optional) receives the winner's milliseconds per forward execution. */
int fyg_batch_autotune(const size_t* lengths, size_t count, int dtype, const char* cache_path, double* best_ms);

/* fyg_batch_create with an explicit execution form (what the batch autotuner chooses between):
 * form 0: one persistent kernel over a device work queue (stage radix cap 16 or 32, single-pass
 * tiles up to single_tile_kb KB of shared memory; 0 = defaults); form 1: one plan per distinct
 * length (register-resident kernels where they apply) as up to 32 parallel chains of one CUDA
 * graph;
 * form 2: lengths up to `split` in the persistent kernel, longer ones as graph chains, both in
 * one graph.  FP64 batches always run form 1. */
int fyg_batch_create_ex(const size_t* lengths, size_t count, int dtype, int flags, int form, size_t split,
                        int radix_cap, int single_tile_kb, fyg_batch** out);
int fyg_batch_destroy(fyg_batch* batch);

/* offsets_dev: device array of `count` int64 element offsets (NULL: packed back to back in the
 * order given).  in/out device pointers.  The work is a CUDA graph captured on the first call
 * with each (direction, in, out, offsets_dev) and replayed on later calls with the same four;
 * the batch keeps every graph it captured until fyg_batch_destroy. */
int fyg_batch_execute(fyg_batch* batch, const void* in, void* out, const int64_t* offsets_dev,
                      int direction, void* stream);

/* Waits for the batch's last fyg_batch_execute on `stream` and reports its device status:
 * FYG_OK, or FYG_ERR_TIMEOUT when a work item waited longer than the batch's wait limit for
 * the pass it depends on (the kernel then abandons the run and returns; the context stays
 * usable). */
int fyg_batch_status(fyg_batch* batch, void* stream);

/* Test hook (host-side fault injection): with enable != 0, the completion count of the first
 * pass another pass waits for becomes unreachable, so the next fyg_batch_execute gives up
 * after `timeout_ms` and fyg_batch_status reports FYG_ERR_TIMEOUT; enable == 0 restores the
 * batch.  No counterpart in the reference. */
int fyg_batch_inject_stall(fyg_batch* batch, int enable, int timeout_ms);

/* Same batch, one launch sequence per transform (the plain one-plan-per-launch path). */
int fyg_batch_execute_plain(fyg_batch* batch, const void* in, void* out, int direction,
                            void* stream);

/* Batch sharding across devices (no collective: transforms are independent; the reference runs
 * one transform per dispatch<>() call, foye_FFT.hpp:128-151, and its plans are one per thread).
 * fyg_partition: contiguous shards of near-equal cost -- bounds[0..parts] with bounds[0] = 0 and
 * bounds[parts] = count; lengths == NULL for a uniform batch (equal counts), else cost
 * n log2 n per transform.  The same split serves one process per device (each rank runs
 * [bounds[rank], bounds[rank+1])) and fyg_multi_create, one plan and stream per device.
 * fyg_multi_execute: host buffers of the whole batch, every shard staged to its device by its
 * own host thread; returns when all outputs are in host memory.
 * fyg_multi_execute_device: ins[i] / outs[i] hold shard i on devices[i]; asynchronous,
 * fyg_multi_synchronize waits.  A device may appear more than once. */
int fyg_partition(const size_t* lengths, size_t count, int parts, size_t* bounds);
int fyg_multi_create(size_t n, int dtype, size_t batch, int flags, const int* devices, int ndev, fyg_multi** out);
int fyg_multi_shards(const fyg_multi* multi, int* ndev, size_t* bounds);
int fyg_multi_execute(fyg_multi* multi, const void* in, void* out, int direction);
int fyg_multi_execute_device(fyg_multi* multi, const void* const* ins, void* const* outs, int direction);
int fyg_multi_synchronize(fyg_multi* multi);
int fyg_multi_destroy(fyg_multi* multi);

/* Allocation-free transform: no counterpart in the reference.  For callers that cannot call
 * cudaMalloc: a host application that owns all device memory and gives a plugin only its input
 * and output buffers (an allocation inside the plugin could fail or break its memory budget),
 * and a loop with a latency budget that cannot take the device-wide synchronization cudaMalloc
 * or cudaFree may cause.  Runs `batch` contiguous transforms of a 13-smooth length n with the
 * multi-pass kernel; its scratch and twiddle tables live in a fixed 20 MiB file-scope device
 * array (held by every GPU that loads the library until exit).  Limit: n * batch * element
 * size <= 16 MiB (half that when n needs three or more passes); larger sizes return
 * FYG_ERR_INVALID_LENGTH.  in/out must be device pointers of the current device; nothing is
 * allocated and nothing is copied from the host: the twiddle tables are computed on the device
 * into the array when n or the type differs from the previous call's.  The first call on a
 * device does a one-time set-up (the array's address via cudaGetSymbolAddress and the codelet
 * constants, both synchronous), so make it before any stream capture.  All calls share the
 * array, which keeps the last call's contents: calls that overlap on the GPU race. */
int fyg_execute_noalloc(size_t n, size_t batch, int dtype, int direction, const void* in, void* out,
                        void* stream);

/* Last error on the calling thread ("" if none). */
const char* fyg_last_error_string(void);

/* Seeded synthetic data (host, no GPU): counter-based splitmix64 stream; dist 0 = uniform
 * [-1, 1), 1 = standard normal (Box-Muller).  n_complex complex elements of `dtype` written
 * to `out` (re then im per element); element i depends only on (seed, i). */
int fyg_fill_random(uint64_t seed, int dist, int dtype, size_t n_complex, void* out);

/* Same stream generated on the device into device memory. */
int fyg_fill_random_device(uint64_t seed, int dist, int dtype, size_t n_complex, void* out,
                           void* stream);

/* Elements [first, first + n_complex) of the same stream (a shard of a larger batch), on the
 * host or on the device. */
int fyg_fill_random_at(uint64_t seed, int dist, int dtype, size_t first, size_t n_complex, void* out);
int fyg_fill_random_device_at(uint64_t seed, int dist, int dtype, size_t first, size_t n_complex, void* out,
                              void* stream);

/* Library version string. */
const char* fyg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FYGPU_H_ */
