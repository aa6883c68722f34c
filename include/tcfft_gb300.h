/*
 * tcfft_gb300.h -- C ABI of the GB300 (sm_103a) half-precision FFT library.
 *
 * This is the drop-in boundary for the reference's plan API (rox906/tcFFT):
 *
 *   reference (C++ linkage, tcfft_half.h:20-21, tcfft_half_2d.h:20-21)
 *     void tcfftCreate(tcfftHandle *plan, int n, int n_batch);
 *     void tcfftCreate(tcfftHandle *plan, int nx, int ny, int n_batch);
 *     void tcfftExec(tcfftHandle plan, half *data);
 *     (no destroy function; errors are undefined behaviour)
 *
 *   this library (extern "C", plain pointers and sizes, status codes)
 *     tcfftPlan1d / tcfftPlan2d / tcfftPlanMany   <- tcfftCreate
 *     tcfftExecute                                <- tcfftExec
 *     tcfftDestroy                                (new: the reference leaks)
 *
 * Semantics kept from the reference (tcfft_doit_half.cpp:31-67):
 *   - `data` is a device pointer owned by the caller, interleaved complex
 *     (re, im), batch-major contiguous: [batch][n] (1D), [batch][nx][ny] (2D,
 *     row-major, ny contiguous);
 *   - the transform is in place, unnormalised, forward sign -1 (the reference
 *     builds F = exp(-2 pi i jk/16), tcfft_half.cu:1339);
 *   - execution is asynchronous on the given stream (the reference uses the
 *     default stream; pass 0 for the same behaviour).
 * Additions: status codes, stream argument, natural input order by default
 * (the reference expects digit-reversed input, tcfft_doit_half.cpp:38-46;
 * TCFFT_ORDER_REFERENCE_DIGIT_REVERSED reproduces that contract), split
 * precision, the adjoint transform, uneven batches, host-buffer execution.
 *
 * Threads: a plan keeps per-plan device state (scratch, counters, tensor maps
 * of the last data pointer, lazily built sub-plans), so calls on one plan from
 * several host threads must be serialised by the caller; different plans are
 * independent.
 */
#ifndef TCFFT_GB300_H
#define TCFFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tcfftStatus {
  TCFFT_SUCCESS = 0,
  TCFFT_INVALID_VALUE = 1,  /* null pointer, bad option value */
  TCFFT_INVALID_SIZE = 2,   /* unsupported n / nx / ny / batch */
  TCFFT_MISALIGNED = 3,     /* data pointer not 128-byte aligned */
  TCFFT_ALLOC_FAILED = 4,   /* device or host allocation failed */
  TCFFT_CUDA_ERROR = 5,     /* a CUDA runtime/driver call failed */
  TCFFT_TIMEOUT = 6,        /* a bounded device-side wait expired */
  TCFFT_NOT_SUPPORTED = 7,  /* valid request this build does not implement */
  TCFFT_INVALID_PLAN = 8    /* null or already destroyed plan */
} tcfftStatus;

typedef enum tcfftPrecision {
  /* fp16 complex in/out (4 bytes per element), fp16 tensor-core operands with
   * fp32 accumulation, fp16 between passes. Same data type as the reference. */
  TCFFT_PRECISION_PLAIN = 0,
  /* fp32 complex in/out (8 bytes per element); every tensor-core product is
   * split into hi+lo fp16 pairs (hi*hi + hi*lo + lo*hi, fp32 accumulation),
   * fp32 twiddles and fp32 storage between passes. */
  TCFFT_PRECISION_SPLIT = 1,
  /* fp32 complex in/out (8 bytes per element, e.g. complex64 tensors), fp16
   * tensor-core operands with fp32 accumulation: the fp32 -> fp16 conversion
   * is fused into the kernels' shared-memory reads and the results are stored
   * from the fp32 accumulators (fp32 between passes).  Plain arithmetic on
   * fp32 data: the schedules and HBM traffic of TCFFT_PRECISION_SPLIT, one
   * tensor-core product per stage instead of three. */
  TCFFT_PRECISION_FP32_IO = 2
} tcfftPrecision;

typedef enum tcfftInputOrder {
  TCFFT_ORDER_NATURAL = 0,
  /* input permuted by the reference's digit-reversal (gen_rev with the
   * reference's radix chain, tcfft_doit_half.cpp:6-29); output natural. Only
   * for sizes the reference supports. */
  TCFFT_ORDER_REFERENCE_DIGIT_REVERSED = 1
} tcfftInputOrder;

typedef enum tcfftDirection {
  /* sign -1: X[k] = sum_n x[n] exp(-2 pi i n k / N), the reference's transform
   * (F = exp(-2 pi i jk/16), tcfft_half.cu:1339) */
  TCFFT_FORWARD = 0,
  /* sign +1: the conjugate direction */
  TCFFT_INVERSE = 1
} tcfftDirection;

typedef enum tcfftNormalization {
  TCFFT_NORM_NONE = 0,   /* unnormalised, as the reference */
  TCFFT_NORM_BY_N = 1    /* every transform scaled by 1/N (N = n, or nx * ny in 2D) */
} tcfftNormalization;

typedef struct tcfftOptions {
  int32_t precision;   /* tcfftPrecision */
  int32_t input_order; /* tcfftInputOrder */
  int32_t autotune;    /* 0: built-in schedule; 1: time candidates at plan time */
  int32_t direction;   /* tcfftDirection of tcfftExecute (default TCFFT_FORWARD) */
  const char* tune_cache_path; /* optional file for autotune results (NULL: none) */
  int32_t normalization; /* tcfftNormalization of tcfftExecute (default TCFFT_NORM_NONE) */
  int32_t reserved;
} tcfftOptions;

typedef struct tcfftPlanImpl* tcfftPlan;

/* Fill `opts` with defaults (plain, natural order, no autotune, forward,
 * unnormalised). */
tcfftStatus tcfftOptionsDefault(tcfftOptions* opts);

/* 1D batched plan: `batch` transforms of length n (power of two, 16 <= n <= 2^27;
 * the split precision stops at n = 64 below 256). The reference plans ten sizes
 * (tcfft_half.cu:1250-1330: 2^8..2^10, 2^17..2^19, 2^24..2^27); all of them are
 * included. */
tcfftStatus tcfftPlan1d(tcfftPlan* plan, int64_t n, int64_t batch, const tcfftOptions* opts);

/* 2D batched plan: `batch` transforms of nx x ny (powers of two, each a valid
 * 1D size). Axes 256..2048 run fused (one HBM round trip); other shapes are
 * composed from 1D plans and transposes. */
tcfftStatus tcfftPlan2d(tcfftPlan* plan, int64_t nx, int64_t ny, int64_t batch, const tcfftOptions* opts);

/* Strided layouts (cuFFT's "advanced layout" for one dimension): `batch`
 * transforms of n points, point j of transform b at element
 *   istride == 1:  b * idist + j            (batch stride; idist >= n, and
 *                                            idist * element bytes a multiple of 128)
 *   istride  > 1:  (b / istride) * n * istride + j * istride + b % istride
 *                  (idist must be 1: istride transforms interleaved, i.e. the FFT
 *                   along the middle axis of a [batch / istride][n][istride] array)
 * The first form is an uneven-batch plan (tcfftPlanMany) with those offsets. The
 * second is plain precision only, without normalisation, n = 128..2048, with
 * istride a multiple of 128 / 32 / 32 / 16 / 8 for n = 128 / 256 / 512 / 1024 / 2048
 * (TCFFT_NOT_SUPPORTED otherwise); it runs as one launch of column FFTs.  No
 * counterpart in the reference (contiguous batches only). */
tcfftStatus tcfftPlanStrided(tcfftPlan* plan, int64_t n, int64_t batch, int64_t istride, int64_t idist,
                             const tcfftOptions* opts);

/* Uneven batch in one launch: `count` independent transforms, transform i has
 * rank ranks[i] (1 or 2), shape (nx[i]) for 1D or (nx[i], ny[i]) for 2D, and
 * starts at element offset offsets[i] of the single device buffer passed to
 * tcfftExecute (in elements; must keep 128-byte alignment). */
tcfftStatus tcfftPlanMany(tcfftPlan* plan, int64_t count, const int32_t* ranks, const int64_t* nx,
                          const int64_t* ny, const int64_t* offsets, const tcfftOptions* opts);

/* The plan's transform (by default forward, unnormalised) in place on device
 * memory `data` on `stream` (a cudaStream_t; NULL = legacy default stream). */
tcfftStatus tcfftExecute(tcfftPlan plan, void* data, void* stream);

/* Adjoint of tcfftExecute: the conjugate direction with the same scale (for
 * the default plan: unnormalised, i.e. N times the inverse DFT), same layout
 * and schedule. */
tcfftStatus tcfftExecuteAdjoint(tcfftPlan plan, void* data, void* stream);

/* Inverse of tcfftExecute: the conjugate direction scaled so that
 * tcfftExecuteInverse(tcfftExecute(x)) = x (for the default plan: the inverse
 * DFT with its 1/N).  The 1/N is folded into a twiddle multiply the kernels
 * already make, so it costs no extra pass over the data, and intermediate
 * values stay within fp16 range.  The reference has no inverse (its kernels
 * use only the exp(-2 pi i jk/N) twiddles). */
tcfftStatus tcfftExecuteInverse(tcfftPlan plan, void* data, void* stream);

/* tcfftExecute with a separate input: `in` (not modified) is transformed into
 * `out`; both device memory of the plan's size and layout, 128-byte aligned,
 * not overlapping (in == out is tcfftExecute).  The 1D schedules of up to
 * 2^22 points (and the composite 1D ones) read `in` directly, so the
 * out-of-place call moves no more data than the in-place one; 2D, uneven-batch
 * and reference-order plans copy `in` to `out` first.  The reference's
 * tcfftExec is in place only (tcfft_half.h:20). */
tcfftStatus tcfftExecuteOutOfPlace(tcfftPlan plan, const void* in, void* out, void* stream);

/* Real 1D transforms (no counterpart in the reference): `batch` sequences of n
 * real values (power of two, 32 <= n <= 2^27), fp16 (TCFFT_PRECISION_PLAIN) or
 * fp32 (TCFFT_PRECISION_SPLIT), contiguous [batch][n], and their Hermitian
 * halves, n/2 + 1 complex values each, [batch][n/2 + 1] (interleaved, half2 /
 * float2).  Computed as complex transforms of n/2 points plus one pass that
 * splits (or, for C2R, merges) the even and odd spectra.  C2R is the inverse of
 * R2C (c2r(r2c(x)) = x): with TCFFT_NORM_NONE (default) R2C is unnormalised and
 * C2R carries the 1/n (numpy's rfft / irfft), with TCFFT_NORM_BY_N R2C carries
 * it and C2R is unnormalised.  Options: precision, normalization, autotune;
 * direction must be TCFFT_FORWARD and input order natural. */
tcfftStatus tcfftPlanReal1d(tcfftPlan* plan, int64_t n, int64_t batch, const tcfftOptions* opts);
/* Real 2D transforms: `batch` real nx x ny arrays [batch][nx][ny] (powers of
 * two, nx >= 16, ny >= 32; the split precision has no 128-point complex
 * transform, so it takes neither nx = 128 nor ny = 256) and their halves
 * [batch][nx][ny/2 + 1] (numpy's rfft2 / irfft2 layout), same precisions,
 * options and normalisation rule as tcfftPlanReal1d (the 1/(nx ny) on C2R by
 * default).  Rows as real 1D transforms, columns as complex 1D transforms of
 * the transposed half spectrum; both calls use tcfftExecuteR2C / C2R. */
tcfftStatus tcfftPlanReal2d(tcfftPlan* plan, int64_t nx, int64_t ny, int64_t batch, const tcfftOptions* opts);
/* X = DFT(x) (sign -1; times 1/n with TCFFT_NORM_BY_N), the n/2 + 1
 * non-redundant values; `in` is not modified. */
tcfftStatus tcfftExecuteR2C(tcfftPlan plan, const void* in, void* out, void* stream);
/* x[j] = c * sum over the full Hermitian spectrum of X[k] exp(+2 pi i jk/n),
 * c = 1/n (TCFFT_NORM_NONE) or 1 (TCFFT_NORM_BY_N); the imaginary parts of
 * X[0] and X[n/2] are ignored; `in` is not modified. */
tcfftStatus tcfftExecuteC2R(tcfftPlan plan, const void* in, void* out, void* stream);

/* Host-buffer execution: the batch is copied in from `host_in`, transformed
 * (forward) in the caller's device buffer `work` (the plan's size, 128-byte
 * aligned) and copied out to `host_out`, pipelined over chunks of the batch on
 * internal streams (host-to-device copy of chunk c+1, transform of chunk c and
 * device-to-host copy of chunk c-1 overlap).  Ordered after the work already in
 * `stream`; work queued in `stream` afterwards waits for the whole call.
 * host_in and host_out should be pinned (cudaHostAlloc / cudaHostRegister) for
 * the copies to be asynchronous; host_out may equal host_in.  Uneven-batch plans
 * run unchunked (copy in, execute, copy out on `stream`).  No counterpart in the
 * reference, whose tcfftExec takes device memory only. */
tcfftStatus tcfftExecuteHost(tcfftPlan plan, const void* host_in, void* host_out, void* work, void* stream);

/* Synchronise `stream` and report device-side errors (TCFFT_TIMEOUT) raised
 * by bounded waits since the last check; clears the flag. */
tcfftStatus tcfftCheckDevice(tcfftPlan plan, void* stream);

/* Limit, in nanoseconds, of every bounded device-side wait of this plan's
 * two-phase kernels (the cross-CTA completion counters and the shared-memory
 * ring barriers, and those of the one-launch uneven-batch plans); 0 restores the
 * default of 2 s.  A wait that runs out stops
 * its kernel early and raises the flag tcfftCheckDevice reports as
 * TCFFT_TIMEOUT.  Applies to the plan's sub-plans too.  No counterpart in the
 * reference, whose kernels never wait on one another. */
tcfftStatus tcfftSetWaitLimit(tcfftPlan plan, int64_t limit_ns);

/* Test hook for the timeout path: the next execute of this plan starts with
 * one completion counter preset (on the host, before the launch) to a value
 * that no number of completed tiles raises to its target, so the waits on it
 * run out after the wait limit and tcfftCheckDevice returns TCFFT_TIMEOUT.
 * Nothing faults; the output of that one execute is undefined, later executes
 * are unaffected.  Two-phase schedules and the one-launch uneven-batch plans of
 * tcfftPlanMany with a transform of two passes (others: TCFFT_NOT_SUPPORTED). */
tcfftStatus tcfftInjectWaitTimeout(tcfftPlan plan);

tcfftStatus tcfftDestroy(tcfftPlan plan);

const char* tcfftGetErrorString(tcfftStatus status);

/* Plan introspection: element count per transform set (sum over the batch),
 * bytes per element (4 plain / 8 split), scratch bytes, number of kernel
 * launches per execute, and the reference-compatible radix chain (up to
 * `max_radices` entries; 2D: x then y) used for
 * TCFFT_ORDER_REFERENCE_DIGIT_REVERSED. */
typedef struct tcfftPlanInfo {
  int64_t total_elements;
  int32_t element_bytes;
  int32_t launches_per_exec;
  int64_t scratch_bytes;
  int32_t n_radices;
  int32_t radices[16];
  int32_t n_radices_y;
  int32_t radices_y[16];
  char schedule[128];
} tcfftPlanInfo;
tcfftStatus tcfftGetPlanInfo(tcfftPlan plan, tcfftPlanInfo* info);

/* Describe the schedule for a 1D size without touching the GPU (host-only
 * planner; used by CPU tests). Writes a short text into buf. */
tcfftStatus tcfftDescribe1d(int64_t n, int64_t batch, int32_t precision, char* buf, size_t buf_len);

/* The same for a 2D shape [batch][nx][ny]: the fused 2D kernel for axes of 256..2048 (split and
 * fp32 I/O: up to 1024), else rows, transpose, rows, transpose through 1D plans. */
tcfftStatus tcfftDescribe2d(int64_t nx, int64_t ny, int64_t batch, int32_t precision, char* buf, size_t buf_len);

/* Diagnostics, host only (no GPU): the work items of the one-launch many-shape executor for the
 * transforms of a tcfftPlanMany call (plain precision) on a GPU with num_sms SMs, in launch
 * order.  Writes min(capacity, *n_items) items, six int32 each, into `items`:
 *   kind      bits 0-7 the work kind; 0x100 a group of listed 1D transforms (N <= 2048, one pass);
 *             0x200 a pass-B item; 0x400 a pass-A item (it releases its transform's pass B)
 *   xf        the transform (pass A / B), or the group's first entry in the listed transforms
 *   tile      the first tile of the transform's pass
 *   count     listed: transforms in the group; pass B: pass-A items of the transform
 *   tiles     consecutive tiles in the item
 *   elements  complex elements the item covers
 * TCFFT_NOT_SUPPORTED when a shape is not one the executor runs (the plan then replays its
 * per-shape graph). */
tcfftStatus tcfftDescribeManyItems(int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                                   const int64_t* offsets, int32_t num_sms, int32_t* items, int64_t capacity,
                                   int64_t* n_items);

/* Library version string. */
const char* tcfftVersion(void);

/* Allocation-free 1D execute (no counterpart in the reference).
 *
 * For callers that cannot call cudaMalloc when they run an FFT: code inside a
 * CUDA stream capture that must not add allocation nodes, runtimes or plug-in
 * hosts that own all device memory, or callbacks that run while a memory
 * pool is locked.  Runs the same two-phase kernel as a tcfftPlan1d plan, in
 * place on `data` ([batch][n] interleaved complex, device memory, 128-byte
 * aligned), forward (direction 0) or adjoint (direction 1), on `stream`.
 *
 * It allocates nothing: its scratch ring, twiddle tables and completion
 * counters live in fixed `static __device__` arrays (32 MiB of scratch, about
 * 32.2 MiB in all) that every GPU loading this library holds until the
 * process exits.  Limits: n a power of two, 2^12 <= n <= 2^21 for
 * TCFFT_PRECISION_PLAIN and <= 2^20 for TCFFT_PRECISION_SPLIT; other sizes
 * return TCFFT_INVALID_SIZE (use a plan).
 *
 * All calls share the arrays and leave the last call's contents in them;
 * each call rewrites its tables and clears its counters on `stream` first, so
 * calls ordered on one stream are independent, but calls that overlap on the
 * GPU (different streams or host threads) race and must not be issued
 * concurrently.  The first call on a device looks up the arrays' device
 * addresses (cudaGetSymbolAddress); make it before any stream capture.
 *
 * A bounded device-side wait that runs out (2 s) stops the kernel early and
 * sets a flag in the static arrays; tcfftCheckDeviceNoAlloc reads it. */
tcfftStatus tcfftExecute1dNoAlloc(void* data, int64_t n, int64_t batch, int32_t precision, int32_t direction,
                                  void* stream);

/* Status of the allocation-free entry point on the current device:
 * synchronises `stream`, then returns TCFFT_TIMEOUT (and clears the flag) if a
 * bounded wait of any tcfftExecute1dNoAlloc call since the last check ran out,
 * else TCFFT_SUCCESS.  Allocates nothing (the flag is read with
 * cudaMemcpyFromSymbol).  No counterpart in the reference. */
tcfftStatus tcfftCheckDeviceNoAlloc(void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TCFFT_GB300_H */
