// tcfft_noalloc.cu -- execute a 1D batched FFT without allocating anything.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they
// run an FFT -- code running inside a CUDA stream capture that must not add
// allocation nodes, allocator-less embedded runtimes, plug-in hosts that own
// all device memory, or callbacks that run while a memory pool is locked.
// tcfftPlan1d allocates twiddle tables, completion counters and the scratch
// ring of the two-phase kernel; this entry point instead uses file-scope
// `static __device__` arrays of fixed size, so it allocates nothing (no
// cudaMalloc, cudaFree, or host heap).
//
// What it runs: the same two-phase executor kernel that tcfftPlan1d selects
// for n = 2^12 .. 2^21, with its scratch ring placed in g_scratch
// (kNoAllocScratchBytes = 32 MiB) and fewer ring slots when the transform is
// large.  Limits: plain fp16 n <= 2^21, split n <= 2^20 (a ring needs at least
// 4 transforms of scratch); n >= 2^12 (smaller sizes use no scratch -- use a
// plan).
//
// Costs of the static arrays: every GPU that loads this library holds them
// (about 32.2 MiB) until the process exits.  Every call shares them and they
// keep the previous call's contents: each call rewrites its twiddle tables and
// clears its completion counters before launching, so calls ordered on one
// stream are independent, but calls that overlap on the GPU (different
// streams, or several host threads) race on the same scratch and must not be
// issued concurrently.
//
// Set-up: the first call on a device looks up the device addresses of the
// arrays with cudaGetSymbolAddress (with that device current).  Make that
// first call before any stream capture; later calls only enqueue work.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

constexpr int64_t kNoAllocScratchBytes = int64_t(32) << 20;
constexpr int kNoAllocMaxSlots = 1024;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];
static __device__ __align__(256) float2 g_tw2048[2048];  // W_2048^j for the call's direction
static __device__ __align__(256) float2 g_twlo[2048];    // W_n^j, j < 2^shift
static __device__ __align__(256) float2 g_twhi[2048];    // W_n^(j << shift)
static __device__ __align__(256) int g_counters[2 * kNoAllocMaxSlots];
static __device__ int g_err;

struct DevicePtrs {
  std::atomic<bool> ready{false};  // set (release) after the fields below are filled
  unsigned char* scratch = nullptr;
  float2* tw2048 = nullptr;
  float2* twlo = nullptr;
  float2* twhi = nullptr;
  int* counters = nullptr;
  int* err = nullptr;
  int num_sms = 0;
};
DevicePtrs g_dev[kNoAllocMaxDevices];
std::mutex g_mu;

// Twiddle tables for one call, computed in FP64 on the device:
// sign -1 (forward) or +1 (adjoint); W_n^j = exp(sign * 2 pi i j / n).
__global__ void noalloc_tables_kernel(float2* tw2048, float2* twlo, float2* twhi, long long n, int shift,
                                      double sign) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 2048) {
    double s, c;
    sincospi(2.0 * (double)i / 2048.0, &s, &c);
    tw2048[i] = make_float2((float)c, (float)(sign * s));
  }
  if (i < (1 << shift)) {
    double s, c;
    sincospi(2.0 * (double)i / (double)n, &s, &c);
    twlo[i] = make_float2((float)c, (float)(sign * s));
  }
  if (i < (int)(n >> shift)) {
    double s, c;
    sincospi(2.0 * (double)((long long)i << shift) / (double)n, &s, &c);
    twhi[i] = make_float2((float)c, (float)(sign * s));
  }
}

cudaError_t setup_device(int dev, DevicePtrs& d) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (d.ready.load(std::memory_order_acquire)) return cudaSuccess;
  cudaError_t e;
  if ((e = cudaGetSymbolAddress((void**)&d.scratch, g_scratch)) != cudaSuccess) return e;
  if ((e = cudaGetSymbolAddress((void**)&d.tw2048, g_tw2048)) != cudaSuccess) return e;
  if ((e = cudaGetSymbolAddress((void**)&d.twlo, g_twlo)) != cudaSuccess) return e;
  if ((e = cudaGetSymbolAddress((void**)&d.twhi, g_twhi)) != cudaSuccess) return e;
  if ((e = cudaGetSymbolAddress((void**)&d.counters, g_counters)) != cudaSuccess) return e;
  if ((e = cudaGetSymbolAddress((void**)&d.err, g_err)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  d.ready.store(true, std::memory_order_release);
  return cudaSuccess;
}

int ilog2_i64(int64_t v) {
  int r = 0;
  while ((int64_t(1) << r) < v) ++r;
  return r;
}

}  // namespace
}  // namespace tcfft

using namespace tcfft;

extern "C" tcfftStatus tcfftCheckDeviceNoAlloc(void* stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return TCFFT_CUDA_ERROR;
  if (cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)) != cudaSuccess) return TCFFT_CUDA_ERROR;
  if (!g_dev[dev].ready.load(std::memory_order_acquire)) return TCFFT_SUCCESS;  // nothing ran on this device
  int e = 0;
  if (cudaMemcpyFromSymbol(&e, g_err, sizeof(int)) != cudaSuccess) return TCFFT_CUDA_ERROR;
  if (e == 0) return TCFFT_SUCCESS;
  const int zero = 0;
  if (cudaMemcpyToSymbol(g_err, &zero, sizeof(int)) != cudaSuccess) return TCFFT_CUDA_ERROR;
  return TCFFT_TIMEOUT;
}

extern "C" tcfftStatus tcfftExecute1dNoAlloc(void* data, int64_t n, int64_t batch, int32_t precision,
                                             int32_t direction, void* stream) {
  const bool debug = getenv("TCFFT_DEBUG") != nullptr;
  if (!data) return TCFFT_INVALID_VALUE;
  if ((reinterpret_cast<uintptr_t>(data) & 127) != 0) return TCFFT_MISALIGNED;
  if (precision != TCFFT_PRECISION_PLAIN && precision != TCFFT_PRECISION_SPLIT) return TCFFT_INVALID_VALUE;
  if (direction != 0 && direction != 1) return TCFFT_INVALID_VALUE;
  const bool split = precision == TCFFT_PRECISION_SPLIT;
  const int es = split ? 8 : 4, er = 128 / es;
  const int lg = ilog2_i64(n);
  const int max_lg = split ? 20 : 21;
  if (n <= 0 || (n & (n - 1)) != 0 || lg < 12 || lg > max_lg || batch < 1 || batch > (int64_t(1) << 40) / n) {
    if (debug)
      fprintf(stderr, "tcfftExecute1dNoAlloc: n must be a power of two in [2^12, 2^%d] (scratch is %lld MiB)\n",
              max_lg, (long long)(kNoAllocScratchBytes >> 20));
    return TCFFT_INVALID_SIZE;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return TCFFT_CUDA_ERROR;
  DevicePtrs& d = g_dev[dev];
  if (!d.ready.load(std::memory_order_acquire)) {
    cudaError_t e = setup_device(dev, d);
    if (e != cudaSuccess) {
      if (debug) fprintf(stderr, "tcfftExecute1dNoAlloc: set-up failed: %s\n", cudaGetErrorString(e));
      return TCFFT_CUDA_ERROR;
    }
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  // schedule (same decomposition as tcfftPlan1d's two-phase executor)
  FusedKey k;
  int64_t n1, n2;
  if (lg <= 15) {
    // 256 x (16..64) short rows; 2^15 as 512 x 64 (the plan's choice, and the split short-row
    // phase's R <= 4 limit)
    n1 = lg == 15 ? 512 : 256;
    n2 = n / n1;
    k.role0 = kRoleCol;
    k.R0 = (int)(n1 / 256);
    k.C0 = lg == 15 ? (split ? 16 : 32) : 16;
    k.role1 = kRoleRow16T;
    k.R1 = (int)(n2 / 16);
    k.C1 = 128;
    if (split && k.R1 > 4) return TCFFT_NOT_SUPPORTED;
  } else {
    // the plan's decompositions: N1 >= N2, except 2^21 as 1024 x 2048
    n1 = lg == 21 ? 1024 : int64_t(1) << ((lg + 1) / 2);
    n2 = n / n1;
    k.role0 = kRoleCol;
    k.R0 = (int)(n1 / 256);
    k.C0 = fused_cols(k.R0, split);
    k.role1 = kRoleRowT;
    k.R1 = (int)(n2 / 256);
    k.C1 = fused_cols(k.R1, split);
    if (k.C0 == 0 || k.C1 == 0) return TCFFT_NOT_SUPPORTED;
  }
  k.split = split;
  const int T0 = (int)(n2 / k.C0 > 0 ? n2 / k.C0 : 1), T1 = (int)(n1 / k.C1);
  // lag and slots: as many as the fixed scratch holds (at least D = 1, S = 4)
  const int64_t slot_bytes = n * es;
  int max_slots = (int)(kNoAllocScratchBytes / slot_bytes);
  if (max_slots > kNoAllocMaxSlots) max_slots = kNoAllocMaxSlots;
  int D = (d.num_sms * 4 + (T0 + T1) - 1) / (T0 + T1) + 1;
  if (D > batch) D = (int)batch;
  if (D > (max_slots - 2) / 2) D = (max_slots - 2) / 2;
  if (D < 1) return TCFFT_INVALID_SIZE;
  const int S = 2 * D + 2;

  // tables for this call, counters cleared (both on `st`, before the launch)
  const int shift = (lg + 1) / 2;
  noalloc_tables_kernel<<<(2048 + 255) / 256, 256, 0, st>>>(d.tw2048, d.twlo, d.twhi, (long long)n, shift,
                                                           direction == 0 ? -1.0 : 1.0);
  if (cudaGetLastError() != cudaSuccess) return TCFFT_CUDA_ERROR;
  if (cudaMemsetAsync(d.counters, 0, sizeof(int) * 2 * S, st) != cudaSuccess) return TCFFT_CUDA_ERROR;

  // tensor maps (host-side encode, no allocation)
  FusedMaps maps;
  if (encode_fused1d_maps(&maps, k, data, d.scratch, n1, n2, batch, S) != CUDA_SUCCESS) return TCFFT_CUDA_ERROR;

  FusedParams fp;
  fp.tw2048 = d.tw2048;
  fp.scratch = reinterpret_cast<unsigned char*>(d.scratch);
  fp.twlo = d.twlo;
  fp.twhi = d.twhi;
  fp.tw_shift = shift;
  fp.wn_global = 0;
  fp.n_mask = (long long)(n - 1);
  fp.batch = (int)batch;
  fp.D = D;
  fp.S = S;
  fp.T0 = T0;
  fp.T1 = T1;
  fp.rows0 = (int)n1;
  fp.rows1 = (int)n1;
  fp.cols0 = T0;
  fp.cols1 = T1;
  fp.cnt0 = d.counters;
  fp.cnt1 = d.counters + S;
  fp.err = d.err;
  fp.dsign = direction == 0 ? 1.f : -1.f;
  fp.wait_ns = 0;  // the default limit
  fp.oscale0 = fp.oscale1 = 1.f;  // unnormalised
  int grid = 0;
  cudaError_t e = launch_fused(k, maps, fp, d.num_sms, st, &grid);
  if (e != cudaSuccess) {
    if (debug) fprintf(stderr, "tcfftExecute1dNoAlloc: launch failed: %s\n", cudaGetErrorString(e));
    return TCFFT_CUDA_ERROR;
  }
  return TCFFT_SUCCESS;
}
