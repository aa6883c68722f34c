// fft_tiny.cu -- 1D FFTs of length N = 16 R (R = 1, 2, 4, 8: N = 16 .. 128).
//
// No reference counterpart (the reference's smallest size is 256,
// tcfft_half.cu:1250-1330); these lengths are the short axes of 2D transforms
// such as 128 x 128 and the sizes below 256 of a 1D plan.
//
// One warp transforms 16 consecutive transforms at once: the 16 transforms are
// the N dimension of the tensor-core product (fft16r_job: one radix-16
// mma.sync stage over the leading digit and a radix-R tail), so a warp moves
// 16 N elements.  The warp stages its 16 transforms in shared memory with
// 16-byte vector copies; rows are padded by 16 bytes so that the 8 transforms
// a warp's lanes touch in one access fall in 8 different bank groups.
#include "fft_job.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

template <int R, int MODE>
struct TinyCfg {
  static constexpr bool kWide = MODE != kModePlain, kSplit = MODE == kModeSplit;
  static constexpr int kN = 16 * R;
  static constexpr int kES = kWide ? 8 : 4;
  static constexpr int kPad = 16 / kES;      // elements of padding per row
  static constexpr int kRow = kN + kPad;     // padded row length (elements)
  static constexpr int kWarps = 4;
  static constexpr int kWarpBytes = 16 * kRow * kES;
  using PI = typename std::conditional<kWide, BitPerm<0, 1, 2, 3>, BitPerm<0, 1, 3, 2>>::type;
  using RHO = BitPerm<0, 2, 3, 1>;
};

template <int R, int MODE>
__global__ void __launch_bounds__(128) fft_tiny_kernel(const unsigned char* in, unsigned char* data, long long batch,
                                                       const float2* __restrict__ tw2048, float dsign, float oscale) {
  using C = TinyCfg<R, MODE>;
  constexpr bool WIDE = C::kWide, SPLIT = C::kSplit;
  constexpr int N = C::kN, ES = C::kES, ROW = C::kRow;
  __shared__ __align__(16) unsigned char buf[C::kWarps][C::kWarpBytes];
  __shared__ float2 tw[N];  // W_N^j
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = threadIdx.x; j < N; j += blockDim.x) tw[j] = tw2048[j * (2048 / N)];
  JobConsts<SPLIT> jc;
  init_job_consts<SPLIT, typename C::PI, typename C::RHO>(jc, tw2048);
  __syncthreads();
  const uint32_t tw_addr = smem_addr(tw);
  const uint32_t wb = smem_addr(buf[warp]);
  constexpr int kVecPerRow = N * ES / 16;
  const long long groups = (batch + 15) / 16;
  for (long long gi = (long long)blockIdx.x * C::kWarps + warp; gi < groups; gi += (long long)gridDim.x * C::kWarps) {
    const long long v0 = gi * 16;
    const int nv = batch - v0 < 16 ? (int)(batch - v0) : 16;
    const uint4* src = reinterpret_cast<const uint4*>(in + v0 * N * ES);
    // global -> shared (padded rows); missing transforms of the last group read as zero
    for (int i = lane; i < 16 * kVecPerRow; i += 32) {
      const int v = i / kVecPerRow, c = i - v * kVecPerRow;
      const uint4 x = v < nv ? src[i] : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(buf[warp] + (v * ROW) * ES + c * 16) = x;
    }
    __syncwarp();
    auto ld = [&](int v, int n) {
      const uint32_t a = wb + (uint32_t)((v * ROW + n) * ES);
      if constexpr (WIDE) return lds64f(a);
      else return unpack_h2(lds32(a));
    };
    auto st = [&](int v, int k, int, int, float2 val) {
      const uint32_t a = wb + (uint32_t)((v * ROW + k) * ES);
      val = make_float2(val.x * oscale, val.y * oscale);  // output scale (1 unless normalised)
      if constexpr (WIDE) sts64f(a, val);
      else sts32(a, pack_h2(val.x, val.y));
    };
    fft16r_job<R, SPLIT, 1, typename C::PI, typename C::RHO>(jc, tw_addr, dsign, ld, st);
    __syncwarp();
    uint4* dst = reinterpret_cast<uint4*>(data + v0 * N * ES);
    for (int i = lane; i < nv * kVecPerRow; i += 32) {
      const int v = i / kVecPerRow, c = i - v * kVecPerRow;
      dst[i] = *reinterpret_cast<const uint4*>(buf[warp] + (v * ROW) * ES + c * 16);
    }
    __syncwarp();
  }
}

template <int R, int MODE>
cudaError_t launch_tiny_t(const void* in, void* data, int64_t batch, const float2* tw, float dsign, int num_sms,
                          cudaStream_t st, float oscale) {
  using C = TinyCfg<R, MODE>;
  const long long groups = (batch + 15) / 16;
  long long blocks = (groups + C::kWarps - 1) / C::kWarps;
  if (blocks > (long long)num_sms * 12) blocks = (long long)num_sms * 12;
  if (blocks < 1) blocks = 1;
  fft_tiny_kernel<R, MODE><<<(unsigned)blocks, 32 * C::kWarps, 0, st>>>(
      static_cast<const unsigned char*>(in), static_cast<unsigned char*>(data), batch, tw, dsign, oscale);
  return cudaGetLastError();
}

}  // namespace

bool tiny_supported(int64_t n, int mode) { return n == 16 || n == 32 || n == 64 || (n == 128 && mode == kModePlain); }

cudaError_t launch_tiny(int64_t n, int mode, void* data, int64_t batch, const float2* tw, float dsign, int num_sms,
                        cudaStream_t st, float oscale, const void* in) {
  if (!in) in = data;
#define TCFFT_TINY(NN, RR, MM) \
  case NN * 4 + MM: return launch_tiny_t<RR, MM>(in, data, batch, tw, dsign, num_sms, st, oscale);
  switch (n * 4 + mode) {
    TCFFT_TINY(16, 1, kModePlain)
    TCFFT_TINY(16, 1, kModeSplit)
    TCFFT_TINY(16, 1, kModeIo32)
    TCFFT_TINY(32, 2, kModePlain)
    TCFFT_TINY(32, 2, kModeSplit)
    TCFFT_TINY(32, 2, kModeIo32)
    TCFFT_TINY(64, 4, kModePlain)
    TCFFT_TINY(64, 4, kModeSplit)
    TCFFT_TINY(64, 4, kModeIo32)
    TCFFT_TINY(128, 8, kModePlain)
    default: return cudaErrorInvalidValue;
  }
#undef TCFFT_TINY
}

}  // namespace tcfft
