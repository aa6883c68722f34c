// fft_small.cu -- instantiations and launcher of the single-pass kernels
// (N = 256, 512, 1024, 2048; plain, split and fp32-I/O modes).
#include <mutex>

#include "fft_small.cuh"
#include "tcfft_host.h"

namespace tcfft {

namespace {
template <int R, int MODE>
cudaError_t launch_one(const CUtensorMap& tmap, const CUtensorMap& omap, int64_t total_elems, const float2* tw,
                       float dsign, int* err, int num_sms, cudaStream_t stream, float oscale) {
  using C = SmallCfg<R, MODE>;
  static std::once_flag once;
  static int blocks_per_sm = 1;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [] {
    init_err = cudaFuncSetAttribute(fft_small_kernel<R, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (init_err == cudaSuccess)
      init_err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, fft_small_kernel<R, MODE>, 256, C::kSmem);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  });
  if (init_err != cudaSuccess) return init_err;
  SmallParams p;
  p.tw = tw;
  p.num_tiles = (int)((total_elems + C::kTE - 1) / C::kTE);
  p.dsign = dsign;
  p.err = err;
  p.oscale = oscale;
  int grid = num_sms * blocks_per_sm;
  if (grid > p.num_tiles) grid = p.num_tiles;
  if (grid < 1) return cudaSuccess;
  fft_small_kernel<R, MODE><<<grid, 256, C::kSmem, stream>>>(tmap, omap, p);
  return cudaGetLastError();
}
}  // namespace

int small_tile_elems(int R, int mode) {
  switch (R * 4 + mode) {
    case 4: return SmallCfg<1, kModePlain>::kTE;
    case 5: return SmallCfg<1, kModeSplit>::kTE;
    case 6: return SmallCfg<1, kModeIo32>::kTE;
    case 8: return SmallCfg<2, kModePlain>::kTE;
    case 9: return SmallCfg<2, kModeSplit>::kTE;
    case 10: return SmallCfg<2, kModeIo32>::kTE;
    case 16: return SmallCfg<4, kModePlain>::kTE;
    case 17: return SmallCfg<4, kModeSplit>::kTE;
    case 18: return SmallCfg<4, kModeIo32>::kTE;
    case 32: return SmallCfg<8, kModePlain>::kTE;
    case 33: return SmallCfg<8, kModeSplit>::kTE;
    case 34: return SmallCfg<8, kModeIo32>::kTE;
    default: return 0;
  }
}

cudaError_t launch_small(int R, int mode, const CUtensorMap& tmap, const CUtensorMap& omap, int64_t total_elems,
                         const float2* tw, float dsign, int* err, int num_sms, cudaStream_t stream, int* launches,
                         float oscale) {
  if (launches) *launches = 1;
#define TCFFT_SMALL(RR, MM) \
  case RR * 4 + MM: return launch_one<RR, MM>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
  switch (R * 4 + mode) {
    TCFFT_SMALL(1, kModePlain)
    TCFFT_SMALL(1, kModeSplit)
    TCFFT_SMALL(1, kModeIo32)
    TCFFT_SMALL(2, kModePlain)
    TCFFT_SMALL(2, kModeSplit)
    TCFFT_SMALL(2, kModeIo32)
    TCFFT_SMALL(4, kModePlain)
    TCFFT_SMALL(4, kModeSplit)
    TCFFT_SMALL(4, kModeIo32)
    TCFFT_SMALL(8, kModePlain)
    TCFFT_SMALL(8, kModeSplit)
    TCFFT_SMALL(8, kModeIo32)
    default: return cudaErrorInvalidValue;
  }
#undef TCFFT_SMALL
}

}  // namespace tcfft
