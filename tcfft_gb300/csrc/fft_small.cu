// fft_small.cu -- instantiations and launcher of the single-pass kernels
// (N = 256, 512, 1024, 2048; plain and split precision).
#include <mutex>

#include "fft_small.cuh"
#include "tcfft_host.h"

namespace tcfft {

namespace {
template <int R, bool SPLIT>
cudaError_t launch_one(const CUtensorMap& tmap, const CUtensorMap& omap, int64_t total_elems, const float2* tw,
                       float dsign, int* err, int num_sms, cudaStream_t stream, float oscale) {
  using C = SmallCfg<R, SPLIT>;
  static std::once_flag once;
  static int blocks_per_sm = 1;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [] {
    init_err = cudaFuncSetAttribute(fft_small_kernel<R, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (init_err == cudaSuccess)
      init_err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, fft_small_kernel<R, SPLIT>, 256, C::kSmem);
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
  fft_small_kernel<R, SPLIT><<<grid, 256, C::kSmem, stream>>>(tmap, omap, p);
  return cudaGetLastError();
}
}  // namespace

int small_tile_elems(int R, bool split) {
  switch (R * 2 + (split ? 1 : 0)) {
    case 2: return SmallCfg<1, false>::kTE;
    case 3: return SmallCfg<1, true>::kTE;
    case 4: return SmallCfg<2, false>::kTE;
    case 5: return SmallCfg<2, true>::kTE;
    case 8: return SmallCfg<4, false>::kTE;
    case 9: return SmallCfg<4, true>::kTE;
    case 16: return SmallCfg<8, false>::kTE;
    default: return 0;
  }
}

cudaError_t launch_small(int R, bool split, const CUtensorMap& tmap, const CUtensorMap& omap, int64_t total_elems,
                         const float2* tw, float dsign, int* err, int num_sms, cudaStream_t stream, int* launches,
                         float oscale) {
  if (launches) *launches = 1;
  switch (R * 2 + (split ? 1 : 0)) {
    case 2: return launch_one<1, false>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 3: return launch_one<1, true>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 4: return launch_one<2, false>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 5: return launch_one<2, true>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 8: return launch_one<4, false>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 9: return launch_one<4, true>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    case 16: return launch_one<8, false>(tmap, omap, total_elems, tw, dsign, err, num_sms, stream, oscale);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace tcfft
