// fft_fused_dispatch.cu -- routes a FusedKey to the translation unit that instantiates it.
#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {

cudaError_t launch_fused_1d(const FusedKey&, const FusedMaps&, const FusedParams&, int, cudaStream_t, int*, bool*);
cudaError_t launch_fused_2d_plain(const FusedKey&, const FusedMaps&, const FusedParams&, int, cudaStream_t, int*, bool*);
cudaError_t launch_fused_2d_split(const FusedKey&, const FusedMaps&, const FusedParams&, int, cudaStream_t, int*, bool*);

int fused_cols(int R, bool split) {
  // columns (or rows) per tile: keep a tile <= 64 KB and its rows at 32, 64 or 128 bytes
  // plain: 32 columns (128-byte rows) while the tile stays <= 64 KB, which measured faster
  // than 16 for R <= 2 (fewer, larger TMA rows and tiles)
  const int es = split ? 8 : 4;
  int c = split ? 16 : 32;
  while (c > 8 && c * 256 * R * es > 64 * 1024) c /= 2;
  if (c * 256 * R * es > 64 * 1024) return 0;
  return c;
}

cudaError_t launch_fused(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms,
                         cudaStream_t st, int* grid_out) {
  bool handled = false;
  cudaError_t e = launch_fused_1d(k, maps, p, num_sms, st, grid_out, &handled);
  if (handled) return e;
  e = k.split ? launch_fused_2d_split(k, maps, p, num_sms, st, grid_out, &handled)
              : launch_fused_2d_plain(k, maps, p, num_sms, st, grid_out, &handled);
  if (handled) return e;
  return cudaErrorNotSupported;
}

}  // namespace tcfft
