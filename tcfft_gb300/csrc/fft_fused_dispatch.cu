// fft_fused_dispatch.cu -- routes a FusedKey to the translation unit that instantiates it.
#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {

cudaError_t launch_fused_1d(const FusedKey&, const FusedMaps*, const FusedParams*, int, cudaStream_t, int*, FusedShape*,
                            bool*);
cudaError_t launch_fused_2d_plain(const FusedKey&, const FusedMaps*, const FusedParams*, int, cudaStream_t, int*,
                                  FusedShape*, bool*);
cudaError_t launch_fused_2d_split(const FusedKey&, const FusedMaps*, const FusedParams*, int, cudaStream_t, int*,
                                  FusedShape*, bool*);
cudaError_t launch_fused_io32(const FusedKey&, const FusedMaps*, const FusedParams*, int, cudaStream_t, int*,
                              FusedShape*, bool*);

namespace {
// Routes `k` to its translation unit: launches, or with `shape` set only reports the ring shape.
cudaError_t route(const FusedKey& k, const FusedMaps* maps, const FusedParams* p, int num_sms, cudaStream_t st,
                  int* grid_out, FusedShape* shape, bool* handled) {
  if (k.split && k.io32) {
    cudaError_t e = launch_fused_io32(k, maps, p, num_sms, st, grid_out, shape, handled);
    return *handled ? e : cudaErrorNotSupported;
  }
  cudaError_t e = launch_fused_1d(k, maps, p, num_sms, st, grid_out, shape, handled);
  if (*handled) return e;
  e = k.split ? launch_fused_2d_split(k, maps, p, num_sms, st, grid_out, shape, handled)
              : launch_fused_2d_plain(k, maps, p, num_sms, st, grid_out, shape, handled);
  if (*handled) return e;
  return cudaErrorNotSupported;
}
}  // namespace

int fused_cols(int R, bool split, int max_tile_bytes) {
  // columns (or rows) per tile: keep a tile <= max_tile_bytes and its rows at 32, 64 or 128 bytes
  // plain: 32 columns (128-byte rows) while the tile fits, which measured faster than 16 for
  // R <= 2 (fewer, larger TMA rows and tiles)
  const int es = split ? 8 : 4;
  int c = split ? 16 : 32;
  while (c > 8 && c * 256 * R * es > max_tile_bytes) c /= 2;
  if (c * 256 * R * es > max_tile_bytes) return 0;
  return c;
}

cudaError_t launch_fused(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms,
                         cudaStream_t st, int* grid_out) {
  bool handled = false;
  return route(k, &maps, &p, num_sms, st, grid_out, nullptr, &handled);
}

bool fused_shape(const FusedKey& k, FusedShape* out) {
  bool handled = false;
  FusedShape tmp;
  return route(k, nullptr, nullptr, 0, nullptr, nullptr, out ? out : &tmp, &handled) == cudaSuccess && handled;
}

}  // namespace tcfft
