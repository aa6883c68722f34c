// fft_fused.cu -- instantiations and launcher of the persistent two-phase
// executor (1D four-step N = N1*N2, 2D row+column).
#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {

namespace {

template <int ROLE0, int R0, int C0, int ROLE1, int R1, int C1, bool SPLIT>
cudaError_t launch_t(const FusedMaps& maps, const FusedParams& p, int num_sms, cudaStream_t st, int* grid_out) {
  using Cfg = FusedCfg<ROLE0, R0, C0, ROLE1, R1, C1, SPLIT>;
  auto kern = fft_fused_kernel<ROLE0, R0, C0, ROLE1, R1, C1, SPLIT>;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [&] {
    init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem);
  });
  if (init_err != cudaSuccess) return init_err;
  const long long items = (long long)(p.batch + p.D) * (p.T0 + p.T1);
  long long grid = num_sms;
  if (grid > items) grid = items;
  if (grid_out) *grid_out = (int)grid;
  kern<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(maps, p);
  return cudaGetLastError();
}

// key: role pair, R0, R1, split (C derived)
#define TCFFT_FUSED_CASE(RO0, RR0, CC0, RO1, RR1, CC1, SP)                                                        \
  if (k.role0 == RO0 && k.R0 == RR0 && k.C0 == CC0 && k.role1 == RO1 && k.R1 == RR1 && k.C1 == CC1 && k.split == SP) \
    return launch_t<RO0, RR0, CC0, RO1, RR1, CC1, SP>(maps, p, num_sms, st, grid_out);

}  // namespace

int fused_cols(int R, bool split) {
  // columns (or rows) per tile: keep a tile <= 64 KB and its rows at 64 or 128 bytes
  const int es = split ? 8 : 4;
  int c = 16;
  while (c > 8 && c * 256 * R * es > 64 * 1024) c /= 2;
  if (c * 256 * R * es > 64 * 1024) return 0;
  return c;
}

cudaError_t launch_fused(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms,
                         cudaStream_t st, int* grid_out) {
  // 1D four-step: phase 0 = columns of N1 = 256*R0, phase 1 = rows of N2 = 256*R1 (N1 >= N2)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 2, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 2, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 4, 8, true)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
