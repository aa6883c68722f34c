// fft_fused_2d.cu -- instantiations of the persistent two-phase executor (2D row + column, plain).
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
  // p.T0 / p.T1 count tiles per transform; the kernel works on items of kSub0 / kSub1 tiles
  if (p.T0 % Cfg::kSub0 != 0 || p.T1 % Cfg::kSub1 != 0) return cudaErrorInvalidValue;
  FusedParams q = p;
  q.T0 = p.T0 / Cfg::kSub0;
  q.T1 = p.T1 / Cfg::kSub1;
  const long long items = (long long)(q.batch + q.D) * (q.T0 + q.T1);
  long long grid = num_sms;
  if (grid > items) grid = items;
  if (grid_out) *grid_out = (int)grid;
  kern<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(maps, q);
  return cudaGetLastError();
}
}  // namespace

#define TCFFT_FUSED_CASE(RO0, RR0, CC0, RO1, RR1, CC1, SP)                                                        \
  if (k.role0 == RO0 && k.R0 == RR0 && k.C0 == CC0 && k.role1 == RO1 && k.R1 == RR1 && k.C1 == CC1 && k.split == SP) { \
    *handled = true;                                                                                                \
    return launch_t<RO0, RR0, CC0, RO1, RR1, CC1, SP>(maps, p, num_sms, st, grid_out);                             \
  }

cudaError_t launch_fused_2d_plain(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms, cudaStream_t st,
                int* grid_out, bool* handled) {
  *handled = false;
  // 2D [NX][NY]: phase 0 = rows of NY = 256*R0 (C0 rows per tile), phase 1 = columns of NX = 256*R1
  TCFFT_FUSED_CASE(kRoleRow, 1, 32, kRoleCol, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 1, 32, kRoleCol, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 1, 32, kRoleCol, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleRow, 1, 32, kRoleCol, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleRow, 2, 32, kRoleCol, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 2, 32, kRoleCol, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 2, 32, kRoleCol, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleRow, 2, 32, kRoleCol, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleRow, 4, 16, kRoleCol, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 4, 16, kRoleCol, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 4, 16, kRoleCol, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleRow, 4, 16, kRoleCol, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleRow, 8, 8, kRoleCol, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 8, 8, kRoleCol, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleRow, 8, 8, kRoleCol, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleRow, 8, 8, kRoleCol, 8, 8, false)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
