// fft_fused.cu -- instantiations of the persistent two-phase executor (1D four-step).
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

cudaError_t launch_fused_1d(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms, cudaStream_t st,
                int* grid_out, bool* handled) {
  *handled = false;
  // 1D four-step: phase 0 = columns of N1 = 256*R0, phase 1 = rows of N2 = 256*R1 (N1 >= N2)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 32, kRoleRowT, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRowT, 1, 32, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRowT, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 2, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 2, 32, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 4, 16, false)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 8, 8, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 2, 16, true)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 4, 8, true)
  // 1D N = 256 x (16..128): phase 1 = 16 short rows per warp
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 1, 128, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 2, 128, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 4, 128, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 8, 128, false)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRow16T, 4, 128, false)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 1, 128, true)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 2, 128, true)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 4, 128, true)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRow16T, 4, 128, true)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
