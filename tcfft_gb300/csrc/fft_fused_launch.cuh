// fft_fused_launch.cuh -- launch one instantiation of the two-phase executor
// (fft_fused.cuh), or report its ring shape to the planner.  Included by the
// translation units that instantiate it (fft_fused.cu, fft_fused_2d*.cu); each
// lists its instantiations with TCFFT_FUSED_CASE.
#pragma once
#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {

template <int ROLE0, int R0, int C0, int ROLE1, int R1, int C1, int MODE, int ITEM_KB>
cudaError_t fused_launch_or_query(const FusedMaps* maps, const FusedParams* p, int num_sms, cudaStream_t st,
                                  int* grid_out, FusedShape* shape) {
  using Cfg = FusedCfg<ROLE0, R0, C0, ROLE1, R1, C1, MODE, ITEM_KB>;
  if (shape) {
    shape->stages = Cfg::kStages;
    shape->sub0 = Cfg::kSub0;
    shape->sub1 = Cfg::kSub1;
    shape->smem = Cfg::kSmem;
    return cudaSuccess;
  }
  auto kern = fft_fused_kernel<ROLE0, R0, C0, ROLE1, R1, C1, MODE, ITEM_KB>;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [&] {
    init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem);
  });
  if (init_err != cudaSuccess) return init_err;
  // p->T0 / p->T1 count tiles per transform; the kernel works on items of kSub0 / kSub1 tiles
  if (p->T0 % Cfg::kSub0 != 0 || p->T1 % Cfg::kSub1 != 0) return cudaErrorInvalidValue;
  FusedParams q = *p;
  q.T0 = p->T0 / Cfg::kSub0;
  q.T1 = p->T1 / Cfg::kSub1;
  const long long items = (long long)(q.batch + q.D) * (q.T0 + q.T1);
  long long grid = num_sms;
  if (grid > items) grid = items;
  if (grid_out) *grid_out = (int)grid;
  kern<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(*maps, q);
  return cudaGetLastError();
}

}  // namespace tcfft

// One instantiation: roles, radices and tile widths of both phases, precision
// (false: plain, true: split; kModeIo32 in fft_fused_io32.cu), work-item size in KiB.
#define TCFFT_FUSED_CASE(RO0, RR0, CC0, RO1, RR1, CC1, SP, KB)                                                  \
  TCFFT_FUSED_CASE_MODE(RO0, RR0, CC0, RO1, RR1, CC1, ((SP) ? kModeSplit : kModePlain), KB)
#define TCFFT_FUSED_CASE_MODE(RO0, RR0, CC0, RO1, RR1, CC1, MM, KB)                                             \
  if (k.role0 == RO0 && k.R0 == RR0 && k.C0 == CC0 && k.role1 == RO1 && k.R1 == RR1 && k.C1 == CC1 &&        \
      fused_mode(k) == (MM) && k.item_kb == KB) {                                                            \
    *handled = true;                                                                                          \
    return fused_launch_or_query<RO0, RR0, CC0, RO1, RR1, CC1, (MM), KB>(maps, p, num_sms, st, grid_out, shape); \
  }
