// fft_fused.cu -- instantiations of the persistent two-phase executor (1D four-step).
#include "fft_fused_launch.cuh"

namespace tcfft {

cudaError_t launch_fused_1d(const FusedKey& k, const FusedMaps* maps, const FusedParams* p, int num_sms, cudaStream_t st,
                int* grid_out, FusedShape* shape, bool* handled) {
  *handled = false;
  // 1D four-step: phase 0 = columns of N1 = 256*R0, phase 1 = rows of N2 = 256*R1 (N1 >= N2)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 32, kRoleRowT, 1, 32, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRowT, 1, 32, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRowT, 2, 32, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 2, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 2, 32, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 4, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 4, 16, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 8, 8, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 16, kRoleRowT, 8, 8, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRowT, 8, 8, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 8, 8, kRoleRowT, 2, 32, false, 64)
  // 32 KiB work items (deeper rings, one tile per item)
  TCFFT_FUSED_CASE(kRoleCol, 1, 32, kRoleRowT, 1, 32, false, 32)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 32, false, 32)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, false, 32)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 2, 16, false, 32)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 4, 8, false, 32)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRowT, 1, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 1, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRowT, 2, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 2, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 4, 8, kRoleRowT, 4, 8, true, 64)
  // 1D N = 256 x (16..128): phase 1 = 16 short rows per warp
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 1, 128, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 2, 128, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 4, 128, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 8, 128, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 32, kRoleRow16T, 4, 128, false, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 1, 128, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 2, 128, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 1, 16, kRoleRow16T, 4, 128, true, 64)
  TCFFT_FUSED_CASE(kRoleCol, 2, 16, kRoleRow16T, 4, 128, true, 64)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
