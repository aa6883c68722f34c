// fft_fused_2d_split.cu -- instantiations of the persistent two-phase executor (2D row + column, split).
#include "fft_fused_launch.cuh"

namespace tcfft {

cudaError_t launch_fused_2d_split(const FusedKey& k, const FusedMaps* maps, const FusedParams* p, int num_sms, cudaStream_t st,
                int* grid_out, FusedShape* shape, bool* handled) {
  *handled = false;
  // 2D [NX][NY]: phase 0 = rows of NY = 256*R0 (C0 rows per tile), phase 1 = columns of NX = 256*R1
  TCFFT_FUSED_CASE(kRoleRow, 1, 16, kRoleCol, 1, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 1, 16, kRoleCol, 2, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 1, 16, kRoleCol, 4, 8, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 2, 16, kRoleCol, 1, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 2, 16, kRoleCol, 2, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 2, 16, kRoleCol, 4, 8, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 4, 8, kRoleCol, 1, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 4, 8, kRoleCol, 2, 16, true, 64)
  TCFFT_FUSED_CASE(kRoleRow, 4, 8, kRoleCol, 4, 8, true, 64)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
