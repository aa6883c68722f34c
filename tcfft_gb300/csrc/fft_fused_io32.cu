// fft_fused_io32.cu -- instantiations of the persistent two-phase executor in the
// fp32-I/O mode (fp32 data and inter-phase storage, fp16 tensor-core operands
// converted as they are read from shared memory, one product per stage): the
// 1D four-step and 2D schedules of the split mode, with plain arithmetic.
#include "fft_fused_launch.cuh"

namespace tcfft {

cudaError_t launch_fused_io32(const FusedKey& k, const FusedMaps* maps, const FusedParams* p, int num_sms,
                              cudaStream_t st, int* grid_out, FusedShape* shape, bool* handled) {
  *handled = false;
  TCFFT_FUSED_CASE_MODE(kRoleCol, 1, 16, kRoleRowT, 1, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 2, 16, kRoleRowT, 1, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 2, 16, kRoleRowT, 2, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 4, 8, kRoleRowT, 2, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 4, 8, kRoleRowT, 4, 8, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 1, 16, kRoleRow16T, 1, 128, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 1, 16, kRoleRow16T, 2, 128, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 1, 16, kRoleRow16T, 4, 128, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleCol, 2, 16, kRoleRow16T, 4, 128, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 1, 16, kRoleCol, 1, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 1, 16, kRoleCol, 2, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 1, 16, kRoleCol, 4, 8, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 2, 16, kRoleCol, 1, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 2, 16, kRoleCol, 2, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 2, 16, kRoleCol, 4, 8, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 4, 8, kRoleCol, 1, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 4, 8, kRoleCol, 2, 16, kModeIo32, 64)
  TCFFT_FUSED_CASE_MODE(kRoleRow, 4, 8, kRoleCol, 4, 8, kModeIo32, 64)
  return cudaErrorNotSupported;
}

}  // namespace tcfft
