// fft_job.cuh -- one warp computes one FFT of length 256*R held in shared
// memory, with caller-supplied addressing (so the same code serves contiguous
// rows and strided columns of a tile).
//
// Algorithm (decimation in frequency, natural-order input):
//   n = m + 256 a, k = q + R k', m = 16 m1 + m0, k' = k0 + 16 k1
//   X[q + R k'] = sum_m0 W16^(m0 k1) W256^(m0 k0) sum_m1 W16^(m1 k0)
//                 [ W_{256R}^(m q) sum_a x[m + 256 a] W_R^(a q) ]
// radix-R butterfly (fp32, registers) -> twiddle -> radix-16 MMA over m1 ->
// twiddle W256 -> radix-16 MMA over m0, chained in registers.
#pragma once
#include "fft_common.cuh"

namespace tcfft {

// Per-thread constants of a 256-point job (independent of the job's location).
template <bool SPLIT>
struct JobConsts {
  uint32_t afr[2][2][4];
  uint32_t afr_lo[SPLIT ? 2 : 1][2][4];
  float2 tw1[2][2][2];  // W256^(m0 k0) at stage-1 output (j, h, e)
  int mval[2][2][2];    // m = 16 m1 + m0 of load slot (kt, r, j)
  int kval[2][2][2];    // k' = k0 + 16 k1 of output slot (h, e, hh)
};

// tw2048: W_2048^j table (direction-specific).
template <bool SPLIT, class PI, class RHO>
__device__ __forceinline__ void init_job_consts(JobConsts<SPLIT>& c, const float2* __restrict__ tw2048) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t dummy[2][2][4];
  if constexpr (SPLIT) build_dft_frags<PI, RHO>(tw2048, 128, c.afr, c.afr_lo, true);
  else build_dft_frags<PI, RHO>(tw2048, 128, c.afr, dummy, false);
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int m0 = PI::apply(2 * t + e + 8 * j), k0 = RHO::apply(g + 8 * h);
        c.tw1[j][h][e] = tw2048[((m0 * k0) & 255) * 8];
      }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) c.mval[kt][r][j] = 16 * PI::apply(2 * t + r + 8 * kt) + PI::apply(g + 8 * j);
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh)
        c.kval[h][e][hh] = RHO::apply(2 * t + e + 8 * h) + 16 * RHO::apply(g + 8 * hh);
}

// LOAD(n) -> float2 element n (0 <= n < 256R) of the job's input.
// STORE(k, q, slot, float2) receives output k = q + R * kval[slot] in fp32
// (slot = 4h + 2e + hh, a compile-time constant after unrolling).
// twR: table with W_{256R}^j at index j*TWS (shared memory), used for the
// radix-R twiddles.
// All LOADs of the warp complete (and are ordered by __syncwarp) before the
// first STORE, so a job may write its output over its own input.
template <int R, bool SPLIT, int TWS = 1, class LoadF, class StoreF>
__device__ __forceinline__ void fft256r_job(const JobConsts<SPLIT>& c, const float2* __restrict__ twR, float dsign,
                                            LoadF&& load, StoreF&& store) {
  uint32_t bhi[R][2][2][2], blo[SPLIT ? R : 1][2][2][2];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float2 x[R];
#pragma unroll
        for (int a = 0; a < R; ++a) x[a] = load(c.mval[kt][r][j] + 256 * a);
        if constexpr (R > 1) {
          dft_small<R>(x, dsign);
#pragma unroll
          for (int q = 1; q < R; ++q) x[q] = cmul(x[q], twR[((c.mval[kt][r][j] * q) & (256 * R - 1)) * TWS]);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
          if constexpr (SPLIT) split_h2(x[q], bhi[q][kt][r][j], blo[q][kt][r][j]);
          else bhi[q][kt][r][j] = pack_h2(x[q].x, x[q].y);
        }
      }
  __syncwarp();  // every lane has read the job's input (stores may alias it)
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float acc[2][2][4];
    if constexpr (SPLIT) dft16_mma_split(c.afr, c.afr_lo, bhi[q], blo[q], acc);
    else dft16_mma(c.afr, bhi[q], acc);
    uint32_t b2[2][2][2], b2lo[2][2][2];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float2 v = cmul(acc_get(acc, kt, h, r), c.tw1[kt][h][r]);
          if constexpr (SPLIT) split_h2(v, b2[kt][r][h], b2lo[kt][r][h]);
          else b2[kt][r][h] = pack_h2(v.x, v.y);
        }
    if constexpr (SPLIT) dft16_mma_split(c.afr, c.afr_lo, b2, b2lo, acc);
    else dft16_mma(c.afr, b2, acc);
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) store(q + R * c.kval[h][e][hh], q, 4 * h + 2 * e + hh, acc_get(acc, h, hh, e));
  }
}

}  // namespace tcfft

namespace tcfft {

// ---------------------------------------------------------------------------
// One warp computes 16 FFTs of length 16*R at once (one radix-16 tensor-core
// stage plus a radix-R tail), the 16 transforms being the MMA's N dimension.
//   n = m1 + 16 a, k = q + R k0:
//   X_v[q + R k0] = sum_m1 W16^(m1 k0) [ W_{16R}^(m1 q) sum_a x_v[m1 + 16 a] W_R^(a q) ]
// LOAD(v, n) -> float2 element n of transform v (0 <= v < 16).
// STORE(v, k, q, slot, float2) receives output k = q + R k0 of transform v;
// slot = 4j + 2h + e (compile-time after unrolling) with v = 2t + e + 8j,
// k0 = RHO(g + 8h).
// tw16R: table with W_{16R}^j at index j*TWS.
template <int R, bool SPLIT, int TWS, class PI, class RHO, class LoadF, class StoreF>
__device__ __forceinline__ void fft16r_job(const JobConsts<SPLIT>& c, const float2* __restrict__ tw16R, float dsign,
                                           LoadF&& load, StoreF&& store) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t bhi[R][2][2][2], blo[SPLIT ? R : 1][2][2][2];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int m1 = PI::apply(2 * t + r + 8 * kt);
        const int v = g + 8 * j;
        float2 x[R];
#pragma unroll
        for (int a = 0; a < R; ++a) x[a] = load(v, m1 + 16 * a);
        if constexpr (R > 1) {
          dft_small<R>(x, dsign);
#pragma unroll
          for (int q = 1; q < R; ++q) x[q] = cmul(x[q], tw16R[((m1 * q) & (16 * R - 1)) * TWS]);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
          if constexpr (SPLIT) split_h2(x[q], bhi[q][kt][r][j], blo[q][kt][r][j]);
          else bhi[q][kt][r][j] = pack_h2(x[q].x, x[q].y);
        }
      }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float acc[2][2][4];
    if constexpr (SPLIT) dft16_mma_split(c.afr, c.afr_lo, bhi[q], blo[q], acc);
    else dft16_mma(c.afr, bhi[q], acc);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int e = 0; e < 2; ++e)
          store(2 * t + e + 8 * j, q + R * RHO::apply(g + 8 * h), q, 4 * j + 2 * h + e, acc_get(acc, j, h, e));
  }
}

}  // namespace tcfft
