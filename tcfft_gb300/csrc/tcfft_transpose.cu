// tcfft_transpose.cu -- batched out-of-place transpose [B][R][C] -> [B][C][R].
//
// Used where a transform is composed from smaller plans: the last step of the
// large 1D sizes (N = N1 N2 with N2 > 2048 is computed as row FFTs of a
// [N1][N2] array whose result X[k1 + N1 k2] is its transpose) and the column
// pass of 2D shapes outside the fused 2D range; with a twiddle, the middle step
// of a four-step 1D FFT built from two short sub-plans.  32 x 32 tiles through
// shared memory: 128-byte coalesced rows on both sides for 4-byte elements.
#include <type_traits>

#include "fft_common.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

template <typename E>
__global__ void __launch_bounds__(256) transpose_kernel(const E* __restrict__ in, E* __restrict__ out, long long B,
                                                        long long R, long long C) {
  __shared__ E tile[32][33];
  const long long tr = (R + 31) / 32, tc = (C + 31) / 32, per = tr * tc, total = B * per;
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const long long b = t / per, rem = t - b * per;
    const long long r0 = (rem / tc) * 32, c0 = (rem % tc) * 32;
    const E* ib = in + b * R * C;
    E* ob = out + b * R * C;
#pragma unroll
    for (int i = threadIdx.y; i < 32; i += 8) {
      const long long r = r0 + i, c = c0 + threadIdx.x;
      if (r < R && c < C) tile[i][threadIdx.x] = ib[r * C + c];
    }
    __syncthreads();
#pragma unroll
    for (int i = threadIdx.y; i < 32; i += 8) {
      const long long c = c0 + i, r = r0 + threadIdx.x;
      if (r < R && c < C) ob[c * R + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}

// R and C multiples of T (T = 64 for 4-byte, 32 for 8-byte elements): T x T tiles,
// every global access a 16-byte vector (16 lanes cover one 256-byte row segment on
// both sides); the tile goes through shared memory with a one-element row pad, so
// the column-wise reads of the transposed side spread over the banks.
template <typename E, int T>
__global__ void __launch_bounds__(256) transpose_vec_kernel(const uint4* __restrict__ in, uint4* __restrict__ out,
                                                            long long B, long long R, long long C) {
  constexpr int V = 16 / sizeof(E);  // elements per 16-byte vector
  static_assert(V * 16 == T, "16 lanes cover one tile row");
  __shared__ E tile[T][T + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long tr = R / T, tc = C / T, per = tr * tc, total = B * per;
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const long long b = t / per, rem = t - b * per;
    const long long r0 = (rem / tc) * T, c0 = (rem % tc) * T;
    const uint4* ib = in + (b * R * C) / V;
    uint4* ob = out + (b * R * C) / V;
#pragma unroll
    for (int i = 0; i < T / 16; ++i) {
      const int r = ty + 16 * i;
      const uint4 v = ib[((r0 + r) * C + c0) / V + tx];
      const E* e = reinterpret_cast<const E*>(&v);
#pragma unroll
      for (int k = 0; k < V; ++k) tile[r][V * tx + k] = e[k];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < T / 16; ++i) {
      const int c = ty + 16 * i;  // output row (input column)
      uint4 v;
      E* e = reinterpret_cast<E*>(&v);
#pragma unroll
      for (int k = 0; k < V; ++k) e[k] = tile[V * tx + k][c];
      ob[((c0 + c) * R + r0) / V + tx] = v;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_transpose(const void* in, void* out, int64_t B, int64_t R, int64_t C, int es, int num_sms,
                             cudaStream_t st) {
  const int TV = es == 4 ? 64 : 32;  // vector-kernel tile
  if ((es == 4 || es == 8) && R % TV == 0 && C % TV == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0 &&
      (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    const long long tv = B * (R / TV) * (C / TV);
    const long long bv = tv < (long long)num_sms * 8 ? tv : (long long)num_sms * 8;
    if (es == 4)
      transpose_vec_kernel<uint32_t, 64><<<(unsigned)bv, 256, 0, st>>>(static_cast<const uint4*>(in),
                                                                       static_cast<uint4*>(out), B, R, C);
    else
      transpose_vec_kernel<uint2, 32><<<(unsigned)bv, 256, 0, st>>>(static_cast<const uint4*>(in),
                                                                    static_cast<uint4*>(out), B, R, C);
    return cudaGetLastError();
  }
  const long long tiles = B * ((R + 31) / 32) * ((C + 31) / 32);
  long long blocks = tiles < (long long)num_sms * 16 ? tiles : (long long)num_sms * 16;
  if (blocks < 1) blocks = 1;
  const dim3 block(32, 8);
  if (es == 4)
    transpose_kernel<uint32_t><<<(unsigned)blocks, block, 0, st>>>(static_cast<const uint32_t*>(in),
                                                                   static_cast<uint32_t*>(out), B, R, C);
  else if (es == 8)
    transpose_kernel<uint2><<<(unsigned)blocks, block, 0, st>>>(static_cast<const uint2*>(in),
                                                                static_cast<uint2*>(out), B, R, C);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace tcfft
