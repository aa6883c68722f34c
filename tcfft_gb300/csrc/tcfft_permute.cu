// tcfft_permute.cu -- the reference's input-order contract (digit-reversed input).
//
// The reference expects its input permuted on the host by gen_rev
// (tcfft_doit_half.cpp:6-29, applied at :38-46; 2D: tcfft_doit_half_2d.cpp:
// 40-50): position i holds x[rev[i]], where rev is the mixed-radix digit
// reversal for the radix chain tcfftCreate picked (tcfft_half.cu:1250-1330,
// tcfft_half_2d.cu:1167-1206).  Plans created with
// TCFFT_ORDER_REFERENCE_DIGIT_REVERSED accept that layout: a scatter kernel
// moves every element back to natural order (into a plan-owned buffer that is
// then copied back), after which the natural-order transform runs.
#include <vector>

#include "tcfft_host.h"

namespace tcfft {

// Reference radix chain for a 1D size (tcfft_half.cu:1250-1330), empty if the
// reference does not support the size.
std::vector<int> reference_radices_1d(int64_t n) {
  switch (n) {
    case 256: return {16, 16};
    case 512: return {16, 16, 2};
    case 1024: return {16, 16, 4};
    case 131072: return {16, 16, 2, 16, 16};
    case 262144: return {16, 16, 2, 16, 16, 2};
    case 524288: return {16, 16, 4, 16, 16, 2};
    case 16777216: return {16, 16, 16, 16, 16, 16};
    case 33554432: return {16, 16, 2, 16, 16, 16, 16};
    case 67108864: return {16, 16, 2, 16, 16, 2, 16, 16};
    case 134217728: return {16, 16, 2, 16, 16, 2, 16, 16, 2};
    default: return {};
  }
}

// Per-axis chain of the reference's 2D planner (tcfft_half_2d.cu:1167-1206).
std::vector<int> reference_radices_2d_axis(int64_t n) {
  switch (n) {
    case 256: return {16, 16};
    case 512: return {16, 16, 2};
    case 1024: return {16, 16, 4};
    default: return {};
  }
}

// Mixed-radix digit reversal: starting from the identity, for each radix from
// the last to the first every block of the current length is split into
// `radix` interleaved sub-sequences laid out one after another; the block
// length then shrinks by that radix (the permutation of tcfft_doit_half.cpp:6-29).
std::vector<int> digit_reversal(int64_t n, const std::vector<int>& radices) {
  std::vector<int> cur(n), nxt(n);
  for (int64_t i = 0; i < n; ++i) cur[i] = (int)i;
  int64_t len = n;
  for (int d = (int)radices.size() - 1; d >= 0; --d) {
    const int64_t r = radices[d], sub = len / r;
    for (int64_t blk = 0; blk < n; blk += len)
      for (int64_t k = 0; k < r; ++k)
        for (int64_t l = 0; l < sub; ++l) nxt[blk + k * sub + l] = cur[blk + l * r + k];
    len = sub;
    cur.swap(nxt);
  }
  return cur;
}

namespace {
template <typename E>
__global__ void scatter_natural_kernel(const E* __restrict__ in, E* __restrict__ out, const int* __restrict__ rev_x,
                                       const int* __restrict__ rev_y, long long nx, long long ny, long long total) {
  const long long per = nx * ny;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / per, r = e - b * per;
    const long long j = r / ny, k = r - j * ny;
    const long long dst = b * per + (long long)(rev_x ? rev_x[j] : j) * ny + rev_y[k];
    out[dst] = in[e];
  }
}
}  // namespace

// data (digit-reversed) -> tmp (natural), then tmp copied back into data.
cudaError_t to_natural_order(void* data, void* tmp, const int* rev_x, const int* rev_y, int64_t nx, int64_t ny,
                             int64_t batch, int es, int num_sms, cudaStream_t st) {
  const long long total = (long long)nx * ny * batch;
  const int threads = 256;
  long long blocks = (total + threads - 1) / threads;
  if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
  if (es == 4)
    scatter_natural_kernel<uint32_t><<<(int)blocks, threads, 0, st>>>(
        (const uint32_t*)data, (uint32_t*)tmp, rev_x, rev_y, nx, ny, total);
  else
    scatter_natural_kernel<uint2><<<(int)blocks, threads, 0, st>>>((const uint2*)data, (uint2*)tmp, rev_x, rev_y,
                                                                    nx, ny, total);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(data, tmp, total * es, cudaMemcpyDeviceToDevice, st);
}

}  // namespace tcfft
