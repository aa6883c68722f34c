// tcfft_gather.cu -- moves many variable-size contiguous blocks in one launch.
//
// An uneven batch (tcfftPlanMany) whose same-shape transforms are scattered
// through the caller's buffer is executed as: gather every shape group into a
// contiguous scratch run (one launch), one batched execute per shape, scatter
// back (one launch).  Block i is `len[i]` 16-byte chunks from src + src_off[i]
// to dst + dst_off[i] (byte offsets, 16-byte aligned); cum[i] = chunks before
// block i.  The grid strides over all chunks; a chunk finds its block by
// binary search in cum.
#include "tcfft_host.h"

namespace tcfft {
namespace {

__global__ void __launch_bounds__(256) move_blocks_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                          const long long* __restrict__ src_off,
                                                          const long long* __restrict__ dst_off,
                                                          const long long* __restrict__ cum, int nblocks,
                                                          long long total_chunks) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total_chunks;
       c += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = nblocks - 1;  // last block with cum <= c
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cum[mid] <= c) lo = mid;
      else hi = mid - 1;
    }
    const long long k = c - cum[lo];
    dst[dst_off[lo] / 16 + k] = src[src_off[lo] / 16 + k];
  }
}

}  // namespace

cudaError_t launch_move_blocks(const void* src, void* dst, const long long* src_off, const long long* dst_off,
                               const long long* cum, int nblocks, long long total_chunks, int num_sms,
                               cudaStream_t st) {
  if (nblocks <= 0 || total_chunks <= 0) return cudaSuccess;
  long long blocks = (total_chunks + 255) / 256;
  if (blocks > (long long)num_sms * 16) blocks = (long long)num_sms * 16;
  move_blocks_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst),
                                                       src_off, dst_off, cum, nblocks, total_chunks);
  return cudaGetLastError();
}

}  // namespace tcfft
