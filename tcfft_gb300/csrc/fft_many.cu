// fft_many.cu -- one persistent pass over the work items of many transforms of
// different shapes (tcfftPlanMany, plain precision).
//
// An uneven batch (1D transforms of 256..65536 points and 2D transforms with
// axes of 128..2048, at arbitrary 128-byte-aligned offsets of one buffer) runs
// as one launch of this kernel over two passes per transform:
//   pass A: 1D N <= 2048 whole (rows of 256R, several transforms per item),
//           1D N >= 4096 phase 0 (columns of N1, times W_N, into a scratch
//           region of the transform), 2D rows;
//   pass B: 1D N >= 4096 phase 1 (rows of N2 from the scratch, written
//           transposed into the transform), 2D columns.
// Columns-only transforms (the element strides of tcfftPlanStrided) have a pass B
// and no pass A.  Every transform has its own tensor maps (four per transform, in
// global memory), so no transform is moved to a batch of its shape first.  An
// item holds up to one 64 KiB stage: consecutive tiles of one transform side by
// side, or up to C whole 1D transforms of 256R points loaded through four
// buffer-wide maps (one per R).  The job bodies are those of the two-phase
// executor (fft_fused.cuh) and of the 16R-point jobs (fft_job.cuh); the four-step
// twiddles of every 1D size come from W_65536 in three shared-memory levels.
//
// CTA = 8 compute warps + 1 TMA-load warp + 1 TMA-store warp (the two-phase
// executor's structure).  The items form one sequence in which a transform's
// pass-B items follow its pass-A items a few hundred items later, so that its
// intermediate is read back from L2.  Each CTA's producer claims the next item
// from a global counter when a stage is free and hands its descriptor to the
// compute and store warps with the stage (kind -1 ends the CTA's work); a pass-B
// item is loaded once its transform's completion counter shows every pass-A item
// stored (release by the storer after the stores complete, acquire by the
// producer; bounded waits).  Pass-A items wait for nothing and are loaded as soon
// as they are claimed, so every wait ends.

#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

using MPI = BitPerm<0, 1, 3, 2>;  // the plain two-phase executor's slot permutations
using MRHO = BitPerm<0, 2, 3, 1>;

constexpr int kManyStage = 64 * 1024;  // bytes of one ring stage (the largest item)
// shared-memory tables: the plain fold tables of R = 2 and 4 and the A part of R = 8's;
// the T part of R = 8's is read from global memory (ManyParams::fold8_t), which leaves
// room for three stages
constexpr int kFold2 = 0, kFold4 = kFold2 + FoldTab<2>::kBytes, kFold8 = kFold4 + FoldTab<4>::kBytes;
constexpr int kWn3 = kFold8 + FoldTab<8>::kABytes;  // W_65536 in three levels: hi[64], mid[32], lo[32]
constexpr int kManyTab = kWn3 + 128 * 8;
constexpr int kManyBudget = 225 * 1024 - kManyTab - 1024 - 256;
constexpr int kManyStages = kManyBudget / kManyStage >= 3 ? 3 : kManyBudget / kManyStage;
static_assert(kManyStages >= 2, "at least two ring stages");
constexpr int kManySmem = kManyStages * kManyStage + kManyTab + 1024 + 256;
static_assert(3 * 8 * kManyStages + 16 * kManyStages <= 256, "barriers and descriptors fit the tail");

__device__ __forceinline__ uint32_t fold_of(uint32_t tab, int R) {
  return tab + (R == 2 ? kFold2 : R == 4 ? kFold4 : kFold8);
}

// W_N^e for any N dividing 65536, from W_65536 in three shared-memory levels:
// W_65536^x = hi[x >> 10] mid[(x >> 5) & 31] lo[x & 31], x = e (65536 / N) mod 65536.
struct Wn3 {
  uint32_t tab;  // hi at tab, mid at tab + 512, lo at tab + 768
  int scale;     // log2(65536 / N)
  int nmask;     // N - 1
  __device__ __forceinline__ float2 operator()(int e) const {
    const int x = (e & nmask) << scale;
    return cmul(cmul(lds64f(tab + (x >> 10) * 8), lds64f(tab + 512 + ((x >> 5) & 31) * 8)),
                lds64f(tab + 768 + (x & 31) * 8));
  }
};

// ---------------------------------------------------------------- job bodies (compute warps)

// C contiguous rows of 256R points, rows warp + 8 jn, in place (the two-phase
// executor's row role).
template <int R, int C>
__device__ __forceinline__ void many_rows(const JobConsts<false>& jc, uint32_t fold, uint32_t base, int warp,
                                          float dsign, const float2* tglob = nullptr) {
  constexpr int JN = C / 8;
  const uint32_t rb0 = base + (uint32_t)(warp * 256 * R * 4);
  uint32_t out[JN][R][8];
  plain_row_jobs<R, JN, MPI, MRHO>(jc, fold, rb0, 8 * 256 * R * 4, dsign, out, tglob);
#pragma unroll
  for (int jn = 0; jn < JN; ++jn)
#pragma unroll
    for (int sl = 0; sl < 8; ++sl) {
      const uint32_t rb = rb0 + (uint32_t)(8 * jn * 256 * R * 4);
      const int k0 = R * jc.kval[sl >> 2][(sl >> 1) & 1][sl & 1];
      if constexpr (R == 1) {
        sts32(rb + swz_w<4>(k0) * 4, out[jn][0][sl]);
      } else if constexpr (R == 2) {
        sts64(rb + swz_w<4>(k0) * 4, out[jn][0][sl], out[jn][1][sl]);
      } else {
#pragma unroll
        for (int q4 = 0; q4 < R; q4 += 4)
          sts128(rb + swz_w<4>(k0 + q4) * 4, out[jn][q4][sl], out[jn][q4 + 1][sl], out[jn][q4 + 2][sl],
                 out[jn][q4 + 3][sl]);
      }
    }
}

// C rows of 256R points (R = 1 here), written transposed as a column tile
// (the two-phase executor's row-transpose role).
template <int R, int C>
__device__ __forceinline__ void many_rows_t(const JobConsts<false>& jc, uint32_t fold, uint32_t base, int warp,
                                            float dsign) {
  constexpr int JN = C / 8;
  constexpr uint32_t kRow = 256 * R * 4;
  constexpr uint32_t kStep = 256 * C * 4;
  const int row0 = JN * warp;
  uint32_t out[JN][R][8];
  plain_row_jobs<R, JN, MPI, MRHO>(jc, fold, base + row0 * kRow, kRow, dsign, out);
  named_bar_sync(1, 256);  // every compute warp finished reading the stage
#pragma unroll
  for (int sl = 0; sl < 8; ++sl) {
    const uint32_t so = base + ctile_off<C, 4>(col_out_row(slot_kval<MPI, MRHO>(sl), 0), row0);
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if constexpr (JN == 4) {
        sts128(so + q * kStep, out[0][q][sl], out[1][q][sl], out[2][q][sl], out[3][q][sl]);
      } else {
#pragma unroll
        for (int jp = 0; jp < JN; jp += 2) sts64(so + jp * 4 + q * kStep, out[jp][q][sl], out[jp + 1][q][sl]);
      }
    }
  }
}

// 128 rows of 16R points (16 per warp), written transposed in boxes of 32
// columns (the two-phase executor's short-row role).
template <int R>
__device__ __forceinline__ void many_rows16_t(const JobConsts<false>& jc, uint32_t fold, uint32_t base, int warp,
                                              int lane, float dsign) {
  constexpr int L = 16 * R;
  uint32_t out[8 * R];
  {
    const uint32_t rb = base + (uint32_t)(warp * 16 * L * 4);
    auto ldr = [&](int v, int n) { return lds32(rb + swz_w<4>(v * L + n) * 4); };
    auto st = [&](int, int, int q, int sl, float2 val) { out[8 * q + sl] = pack_h2(val.x, val.y); };
    fft16r_job_fold<R, MPI, MRHO>(jc, fold, dsign, ldr, st);
  }
  named_bar_sync(1, 256);
  const int lane_g = lane >> 2, lane_t = lane & 3;
#pragma unroll
  for (int q = 0; q < R; ++q)
#pragma unroll
    for (int sl = 0; sl < 8; ++sl) {
      const int jj = sl >> 2, h = (sl >> 1) & 1, e = sl & 1;
      const int col = warp * 16 + 2 * lane_t + e + 8 * jj;
      const int row = MRHO::apply(lane_g + 8 * h) + 16 * q;
      sts32(base + (uint32_t)((col / 32) * (32 * L * 4)) + ctile_off<32, 4>(row, col % 32), out[8 * q + sl]);
    }
}

// 128 contiguous rows of 128 points (16 per warp), in place: the warp's loads all
// precede its stores (fft16r_job_fold), and no other warp touches its rows.
__device__ __forceinline__ void many_rows128(const JobConsts<false>& jc, uint32_t fold8, uint32_t base, int warp,
                                             float dsign) {
  const uint32_t rb = base + (uint32_t)(warp * 16 * 128 * 4);
  auto ldr = [&](int v, int n) { return lds32(rb + swz_w<4>(v * 128 + n) * 4); };
  auto st = [&](int v, int k, int, int, float2 val) { sts32(rb + swz_w<4>(v * 128 + k) * 4, pack_h2(val.x, val.y)); };
  fft16r_job_fold<8, MPI, MRHO>(jc, fold8, dsign, ldr, st);
}

// 128 columns of 128 points (16 per warp), in place; the tile is four boxes of
// [128 rows][32 columns] with the 128-byte swizzle.
__device__ __forceinline__ void many_cols128(const JobConsts<false>& jc, uint32_t fold8, uint32_t base, int warp,
                                             float dsign) {
  const uint32_t cb = base + (uint32_t)((warp >> 1) * (128 * 32 * 4));
  const int c0 = (warp & 1) * 16;
  auto ldr = [&](int v, int n) { return lds32(cb + ctile_off<32, 4>(n, c0 + v)); };
  auto st = [&](int v, int k, int, int, float2 val) { sts32(cb + ctile_off<32, 4>(k, c0 + v), pack_h2(val.x, val.y)); };
  fft16r_job_fold<8, MPI, MRHO>(jc, fold8, dsign, ldr, st);
}

// ---------------------------------------------------------------- TMA per kind (one thread)
// The maps live in global memory and are rewritten by the host when the data
// buffer changes: order this thread's tensor-map reads after those writes.
__device__ __forceinline__ const CUtensorMap* tmap_acquire(const CUtensorMap* m, int count) {
  for (int i = 0; i < count; ++i)
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m + i) : "memory");
  return m;
}

__device__ __forceinline__ int ilog2_small(int v) { return v >= 8 ? 3 : v >= 4 ? 2 : v >= 2 ? 1 : 0; }
// Bytes of one tile of a (non-listed) kind.
__device__ __forceinline__ uint32_t tile_bytes(int kind) { return (uint32_t)many_item_elems(kind) * 4u; }

// Bytes an item moves (listed rows: `count` transforms of 256R points).
__device__ __forceinline__ uint32_t item_bytes(const ManyItem& it) {
  const int kind = it.kind & 0xff;
  if (it.kind & kMkList) return (uint32_t)it.count * 256u * (uint32_t)many_r(kind) * 4u;
  return (uint32_t)it.nsub * tile_bytes(kind);
}

__device__ __forceinline__ void many_load(const ManyParams& p, const ManyItem& it, unsigned char* dst, uint64_t* bar) {
  const int kind = it.kind & 0xff;
  const int R = many_r(kind), C = many_c(kind);
  if (it.kind & kMkList) {  // whole transforms of 256R points, one box each, through the buffer-wide map
    const CUtensorMap* bm = tmap_acquire(p.maps + 4 * (size_t)p.n_xf + ilog2_small(R), 1);
    for (int j = 0; j < it.count; ++j) tma_load_2d(dst + j * (256 * R * 4), bm, 0, p.row_list[it.xf + j], bar);
    return;
  }
  const CUtensorMap* m = tmap_acquire(p.maps + 4 * (size_t)it.xf, 4);
  const uint32_t tb = tile_bytes(kind);
  switch (kind) {
    case kMkRow1: case kMkRow2: case kMkRow4: case kMkRow8: {  // consecutive rows of one transform
      const int rows = C * 256 * R / 32, bh = rows < 256 ? rows : 256;
      for (int i = 0; i < it.nsub * rows / bh; ++i)
        tma_load_2d(dst + i * bh * 128, m, 0, it.tile * rows + i * bh, bar);
      break;
    }
    case kMkColWn1x16: case kMkColWn1x32: case kMkColWn2x32:
      for (int u = 0; u < it.nsub; ++u) tma_load_5d(dst + u * tb, m, (it.tile + u) * C, 0, 0, 0, 0, bar);
      break;
    case kMkRowT1:  // 32 rows of 256 from the scratch: 256 rows of 128 bytes per tile
      for (int u = 0; u < it.nsub; ++u) tma_load_2d(dst + u * tb, m + 2, 0, (it.tile + u) * 256, bar);
      break;
    case kMkRow16T1: case kMkRow16T2: case kMkRow16T4:  // 128 rows of 16R: 64R rows of 128 bytes per tile
      for (int u = 0; u < it.nsub; ++u) tma_load_2d(dst + u * tb, m + 2, 0, (it.tile + u) * 64 * R, bar);
      break;
    case kMkCol1: case kMkCol2: case kMkCol4: case kMkCol8:
      for (int u = 0; u < it.nsub; ++u) tma_load_5d(dst + u * tb, m + 2, (it.tile + u) * C, 0, 0, 0, 0, bar);
      break;
    case kMkRow128:  // 128 rows of 128 points: 512 rows of 128 bytes, two boxes
      tma_load_2d(dst, m, 0, it.tile * 512, bar);
      tma_load_2d(dst + 256 * 128, m, 0, it.tile * 512 + 256, bar);
      break;
    case kMkCol128:  // 128 columns: four boxes of 32 columns x 128 rows
      for (int b = 0; b < 4; ++b) tma_load_2d(dst + b * (128 * 32 * 4), m + 2, it.tile * 128 + 32 * b, 0, bar);
      break;
    default:
      break;
  }
}

__device__ __forceinline__ void many_store(const ManyParams& p, const ManyItem& it, const unsigned char* src) {
  const int kind = it.kind & 0xff;
  const int R = many_r(kind), C = many_c(kind);
  if (it.kind & kMkList) {
    const CUtensorMap* bm = tmap_acquire(p.maps + 4 * (size_t)p.n_xf + ilog2_small(R), 1);
    for (int j = 0; j < it.count; ++j) tma_store_2d(bm, 0, p.row_list[it.xf + j], src + j * (256 * R * 4));
    return;
  }
  const CUtensorMap* m = tmap_acquire(p.maps + 4 * (size_t)it.xf, 4);
  const uint32_t tb = tile_bytes(kind);
  switch (kind) {
    case kMkRow1: case kMkRow2: case kMkRow4: case kMkRow8: {
      const int rows = C * 256 * R / 32, bh = rows < 256 ? rows : 256;
      for (int i = 0; i < it.nsub * rows / bh; ++i)
        tma_store_2d(m, 0, it.tile * rows + i * bh, src + i * bh * 128);
      break;
    }
    case kMkColWn1x16: case kMkColWn1x32: case kMkColWn2x32:  // into the transform's scratch
      for (int u = 0; u < it.nsub; ++u) tma_store_5d(m + 1, (it.tile + u) * C, 0, 0, 0, 0, src + u * tb);
      break;
    case kMkRowT1:  // output columns k1 of [N2 rows k2][N1 cols k1]
      for (int u = 0; u < it.nsub; ++u) tma_store_5d(m + 3, (it.tile + u) * C, 0, 0, 0, 0, src + u * tb);
      break;
    case kMkRow16T1: case kMkRow16T2: case kMkRow16T4:  // 4D [N1][k0][q][1], boxes of 32 columns
      for (int u = 0; u < it.nsub; ++u)
        for (int bx = 0; bx < 4; ++bx)
          tma_store_4d(m + 3, (it.tile + u) * 128 + bx * 32, 0, 0, 0, src + u * tb + bx * (32 * 16 * R * 4));
      break;
    case kMkCol1: case kMkCol2: case kMkCol4: case kMkCol8:
      for (int u = 0; u < it.nsub; ++u) tma_store_5d(m + 3, (it.tile + u) * C, 0, 0, 0, 0, src + u * tb);
      break;
    case kMkRow128:
      tma_store_2d(m, 0, it.tile * 512, src);
      tma_store_2d(m, 0, it.tile * 512 + 256, src + 256 * 128);
      break;
    case kMkCol128:
      for (int b = 0; b < 4; ++b) tma_store_2d(m + 2, it.tile * 128 + 32 * b, 0, src + b * (128 * 32 * 4));
      break;
    default:
      break;
  }
}

__global__ void __launch_bounds__(384, 1) fft_many_kernel(const __grid_constant__ ManyParams p) {
  constexpr int NST = kManyStages;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* s_tab = smem + NST * kManyStage;
  uint64_t* full = reinterpret_cast<uint64_t*>(s_tab + kManyTab);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;
  ManyItem* s_meta = reinterpret_cast<ManyItem*>(empty + NST);  // descriptor of each stage's item
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned long long lim = p.wait_ns ? p.wait_ns : kTimeoutNs;

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
    }
    fence_barrier_init();
  }
  build_fold_table<2, MPI, MRHO>(s_tab + kFold2, p.tw2048, tid, blockDim.x);
  build_fold_table<4, MPI, MRHO>(s_tab + kFold4, p.tw2048, tid, blockDim.x);
  build_fold_table<8, MPI, MRHO, false>(s_tab + kFold8, p.tw2048, tid, blockDim.x);
  if (tid < 128) reinterpret_cast<float2*>(s_tab + kWn3)[tid] = p.wn3[p.dir][tid];
  __syncthreads();

  if (warp >= 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(56));
  if (warp >= 10) return;
  if (warp == 8) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int cnt = 0;
      bool failed = false;
      // the next item is claimed, read and its maps prefetched before the wait for a free
      // stage, so that their latency overlaps the work already in flight; in the last two
      // rounds of the grid the claim waits for the free stage instead, so that no CTA sits on
      // items that an idle CTA could run
      int last = -1;
      auto claim = [&](ManyItem& it) {
        const int idx = atomicAdd(p.claim, 1);
        last = idx;
        if (idx >= p.n_items) {
          it.kind = -1;
          return;
        }
        it = p.items[idx];
        if (!(it.kind & kMkList)) {
          const CUtensorMap* m = p.maps + 4 * (size_t)it.xf;
          for (int i = 0; i < 4; ++i) prefetch_tmap(m + i);
        }
      };
      ManyItem it;
      bool have = false;
      while (true) {
        const int s = cnt % NST;
        if (!mbar_wait(&empty[s], ((cnt / NST) + 1) & 1, p.err, lim)) {
          failed = true;
          break;
        }
        if (!have) claim(it);
        have = false;
        if (it.kind < 0) {  // the end of the work: a descriptor of kind -1, no bytes
          s_meta[s].kind = -1;
          mbar_arrive(&full[s]);
          break;
        }
        if (it.kind & kMkB) {  // every pass-A item of the transform stored
          if (!wait_counter(&p.done[it.xf], it.count, p.err, lim)) {
            failed = true;
            break;
          }
          fence_proxy_async_global();
        }
        unsigned char* dst = smem + s * kManyStage;
        s_meta[s] = it;  // published to the other warps by the arrive below
        mbar_arrive_expect_tx(&full[s], item_bytes(it));
        many_load(p, it, dst, &full[s]);
        ++cnt;
        if (last + 2 * (int)gridDim.x < p.n_items) {
          claim(it);
          have = true;
        }
      }
      // on an early exit let the loads still in flight land before the CTA ends (bounded); on the
      // normal exit the compute warps have waited for every load
      if (failed)
        for (int i = (cnt > NST ? cnt - NST : 0); i < cnt; ++i) mbar_wait(&full[i % NST], (i / NST) & 1, nullptr);
    }
    return;
  }
  if (warp == 9) {
    // ------------------------------------------------------------ TMA storer
    // A pass-A item's completion is released (done[xf] += 1) once its stores are
    // complete: up to kMaxPending stay in flight, and before the storer blocks it
    // releases every pending one, so a producer waiting on this CTA's output never
    // waits behind this CTA's own pipeline.
    if (lane == 0) {
      constexpr int kMaxPending = 2;
      int* pend[kMaxPending + 1];
      int npend = 0;
      auto release_all = [&]() {
        if (npend == 0) return;
        bulk_wait<0>();
        fence_proxy_async_global();
        for (int i = 0; i < npend; ++i)
          if (pend[i]) red_release_add(pend[i], 1);
        npend = 0;
      };
      auto wait_stage = [&](uint64_t* bar, uint32_t par) {
        if (mbar_try_wait(bar, par)) return true;
        release_all();
        return mbar_wait(bar, par, p.err, lim);
      };
      int cnt = 0;
      while (true) {
        const int s = cnt % NST;
        // the stage's descriptor first (the end of the work has no computed phase)
        if (!wait_stage(&full[s], (cnt / NST) & 1)) break;
        const ManyItem it = s_meta[s];
        if (it.kind < 0) break;
        if (!wait_stage(&computed[s], (cnt / NST) & 1)) break;
        many_store(p, it, smem + s * kManyStage);
        bulk_commit();
        if (it.kind & kMkRelease) pend[npend++] = &p.done[it.xf];
        else if (npend > 0) pend[npend++] = nullptr;  // keeps the groups and entries in step
        bulk_wait_read<0>();  // the stage has been read: the producer may refill it
        mbar_arrive(&empty[s]);
        if (npend > kMaxPending) {
          // the oldest group is complete once at most kMaxPending remain
          bulk_wait<kMaxPending>();
          fence_proxy_async_global();
          if (pend[0]) red_release_add(pend[0], 1);
          for (int i = 1; i < npend; ++i) pend[i - 1] = pend[i];
          --npend;
        }
        ++cnt;
      }
      release_all();
      bulk_wait<0>();
    }
    return;
  }

  // -------------------------------------------------------------- compute warps
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(224));
  JobConsts<false> jc;
  init_job_consts<false, MPI, MRHO>(jc, p.tw2048);
  const uint32_t tab = smem_addr(s_tab);
  int cnt = 0;
  while (true) {
    const int s = cnt % NST;
    const bool ok = named_bar_and(2, 256, mbar_wait(&full[s], (cnt / NST) & 1, p.err, lim));
    const ManyItem it = s_meta[s];
    if (ok && it.kind < 0) break;  // end of the pass (every compute warp sees the same descriptor)
    const uint32_t stage = smem_addr(smem + s * kManyStage);
    const int kind = it.kind & 0xff;
    const int nsub = (it.kind & kMkList) ? 1 : it.nsub;
#pragma unroll 1
    for (int u = 0; ok && u < nsub; ++u) {
      const uint32_t base = stage + u * tile_bytes(kind);
      const int tile = it.tile + u;
      switch (kind) {
        case kMkRow1: many_rows<1, 32>(jc, tab, base, warp, p.dsign); break;
        case kMkRow2: many_rows<2, 32>(jc, fold_of(tab, 2), base, warp, p.dsign); break;
        case kMkRow4: many_rows<4, 16>(jc, fold_of(tab, 4), base, warp, p.dsign); break;
        case kMkRow8: many_rows<8, 8>(jc, fold_of(tab, 8), base, warp, p.dsign, p.fold8_t[p.dir]); break;
        case kMkColWn1x16: case kMkColWn1x32: case kMkColWn2x32: {
          Wn3 wn;
          wn.tab = tab + kWn3;
          wn.nmask = it.wn;  // N - 1
          wn.scale = 16 - (31 - __clz(wn.nmask + 1));
          if (kind == kMkColWn1x16)
            plain_col_tile<1, 16, true, MPI, MRHO, 2, Wn3>(jc, tab, base, warp, p.dsign, tile * 16, wn);
          else if (kind == kMkColWn1x32)
            plain_col_tile<1, 32, true, MPI, MRHO, 4, Wn3>(jc, tab, base, warp, p.dsign, tile * 32, wn);
          else
            plain_col_tile<2, 32, true, MPI, MRHO, 4, Wn3>(jc, fold_of(tab, 2), base, warp, p.dsign, tile * 32, wn);
          break;
        }
        case kMkRowT1: many_rows_t<1, 32>(jc, tab, base, warp, p.dsign); break;
        case kMkRow16T1: many_rows16_t<1>(jc, tab, base, warp, lane, p.dsign); break;
        case kMkRow16T2: many_rows16_t<2>(jc, fold_of(tab, 2), base, warp, lane, p.dsign); break;
        case kMkRow16T4: many_rows16_t<4>(jc, fold_of(tab, 4), base, warp, lane, p.dsign); break;
        case kMkCol1: case kMkCol2: case kMkCol4: case kMkCol8: {
          WnTable wn;  // unused without the W_N twiddle
          wn.hi = wn.lo = 0;
          wn.ghi = wn.glo = nullptr;
          wn.global = true;
          wn.shift = 0;
          wn.nmask = 0;
          if (kind == kMkCol1) plain_col_tile<1, 32, false, MPI, MRHO>(jc, tab, base, warp, p.dsign, 0, wn);
          else if (kind == kMkCol2)
            plain_col_tile<2, 32, false, MPI, MRHO>(jc, fold_of(tab, 2), base, warp, p.dsign, 0, wn);
          else if (kind == kMkCol4)
            plain_col_tile<4, 16, false, MPI, MRHO>(jc, fold_of(tab, 4), base, warp, p.dsign, 0, wn);
          else
            plain_col_tile<8, 8, false, MPI, MRHO>(jc, fold_of(tab, 8), base, warp, p.dsign, 0, wn, 1.f,
                                                   p.fold8_t[p.dir]);
          break;
        }
        case kMkRow128: many_rows128(jc, fold_of(tab, 8), base, warp, p.dsign); break;
        case kMkCol128: many_cols128(jc, fold_of(tab, 8), base, warp, p.dsign); break;
        default: break;
      }
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&computed[s]);
    if (!ok) break;
    ++cnt;
  }
}

__global__ void __launch_bounds__(256) many_fold8_kernel(unsigned char* out, const float2* tw2048) {
  build_fold_table<8, MPI, MRHO>(out, tw2048, threadIdx.x, blockDim.x);
}

}  // namespace

int many_stages() { return kManyStages; }
int many_fold8_bytes() { return FoldTab<8>::kBytes; }
int many_fold8_t_offset() { return FoldTab<8>::kABytes; }
cudaError_t many_fold8_init(unsigned char* out, const float2* tw2048, cudaStream_t st) {
  many_fold8_kernel<<<1, 256, 0, st>>>(out, tw2048);
  return cudaGetLastError();
}

cudaError_t launch_many(const ManyParams& p, int num_sms, cudaStream_t st) {
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [] {
    init_err = cudaFuncSetAttribute(fft_many_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kManySmem);
  });
  if (init_err != cudaSuccess) return init_err;
  if (p.n_items <= 0) return cudaSuccess;
  const int grid = p.n_items < num_sms ? p.n_items : num_sms;
  fft_many_kernel<<<grid, 384, kManySmem, st>>>(p);
  return cudaGetLastError();
}

}  // namespace tcfft
