// fft_resident.cu -- 1D FFTs of N = 256 x 16 R1 (R1 = 1, 2, 4, 8: N = 4096, 8192,
// 16384, 32768) held entirely in one CTA's shared memory (32768: a variant with one
// transform in two stages, after the first kernel below).
//
// Same four-step factorisation as the two-phase kernel (fft_fused.cuh), but a
// whole transform (16-64 KiB) fits in one 64 KiB stage, so both phases run on
// the stage in place: no scratch ring, no cross-CTA dependency, and HBM is
// touched once per element each way with contiguous TMA copies.  (The
// reference has no sizes between 1024 and 2^17, tcfft_half.cu:1250-1330.)
//
//   stage = T transforms (T = 16 KiB-transforms per 64 KiB), loaded as column
//           tiles of the [256 rows n1][N2 cols n2] view (5D boxes in the
//           digit-ordered row layout of the column role, one box per group of
//           C <= 32 columns);
//   phase 0: 256-point column FFTs (plain_col_tile) times W_N^(n2 k1);
//   phase 1: N2-point FFTs of the 256 rows k1, 16 rows per warp job
//           (fft16r_job_q_fold, 16-byte loads), results held in registers;
//   output: after a barrier, X[k1 + 256 k2] written into the stage in a
//           digit order of (k1, k2) and stored with one 5D TMA box per stage.
//
// Bank conflicts (the former natural-order write-back hit one bank 8 times
// per instruction): a job's 16 rows are the k1 of one 16-aligned group with
// the row digits permuted (kap_of) so that the two rows a quarter-warp reads
// sit in different halves of the 128-byte bank window, and the lanes of one
// output store differ in k1 bits 0-1 (one 16-byte chunk) and in the k2 bits
// that select the stage row's swizzle phase (8 different chunks).
#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

template <int R1>
struct ResCfg {
  static constexpr int kN2 = 16 * R1;
  static constexpr int kN = 256 * kN2;
  static constexpr int kC = kN2 < 32 ? kN2 : 32;          // columns per column tile
  static constexpr int kCG = kN2 / kC;                     // column tiles per transform
  static constexpr int kT = 65536 / (kN * 4);              // transforms per stage
  static constexpr int kTileBytes = 256 * kC * 4;          // one column tile
  static constexpr int kStageBytes = 65536;
  static constexpr int kStages = 3;
  static constexpr int kLog2N = 8 + 4 + (R1 == 1 ? 0 : (R1 == 2 ? 1 : 2));
  static constexpr int kTwShift = (kLog2N + 1) / 2;
  static constexpr int kTwLo = 1 << kTwShift, kTwHi = kN >> kTwShift;
  static constexpr int kTabBytes = (kTwLo + kTwHi + kN2) * 8 + FoldTab<R1>::kBytes;  // + phase-1 fold table
  static constexpr int kSmem = kStages * kStageBytes + kTabBytes + 1024 + 256;
  static constexpr int kThreads = 384;
  static constexpr int kL = R1 == 1 ? 0 : (R1 == 2 ? 1 : 2);  // log2 R1
  using PI = BitPerm<0, 1, 3, 2>;   // phase 0 (column jobs)
  using PI1 = BitPerm<0, 2, 3, 1>;  // phase 1: lane t reads points 4t .. 4t + 3
  using RHO = BitPerm<0, 2, 3, 1>;
  static_assert(kT >= 1 && kT * kN * 4 == kStageBytes, "a stage holds whole transforms");
};

// Row k1 of transform-row v (0..15) in phase-1 job jl (0..15): a bit permutation
// of k1 = 16 jl + v.  v bit 0 goes to the k1 bit that makes the tile rows of
// v and v + 1 differ in the bank half (tile row bit 0 for 64-byte rows, bit 2
// for 128-byte rows); v bits 1-2 go to k1 bits 0-1 (the output chunk).
template <int C>
__device__ __forceinline__ int kap_of(int v, int jl) {
  const int v0 = v & 1, v1 = (v >> 1) & 1, v2 = (v >> 2) & 1, v3 = (v >> 3) & 1;
  if constexpr (C == 16) return v1 | (v2 << 1) | (v0 << 2) | (v3 << 3) | (jl << 4);
  else return v1 | (v2 << 1) | ((jl & 1) << 2) | (v3 << 3) | (v0 << 4) | ((jl >> 1) << 5);
}

// Stage row (128-byte rows of 32 k1, 128B swizzle) of output X[k1 + 256 k2] of
// stage transform t: rho = k2 bit L | (k2 bits L+2..L+3, t) << 1 |
// (k2 bit L+1 | (k1 >> 5 | (k2 & (R1 - 1)) << 3) << 1) << (3 + log2 T).
template <int R1>
__device__ __forceinline__ int res_rho(int kap, int k2, int t) {
  constexpr int L = ResCfg<R1>::kL, T = ResCfg<R1>::kT;
  return ((k2 >> L) & 1) +
         2 * ((((k2 >> (L + 2)) & 3) + 4 * t) + 4 * T * (((k2 >> (L + 1)) & 1) + 2 * ((kap >> 5) + 8 * (k2 & (R1 - 1)))));
}

struct ResParams {
  const float2* tw2048;
  const float2* twlo;
  const float2* twhi;
  long long batch;
  long long rows;  // transposed output: transforms per matrix (the destination's row length)
  int* err;
  float dsign;
  float oscale;  // output scale (a power of two), carried by the phase-0 W_N factors
};

// TOUT (N = 4096): the output is written transposed, as dst[m][k][r] for transform
// m * rows + r (a [rows][4096] matrix of transforms becomes the [4096][rows] matrix of
// their outputs), out of place.  The stage's four transforms are adjacent rows r, so
// after the natural-order write-back all compute threads re-read it as 16-byte
// groups of 4 outputs of one transform and write 16-byte groups of one output of the
// 4 transforms, in the layout of a 5D box (r: 4, k bits 2-4, k bits 0-1, k bits 5-11,
// matrix): both passes one wavefront per quarter-warp.
template <int R1, bool TOUT>
__global__ void __launch_bounds__(384, 1) fft_resident_kernel(const __grid_constant__ CUtensorMap load_map,
                                                               const __grid_constant__ CUtensorMap store_map,
                                                               const ResParams p) {
  using Cfg = ResCfg<R1>;
  using PI = typename Cfg::PI;
  using PI1 = typename Cfg::PI1;
  using RHO = typename Cfg::RHO;
  constexpr int NST = Cfg::kStages, T = Cfg::kT, CG = Cfg::kCG, C = Cfg::kC, L = Cfg::kL;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* tab = smem + NST * Cfg::kStageBytes;
  float2* s_twlo = reinterpret_cast<float2*>(tab);
  float2* s_twhi = s_twlo + Cfg::kTwLo;
  float2* s_tw16 = s_twhi + Cfg::kTwHi;  // W_{N2}^j
  unsigned char* s_fold = reinterpret_cast<unsigned char*>(s_tw16 + Cfg::kN2);
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + Cfg::kTabBytes);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long tiles = (p.batch + T - 1) / T;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
    }
    fence_barrier_init();
  }
  for (int j = tid; j < Cfg::kTwLo; j += blockDim.x) s_twlo[j] = p.twlo[j];
  for (int j = tid; j < Cfg::kTwHi; j += blockDim.x) s_twhi[j] = p.twhi[j];
  for (int j = tid; j < Cfg::kN2; j += blockDim.x) s_tw16[j] = p.tw2048[j * (2048 / Cfg::kN2)];
  build_fold_table<R1, PI1, RHO>(s_fold, p.tw2048, tid, blockDim.x);  // phase-1 radix-R1 fold
  __syncthreads();

  if (warp >= 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(56));
  if (warp >= 10) return;
  if (warp == 8) {  // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&load_map);
      int cnt = 0;
      for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&empty[s], ((cnt / NST) + 1) & 1, p.err)) break;
        unsigned char* dst = smem + s * Cfg::kStageBytes;
        mbar_arrive_expect_tx(&full[s], Cfg::kStageBytes);
#pragma unroll 1
        for (int t = 0; t < T; ++t)
#pragma unroll 1
          for (int cg = 0; cg < CG; ++cg)
            tma_load_5d(dst + (t * CG + cg) * Cfg::kTileBytes, &load_map, cg * C, 0, 0, 0, (int)(it * T + t),
                        &full[s]);
      }
      for (int i = (cnt > NST ? cnt - NST : 0); i < cnt; ++i) mbar_wait(&full[i % NST], (i / NST) & 1, nullptr);
    }
    return;
  }
  if (warp == 9) {  // ------------------------------------------------ TMA storer
    if (lane == 0) {
      prefetch_tmap(&store_map);
      int cnt = 0;
      for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&computed[s], (cnt / NST) & 1, p.err)) break;
        const unsigned char* src = smem + s * Cfg::kStageBytes;
        if constexpr (TOUT) {
          const long long m0 = it * T;  // first transform of the stage
          tma_store_5d(&store_map, (int)(m0 % p.rows), 0, 0, 0, (int)(m0 / p.rows), src);
        } else {
          tma_store_5d(&store_map, 0, 0, (int)(4 * T * it), 0, 0, src);
        }
        bulk_commit();
        bulk_wait_read<0>();
        mbar_arrive(&empty[s]);
      }
      bulk_wait<0>();
    }
    return;
  }

  // ------------------------------------------------------------------ compute warps
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(224));
  JobConsts<false> jc, jc1;
  init_job_consts<false, PI, RHO>(jc, p.tw2048);
  init_job_consts<false, PI1, RHO>(jc1, p.tw2048);
  const uint32_t fold = smem_addr(s_fold), tw16 = smem_addr(s_tw16);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = false;
  wn.shift = Cfg::kTwShift;
  wn.nmask = Cfg::kN - 1;
  const int g = lane >> 2, tq = lane & 3;
  int cnt = 0;
  for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
    const int s = cnt % NST;
    const bool ok = named_bar_and(2, 256, mbar_wait(&full[s], (cnt / NST) & 1, p.err));
    const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes);
    if (ok) {
      // phase 0: columns of 256 (in place, digit-ordered rows), twiddle W_N^(n2 k1)
#pragma unroll 1
      for (int tile = 0; tile < T * CG; ++tile) {
        if constexpr (C == 32 && R1 == 4) {
          // one-transform stages (16384): two passes of two columns, fewer live registers than
          // one of four (0.641 -> 0.534 ms for 2^28 elements; 8192 measured better with four)
#pragma unroll 1
          for (int h = 0; h < 2; ++h)
            plain_col_tile<1, C, true, PI, RHO, 2>(jc, fold, base + tile * Cfg::kTileBytes, warp + 8 * h,
                                                   p.dsign, (tile % CG) * C, wn, p.oscale);
        } else {
          plain_col_tile<1, C, true, PI, RHO>(jc, fold, base + tile * Cfg::kTileBytes, warp, p.dsign,
                                              (tile % CG) * C, wn, p.oscale);
        }
      }
      named_bar_sync(1, 256);
      // phase 1: 16 rows k1 per job, FFT over n2 (length 16 R1); jobs j = warp + 8 i
      constexpr int JOBS = 2 * T;  // per warp: 16 T jobs per stage / 8 warps
      uint32_t out[JOBS][8 * R1];
#pragma unroll
      for (int i = 0; i < JOBS; ++i) {
        const int job = warp + 8 * i, t = job >> 4, jl = job & 15;
        const uint32_t tbase = base + t * (CG * Cfg::kTileBytes);
        auto ld4 = [&](int v, int a, uint32_t(&w)[4]) {
          const int n = 4 * tq + 16 * a;
          lds128(tbase + (n / C) * Cfg::kTileBytes + ctile_off<C, 4>(col_out_row(kap_of<C>(v, jl), 0), n % C), w);
        };
        auto st = [&](int, int, int q, int slot, float2 val) { out[i][8 * q + slot] = pack_h2(val.x, val.y); };
        fft16r_job_q_fold<R1, PI1, RHO>(jc1, fold, p.dsign, ld4, st);
      }
      named_bar_sync(1, 256);  // every warp has read the stage
      // X[k1 + 256 k2] of transform t at stage row rho (128-byte rows of 32 k1, 128B swizzle):
      // rho = k2 bit L | (k2 bits L+2..L+3, t) << 1 | k2 bit L+1 << (3 + log2 T) |
      //       (k1 >> 5 | (k2 & (R1 - 1)) << 3) << (4 + log2 T); the store box has these digits as dims
#pragma unroll
      for (int i = 0; i < JOBS; ++i) {
        const int job = warp + 8 * i, t = job >> 4, jl = job & 15;
#pragma unroll
        for (int q = 0; q < R1; ++q)
#pragma unroll
          for (int slot = 0; slot < 8; ++slot) {
            const int jj = slot >> 2, h = (slot >> 1) & 1, e = slot & 1;
            const int kap = kap_of<C>(2 * tq + e + 8 * jj, jl), k2 = q + R1 * RHO::apply(g + 8 * h);
            const int rho = res_rho<R1>(kap, k2, t);
            sts32(base + swz_w<4>((uint32_t)((kap & 31) + 32 * rho)) * 4, out[i][8 * q + slot]);
          }
      }
      if constexpr (TOUT) {
        static_assert(R1 == 1 && T == 4, "transposed output: four 4096-point transforms per stage");
        named_bar_sync(1, 256);  // natural-order write-back complete
        uint32_t w[4][4][4];     // [group][transform][output]
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int gi = threadIdx.x + 256 * i, K = 4 * (gi & 7) + 32 * (gi >> 3);
#pragma unroll
          for (int t = 0; t < 4; ++t)
            lds128(base + swz_w<4>((uint32_t)((K & 31) + 32 * res_rho<1>(K & 255, K >> 8, t))) * 4, w[i][t]);
        }
        named_bar_sync(1, 256);  // every group read before any is overwritten
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int gi = threadIdx.x + 256 * i, K = 4 * (gi & 7) + 32 * (gi >> 3);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            sts128(base + 16 * (((K >> 2) & 7) + 8 * j + 32 * (K >> 5)), w[i][0][j], w[i][1][j], w[i][2][j],
                   w[i][3][j]);
        }
      }
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&computed[s]);
    if (!ok) break;
  }
}

// ---------------------------------------------------------------------------
// Split precision (fp32 complex in and out, hi/lo fp16 operands, three tensor-core
// products per stage): N = 4096 (two transforms per 64 KiB stage) and 8192 (one).
// Same schedule as the plain kernel: column tiles of 16 columns (128-byte rows of
// 8-byte elements), the 256-point split column jobs with W_N, the 16 R1-point
// split row jobs of 16 rows, natural-order write-back, 128-byte-row stores.
template <int R1>
struct ResSplitCfg {
  static constexpr int kES = 8;
  static constexpr int kN2 = 16 * R1, kN = 256 * kN2;
  static constexpr int kC = 16;
  static constexpr int kCG = kN2 / kC;
  static constexpr int kTileBytes = 256 * kC * kES;
  static constexpr int kStageBytes = 65536;
  static constexpr int kT = kStageBytes / (kN * kES);
  static constexpr int kStages = 3;
  static constexpr int kLog2N = R1 == 1 ? 12 : 13;
  static constexpr int kTwShift = (kLog2N + 1) / 2;
  static constexpr int kTwLo = 1 << kTwShift, kTwHi = kN >> kTwShift;
  static constexpr int kTabBytes = (kTwLo + kTwHi + kN2) * 8;
  static constexpr int kSmem = kStages * kStageBytes + kTabBytes + 1024 + 256;
  static constexpr int kThreads = 384;
  using PI = BitPerm<0, 1, 2, 3>;
  using RHO = BitPerm<0, 2, 3, 1>;
  static_assert(kT >= 1 && kT * kN * kES == kStageBytes, "a stage holds whole transforms");
};

template <int R1, bool SPLIT>  // SPLIT: three products per stage; else fp16 operands (fp32-I/O mode)
__global__ void __launch_bounds__(384, 1) fft_resident_split_kernel(const __grid_constant__ CUtensorMap load_map,
                                                                     const __grid_constant__ CUtensorMap store_map,
                                                                     const ResParams p) {
  using Cfg = ResSplitCfg<R1>;
  using PI = typename Cfg::PI;
  using RHO = typename Cfg::RHO;
  constexpr int NST = Cfg::kStages, T = Cfg::kT, CG = Cfg::kCG, C = Cfg::kC, ES = Cfg::kES;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* tab = smem + NST * Cfg::kStageBytes;
  float2* s_twlo = reinterpret_cast<float2*>(tab);
  float2* s_twhi = s_twlo + Cfg::kTwLo;
  float2* s_tw16 = s_twhi + Cfg::kTwHi;  // W_{N2}^j
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + Cfg::kTabBytes);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long tiles = (p.batch + T - 1) / T;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
    }
    fence_barrier_init();
  }
  for (int j = tid; j < Cfg::kTwLo; j += blockDim.x) s_twlo[j] = p.twlo[j];
  for (int j = tid; j < Cfg::kTwHi; j += blockDim.x) s_twhi[j] = p.twhi[j];
  for (int j = tid; j < Cfg::kN2; j += blockDim.x) s_tw16[j] = p.tw2048[j * (2048 / Cfg::kN2)];
  __syncthreads();

  if (warp >= 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(56));
  if (warp >= 10) return;
  if (warp == 8) {  // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&load_map);
      int cnt = 0;
      for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&empty[s], ((cnt / NST) + 1) & 1, p.err)) break;
        unsigned char* dst = smem + s * Cfg::kStageBytes;
        mbar_arrive_expect_tx(&full[s], Cfg::kStageBytes);
#pragma unroll 1
        for (int t = 0; t < T; ++t)
#pragma unroll 1
          for (int cg = 0; cg < CG; ++cg)
            tma_load_5d(dst + (t * CG + cg) * Cfg::kTileBytes, &load_map, cg * C, 0, 0, 0,
                        col_blk<true>((int)(it * T + t), 1), &full[s]);
      }
      for (int i = (cnt > NST ? cnt - NST : 0); i < cnt; ++i) mbar_wait(&full[i % NST], (i / NST) & 1, nullptr);
    }
    return;
  }
  if (warp == 9) {  // ------------------------------------------------ TMA storer
    if (lane == 0) {
      prefetch_tmap(&store_map);
      int cnt = 0;
      for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&computed[s], (cnt / NST) & 1, p.err)) break;
        const unsigned char* src = smem + s * Cfg::kStageBytes;
        const int row0 = (int)(it * (Cfg::kStageBytes / 128));
#pragma unroll 1
        for (int b = 0; b < Cfg::kStageBytes / (256 * 128); ++b)
          tma_store_2d(&store_map, 0, row0 + 256 * b, src + b * 256 * 128);
        bulk_commit();
        bulk_wait_read<0>();
        mbar_arrive(&empty[s]);
      }
      bulk_wait<0>();
    }
    return;
  }

  // ------------------------------------------------------------------ compute warps
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(224));
  JobConsts<SPLIT> jc;
  init_job_consts<SPLIT, PI, RHO>(jc, p.tw2048);
  const uint32_t tw16 = smem_addr(s_tw16);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = false;
  wn.shift = Cfg::kTwShift;
  wn.nmask = Cfg::kN - 1;
  const int g = lane >> 2, tq = lane & 3;
  constexpr int JN = C / 8;  // two side-by-side columns per warp
  const int col0 = JN * warp;
  int cnt = 0;
  for (long long it = blockIdx.x; it < tiles; it += gridDim.x, ++cnt) {
    const int s = cnt % NST;
    const bool ok = named_bar_and(2, 256, mbar_wait(&full[s], (cnt / NST) & 1, p.err));
    const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes);
    if (ok) {
      // phase 0: columns of 256 in place, times W_N^(n2 k1)
#pragma unroll 1
      for (int tile = 0; tile < T * CG; ++tile) {
        const uint32_t tb = base + tile * Cfg::kTileBytes;
        float2 fk[JN][8];
#pragma unroll
        for (int jn = 0; jn < JN; ++jn) {
          const int n2 = (tile % CG) * C + col0 + jn;
#pragma unroll
          for (int sl = 0; sl < 8; ++sl) {
            const float2 f = wn(n2 * jc.kval[sl >> 2][(sl >> 1) & 1][sl & 1]);
            fk[jn][sl] = make_float2(f.x * p.oscale, f.y * p.oscale);
          }
        }
        auto ldp = [&](int jp, int n, float2& x0, float2& x1) {
          lds_pair<true>(tb + ctile_off<C, ES>(col_in_row_t<true>(n), col0 + jp), x0, x1);
        };
        auto st = [&](int jp, int k, int, int sl, float2 v0, float2 v1) {
          sts_pair<true>(tb + ctile_off<C, ES>(col_out_row(k, 0), col0 + jp), cmul(v0, fk[jp][sl]),
                         cmul(v1, fk[jp + 1][sl]));
        };
        fft256r_jobs<1, SPLIT, 1, JN, true>(jc, tw16, p.dsign, ldp, st);
      }
      named_bar_sync(1, 256);
      // phase 1: 16 rows k1 per job, FFT over n2 (length 16 R1); jobs j = warp + 8 i
      constexpr int JOBS = 2 * T;
      float2 out[JOBS][8 * R1];
#pragma unroll
      for (int i = 0; i < JOBS; ++i) {
        const int job = warp + 8 * i, t = job >> 4, k1base = (job & 15) * 16;
        const uint32_t tbase = base + t * (CG * Cfg::kTileBytes);
        auto ld = [&](int v, int n) {
          return lds_elem<true>(tbase + (n / C) * Cfg::kTileBytes +
                                ctile_off<C, ES>(col_out_row(k1base + v, 0), n % C));
        };
        auto st = [&](int, int, int q, int slot, float2 val) { out[i][8 * q + slot] = val; };
        fft16r_job<R1, SPLIT, 1, PI, RHO>(jc, tw16, p.dsign, ld, st);
      }
      named_bar_sync(1, 256);  // every warp has read the stage
      // natural order X[k1 + 256 k2] of transform t at element t N + k1 + 256 k2 (128B-swizzled rows)
#pragma unroll
      for (int i = 0; i < JOBS; ++i) {
        const int job = warp + 8 * i, t = job >> 4, k1base = (job & 15) * 16;
#pragma unroll
        for (int q = 0; q < R1; ++q)
#pragma unroll
          for (int slot = 0; slot < 8; ++slot) {
            const int jj = slot >> 2, h = (slot >> 1) & 1, e = slot & 1;
            const int v = 2 * tq + e + 8 * jj, k = q + R1 * RHO::apply(g + 8 * h);
            const uint32_t el = (uint32_t)(t * Cfg::kN + k1base + v + 256 * k);
            sts64f(base + swz_w<8>(el) * 8, out[i][8 * q + slot]);
          }
      }
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&computed[s]);
    if (!ok) break;
  }
}

template <int R1, bool SPLIT>
cudaError_t launch_resident_split_t(const CUtensorMap& lm, const CUtensorMap& sm, const ResParams& p, int num_sms,
                                    cudaStream_t st) {
  using Cfg = ResSplitCfg<R1>;
  auto kern = fft_resident_split_kernel<R1, SPLIT>;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [&] { init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem); });
  if (init_err != cudaSuccess) return init_err;
  const long long tiles = (p.batch + Cfg::kT - 1) / Cfg::kT;
  const long long grid = tiles < num_sms ? tiles : num_sms;
  kern<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(lm, sm, p);
  return cudaGetLastError();
}

template <int R1, bool TOUT = false>
cudaError_t launch_resident_t(const CUtensorMap& lm, const CUtensorMap& sm, const ResParams& p, int num_sms,
                              cudaStream_t st) {
  using Cfg = ResCfg<R1>;
  auto kern = fft_resident_kernel<R1, TOUT>;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [&] { init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem); });
  if (init_err != cudaSuccess) return init_err;
  const long long tiles = (p.batch + Cfg::kT - 1) / Cfg::kT;
  const long long grid = tiles < num_sms ? tiles : num_sms;
  kern<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(lm, sm, p);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// N = 32768 = 256 x 128 plain.  Shared memory holds three 64 KiB regions.  Transform c
// takes its four 32-column tiles in regions in0 = -c mod 3 (tiles 0, 1) and in1 = in0 + 1
// (tiles 2, 3), and half of its output in out = in0 + 2:
//   phase 0: 256-point column FFTs of the four tiles in place, times W_N^(n2 k1)
//            (tiles 0, 1 as soon as they have landed, then tiles 2, 3);
//   phase 1, first half: the 8 jobs of rows k1 < 128 (one 16-row job of 128 points per
//            warp), outputs written straight into region out, which is then stored;
//   second half: the 8 jobs of rows k1 >= 128, outputs written into the tile rows the
//            first half consumed (in the column role's row order, k1 < 128 are the tile rows with
//            bit 5 clear: 4 runs of 32 rows per tile, 4 KiB each), stored the same way.
// Transform c + 1 loads its tiles 0, 1 into region out(c) as soon as the first half's store
// has read it (during the second half), and its tiles 2, 3 into in0(c) once the second
// half's store has read the runs; its first-half output goes to in1(c).  So the loads
// overlap the second half and the next transform's first column tiles.
// Output box (one TMA store, 4 KiB): 32 consecutive k1 x k2 bits 3-5 x k2 bits 0-1,
// at fixed k1 bits 5-7, k2 bit 2 and k2 bit 6.  The row jobs run with the identity
// output digit order (k2 = q + 8 (g + 8 h)), so the 8 lanes g of one store
// instruction write 8 box rows of different swizzle phases and the 4 lanes t write
// k1 bits 0-1 of one chunk: one wavefront per instruction.
struct Res32kCfg {
  static constexpr int kN = 32768, kC = 32, kCG = 4;  // N2 = 128 = 16 x 8
  static constexpr int kTileBytes = 256 * kC * 4;     // 32 KiB
  static constexpr int kRegionBytes = 65536;          // two tiles, or half of the output
  static constexpr int kHalfBytes = 2 * kTileBytes;
  static constexpr int kBoxBytes = 4096;
  static constexpr int kTwShift = 8, kTwLo = 256, kTwHi = 128;
  static constexpr int kTabBytes = (kTwLo + kTwHi) * 8 + FoldTab<8>::kABytes;
  static constexpr int kSmem = 3 * kRegionBytes + kTabBytes + 1024 + 256;
  static constexpr int kThreads = 384;
  using PI = BitPerm<0, 1, 3, 2>;    // phase 0 (column jobs)
  using PI1 = BitPerm<0, 2, 3, 1>;   // phase 1: lane t reads points 4t .. 4t + 3
  using RHO = BitPerm<0, 2, 3, 1>;   // phase 0
  using RHO1 = BitPerm<0, 1, 2, 3>;  // phase 1: output digit k0 = g + 8 h
  static_assert(kHalfBytes == kRegionBytes, "two tiles fill a region");
  static_assert(16 * kBoxBytes == kRegionBytes, "half an output is 16 boxes");
};

// Regions of transform c (shared-memory addresses): tiles 0-1, tiles 2-3, first-half output.
struct Res32kRegions {
  uint32_t t01, t23, out;
  __device__ __forceinline__ Res32kRegions(uint32_t base, int cnt) {
    const int r0 = (3 - cnt % 3) % 3;
    t01 = base + (uint32_t)(r0 * Res32kCfg::kRegionBytes);
    t23 = base + (uint32_t)(((r0 + 1) % 3) * Res32kCfg::kRegionBytes);
    out = base + (uint32_t)(((r0 + 2) % 3) * Res32kCfg::kRegionBytes);
  }
  __device__ __forceinline__ uint32_t tile(int t) const {
    return (t < 2 ? t01 : t23) + (uint32_t)((t & 1) * Res32kCfg::kTileBytes);
  }
  // box u of a row half: in region out (first half, rh 0) or run u & 3 of tile u >> 2 (rh 1)
  __device__ __forceinline__ uint32_t box(int rh, int u) const {
    return rh == 0 ? out + (uint32_t)(u * Res32kCfg::kBoxBytes) : tile(u >> 2) + (uint32_t)((u & 3) * 8192);
  }
};

// Byte address of output X[k1 + 256 k2] (k1 in row half rh): box u = 4 c + k2
// bit 2 + 2 k2 bit 6 (c = k1 bits 5-6), box row k2 bits 3-5 | k2 bits 0-1 << 3, 128-byte
// swizzle.
__device__ __forceinline__ uint32_t res32k_out(const Res32kRegions& rg, int rh, int k1, int k2) {
  const int u = 4 * ((k1 >> 5) & 3) + ((k2 >> 2) & 1) + 2 * (k2 >> 6);
  const int row = ((k2 >> 3) & 7) | ((k2 & 3) << 3);
  return rg.box(rh, u) + ctile_off<32, 4>(row, k1 & 31);
}

__global__ void __launch_bounds__(384, 1) fft_resident32k_kernel(const __grid_constant__ CUtensorMap load_map,
                                                                  const __grid_constant__ CUtensorMap store_map,
                                                                  const ResParams p) {
  using Cfg = Res32kCfg;
  using PI = Cfg::PI;
  using PI1 = Cfg::PI1;
  using RHO = Cfg::RHO;
  using RHO1 = Cfg::RHO1;
  constexpr int C = Cfg::kC;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* tab = smem + 3 * Cfg::kRegionBytes;
  float2* s_twlo = reinterpret_cast<float2*>(tab);
  float2* s_twhi = s_twlo + Cfg::kTwLo;
  unsigned char* s_fold = reinterpret_cast<unsigned char*>(s_twhi + Cfg::kTwHi);
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + Cfg::kTabBytes);  // [2]: tiles 0-1, tiles 2-3 landed
  uint64_t* outfree = full + 2;  // the first half's output region read out by its store
  uint64_t* runsfree = full + 3; // the second half's runs read out by their store
  uint64_t* half = full + 4;     // [2]: a half of the output written (8 compute warps)
  const uint32_t base = smem_addr(smem);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(outfree, 1);
    mbar_init(runsfree, 1);
    mbar_init(&half[0], 8);
    mbar_init(&half[1], 8);
    fence_barrier_init();
  }
  for (int j = tid; j < Cfg::kTwLo; j += blockDim.x) s_twlo[j] = p.twlo[j];
  for (int j = tid; j < Cfg::kTwHi; j += blockDim.x) s_twhi[j] = p.twhi[j];
  build_fold_table<8, PI1, RHO1, false>(s_fold, p.tw2048, tid, blockDim.x);  // phase-1 radix-8 fold (A part)
  __syncthreads();

  if (warp >= 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(56));
  if (warp >= 10) return;
  if (warp == 8) {  // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&load_map);
      int issued[2] = {0, 0};
      int cnt = 0;
      for (long long it = blockIdx.x; it < p.batch; it += gridDim.x, ++cnt) {
        const Res32kRegions rg(base, cnt);
        bool ok = true;
#pragma unroll 1
        for (int h = 0; h < 2 && ok; ++h) {
          // tiles 0-1 go to the previous transform's first-half output region, tiles 2-3 to its
          // tiles 0-1 region (which held its second-half runs)
          ok = mbar_wait(h == 0 ? outfree : runsfree, (uint32_t)(cnt + 1) & 1, p.err);
          if (!ok) break;
          mbar_arrive_expect_tx(&full[h], Cfg::kHalfBytes);
#pragma unroll 1
          for (int t = 2 * h; t < 2 * h + 2; ++t)
            tma_load_5d(smem + (rg.tile(t) - base), &load_map, t * C, 0, 0, 0, (int)it, &full[h]);
          ++issued[h];
        }
        if (!ok) break;
      }
      for (int h = 0; h < 2; ++h)  // the last loads have landed
        if (issued[h] > 0) mbar_wait(&full[h], (uint32_t)(issued[h] - 1) & 1, nullptr);
    }
    return;
  }
  if (warp == 9) {  // ------------------------------------------------ TMA storer
    if (lane == 0) {
      prefetch_tmap(&store_map);
      int cnt = 0;
      bool ok = true;
      for (long long it = blockIdx.x; it < p.batch && ok; it += gridDim.x, ++cnt) {
        const Res32kRegions rg(base, cnt);
#pragma unroll 1
        for (int rh = 0; rh < 2; ++rh) {
          ok = mbar_wait(&half[rh], (uint32_t)cnt & 1, p.err);
          if (!ok) break;
#pragma unroll 1
          for (int u = 0; u < 16; ++u)
            tma_store_5d(&store_map, 128 * rh + 32 * (u >> 2), 0, 0, u & 1, ((u >> 1) & 1) + 2 * (int)it,
                         smem + (rg.box(rh, u) - base));
          bulk_commit();
          bulk_wait_read<0>();
          mbar_arrive(rh == 0 ? outfree : runsfree);
        }
      }
      bulk_wait<0>();
    }
    return;
  }

  // ------------------------------------------------------------------ compute warps
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(224));
  JobConsts<false> jc, jc1;
  init_job_consts<false, PI, RHO>(jc, p.tw2048);
  init_job_consts<false, PI1, RHO1>(jc1, p.tw2048);
  const uint32_t fold = smem_addr(s_fold);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = false;
  wn.shift = Cfg::kTwShift;
  wn.nmask = Cfg::kN - 1;
  const int tq = lane & 3;
  int cnt = 0;
  for (long long it = blockIdx.x; it < p.batch; it += gridDim.x, ++cnt) {
    const Res32kRegions rg(base, cnt);
    bool ok = true;
    // phase 0: columns of 256 (in place, digit-ordered rows), twiddle W_N^(n2 k1); two passes of
    // two columns per warp, as for the one-transform stages of 16384.  Tiles 0-1 start before
    // tiles 2-3 have landed.
#pragma unroll 1
    for (int hh = 0; hh < 2; ++hh) {
      ok = named_bar_and(2, 256, ok && mbar_wait(&full[hh], (uint32_t)cnt & 1, p.err));
      if (ok) {
#pragma unroll 1
        for (int tile = 2 * hh; tile < 2 * hh + 2; ++tile)
#pragma unroll 1
          for (int h = 0; h < 2; ++h)
            plain_col_tile<1, C, true, PI, RHO, 2>(jc, fold, rg.tile(tile), warp + 8 * h, p.dsign, tile * C, wn,
                                                   p.oscale);
      }
    }
    // every column tile is complete; the first half's output region was freed before tiles 2-3
    // were loaded (it held the previous transform's second-half runs)
    ok = named_bar_and(2, 256, ok);
#pragma unroll 1
    for (int rh = 0; rh < 2; ++rh) {
      if (ok) {
        // 16 rows k1 per job, FFT over n2 (length 128); job jl = warp + 8 rh
        const int jl = warp + 8 * rh;
        auto ld4 = [&](int v, int a, uint32_t(&w)[4]) {
          const int n = 4 * tq + 16 * a;
          lds128(rg.tile(n >> 5) + ctile_off<C, 4>(col_out_row(kap_of<C>(v, jl), 0), n & (C - 1)), w);
        };
        auto st = [&](int v, int k2, int, int, float2 val) {
          sts32(res32k_out(rg, rh, kap_of<C>(v, jl), k2), pack_h2(val.x, val.y));
        };
        fft16r_job_q_fold<8, PI1, RHO1>(jc1, fold, p.dsign, ld4, st);
      }
      fence_proxy_async_smem();  // the half is read by TMA stores
      __syncwarp();
      if (lane == 0) mbar_arrive(&half[rh]);
      // the second half overwrites the rows the first half read: every warp has finished it
      if (rh == 0) ok = named_bar_and(2, 256, ok);
    }
    if (!ok) break;
  }
}

cudaError_t launch_resident32k(const CUtensorMap& lm, const CUtensorMap& sm, const ResParams& p, int num_sms,
                               cudaStream_t st) {
  using Cfg = Res32kCfg;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  std::call_once(once, [&] {
    init_err = cudaFuncSetAttribute(fft_resident32k_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem);
  });
  if (init_err != cudaSuccess) return init_err;
  const long long grid = p.batch < num_sms ? p.batch : num_sms;
  fft_resident32k_kernel<<<(int)grid, Cfg::kThreads, Cfg::kSmem, st>>>(lm, sm, p);
  return cudaGetLastError();
}

}  // namespace

bool resident_supported(int64_t n, bool split) {
  return split ? (n == 4096 || n == 8192) : (n == 4096 || n == 8192 || n == 16384 || n == 32768);
}

// Tensor maps: column-tile loads of the [B*256 rows][N2 cols] view; stores of
// X[k1 + 256 k2] as a 5D box with dims (k1 bits 0-4, k2 bit L, k2 bits L+2..L+3
// together with the transform index, k2 bit L+1, k1 bits 5-7 together with
// k2 bits 0..L-1), L = log2(N2 / 16), matching the stage layout above.
cudaError_t launch_resident_split(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                                  const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st,
                                  CUtensorMap* lm, CUtensorMap* sm, bool encode, float oscale, const void* in,
                                  bool io32) {
  const int64_t n2 = n / 256;
  if (encode) {
    void* src = const_cast<void*>(in ? in : data);  // loads from the input, stores to data
    if (encode_col_load(lm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, src, n2, batch, 8, 16, 1) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    uint64_t dims[2] = {16, (uint64_t)(n * batch / 16)};
    uint64_t str[1] = {128};
    uint32_t box[2] = {16, 256};
    if (encode_tmap(sm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, data, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B) !=
        CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  ResParams p;
  p.tw2048 = tw2048;
  p.twlo = twlo;
  p.twhi = twhi;
  p.batch = batch;
  p.rows = 0;
  p.err = err;
  p.dsign = dsign;
  p.oscale = oscale;
  switch (n) {
    case 4096: return io32 ? launch_resident_split_t<1, false>(*lm, *sm, p, num_sms, st)
                           : launch_resident_split_t<1, true>(*lm, *sm, p, num_sms, st);
    case 8192: return io32 ? launch_resident_split_t<2, false>(*lm, *sm, p, num_sms, st)
                           : launch_resident_split_t<2, true>(*lm, *sm, p, num_sms, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_resident(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                            const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st,
                            CUtensorMap* lm, CUtensorMap* sm, bool encode, float oscale, const void* in) {
  const int64_t n2 = n / 256;
  const int C = n2 < 32 ? (int)n2 : 32;
  if (encode && n == 32768) {
    // stores: 4 KiB boxes of X[k1 + 256 k2] with dims (k1, k2 bits 3-5, k2 bits 0-1, k2 bit 2,
    // k2 bit 6 together with the transform index), the layout of res32k_out
    void* src = const_cast<void*>(in ? in : data);
    if (encode_col_load(lm, CU_TENSOR_MAP_DATA_TYPE_UINT32, src, n2, batch, 4, C, 1) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    uint64_t dims[5] = {256, 8, 4, 2, (uint64_t)(2 * batch)};
    uint64_t str[4] = {8 * 1024, 1024, 4 * 1024, 64 * 1024};
    uint32_t box[5] = {32, 8, 4, 1, 1};
    if (encode_tmap(sm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 5, data, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B) !=
        CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  } else if (encode) {
    void* src = const_cast<void*>(in ? in : data);  // loads from the input, stores to data
    if (encode_col_load(lm, CU_TENSOR_MAP_DATA_TYPE_UINT32, src, n2, batch, 4, C, 1) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    const uint64_t r1 = (uint64_t)(n2 / 16), row = 256 * 4;  // R1; bytes per k2 step
    const uint32_t T = (uint32_t)(4 / r1);                    // transforms per stage
    uint64_t dims[5] = {32, 2, (uint64_t)(4 * batch), 2, 8 * r1};
    uint64_t str[4] = {row * r1, row * r1 * 4, row * r1 * 2, 128};
    uint32_t box[5] = {32, 2, 4 * T, 2, (uint32_t)(8 * r1)};
    if (encode_tmap(sm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 5, data, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B) !=
        CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  ResParams p;
  p.tw2048 = tw2048;
  p.twlo = twlo;
  p.twhi = twhi;
  p.batch = batch;
  p.rows = 0;
  p.err = err;
  p.dsign = dsign;
  p.oscale = oscale;
  switch (n) {
    case 4096: return launch_resident_t<1>(*lm, *sm, p, num_sms, st);
    case 8192: return launch_resident_t<2>(*lm, *sm, p, num_sms, st);
    case 16384: return launch_resident_t<4>(*lm, *sm, p, num_sms, st);
    case 32768: return launch_resident32k(*lm, *sm, p, num_sms, st);
    default: return cudaErrorInvalidValue;
  }
}

// N = 4096 with transposed output: transform m * rows + r of `in` (batch = rows x
// matrices) goes to out[m][k][r], k < 4096 (out of place; rows a multiple of 4).
bool resident_tout_supported(int64_t n, int64_t batch, int64_t rows) {
  return n == 4096 && rows >= 4 && rows % 4 == 0 && batch % rows == 0;
}
cudaError_t launch_resident_tout(int64_t n, const void* in, void* out, int64_t batch, int64_t rows,
                                 const float2* tw2048, const float2* twlo, const float2* twhi, float dsign, int* err,
                                 int num_sms, cudaStream_t st, CUtensorMap* lm, CUtensorMap* sm, bool encode,
                                 float oscale) {
  if (!resident_tout_supported(n, batch, rows)) return cudaErrorInvalidValue;
  if (encode) {
    if (encode_col_load(lm, CU_TENSOR_MAP_DATA_TYPE_UINT32, const_cast<void*>(in), 16, batch, 4, 16, 1) !=
        CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    const uint64_t rb = (uint64_t)rows * 4;  // bytes per output k
    uint64_t dims[5] = {(uint64_t)rows, 8, 4, 128, (uint64_t)(batch / rows)};
    uint64_t str[4] = {4 * rb, rb, 32 * rb, 4096 * rb};
    uint32_t box[5] = {4, 8, 4, 128, 1};
    if (encode_tmap(sm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 5, out, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE) !=
        CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  ResParams p;
  p.tw2048 = tw2048;
  p.twlo = twlo;
  p.twhi = twhi;
  p.batch = batch;
  p.rows = rows;
  p.err = err;
  p.dsign = dsign;
  p.oscale = oscale;
  return launch_resident_t<1, true>(*lm, *sm, p, num_sms, st);
}

}  // namespace tcfft
