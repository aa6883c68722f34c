// fft_fused.cuh -- persistent two-phase FFT executor (large 1D sizes and 2D).
//
// A transform is processed in two phases with TMA-fed shared-memory tiles:
//
//   1D, N = N1*N2 (four-step, replaces the reference's chain of layer_*_0 +
//   layer_*_1 launches, tcfft_half.cu:1205-1232, which make one full HBM
//   round trip per launch):
//     phase 0  (COL):   data[n1][n2] -> FFT over n1 (length N1, stride N2)
//                       -> twiddle W_N^(n2 k1) -> scratch[k1][n2]
//     phase 1  (ROW_T): scratch row k1 -> FFT over n2 (length N2)
//                       -> data[k1 + N1 k2]  (transposed write)
//   2D, [NX][NY] row-major (replaces tcfft_half_2d.cu:1128-1149's two
//   launches):
//     phase 0  (ROW):   FFT of each contiguous row (length NY), in place
//     phase 1  (COL):   FFT of each column (length NX, stride NY), in place
//
// One launch processes every transform of the batch.  Work items (tiles) are
// ordered in blocks: block s holds the phase-0 tiles of transform s followed by
// the phase-1 tiles of transform s - D, so the intermediate of a transform is
// consumed D blocks after it was produced, while it is still in L2.  The 1D
// intermediate lives in a ring of S >= D + 1 scratch slots.  Cross-CTA
// ordering uses per-slot completion counters (release/acquire, bounded spins
// that raise kDevTimeout instead of hanging).
//
// CTA = 8 compute warps + 1 TMA-load warp + 1 TMA-store warp, a ring of
// kStages shared-memory tiles (full / computed / empty mbarriers).
#pragma once
#include "fft_job.cuh"

namespace tcfft {

// kRoleCol:    FFT of length 256R down tile columns, in place (TMA 5D store, digit-ordered rows)
// kRoleRowT:   FFT of length 256R along contiguous rows, written transposed (1D phase 1)
// kRoleRow:    FFT of length 256R along contiguous rows, in place (2D phase 0)
// kRoleRow16T: 16 rows at a time, FFT of length 16R along each, written transposed (1D phase 1, short rows)
enum Role : int { kRoleCol = 0, kRoleRowT = 1, kRoleRow = 2, kRoleRow16T = 3 };
__host__ __device__ constexpr int role_len(int role, int R) { return role == kRoleRow16T ? 16 * R : 256 * R; }
__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

struct FusedMaps {
  CUtensorMap load0, store0, load1, store1;
};

struct FusedParams {
  const float2* tw2048;
  unsigned char* scratch;  // 1D: the scratch ring (phase-0 output, phase-1 input); 2D: unused
  const float2* twlo;  // W_N^j, j < 2^tw_shift        (1D phase-0 twiddle)
  const float2* twhi;  // W_N^(j << tw_shift)
  int tw_shift;
  int wn_global;       // 1: W_N factors read from twlo/twhi in global memory (tables too large to
                       //    stage in shared memory: the column pass of N > 2^22); 0: staged
  long long n_mask;    // N - 1 (1D)
  int batch;           // transforms
  int D;               // lag in blocks between phase 0 and phase 1 of a transform
  int S;               // counter / scratch slots
  int T0, T1;          // tiles per transform in each phase
  int rows0, rows1;    // rows per transform in the phase's load geometry (see launcher)
  int cols0, cols1;    // column groups per transform (COL tiles) / row groups (ROW tiles)
  int* cnt0;           // [S] completed phase-0 tiles per slot (monotonic within an execute)
  int* cnt1;           // [S] completed phase-1 tiles per slot
  int* err;
  float dsign;
  unsigned long long wait_ns;  // limit of every bounded wait (0: kTimeoutNs)
  float oscale0, oscale1;      // output scale of each phase (powers of two; 0 reads as 1): 1D carries
                               // the 1/N of a normalised transform in phase 0's W_N factors
};

// Column tiles: C columns x L rows of C*ES bytes (32, 64 or 128), moved by TMA
// with the swizzle of that width (the 16-byte chunk bits [4:4+w) of the byte
// offset XOR bits [7:7+w), w = 1, 2, 3 for 32-, 64-, 128-byte rows).  A column of such a tile
// reaches only 8 of the 16-byte bank groups, and which one is picked by the low
// row bits, so rows are placed in a digit order that spreads the rows a warp
// touches in one instruction over all 8 groups (checked exhaustively for every
// tile shape: 2 wavefronts per 128 bytes and half-warp, the minimum for two
// side-by-side jobs):
//  * input row n = m0 + 16 m1 + 256 a sits at tile row
//    (m1 bit 3 | m0 << 1 | m1 bits 0-2 << 5 | a << 8);
//  * output row k = q + R (k0 + 16 k1) sits at tile row
//    (k0 bits 2-3 | k1 << 2 | k0 bits 0-1 << 6 | q << 8).
// 5D TMA boxes whose dimensions are these digit groups move the rows between
// natural order in global memory and this order in the tile.
template <int C, int ES>
__device__ __forceinline__ uint32_t ctile_off(int row, int col) {
  constexpr int RB = C * ES;
  static_assert(RB == 32 || RB == 64 || RB == 128, "column tiles are 32-, 64- or 128-byte rows");
  constexpr uint32_t kMask = RB == 128 ? 7u : (RB == 64 ? 3u : 1u);
  const uint32_t L = (uint32_t)(row * RB + col * ES);
  return L ^ (((L >> 7) & kMask) << 4);
}
__device__ __forceinline__ int col_in_row(int n) {
  return ((n >> 7) & 1) | ((n & 15) << 1) | (((n >> 4) & 7) << 5) | (n & ~255);
}
// Split precision (8-byte elements, identity slot permutation, 16-byte accesses of
// two columns): the eight lanes of a quarter-warp read rows n whose bits 0, 5 and 6
// differ, so those bits are the tile row's low bits (the swizzle phase):
// tile row (n bits 5-6 | n bit 0 << 2 | n bits 1-4 << 3 | (n >> 7) << 7).
template <bool SPLIT>
__device__ __forceinline__ int col_in_row_t(int n) {
  if constexpr (SPLIT) return ((n >> 5) & 3) | ((n & 1) << 2) | (((n >> 1) & 15) << 3) | ((n >> 7) << 7);
  else return col_in_row(n);
}
// Block coordinate of transform b in a column-load box (the outermost box dimension
// holds R blocks of 256 rows, 2R half-blocks of 128 in the split order).
template <bool SPLIT>
__host__ __device__ constexpr int col_blk(int b, int R) {
  return SPLIT ? 2 * R * b : R * b;
}
__device__ __forceinline__ int col_out_row(int kp, int q) {
  return ((kp >> 2) & 3) | ((kp >> 4) << 2) | ((kp & 3) << 6) | (q << 8);
}

template <bool SPLIT>
__device__ __forceinline__ float2 lds_elem(uint32_t addr) {
  if constexpr (SPLIT) return lds64f(addr);
  else return unpack_h2(lds32(addr));
}
template <bool SPLIT>
__device__ __forceinline__ void sts_elem(uint32_t addr, float2 v) {
  if constexpr (SPLIT) sts64f(addr, v);
  else sts32(addr, pack_h2(v.x, v.y));
}
// two side-by-side elements (adjacent columns of a column tile)
template <bool SPLIT>
__device__ __forceinline__ void lds_pair(uint32_t addr, float2& x0, float2& x1) {
  if constexpr (SPLIT) {
    lds128f(addr, x0, x1);
  } else {
    uint32_t a, b;
    lds64(addr, a, b);
    x0 = unpack_h2(a);
    x1 = unpack_h2(b);
  }
}
template <bool SPLIT>
__device__ __forceinline__ void sts_pair(uint32_t addr, float2 v0, float2 v1) {
  if constexpr (SPLIT) sts128f(addr, v0, v1);
  else sts64(addr, pack_h2(v0.x, v0.y), pack_h2(v1.x, v1.y));
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Bounded spin until *p >= target (at most limit_ns).
__device__ __forceinline__ bool wait_counter(const int* p, int target, int* err, unsigned long long limit_ns) {
  if (ld_acquire(p) >= target) return true;
  const unsigned long long t0 = global_ns();
  while (ld_acquire(p) < target) {
    if (global_ns() - t0 > limit_ns) {
      if (err) atomicExch(err, kDevTimeout);
      return false;
    }
    __nanosleep(64);
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void named_bar_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// Barrier over `n` threads that also returns the AND of `pred` across them.
__device__ __forceinline__ bool named_bar_and(int id, int n, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

// ---------------------------------------------------------------- plain-precision tile bodies
// (fft256r_jobs_fold with per-lane slot offsets computed once per tile)

// Input digit m of B-fragment slot 4kt + 2r + j and output index k' of
// accumulator slot 4h + 2e + hh for this lane (fft_common.cuh conventions).
template <class PI, class RHO>
__device__ __forceinline__ int slot_m(int slot) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  return 16 * PI::apply(2 * t + ((slot >> 1) & 1) + 8 * (slot >> 2)) + PI::apply(g + 8 * (slot & 1));
}
template <class PI, class RHO>
__device__ __forceinline__ int slot_kval(int osl) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  return RHO::apply(2 * t + ((osl >> 1) & 1) + 8 * (osl >> 2)) + 16 * RHO::apply(g + 8 * (osl & 1));
}

// W_N^e from the two-level table (e reduced mod N by nmask): staged in shared
// memory (hi, lo addresses) or, for very large N, read from global memory.
struct WnTable {
  uint32_t hi, lo;
  const float2* ghi;
  const float2* glo;
  int shift, nmask;
  bool global;
  __device__ __forceinline__ float2 operator()(int e) const {
    e &= nmask;
    if (global) return cmul(__ldg(ghi + (e >> shift)), __ldg(glo + (e & ((1 << shift) - 1))));
    return cmul(lds64f(hi + (e >> shift) * 8), lds64f(lo + (e & ((1 << shift) - 1)) * 8));
  }
};

// Column tile, in place: JN = C/8 side-by-side columns col0 = JN warp + jn per
// warp, each an FFT of length 256R down the tile.  With WN (1D four-step phase
// 0) the output k of column n2 = n2base + jn is multiplied by W_N^(n2 k).
// JNW: columns per call (default C/8: the 8 warps share the tile in one call; 2 with
// 32-column tiles: two calls per warp, `warp` and `warp + 8`, fewer live registers).
// wscale (WN only) multiplies the W_N factors: the outputs come out scaled by it.
// WnT: the W_N lookup (WnTable, or any functor int e -> W_N^e).
template <int R, int C, bool WN, class PI, class RHO, int JNW = C / 8, class WnT = WnTable>
__device__ __forceinline__ void plain_col_tile(const JobConsts<false>& jc, uint32_t fold, uint32_t base, int warp,
                                               float dsign, int n2base, const WnT& wn, float wscale = 1.f,
                                               const float2* tglob = nullptr) {
  constexpr int ES = 4, JN = JNW;
  static_assert(JN * 8 == C || (JN == 2 && C == 32), "columns per call");
  constexpr bool PAIR = JN % 2 == 0;
  constexpr bool QUAD = JN == 4;  // 128-byte rows: the four columns move as one 16-byte access
  constexpr uint32_t kStep = 256 * C * ES;  // one digit a (input) or q (output) further down
  const int col0 = JN * warp;
  uint32_t lo[8], so[8];
#pragma unroll
  for (int sl = 0; sl < 8; ++sl) {
    lo[sl] = base + ctile_off<C, ES>(col_in_row(slot_m<PI, RHO>(sl)), col0);
    so[sl] = base + ctile_off<C, ES>(col_out_row(slot_kval<PI, RHO>(sl), 0), col0);
  }
  if constexpr (WN) {
    // W_N^(n2 (q + R k')), k' = kbase + e + 2h + 32hh (RHO digit structure):
    // fk[osl] = W^(n2 R kbase) u^(e + 2h) u32^hh with u = W^(n2 R); fq[q] = W^(n2 q)
    // Only the even-slot factors and u32 are held; an odd slot costs one product at the store
    // (four jobs: 40 registers instead of 64; two jobs at 2^20: no spills instead of 8/40 bytes,
    // 1 % faster at 2^19..2^22).
    const int kbase = slot_kval<PI, RHO>(0);
    constexpr int NK = 4;
    float2 fk[JN][NK], fu[JN], fq[JN][R];
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) {
      const int n2 = n2base + col0 + jn;
      float2 F = wn(n2 * R * kbase);
      F = make_float2(F.x * wscale, F.y * wscale);
      const float2 u = wn(n2 * R), u32 = wn(32 * n2 * R);
      const float2 u2 = cmul(u, u), u3 = cmul(u2, u);
      const float2 f0[4] = {F, cmul(F, u), cmul(F, u2), cmul(F, u3)};
      fu[jn] = u32;
#pragma unroll
      for (int osl = 0; osl < NK; ++osl) fk[jn][osl] = f0[osl];
      fq[jn][0] = make_float2(1.f, 0.f);
      if constexpr (R > 1) fq[jn][1] = wn(n2);
#pragma unroll
      for (int q = 2; q < R; ++q) fq[jn][q] = cmul(fq[jn][q - 1], fq[jn][1]);
    }
    // W_N^(n2 (q + R k')) of job jn, output slot osl (osl and q are compile-time constants
    // after unrolling: q = 0 needs no product)
    auto wfac = [&](int jn, int osl, int q) {
      float2 f = fk[jn][((osl >> 1) & 1) + 2 * (osl >> 2)];
      if (osl & 1) f = cmul(f, fu[jn]);
      return q == 0 ? f : cmul(f, fq[jn][q]);
    };
    if constexpr (QUAD) {
      auto ld = [&](int, int sl, int a, uint32_t& x0, uint32_t& x1, uint32_t& x2, uint32_t& x3) {
        uint32_t w[4];
        lds128(lo[sl] + a * kStep, w);
        x0 = w[0];
        x1 = w[1];
        x2 = w[2];
        x3 = w[3];
      };
      auto st = [&](int, int osl, int q, float2 v0, float2 v1, float2 v2, float2 v3) {
        v0 = cmul(v0, wfac(0, osl, q));
        v1 = cmul(v1, wfac(1, osl, q));
        v2 = cmul(v2, wfac(2, osl, q));
        v3 = cmul(v3, wfac(3, osl, q));
        sts128(so[osl] + q * kStep, pack_h2(v0.x, v0.y), pack_h2(v1.x, v1.y), pack_h2(v2.x, v2.y),
               pack_h2(v3.x, v3.y));
      };
      fft256r_jobs_fold_quad<R>(jc, fold, dsign, ld, st, tglob);
    } else if constexpr (PAIR) {
      auto ld = [&](int jp, int sl, int a, uint32_t& x0, uint32_t& x1) { lds64(lo[sl] + jp * ES + a * kStep, x0, x1); };
      auto st = [&](int jp, int osl, int q, float2 v0, float2 v1) {
        v0 = cmul(v0, wfac(jp, osl, q));
        v1 = cmul(v1, wfac(jp + 1, osl, q));
        sts_pair<false>(so[osl] + jp * ES + q * kStep, v0, v1);
      };
      fft256r_jobs_fold<R, JN, true>(jc, fold, dsign, ld, st, tglob);
    } else {
      auto ld = [&](int jn, int sl, int a) { return lds32(lo[sl] + jn * ES + a * kStep); };
      auto st = [&](int jn, int osl, int q, float2 v) {
        sts_elem<false>(so[osl] + jn * ES + q * kStep, cmul(v, wfac(jn, osl, q)));
      };
      fft256r_jobs_fold<R, JN, false>(jc, fold, dsign, ld, st, tglob);
    }
  } else {
    if constexpr (QUAD) {
      auto ld = [&](int, int sl, int a, uint32_t& x0, uint32_t& x1, uint32_t& x2, uint32_t& x3) {
        uint32_t w[4];
        lds128(lo[sl] + a * kStep, w);
        x0 = w[0];
        x1 = w[1];
        x2 = w[2];
        x3 = w[3];
      };
      auto st = [&](int, int osl, int q, float2 v0, float2 v1, float2 v2, float2 v3) {
        sts128(so[osl] + q * kStep, pack_h2(v0.x, v0.y), pack_h2(v1.x, v1.y), pack_h2(v2.x, v2.y),
               pack_h2(v3.x, v3.y));
      };
      fft256r_jobs_fold_quad<R>(jc, fold, dsign, ld, st, tglob);
    } else if constexpr (PAIR) {
      auto ld = [&](int jp, int sl, int a, uint32_t& x0, uint32_t& x1) { lds64(lo[sl] + jp * ES + a * kStep, x0, x1); };
      auto st = [&](int jp, int osl, int q, float2 v0, float2 v1) {
        sts_pair<false>(so[osl] + jp * ES + q * kStep, v0, v1);
      };
      fft256r_jobs_fold<R, JN, true>(jc, fold, dsign, ld, st, tglob);
    } else {
      auto ld = [&](int jn, int sl, int a) { return lds32(lo[sl] + jn * ES + a * kStep); };
      auto st = [&](int jn, int osl, int q, float2 v) { sts_elem<false>(so[osl] + jn * ES + q * kStep, v); };
      fft256r_jobs_fold<R, JN, false>(jc, fold, dsign, ld, st, tglob);
    }
  }
}

// Contiguous rows of length 256R (JN per warp); the outputs stay in registers
// (out[jn][q][osl], packed half2) for the caller to store.
template <int R, int JN, class PI, class RHO>
__device__ __forceinline__ void plain_row_jobs(const JobConsts<false>& jc, uint32_t fold, uint32_t row_addr0,
                                               uint32_t row_stride, float dsign, uint32_t (&out)[JN][R][8],
                                               const float2* tglob = nullptr) {
  uint32_t lo[8];
#pragma unroll
  for (int sl = 0; sl < 8; ++sl) lo[sl] = row_addr0 + swz_w<4>(slot_m<PI, RHO>(sl)) * 4;
  auto ld = [&](int jn, int sl, int a) { return lds32(lo[sl] + jn * row_stride + a * 1024); };
  auto st = [&](int jn, int osl, int q, float2 v) { out[jn][q][osl] = pack_h2(v.x, v.y); };
  fft256r_jobs_fold<R, JN, false>(jc, fold, dsign, ld, st, tglob);
}

// Tiles per work item of a 1D row-transpose schedule: as many tiles as fill an
// item of `item_bytes` (at most 4); other schedules move one tile per item.
__host__ __device__ constexpr int fused_sub_of(bool sub_ok, int tile_bytes, int item_bytes = 65536) {
  return !sub_ok || tile_bytes >= item_bytes ? 1 : (item_bytes / tile_bytes > 4 ? 4 : item_bytes / tile_bytes);
}

// ITEM_KB: target bytes of one work item (KiB).  64 KiB items run a ring of at
// most 4 stages; smaller items run deeper rings (up to 8 stages), which keeps
// more loads in flight per SM for the same shared memory.
template <int ROLE0, int R0, int C0, int ROLE1, int R1, int C1, int MODE, int ITEM_KB = 64>
struct FusedCfg {
  static constexpr bool kWide = MODE != kModePlain;   // 8-byte (float2) elements
  static constexpr bool kSplit = MODE == kModeSplit;  // three products per stage
  static constexpr int kES = kWide ? 8 : 4;
  static constexpr int kER = 128 / kES;
  static constexpr bool k1D = ROLE1 == kRoleRowT || ROLE1 == kRoleRow16T;
  static constexpr int kLen0 = role_len(ROLE0, R0), kLen1 = role_len(ROLE1, R1);  // FFT lengths
  static constexpr int kTile0 = C0 * kLen0;  // elements per tile
  static constexpr int kTile1 = C1 * kLen1;
  // 1D row-transpose and 2D schedules move up to 4 tiles per work item (kSub0/kSub1),
  // so that every item fills a 64 KiB stage: fewer, larger TMA transactions and
  // fewer per-item waits for tiles smaller than a stage (host T0/T1 count tiles;
  // the launcher passes items)
  static constexpr bool kSubOK = (k1D && ROLE1 == kRoleRowT) || (ROLE0 == kRoleRow && ROLE1 == kRoleCol);
  static constexpr int kSub0 = fused_sub_of(kSubOK, kTile0 * kES, ITEM_KB * 1024);
  static constexpr int kSub1 = fused_sub_of(kSubOK, kTile1 * kES, ITEM_KB * 1024);
  static constexpr int kItem0 = kSub0 * kTile0, kItem1 = kSub1 * kTile1;  // elements per work item
  static constexpr int kTileMax = kItem0 > kItem1 ? kItem0 : kItem1;
  static constexpr int kStageBytes = kTileMax * kES;
  // shared-memory tables: W_L^j (L = the longer job length; the fp32 job paths),
  // the two halves of W_N^j (1D four-step, N = kLen0 * kLen1) and the per-lane
  // fold tables of the plain 256R-point jobs (one per distinct R)
  static constexpr int kLmax = kLen0 > kLen1 ? kLen0 : kLen1;
  static constexpr int kLog2N = ilog2c(kLen0) + ilog2c(kLen1);
  static constexpr int kTwShift = (kLog2N + 1) / 2;          // log2 of the low table length
  static constexpr int kTwHi = 1 << (kLog2N - kTwShift);     // N >> shift
  static constexpr bool kFold = !kWide;                       // plain 256R-point jobs use fft256r_jobs_fold
  // (short-row phases use the A_q part only; with R1 == R0 they share the phase-0 table,
  // whose A part comes first)
  static constexpr bool kFold1Own = kFold && R1 != R0 && R1 > 1;
  static constexpr int kTwRBytes = (kWide || ROLE1 == kRoleRow16T) ? kLmax * 8 : 0;
  static constexpr int kWnBytes = k1D ? ((1 << kTwShift) + kTwHi) * 8 : 0;
  static constexpr int kFold0Bytes = kFold ? FoldTab<R0>::kBytes : 0;
  static constexpr int kFold1Bytes =
      kFold1Own ? (ROLE1 == kRoleRow16T ? FoldTab<R1>::kABytes : FoldTab<R1>::kBytes) : 0;
  static constexpr int kOffWn = kTwRBytes, kOffFold0 = kTwRBytes + kWnBytes, kOffFold1 = kOffFold0 + kFold0Bytes;
  static constexpr int kTabBytes = kTwRBytes + kWnBytes + kFold0Bytes + kFold1Bytes;
  // kRoleRow16T output boxes: kBW columns (128 bytes) each
  static constexpr int kBW = 128 / kES;
  // contiguous-row tiles move as boxes of [kER elements][kBH rows] (kBH <= 256)
  static constexpr int kBH0 = kTile0 / kER < 256 ? kTile0 / kER : 256;
  static constexpr int kBH1 = kTile1 / kER < 256 ? kTile1 / kER : 256;
  static constexpr int kBudget = 225 * 1024 - kTabBytes - 1024 - 256;
  static constexpr int kMaxStages = ITEM_KB >= 64 ? 4 : 8;
  static constexpr int kStages = kBudget / kStageBytes >= kMaxStages ? kMaxStages : kBudget / kStageBytes;
  static constexpr int kSmem = kStages * kStageBytes + kTabBytes + 1024 + 256;
  static_assert(kStages >= 2, "at least two tile stages");
  // 3 warpgroups: two of compute warps, one holding the producer and storer warps.
  // Launched at 168 registers/thread (384 x 168 = 64512); setmaxnreg moves
  // registers to the compute warpgroups: 256 x kComputeRegs + 128 x kAuxRegs = 64512.
  static constexpr int kThreads = 384;
  static constexpr int kComputeRegs = 224;
  static constexpr int kAuxRegs = 56;
  static_assert(256 * kComputeRegs + 128 * kAuxRegs == 384 * 168, "register split must match the launch");
  using PI = typename std::conditional<kWide, BitPerm<0, 1, 2, 3>, BitPerm<0, 1, 3, 2>>::type;
  using RHO = BitPerm<0, 2, 3, 1>;
};

// Item decode: block s = idx / (T0+T1); phase-0 tiles of transform s, then
// phase-1 tiles of transform s - D.
struct Item {
  int phase, b, tile;
  bool valid;
};
__device__ __forceinline__ Item decode_item(long long idx, const FusedParams& p) {
  const int per = p.T0 + p.T1;
  const long long blk = idx / per;
  const int r = (int)(idx - blk * per);
  Item it;
  if (r < p.T0) {
    it.phase = 0;
    it.b = (int)blk;
    it.tile = r;
  } else {
    it.phase = 1;
    it.b = (int)(blk - p.D);
    it.tile = r - p.T0;
  }
  it.valid = it.b >= 0 && it.b < p.batch;
  return it;
}

template <int ROLE0, int R0, int C0, int ROLE1, int R1, int C1, int MODE, int ITEM_KB>
__global__ void __launch_bounds__(384, 1)  // 12 warps at launch: 168 registers (3 warps per SM sub-partition)
    fft_fused_kernel(const __grid_constant__ FusedMaps maps, const FusedParams p) {
  using Cfg = FusedCfg<ROLE0, R0, C0, ROLE1, R1, C1, MODE, ITEM_KB>;
  constexpr bool WIDE = Cfg::kWide, SPLIT = Cfg::kSplit;  // element width; split arithmetic
  constexpr int ES = Cfg::kES, ER = Cfg::kER, NST = Cfg::kStages;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* s_tab = smem + NST * Cfg::kStageBytes;
  float2* s_twR = reinterpret_cast<float2*>(s_tab);                            // W_Lmax^j
  float2* s_twlo = reinterpret_cast<float2*>(s_tab + Cfg::kOffWn);             // W_N^j, j < 2^shift
  float2* s_twhi = s_twlo + (1 << Cfg::kTwShift);                              // W_N^(j << shift)
  unsigned char* s_fold0 = s_tab + Cfg::kOffFold0;                             // fold table for R0
  unsigned char* s_fold1 = Cfg::kFold1Own ? s_tab + Cfg::kOffFold1 : s_fold0;  // fold table for R1
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * Cfg::kStageBytes + Cfg::kTabBytes);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long total = (long long)(p.batch + p.D) * (p.T0 + p.T1);
  const unsigned long long lim = p.wait_ns ? p.wait_ns : kTimeoutNs;

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
    }
    fence_barrier_init();
  }
  // twiddle tables into shared memory (the inner loops never touch global tables)
  if constexpr (Cfg::kTwRBytes > 0)
    for (int j = tid; j < Cfg::kLmax; j += blockDim.x) s_twR[j] = p.tw2048[j * (2048 / Cfg::kLmax)];
  if (Cfg::k1D && !p.wn_global) {
    for (int j = tid; j < (1 << Cfg::kTwShift); j += blockDim.x) s_twlo[j] = p.twlo[j];
    for (int j = tid; j < Cfg::kTwHi; j += blockDim.x) s_twhi[j] = p.twhi[j];
  }
  // Output scales (powers of two; a normalised transform splits its 1/N between the
  // phases, so the intermediate keeps its magnitude and never drifts into fp16's
  // subnormal range).  2D: each phase's stage-1 twiddles (fold tables here,
  // JobConsts::tw1 per item below).  1D: the stage-1 twiddles of both phases carry
  // phase 1's scale and phase 0's W_N factors the ratio os0 / os1 (the short-row
  // phase has no stage-1 twiddle: its plans pass os1 = 1).
  const float os0 = p.oscale0 != 0.f ? p.oscale0 : 1.f, os1 = p.oscale1 != 0.f ? p.oscale1 : 1.f;
  const float wscale0 = Cfg::k1D ? os0 / os1 : 1.f;  // phase 0's W_N factors (1D)
  if constexpr (Cfg::kFold) {
    build_fold_table<R0, typename Cfg::PI, typename Cfg::RHO>(s_fold0, p.tw2048, tid, blockDim.x,
                                                              Cfg::k1D ? os1 : os0);
    if constexpr (Cfg::kFold1Own)
      build_fold_table<R1, typename Cfg::PI, typename Cfg::RHO, ROLE1 != kRoleRow16T>(s_fold1, p.tw2048, tid,
                                                                                       blockDim.x, os1);
  }
  __syncthreads();

  if (warp >= 8) {
    // auxiliary warpgroup: give registers back; each path below ends in return,
    // so the compute code is reached only through the setmaxnreg.inc further down
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(Cfg::kAuxRegs));
  }

  // Warp 8 is the TMA producer, warp 9 the TMA storer; warps 10-11 idle.
  if (warp >= 10) return;
  if (warp == 8) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&maps.load0);
      prefetch_tmap(&maps.load1);
      int cnt = 0, issued = 0;
      for (long long idx = blockIdx.x; idx < total; idx += gridDim.x) {
        const Item it = decode_item(idx, p);
        if (!it.valid) continue;
        const int s = cnt % NST;
        const int slot = it.b % p.S, epoch = it.b / p.S;
        // dependencies first (their latency overlaps the wait for a free stage)
        if (it.phase == 0) {
          // the previous occupant of this slot (transform b - S) must be finished, so that
          // the slot's scratch (1D) and completion counters (1D and 2D) are free
          if (epoch > 0 && !wait_counter(&p.cnt1[slot], epoch * p.T1, p.err, lim)) break;
        } else {
          if (!wait_counter(&p.cnt0[slot], (epoch + 1) * p.T0, p.err, lim)) break;
        }
        if (!mbar_wait(&empty[s], ((cnt / NST) + 1) & 1, p.err, lim)) break;
        if (it.phase == 1) fence_proxy_async_global();
        unsigned char* dst = smem + s * Cfg::kStageBytes;
        if (it.phase == 0) {
          mbar_arrive_expect_tx(&full[s], Cfg::kItem0 * ES);
          if constexpr (ROLE0 == kRoleCol) {  // 5D boxes: rows in the column-tile digit order
#pragma unroll 1
            for (int u = 0; u < Cfg::kSub0; ++u) {
              const int cg = (it.tile * Cfg::kSub0 + u) % p.cols0;
              tma_load_5d(dst + u * (Cfg::kTile0 * ES), &maps.load0, cg * C0, 0, 0, 0, col_blk<WIDE>(it.b, R0),
                          &full[s]);
            }
          } else {  // contiguous rows (the item's tiles are consecutive row groups)
            const int y0 =
                (int)(((long long)it.b * p.rows0 + (long long)it.tile * (Cfg::kSub0 * C0)) * (256 * R0) / ER);
#pragma unroll 1
            for (int i = 0; i < Cfg::kItem0 / (ER * Cfg::kBH0); ++i)
              tma_load_2d(dst + i * (ER * Cfg::kBH0 * ES), &maps.load0, 0, y0 + Cfg::kBH0 * i, &full[s]);
          }
        } else {
          mbar_arrive_expect_tx(&full[s], Cfg::kItem1 * ES);
          if constexpr (ROLE1 == kRoleCol) {
#pragma unroll 1
            for (int u = 0; u < Cfg::kSub1; ++u) {
              const int cg = (it.tile * Cfg::kSub1 + u) % p.cols1;
              tma_load_5d(dst + u * (Cfg::kTile1 * ES), &maps.load1, cg * C1, 0, 0, 0, col_blk<WIDE>(it.b, R1),
                          &full[s]);
            }
          } else {
            // 1D: source is the scratch slot; 2D never has a contiguous phase 1
            const long long row0 = (long long)slot * p.rows1 + (long long)it.tile * (Cfg::kSub1 * C1);
            const int y0 = (int)(row0 * Cfg::kLen1 / ER);
#pragma unroll 1
            for (int i = 0; i < Cfg::kItem1 / (ER * Cfg::kBH1); ++i)
              tma_load_2d(dst + i * (ER * Cfg::kBH1 * ES), &maps.load1, 0, y0 + Cfg::kBH1 * i, &full[s]);
          }
        }
        ++cnt;
        ++issued;
      }
      // on an early exit let this warp's loads still in flight land before the CTA ends (bounded)
      for (int i = (cnt > NST ? cnt - NST : 0); i < cnt; ++i) mbar_wait(&full[i % NST], (i / NST) & 1, nullptr);
      (void)issued;
    }
    return;
  }
  if (warp == 9) {
    // ------------------------------------------------------------ TMA storer
    // Up to kMaxPending stores stay in flight; their completion counters are
    // released in order once the bulk group reports them written.  Before the
    // storer blocks on the next computed tile it drains and releases every
    // pending store, so a consumer waiting on this CTA's output never waits
    // behind this CTA's own pipeline.
    if (lane == 0) {
      prefetch_tmap(&maps.store0);
      prefetch_tmap(&maps.store1);
      constexpr int kMaxPending = 2;
      int* pend[kMaxPending + 1];
      int npend = 0;
      auto release_all = [&]() {
        if (npend == 0) return;
        bulk_wait<0>();
        fence_proxy_async_global();
        for (int i = 0; i < npend; ++i) red_release_add(pend[i], 1);
        npend = 0;
      };
      int cnt = 0;
      bool failed = false;
      for (long long idx = blockIdx.x; idx < total && !failed; idx += gridDim.x) {
        const Item it = decode_item(idx, p);
        if (!it.valid) continue;
        const int s = cnt % NST;
        const uint32_t cpar = (cnt / NST) & 1;
        if (!mbar_try_wait(&computed[s], cpar)) {
          release_all();
          if (!mbar_wait(&computed[s], cpar, p.err, lim)) {
            failed = true;
            break;
          }
        }
        const unsigned char* src = smem + s * Cfg::kStageBytes;
        const int slot = it.b % p.S;
        if (it.phase == 0) {
          if constexpr (ROLE0 == kRoleCol) {
            // 5D box [C0][k0 hi][k1 (+16 transform)][k0 lo][q]: 1D -> scratch slot, 2D -> the data
#pragma unroll 1
            for (int u = 0; u < Cfg::kSub0; ++u) {
              const int cg = (it.tile * Cfg::kSub0 + u) % p.cols0;
              tma_store_5d(&maps.store0, cg * C0, 0, 16 * (Cfg::k1D ? slot : it.b), 0, 0,
                           src + u * (Cfg::kTile0 * ES));
            }
          } else {
            const int y0 =
                (int)(((long long)it.b * p.rows0 + (long long)it.tile * (Cfg::kSub0 * C0)) * (256 * R0) / ER);
#pragma unroll 1
            for (int i = 0; i < Cfg::kItem0 / (ER * Cfg::kBH0); ++i)
              tma_store_2d(&maps.store0, 0, y0 + Cfg::kBH0 * i, src + i * (ER * Cfg::kBH0 * ES));
          }
        } else {
          if constexpr (ROLE1 == kRoleCol) {
#pragma unroll 1
            for (int u = 0; u < Cfg::kSub1; ++u) {
              const int cg = (it.tile * Cfg::kSub1 + u) % p.cols1;
              tma_store_5d(&maps.store1, cg * C1, 0, 16 * it.b, 0, 0, src + u * (Cfg::kTile1 * ES));
            }
          } else if constexpr (ROLE1 == kRoleRowT) {  // output columns k1 of data viewed [B][N2 rows k2][N1 cols]
#pragma unroll 1
            for (int u = 0; u < Cfg::kSub1; ++u)
              tma_store_5d(&maps.store1, (it.tile * Cfg::kSub1 + u) * C1, 0, 16 * it.b, 0, 0,
                           src + u * (Cfg::kTile1 * ES));
          } else {  // kRoleRow16T: C1 columns as boxes of kBW, 4D [cols][k0][q][B]
#pragma unroll 1
            for (int bx = 0; bx < C1 / Cfg::kBW; ++bx)
              tma_store_4d(&maps.store1, it.tile * C1 + bx * Cfg::kBW, 0, 0, it.b,
                           src + bx * (Cfg::kBW * Cfg::kLen1 * ES));
          }
        }
        bulk_commit();
        pend[npend++] = it.phase == 0 ? &p.cnt0[slot] : &p.cnt1[slot];
        bulk_wait_read<0>();
        mbar_arrive(&empty[s]);
        if (npend > kMaxPending) {
          // the oldest group is complete once at most kMaxPending remain
          bulk_wait<kMaxPending>();
          fence_proxy_async_global();
          red_release_add(pend[0], 1);
          for (int i = 1; i < npend; ++i) pend[i - 1] = pend[i];
          --npend;
        }
        ++cnt;
      }
      release_all();
    }
    return;
  }

  // -------------------------------------------------------------- compute warps
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(Cfg::kComputeRegs));
  using PI = typename Cfg::PI;
  using RHO = typename Cfg::RHO;
  using Hold = typename std::conditional<WIDE, float2, uint32_t>::type;
  JobConsts<SPLIT> jc;
  init_job_consts<SPLIT, PI, RHO>(jc, p.tw2048);
  const uint32_t twR = smem_addr(s_twR);
  const uint32_t fold0 = smem_addr(s_fold0), fold1 = smem_addr(s_fold1);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = p.wn_global != 0;
  wn.shift = wn.global ? p.tw_shift : Cfg::kTwShift;
  wn.nmask = (int)p.n_mask;
  float tw1_scale = 1.f;  // the scale currently folded into jc.tw1
  if constexpr (Cfg::k1D) {
    scale_tw1(jc, os1);
    tw1_scale = os1;
  }
  int cnt = 0;
  for (long long idx = blockIdx.x; idx < total; idx += gridDim.x) {
    const Item it = decode_item(idx, p);
    if (!it.valid) continue;
    const int s = cnt % NST;
    if constexpr (!Cfg::k1D) {
      const float want = it.phase == 0 ? os0 : os1;
      if (want != tw1_scale) {  // powers of two: the ratio is exact
        scale_tw1(jc, want / tw1_scale);
        tw1_scale = want;
      }
    }
    // all compute warps agree on success before any of them enters a named barrier
    const bool ok = named_bar_and(2, 256, mbar_wait(&full[s], (cnt / NST) & 1, p.err, lim));
    const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes);
    if constexpr (Cfg::k1D) {
      if (ok && it.phase == 1) {
        // the tile's scratch rows are in shared memory now and never read again: drop
        // them from L2 without writing them back to HBM
        const long long row0 = (long long)(it.b % p.S) * p.rows1 + (long long)it.tile * (Cfg::kSub1 * C1);
        const unsigned char* src = p.scratch + row0 * Cfg::kLen1 * ES;
        for (int i = threadIdx.x; i < Cfg::kItem1 * ES / 128; i += 256)
          asm volatile("discard.global.L2 [%0], 128;" ::"l"(src + i * 128) : "memory");
      }
    }
    if (ok) {
      if (it.phase == 0) {
        if constexpr (ROLE0 == kRoleCol && !WIDE) {
#pragma unroll 1
          for (int u = 0; u < Cfg::kSub0; ++u)
            plain_col_tile<R0, C0, Cfg::k1D, PI, RHO>(jc, fold0, base + u * (Cfg::kTile0 * ES), warp, p.dsign,
                                                      ((it.tile * Cfg::kSub0 + u) % p.cols0) * C0, wn, wscale0);
        } else if constexpr (ROLE0 == kRoleCol) {
#pragma unroll 1
         for (int u = 0; u < Cfg::kSub0; ++u) {
          const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes) + u * (Cfg::kTile0 * ES);
          // columns JN*warp + jn in place (side by side, moved in pairs); 1D adds the
          // four-step twiddle W_N^(n2 k1)
          constexpr int JN = C0 / 8;
          constexpr bool PAIR = JN % 2 == 0;
          constexpr int TWS = Cfg::kLmax / (256 * R0);
          const int cg = (it.tile * Cfg::kSub0 + u) % p.cols0;
          const int col0 = JN * warp;
          auto ld = [&](int jn, int n) {
            return lds_elem<WIDE>(base + ctile_off<C0, ES>(col_in_row_t<WIDE>(n), col0 + jn));
          };
          auto ldp = [&](int jp, int n, float2& x0, float2& x1) {
            lds_pair<WIDE>(base + ctile_off<C0, ES>(col_in_row_t<WIDE>(n), col0 + jp), x0, x1);
          };
          auto oaddr = [&](int jn, int k, int q) {
            return base + ctile_off<C0, ES>(col_out_row((k - q) / R0, q), col0 + jn);
          };
          if constexpr (Cfg::k1D) {
            // W^(n2 k), k = q + R0 k' = W^(n2 q) * W^(n2 R0 k'): factors per job and thread
            float2 fk[JN][8], fq[JN][R0];
#pragma unroll
            for (int jn = 0; jn < JN; ++jn) {
              const int n2 = cg * C0 + col0 + jn;
#pragma unroll
              for (int sl = 0; sl < 8; ++sl) {
                const float2 f = wn(n2 * R0 * jc.kval[sl >> 2][(sl >> 1) & 1][sl & 1]);
                fk[jn][sl] = make_float2(f.x * wscale0, f.y * wscale0);
              }
#pragma unroll
              for (int q = 0; q < R0; ++q) fq[jn][q] = wn(n2 * q);
            }
            if constexpr (PAIR) {
              auto st = [&](int jp, int k, int q, int sl, float2 v0, float2 v1) {
                v0 = cmul(v0, cmul(fk[jp][sl], fq[jp][q]));
                v1 = cmul(v1, cmul(fk[jp + 1][sl], fq[jp + 1][q]));
                sts_pair<WIDE>(oaddr(jp, k, q), v0, v1);
              };
              fft256r_jobs<R0, SPLIT, TWS, JN, true>(jc, twR, p.dsign, ldp, st);
            } else {
              auto st = [&](int jn, int k, int q, int sl, float2 v) {
                sts_elem<WIDE>(oaddr(jn, k, q), cmul(v, cmul(fk[jn][sl], fq[jn][q])));
              };
              fft256r_jobs<R0, SPLIT, TWS, JN>(jc, twR, p.dsign, ld, st);
            }
          } else {
            if constexpr (PAIR) {
              auto st = [&](int jp, int k, int q, int, float2 v0, float2 v1) {
                sts_pair<WIDE>(oaddr(jp, k, q), v0, v1);
              };
              fft256r_jobs<R0, SPLIT, TWS, JN, true>(jc, twR, p.dsign, ldp, st);
            } else {
              auto st = [&](int jn, int k, int q, int, float2 v) { sts_elem<WIDE>(oaddr(jn, k, q), v); };
              fft256r_jobs<R0, SPLIT, TWS, JN>(jc, twR, p.dsign, ld, st);
            }
          }
         }
        } else {  // kRoleRow: contiguous rows j = warp + 8 jn in place (2D phase 0)
#pragma unroll 1
         for (int u = 0; u < Cfg::kSub0; ++u) {
          const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes) + u * (Cfg::kTile0 * ES);
          constexpr int JN = C0 / 8;
          auto rowb = [&](int jn) { return base + (uint32_t)((warp + 8 * jn) * 256 * R0 * ES); };
          auto ld = [&](int jn, int n) { return lds_elem<WIDE>(rowb(jn) + swz_w<ES>(n) * ES); };
          // outputs k = q + R0 k' of one slot are R0 consecutive elements: hold all q, then
          // store each slot's run with vector stores (conflict-free, like the single-pass kernel)
          Hold out[JN][R0][8];
          if constexpr (!WIDE) {
            plain_row_jobs<R0, JN, PI, RHO>(jc, fold0, rowb(0), 8 * 256 * R0 * ES, p.dsign, out);
          } else {
            auto st = [&](int jn, int k, int q, int sl, float2 v) { out[jn][q][sl] = v; };
            fft256r_jobs<R0, SPLIT, Cfg::kLmax / (256 * R0), JN>(jc, twR, p.dsign, ld, st);
          }
#pragma unroll
          for (int jn = 0; jn < JN; ++jn)
#pragma unroll
            for (int sl = 0; sl < 8; ++sl) {
              const uint32_t rb = rowb(jn);
              const int k0 = R0 * jc.kval[sl >> 2][(sl >> 1) & 1][sl & 1];
              if constexpr (!WIDE) {
                if constexpr (R0 == 1) sts32(rb + swz_w<4>(k0) * 4, out[jn][0][sl]);
                else if constexpr (R0 == 2) sts64(rb + swz_w<4>(k0) * 4, out[jn][0][sl], out[jn][1][sl]);
                else {
#pragma unroll
                  for (int q4 = 0; q4 < R0; q4 += 4)
                    sts128(rb + swz_w<4>(k0 + q4) * 4, out[jn][q4][sl], out[jn][q4 + 1][sl], out[jn][q4 + 2][sl],
                           out[jn][q4 + 3][sl]);
                }
              } else {
                if constexpr (R0 == 1) sts64f(rb + swz_w<8>(k0) * 8, out[jn][0][sl]);
                else {
#pragma unroll
                  for (int q2 = 0; q2 < R0; q2 += 2)
                    sts128f(rb + swz_w<8>(k0 + q2) * 8, out[jn][q2][sl], out[jn][q2 + 1][sl]);
                }
              }
            }
         }
        }
      } else {
        if constexpr (ROLE1 == kRoleCol && !WIDE) {
#pragma unroll 1
          for (int u = 0; u < Cfg::kSub1; ++u)
            plain_col_tile<R1, C1, false, PI, RHO>(jc, fold1, base + u * (Cfg::kTile1 * ES), warp, p.dsign, 0, wn);
        } else if constexpr (ROLE1 == kRoleCol) {
#pragma unroll 1
         for (int u = 0; u < Cfg::kSub1; ++u) {
          const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes) + u * (Cfg::kTile1 * ES);
          constexpr int JN = C1 / 8;
          constexpr int TWS = Cfg::kLmax / (256 * R1);
          const int col0 = JN * warp;
          auto oaddr = [&](int jn, int k, int q) {
            return base + ctile_off<C1, ES>(col_out_row((k - q) / R1, q), col0 + jn);
          };
          if constexpr (JN % 2 == 0) {
            auto ldp = [&](int jp, int n, float2& x0, float2& x1) {
              lds_pair<WIDE>(base + ctile_off<C1, ES>(col_in_row_t<WIDE>(n), col0 + jp), x0, x1);
            };
            auto st = [&](int jp, int k, int q, int, float2 v0, float2 v1) {
              sts_pair<WIDE>(oaddr(jp, k, q), v0, v1);
            };
            fft256r_jobs<R1, SPLIT, TWS, JN, true>(jc, twR, p.dsign, ldp, st);
          } else {
            auto ld = [&](int jn, int n) {
              return lds_elem<WIDE>(base + ctile_off<C1, ES>(col_in_row_t<WIDE>(n), col0 + jn));
            };
            auto st = [&](int jn, int k, int q, int, float2 v) { sts_elem<WIDE>(oaddr(jn, k, q), v); };
            fft256r_jobs<R1, SPLIT, TWS, JN>(jc, twR, p.dsign, ld, st);
          }
         }
        } else if constexpr (ROLE1 == kRoleRow16T) {
          // 16 short rows per warp (one S1 job), held in registers, then written
          // transposed as [k0 + 16 q rows][C1 cols] in boxes of kBW columns
          static_assert(C1 == 128, "short-row tiles hold 8 warps x 16 rows");
          Hold out[8 * R1];
          {
            const uint32_t rb = base + (uint32_t)(warp * 16 * Cfg::kLen1 * ES);
            auto ld = [&](int v, int n) { return lds_elem<WIDE>(rb + swz_w<ES>(v * Cfg::kLen1 + n) * ES); };
            auto st = [&](int v, int k, int q, int sl, float2 val) {
              if constexpr (WIDE) out[8 * q + sl] = val;
              else out[8 * q + sl] = pack_h2(val.x, val.y);
            };
            if constexpr (WIDE) {
              fft16r_job<R1, SPLIT, Cfg::kLmax / (16 * R1), PI, RHO>(jc, twR, p.dsign, ld, st);
            } else {
              auto ldr = [&](int v, int n) { return lds32(rb + swz_w<4>(v * Cfg::kLen1 + n) * 4); };
              fft16r_job_fold<R1, PI, RHO>(jc, fold1, p.dsign, ldr, st);
            }
          }
          named_bar_sync(1, 256);
          {
            const int lane_g = lane >> 2, lane_t = lane & 3;
#pragma unroll
            for (int q = 0; q < R1; ++q)
#pragma unroll
              for (int sl = 0; sl < 8; ++sl) {
                const int jj = sl >> 2, h = (sl >> 1) & 1, e = sl & 1;
                const int col = warp * 16 + 2 * lane_t + e + 8 * jj;
                const int row = RHO::apply(lane_g + 8 * h) + 16 * q;
                const uint32_t addr = base + (uint32_t)((col / Cfg::kBW) * (Cfg::kBW * Cfg::kLen1 * ES)) +
                                      ctile_off<Cfg::kBW, ES>(row, col % Cfg::kBW);
                if constexpr (WIDE) sts64f(addr, out[8 * q + sl]);
                else sts32(addr, out[8 * q + sl]);
              }
          }
        } else {  // kRoleRowT: rows j = JN warp + jn -> transposed output tile in the same stage
          static_assert(C1 % 8 == 0, "row-transpose tiles hold a multiple of 8 rows");
          constexpr int JN = C1 / 8;
          constexpr uint32_t kRow = 256 * R1 * ES;   // bytes per input row
          constexpr uint32_t kStep = 256 * C1 * ES;  // output tile: one q further down
          const int row0 = JN * warp;                // output columns row0 + jn sit side by side
#pragma unroll 1
         for (int u = 0; u < Cfg::kSub1; ++u) {       // the item's tiles, one after the other
          const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes) + u * (Cfg::kTile1 * ES);
          Hold out[JN][R1][8];
          if constexpr (!WIDE) {
            plain_row_jobs<R1, JN, PI, RHO>(jc, fold1, base + row0 * kRow, kRow, p.dsign, out);
          } else {
            auto ld = [&](int jn, int n) { return lds_elem<WIDE>(base + (row0 + jn) * kRow + swz_w<ES>(n) * ES); };
            auto st = [&](int jn, int k, int q, int sl, float2 v) { out[jn][q][sl] = v; };
            fft256r_jobs<R1, SPLIT, Cfg::kLmax / (256 * R1), JN>(jc, twR, p.dsign, ld, st);
          }
          named_bar_sync(1, 256);  // every compute warp finished reading the stage
#pragma unroll
          for (int sl = 0; sl < 8; ++sl) {
            const uint32_t so = base + ctile_off<C1, ES>(col_out_row(slot_kval<PI, RHO>(sl), 0), row0);
#pragma unroll
            for (int q = 0; q < R1; ++q) {
              if constexpr (!WIDE && JN == 4) {  // 128-byte rows: one 16-byte store per slot
                sts128(so + q * kStep, out[0][q][sl], out[1][q][sl], out[2][q][sl], out[3][q][sl]);
              } else if constexpr (JN % 2 == 0) {
#pragma unroll
                for (int jp = 0; jp < JN; jp += 2) {
                  const uint32_t addr = so + jp * ES + q * kStep;
                  if constexpr (WIDE) sts128f(addr, out[jp][q][sl], out[jp + 1][q][sl]);
                  else sts64(addr, out[jp][q][sl], out[jp + 1][q][sl]);
                }
              } else {
#pragma unroll
                for (int jn = 0; jn < JN; ++jn) {
                  const uint32_t addr = so + jn * ES + q * kStep;
                  if constexpr (WIDE) sts64f(addr, out[jn][q][sl]);
                  else sts32(addr, out[jn][q][sl]);
                }
              }
            }
          }
         }
        }
      }
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&computed[s]);
    if (!ok) break;
    ++cnt;
  }
}

}  // namespace tcfft
