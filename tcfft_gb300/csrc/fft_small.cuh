// fft_small.cuh -- single-pass kernels for transforms of N = 256*R points
// (R in {1,2,4,8}: N = 256 ... 2048), one HBM round trip per element.
//
// Replaces the reference's layer_{256,512,1024}_0 kernels
// (tcfft_half.cu:69-161, 586-699, 1011-1095), which compute the same
// contiguous sub-FFTs with WMMA and fp16 accumulation on digit-reversed input.
// Here the input is in natural order and the algorithm is decimation in
// frequency:  n = m + 256 a,  k = q + R k',
//   X[q + R k'] = sum_m W256^(m k') [ W_N^(m q) sum_a x[m + 256 a] W_R^(a q) ]
// i.e. a radix-R butterfly over a (fp32, registers), a twiddle, then a
// 256-point FFT per q done as two radix-16 tensor-core stages
// (m = 16 m1 + m0:  sum over m1 -> k0, twiddle W256^(m0 k0), sum over m0 -> k1,
// k' = k0 + 16 k1).  Everything between the TMA load and the TMA store stays
// in registers.
//
// CTA structure: persistent CTAs, 8 warps, a ring of NSTAGE shared-memory
// tiles filled by 2D TMA loads (128B swizzle) and drained by TMA stores; tiles
// are loaded through one tensor map and stored to the same rows through another
// (the same map in place, the output buffer's map out of place).
#pragma once
#include "fft_common.cuh"
#include "fft_job.cuh"

namespace tcfft {

// MODE: kModePlain (fp16 data and arithmetic), kModeSplit (fp32 data, hi/lo
// split products), kModeIo32 (fp32 data converted to fp16 operands as they are
// read from shared memory, fp32 results stored: one product per stage).
template <int R, int MODE>
struct SmallCfg {
  static constexpr bool kWide = MODE != kModePlain;      // 8-byte (float2) elements
  static constexpr bool kSplit = MODE == kModeSplit;     // three products per stage
  static constexpr int kN = 256 * R;
  static constexpr int kES = kWide ? 8 : 4;              // bytes per complex element
  static constexpr int kER = 128 / kES;                  // elements per 128-byte row
  static constexpr int kBoxElems = kER * 256;            // one TMA box: 256 rows
  static constexpr int kJPW = kWide ? (R >= 2 ? 1 : 2) : (R >= 4 ? 1 : 4 / R);  // jobs per warp
  // 8-byte elements at N = 2048: two warps per transform, each computing four of the eight
  // radix-8 sub-transforms, so that a tile of four transforms is one 64 KiB stage
  static constexpr bool kPair = kWide && R == 8;
  static constexpr int kQH = kPair ? R / 2 : R;           // sub-transforms q per warp
  static constexpr int kJobs = kPair ? 4 : 8 * kJPW;      // transforms per tile
  static constexpr int kTE = kJobs * kN;                  // elements per tile
  static constexpr int kBoxes = kTE / kBoxElems;
  static constexpr int kTileBytes = kTE * kES;
  static constexpr int kStages = 3;
  // split: W_N^j table (radix-R twiddles); plain: the folded radix-R tables (per-q DFT
  // matrices and stage-1 twiddles, fft256r_jobs_fold) in place of it
  static constexpr bool kFold = !kWide && R > 1;
  static constexpr int kTabBytes = kFold ? FoldTab<R>::kBytes : (R > 1 ? kN * 8 : 0);
  static constexpr int kSmem = kStages * kTileBytes + kTabBytes + 1024 + 64;
  static constexpr int kMinBlocks = (kSmem <= 112 * 1024) ? 2 : 1;
  static_assert(kTE % kBoxElems == 0, "tile must be whole TMA boxes");
  // bank-conflict-free slot permutations (see fft_common.cuh)
  using PI = typename std::conditional<kWide, BitPerm<0, 1, 2, 3>, BitPerm<0, 1, 3, 2>>::type;
  using RHO = typename std::conditional<
      kWide,
      typename std::conditional<R == 1, BitPerm<1, 0, 3, 2>, BitPerm<0, 2, 3, 1>>::type,
      typename std::conditional<R == 1, BitPerm<2, 0, 1, 3>,
                                typename std::conditional<R == 2, BitPerm<1, 0, 3, 2>, BitPerm<0, 2, 3, 1>>::type>::type>::type;
};

struct SmallParams {
  const float2* tw;  // W_2048^j, j < 2048, direction-specific (fp32 from fp64)
  int num_tiles;
  float dsign;       // +1 forward, -1 adjoint (conjugate direction)
  int* err;
  float oscale;      // output scale (a power of two; 1/N for a normalised transform), carried
                     // by the stage-1 twiddles, so it costs nothing per element
};

template <int R, int MODE>
__global__ void __launch_bounds__(256, SmallCfg<R, MODE>::kMinBlocks)
    fft_small_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap omap,
                     const SmallParams p) {
  using C = SmallCfg<R, MODE>;
  constexpr bool WIDE = C::kWide, SPLIT = C::kSplit;
  using PI = typename C::PI;
  using RHO = typename C::RHO;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float2* s_tw = reinterpret_cast<float2*>(smem + C::kStages * C::kTileBytes);
  const uint32_t s_tw_addr = smem_addr(s_tw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::kStages * C::kTileBytes + C::kTabBytes);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int ntile_cta = (p.num_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;

  if (tid == 0) {
    prefetch_tmap(&tmap);
    prefetch_tmap(&omap);
    for (int s = 0; s < C::kStages; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  if constexpr (C::kFold)
    build_fold_table<R, PI, RHO>(reinterpret_cast<unsigned char*>(s_tw), p.tw, tid, blockDim.x, p.oscale);
  else if constexpr (R > 1)
    for (int j = tid; j < C::kN; j += blockDim.x) s_tw[j] = p.tw[j * (2048 / C::kN)];
  __syncthreads();

  auto issue_load = [&](int i) {  // thread 0 only: tile #i of this CTA into stage i % kStages
    const int tile = blockIdx.x + i * gridDim.x;
    const int s = i % C::kStages;
    mbar_arrive_expect_tx(&full[s], C::kTileBytes);
#pragma unroll
    for (int b = 0; b < C::kBoxes; ++b)
      tma_load_2d(smem + s * C::kTileBytes + b * C::kBoxElems * C::kES, &tmap, 0,
                  tile * (C::kTE / C::kER) + b * 256, &full[s]);
  };
  if (tid == 0)
    for (int i = 0; i < C::kStages && i < ntile_cta; ++i) issue_load(i);

  // ---- per-thread constants
  JobConsts<false> jc;  // the fold path's fragments and stage-1 twiddles
  if constexpr (C::kFold) {
    init_job_consts<false, PI, RHO>(jc, p.tw);
    scale_tw1(jc, p.oscale);
  }
  uint32_t afr[2][2][4], afr_lo[2][2][4];
  build_dft_frags<PI, RHO>(p.tw, 128, afr, afr_lo, SPLIT);
  float2 tw1[2][2][2];  // W256^(m0 k0) for stage-1 output (j, h, e)
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int m0 = PI::apply(2 * t + e + 8 * j), k0 = RHO::apply(g + 8 * h);
        const float2 w = p.tw[((m0 * k0) & 255) * 8];
        tw1[j][h][e] = make_float2(w.x * p.oscale, w.y * p.oscale);
      }
  uint32_t in_off[2][2][2];   // physical element offset of load slot (kt, r, j) in tile a = 0
  int mval[2][2][2];          // m = 16 m1 + m0 of that slot
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int m = 16 * PI::apply(2 * t + r + 8 * kt) + PI::apply(g + 8 * j);
        mval[kt][r][j] = m;
        in_off[kt][r][j] = swz_w<C::kES>(m);
      }
  uint32_t out_off[2][2][2];  // physical offset of output slot (h, e, hh) for q = 0 (k = R k')
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int kp = RHO::apply(2 * t + e + 8 * h) + 16 * RHO::apply(g + 8 * hh);
        out_off[h][e][hh] = swz_w<C::kES>(R * kp);
      }

  int issued = 0;  // thread 0: loads issued so far (tiles [0, issued) of this CTA)
  if (tid == 0) issued = ntile_cta < C::kStages ? ntile_cta : C::kStages;
  bool failed = false;
  for (int i = 0; i < ntile_cta; ++i) {
    const int s = i % C::kStages;
    const bool ok = mbar_wait(&full[s], (i / C::kStages) & 1, p.err);
    unsigned char* tile_base = smem + s * C::kTileBytes;

#pragma unroll 1
    for (int jj = 0; jj < (ok ? C::kJPW : 0); ++jj) {
      const int job_idx = C::kPair ? (warp >> 1) : warp * C::kJPW + jj;
      const uint32_t job = smem_addr(tile_base) + (uint32_t)(job_idx * C::kN * C::kES);
      if constexpr (C::kFold) {
        // plain R > 1: radix-R butterfly on packed half2, twiddles folded into the
        // per-q tensor-core stages; outputs k = q + R k' collected, then stored as R-runs
        uint32_t res[R][8];
        auto ld = [&](int, int slot, int a) {
          return lds32(job + (uint32_t)(a * 256 + in_off[slot >> 2][(slot >> 1) & 1][slot & 1]) * 4);
        };
        auto st = [&](int, int osl, int q, float2 v) { res[q][osl] = pack_h2(v.x, v.y); };
        fft256r_jobs_fold<R, 1, false>(jc, s_tw_addr, p.dsign, ld, st);
#pragma unroll
        for (int osl = 0; osl < 8; ++osl) {
          const uint32_t ob = out_off[osl >> 2][(osl >> 1) & 1][osl & 1];
          if constexpr (R == 2) {
            sts64(job + ob * 4, res[0][osl], res[1][osl]);
          } else {
#pragma unroll
            for (int q4 = 0; q4 < R; q4 += 4)
              sts128(job + swz_w<4>(swz_w<4>(ob) + q4) * 4, res[q4][osl], res[q4 + 1][osl], res[q4 + 2][osl],
                     res[q4 + 3][osl]);
          }
        }
        continue;
      }
      // ---------------- load + radix-R (DIF) + twiddle -> B operands per tile q
      // (kPair: this warp keeps the sub-transforms q0 .. q0 + QH - 1)
      constexpr int QH = C::kQH;
      const int q0 = C::kPair ? (warp & 1) * QH : 0;
      uint32_t bhi[QH][2][2][2], blo[SPLIT ? QH : 1][2][2][2];
      float2 xs[SPLIT ? QH : 1][2][2][2];  // split: fp32 operands until the job's scale is known
      float inv = 1.f;
#pragma unroll
      for (int kt = 0; kt < 2; ++kt)
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            if constexpr (!WIDE && R == 1) {
              bhi[0][kt][r][j] = lds32(job + in_off[kt][r][j] * 4);
            } else {
              float2 x[R];
#pragma unroll
              for (int a = 0; a < R; ++a) {
                const uint32_t addr = job + (uint32_t)(a * 256 + in_off[kt][r][j]) * C::kES;
                if constexpr (WIDE) x[a] = lds64f(addr);
                else x[a] = unpack_h2(lds32(addr));
              }
              if constexpr (R > 1) dft_small<R>(x, p.dsign);
#pragma unroll
              for (int qq = 0; qq < QH; ++qq) {
                // this warp's half of the outputs (constant indices: x stays in registers)
                float2 v = (C::kPair && q0 != 0) ? x[(QH + qq) % R] : x[qq];
                const int q = q0 + qq;
                if (R > 1 && q > 0) v = cmul(v, lds64f(s_tw_addr + ((mval[kt][r][j] * q) & (C::kN - 1)) * 8));
                if constexpr (SPLIT) xs[qq][kt][r][j] = v;
                else bhi[qq][kt][r][j] = pack_h2(v.x, v.y);
              }
            }
          }
      if constexpr (SPLIT) {
        float m = 0.f;
#pragma unroll
        for (int q = 0; q < QH; ++q)
#pragma unroll
          for (int kt = 0; kt < 2; ++kt)
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
              for (int j = 0; j < 2; ++j)
                m = fmaxf(m, fmaxf(fabsf(xs[q][kt][r][j].x), fabsf(xs[q][kt][r][j].y)));
        float sc;
        split_scale(warp_max(m), sc, inv);
#pragma unroll
        for (int q = 0; q < QH; ++q)
#pragma unroll
          for (int kt = 0; kt < 2; ++kt)
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
              for (int j = 0; j < 2; ++j) {
                const float2 v = xs[q][kt][r][j];
                split_h2(make_float2(v.x * sc, v.y * sc), bhi[q][kt][r][j], blo[q][kt][r][j]);
              }
      }
      // all lanes (kPair: of both warps of the transform) finished reading its region (in place)
      if constexpr (C::kPair) asm volatile("bar.sync %0, 64;" ::"r"(1 + (warp >> 1)) : "memory");
      else __syncwarp();

      // ---------------- two radix-16 tensor-core stages per tile q
      float2 res[QH][2][2][2];  // wide: fp32 results; plain: packed half2 in .x bits
#pragma unroll
      for (int q = 0; q < QH; ++q) {
        float acc[2][2][4];
        if constexpr (SPLIT) dft16_mma_split(afr, afr_lo, bhi[q], blo[q], acc);
        else dft16_mma(afr, bhi[q], acc);
        uint32_t b2[2][2][2], b2lo[2][2][2];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt)
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const float2 v = cmul(acc_get(acc, kt, h, r), tw1[kt][h][r]);
              if constexpr (SPLIT) split_h2(v, b2[kt][r][h], b2lo[kt][r][h]);
              else b2[kt][r][h] = pack_h2(v.x, v.y);
            }
        if constexpr (SPLIT) dft16_mma_split(afr, afr_lo, b2, b2lo, acc);
        else dft16_mma(afr, b2, acc);
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              const float2 v = acc_get(acc, h, hh, e);
              if constexpr (SPLIT) res[q][h][e][hh] = make_float2(v.x * inv, v.y * inv);
              else if constexpr (WIDE) res[q][h][e][hh] = v;
              else res[q][h][e][hh].x = __uint_as_float(pack_h2(v.x, v.y));
            }
      }
      // ---------------- store natural order: k = q + R k'
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const uint32_t base = job + out_off[h][e][hh] * C::kES;
            if constexpr (!WIDE) {
              if constexpr (R == 1) sts32(base, __float_as_uint(res[0][h][e][hh].x));
              else if constexpr (R == 2)
                sts64(base, __float_as_uint(res[0][h][e][hh].x), __float_as_uint(res[1][h][e][hh].x));
              else {
#pragma unroll
                for (int q4 = 0; q4 < R; q4 += 4) {
                  // consecutive 16-byte chunks of the same row: chunk index differs by one
                  const uint32_t addr = job + swz_w<4>(swz_w<4>(out_off[h][e][hh]) + q4) * 4;
                  sts128(addr, __float_as_uint(res[q4][h][e][hh].x), __float_as_uint(res[q4 + 1][h][e][hh].x),
                         __float_as_uint(res[q4 + 2][h][e][hh].x), __float_as_uint(res[q4 + 3][h][e][hh].x));
                }
              }
            } else {
              if constexpr (R == 1) sts64f(base, res[0][h][e][hh]);
              else {
#pragma unroll
                for (int q2 = 0; q2 < QH; q2 += 2) {
                  const uint32_t addr = job + swz_w<8>(swz_w<8>(out_off[h][e][hh]) + q0 + q2) * 8;
                  sts128f(addr, res[q2][h][e][hh], res[q2 + 1][h][e][hh]);
                }
              }
            }
          }
    }
    // ---------------- hand the tile to the TMA store, refill the ring
    fence_proxy_async_smem();
    if (__syncthreads_or(!ok)) {  // a bounded wait expired somewhere: stop consistently
      failed = true;
      break;
    }
    if (tid == 0) {
      const int tile = blockIdx.x + i * gridDim.x;
#pragma unroll
      for (int b = 0; b < C::kBoxes; ++b)
        tma_store_2d(&omap, 0, tile * (C::kTE / C::kER) + b * 256, tile_base + b * C::kBoxElems * C::kES);
      bulk_commit();
      // the store issued in iteration i-1 has finished reading its stage -> reuse it
      if (i >= 1 && i - 1 + C::kStages < ntile_cta) {
        bulk_wait_read<1>();
        issue_load(i - 1 + C::kStages);
        ++issued;
      }
    }
  }
  if (tid == 0) {
    if (failed) {  // let loads still in flight land before the CTA exits (bounded)
      for (int i = 0; i < issued; ++i) mbar_wait(&full[i % C::kStages], (i / C::kStages) & 1, nullptr);
    }
    bulk_wait<0>();
  }
}

}  // namespace tcfft
