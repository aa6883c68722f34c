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

// Multiply the stage-1 -> stage-2 twiddles by s (a power of two): every job
// output then comes out scaled by s exactly, at no cost per element.
template <bool SPLIT>
__device__ __forceinline__ void scale_tw1(JobConsts<SPLIT>& c, float s) {
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e) c.tw1[j][h][e] = make_float2(c.tw1[j][h][e].x * s, c.tw1[j][h][e].y * s);
}

// JN independent jobs computed in lockstep by one warp (JN = 1 or 2): their
// instruction streams interleave, which hides MMA/shared-memory latency when
// only two warps share a scheduler.
// LOAD(jn, n) -> float2 element n (0 <= n < 256R) of job jn's input.
// STORE(jn, k, q, slot, float2) receives output k = q + R * kval[slot] of job
// jn in fp32 (slot = 4h + 2e + hh; jn, q, slot compile-time after unrolling).
// PAIR (JN even): jobs 2i and 2i+1 sit side by side in memory and move together,
// LOAD(2i, n, float2& x0, float2& x1) and STORE(2i, k, q, slot, v0, v1), so one
// 8- or 16-byte shared access serves both.
// All LOADs of the warp complete (and are ordered by __syncwarp) before the
// first STORE, so a job may write its output over its own input.
// twR: shared-memory address of a table with W_{256R}^j at index j*TWS (read
// with ld.shared), used for the radix-R twiddles.
template <int R, bool SPLIT, int TWS, int JN, bool PAIR = false, class LoadF, class StoreF>
__device__ __forceinline__ void fft256r_jobs(const JobConsts<SPLIT>& c, uint32_t twR, float dsign, LoadF&& load,
                                             StoreF&& store) {
  static_assert(!PAIR || JN % 2 == 0, "paired jobs come in twos");
  uint32_t bhi[JN][R][2][2][2], blo[JN][SPLIT ? R : 1][2][2][2];
  float2 xs[SPLIT ? JN : 1][SPLIT ? R : 1][2][2][2];  // split: fp32 operands until the scale is known
  float inv[JN];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int m = c.mval[kt][r][j];
        float2 x[JN][R];
#pragma unroll
        for (int a = 0; a < R; ++a) {
          if constexpr (PAIR) {
#pragma unroll
            for (int jp = 0; jp < JN; jp += 2) load(jp, m + 256 * a, x[jp][a], x[jp + 1][a]);
          } else {
#pragma unroll
            for (int jn = 0; jn < JN; ++jn) x[jn][a] = load(jn, m + 256 * a);
          }
        }
        if constexpr (R > 1) {
          float2 w[R];  // W_{256R}^(m q), shared by the jobs
#pragma unroll
          for (int q = 1; q < R; ++q) w[q] = lds64f(twR + ((m * q) & (256 * R - 1)) * TWS * 8);
#pragma unroll
          for (int jn = 0; jn < JN; ++jn) {
            dft_small<R>(x[jn], dsign);
#pragma unroll
            for (int q = 1; q < R; ++q) x[jn][q] = cmul(x[jn][q], w[q]);
          }
        }
#pragma unroll
        for (int jn = 0; jn < JN; ++jn)
#pragma unroll
          for (int q = 0; q < R; ++q) {
            if constexpr (SPLIT) xs[jn][q][kt][r][j] = x[jn][q];
            else bhi[jn][q][kt][r][j] = pack_h2(x[jn][q].x, x[jn][q].y);
          }
      }
  if constexpr (SPLIT) {
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) {
      float m = 0.f;
#pragma unroll
      for (int q = 0; q < R; ++q)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt)
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int j = 0; j < 2; ++j)
              m = fmaxf(m, fmaxf(fabsf(xs[jn][q][kt][r][j].x), fabsf(xs[jn][q][kt][r][j].y)));
      float sc;
      split_scale(warp_max(m), sc, inv[jn]);
#pragma unroll
      for (int q = 0; q < R; ++q)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt)
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const float2 v = xs[jn][q][kt][r][j];
              split_h2(make_float2(v.x * sc, v.y * sc), bhi[jn][q][kt][r][j], blo[jn][q][kt][r][j]);
            }
    }
  } else {
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) inv[jn] = 1.f;
  }
  __syncwarp();  // every lane has read the jobs' inputs (stores may alias them)
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float acc[JN][2][2][4];
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) {
      if constexpr (SPLIT) dft16_mma_split(c.afr, c.afr_lo, bhi[jn][q], blo[jn][q], acc[jn]);
      else dft16_mma(c.afr, bhi[jn][q], acc[jn]);
    }
    uint32_t b2[JN][2][2][2], b2lo[JN][2][2][2];
#pragma unroll
    for (int jn = 0; jn < JN; ++jn)
#pragma unroll
      for (int kt = 0; kt < 2; ++kt)
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float2 v = cmul(acc_get(acc[jn], kt, h, r), c.tw1[kt][h][r]);
            if constexpr (SPLIT) split_h2(v, b2[jn][kt][r][h], b2lo[jn][kt][r][h]);
            else b2[jn][kt][r][h] = pack_h2(v.x, v.y);
          }
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) {
      if constexpr (SPLIT) dft16_mma_split(c.afr, c.afr_lo, b2[jn], b2lo[jn], acc[jn]);
      else dft16_mma(c.afr, b2[jn], acc[jn]);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          float2 v[JN];
#pragma unroll
          for (int jn = 0; jn < JN; ++jn) {
            v[jn] = acc_get(acc[jn], h, hh, e);
            if constexpr (SPLIT) v[jn] = make_float2(v[jn].x * inv[jn], v[jn].y * inv[jn]);
          }
          const int k = q + R * c.kval[h][e][hh], sl = 4 * h + 2 * e + hh;
          if constexpr (PAIR) {
#pragma unroll
            for (int jp = 0; jp < JN; jp += 2) store(jp, k, q, sl, v[jp], v[jp + 1]);
          } else {
#pragma unroll
            for (int jn = 0; jn < JN; ++jn) store(jn, k, q, sl, v[jn]);
          }
        }
  }
}


// ---------------------------------------------------------------------------
// Plain precision with the radix-R twiddle folded into the two MMA stages.
//
// W_{256R}^(m q) = W_{16R}^(m1 q) W_{256R}^(m0 q) for m = 16 m1 + m0, so the
// sub-transform q is computed as
//   stage 1:  A_q[k0][m1] = W16^(m1 k0) W_{16R}^(m1 q)      (a per-q DFT matrix)
//   twiddle:  T_q[m0][k0] = W_{256R}^(m0 (R k0 + q))        (= W256^(m0 k0) W_{256R}^(m0 q))
//   stage 2:  F16 over m0
// and the radix-R step is only the butterfly.  A_0 = F16 and T_0 = W256 stay in
// registers (JobConsts); A_q and T_q for q >= 1 are per-lane tables in shared
// memory, entry-major ([entry][lane]) so that the 32 lanes of a warp read 32
// consecutive words (no bank conflicts).
template <int R>
struct FoldTab {
  static constexpr int kABytes = (R - 1) * 16 * 32 * 4;  // A_q fragments: [q-1][ct kt reg][lane] u32
  static constexpr int kTBytes = (R - 1) * 8 * 32 * 8;   // T_q: [q-1][j h e][lane] float2
  static constexpr int kBytes = kABytes + kTBytes;
};

// Fill one fold table (all threads of the CTA take part; tw2048 = W_2048^j).
// WITH_T = false: the A_q part only (16R-point row jobs have no second stage).
// tscale multiplies the stage-1 twiddles T_q (a power of two: the jobs' outputs
// come out scaled by it exactly; together with JobConsts::tw1 it carries the
// 1/N of a normalised transform).
template <int R, class PI, class RHO, bool WITH_T = true>
__device__ void build_fold_table(unsigned char* tab, const float2* __restrict__ tw2048, int tid, int nthreads,
                                 float tscale = 1.f) {
  if constexpr (R > 1) {
    uint32_t* A = reinterpret_cast<uint32_t*>(tab);
    for (int idx = tid; idx < (R - 1) * 16 * 32; idx += nthreads) {
      const int q = idx / 512 + 1, e = (idx >> 5) & 15, lane = idx & 31, g = lane >> 2, t = lane & 3;
      const int ct = e >> 3, kt = (e >> 2) & 1, reg = e & 3;
      const int k0 = RHO::apply(g + 8 * (reg & 1)), m1 = PI::apply(2 * t + (reg >> 1) + 8 * kt);
      const float2 w = tw2048[((m1 * (R * k0 + q)) & (16 * R - 1)) * (128 / R)];  // W_{16R}^(m1 (R k0 + q))
      A[idx] = ct == 0 ? pack_h2(w.x, -w.y) : pack_h2(w.y, w.x);
    }
    float2* T = reinterpret_cast<float2*>(tab + FoldTab<R>::kABytes);
    for (int idx = tid; idx < (WITH_T ? (R - 1) * 8 * 32 : 0); idx += nthreads) {
      const int q = idx / 256 + 1, sl = (idx >> 5) & 7, lane = idx & 31, g = lane >> 2, t = lane & 3;
      const int j = sl >> 2, h = (sl >> 1) & 1, e = sl & 1;
      const int m0 = PI::apply(2 * t + e + 8 * j), k0 = RHO::apply(g + 8 * h);
      const float2 w = tw2048[((m0 * (R * k0 + q)) & (256 * R - 1)) * (8 / R)];  // W_{256R}^(m0 (R k0 + q))
      T[idx] = make_float2(w.x * tscale, w.y * tscale);
    }
  }
}

// JN jobs of length 256R in lockstep, plain precision, folded twiddles; the
// radix-R butterfly runs on the packed half2 inputs (no fp32 round trip).
// LOAD(jn, slot, a) -> packed half2 input element m(slot) + 256 a of job jn,
// where slot = 4 kt + 2 r + j is the B-fragment slot (m = 16 PI(2t + r + 8kt) +
// PI(g + 8j)); with PAIR, LOAD(jp, slot, a, uint32_t& x0, uint32_t& x1) for jobs
// jp, jp + 1.  STORE(jn, osl, q, float2) receives output q + R kval(osl) of
// job jn (osl = 4h + 2e + hh, kval = RHO(2t + e + 8h) + 16 RHO(g + 8hh)); with
// PAIR, STORE(jp, osl, q, v0, v1).  All loads precede the first store.
// tab: shared-memory address of this R's fold table.
// QUAD (JN = 4, with PAIR): the four jobs' elements of one slot move together,
// LOAD(0, slot, a, x0, x1, x2, x3) and STORE(0, osl, q, v0, v1, v2, v3).
template <int R, int JN, bool PAIR, class LoadF, class StoreF, bool QUAD = false>
__device__ __forceinline__ void fft256r_jobs_fold_impl(const JobConsts<false>& c, uint32_t tab, float dsign,
                                                       LoadF&& load, StoreF&& store, const float2* tglob) {
  static_assert(!PAIR || JN % 2 == 0, "paired jobs come in twos");
  static_assert(!QUAD || (PAIR && JN == 4), "quads are four paired jobs");
  const uint32_t lane4 = (threadIdx.x & 31) * 4;
  const uint32_t negmask = dsign > 0.f ? 0x80000000u : 0x00008000u;
  const uint32_t c8 = pack_h2(0.70710678118654752440f, 0.70710678118654752440f);
  uint32_t bhi[JN][R][2][2][2];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int slot = 4 * kt + 2 * r + j;
        uint32_t x[JN][R];
#pragma unroll
        for (int a = 0; a < R; ++a) {
          if constexpr (QUAD) {
            load(0, slot, a, x[0][a], x[1][a], x[2][a], x[3][a]);
          } else if constexpr (PAIR) {
#pragma unroll
            for (int jp = 0; jp < JN; jp += 2) load(jp, slot, a, x[jp][a], x[jp + 1][a]);
          } else {
#pragma unroll
            for (int jn = 0; jn < JN; ++jn) x[jn][a] = load(jn, slot, a);
          }
        }
#pragma unroll
        for (int jn = 0; jn < JN; ++jn) {
          if constexpr (R > 1) dft_small_h<R>(x[jn], negmask, c8);
#pragma unroll
          for (int q = 0; q < R; ++q) bhi[jn][q][kt][r][j] = x[jn][q];
        }
      }
  __syncwarp();  // every lane has read the jobs' inputs (stores may alias them)
#pragma unroll
  for (int q = 0; q < R; ++q) {
    uint32_t aq[2][2][4];
    if (q == 0) {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = c.afr[i >> 3][(i >> 2) & 1][i & 3];
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = lds32(tab + ((q - 1) * 16 + i) * 128 + lane4);
    }
    float acc[JN][2][2][4];
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) dft16_mma(aq, bhi[jn][q], acc[jn]);
    uint32_t b2[JN][2][2][2];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          // T_q from the table's T part in shared memory or, with tglob, from a copy of it in
          // global memory (same [q - 1][slot][lane] layout)
          const int ti = ((q - 1) * 8 + 4 * kt + 2 * h + r) * 32;
          const float2 w = q == 0 ? c.tw1[kt][h][r]
                           : tglob ? __ldg(tglob + ti + (threadIdx.x & 31))
                                   : lds64f(tab + FoldTab<R>::kABytes + ti * 8 + lane4 * 2);
#pragma unroll
          for (int jn = 0; jn < JN; ++jn) {
            const float2 v = cmul(acc_get(acc[jn], kt, h, r), w);
            b2[jn][kt][r][h] = pack_h2(v.x, v.y);
          }
        }
#pragma unroll
    for (int jn = 0; jn < JN; ++jn) dft16_mma(c.afr, b2[jn], acc[jn]);
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int osl = 4 * h + 2 * e + hh;
          if constexpr (QUAD) {
            store(0, osl, q, acc_get(acc[0], h, hh, e), acc_get(acc[1], h, hh, e), acc_get(acc[2], h, hh, e),
                  acc_get(acc[3], h, hh, e));
          } else if constexpr (PAIR) {
#pragma unroll
            for (int jp = 0; jp < JN; jp += 2)
              store(jp, osl, q, acc_get(acc[jp], h, hh, e), acc_get(acc[jp + 1], h, hh, e));
          } else {
#pragma unroll
            for (int jn = 0; jn < JN; ++jn) store(jn, osl, q, acc_get(acc[jn], h, hh, e));
          }
        }
  }
}

// tglob: the fold table's T part in global memory (nullptr: in shared memory after the A part).
template <int R, int JN, bool PAIR, class LoadF, class StoreF>
__device__ __forceinline__ void fft256r_jobs_fold(const JobConsts<false>& c, uint32_t tab, float dsign, LoadF&& load,
                                                  StoreF&& store, const float2* tglob = nullptr) {
  fft256r_jobs_fold_impl<R, JN, PAIR, LoadF, StoreF, false>(c, tab, dsign, static_cast<LoadF&&>(load),
                                                            static_cast<StoreF&&>(store), tglob);
}
template <int R, class LoadF, class StoreF>
__device__ __forceinline__ void fft256r_jobs_fold_quad(const JobConsts<false>& c, uint32_t tab, float dsign,
                                                       LoadF&& load, StoreF&& store, const float2* tglob = nullptr) {
  fft256r_jobs_fold_impl<R, 4, true, LoadF, StoreF, true>(c, tab, dsign, static_cast<LoadF&&>(load),
                                                          static_cast<StoreF&&>(store), tglob);
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
// tw16R: shared-memory address of a table with W_{16R}^j at index j*TWS.
template <int R, bool SPLIT, int TWS, class PI, class RHO, class LoadF, class StoreF>
__device__ __forceinline__ void fft16r_job(const JobConsts<SPLIT>& c, uint32_t tw16R, float dsign, LoadF&& load,
                                           StoreF&& store) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t bhi[R][2][2][2], blo[SPLIT ? R : 1][2][2][2];
  float2 xs[SPLIT ? R : 1][2][2][2];
  float inv = 1.f;
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
          for (int q = 1; q < R; ++q) x[q] = cmul(x[q], lds64f(tw16R + ((m1 * q) & (16 * R - 1)) * TWS * 8));
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
          if constexpr (SPLIT) xs[q][kt][r][j] = x[q];
          else bhi[q][kt][r][j] = pack_h2(x[q].x, x[q].y);
        }
      }
  if constexpr (SPLIT) {
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < R; ++q)
#pragma unroll
      for (int kt = 0; kt < 2; ++kt)
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int j = 0; j < 2; ++j) m = fmaxf(m, fmaxf(fabsf(xs[q][kt][r][j].x), fabsf(xs[q][kt][r][j].y)));
    float sc;
    split_scale(warp_max(m), sc, inv);
#pragma unroll
    for (int q = 0; q < R; ++q)
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
        for (int e = 0; e < 2; ++e) {
          float2 v = acc_get(acc, j, h, e);
          if constexpr (SPLIT) v = make_float2(v.x * inv, v.y * inv);
          store(2 * t + e + 8 * j, q + R * RHO::apply(g + 8 * h), q, 4 * j + 2 * h + e, v);
        }
  }
}

// One warp computes 16 FFTs of length 16R (fft16r_job's algorithm and output
// slots), plain precision, with each lane's inputs read as 16-byte quads and the
// radix-R step folded like fft256r_jobs_fold: with PI = BitPerm<0, 2, 3, 1> the
// slots (kt, r) of lane t are the points m1 = 4t + r + 2kt, so LOAD4(v, a, w)
// fills w[0..3] with the half2 words of points 16a + 4t .. 16a + 4t + 3 of
// transform v (word r + 2kt is slot (kt, r)); the butterfly runs on the packed
// half2 inputs and the twiddle W_{16R}^(m1 q) is part of the per-q DFT matrix A_q
// (the A part of FoldTab<R>, built with this PI and RHO).  STORE(v, k, q, slot,
// float2) as in fft16r_job.
template <int R, class PI, class RHO, class Load4F, class StoreF>
__device__ __forceinline__ void fft16r_job_q_fold(const JobConsts<false>& c, uint32_t tab, float dsign,
                                                  Load4F&& load4, StoreF&& store) {
  static_assert(PI::apply(1) == 1 && PI::apply(2) == 4 && PI::apply(4) == 8 && PI::apply(8) == 2,
                "quad loads need PI = BitPerm<0, 2, 3, 1>");
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t lane4 = (uint32_t)lane * 4;
  const uint32_t negmask = dsign > 0.f ? 0x80000000u : 0x00008000u;
  const uint32_t c8 = pack_h2(0.70710678118654752440f, 0.70710678118654752440f);
  uint32_t bhi[R][2][2][2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    uint32_t w[R][4];
#pragma unroll
    for (int a = 0; a < R; ++a) load4(g + 8 * j, a, w[a]);
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        uint32_t x[R];
#pragma unroll
        for (int a = 0; a < R; ++a) x[a] = w[a][r + 2 * kt];
        if constexpr (R > 1) dft_small_h<R>(x, negmask, c8);
#pragma unroll
        for (int q = 0; q < R; ++q) bhi[q][kt][r][j] = x[q];
      }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    uint32_t aq[2][2][4];
    if (q == 0) {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = c.afr[i >> 3][(i >> 2) & 1][i & 3];
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = lds32(tab + ((q - 1) * 16 + i) * 128 + lane4);
    }
    float acc[2][2][4];
    dft16_mma(aq, bhi[q], acc);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int e = 0; e < 2; ++e) store(2 * t + e + 8 * j, q + R * RHO::apply(g + 8 * h), q, 4 * j + 2 * h + e,
                                          acc_get(acc, j, h, e));
  }
}

// The same with one element per load: LOAD(v, n) -> packed half2 point n of
// transform v (fft16r_job's slot layout, any PI).
template <int R, class PI, class RHO, class LoadF, class StoreF>
__device__ __forceinline__ void fft16r_job_fold(const JobConsts<false>& c, uint32_t tab, float dsign, LoadF&& load,
                                                StoreF&& store) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t lane4 = (uint32_t)lane * 4;
  const uint32_t negmask = dsign > 0.f ? 0x80000000u : 0x00008000u;
  const uint32_t c8 = pack_h2(0.70710678118654752440f, 0.70710678118654752440f);
  uint32_t bhi[R][2][2][2];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int m1 = PI::apply(2 * t + r + 8 * kt), v = g + 8 * j;
        uint32_t x[R];
#pragma unroll
        for (int a = 0; a < R; ++a) x[a] = load(v, m1 + 16 * a);
        if constexpr (R > 1) dft_small_h<R>(x, negmask, c8);
#pragma unroll
        for (int q = 0; q < R; ++q) bhi[q][kt][r][j] = x[q];
      }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    uint32_t aq[2][2][4];
    if (q == 0) {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = c.afr[i >> 3][(i >> 2) & 1][i & 3];
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) aq[i >> 3][(i >> 2) & 1][i & 3] = lds32(tab + ((q - 1) * 16 + i) * 128 + lane4);
    }
    float acc[2][2][4];
    dft16_mma(aq, bhi[q], acc);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int e = 0; e < 2; ++e) store(2 * t + e + 8 * j, q + R * RHO::apply(g + 8 * h), q, 4 * j + 2 * h + e,
                                          acc_get(acc, j, h, e));
  }
}

}  // namespace tcfft
