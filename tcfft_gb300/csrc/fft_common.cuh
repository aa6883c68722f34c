// fft_common.cuh -- device building blocks shared by every tcfft_gb300 kernel.
//
// Data model.  A complex element is either a packed half2 (PLAIN mode: low 16
// bits = real, high 16 bits = imaginary, i.e. the interleaved `half` layout of
// tcfft_half.h:20 `tcfftExec(tcfftHandle, half*)`) or a float2 (SPLIT mode).
// Shared-memory tiles are always written/read by TMA with the 128-byte swizzle,
// so a tile is a stack of 128-byte rows and the 16-byte chunk c of row r sits
// at chunk position c ^ (r & 7).  `swz_w` maps a logical element index inside
// a 1024-byte-aligned tile to its physical element index.
//
// Radix-16 on the tensor cores.  A 16-point DFT applied to 16 vectors is the
// complex product Y = F * X with F[k][m] = W16^(k*m).  Interleaving real and
// imaginary parts turns it into a real 32x32 by 32x16 product that maps onto
// two m16 x two k16 x two n8 `mma.sync.m16n8k16` tiles (8 MMAs), with fp16
// operands and fp32 accumulation.  The fragment slots are chosen so that the
// accumulator of one stage, packed to half2, is already the B operand of the
// next stage (two radix-16 stages per register pass, no shared-memory round
// trip in between).  The index permutations PI (operand slots) and RHO (output
// rows) are bit permutations picked so that every shared-memory access of a
// warp is bank-conflict free on the swizzled tile.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace tcfft {

// ---------------------------------------------------------------- constants
constexpr unsigned long long kTimeoutNs = 2000000000ull;  // every device-side wait gives up after 2 s
// Precision modes of the kernels: fp16 data and arithmetic; fp32 data with
// hi/lo split products; fp32 data with fp16 operands (one product per stage).
enum KernelMode : int { kModePlain = 0, kModeSplit = 1, kModeIo32 = 2 };
enum DeviceError : int { kDevOk = 0, kDevTimeout = 1 };

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// 4-bit index permutation: bit i of x moves to bit P_i.
template <int P0, int P1, int P2, int P3>
struct BitPerm {
  __host__ __device__ static constexpr int apply(int x) {
    return (((x >> 0) & 1) << P0) | (((x >> 1) & 1) << P1) | (((x >> 2) & 1) << P2) | (((x >> 3) & 1) << P3);
  }
};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Physical index of logical element e inside a 128B-swizzled, 1024B-aligned tile.
template <int ELEM_BYTES>
__device__ __forceinline__ uint32_t swz_w(uint32_t e) {
  if constexpr (ELEM_BYTES == 4) {
    return e ^ (((e >> 5) & 7u) << 2);  // 32 elements per 128-byte row, 4 per chunk
  } else {
    return e ^ (((e >> 4) & 7u) << 1);  // 16 elements per row, 2 per chunk
  }
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (wall clock, `limit_ns`, by default kTimeoutNs); on expiry
// records kDevTimeout in *err and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          unsigned long long limit_ns = kTimeoutNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) {
      if (err) atomicExch(err, kDevTimeout);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// 2D tiled TMA load (global -> shared), completion counted on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}
// 2D/3D tiled TMA store (shared -> global), tracked by the bulk async-group.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map), "r"(x),
               "r"(y), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void tma_store_4d(const CUtensorMap* map, int c0, int c1, int c2, int c3, const void* src) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(map),
               "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void tma_store_5d(const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                             const void* src) {
  asm volatile(
      "cp.async.bulk.tensor.5d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4, %5}], [%6];" ::"l"(map),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(src))
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N>
__device__ __forceinline__ void bulk_wait() {
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// ---------------------------------------------------------------- shared memory I/O
__device__ __forceinline__ uint32_t lds32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void sts32(uint32_t addr, uint32_t v) {
  asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void lds64(uint32_t addr, uint32_t& a, uint32_t& b) {
  asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(a), "=r"(b) : "r"(addr) : "memory");
}
__device__ __forceinline__ void lds128(uint32_t addr, uint32_t (&w)[4]) {
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]) : "r"(addr)
               : "memory");
}
__device__ __forceinline__ void lds128f(uint32_t addr, float2& a, float2& b) {
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(a.x), "=f"(a.y), "=f"(b.x), "=f"(b.y) : "r"(addr)
               : "memory");
}
__device__ __forceinline__ float2 lds64f(uint32_t addr) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void sts64f(uint32_t addr, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void sts64(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void sts128f(uint32_t addr, float2 a, float2 b) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y) : "memory");
}

// ---------------------------------------------------------------- complex helpers
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by -i (forward, dsign=+1) or +i (adjoint, dsign=-1)
__device__ __forceinline__ float2 cmul_mi(float2 a, float dsign) { return make_float2(dsign * a.y, -dsign * a.x); }

__device__ __forceinline__ uint32_t pack_h2(float re, float im) {
  __half2 h = __floats2half2_rn(re, im);
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float2 unpack_h2(uint32_t v) {
  __half2 h = *reinterpret_cast<__half2*>(&v);
  return __half22float2(h);
}
// hi/lo fp16 split of an fp32 complex value: x ~= hi + lo to ~22 bits.
__device__ __forceinline__ void split_h2(float2 x, uint32_t& hi, uint32_t& lo) {
  hi = pack_h2(x.x, x.y);
  float2 h = unpack_h2(hi);
  lo = pack_h2(x.x - h.x, x.y - h.y);
}

// Split precision keeps each stage's operands inside fp16's range with a
// per-job power-of-two scale: the job's inputs are scaled so that their largest
// component lies in [512, 1024), which leaves room for the x16 growth of one
// radix-16 stage before the next hi/lo split (16384 < 65504); the fp32 results
// are scaled back exactly.
__device__ __forceinline__ float warp_max(float m) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  return m;
}
// scale and inverse scale (powers of two) for a job whose max |component| is m
__device__ __forceinline__ void split_scale(float m, float& scale, float& inv) {
  int e = (int)((__float_as_uint(m) >> 23) & 0xff) - 127;  // floor(log2 m) for normal m
  if (m == 0.f || e < -100) e = 9;
  if (e > 100) e = 100;
  scale = __uint_as_float((uint32_t)(127 + 9 - e) << 23);
  inv = __uint_as_float((uint32_t)(127 - 9 + e) << 23);
}

// D += A(16x16 fp16, row) * B(16x8 fp16, col), fp32 accumulate.
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------- radix-16 MMA stage
// Thread (g = lane/4, t = lane%4) fragment conventions used everywhere:
//  * B operand slot (kt, r, j): K-slot kappa = 8*kt + 4*r + t carries the input
//    digit value PI(2t + r + 8kt); N column g + 8j carries vector PI(g + 8j)
//    (first stage) -- later stages inherit the vector order of the previous
//    stage's output rows.
//  * accumulator (ct, j, 2h + e): ct = real/imag m-tile, n-tile j, row g + 8h
//    (output digit RHO(g + 8h)), column 2t + e (vector at N position
//    2t + e + 8j).
// A = real-ified F with rows RHO and K columns PI(2t + r + 8kt):
//   real rows: [Re F, -Im F], imag rows: [Im F, Re F] (interleaved re/im in K).
// `w16` points at W16^0 of a twiddle table whose entry j*w16_stride is W16^j.
template <class PI, class RHO>
__device__ __forceinline__ void build_dft_frags(const float2* __restrict__ w16, int w16_stride, uint32_t (&a)[2][2][4],
                                                uint32_t (&alo)[2][2][4], bool want_lo) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int ct = 0; ct < 2; ++ct)
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int reg = 0; reg < 4; ++reg) {
        const int row = g + 8 * (reg & 1);   // a0,a2: row g; a1,a3: row g+8
        const int r = reg >> 1;              // a0,a1: cols 2t..; a2,a3: cols 2t+8.. (kappa + 4)
        const int k = RHO::apply(row);
        const int m = PI::apply(2 * t + r + 8 * kt);
        const float2 w = w16[((k * m) & 15) * w16_stride];
        // ct=0 (real output): (Re, -Im); ct=1 (imag output): (Im, Re)
        const float lo_part = ct == 0 ? w.x : w.y;
        const float hi_part = ct == 0 ? -w.y : w.x;
        a[ct][kt][reg] = pack_h2(lo_part, hi_part);
        if (want_lo) {
          const float2 h = unpack_h2(a[ct][kt][reg]);
          alo[ct][kt][reg] = pack_h2(lo_part - h.x, hi_part - h.y);
        }
      }
}

// One radix-16 stage on a 16x16 complex tile held as B fragments.
// b[kt][r][j] are packed half2 operands; acc[ct][j][4] receives fp32 results.
__device__ __forceinline__ void dft16_mma(const uint32_t (&a)[2][2][4], const uint32_t (&b)[2][2][2],
                                          float (&acc)[2][2][4]) {
#pragma unroll
  for (int ct = 0; ct < 2; ++ct)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      acc[ct][j][0] = acc[ct][j][1] = acc[ct][j][2] = acc[ct][j][3] = 0.f;
#pragma unroll
      for (int kt = 0; kt < 2; ++kt) mma16816(acc[ct][j], a[ct][kt], b[kt][0][j], b[kt][1][j]);
    }
}
// Split-precision stage: acc = Ahi*Bhi + Ahi*Blo + Alo*Bhi (fp32 accumulate).
__device__ __forceinline__ void dft16_mma_split(const uint32_t (&a)[2][2][4], const uint32_t (&alo)[2][2][4],
                                                const uint32_t (&b)[2][2][2], const uint32_t (&blo)[2][2][2],
                                                float (&acc)[2][2][4]) {
#pragma unroll
  for (int ct = 0; ct < 2; ++ct)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      acc[ct][j][0] = acc[ct][j][1] = acc[ct][j][2] = acc[ct][j][3] = 0.f;
#pragma unroll
      for (int kt = 0; kt < 2; ++kt) {
        mma16816(acc[ct][j], alo[ct][kt], b[kt][0][j], b[kt][1][j]);
        mma16816(acc[ct][j], a[ct][kt], blo[kt][0][j], blo[kt][1][j]);
        mma16816(acc[ct][j], a[ct][kt], b[kt][0][j], b[kt][1][j]);
      }
    }
}

// Accumulator entry (ct re/im pair) for n-tile j, row-half h, column e.
__device__ __forceinline__ float2 acc_get(const float (&acc)[2][2][4], int j, int h, int e) {
  return make_float2(acc[0][j][2 * h + e], acc[1][j][2 * h + e]);
}

// ---------------------------------------------------------------- packed half2 complex arithmetic
// A complex value as one 32-bit register: real part in the low half, imaginary
// part in the high half (the layout of the interleaved half2 data).
__device__ __forceinline__ uint32_t h2add(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("add.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t h2sub(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t h2mul(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
// v * (-i * dsign): swap the halves, then negate one of them; negmask =
// 0x80000000 for dsign = +1 ((re, im) -> (im, -re)), 0x00008000 for dsign = -1.
__device__ __forceinline__ uint32_t h2mi(uint32_t v, uint32_t negmask) { return __byte_perm(v, 0, 0x1032) ^ negmask; }

// In-place radix-R DFT on packed half2 values (same convention as dft_small).
// c8 = cos(pi/4) broadcast to both halves (used by R = 8).
template <int R>
__device__ __forceinline__ void dft_small_h(uint32_t (&x)[R], uint32_t negmask, uint32_t c8) {
  if constexpr (R == 2) {
    const uint32_t a = x[0], b = x[1];
    x[0] = h2add(a, b);
    x[1] = h2sub(a, b);
  } else if constexpr (R == 4) {
    const uint32_t a0 = h2add(x[0], x[2]), a1 = h2sub(x[0], x[2]);
    const uint32_t b0 = h2add(x[1], x[3]), b1 = h2mi(h2sub(x[1], x[3]), negmask);
    x[0] = h2add(a0, b0);
    x[2] = h2sub(a0, b0);
    x[1] = h2add(a1, b1);
    x[3] = h2sub(a1, b1);
  } else if constexpr (R == 8) {
    uint32_t u[4], v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      u[a] = h2add(x[a], x[a + 4]);
      v[a] = h2sub(x[a], x[a + 4]);
    }
    // v[a] *= W8^a: W8 = c (1 - i dsign) -> c (v + mi(v)); W8^2 = -i dsign; W8^3 = c (mi(v) - v)
    v[1] = h2mul(h2add(v[1], h2mi(v[1], negmask)), c8);
    v[2] = h2mi(v[2], negmask);
    v[3] = h2mul(h2sub(h2mi(v[3], negmask), v[3]), c8);
    dft_small_h<4>(u, negmask, c8);
    dft_small_h<4>(v, negmask, c8);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      x[2 * q] = u[q];
      x[2 * q + 1] = v[q];
    }
  }
}

// ---------------------------------------------------------------- small radix-R DFT (fp32)
// In-place DFT of R values, x_q <- sum_a x_a W_R^(a q) (W_R = exp(-2 pi i dsign / R)).
template <int R>
__device__ __forceinline__ void dft_small(float2 (&x)[R], float dsign) {
  if constexpr (R == 2) {
    const float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (R == 4) {
    const float2 a0 = cadd(x[0], x[2]), a1 = csub(x[0], x[2]);
    const float2 b0 = cadd(x[1], x[3]), b1 = cmul_mi(csub(x[1], x[3]), dsign);
    x[0] = cadd(a0, b0);
    x[2] = csub(a0, b0);
    x[1] = cadd(a1, b1);
    x[3] = csub(a1, b1);
  } else if constexpr (R == 8) {
    // radix-2 over the top bit, twiddle W8^(a*q), then two radix-4s
    constexpr float c = 0.70710678118654752440f;
    float2 u[4], v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      u[a] = cadd(x[a], x[a + 4]);
      v[a] = csub(x[a], x[a + 4]);
    }
    // v[a] *= W8^a : W8 = (c, -c*dsign)
    v[1] = make_float2(c * (v[1].x + dsign * v[1].y), c * (v[1].y - dsign * v[1].x));
    v[2] = cmul_mi(v[2], dsign);
    v[3] = make_float2(c * (-v[3].x + dsign * v[3].y), c * (-v[3].y - dsign * v[3].x));
    dft_small<4>(u, dsign);
    dft_small<4>(v, dsign);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      x[2 * q] = u[q];
      x[2 * q + 1] = v[q];
    }
  }
}

}  // namespace tcfft
