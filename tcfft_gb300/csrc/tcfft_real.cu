// tcfft_real.cu -- real-to-complex and complex-to-real 1D transforms of N
// points through a complex transform of N/2 points (no counterpart in the
// reference, whose plan API is complex-to-complex only, tcfft_half.h:20).
//
// A real sequence x[0..N-1] stored as N values is, byte for byte, the complex
// sequence z[m] = x[2m] + i x[2m+1] of h = N/2 points.  With Z = DFT_h(z), the
// DFTs of the even and odd samples are
//   E[k] = (Z[k] + conj(Z[h-k])) / 2,   O[k] = (Z[k] - conj(Z[h-k])) / (2i),
// and the spectrum of x is X[k] = E[k] + W_N^k O[k], X[h-k] = conj(E[k] - W_N^k O[k])
// (W_N = exp(-2 pi i / N)), for k = 0..h/2; indices are mod h.  The R2C pass
// below turns Z into X[0..h] (h + 1 values, the Hermitian half).  The C2R pass
// inverts it: Z'[k] = (E2 + i O2), E2 = X[k] + conj(X[h-k]), O2 = (X[k] -
// conj(X[h-k])) W_N^-k, whose unnormalised inverse DFT of h points is N x; the
// imaginary parts of X[0] and X[h] are taken as zero (they are for a real x).
// Both passes read each input element once and write each output once: one
// thread per pair (k, h - k), coalesced from both ends; W_N^k from the plan's
// two-level table (hi[k >> s] * lo[k & (2^s - 1)], fp32 from long double).
#include "fft_common.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

template <bool SPLIT>
struct Elem {
  using T = typename std::conditional<SPLIT, float2, uint32_t>::type;
  static __device__ __forceinline__ float2 get(const T* p, long long i) {
    if constexpr (SPLIT) return p[i];
    else return unpack_h2(p[i]);
  }
  static __device__ __forceinline__ void put(T* p, long long i, float2 v) {
    if constexpr (SPLIT) p[i] = v;
    else p[i] = pack_h2(v.x, v.y);
  }
};

__device__ __forceinline__ float2 twiddle(const float2* __restrict__ lo, const float2* __restrict__ hi, int shift,
                                          long long k) {
  return cmul(__ldg(hi + (k >> shift)), __ldg(lo + (k & ((1ll << shift) - 1))));
}

// Z [batch][h] -> X [batch][h + 1]; tables of W_N^j (forward sign).
template <bool SPLIT>
__global__ void __launch_bounds__(256) r2c_post_kernel(const void* __restrict__ zin, void* __restrict__ xout,
                                                       long long batch, long long h, const float2* __restrict__ lo,
                                                       const float2* __restrict__ hi, int shift, float scale) {
  using E = Elem<SPLIT>;
  const typename E::T* Z = static_cast<const typename E::T*>(zin);
  typename E::T* X = static_cast<typename E::T*>(xout);
  const long long per = h / 2 + 1, total = batch * per;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / per, k = i - b * per;
    const float2 a = E::get(Z, b * h + k % h);
    const float2 c = E::get(Z, b * h + (h - k) % h);  // B = conj(c)
    const float2 ev = make_float2(0.5f * (a.x + c.x), 0.5f * (a.y - c.y));
    const float2 od = make_float2(0.5f * (a.y + c.y), -0.5f * (a.x - c.x));
    const float2 wo = cmul(twiddle(lo, hi, shift, k), od);
    E::put(X, b * (h + 1) + k, make_float2(scale * (ev.x + wo.x), scale * (ev.y + wo.y)));
    if (k != h - k) E::put(X, b * (h + 1) + (h - k), make_float2(scale * (ev.x - wo.x), -scale * (ev.y - wo.y)));
  }
}

// X [batch][h + 1] -> Z' [batch][h]; tables of W_N^-j (conjugate sign).
template <bool SPLIT>
__global__ void __launch_bounds__(256) c2r_pre_kernel(const void* __restrict__ xin, void* __restrict__ zout,
                                                      long long batch, long long h, const float2* __restrict__ lo,
                                                      const float2* __restrict__ hi, int shift, float scale) {
  using E = Elem<SPLIT>;
  const typename E::T* X = static_cast<const typename E::T*>(xin);
  typename E::T* Z = static_cast<typename E::T*>(zout);
  const long long per = h / 2 + 1, total = batch * per;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / per, k = i - b * per;
    float2 a = E::get(X, b * (h + 1) + k);
    float2 c = E::get(X, b * (h + 1) + (h - k));  // B = conj(c)
    if (k == 0) {  // X[0] and X[h] of a real sequence are real
      a.y = 0.f;
      c.y = 0.f;
    }
    const float2 e2 = make_float2(a.x + c.x, a.y - c.y);
    const float2 o2 = cmul(make_float2(a.x - c.x, a.y + c.y), twiddle(lo, hi, shift, k));
    // Z'[k] = e2 + i o2;  Z'[h - k] = conj(e2) + i conj(o2)
    if (k < h) E::put(Z, b * h + k, make_float2(scale * (e2.x - o2.y), scale * (e2.y + o2.x)));
    if (k != 0 && k != h - k) E::put(Z, b * h + (h - k), make_float2(scale * (e2.x + o2.y), scale * (o2.x - e2.y)));
  }
}

long long grid_for(long long work, int num_sms) {
  long long g = (work + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  return g < 1 ? 1 : (g > cap ? cap : g);
}

}  // namespace

cudaError_t launch_r2c_post(const void* z, void* x, int64_t batch, int64_t h, const float2* lo, const float2* hi,
                            int shift, float scale, bool split, int num_sms, cudaStream_t st) {
  const long long g = grid_for(batch * (h / 2 + 1), num_sms);
  if (split) r2c_post_kernel<true><<<(unsigned)g, 256, 0, st>>>(z, x, batch, h, lo, hi, shift, scale);
  else r2c_post_kernel<false><<<(unsigned)g, 256, 0, st>>>(z, x, batch, h, lo, hi, shift, scale);
  return cudaGetLastError();
}

cudaError_t launch_c2r_pre(const void* x, void* z, int64_t batch, int64_t h, const float2* lo, const float2* hi,
                           int shift, float scale, bool split, int num_sms, cudaStream_t st) {
  const long long g = grid_for(batch * (h / 2 + 1), num_sms);
  if (split) c2r_pre_kernel<true><<<(unsigned)g, 256, 0, st>>>(x, z, batch, h, lo, hi, shift, scale);
  else c2r_pre_kernel<false><<<(unsigned)g, 256, 0, st>>>(x, z, batch, h, lo, hi, shift, scale);
  return cudaGetLastError();
}

}  // namespace tcfft
