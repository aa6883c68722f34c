// fft_cluster.cu -- 1D FFTs of N = 256 x 64 CL (CL = 2, 4, 8, 16: N = 2^15 .. 2^18)
// by a thread-block cluster of CL CTAs sharing the transform through
// distributed shared memory.
//
// The reference computes these sizes (2^17..2^19 in its table,
// tcfft_half.cu:1280-1305) with two launches and an HBM round trip between
// them; the two-phase kernel of this library keeps the intermediate in L2.
// Here the intermediate never leaves the SMs:
//
//   CTA r of the cluster holds columns [64 r, 64 r + 64) of the transform's
//   [256 rows n1][N2 cols n2] view (two 32-column tiles, 64 KiB, loaded with
//   the digit-ordered 5D boxes of the column role);
//   phase 0: 256-point column FFTs in place, times W_N^(n2 k1);
//   cluster barrier (remote mbarrier arrivals, release/acquire at cluster scope);
//   phase 1: CTA r transforms rows k1 in [r 256/CL, (r+1) 256/CL) of length N2,
//            reading each row's elements from the CTA that holds them
//            (ld.shared::cluster); results stay in registers;
//   cluster barrier (every CTA has read every slice);
//   output: X[k1 + 256 k2] of its rows written into its own stage and stored
//            with 2D TMA boxes (rows k2 of 256/CL contiguous k1).
// One HBM read and one write per element, no scratch, no global counters.
#include <mutex>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {
namespace {

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t nclusters_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// shared::cta address -> the same offset in CTA `rank`'s shared memory (shared::cluster window)
__device__ __forceinline__ uint32_t mapa(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ uint32_t ld_cluster(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ bool try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool wait_cluster(uint64_t* bar, uint32_t parity, int* err) {
  if (try_wait_cluster(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!try_wait_cluster(bar, parity)) {
    if (global_ns() - t0 > kTimeoutNs) {
      if (err) atomicExch(err, kDevTimeout);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int CL>
struct ClCfg {
  static constexpr int kN2 = 64 * CL;
  static constexpr int kN = 256 * kN2;
  static constexpr int kRPC = 256 / CL;                  // phase-1 rows per CTA
  static constexpr int kR1 = CL == 2 ? 8 : CL / 4;      // row FFT: 16*8 (CL=2) or 256*R1
  static constexpr int kW = kRPC < 32 ? kRPC : 32;       // output box width (elements)
  static constexpr int kChunks = kRPC / kW;
  static constexpr int kBH = kN2 < 256 ? kN2 : 256;      // output box height (rows k2)
  static constexpr int kTileBytes = 256 * 32 * 4;        // one 32-column tile
  static constexpr int kStageBytes = 65536;
  static constexpr int kStages = 3;
  static constexpr int kLog2N = 14 + (CL == 2 ? 1 : CL == 4 ? 2 : CL == 8 ? 3 : 4);
  static constexpr int kTwShift = (kLog2N + 1) / 2;
  static constexpr int kTwLo = 1 << kTwShift, kTwHi = kN >> kTwShift;
  static constexpr int kFold1 = (CL >= 4) ? FoldTab<kR1>::kBytes : 0;
  static constexpr int kTabBytes = (kTwLo + kTwHi + 128) * 8 + FoldTab<1>::kBytes + kFold1;
  static constexpr int kBars = 5 * kStages;
  static constexpr int kSmem = kStages * kStageBytes + kTabBytes + 1024 + kBars * 8 + 64;
  using PI = BitPerm<0, 1, 3, 2>;
  // row phase: lane digit t in bits 0-1 of m1, so that one load instruction (fixed r, kt, j, a)
  // reads a single 64-column slice, i.e. a single peer CTA
  using PI1 = BitPerm<2, 0, 1, 3>;
  using RHO = BitPerm<0, 2, 3, 1>;
  static_assert(kRPC * kN2 * 4 == kStageBytes, "a CTA's output slice is one stage");
};

struct ClParams {
  const float2* tw2048;
  const float2* twlo;
  const float2* twhi;
  long long batch;
  int* err;
  float dsign;
  float oscale = 1.f;  // output scale (a power of two), carried by the phase-0 W_N factors
};

template <int CL>
__device__ __forceinline__ void compute_warps(unsigned char* smem, uint64_t* full, uint64_t* computed, uint64_t* p0,
                                              uint64_t* p1, unsigned char* s_fold0, unsigned char* s_fold1,
                                              float2* s_tw128, float2* s_twlo, float2* s_twhi, const ClParams& p,
                                              uint32_t rank, long long first, long long step);

template <int CL>
__global__ void __launch_bounds__(384, 1) fft_cluster_kernel(const __grid_constant__ CUtensorMap load_map,
                                                              const __grid_constant__ CUtensorMap store_map,
                                                              const ClParams p) {
  using Cfg = ClCfg<CL>;
  using PI = typename Cfg::PI;
  using RHO = typename Cfg::RHO;
  constexpr int NST = Cfg::kStages, N2 = Cfg::kN2, RPC = Cfg::kRPC, R1 = Cfg::kR1, W = Cfg::kW;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // the dynamic shared window starts at the same offset in every CTA of the cluster, so
  // aligning it the same way keeps local and remote offsets equal
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* tab = smem + NST * Cfg::kStageBytes;
  float2* s_twlo = reinterpret_cast<float2*>(tab);
  float2* s_twhi = s_twlo + Cfg::kTwLo;
  float2* s_tw128 = s_twhi + Cfg::kTwHi;  // W_128^j (CL = 2 rows)
  unsigned char* s_fold0 = reinterpret_cast<unsigned char*>(s_tw128 + 128);
  unsigned char* s_fold1 = Cfg::kFold1 ? s_fold0 + FoldTab<1>::kBytes : s_fold0;
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + Cfg::kTabBytes);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;
  uint64_t* p0 = empty + NST;  // column phase done, all CTAs (8 CL arrivals)
  uint64_t* p1 = p0 + NST;     // row phase has read every slice (8 CL arrivals)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = cluster_rank();
  const long long first = cluster_id_x(), step = nclusters_x();
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
      mbar_init(&p0[s], 8 * CL);
      mbar_init(&p1[s], 8 * CL);
    }
    fence_barrier_init();
  }
  for (int j = tid; j < Cfg::kTwLo; j += blockDim.x) s_twlo[j] = p.twlo[j];
  for (int j = tid; j < Cfg::kTwHi; j += blockDim.x) s_twhi[j] = p.twhi[j];
  for (int j = tid; j < 128; j += blockDim.x) s_tw128[j] = p.tw2048[j * 16];
  build_fold_table<1, PI, RHO>(s_fold0, p.tw2048, tid, blockDim.x);
  if constexpr (Cfg::kFold1 > 0) build_fold_table<R1, typename Cfg::PI1, RHO>(s_fold1, p.tw2048, tid, blockDim.x);
  __syncthreads();
  cluster_sync_all();  // every CTA's barriers are initialised before any remote arrival

  if (warp >= 8) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(56));
  // every warp, the auxiliary ones included, ends at the closing cluster barrier
  if (warp >= 10) {
    // idle
  } else if (warp == 8) {  // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tmap(&load_map);
      int cnt = 0;
      for (long long it = first; it < p.batch; it += step, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&empty[s], ((cnt / NST) + 1) & 1, p.err)) break;
        unsigned char* dst = smem + s * Cfg::kStageBytes;
        mbar_arrive_expect_tx(&full[s], Cfg::kStageBytes);
        tma_load_5d(dst, &load_map, (int)(64 * rank), 0, 0, 0, (int)it, &full[s]);
        tma_load_5d(dst + Cfg::kTileBytes, &load_map, (int)(64 * rank + 32), 0, 0, 0, (int)it, &full[s]);
      }
      for (int i = (cnt > NST ? cnt - NST : 0); i < cnt; ++i) mbar_wait(&full[i % NST], (i / NST) & 1, nullptr);
    }
    __syncwarp();
  } else if (warp == 9) {  // ------------------------------------------------ TMA storer
    if (lane == 0) {
      prefetch_tmap(&store_map);
      int cnt = 0;
      for (long long it = first; it < p.batch; it += step, ++cnt) {
        const int s = cnt % NST;
        if (!mbar_wait(&computed[s], (cnt / NST) & 1, p.err)) break;
        const unsigned char* src = smem + s * Cfg::kStageBytes;
#pragma unroll 1
        for (int c = 0; c < Cfg::kChunks; ++c)
#pragma unroll 1
          for (int h = 0; h < N2 / Cfg::kBH; ++h)
            tma_store_2d(&store_map, (int)(rank * RPC + c * W), (int)(it * N2 + h * Cfg::kBH),
                         src + (c * N2 + h * Cfg::kBH) * W * 4);
        bulk_commit();
        bulk_wait_read<0>();
        mbar_arrive(&empty[s]);
      }
      bulk_wait<0>();
    }
    __syncwarp();
  } else {
    compute_warps<CL>(smem, full, computed, p0, p1, s_fold0, s_fold1, s_tw128, s_twlo, s_twhi, p, rank, first, step);
  }
  cluster_sync_all();  // no CTA leaves while another may still read its shared memory
}

template <int CL>
__device__ __forceinline__ void compute_warps(unsigned char* smem, uint64_t* full, uint64_t* computed, uint64_t* p0,
                                              uint64_t* p1, unsigned char* s_fold0, unsigned char* s_fold1,
                                              float2* s_tw128, float2* s_twlo, float2* s_twhi, const ClParams& p,
                                              uint32_t rank, long long first, long long step) {
  using Cfg = ClCfg<CL>;
  using PI = typename Cfg::PI;
  using RHO = typename Cfg::RHO;
  constexpr int NST = Cfg::kStages, N2 = Cfg::kN2, RPC = Cfg::kRPC, R1 = Cfg::kR1, W = Cfg::kW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(224));
  using PI1 = typename Cfg::PI1;
  JobConsts<false> jc, jc1;
  init_job_consts<false, PI, RHO>(jc, p.tw2048);
  if constexpr (CL >= 4) init_job_consts<false, PI1, RHO>(jc1, p.tw2048);
  const uint32_t fold0 = smem_addr(s_fold0), fold1 = smem_addr(s_fold1), tw128 = smem_addr(s_tw128);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = false;
  wn.shift = Cfg::kTwShift;
  wn.nmask = Cfg::kN - 1;
  uint32_t remote_p0[CL], remote_p1[CL];
  const int g = lane >> 2, tq = lane & 3;
  int cnt = 0;
  for (long long it = first; it < p.batch; it += step, ++cnt) {
    const int s = cnt % NST;
    const uint32_t par = (cnt / NST) & 1;
    bool ok = named_bar_and(2, 256, mbar_wait(&full[s], par, p.err));
    const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes);
    if (ok) {
#pragma unroll
      for (int q = 0; q < CL; ++q) {
        remote_p0[q] = mapa(smem_addr(&p0[s]), q);
        remote_p1[q] = mapa(smem_addr(&p1[s]), q);
      }
      // phase 0: the two 32-column tiles of this CTA's slice
#pragma unroll 1
      for (int t = 0; t < 2; ++t)
        plain_col_tile<1, 32, true, PI, RHO>(jc, fold0, base + t * Cfg::kTileBytes, warp, p.dsign,
                                             (int)(64 * rank + 32 * t), wn, p.oscale);
      __syncwarp();
      if (lane == 0)
        for (int q = 0; q < CL; ++q) arrive_remote(remote_p0[q]);
      ok = named_bar_and(2, 256, wait_cluster(&p0[s], par, p.err));
    }
    constexpr int OUTN = 64;  // output values held per lane
    uint32_t out[OUTN];
    if (ok) {
      // phase 1: rows k1 = rank RPC + ...; element (k1, n2) lives in CTA n2 / 64
      auto elem = [&](int k1, int n2) {
        const uint32_t local = base + (uint32_t)(((n2 & 63) >> 5) * Cfg::kTileBytes) +
                               ctile_off<32, 4>(col_out_row(k1, 0), n2 & 31);
        return ld_cluster(mapa(local, (uint32_t)(n2 >> 6)));
      };
      if constexpr (CL == 2) {
        // 128 rows per CTA: one job of 16 rows (length 128 = 16 x 8) per warp
        const int k1base = (int)rank * RPC + 16 * warp;
        auto ld = [&](int v, int n) { return unpack_h2(elem(k1base + v, n)); };
        auto st = [&](int, int, int q, int slot, float2 val) { out[8 * q + slot] = pack_h2(val.x, val.y); };
        fft16r_job<8, false, 1, PI, RHO>(jc, tw128, p.dsign, ld, st);
      } else {
        // RPC / 8 rows per warp, two at a time, length 256 R1
        constexpr int RPW = RPC / 8;
#pragma unroll
        for (int pr = 0; pr < RPW; pr += 2) {
          const int k1 = (int)rank * RPC + RPW * warp + pr;
          int mrow[8];
#pragma unroll
          for (int sl = 0; sl < 8; ++sl) mrow[sl] = slot_m<PI1, RHO>(sl);
          auto ld = [&](int jn, int sl, int a) { return elem(k1 + jn, mrow[sl] + 256 * a); };
          auto st = [&](int jn, int osl, int q, float2 v) { out[(pr + jn) * 8 * R1 + 8 * q + osl] = pack_h2(v.x, v.y); };
          fft256r_jobs_fold<R1, 2, false>(jc1, fold1, p.dsign, ld, st);
        }
      }
      __syncwarp();
      if (lane == 0)
        for (int q = 0; q < CL; ++q) arrive_remote(remote_p1[q]);
      ok = named_bar_and(2, 256, wait_cluster(&p1[s], par, p.err));
    }
    if (ok) {
      // output rows k2 of this CTA's RPC consecutive k1, chunks of W columns
      auto put = [&](int k1l, int k2, uint32_t v) {
        const int c = k1l / W, j = k1l % W;
        sts32(base + (uint32_t)(c * N2 * W * 4) + ctile_off<W, 4>(k2, j), v);
      };
      if constexpr (CL == 2) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int slot = 0; slot < 8; ++slot) {
            const int jj = slot >> 2, h = (slot >> 1) & 1, e = slot & 1;
            put(16 * warp + 2 * tq + e + 8 * jj, q + 8 * RHO::apply(g + 8 * h), out[8 * q + slot]);
          }
      } else {
        constexpr int RPW = RPC / 8;
#pragma unroll
        for (int r = 0; r < RPW; ++r)
#pragma unroll
          for (int q = 0; q < R1; ++q)
#pragma unroll
            for (int osl = 0; osl < 8; ++osl)
              put(RPW * warp + r, q + R1 * slot_kval<PI, RHO>(osl), out[r * 8 * R1 + 8 * q + osl]);
      }
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&computed[s]);
    if (!ok) break;
  }
}

template <int CL>
cudaError_t launch_cluster_t(const CUtensorMap& lm, const CUtensorMap& sm, const ClParams& p, int num_sms,
                             cudaStream_t st, int* max_clusters) {
  using Cfg = ClCfg<CL>;
  auto kern = fft_cluster_kernel<CL>;
  static std::once_flag once;
  static cudaError_t init_err = cudaSuccess;
  static int active = 0;
  std::call_once(once, [&] {
    init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem);
    if (init_err == cudaSuccess && CL > 8)
      init_err = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (init_err != cudaSuccess) return;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(CL * (num_sms / CL));
    cfg.blockDim = dim3(384);
    cfg.dynamicSmemBytes = Cfg::kSmem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    init_err = cudaOccupancyMaxActiveClusters(&active, kern, &cfg);
  });
  if (max_clusters) *max_clusters = active;
  if (init_err != cudaSuccess) return init_err;
  if (active < 1) return cudaErrorNotSupported;
  if (!p.twlo) return cudaSuccess;  // capability query only
  long long clusters = active;
  if (clusters > p.batch) clusters = p.batch;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(CL * clusters));
  cfg.blockDim = dim3(384);
  cfg.dynamicSmemBytes = Cfg::kSmem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, lm, sm, p);
}

cudaError_t dispatch_cluster(int64_t n, const CUtensorMap& lm, const CUtensorMap& sm, const ClParams& p,
                             int num_sms, cudaStream_t st, int* max_clusters) {
  switch (n) {
    case 1 << 15: return launch_cluster_t<2>(lm, sm, p, num_sms, st, max_clusters);
    case 1 << 16: return launch_cluster_t<4>(lm, sm, p, num_sms, st, max_clusters);
    case 1 << 17: return launch_cluster_t<8>(lm, sm, p, num_sms, st, max_clusters);
    case 1 << 18: return launch_cluster_t<16>(lm, sm, p, num_sms, st, max_clusters);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// Whether this GPU can run the cluster kernel for n (plain): it needs CL co-resident CTAs of
// ~215 KiB shared memory each in one GPU processing cluster.
bool cluster_supported(int64_t n, bool split, int num_sms) {
  if (split || n < (1 << 15) || n > (1 << 18)) return false;
  CUtensorMap dummy;
  memset(&dummy, 0, sizeof dummy);
  ClParams p = {};
  int active = 0;
  return dispatch_cluster(n, dummy, dummy, p, num_sms, nullptr, &active) == cudaSuccess && active > 0;
}

cudaError_t launch_cluster(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                           const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st, CUtensorMap* lm,
                           CUtensorMap* sm, bool encode, float oscale, const void* in) {
  const int64_t n2 = n / 256;
  const int cl = (int)(n2 / 64), rpc = 256 / cl, w = rpc < 32 ? rpc : 32;
  const int bh = n2 < 256 ? (int)n2 : 256;
  if (encode) {
    void* src = const_cast<void*>(in ? in : data);  // loads from the input, stores to data
    if (encode_col_load(lm, CU_TENSOR_MAP_DATA_TYPE_UINT32, src, n2, batch, 4, 32, 1) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    uint64_t dims[2] = {256, (uint64_t)(n2 * batch)};  // X[b][k1 + 256 k2] as rows k2 of 256 k1
    uint64_t str[1] = {1024};
    uint32_t box[2] = {(uint32_t)w, (uint32_t)bh};
    const CUtensorMapSwizzle sw = w * 4 == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    if (encode_tmap(sm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, data, dims, str, box, sw) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  ClParams p;
  p.tw2048 = tw2048;
  p.twlo = twlo;
  p.twhi = twhi;
  p.batch = batch;
  p.err = err;
  p.dsign = dsign;
  p.oscale = oscale;
  int active = 0;
  return dispatch_cluster(n, *lm, *sm, p, num_sms, st, &active);
}

}  // namespace tcfft
