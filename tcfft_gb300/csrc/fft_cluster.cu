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
//   exchange: CTA r pushes to every CTA q of the cluster, itself included, the rows
//            k1 in [q RPC, (q+1) RPC) of its two tiles (RPC = 256 / CL).  In the
//            column role's row order those rows are 4 runs of 64 / CL consecutive
//            tile rows per tile, so the exchange is 8 CL bulk shared::cluster copies
//            per CTA, each completing on the receiver's mbarrier for that sender.
//            The receive buffer keeps the bytes as they were (the swizzle phase of
//            each row is that of its original row), so the row phase reads them
//            with the bank pattern of a local tile;
//   phase 1: CTA r transforms its RPC rows k1 of length N2 from its receive buffer
//            (local shared-memory loads only); results stay in registers;
//   output: X[k1 + 256 k2] of its rows written into its own stage and stored
//            with 2D TMA boxes (rows k2 of 256/CL contiguous k1).
// One HBM read and one write per element, no scratch, no global counters.
//
// Per transform c (every CTA of a cluster runs the same sequence of transforms),
// three kinds of mbarrier, every wait on them bounded:
//   recv[y]  (one per sender y, this CTA included: 1 arrival, this CTA arming it at
//            the start of c, plus the 64 KiB / CL bytes of y's pieces): y's pieces of
//            c have landed;
//   pfree    (8 (CL - 1) arrivals, every compute warp of every peer after its row
//            phase of c): the peers' receive buffers may take the pieces of c + 1;
//   sent     (CL - 1 arrivals, each peer once it has all its pieces of c): this
//            CTA's stage may be overwritten by the output of c (its own pieces have
//            landed before its row phase).  The pieces of c + 1 into its own receive
//            buffer follow its row phase of c in program order.
// At exit every CTA passes a cluster barrier (no piece is pushed after it), waits
// until the pieces its peers pushed to it (their counts, read remotely) have
// landed, and passes a second barrier, so no CTA leaves while a copy into it is
// in flight.
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
// bulk copy of `bytes` (a multiple of 16) from this CTA's shared memory to a peer's,
// completing `bytes` transactions on the peer's mbarrier `bar` (shared::cluster addresses)
__device__ __forceinline__ void bulk_push(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "r"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int CL>
struct ClCfg {
  static constexpr int kLgCL = CL == 2 ? 1 : CL == 4 ? 2 : CL == 8 ? 3 : 4;
  static constexpr int kN2 = 64 * CL;
  static constexpr int kN = 256 * kN2;
  static constexpr int kRPC = 256 / CL;                  // phase-1 rows per CTA
  static constexpr int kR1 = CL == 2 ? 8 : CL / 4;      // row FFT: 16*8 (CL=2) or 256*R1
  static constexpr int kW = kRPC < 32 ? kRPC : 32;       // output box width (elements)
  static constexpr int kChunks = kRPC / kW;
  static constexpr int kBH = kN2 < 256 ? kN2 : 256;      // output box height (rows k2)
  static constexpr int kTileBytes = 256 * 32 * 4;        // one 32-column tile
  static constexpr int kStageBytes = 65536;
  static constexpr int kStages = 2;
  // receive buffer: per sender q and tile t a block of the RPC tile rows of this CTA's k1
  // range (4 pieces of kPieceRows consecutive rows), at (2 q + t) kBlockBytes
  static constexpr int kRecvBytes = 65536;
  static constexpr int kPieceRows = 64 / CL;
  static constexpr int kPieceBytes = kPieceRows * 128;
  static constexpr int kBlockBytes = kRPC * 128;
  static constexpr int kPieces = 8 * CL;                          // pushed per transform
  static constexpr uint32_t kSenderTx = 8u * kPieceBytes;         // bytes from one sender
  static constexpr int kLog2N = 14 + kLgCL;
  static constexpr int kTwShift = (kLog2N + 1) / 2;
  static constexpr int kTwLo = 1 << kTwShift, kTwHi = kN >> kTwShift;
  static constexpr int kFold1 = (CL >= 4) ? FoldTab<kR1>::kBytes : 0;
  static constexpr int kTabBytes = (kTwLo + kTwHi + 128) * 8 + FoldTab<1>::kBytes + kFold1;
  static constexpr int kBars = 3 * kStages + CL + 2;
  static constexpr int kCtl = 2 + CL;  // ints: transforms pushed, transforms armed, received per sender
  static constexpr int kSmem = kStages * kStageBytes + kRecvBytes + kTabBytes + 1024 + kBars * 8 + kCtl * 4 + 64;
  using PI = BitPerm<0, 1, 3, 2>;
  // row phase: lane digit t in bits 0-1 of m1, so that one load instruction (fixed r, kt, j, a)
  // reads a single 64-column slice, i.e. a single sender's block
  using PI1 = BitPerm<2, 0, 1, 3>;
  using RHO = BitPerm<0, 2, 3, 1>;
  static_assert(kRPC * kN2 * 4 == kStageBytes, "a CTA's output slice is one stage");
  static_assert(2 * CL * kBlockBytes == kRecvBytes && 4 * kPieceBytes == kBlockBytes, "receive buffer layout");
  static_assert(kPieceBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
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
__device__ __forceinline__ void compute_warps(unsigned char* smem, uint64_t* full, uint64_t* computed, uint64_t* recv,
                                              uint64_t* pfree, uint64_t* sent, int* ctl, unsigned char* s_fold0,
                                              unsigned char* s_fold1, float2* s_tw128, float2* s_twlo,
                                              float2* s_twhi, const ClParams& p, uint32_t rank, long long first,
                                              long long step);

// Exit: wait until every piece a peer pushed to this CTA has landed (the peers' push counts are
// read after a cluster barrier, so no further piece follows).  One thread.
template <int CL>
__device__ __forceinline__ void drain_pieces(uint64_t* recv, int* ctl, uint32_t rank, int* err) {
  using Cfg = ClCfg<CL>;
  for (int y = 0; y < CL; ++y) {
    const int pushed = (int)ld_cluster(mapa(smem_addr(&ctl[0]), (uint32_t)y));
    for (int c = ctl[2 + y]; c < pushed; ++c) {
      if (c >= ctl[1]) mbar_arrive_expect_tx(&recv[y], Cfg::kSenderTx);  // a phase not armed yet
      if (!mbar_wait(&recv[y], (uint32_t)c & 1, err)) break;
    }
  }
}

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
  unsigned char* tab = smem + NST * Cfg::kStageBytes + Cfg::kRecvBytes;
  float2* s_twlo = reinterpret_cast<float2*>(tab);
  float2* s_twhi = s_twlo + Cfg::kTwLo;
  float2* s_tw128 = s_twhi + Cfg::kTwHi;  // W_128^j (CL = 2 rows)
  unsigned char* s_fold0 = reinterpret_cast<unsigned char*>(s_tw128 + 128);
  unsigned char* s_fold1 = Cfg::kFold1 ? s_fold0 + FoldTab<1>::kBytes : s_fold0;
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + Cfg::kTabBytes);
  uint64_t* computed = full + NST;
  uint64_t* empty = computed + NST;
  uint64_t* recv = empty + NST;  // [CL] by sender rank
  uint64_t* pfree = recv + CL;
  uint64_t* sent = pfree + 1;
  int* ctl = reinterpret_cast<int*>(sent + 1);  // [0] transforms pushed, [1] armed, [2 + y] received from y

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = cluster_rank();
  const long long first = cluster_id_x(), step = nclusters_x();
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&computed[s], 8);
      mbar_init(&empty[s], 1);
    }
    for (int y = 0; y < CL; ++y) mbar_init(&recv[y], 1);
    mbar_init(pfree, 8 * (CL - 1));
    mbar_init(sent, CL - 1);
    for (int i = 0; i < Cfg::kCtl; ++i) ctl[i] = 0;
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
  // every warp, the auxiliary ones included, ends at the closing cluster barriers
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
    compute_warps<CL>(smem, full, computed, recv, pfree, sent, ctl, s_fold0, s_fold1, s_tw128, s_twlo, s_twhi, p,
                      rank, first, step);
  }
  __syncwarp();
  cluster_sync_all();  // no piece is pushed after this barrier
  if (tid == 0) drain_pieces<CL>(recv, ctl, rank, p.err);
  __syncwarp();
  cluster_sync_all();  // no CTA leaves while a piece may land in it or a peer reads its count
}

template <int CL>
__device__ __forceinline__ void compute_warps(unsigned char* smem, uint64_t* full, uint64_t* computed, uint64_t* recv,
                                              uint64_t* pfree, uint64_t* sent, int* ctl, unsigned char* s_fold0,
                                              unsigned char* s_fold1, float2* s_tw128, float2* s_twlo,
                                              float2* s_twhi, const ClParams& p, uint32_t rank, long long first,
                                              long long step) {
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
  const uint32_t rbuf = smem_addr(smem + NST * Cfg::kStageBytes);
  WnTable wn;
  wn.hi = smem_addr(s_twhi);
  wn.lo = smem_addr(s_twlo);
  wn.ghi = p.twhi;
  wn.glo = p.twlo;
  wn.global = false;
  wn.shift = Cfg::kTwShift;
  wn.nmask = Cfg::kN - 1;
  const int g = lane >> 2, tq = lane & 3;
  const bool leader = warp == 0 && lane == 0;
  int cnt = 0;
  for (long long it = first; it < p.batch; it += step, ++cnt) {
    const int s = cnt % NST;
    const uint32_t par = (cnt / NST) & 1, tpar = (uint32_t)cnt & 1;
    const uint32_t base = smem_addr(smem + s * Cfg::kStageBytes);
    if (leader) {  // arm the receive barriers of this transform (pieces may already be landing)
      for (int y = 0; y < CL; ++y) mbar_arrive_expect_tx(&recv[y], Cfg::kSenderTx);
      ctl[1] = cnt + 1;
    }
    bool ok = named_bar_and(2, 256, mbar_wait(&full[s], par, p.err));
    if (ok) {
      // phase 0: the two 32-column tiles of this CTA's slice
#pragma unroll 1
      for (int t = 0; t < 2; ++t)
        plain_col_tile<1, 32, true, PI, RHO>(jc, fold0, base + t * Cfg::kTileBytes, warp, p.dsign,
                                             (int)(64 * rank + 32 * t), wn, p.oscale);
      fence_proxy_async_smem();  // the pieces are read by bulk copies
    }
    ok = named_bar_and(2, 256, ok);
    if (warp == 0) {
      // push: once every peer's receive buffer is free (their row phase of the previous
      // transform is done), piece i = (receiver q, tile t, run hi) goes to q's block (rank, t)
      bool go = ok;
      if (lane == 0 && go) go = wait_cluster(pfree, (uint32_t)(cnt + 1) & 1, p.err);
      go = __shfl_sync(0xffffffffu, go, 0);
      if (go) {
        for (int i = lane; i < Cfg::kPieces; i += 32) {
          const int t = (i >> 2) & 1, hi = i & 3;
          const uint32_t q = (uint32_t)(i >> 3);
          const uint32_t src =
              base + (uint32_t)(t * Cfg::kTileBytes + ((hi << 6) | ((int)q << (6 - Cfg::kLgCL))) * 128);
          const uint32_t dst =
              mapa(rbuf + (uint32_t)((2 * (int)rank + t) * Cfg::kBlockBytes + hi * Cfg::kPieceBytes), q);
          bulk_push(dst, src, (uint32_t)Cfg::kPieceBytes, mapa(smem_addr(&recv[rank]), q));
        }
      }
      __syncwarp();
      if (lane == 0 && go) ctl[0] = cnt + 1;
      ok = go;
    }
    // every sender's pieces of this transform
    bool got = ok;
#pragma unroll 1
    for (int y = 0; y < CL; ++y)
      if (got) {
        got = mbar_wait(&recv[y], tpar, p.err);
        if (got && leader) ctl[2 + y] = cnt + 1;
      }
    ok = named_bar_and(2, 256, got);
    if (ok && leader)
      for (int y = 0; y < CL; ++y)
        if (y != (int)rank) arrive_remote(mapa(smem_addr(sent), (uint32_t)y));
    constexpr int OUTN = 64;  // output values held per lane
    uint32_t out[OUTN];
    if (ok) {
      // phase 1: rows k1 = rank RPC + ...; element (k1, n2) was computed by CTA n2 / 64 and sits in
      // that sender's block of the receive buffer, at its tile row's rank among the rows of this
      // k1 range, with the swizzle of the original row
      auto elem = [&](int k1, int n2) {
        const int q = n2 >> 6, t = (n2 >> 5) & 1;
        const int row = col_out_row(k1, 0);
        const uint32_t off = ctile_off<32, 4>(row, n2 & 31);
        const int crow = (row & (Cfg::kPieceRows - 1)) | ((row >> 6) * Cfg::kPieceRows);
        return lds32(rbuf + (uint32_t)((2 * q + t) * Cfg::kBlockBytes + crow * 128) + (off & 127u));
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
      if (lane == 0)  // this warp has read its part of the receive buffer
        for (int y = 0; y < CL; ++y)
          if (y != (int)rank) arrive_remote(mapa(smem_addr(pfree), (uint32_t)y));
    }
    // the stage is overwritten only once every peer holds its pieces of this transform
    ok = named_bar_and(2, 256, ok && wait_cluster(sent, tpar, p.err));
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
// ~215 KiB shared memory each in one GPU processing cluster.  *active_clusters: how many such
// clusters the device holds at once.
bool cluster_supported(int64_t n, bool split, int num_sms, int* active_clusters) {
  if (split || n < (1 << 15) || n > (1 << 18)) return false;
  CUtensorMap dummy;
  memset(&dummy, 0, sizeof dummy);
  ClParams p = {};
  int active = 0;
  const bool ok = dispatch_cluster(n, dummy, dummy, p, num_sms, nullptr, &active) == cudaSuccess && active > 0;
  if (active_clusters) *active_clusters = active;
  return ok;
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
