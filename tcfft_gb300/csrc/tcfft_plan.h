// tcfft_plan.h -- the opaque plan object behind `tcfftPlan`.
#pragma once
#include <string>
#include <vector>

#include "fft_fused.cuh"
#include "tcfft_host.h"

namespace tcfft {

// Execution schedule chosen at plan time (host-only, no CUDA calls).
struct Schedule {
  // kTiny: N = 16..128, one launch (fft_tiny.cu).
  // kLarge1d: N = N1 N2 with N2 > 2048: column pass (fused kernel, phase 0 only) into a
  //   full-size scratch, row FFTs of length N2 by a sub-plan, transpose back.
  // kGeneric2d: axes outside the fused 2D range: row FFTs (sub-plan), transpose, row FFTs of
  //   the other axis (sub-plan), transpose back.
  enum Kind {
    kNone = 0, kSmall = 1, kFused1d = 2, kFused2d = 3, kTiny = 4, kLarge1d = 5, kGeneric2d = 6,
    kResident = 8,  // N = 4096..16384 plain: whole transforms in one CTA's shared memory (fft_resident.cu)
    kCluster = 9    // N = 2^15..2^18 plain: one transform per thread-block cluster (fft_cluster.cu)
  } kind = kNone;
  int R = 1;             // small: N = 256 R
  int64_t N1 = 0, N2 = 0;  // fused 1D: N = N1 N2 (phase 0 columns of N1, phase 1 rows of N2)
  FusedKey key;          // fused: kernel instantiation
  int T0 = 0, T1 = 0, D = 0, S = 0;
  int launches = 0;      // kernel launches per execute
  std::string text;      // human-readable description
};

}  // namespace tcfft

struct tcfftPlanImpl {
  static constexpr uint32_t kMagic = 0x7cff7600u;
  uint32_t magic = kMagic;
  int kind = 0;  // 1: 1D, 2: 2D, 3: many, 4: real 1D (R2C / C2R through subs[0], a complex plan of n / 2),
                 // 5: real 2D (subs[0] the real row plan, subs[1] the complex column plan)
  int64_t n = 0, nx = 0, ny = 0, batch = 0;
  int precision = 0, input_order = 0;
  int direction = 0, normalize = 0;  // of tcfftExecute (tcfftOptions)
  int device = -1, num_sms = 0;
  int64_t total_elems = 0;
  int64_t span_elems = 0;  // elements from the buffer start to the end of the last transform
  tcfft::Schedule sched;
  tcfft::DeviceTables tables;
  // fused executor resources
  float2* twlo[2] = {nullptr, nullptr};
  float2* twhi[2] = {nullptr, nullptr};
  int tw_shift = 0;
  int* counters = nullptr;  // [2 * S]
  void* scratch = nullptr;
  int64_t scratch_bytes = 0;
  // composite schedules (kLarge1d, kGeneric2d): full-size intermediate and sub-plans
  void* big = nullptr;
  std::vector<tcfftPlanImpl*> subs;
  // tcfftPlanMany: runs of same-shape, back-to-back transforms, each executed by a
  // sub-plan shared by every run of that shape and length (owned in `subs`); the
  // sequence is captured once per (data pointer, direction) into a CUDA graph on a
  // private stream and replayed with one graph launch.
  struct Run {
    tcfftPlanImpl* sub;
    int64_t offset;  // elements, in the caller's buffer or (in_big) in `big`
    bool in_big;
  };
  std::vector<Run> runs;
  // same-shape transforms that are not back to back are gathered into `big`
  // (one launch), transformed as one batch and scattered back (one launch):
  // per moved transform its byte offset in the caller's buffer and in `big`,
  // and the 16-byte chunks before it (device tables)
  long long* mv_user = nullptr;
  long long* mv_big = nullptr;
  long long* mv_cum = nullptr;
  int mv_n = 0;
  long long mv_chunks = 0;
  cudaStream_t cap_stream = nullptr;
  // independent runs are captured on branch streams (forked after the gather, joined
  // before the scatter), so the graph runs them concurrently
  static constexpr int kBranches = 8;
  cudaStream_t branch[kBranches] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kBranches] = {};
  void* graph_ptr[4] = {};  // per (direction, normalisation)
  cudaGraphExec_t graph_exec[4] = {};
  // tcfftPlanMany, plain precision, every shape supported: the two-pass many-shape
  // executor (fft_many.cu) in place of the graph.  Per transform its element offset,
  // shape and scratch offset (1D N >= 4096); device item lists of both passes, the
  // row list, the transforms' tensor maps (re-encoded when the data pointer changes,
  // through a pinned staging copy).
  struct ManyXf {
    int rank;
    int64_t nx, ny, off, soff;
  };
  bool many_ok = false;
  bool many_only = false;                  // no per-shape graph (strided column plans)
  int many_xf_b = -1;                      // first transform with a pass B (timeout test hook)
  std::vector<ManyXf> many_xf;
  tcfft::ManyItem* many_items = nullptr;  // the item sequence of the one launch
  int many_n[2] = {0, 0};                 // [0]: items
  int* many_rows = nullptr;
  int* many_claim = nullptr;               // per transform its completed pass-A items, then the claim counter
  CUtensorMap* many_maps = nullptr;
  CUtensorMap* many_hmaps = nullptr;      // pinned
  void* many_maps_ptr = nullptr;
  void* many_scratch = nullptr;
  unsigned char* many_fold8 = nullptr;     // R = 8 fold tables of both directions
  float2* many_wn3 = nullptr;              // W_65536 in three levels, both directions
  // tcfftExecuteHost: sub-plans for the chunk batches (created on first use), copy-in,
  // compute and copy-out streams, per-chunk events
  static constexpr int kHostChunks = 32;  // most chunks (events); 16 used unless TCFFT_HOST_CHUNKS says otherwise
  tcfftPlanImpl* host_sub[2] = {nullptr, nullptr};  // chunk batches b0 and b0 + 1
  int64_t host_b0 = 0;
  cudaStream_t host_st[3] = {};
  cudaEvent_t host_ev_in[kHostChunks] = {}, host_ev_fft[kHostChunks] = {};
  cudaEvent_t host_fork = nullptr, host_join[2] = {};
  // autotuner: chosen lag multiplier of the fused executor (1 = built-in)
  double lag_scale = 1.0;
  // limit of the two-phase kernels' bounded waits (0: the default, 2 s) and the
  // one-shot stall injection of tcfftInjectWaitTimeout
  unsigned long long wait_ns = 0;
  bool inject_timeout = false;
  // reference input order (TCFFT_ORDER_REFERENCE_DIGIT_REVERSED)
  std::vector<int> radices_x, radices_y;  // reported chains (x = the 1D chain)
  int* rev_x = nullptr;                   // device digit-reversal tables (nullptr: natural)
  int* rev_y = nullptr;
  void* perm_tmp = nullptr;               // natural-order staging buffer
  // tensor maps encoded for the last data pointer
  void* tmap_ptr = nullptr;        // output buffer the maps were encoded for
  const void* tmap_in = nullptr;   // input buffer (== tmap_ptr in place)
  CUtensorMap tmap0, tmap1;        // single-pass schedule: loads, stores
  tcfft::FusedMaps fmaps;
};
