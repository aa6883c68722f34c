// tcfft_api.cu -- C-ABI implementation: planner, device tables, execute.
//
// Plan creation replaces the reference's tcfftCreate (tcfft_half.cu:1235-1345,
// tcfft_half_2d.cu:1151-1221): instead of a hard-coded size table it derives
// a schedule for every power-of-two size, validates its arguments, owns its
// device tables and can be destroyed.  tcfftExecute replaces tcfftExec
// (tcfft_half.cu:1177-1233): it launches the schedule on a caller-chosen
// stream and returns a status.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "tcfft_host.h"
#include <algorithm>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "tcfft_plan.h"

namespace tcfft {

// ------------------------------------------------------------------ driver entry
namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;
std::once_flag g_encode_once;
}  // namespace

CUresult encode_tmap(CUtensorMap* map, CUtensorMapDataType dtype, int rank, void* addr, const uint64_t* dims,
                     const uint64_t* strides_bytes, const uint32_t* box, CUtensorMapSwizzle swizzle) {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  });
  if (!g_encode) return CUDA_ERROR_NOT_FOUND;
  cuuint64_t d[5], st[4];
  cuuint32_t b[5], es[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    es[i] = 1;
    if (i + 1 < rank) st[i] = strides_bytes[i];
  }
  return g_encode(map, dtype, (cuuint32_t)rank, addr, d, st, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

// Column-tile maps (the digit orders of fft_fused.cuh's ctile_off/col_in_row/
// col_out_row; the swizzle of the tile's row width C*es).  The global data is
// rows of `ncols` elements; transforms are blocks of 256R consecutive rows.
CUtensorMapSwizzle col_swizzle(int C, int es) {
  return C * es == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                      : (C * es == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B);
}
// Load box [C][m1 bit 3][m0][m1 bits 0-2][a + R block]: input row n = m0 + 16 m1 + 256 a.
CUresult encode_col_load(CUtensorMap* m, CUtensorMapDataType dt, void* base, int64_t ncols, int64_t nblk, int es,
                         int C, int R) {
  const uint64_t rp = (uint64_t)ncols * es;
  if (es == 8) {
    // split precision (8-byte elements, identity slot permutation): box
    // [C][n bits 5-6][n bit 0][n bits 1-4][n bit 7 + 2 a]: tile row
    // (n bits 5-6 | n bit 0 << 2 | n bits 1-4 << 3 | (n >> 7) << 7), see col_in_row_t
    uint64_t dims[5] = {(uint64_t)ncols, 4, 2, 16, (uint64_t)(2 * nblk * R)};
    uint64_t str[4] = {32 * rp, rp, 2 * rp, 128 * rp};
    uint32_t box[5] = {(uint32_t)C, 4, 2, 16, (uint32_t)(2 * R)};
    return encode_tmap(m, dt, 5, base, dims, str, box, col_swizzle(C, es));
  }
  uint64_t dims[5] = {(uint64_t)ncols, 2, 16, 8, (uint64_t)(nblk * R)};
  uint64_t str[4] = {128 * rp, rp, 16 * rp, 256 * rp};
  uint32_t box[5] = {(uint32_t)C, 2, 16, 8, (uint32_t)R};
  return encode_tmap(m, dt, 5, base, dims, str, box, col_swizzle(C, es));
}
// Store box [C][k0 bits 2-3][k1 + 16 block][k0 bits 0-1][q]: output row k = q + R (k0 + 16 k1).
CUresult encode_col_store(CUtensorMap* m, CUtensorMapDataType dt, void* base, int64_t ncols, int64_t nblk, int es,
                          int C, int R) {
  const uint64_t rp = (uint64_t)ncols * es;
  uint64_t dims[5] = {(uint64_t)ncols, 4, (uint64_t)(16 * nblk), 4, (uint64_t)R};
  uint64_t str[4] = {4 * R * rp, 16 * R * rp, R * rp, rp};
  uint32_t box[5] = {(uint32_t)C, 4, 16, 4, (uint32_t)R};
  return encode_tmap(m, dt, 5, base, dims, str, box, col_swizzle(C, es));
}

// Tensor maps of the 1D fused executor (the plan path and the allocation-free
// entry point share them): phase 0 reads `data` as column tiles and writes the
// scratch slots [S][N1 rows][N2 cols]; phase 1 reads scratch rows and writes
// `data` transposed (X[k1 + N1 k2]).
CUresult encode_fused1d_maps(FusedMaps* maps, const FusedKey& k, void* data, void* scratch, int64_t n1, int64_t n2,
                             int64_t batch, int S, const void* in) {
  const int es = k.split ? 8 : 4, er = 128 / es;
  const CUtensorMapDataType dt = k.split ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  CUresult r = encode_col_load(&maps->load0, dt, const_cast<void*>(in ? in : data), n2, batch, es, k.C0, k.R0);
  if (r != CUDA_SUCCESS) return r;
  r = encode_col_store(&maps->store0, dt, scratch, n2, S, es, k.C0, k.R0);
  if (r != CUDA_SUCCESS) return r;
  {  // phase-1 load: scratch as contiguous 128-byte rows, boxes of one tile (<= 256 rows)
    const int64_t tile_rows = (int64_t)k.C1 * n2 / er;
    uint64_t dims[2] = {(uint64_t)er, (uint64_t)(S * n1 * n2 / er)};
    uint64_t str[1] = {128};
    uint32_t box[2] = {(uint32_t)er, (uint32_t)(tile_rows < 256 ? tile_rows : 256)};
    r = encode_tmap(&maps->load1, dt, 2, scratch, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
    if (r != CUDA_SUCCESS) return r;
  }
  if (k.role1 == kRoleRow16T) {  // phase-1 store: X[k1 + N1 k2], k2 = q + R1 k0: dims [N1][k0][q][B]
    const uint64_t rowb = (uint64_t)n1 * es;
    uint64_t dims[4] = {(uint64_t)n1, 16, (uint64_t)k.R1, (uint64_t)batch};
    uint64_t str[3] = {rowb * k.R1, rowb, rowb * n2};
    uint32_t box[4] = {(uint32_t)(128 / es), 16, (uint32_t)k.R1, 1};
    return encode_tmap(&maps->store1, dt, 4, data, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
  }
  // phase-1 store: data as [B*N2 rows k2][N1 cols k1]
  return encode_col_store(&maps->store1, dt, data, n1, batch, es, k.C1, k.R1);
}
}  // namespace tcfft

using namespace tcfft;

// ------------------------------------------------------------------ helpers
namespace {


bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

// With TCFFT_DEBUG set, failing CUDA calls are reported on stderr.
bool debug_on() {
  static const bool on = getenv("TCFFT_DEBUG") != nullptr;
  return on;
}
tcfftStatus cuda_status(cudaError_t e, const char* what = "launch") {
  if (e == cudaSuccess) return TCFFT_SUCCESS;
  if (debug_on()) fprintf(stderr, "tcfft: %s failed: %s\n", what, cudaGetErrorString(e));
  return TCFFT_CUDA_ERROR;
}
tcfftStatus cu_status(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return TCFFT_SUCCESS;
  if (debug_on()) fprintf(stderr, "tcfft: %s failed: CUresult %d\n", what, (int)r);
  return TCFFT_CUDA_ERROR;
}

// W_2048^j in fp32, computed in fp64 with exact octant reduction.
void host_twiddles(int n, int sign, std::vector<float2>& out) {
  out.resize(n);
  for (int j = 0; j < n; ++j) {
    const long double th = 2.0L * 3.141592653589793238462643383279502884L * (long double)j / (long double)n;
    const double c = (double)cosl(th), s = (double)sinl(th);
    out[j] = make_float2((float)c, (float)(sign < 0 ? -s : s));
  }
}

tcfftStatus alloc_tables(tcfftPlanImpl* p) {
  if (cudaGetDevice(&p->device) != cudaSuccess) return TCFFT_CUDA_ERROR;
  if (cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    return TCFFT_CUDA_ERROR;
  std::vector<float2> fw, bw;
  host_twiddles(2048, -1, fw);
  host_twiddles(2048, +1, bw);
  for (int d = 0; d < 2; ++d) {
    if (cudaMalloc(&p->tables.tw2048[d], 2048 * sizeof(float2)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (cudaMemcpy(p->tables.tw2048[d], d == 0 ? fw.data() : bw.data(), 2048 * sizeof(float2),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return TCFFT_CUDA_ERROR;
  }
  if (cudaMalloc(&p->tables.err, sizeof(int)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  if (cudaMemset(p->tables.err, 0, sizeof(int)) != cudaSuccess) return TCFFT_CUDA_ERROR;
  return TCFFT_SUCCESS;
}

void free_tables(tcfftPlanImpl* p) {
  for (int d = 0; d < 2; ++d)
    if (p->tables.tw2048[d]) cudaFree(p->tables.tw2048[d]);
  if (p->tables.err) cudaFree(p->tables.err);
  if (p->scratch) cudaFree(p->scratch);
  for (int d = 0; d < 2; ++d) {
    if (p->twlo[d]) cudaFree(p->twlo[d]);
    if (p->twhi[d]) cudaFree(p->twhi[d]);
    p->twlo[d] = p->twhi[d] = nullptr;
  }
  if (p->counters) cudaFree(p->counters);
  p->counters = nullptr;
  if (p->rev_x) cudaFree(p->rev_x);
  if (p->rev_y) cudaFree(p->rev_y);
  if (p->perm_tmp) cudaFree(p->perm_tmp);
  p->rev_x = p->rev_y = nullptr;
  p->perm_tmp = nullptr;
  p->tables = DeviceTables();
  p->scratch = nullptr;
  if (p->big) cudaFree(p->big);
  p->big = nullptr;
  for (tcfftPlanImpl* sp : p->subs) tcfftDestroy(sp);
  p->subs.clear();
  p->runs.clear();
  for (long long** q : {&p->mv_user, &p->mv_big, &p->mv_cum}) {
    if (*q) cudaFree(*q);
    *q = nullptr;
  }
  p->mv_n = 0;
  for (int d = 0; d < 4; ++d) {
    if (p->graph_exec[d]) cudaGraphExecDestroy(p->graph_exec[d]);
    p->graph_exec[d] = nullptr;
    p->graph_ptr[d] = nullptr;
  }
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  p->cap_stream = nullptr;
  if (p->many_items) cudaFree(p->many_items);
  if (p->many_rows) cudaFree(p->many_rows);
  if (p->many_claim) cudaFree(p->many_claim);
  p->many_claim = nullptr;
  if (p->many_fold8) cudaFree(p->many_fold8);
  p->many_fold8 = nullptr;
  if (p->many_wn3) cudaFree(p->many_wn3);
  p->many_wn3 = nullptr;
  if (p->many_maps) cudaFree(p->many_maps);
  if (p->many_hmaps) cudaFreeHost(p->many_hmaps);
  if (p->many_scratch) cudaFree(p->many_scratch);
  p->many_items = nullptr;
  p->many_rows = nullptr;
  p->many_maps = nullptr;
  p->many_hmaps = nullptr;
  p->many_scratch = nullptr;
  p->many_ok = false;
  for (int b = 0; b < tcfftPlanImpl::kBranches; ++b) {
    if (p->branch[b]) cudaStreamDestroy(p->branch[b]);
    if (p->join_ev[b]) cudaEventDestroy(p->join_ev[b]);
    p->branch[b] = nullptr;
    p->join_ev[b] = nullptr;
  }
  if (p->fork_ev) cudaEventDestroy(p->fork_ev);
  p->fork_ev = nullptr;
  for (int i = 0; i < 2; ++i) {
    if (p->host_sub[i]) tcfftDestroy(p->host_sub[i]);
    p->host_sub[i] = nullptr;
    if (p->host_join[i]) cudaEventDestroy(p->host_join[i]);
    p->host_join[i] = nullptr;
  }
  for (int i = 0; i < 3; ++i) {
    if (p->host_st[i]) cudaStreamDestroy(p->host_st[i]);
    p->host_st[i] = nullptr;
  }
  for (int c = 0; c < tcfftPlanImpl::kHostChunks; ++c) {
    if (p->host_ev_in[c]) cudaEventDestroy(p->host_ev_in[c]);
    if (p->host_ev_fft[c]) cudaEventDestroy(p->host_ev_fft[c]);
    p->host_ev_in[c] = p->host_ev_fft[c] = nullptr;
  }
  if (p->host_fork) cudaEventDestroy(p->host_fork);
  p->host_fork = nullptr;
}

// Name of a precision in schedule descriptions.
const char* prec_name(int precision) {
  return precision == TCFFT_PRECISION_SPLIT ? "split" : (precision == TCFFT_PRECISION_FP32_IO ? "fp32io" : "plain");
}

// SM count of the current device (152 on GB300 when it cannot be queried).
int current_num_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      n > 0)
    return n;
  cudaGetLastError();
  return 152;
}

int ilog2_exact(int64_t v) {
  int r = 0;
  while ((int64_t(1) << r) < v) ++r;
  return r;
}

// Lag (in blocks) between the two phases of the fused executor and the number
// of slots: enough tiles in flight across the GPU to cover, L2-sized ring.
// Tiles in flight span about (CTAs x stages) items; a transform's phase 1 is
// placed D blocks after its phase 0, and a slot is reused S blocks later, so
// both D and S - D must exceed the blocks in flight.
// Lag multiplier, 1D column length N1 and work-item size chosen by the autotuner
// while it times candidates (0: none).
thread_local double g_lag_override = 0.0;
thread_local int64_t g_n1_override = 0;
thread_local int g_item_kb_override = 0;

// Items of several tiles keep more tiles in flight per CTA: the lag grows with
// the tiles per item (x 1.25, measured at N = 2^16 and 2^17).  Rings deeper than
// four stages (32 KiB items) keep that many items in flight per CTA.
void fused_lag(int T0, int T1, int64_t batch, Schedule& s, const FusedKey* key, int num_sms) {
  static const double env_scale = getenv("TCFFT_LAG_SCALE") ? atof(getenv("TCFFT_LAG_SCALE")) : 1.0;
  double scale = g_lag_override > 0.0 ? g_lag_override : env_scale;
  int per_cta = 4;
  FusedShape sh;
  if (key && fused_shape(*key, &sh)) {
    if (sh.stages > per_cta) per_cta = sh.stages;
    if (sh.sub0 > 1 || sh.sub1 > 1) scale *= 1.25 * (double)(T0 * sh.sub0 + T1 * sh.sub1) / (double)(T0 + T1);
  }
  const int in_flight = (int)(num_sms * per_cta * scale);  // CTAs x tiles per CTA
  int D = (in_flight + (T0 + T1) - 1) / (T0 + T1) + 1;
  if (D > batch) D = (int)batch;
  if (D < 1) D = 1;
  s.D = D;
  s.S = 2 * D + 2;
}

// Work-item size of the 1D two-phase schedules (TCFFT_ITEM_KB overrides it, for measurements).
int item_kb_1d(int lg, bool split) {
  static const int env = getenv("TCFFT_ITEM_KB") ? atoi(getenv("TCFFT_ITEM_KB")) : 0;
  if (g_item_kb_override == 32 || g_item_kb_override == 64) return g_item_kb_override;
  if (env == 32 || env == 64) return env;
  // 2^16 plain (256 x 256): 32 KiB items with a deeper ring, 948 us per 2^28 elements against
  // 1032 us (the autotuner's choice); 64 KiB elsewhere (its choice from 2^17 to 2^22)
  return lg == 16 && !split ? 32 : 64;
}

// Host-only schedule selection for a 1D size (no CUDA calls).
tcfftStatus choose_1d(int64_t n, int64_t batch, int precision, Schedule& s, int num_sms = 152) {
  if (!is_pow2(n) || n < 16 || n > (int64_t(1) << 27)) return TCFFT_INVALID_SIZE;
  if (batch < 1 || batch > (int64_t(1) << 40) / n) return TCFFT_INVALID_SIZE;
  // split and fp32-I/O share the 8-byte-element schedules; they differ in arithmetic only
  const bool split = precision != TCFFT_PRECISION_PLAIN;
  const bool io32 = precision == TCFFT_PRECISION_FP32_IO;
  const char* pname = prec_name(precision);
  s = Schedule();
  char buf[160];
  if (n < 256) {
    if (!tiny_supported(n, precision)) return TCFFT_NOT_SUPPORTED;
    s.kind = Schedule::kTiny;
    s.R = (int)(n / 16);
    s.launches = 1;
    snprintf(buf, sizeof buf, "tiny(N=%lld,%s): 16 transforms per warp, 1 mma stage + radix-%d", (long long)n,
             pname, s.R);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  if (n <= 2048) {
    s.kind = Schedule::kSmall;
    s.R = (int)(n / 256);
    s.launches = 1;
    snprintf(buf, sizeof buf, "small(R=%d,%s): 1 pass, 2 mma stages + radix-%d", s.R, pname, s.R);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  const int lg = ilog2_exact(n);
  if (resident_supported(n, split) && !getenv("TCFFT_NO_RESIDENT")) {
    s.kind = Schedule::kResident;
    s.N1 = 256;
    s.N2 = n / 256;
    s.launches = 1;
    snprintf(buf, sizeof buf, "resident(%s): N=256 x %lld, whole transforms in shared memory, one HBM pass",
             pname, (long long)s.N2);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  if (lg >= 12 && lg <= 15) {
    // N = 256 x N2 with short rows N2 = 16 R1: phase 0 columns of 256, phase 1 16 rows per warp
    FusedKey k;
    // 2^15 (split, or plain with the resident kernel turned off): 512 x 64 (plain: 1.24 ms for
    // 2^28 elements against 1.48 ms for 256 x 128 and 1.38 ms for 1024 x 32: 64 KiB column tiles
    // and a radix-4 short-row phase; split: the short-row phase's R <= 4 limit)
    int64_t n1 = lg == 15 ? 512 : 256;
    if (getenv("TCFFT_N1")) n1 = atoll(getenv("TCFFT_N1"));  // decomposition override (measurements)
    if (n1 < 256 || n1 > 2048 || n / n1 < 16 || n / n1 > 128) return TCFFT_NOT_SUPPORTED;
    k.role0 = kRoleCol;
    k.R0 = (int)(n1 / 256);
    k.C0 = n1 == 512 ? (split ? 16 : 32) : 16;
    k.role1 = kRoleRow16T;
    k.R1 = (int)(n / n1 / 16);
    k.C1 = 128;
    k.split = split;
    k.io32 = io32;
    if (split && k.R1 > 4) return TCFFT_NOT_SUPPORTED;
    if (!fused_shape(k, nullptr)) return TCFFT_NOT_SUPPORTED;  // e.g. an override naming no compiled kernel
    s.kind = Schedule::kFused1d;
    s.N1 = n1;
    s.N2 = n / n1;
    s.key = k;
    s.T0 = (int)(s.N2 / k.C0 > 0 ? s.N2 / k.C0 : 1);
    s.T1 = (int)(s.N1 / k.C1);
    fused_lag(s.T0, s.T1, batch, s, &k, num_sms);
    s.launches = 1;
    snprintf(buf, sizeof buf, "fused1d(%s): N=%lld x %lld, phase0 columns R=%d C=%d, phase1 16-row groups R=%d, lag %d, %d slots",
             pname, (long long)s.N1, (long long)s.N2, k.R0, k.C0, k.R1, s.D, s.S);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  if (lg >= 16 && lg <= 22 && !(split && lg >= 21)) {
    // N1 >= N2 except 2^21: 1024 x 2048 (0.90 ms for 2^28 elements) against 2048 x 1024 (0.94 ms)
    int64_t n1 = int64_t(1) << ((lg + 1) / 2);
    if (lg == 21) n1 = 1024;
    if (getenv("TCFFT_N1")) n1 = atoll(getenv("TCFFT_N1"));  // decomposition override (measurements)
    if (g_n1_override) n1 = g_n1_override;                     // the autotuner's candidate
    if (n1 < 256 || n1 > 2048 || n / n1 < 256 || n / n1 > 2048) return TCFFT_NOT_SUPPORTED;
    const int64_t n2 = n / n1;
    FusedKey k;
    k.role0 = kRoleCol;
    k.R0 = (int)(n1 / 256);
    k.role1 = kRoleRowT;
    k.R1 = (int)(n2 / 256);
    k.split = split;
    k.io32 = io32;
    for (int ikb : {item_kb_1d(lg, split), 64}) {  // the preferred item size, else 64 KiB items
      k.item_kb = ikb;
      k.C0 = fused_cols(k.R0, split, ikb * 1024);
      k.C1 = fused_cols(k.R1, split, ikb * 1024);
      if (getenv("TCFFT_FUSED_C")) k.C0 = k.C1 = atoi(getenv("TCFFT_FUSED_C"));
      if (k.C0 != 0 && k.C1 != 0 && fused_shape(k, nullptr)) break;
    }
    if (k.C0 == 0 || k.C1 == 0) return TCFFT_NOT_SUPPORTED;
    s.kind = Schedule::kFused1d;
    s.N1 = n1;
    s.N2 = n2;
    s.key = k;
    s.T0 = (int)(n2 / k.C0);
    s.T1 = (int)(n1 / k.C1);
    fused_lag(s.T0, s.T1, batch, s, &k, num_sms);
    s.launches = 1;
    snprintf(buf, sizeof buf,
             "fused1d(%s): N=%lld x %lld, phase0 columns R=%d C=%d, phase1 rows R=%d C=%d, %d KiB items, lag %d, %d slots",
             pname, (long long)n1, (long long)n2, k.R0, k.C0, k.R1, k.C1, k.item_kb, s.D, s.S);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  if ((lg >= 23 || (split && lg >= 21)) && lg <= 27) {
    // N = N1 x N2, N1 = 2048 (split 1024; split 2^21: 512, so that the rows are 4096-point
    // resident transforms rather than a four-step of 2048): column FFTs of N1 with the W_N
    // twiddle into a full-size scratch (fused kernel, phase 0 only), N1 rows of N2 by a 1D
    // sub-plan, transpose back
    const int64_t n1 = split ? (lg == 21 ? 512 : 1024) : 2048, n2 = n / n1;
    if (batch > (1 << 30)) return TCFFT_INVALID_SIZE;
    FusedKey k;
    k.role0 = kRoleCol;
    k.R0 = (int)(n1 / 256);
    k.C0 = fused_cols(k.R0, split);
    k.role1 = kRoleRowT;
    k.R1 = k.R0;
    k.C1 = k.C0;
    k.split = split;
    k.io32 = io32;
    s.kind = Schedule::kLarge1d;
    s.N1 = n1;
    s.N2 = n2;
    s.key = k;
    s.T0 = (int)(n2 / k.C0);
    s.T1 = 0;
    s.D = 0;
    s.S = (int)batch;
    s.launches = 3;  // updated with the sub-plan's count at plan time
    snprintf(buf, sizeof buf, "large1d(%s): N=%lld x %lld, column pass R=%d C=%d -> rows of %lld (sub-plan) -> transpose",
             pname, (long long)n1, (long long)n2, k.R0, k.C0, (long long)n2);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  return TCFFT_NOT_SUPPORTED;
}

// Host-only schedule selection for a 2D size.
tcfftStatus choose_2d(int64_t nx, int64_t ny, int64_t batch, int precision, Schedule& s, int num_sms = 152) {
  if (!is_pow2(nx) || !is_pow2(ny) || nx < 256 || ny < 256 || nx > 2048 || ny > 2048) return TCFFT_INVALID_SIZE;
  if (batch < 1 || batch > (int64_t(1) << 40) / (nx * ny)) return TCFFT_INVALID_SIZE;
  const bool split = precision != TCFFT_PRECISION_PLAIN;  // 8-byte elements
  const char* pname = prec_name(precision);
  const int es = split ? 8 : 4;
  s = Schedule();
  FusedKey k;
  k.role0 = kRoleRow;
  k.R0 = (int)(ny / 256);
  k.C0 = fused_cols(k.R0, split);
  k.role1 = kRoleCol;
  k.R1 = (int)(nx / 256);
  k.C1 = fused_cols(k.R1, split);
  if (getenv("TCFFT_FUSED_C")) k.C0 = k.C1 = atoi(getenv("TCFFT_FUSED_C"));
  k.split = split;
  k.io32 = precision == TCFFT_PRECISION_FP32_IO;
  if (k.C1 == 0 || k.C0 * 256 * k.R0 * es > 64 * 1024 || (split && (k.R0 > 4 || k.R1 > 4))) return TCFFT_NOT_SUPPORTED;
  s.kind = Schedule::kFused2d;
  s.N1 = nx;
  s.N2 = ny;
  s.key = k;
  s.T0 = (int)(nx / k.C0);
  s.T1 = (int)(ny / k.C1);
  fused_lag(s.T0, s.T1, batch, s, &k, num_sms);
  s.launches = 1;
  char buf[160];
  snprintf(buf, sizeof buf, "fused2d(%s): %lld x %lld, phase0 rows R=%d C=%d, phase1 columns R=%d C=%d, lag %d",
           pname, (long long)nx, (long long)ny, k.R0, k.C0, k.R1, k.C1, s.D);
  s.text = buf;
  return TCFFT_SUCCESS;
}

// The 2D schedule: the fused 2D kernel where choose_2d takes the shape, otherwise rows of ny,
// transpose, rows of nx, transpose, from 1D plans (both axes must be valid 1D sizes).
tcfftStatus choose_2d_any(int64_t nx, int64_t ny, int64_t batch, int precision, Schedule& s, int num_sms = 152) {
  if (choose_2d(nx, ny, batch, precision, s, num_sms) == TCFFT_SUCCESS) return TCFFT_SUCCESS;
  Schedule sx, sy;
  if (!is_pow2(nx) || !is_pow2(ny) || batch < 1 || nx * ny > (int64_t(1) << 40) / batch) return TCFFT_INVALID_SIZE;
  tcfftStatus ex = choose_1d(nx, ny * batch, precision, sx), ey = choose_1d(ny, nx * batch, precision, sy);
  if (ex != TCFFT_SUCCESS) return ex;
  if (ey != TCFFT_SUCCESS) return ey;
  s = Schedule();
  s.kind = Schedule::kGeneric2d;
  s.N1 = nx;
  s.N2 = ny;
  char buf[160];
  snprintf(buf, sizeof buf, "generic2d(%s): rows of %lld, transpose, rows of %lld, transpose", prec_name(precision),
           (long long)ny, (long long)nx);
  s.text = buf;
  return TCFFT_SUCCESS;
}

// Device tables for the reference input order; chains must be supported by the reference.
tcfftStatus setup_reference_order(tcfftPlanImpl* p) {
  const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  auto upload = [&](const std::vector<int>& h, int** d) -> tcfftStatus {
    if (cudaMalloc(d, h.size() * sizeof(int)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (cudaMemcpy(*d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      return TCFFT_CUDA_ERROR;
    return TCFFT_SUCCESS;
  };
  tcfftStatus st;
  if (p->kind == 1) {
    if ((st = upload(digit_reversal(p->n, p->radices_x), &p->rev_y)) != TCFFT_SUCCESS) return st;
  } else {
    if ((st = upload(digit_reversal(p->nx, p->radices_x), &p->rev_x)) != TCFFT_SUCCESS) return st;
    if ((st = upload(digit_reversal(p->ny, p->radices_y), &p->rev_y)) != TCFFT_SUCCESS) return st;
  }
  if (cudaMalloc(&p->perm_tmp, p->total_elems * es) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  return TCFFT_SUCCESS;
}

tcfftStatus validate_opts(const tcfftOptions* o) {
  if (!o) return TCFFT_SUCCESS;
  if (o->precision != TCFFT_PRECISION_PLAIN && o->precision != TCFFT_PRECISION_SPLIT &&
      o->precision != TCFFT_PRECISION_FP32_IO)
    return TCFFT_INVALID_VALUE;
  if (o->input_order != TCFFT_ORDER_NATURAL && o->input_order != TCFFT_ORDER_REFERENCE_DIGIT_REVERSED)
    return TCFFT_INVALID_VALUE;
  if (o->direction != TCFFT_FORWARD && o->direction != TCFFT_INVERSE) return TCFFT_INVALID_VALUE;
  if (o->normalization != TCFFT_NORM_NONE && o->normalization != TCFFT_NORM_BY_N) return TCFFT_INVALID_VALUE;
  return TCFFT_SUCCESS;
}

tcfftStatus exec_many(tcfftPlanImpl* plan, void* data, cudaStream_t st, int dir, int norm);

// Composite schedules whose 4096-point row pass writes its output transposed
// (resident kernel, plain): 1D N1 x 4096 (no final transpose) and 2D axes of 4096.
// Its 16-byte output pieces only merge into full lines while the output stays in
// L2, so it is used up to 64 MiB per call (4096^2 x 1: 92 against 120 us with row
// pass + transpose; 4096^2 x 16: 2.39 against 1.65 ms; 2^23 x 32: 1.56 against 1.40 ms).
constexpr int64_t kToutMaxBytes = int64_t(64) << 20;
tcfftStatus exec_plan(tcfftPlan plan, void* data, void* stream, int dir, int norm, const void* in);

// Real 2D (kind 5).  R2C: real rows -> A [B][nx][h], transpose -> T [B][h][nx], complex
// columns in place on T, transpose -> out [B][nx][h].  C2R: the same backwards (the
// column inverse carries 1/nx unless R2C did, the row C2R 1/ny under the same rule).
tcfftStatus exec_real2d(tcfftPlanImpl* p, const void* in, void* out, void* stream, bool forward) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  const int64_t h = p->ny / 2 + 1;
  unsigned char* A = static_cast<unsigned char*>(p->big);
  unsigned char* T = A + p->span_elems;
  if (forward) {
    tcfftStatus r = tcfftExecuteR2C(p->subs[0], in, A, stream);
    if (r != TCFFT_SUCCESS) return r;
    if (cuda_status(launch_transpose(A, T, p->batch, p->nx, h, es, p->num_sms, st), "transpose")) return TCFFT_CUDA_ERROR;
    r = exec_plan(p->subs[1], T, stream, 0, p->normalize, nullptr);
    if (r != TCFFT_SUCCESS) return r;
    return cuda_status(launch_transpose(T, out, p->batch, h, p->nx, es, p->num_sms, st), "transpose");
  }
  if (cuda_status(launch_transpose(in, T, p->batch, p->nx, h, es, p->num_sms, st), "transpose")) return TCFFT_CUDA_ERROR;
  tcfftStatus r = exec_plan(p->subs[1], T, stream, 1, p->normalize ? 0 : 1, nullptr);
  if (r != TCFFT_SUCCESS) return r;
  if (cuda_status(launch_transpose(T, A, p->batch, h, p->nx, es, p->num_sms, st), "transpose")) return TCFFT_CUDA_ERROR;
  return tcfftExecuteC2R(p->subs[0], A, out, stream);
}

bool large1d_tout(const tcfftPlanImpl* p) {
  if (p->total_elems * 4 > kToutMaxBytes) return false;
  return p->precision == TCFFT_PRECISION_PLAIN && p->sched.N2 == 4096 &&
         resident_tout_supported(4096, p->sched.N1 * p->batch, p->sched.N1);
}
bool generic2d_tout(const tcfftPlanImpl* p, int axis) {
  if (p->precision != TCFFT_PRECISION_PLAIN || p->total_elems * 4 > kToutMaxBytes) return false;
  return axis == 0 ? p->ny == 4096 && resident_tout_supported(4096, p->nx * p->batch, p->nx)
                   : p->nx == 4096 && resident_tout_supported(4096, p->ny * p->batch, p->ny);
}

// Armed by tcfftInjectWaitTimeout: after the counter reset, phase-0 completion
// counter 0 is set to 0x80808080 (a large negative count), which no number of
// completed tiles raises to its target, so every wait on it runs out.
bool inject_stall(tcfftPlanImpl* plan, cudaStream_t st) {
  if (!plan->inject_timeout) return false;
  plan->inject_timeout = false;
  return cudaMemsetAsync(plan->counters, 0x80, sizeof(int), st) != cudaSuccess;
}

// dir: 0 = sign -1 (the reference's forward), 1 = sign +1 (conjugate direction);
// norm: 1 = scale every transform by 1 / (its element count).  The scale is a
// power of two, so it is exact; each kernel folds it into a twiddle it already
// applies (no extra pass, no extra work per element except in the tiny kernel).
// in: out of place, the input (not modified; `data` receives the output);
// nullptr or data: in place.  The single-pass, tiny, resident, cluster,
// two-phase 1D and composite 1D schedules read `in` directly; the others copy
// it to `data` first.
tcfftStatus exec_plan(tcfftPlan plan, void* data, void* stream, int dir, int norm, const void* in = nullptr) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (!data) return TCFFT_INVALID_VALUE;
  if ((reinterpret_cast<uintptr_t>(data) & 127) != 0 || (reinterpret_cast<uintptr_t>(in) & 127) != 0)
    return TCFFT_MISALIGNED;
  if (plan->kind == 4 || plan->kind == 5) return TCFFT_INVALID_VALUE;  // real plans: tcfftExecuteR2C / C2R
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const bool split = plan->precision != TCFFT_PRECISION_PLAIN;  // 8-byte elements (split or fp32 I/O)
  const int mode = plan->precision;                             // kernel mode: kModePlain/Split/Io32
  const int es = split ? 8 : 4;
  const Schedule& s = plan->sched;
  const void* src = in ? in : data;
  const bool direct = plan->kind != 3 && !plan->perm_tmp &&
                      (s.kind == Schedule::kSmall || s.kind == Schedule::kTiny || s.kind == Schedule::kResident ||
                       s.kind == Schedule::kCluster || s.kind == Schedule::kFused1d || s.kind == Schedule::kLarge1d);
  if (src != data && !direct) {  // schedules without a separate input: copy, then in place
    const int64_t bytes = (plan->kind == 3 ? plan->span_elems : plan->total_elems) * es;
    if (cuda_status(cudaMemcpyAsync(data, src, bytes, cudaMemcpyDeviceToDevice, st), "copy input")) return TCFFT_CUDA_ERROR;
    src = data;
  }
  if (plan->kind == 3) return exec_many(plan, data, st, dir, norm);
  const float oscale = norm ? 1.f / (float)(plan->kind == 2 ? plan->nx * plan->ny : plan->n) : 1.f;
  const float2* tw = plan->tables.tw2048[dir];
  const float dsign = dir == 0 ? 1.f : -1.f;
  // tensor maps name the buffers: re-encode when the (input, output) pair changes
  const bool fresh_maps = plan->tmap_ptr != data || plan->tmap_in != src;
  auto maps_done = [&]() {
    plan->tmap_ptr = data;
    plan->tmap_in = src;
  };
  if (plan->perm_tmp) {  // reference input order: move the input to natural order first
    const int64_t nx = plan->kind == 1 ? 1 : plan->nx, ny = plan->kind == 1 ? plan->n : plan->ny;
    if (cuda_status(to_natural_order(data, plan->perm_tmp, plan->rev_x, plan->rev_y, nx, ny, plan->batch,
                                     split ? 8 : 4, plan->num_sms, st),
                    "input reorder"))
      return TCFFT_CUDA_ERROR;
  }
  if (s.kind == Schedule::kCluster) {
    cudaError_t e = launch_cluster(plan->n, data, plan->batch, tw, plan->twlo[dir], plan->twhi[dir], dsign,
                                   plan->tables.err, plan->num_sms, st, &plan->fmaps.load0, &plan->fmaps.store0,
                                   fresh_maps, oscale, src);
    if (e == cudaSuccess) maps_done();
    return cuda_status(e, "cluster launch");
  }
  if (s.kind == Schedule::kResident) {
    cudaError_t e =
        split ? launch_resident_split(plan->n, data, plan->batch, tw, plan->twlo[dir], plan->twhi[dir], dsign,
                                      plan->tables.err, plan->num_sms, st, &plan->fmaps.load0, &plan->fmaps.store0,
                                      fresh_maps, oscale, src, mode == TCFFT_PRECISION_FP32_IO)
              : launch_resident(plan->n, data, plan->batch, tw, plan->twlo[dir], plan->twhi[dir], dsign,
                                plan->tables.err, plan->num_sms, st, &plan->fmaps.load0, &plan->fmaps.store0,
                                fresh_maps, oscale, src);
    if (e == cudaSuccess) maps_done();
    return cuda_status(e, "resident launch");
  }
  if (s.kind == Schedule::kTiny)
    return cuda_status(launch_tiny(plan->n, mode, data, plan->batch, tw, dsign, plan->num_sms, st, oscale, src),
                       "tiny launch");
  if (s.kind == Schedule::kLarge1d) {
    const FusedKey& k = s.key;
    const bool fresh = fresh_maps;
    if (fresh) {
      const CUtensorMapDataType dt = split ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
      if (cu_status(encode_col_load(&plan->fmaps.load0, dt, const_cast<void*>(src), s.N2, plan->batch, es, k.C0,
                                    k.R0),
                    "tmap load0") ||
          cu_status(encode_col_store(&plan->fmaps.store0, dt, plan->big, s.N2, plan->batch, es, k.C0, k.R0),
                    "tmap store0"))
        return TCFFT_CUDA_ERROR;
      plan->fmaps.load1 = plan->fmaps.load0;  // phase 1 has no work items
      plan->fmaps.store1 = plan->fmaps.store0;
      maps_done();
    }
    FusedParams fp;
    memset(&fp, 0, sizeof fp);
    fp.tw2048 = tw;
    fp.scratch = static_cast<unsigned char*>(plan->big);
    fp.twlo = plan->twlo[dir];
    fp.twhi = plan->twhi[dir];
    fp.tw_shift = plan->tw_shift;
    fp.wn_global = 1;
    fp.n_mask = (long long)(plan->n - 1);
    fp.batch = (int)plan->batch;
    fp.D = 0;
    fp.S = s.S;
    fp.T0 = s.T0;
    fp.T1 = 0;
    fp.rows0 = (int)s.N1;
    fp.rows1 = (int)s.N1;
    fp.cols0 = s.T0;
    fp.cols1 = 1;
    fp.cnt0 = plan->counters;
    fp.cnt1 = plan->counters + s.S;
    fp.err = plan->tables.err;
    fp.dsign = dsign;
    fp.wait_ns = plan->wait_ns;
    fp.oscale0 = norm ? 1.f / (float)s.N1 : 1.f;  // the column pass scales by 1/N1, the rows by 1/N2
    fp.oscale1 = 1.f;
    if (cuda_status(cudaMemsetAsync(plan->counters, 0, sizeof(int) * 2 * s.S, st), "counter reset"))
      return TCFFT_CUDA_ERROR;
    int grid = 0;
    if (cuda_status(launch_fused(k, plan->fmaps, fp, plan->num_sms, st, &grid), "column pass")) return TCFFT_CUDA_ERROR;
    if (large1d_tout(plan)) {
      // rows of N2 = 4096 written transposed straight into data: X[k1 + N1 k2]
      const tcfftPlanImpl* rp = plan->subs[0];
      return cuda_status(launch_resident_tout(4096, plan->big, data, s.N1 * plan->batch, s.N1, tw, rp->twlo[dir],
                                              rp->twhi[dir], dsign, plan->tables.err, plan->num_sms, st,
                                              &plan->fmaps.load1, &plan->fmaps.store1, fresh,
                                              norm ? 1.f / 4096 : 1.f),
                         "rows (transposed output)");
    }
    tcfftStatus r = exec_plan(plan->subs[0], plan->big, stream, dir, norm);  // rows of N2 (scaled by 1/N2)
    if (r != TCFFT_SUCCESS) return r;
    // [B][N1 rows k1][N2 cols k2] -> X[k1 + N1 k2] = [B][N2][N1]
    return cuda_status(launch_transpose(plan->big, data, plan->batch, s.N1, s.N2, es, plan->num_sms, st), "transpose");
  }
  if (s.kind == Schedule::kGeneric2d) {
    // an axis of 4096 runs as the resident kernel with transposed output, which
    // replaces that axis' transpose
    const bool fresh = fresh_maps;
    maps_done();
    const int64_t nx = plan->nx, ny = plan->ny, B = plan->batch;
    if (generic2d_tout(plan, 0)) {  // rows of ny -> big = [B][ny][nx]
      const tcfftPlanImpl* rp = plan->subs[0];
      if (cuda_status(launch_resident_tout(4096, data, plan->big, nx * B, nx, tw, rp->twlo[dir], rp->twhi[dir], dsign,
                                           plan->tables.err, plan->num_sms, st, &plan->fmaps.load0,
                                           &plan->fmaps.store0, fresh, norm ? 1.f / 4096 : 1.f),
                      "rows (transposed output)"))
        return TCFFT_CUDA_ERROR;
    } else {
      tcfftStatus r = exec_plan(plan->subs[0], data, stream, dir, norm);  // rows of ny (scaled by 1/ny)
      if (r != TCFFT_SUCCESS) return r;
      if (cuda_status(launch_transpose(data, plan->big, B, nx, ny, es, plan->num_sms, st), "transpose"))
        return TCFFT_CUDA_ERROR;
    }
    if (generic2d_tout(plan, 1)) {  // columns of nx (rows of big) -> data = [B][nx][ny]
      const tcfftPlanImpl* cp = plan->subs[1];
      return cuda_status(launch_resident_tout(4096, plan->big, data, ny * B, ny, tw, cp->twlo[dir], cp->twhi[dir],
                                              dsign, plan->tables.err, plan->num_sms, st, &plan->fmaps.load1,
                                              &plan->fmaps.store1, fresh, norm ? 1.f / 4096 : 1.f),
                         "columns (transposed output)");
    }
    tcfftStatus r = exec_plan(plan->subs[1], plan->big, stream, dir, norm);  // columns of nx, now rows
    if (r != TCFFT_SUCCESS) return r;
    return cuda_status(launch_transpose(plan->big, data, B, ny, nx, es, plan->num_sms, st), "transpose");
  }
  if (s.kind == Schedule::kSmall) {
    // 2D view of the whole batch: rows of 128 bytes
    const int er = 128 / es;
    const uint64_t rows = (uint64_t)plan->total_elems / er;
    if (fresh_maps) {  // loads through tmap0 (the input), stores through tmap1 (the output)
      uint64_t dims[2] = {(uint64_t)er, rows};
      uint64_t strides[1] = {128};
      uint32_t box[2] = {(uint32_t)er, 256};
      const CUtensorMapDataType dt = split ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
      if (cu_status(encode_tmap(&plan->tmap0, dt, 2, const_cast<void*>(src), dims, strides, box,
                                CU_TENSOR_MAP_SWIZZLE_128B),
                    "tmap small") ||
          cu_status(encode_tmap(&plan->tmap1, dt, 2, data, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B),
                    "tmap small"))
        return TCFFT_CUDA_ERROR;
      maps_done();
    }
    int launches = 0;
    return cuda_status(launch_small(s.R, mode, plan->tmap0, plan->tmap1, plan->total_elems, tw, dsign,
                                    plan->tables.err, plan->num_sms, st, &launches, oscale));
  }
  if (s.kind == Schedule::kFused1d) {
    if (fresh_maps) {
      const FusedKey& k = s.key;
      if (cu_status(encode_fused1d_maps(&plan->fmaps, k, data, plan->scratch, s.N1, s.N2, plan->batch, s.S, src),
                    "tmap fused1d"))
        return TCFFT_CUDA_ERROR;
      maps_done();
    }
    FusedParams fp;
    fp.tw2048 = tw;
    fp.scratch = static_cast<unsigned char*>(plan->scratch);
    fp.twlo = plan->twlo[dir];
    fp.twhi = plan->twhi[dir];
    fp.tw_shift = plan->tw_shift;
    fp.n_mask = (long long)(plan->n - 1);
    fp.batch = (int)plan->batch;
    fp.D = s.D;
    fp.S = s.S;
    fp.T0 = s.T0;
    fp.T1 = s.T1;
    fp.rows0 = (int)s.N1;
    fp.rows1 = (int)s.N1;
    fp.cols0 = s.T0;
    fp.cols1 = s.T1;
    fp.cnt0 = plan->counters;
    fp.cnt1 = plan->counters + s.S;
    fp.err = plan->tables.err;
    fp.dsign = dsign;
    fp.wait_ns = plan->wait_ns;
    // 1/N split as 1/N1 (columns) and 1/N2 (rows); the short-row phase takes no scale
    const bool short_rows = s.key.role1 == kRoleRow16T;
    fp.oscale0 = norm ? (short_rows ? oscale : 1.f / (float)s.N1) : 1.f;
    fp.oscale1 = norm && !short_rows ? 1.f / (float)s.N2 : 1.f;
    if (cuda_status(cudaMemsetAsync(plan->counters, 0, sizeof(int) * 2 * s.S, st), "counter reset") ||
        inject_stall(plan, st))
      return TCFFT_CUDA_ERROR;
    int grid = 0;
    return cuda_status(launch_fused(s.key, plan->fmaps, fp, plan->num_sms, st, &grid), "fused launch");
  }
  if (s.kind == Schedule::kFused2d) {
    const int er = 128 / es;
    const CUtensorMapDataType dt = split ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
    const FusedKey& k = s.key;
    const int64_t nx = s.N1, ny = s.N2;
    if (fresh_maps) {
      {  // phase 0 (rows, in place): contiguous 128-byte rows, one tile per box group
        const int64_t tile_rows = (int64_t)k.C0 * ny / er;
        uint64_t dims[2] = {(uint64_t)er, (uint64_t)(plan->batch * nx * ny / er)};
        uint64_t str[1] = {128};
        uint32_t box[2] = {(uint32_t)er, (uint32_t)(tile_rows < 256 ? tile_rows : 256)};
        if (cu_status(encode_tmap(&plan->fmaps.load0, dt, 2, data, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B),
                      "tmap2d load0"))
          return TCFFT_CUDA_ERROR;
        plan->fmaps.store0 = plan->fmaps.load0;
      }
      // phase 1 (columns, in place): data as [B*NX][NY], NX = 256 R1 rows per transform
      if (cu_status(encode_col_load(&plan->fmaps.load1, dt, data, ny, plan->batch, es, k.C1, k.R1), "tmap2d load1"))
        return TCFFT_CUDA_ERROR;
      if (cu_status(encode_col_store(&plan->fmaps.store1, dt, data, ny, plan->batch, es, k.C1, k.R1),
                    "tmap2d store1"))
        return TCFFT_CUDA_ERROR;
      maps_done();
    }
    FusedParams fp;
    memset(&fp, 0, sizeof fp);
    fp.tw2048 = tw;
    fp.batch = (int)plan->batch;
    fp.D = s.D;
    fp.S = s.S;
    fp.T0 = s.T0;
    fp.T1 = s.T1;
    fp.rows0 = (int)nx;
    fp.rows1 = (int)nx;
    fp.cols0 = s.T0;
    fp.cols1 = s.T1;
    fp.cnt0 = plan->counters;
    fp.cnt1 = plan->counters + s.S;
    fp.err = plan->tables.err;
    fp.dsign = dsign;
    fp.wait_ns = plan->wait_ns;
    fp.oscale0 = norm ? 1.f / (float)ny : 1.f;  // rows
    fp.oscale1 = norm ? 1.f / (float)nx : 1.f;  // columns
    if (cuda_status(cudaMemsetAsync(plan->counters, 0, sizeof(int) * 2 * s.S, st), "counter reset") ||
        inject_stall(plan, st))
      return TCFFT_CUDA_ERROR;
    int grid = 0;
    return cuda_status(launch_fused(s.key, plan->fmaps, fp, plan->num_sms, st, &grid), "fused2d launch");
  }
  return TCFFT_NOT_SUPPORTED;
}

// Two-level W_N table (fp32 from long double): W_N^j = hi[j >> shift] * lo[j & mask].
tcfftStatus alloc_wn_tables(tcfftPlanImpl* p, int64_t n) {
  const int lg = ilog2_exact(n);
  p->tw_shift = (lg + 1) / 2;
  const int64_t nlo = int64_t(1) << p->tw_shift, nhi = n >> p->tw_shift;
  std::vector<float2> lo(nlo), hi(nhi);
  for (int d = 0; d < 2; ++d) {
    const long double sgn = d == 0 ? -1.0L : 1.0L;
    const long double twopi = 2.0L * 3.141592653589793238462643383279502884L;
    for (int64_t j = 0; j < nlo; ++j) {
      const long double th = twopi * (long double)j / (long double)n;
      lo[j] = make_float2((float)cosl(th), (float)(sgn * sinl(th)));
    }
    for (int64_t j = 0; j < nhi; ++j) {
      const long double th = twopi * (long double)(j << p->tw_shift) / (long double)n;
      hi[j] = make_float2((float)cosl(th), (float)(sgn * sinl(th)));
    }
    if (cudaMalloc(&p->twlo[d], nlo * sizeof(float2)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (cudaMalloc(&p->twhi[d], nhi * sizeof(float2)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (cudaMemcpy(p->twlo[d], lo.data(), nlo * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->twhi[d], hi.data(), nhi * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
      return TCFFT_CUDA_ERROR;
  }
  return TCFFT_SUCCESS;
}

// Counters and (1D) scratch ring for the current schedule's slot count.
tcfftStatus alloc_ring(tcfftPlanImpl* p) {
  const Schedule& s = p->sched;
  const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  if (p->counters) cudaFree(p->counters);
  if (p->scratch) cudaFree(p->scratch);
  p->counters = nullptr;
  p->scratch = nullptr;
  p->scratch_bytes = 0;
  p->tmap_ptr = nullptr;  // the maps name the scratch
  if (cudaMalloc(&p->counters, sizeof(int) * 2 * s.S) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  if (s.kind == Schedule::kFused1d) {
    p->scratch_bytes = (int64_t)s.S * p->n * es;
    if (cudaMalloc(&p->scratch, p->scratch_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  }
  return TCFFT_SUCCESS;
}

tcfftStatus alloc_fused(tcfftPlanImpl* p) {
  if (p->sched.kind == Schedule::kFused1d) {
    tcfftStatus st = alloc_wn_tables(p, p->n);
    if (st != TCFFT_SUCCESS) return st;
  }
  return alloc_ring(p);
}

// Large 1D: full-size intermediate, counters (one slot per transform), W_N
// tables for N (read from global memory by the column pass) and the row plan.
tcfftStatus setup_large1d(tcfftPlanImpl* p) {
  const Schedule& s = p->sched;
  const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  if (cudaMalloc(&p->counters, sizeof(int) * 2 * s.S) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  tcfftStatus st = alloc_wn_tables(p, p->n);
  if (st != TCFFT_SUCCESS) return st;
  p->scratch_bytes = p->n * p->batch * es;
  if (cudaMalloc(&p->big, p->scratch_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  o.precision = p->precision;
  tcfftPlan rows = nullptr;
  st = tcfftPlan1d(&rows, s.N2, s.N1 * p->batch, &o);
  if (st != TCFFT_SUCCESS) return st;
  p->subs.push_back(rows);
  p->sched.launches = 2 + rows->sched.launches;
  if (large1d_tout(p)) {
    p->sched.launches = 2;
    p->sched.text += ", rows written transposed (no transpose pass)";
  }
  p->scratch_bytes += rows->scratch_bytes;
  return TCFFT_SUCCESS;
}

// Generic 2D: row plan over ny, column plan over nx (run on the transpose), one
// full-size intermediate.
tcfftStatus setup_generic2d(tcfftPlanImpl* p) {
  const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  p->scratch_bytes = p->nx * p->ny * p->batch * es;
  if (cudaMalloc(&p->big, p->scratch_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  o.precision = p->precision;
  tcfftPlan rows = nullptr, cols = nullptr;
  tcfftStatus st = tcfftPlan1d(&rows, p->ny, p->nx * p->batch, &o);
  if (st != TCFFT_SUCCESS) return st;
  p->subs.push_back(rows);
  st = tcfftPlan1d(&cols, p->nx, p->ny * p->batch, &o);
  if (st != TCFFT_SUCCESS) return st;
  p->subs.push_back(cols);
  p->sched.launches = rows->sched.launches + cols->sched.launches + 2;
  if (generic2d_tout(p, 0) || generic2d_tout(p, 1)) {
    p->sched.launches = (generic2d_tout(p, 0) ? 1 : rows->sched.launches + 1) +
                        (generic2d_tout(p, 1) ? 1 : cols->sched.launches + 1);
    p->sched.text += generic2d_tout(p, 0) && generic2d_tout(p, 1) ? " (both axes: 4096-point rows written transposed)"
                                                                  : " (one 4096 axis written transposed)";
  }
  p->scratch_bytes += rows->scratch_bytes + cols->scratch_bytes;
  return TCFFT_SUCCESS;
}

// ------------------------------------------------------------------ autotuner
// For the two-phase executor the free parameters with measured effect are the
// lag (how many transforms are between their first and second phase, which
// sets the L2 footprint of the intermediate and the slack of the cross-CTA
// dependency) and, for 1D sizes N = N1 x N2, the decomposition N1 and the
// work-item size (64 or 32 KiB).  At plan time, with tcfftOptions.autotune = 1,
// the plan times each decomposition / item-size candidate at the built-in lag,
// then a few lag multipliers for the fastest, on a scratch buffer of its own
// size, and keeps the fastest; results are cached per (shape, batch,
// precision) in the process and, if tune_cache_path is set, in that text file
// ("key|lag|N1|item KiB" lines; "key|lag" lines of older files still load).
struct TuneChoice {
  double lag = 1.0;
  int64_t n1 = 0;  // 0: the built-in decomposition
  int item_kb = 0; // 0: the built-in item size
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_cache;
std::set<std::string> g_tune_files_read;

void load_tune_file(const char* path) {
  if (!path || g_tune_files_read.count(path)) return;
  g_tune_files_read.insert(path);
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[256];
  while (fgets(line, sizeof line, f)) {
    char key[200];
    TuneChoice c;
    long long n1 = 0;
    int kb = 0;
    const int got = sscanf(line, "%199[^|]|%lf|%lld|%d", key, &c.lag, &n1, &kb);
    if (got < 2 || !(c.lag > 0)) continue;
    if (got == 4) {
      c.n1 = n1;
      c.item_kb = kb;
    }
    g_tune_cache[key] = c;
  }
  fclose(f);
}

tcfftStatus choose_again(tcfftPlanImpl* p, const TuneChoice& c, Schedule& s) {
  g_lag_override = c.lag;
  g_n1_override = c.n1;
  g_item_kb_override = c.item_kb;
  tcfftStatus st = p->kind == 1 ? choose_1d(p->n, p->batch, p->precision, s, p->num_sms)
                                : choose_2d(p->nx, p->ny, p->batch, p->precision, s, p->num_sms);
  g_lag_override = 0.0;
  g_n1_override = 0;
  g_item_kb_override = 0;
  return st;
}

tcfftStatus apply_choice(tcfftPlanImpl* p, const TuneChoice& c) {
  Schedule s;
  tcfftStatus st = choose_again(p, c, s);
  if (st != TCFFT_SUCCESS) return st;
  if (s.kind != p->sched.kind) return TCFFT_NOT_SUPPORTED;  // candidates never change the schedule kind
  p->sched = s;
  p->lag_scale = c.lag;
  return alloc_ring(p);
}

// 1D decomposition / item-size candidates for the tuner: N1 = 2^ceil(lg/2) and
// 2^floor(lg/2) (the schedule's bounds keep N1, N2 in 256..2048), each with
// 64 and 32 KiB items; choose_1d falls back to 64 KiB where 32 is not built.
std::vector<TuneChoice> shape_candidates(const tcfftPlanImpl* p) {
  std::vector<TuneChoice> out;
  out.push_back(TuneChoice());
  if (p->kind != 1) return out;
  const int lg = ilog2_exact(p->n);
  if (lg < 16 || lg > 22) return out;
  for (int e : {(lg + 1) / 2, lg / 2, (lg + 1) / 2 + 1, lg / 2 - 1}) {
    const int64_t n1 = int64_t(1) << e;
    if (n1 < 256 || n1 > 2048 || p->n / n1 < 256 || p->n / n1 > 2048) continue;
    for (int kb : {64, 32}) {
      TuneChoice c;
      c.n1 = n1;
      c.item_kb = kb;
      out.push_back(c);
    }
  }
  return out;
}

tcfftStatus autotune_plan(tcfftPlanImpl* p, const tcfftOptions& o) {
  if (p->sched.kind != Schedule::kFused1d && p->sched.kind != Schedule::kFused2d) return TCFFT_SUCCESS;
  char kb[200];
  snprintf(kb, sizeof kb, "%d %lld %lld %lld %d", p->kind, (long long)p->nx, (long long)p->ny, (long long)p->batch,
           p->precision);
  const std::string key = kb;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_tune_file(o.tune_cache_path);
  TuneChoice best;
  auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    best = it->second;
  } else {
    const int es = p->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, p->total_elems * es) != cudaSuccess) {
      cudaGetLastError();
      return TCFFT_SUCCESS;  // not enough memory to time: keep the built-in schedule
    }
    cudaMemset(tmp, 0, p->total_elems * es);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    bool failed = false;
    // one timing: a warm-up execute, then three timed ones
    auto time_choice = [&](const TuneChoice& c, float* ms) {
      if (apply_choice(p, c) != TCFFT_SUCCESS) return false;
      if (exec_plan(p, tmp, nullptr, 0, 0) != TCFFT_SUCCESS) return false;
      cudaEventRecord(e0, nullptr);
      for (int r = 0; r < 3; ++r) exec_plan(p, tmp, nullptr, 0, 0);
      cudaEventRecord(e1, nullptr);
      if (cudaEventSynchronize(e1) != cudaSuccess) return false;
      cudaEventElapsedTime(ms, e0, e1);
      return true;
    };
    // stage 1: decomposition and item size at the built-in lag (distinct schedules only)
    std::set<std::string> seen;
    for (const TuneChoice& c : shape_candidates(p)) {
      Schedule s;
      if (choose_again(p, c, s) != TCFFT_SUCCESS || s.kind != p->sched.kind) continue;
      char sig[64];
      snprintf(sig, sizeof sig, "%lld %d %d %d", (long long)s.N1, s.key.item_kb, s.key.C0, s.key.C1);
      if (!seen.insert(sig).second) continue;
      float ms = 0;
      if (!time_choice(c, &ms)) {
        failed = true;
        break;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    // stage 2: the lag for the chosen shape
    std::set<int> seen_d;
    {
      Schedule s;
      if (!failed && choose_again(p, best, s) == TCFFT_SUCCESS) seen_d.insert(s.D);
    }
    for (double lag : {0.6, 1.6, 2.5}) {
      if (failed) break;
      TuneChoice c = best;
      c.lag = lag;
      Schedule s;
      if (choose_again(p, c, s) != TCFFT_SUCCESS || !seen_d.insert(s.D).second) continue;
      float ms = 0;
      if (!time_choice(c, &ms)) {
        failed = true;
        break;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(tmp);
    if (failed) {
      cudaGetLastError();
      best = TuneChoice();  // a candidate failed to run: keep the built-in schedule, cache nothing
    } else {
      g_tune_cache[key] = best;
      if (o.tune_cache_path) {
        FILE* f = fopen(o.tune_cache_path, "a");
        if (f) {
          fprintf(f, "%s|%.3f|%lld|%d\n", key.c_str(), best.lag, (long long)best.n1, best.item_kb);
          fclose(f);
        }
      }
    }
  }
  tcfftStatus st = apply_choice(p, best);
  if (st != TCFFT_SUCCESS) {
    st = apply_choice(p, TuneChoice());  // e.g. a cache line for another build's instantiations
    if (st != TCFFT_SUCCESS) return st;
    best = TuneChoice();
  }
  // in front: the plan-info string is 128 characters
  char buf[96];
  if (p->kind == 1 && p->sched.kind == Schedule::kFused1d)
    snprintf(buf, sizeof buf, "[tuned: N1=%lld, %d KiB items, lag x%.2g] ", (long long)p->sched.N1,
             p->sched.key.item_kb, best.lag);
  else
    snprintf(buf, sizeof buf, "[tuned: lag x%.2g] ", best.lag);
  p->sched.text = buf + p->sched.text;
  return TCFFT_SUCCESS;
}

tcfftStatus check_errors(tcfftPlanImpl* p) {
  int e = 0;
  if (cudaMemcpy(&e, p->tables.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return TCFFT_CUDA_ERROR;
  tcfftStatus r = TCFFT_SUCCESS;
  if (e != 0) {
    cudaMemset(p->tables.err, 0, sizeof(int));
    r = TCFFT_TIMEOUT;
  }
  for (tcfftPlanImpl* sp : p->subs) {
    tcfftStatus rs = check_errors(sp);
    if (r == TCFFT_SUCCESS) r = rs;
  }
  for (tcfftPlanImpl* sp : p->host_sub)
    if (sp) {
      tcfftStatus rs = check_errors(sp);
      if (r == TCFFT_SUCCESS) r = rs;
    }
  return r;
}

// ------------------------------------------------------------------ many-shape executor (plain)
// Pass A / pass B kinds of a transform (kMkKinds: not supported by the executor).
// Rank 3 is a "columns" transform: FFTs of nx points down the ny columns of an
// [nx][ny] matrix (no pass A; tcfftPlanStrided with istride = ny).
int many_kind_a(int rank, int64_t nx, int64_t ny) {
  if (rank == 3) return -1;
  if (rank == 1) {
    switch (nx) {
      case 256: return kMkRow1 | kMkList;
      case 512: return kMkRow2 | kMkList;
      case 1024: return kMkRow4 | kMkList;
      case 2048: return kMkRow8 | kMkList;
      case 4096: case 8192: case 16384: return kMkColWn1x16;
      case 32768: return kMkColWn2x32;
      case 65536: return kMkColWn1x32;
      default: return kMkKinds;
    }
  }
  switch (ny) {
    case 128: return kMkRow128;
    case 256: return kMkRow1;
    case 512: return kMkRow2;
    case 1024: return kMkRow4;
    case 2048: return kMkRow8;
    default: return kMkKinds;
  }
}
int many_kind_b(int rank, int64_t nx, int64_t ny) {
  if (rank == 1) {
    switch (nx) {
      case 4096: return kMkRow16T1;
      case 8192: return kMkRow16T2;
      case 16384: case 32768: return kMkRow16T4;
      case 65536: return kMkRowT1;
      default: return nx <= 2048 ? -1 : kMkKinds;  // -1: no pass B
    }
  }
  const int k = nx == 128 ? kMkCol128 : nx == 256 ? kMkCol1 : nx == 512 ? kMkCol2 : nx == 1024 ? kMkCol4
              : nx == 2048 ? kMkCol8 : kMkKinds;
  // whole tiles of columns (2D shapes have ny >= 128, a multiple of every tile width)
  if (k != kMkKinds && ny % (k == kMkCol128 ? 128 : many_c(k)) != 0) return kMkKinds;
  return k;
}
// 1D N >= 4096 = N1 x N2 in the executor (N1 = 256, 2^15: 512)
int64_t many_n1(int64_t n) { return n == 32768 ? 512 : 256; }

// Tiles of a transform's pass for a (non-listed) kind.
int64_t many_tiles(int kind, int rank, int64_t nx, int64_t ny) {
  const int C = many_c(kind);
  switch (kind) {
    case kMkRow1: case kMkRow2: case kMkRow4: case kMkRow8: return nx / C;
    case kMkRow128: return nx / 128;
    case kMkColWn1x16: case kMkColWn1x32: case kMkColWn2x32: return (nx / many_n1(nx)) / C;
    case kMkRowT1: return many_n1(nx) / C;
    case kMkRow16T1: case kMkRow16T2: case kMkRow16T4: return many_n1(nx) / 128;
    case kMkCol1: case kMkCol2: case kMkCol4: case kMkCol8: return ny / C;
    case kMkCol128: return ny / 128;
    default: (void)rank; return 0;
  }
}

// The executor's work (host logic only): per transform its shape and scratch offset, the item
// sequence of the one launch and the row list of the listed 1D transforms.  False when a shape is
// not one the executor runs.
bool build_many_items(int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                      const int64_t* offsets, int num_sms, std::vector<tcfftPlanImpl::ManyXf>& xf,
                      std::vector<ManyItem>& seq, std::vector<int>& rows, int64_t& soff) {
  xf.assign((size_t)count, tcfftPlanImpl::ManyXf{});
  seq.clear();
  rows.clear();
  soff = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int r = ranks[i];
    const int64_t x = nx[i], y = r >= 2 ? ny[i] : 1;
    if (many_kind_a(r, x, y) == kMkKinds || many_kind_b(r, x, y) == kMkKinds) return false;
    if (r == 3 && many_kind_b(r, x, y) < 0) return false;
    xf[i] = {r, x, y, offsets[i], 0};
    if (r == 1 && x >= 4096) {
      xf[i].soff = soff;
      soff += x;
    }
  }
  // Items: the listed 1D transforms (no pass B) first, then per transform its pass-A
  // items, with its pass-B items following lag items later (its intermediate is still in
  // L2 then and its pass A complete).  Transforms are taken in order of their kinds, so
  // that the CTAs run at most a few kinds at a time.
  {
    std::vector<int64_t> listed[kMkKinds];
    std::vector<int64_t> order;
    for (int64_t i = 0; i < count; ++i) {
      const auto& t = xf[i];
      const int k = many_kind_a(t.rank, t.nx, t.ny);
      if (k >= 0 && (k & kMkList)) listed[k & 0xff].push_back(i);
      else order.push_back(i);
    }
    for (int kind = 0; kind < kMkKinds; ++kind) {
      const int C = many_c(kind);
      for (size_t j = 0; j < listed[kind].size(); j += C) {
        const int cnt = (int)std::min<size_t>(C, listed[kind].size() - j);
        seq.push_back({kind | kMkList, (int)rows.size(), 0, cnt, 1, 0, {0, 0}});
        // the transform's offset in rows of 128 bytes (a coordinate of the buffer-wide maps)
        for (int q = 0; q < cnt; ++q) rows.push_back((int)(xf[listed[kind][j + q]].off / 32));
      }
    }
    auto kinds_of = [&](int64_t i) {
      const auto& t = xf[i];
      return std::make_pair(many_kind_a(t.rank, t.nx, t.ny), many_kind_b(t.rank, t.nx, t.ny));
    };
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return kinds_of(a) < kinds_of(b); });
    // lag (in items) between a transform's pass A and its pass B, in multiples of the SM
    // count (TCFFT_MANY_LAG overrides it): on the uneven-batch workload 4 x gave 139 us, 6 x 130,
    // 8 x 134 and 12 x 123 (a pass-B item that waits stalls its CTA's producer)
    static const double lag_env = getenv("TCFFT_MANY_LAG") ? atof(getenv("TCFFT_MANY_LAG")) : 0.0;
    const double lag_mult = lag_env > 0.0 ? lag_env : 10.0;
    const size_t lag = (size_t)(lag_mult * (double)num_sms);
    std::vector<std::pair<int64_t, size_t>> waiting;  // (transform, sequence length after its pass A)
    size_t head = 0;
    // consecutive tiles of a transform share an item up to one 64 KiB stage
    auto sub_of = [](int kind) {
      const int per = (64 * 1024) / (many_item_elems(kind) * 4);
      return per < 1 ? 1 : per;
    };
    auto items_of = [&](int kind, int64_t tiles) { return (tiles + sub_of(kind) - 1) / sub_of(kind); };
    auto emit_b = [&](int64_t i) {
      const auto& t = xf[i];
      const auto k = kinds_of(i);
      const int na = k.first < 0 ? 0 : (int)items_of(k.first, many_tiles(k.first, t.rank, t.nx, t.ny));
      const int64_t tiles = many_tiles(k.second, t.rank, t.nx, t.ny);
      for (int64_t tile = 0; tile < tiles; tile += sub_of(k.second)) {
        const int nsub = (int)std::min<int64_t>(sub_of(k.second), tiles - tile);
        seq.push_back({k.second | kMkB, (int)i, (int)tile, na, nsub, 0, {0, 0}});
      }
    };
    for (int64_t i : order) {
      const auto& t = xf[i];
      const auto k = kinds_of(i);
      if (k.first < 0) {  // columns only: no pass A, its pass-B items wait for nothing
        emit_b(i);
        continue;
      }
      int wn = 0;
      if (k.first == kMkColWn1x16 || k.first == kMkColWn1x32 || k.first == kMkColWn2x32)
        wn = (int)(t.nx - 1);
      const int64_t tiles = many_tiles(k.first, t.rank, t.nx, t.ny);
      for (int64_t tile = 0; tile < tiles; tile += sub_of(k.first)) {
        const int nsub = (int)std::min<int64_t>(sub_of(k.first), tiles - tile);
        seq.push_back({k.first | kMkRelease, (int)i, (int)tile, 0, nsub, wn, {0, 0}});
      }
      waiting.push_back({i, seq.size()});
      while (head < waiting.size() && waiting[head].second + lag <= seq.size()) emit_b(waiting[head++].first);
    }
    // the pass-B items left after the last pass A run largest first: the smallest finish the launch
    const size_t tail = seq.size();
    while (head < waiting.size()) emit_b(waiting[head++].first);
    std::stable_sort(seq.begin() + tail, seq.end(), [](const ManyItem& a, const ManyItem& b) {
      return a.nsub * many_item_elems(a.kind & 0xff) > b.nsub * many_item_elems(b.kind & 0xff);
    });
  }
  return true;
}

// Builds the executor's items, row list, scratch and W_N tables; false (nothing
// allocated that the plan does not free) when a shape is not supported.
bool setup_many_pass(tcfftPlanImpl* p, int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                     const int64_t* offsets) {
  if (p->precision != TCFFT_PRECISION_PLAIN || getenv("TCFFT_MANY_GRAPH")) return false;
  if (count > (int64_t)1 << 24) return false;
  // tensor-map coordinates are 32-bit: the buffer-wide maps address the span in rows of 128 bytes
  if (p->span_elems / 32 > (int64_t)INT32_MAX - 256) return false;
  std::vector<tcfftPlanImpl::ManyXf> xf;
  std::vector<ManyItem> seq;
  std::vector<int> rows;
  int64_t soff = 0;
  if (!build_many_items(count, ranks, nx, ny, offsets, p->num_sms, xf, seq, rows, soff)) return false;
  // device arrays
  const size_t nit = seq.size();
  if (cudaMalloc(&p->many_items, std::max<size_t>(nit, 1) * sizeof(ManyItem)) != cudaSuccess ||
      cudaMalloc(&p->many_rows, std::max<size_t>(rows.size(), 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&p->many_maps, (size_t)(count + 1) * 4 * sizeof(CUtensorMap)) != cudaSuccess ||
      cudaMallocHost(&p->many_hmaps, (size_t)(count + 1) * 4 * sizeof(CUtensorMap)) != cudaSuccess ||
      (soff > 0 && cudaMalloc(&p->many_scratch, soff * 4) != cudaSuccess)) {
    cudaGetLastError();
    return false;
  }
  const std::vector<ManyItem>& all = seq;
  {  // W_65536 in three levels, both directions (fp32 from long double)
    std::vector<float2> w3(256);
    const long double twopi = 2.0L * 3.141592653589793238462643383279502884L;
    for (int d = 0; d < 2; ++d)
      for (int i = 0; i < 128; ++i) {
        const int e = i < 64 ? i * 1024 : i < 96 ? (i - 64) * 32 : i - 96;
        const long double th = twopi * (long double)e / 65536.0L;
        w3[d * 128 + i] = make_float2((float)cosl(th), (float)((d == 0 ? -1.0L : 1.0L) * sinl(th)));
      }
    if (cudaMalloc(&p->many_wn3, 256 * sizeof(float2)) != cudaSuccess ||
        cudaMemcpy(p->many_wn3, w3.data(), 256 * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  }
  if (cudaMalloc(&p->many_claim, (size_t)(count + 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&p->many_fold8, 2 * (size_t)many_fold8_bytes()) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  for (int d = 0; d < 2; ++d)
    if (many_fold8_init(p->many_fold8 + d * many_fold8_bytes(), p->tables.tw2048[d], nullptr) != cudaSuccess)
      return false;
  if (cudaDeviceSynchronize() != cudaSuccess) return false;
  if ((nit && cudaMemcpy(p->many_items, all.data(), nit * sizeof(ManyItem), cudaMemcpyHostToDevice) != cudaSuccess) ||
      (!rows.empty() &&
       cudaMemcpy(p->many_rows, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess))
    return false;
  for (int64_t i = 0; i < count && p->many_xf_b < 0; ++i)
    if (many_kind_b(xf[i].rank, xf[i].nx, xf[i].ny) >= 0) p->many_xf_b = (int)i;
  p->many_xf = std::move(xf);
  p->many_n[0] = (int)seq.size();
  p->many_n[1] = 0;
  p->scratch_bytes += soff * 4;
  p->many_ok = true;
  return true;
}

// The transforms' tensor maps for data buffer `data` (into the pinned staging copy).
CUresult encode_many_maps(tcfftPlanImpl* p, void* data) {
  const CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_UINT32;
  unsigned char* d = static_cast<unsigned char*>(data);
  unsigned char* sc = static_cast<unsigned char*>(p->many_scratch);
  for (size_t i = 0; i < p->many_xf.size(); ++i) {
    const auto& t = p->many_xf[i];
    CUtensorMap* m = p->many_hmaps + 4 * i;
    memset(m, 0, 4 * sizeof(CUtensorMap));
    void* base = d + t.off * 4;
    CUresult r = CUDA_SUCCESS;
    auto rows_map = [&](CUtensorMap* mm, void* b, int64_t elems, int64_t box_rows) {
      uint64_t dims[2] = {32, (uint64_t)(elems / 32)};
      uint64_t str[1] = {128};
      uint32_t box[2] = {32, (uint32_t)box_rows};
      return encode_tmap(mm, dt, 2, b, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
    };
    if (t.rank == 1 && t.nx <= 2048) {
      continue;  // listed: the buffer-wide maps below
    } else if (t.rank == 1) {
      const int64_t n1 = many_n1(t.nx), n2 = t.nx / n1;
      const int ka = many_kind_a(1, t.nx, 1), kb = many_kind_b(1, t.nx, 1);
      void* sbase = sc + t.soff * 4;
      r = encode_col_load(&m[0], dt, base, n2, 1, 4, many_c(ka), many_r(ka));
      if (r == CUDA_SUCCESS) r = encode_col_store(&m[1], dt, sbase, n2, 1, 4, many_c(ka), many_r(ka));
      if (kb == kMkRowT1) {
        if (r == CUDA_SUCCESS) r = rows_map(&m[2], sbase, t.nx, 256);
        if (r == CUDA_SUCCESS) r = encode_col_store(&m[3], dt, base, n1, 1, 4, many_c(kb), many_r(kb));
      } else {  // 128 rows of 16 R per item; store [N1][k0][q][1] in boxes of 32 columns
        const int R1 = many_r(kb);
        if (r == CUDA_SUCCESS) r = rows_map(&m[2], sbase, t.nx, 64 * R1);
        const uint64_t rowb = (uint64_t)n1 * 4;
        uint64_t dims[4] = {(uint64_t)n1, 16, (uint64_t)R1, 1};
        uint64_t str[3] = {rowb * R1, rowb, rowb * n2};
        uint32_t box[4] = {32, 16, (uint32_t)R1, 1};
        if (r == CUDA_SUCCESS) r = encode_tmap(&m[3], dt, 4, base, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
      }
    } else {
      const int ka = many_kind_a(t.rank, t.nx, t.ny), kb = many_kind_b(t.rank, t.nx, t.ny);
      const int64_t elems = t.nx * t.ny;
      if (ka < 0) {
        // columns only: no pass-A map
      } else if (ka == kMkRow128) {
        r = rows_map(&m[0], base, elems, 256);
      } else {
        const int64_t rows = (int64_t)many_c(ka) * t.ny / 32;
        r = rows_map(&m[0], base, elems, rows < 256 ? rows : 256);
      }
      if (kb == kMkCol128) {  // [128 rows][ny cols], boxes of 32 columns x 128 rows
        uint64_t dims[2] = {(uint64_t)t.ny, 128};
        uint64_t str[1] = {(uint64_t)t.ny * 4};
        uint32_t box[2] = {32, 128};
        if (r == CUDA_SUCCESS) r = encode_tmap(&m[2], dt, 2, base, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
        m[3] = m[2];
      } else {
        if (r == CUDA_SUCCESS) r = encode_col_load(&m[2], dt, base, t.ny, 1, 4, many_c(kb), many_r(kb));
        if (r == CUDA_SUCCESS) r = encode_col_store(&m[3], dt, base, t.ny, 1, 4, many_c(kb), many_r(kb));
      }
    }
    if (r != CUDA_SUCCESS) return r;
  }
  // the whole buffer as rows of 128 bytes, boxes of one listed transform of 256 << i points
  CUtensorMap* bm = p->many_hmaps + 4 * p->many_xf.size();
  for (int i = 0; i < 4; ++i) {
    uint64_t dims[2] = {32, (uint64_t)((p->span_elems + 31) / 32)};
    uint64_t str[1] = {128};
    uint32_t box[2] = {32, (uint32_t)(8 << i)};
    const CUresult r = encode_tmap(&bm[i], dt, 2, d, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
    if (r != CUDA_SUCCESS) return r;
  }
  return CUDA_SUCCESS;
}

tcfftStatus exec_many_pass(tcfftPlanImpl* plan, void* data, cudaStream_t st, int dir) {
  if (plan->many_maps_ptr != data) {
    // the staging copy may still be read by an earlier execute's copy: let it finish first
    if (cuda_status(cudaStreamSynchronize(st), "many maps")) return TCFFT_CUDA_ERROR;
    if (cu_status(encode_many_maps(plan, data), "many maps")) return TCFFT_CUDA_ERROR;
    const size_t bytes = (plan->many_xf.size() + 1) * 4 * sizeof(CUtensorMap);
    if (cuda_status(cudaMemcpyAsync(plan->many_maps, plan->many_hmaps, bytes, cudaMemcpyHostToDevice, st),
                    "many maps"))
      return TCFFT_CUDA_ERROR;
    plan->many_maps_ptr = data;
  }
  ManyParams mp;
  memset(&mp, 0, sizeof mp);
  mp.maps = plan->many_maps;
  mp.row_list = plan->many_rows;
  mp.n_xf = (int)plan->many_xf.size();
  mp.tw2048 = plan->tables.tw2048[dir];
  for (int d = 0; d < 2; ++d) {
    mp.fold8_t[d] = reinterpret_cast<const float2*>(plan->many_fold8 + d * many_fold8_bytes() + many_fold8_t_offset());
    mp.wn3[d] = plan->many_wn3 + 128 * d;
  }
  mp.dir = dir;
  mp.dsign = dir == 0 ? 1.f : -1.f;
  mp.err = plan->tables.err;
  mp.wait_ns = plan->wait_ns;
  // the claim counter and the per-transform completion counters start at zero
  const int64_t ntf = (int64_t)plan->many_xf.size();
  if (cuda_status(cudaMemsetAsync(plan->many_claim, 0, (size_t)(ntf + 1) * sizeof(int), st), "many counters"))
    return TCFFT_CUDA_ERROR;
  if (plan->inject_timeout) {  // test hook: one transform's pass B waits for a count that never comes
    plan->inject_timeout = false;
    if (cuda_status(cudaMemsetAsync(plan->many_claim + plan->many_xf_b, 0x80, sizeof(int), st), "inject"))
      return TCFFT_CUDA_ERROR;
  }
  mp.items = plan->many_items;
  mp.n_items = plan->many_n[0];
  mp.claim = plan->many_claim + ntf;
  mp.done = plan->many_claim;
  if (cuda_status(launch_many(mp, plan->num_sms, st), "many launch")) return TCFFT_CUDA_ERROR;
  return TCFFT_SUCCESS;
}

tcfftStatus exec_many(tcfftPlanImpl* plan, void* data, cudaStream_t st, int dir, int norm) {
  if (plan->many_ok && !norm) return exec_many_pass(plan, data, st, dir);
  if (plan->many_only) return TCFFT_NOT_SUPPORTED;  // no per-shape graph to normalise with
  const int es = plan->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  const int g = 2 * dir + norm;  // one captured graph per direction and normalisation
  if (!plan->graph_exec[g] || plan->graph_ptr[g] != data) {
    if (plan->graph_exec[g]) cudaGraphExecDestroy(plan->graph_exec[g]);
    plan->graph_exec[g] = nullptr;
    plan->graph_ptr[g] = nullptr;
    if (cuda_status(cudaStreamBeginCapture(plan->cap_stream, cudaStreamCaptureModeThreadLocal), "graph capture"))
      return TCFFT_CUDA_ERROR;
    tcfftStatus r = TCFFT_SUCCESS;
    if (plan->mv_n > 0)
      r = cuda_status(launch_move_blocks(data, plan->big, plan->mv_user, plan->mv_big, plan->mv_cum, plan->mv_n,
                                         plan->mv_chunks, plan->num_sms, plan->cap_stream),
                      "gather");
    // runs on branch streams: runs of one sub-plan share its scratch, so they stay on one
    // branch (in order); different sub-plans touch disjoint data and run concurrently
    if (r == TCFFT_SUCCESS) r = cuda_status(cudaEventRecord(plan->fork_ev, plan->cap_stream), "graph fork");
    std::map<const tcfftPlanImpl*, int> branch_of;
    bool used[tcfftPlanImpl::kBranches] = {};
    for (const auto& run : plan->runs) {
      if (r != TCFFT_SUCCESS) break;
      auto ins = branch_of.emplace(run.sub, (int)(branch_of.size() % tcfftPlanImpl::kBranches));
      const int b = ins.first->second;
      if (!used[b]) {
        used[b] = true;
        if (cuda_status(cudaStreamWaitEvent(plan->branch[b], plan->fork_ev, 0), "graph fork")) {
          r = TCFFT_CUDA_ERROR;
          break;
        }
      }
      unsigned char* base = static_cast<unsigned char*>(run.in_big ? plan->big : data);
      r = exec_plan(run.sub, base + run.offset * es, plan->branch[b], dir, norm);
    }
    for (int b = 0; b < tcfftPlanImpl::kBranches; ++b)  // join every forked branch (also after a failure)
      if (used[b] && (cudaEventRecord(plan->join_ev[b], plan->branch[b]) != cudaSuccess ||
                      cudaStreamWaitEvent(plan->cap_stream, plan->join_ev[b], 0) != cudaSuccess))
        r = TCFFT_CUDA_ERROR;
    if (r == TCFFT_SUCCESS && plan->mv_n > 0)
      r = cuda_status(launch_move_blocks(plan->big, data, plan->mv_big, plan->mv_user, plan->mv_cum, plan->mv_n,
                                         plan->mv_chunks, plan->num_sms, plan->cap_stream),
                      "scatter");
    cudaGraph_t gr = nullptr;
    cudaError_t ce = cudaStreamEndCapture(plan->cap_stream, &gr);
    if (r != TCFFT_SUCCESS || ce != cudaSuccess) {
      if (gr) cudaGraphDestroy(gr);
      return r != TCFFT_SUCCESS ? r : cuda_status(ce, "graph capture");
    }
    ce = cudaGraphInstantiate(&plan->graph_exec[g], gr, 0);
    cudaGraphDestroy(gr);
    if (cuda_status(ce, "graph instantiate")) return TCFFT_CUDA_ERROR;
    plan->graph_ptr[g] = data;
  }
  return cuda_status(cudaGraphLaunch(plan->graph_exec[g], st), "graph launch");
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

const char* tcfftVersion(void) { return "tcfft_gb300 0.1 (sm_103a)"; }

const char* tcfftGetErrorString(tcfftStatus s) {
  switch (s) {
    case TCFFT_SUCCESS: return "success";
    case TCFFT_INVALID_VALUE: return "invalid value (null pointer or bad option)";
    case TCFFT_INVALID_SIZE: return "unsupported transform size or batch";
    case TCFFT_MISALIGNED: return "data pointer is not 128-byte aligned";
    case TCFFT_ALLOC_FAILED: return "allocation failed";
    case TCFFT_CUDA_ERROR: return "CUDA error";
    case TCFFT_TIMEOUT: return "device-side bounded wait expired";
    case TCFFT_NOT_SUPPORTED: return "not supported by this build";
    case TCFFT_INVALID_PLAN: return "invalid or destroyed plan";
  }
  return "unknown status";
}

tcfftStatus tcfftOptionsDefault(tcfftOptions* o) {
  if (!o) return TCFFT_INVALID_VALUE;
  memset(o, 0, sizeof(*o));
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftDescribe1d(int64_t n, int64_t batch, int32_t precision, char* buf, size_t len) {
  if (!buf || len == 0) return TCFFT_INVALID_VALUE;
  if (precision != TCFFT_PRECISION_PLAIN && precision != TCFFT_PRECISION_SPLIT &&
      precision != TCFFT_PRECISION_FP32_IO)
    return TCFFT_INVALID_VALUE;
  Schedule s;
  tcfftStatus st = choose_1d(n, batch, precision, s);
  if (st != TCFFT_SUCCESS) return st;
  snprintf(buf, len, "%s", s.text.c_str());
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftDescribe2d(int64_t nx, int64_t ny, int64_t batch, int32_t precision, char* buf, size_t len) {
  if (!buf || len == 0) return TCFFT_INVALID_VALUE;
  if (precision != TCFFT_PRECISION_PLAIN && precision != TCFFT_PRECISION_SPLIT &&
      precision != TCFFT_PRECISION_FP32_IO)
    return TCFFT_INVALID_VALUE;
  Schedule s;
  tcfftStatus st = choose_2d_any(nx, ny, batch, precision, s);
  if (st != TCFFT_SUCCESS) return st;
  snprintf(buf, len, "%s", s.text.c_str());
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftDescribeManyItems(int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                                   const int64_t* offsets, int32_t num_sms, int32_t* items, int64_t capacity,
                                   int64_t* n_items) {
  if (count < 1 || !ranks || !nx || !offsets || !n_items || num_sms < 1 || (capacity > 0 && !items))
    return TCFFT_INVALID_VALUE;
  for (int64_t i = 0; i < count; ++i)
    if ((ranks[i] != 1 && !ny) || ranks[i] < 1 || ranks[i] > 3 || nx[i] < 1 || (ranks[i] >= 2 && ny[i] < 1))
      return TCFFT_INVALID_VALUE;
  std::vector<tcfftPlanImpl::ManyXf> xf;
  std::vector<ManyItem> seq;
  std::vector<int> rows;
  int64_t soff = 0;
  if (!build_many_items(count, ranks, nx, ny ? ny : nx, offsets, num_sms, xf, seq, rows, soff))
    return TCFFT_NOT_SUPPORTED;
  *n_items = (int64_t)seq.size();
  for (int64_t i = 0; i < capacity && i < (int64_t)seq.size(); ++i) {
    const ManyItem& it = seq[(size_t)i];
    int32_t* o = items + 6 * i;
    const int k = it.kind & 0xff;
    o[0] = it.kind;
    o[1] = it.xf;
    o[2] = it.tile;
    o[3] = it.count;
    o[4] = it.nsub;
    o[5] = (it.kind & kMkList) ? it.count * 256 * many_r(k) : it.nsub * many_item_elems(k);
  }
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftPlan1d(tcfftPlan* out, int64_t n, int64_t batch, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  Schedule s;
  st = choose_1d(n, batch, o.precision, s, current_num_sms());
  if (st != TCFFT_SUCCESS) return st;
  std::vector<int> chain = {(int)n};  // natural order reads as a single radix-N digit
  if (o.input_order == TCFFT_ORDER_REFERENCE_DIGIT_REVERSED) {
    chain = reference_radices_1d(n);
    if (chain.empty()) return TCFFT_INVALID_SIZE;  // the reference defines no order for this size
  }
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 1;
  p->n = n;
  p->nx = n;
  p->ny = 1;
  p->batch = batch;
  p->precision = o.precision;
  p->input_order = o.input_order;
  p->direction = o.direction;
  p->normalize = o.normalization;
  p->total_elems = n * batch;
  p->sched = s;
  p->radices_x = chain;
  st = alloc_tables(p);
  const char* cl_env = getenv("TCFFT_CLUSTER");
  int active_clusters = 0;
  if (st == TCFFT_SUCCESS && s.kind == Schedule::kFused1d && cl_env && atoi(cl_env) != 0 &&
      cluster_supported(n, o.precision != TCFFT_PRECISION_PLAIN, p->num_sms, &active_clusters)) {
    // opt-in: clusters of N / 2^14 CTAs, one transform per cluster, no L2 round trip.  Correct at
    // N = 2^15..2^18 but slower than the two-phase kernel (warps waiting at the exchange barriers,
    // bank conflicts of its write-back and row phase: 1.32 against 1.13 ms at 2^15 for 2^28
    // elements, 4.3 against 0.9 ms at 2^18), so the planner does not pick it by itself.
    p->sched = Schedule();
    p->sched.kind = Schedule::kCluster;
    p->sched.N1 = 256;
    p->sched.N2 = n / 256;
    p->sched.launches = 1;
    char buf[160];
    snprintf(buf, sizeof buf, "cluster(plain): N=256 x %lld on %lld CTAs sharing shared memory, %d clusters, one HBM pass",
             (long long)(n / 256), (long long)(n >> 14), active_clusters);
    p->sched.text = buf;
    st = alloc_wn_tables(p, n);
  }
  if (st == TCFFT_SUCCESS && (p->sched.kind == Schedule::kFused1d || p->sched.kind == Schedule::kFused2d))
    st = alloc_fused(p);
  if (st == TCFFT_SUCCESS && s.kind == Schedule::kLarge1d) st = setup_large1d(p);
  if (st == TCFFT_SUCCESS && s.kind == Schedule::kResident) st = alloc_wn_tables(p, n);
  if (st == TCFFT_SUCCESS && o.autotune) st = autotune_plan(p, o);
  if (st == TCFFT_SUCCESS && o.input_order == TCFFT_ORDER_REFERENCE_DIGIT_REVERSED) st = setup_reference_order(p);
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftPlan2d(tcfftPlan* out, int64_t nx, int64_t ny, int64_t batch, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  Schedule s;
  st = choose_2d_any(nx, ny, batch, o.precision, s, current_num_sms());
  if (st != TCFFT_SUCCESS) return st;
  std::vector<int> cx = {(int)nx}, cy = {(int)ny};
  if (o.input_order == TCFFT_ORDER_REFERENCE_DIGIT_REVERSED) {
    cx = reference_radices_2d_axis(nx);
    cy = reference_radices_2d_axis(ny);
    if (cx.empty() || cy.empty()) return TCFFT_INVALID_SIZE;
  }
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 2;
  p->nx = nx;
  p->ny = ny;
  p->n = nx * ny;
  p->batch = batch;
  p->precision = o.precision;
  p->input_order = o.input_order;
  p->direction = o.direction;
  p->normalize = o.normalization;
  p->total_elems = nx * ny * batch;
  p->sched = s;
  p->radices_x = cx;
  p->radices_y = cy;
  st = alloc_tables(p);
  if (st == TCFFT_SUCCESS) st = s.kind == Schedule::kGeneric2d ? setup_generic2d(p) : alloc_fused(p);
  if (st == TCFFT_SUCCESS && o.autotune) st = autotune_plan(p, o);
  if (st == TCFFT_SUCCESS && o.input_order == TCFFT_ORDER_REFERENCE_DIGIT_REVERSED) st = setup_reference_order(p);
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftPlanStrided(tcfftPlan* out, int64_t n, int64_t batch, int64_t istride, int64_t idist,
                             const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  if (batch < 1 || istride < 1 || idist < 1) return TCFFT_INVALID_VALUE;
  if (!is_pow2(n)) return TCFFT_INVALID_SIZE;
  if (istride == 1) {  // batch stride: an uneven-batch plan with offsets b * idist
    if (idist < n) return TCFFT_INVALID_VALUE;
    if (batch > (int64_t)1 << 24) return TCFFT_INVALID_SIZE;
    std::vector<int32_t> r((size_t)batch, 1);
    std::vector<int64_t> x((size_t)batch, n), y((size_t)batch, 1), off((size_t)batch);
    for (int64_t b = 0; b < batch; ++b) off[b] = b * idist;
    tcfftStatus st = tcfftPlanMany(out, batch, r.data(), x.data(), y.data(), off.data(), opts);
    if (st == TCFFT_SUCCESS) {
      char buf[64];
      snprintf(buf, sizeof buf, "strided(idist=%lld) ", (long long)idist);
      (*out)->sched.text = buf + (*out)->sched.text;
    }
    return st;
  }
  // element stride: groups of istride interleaved transforms, each a columns transform
  if (idist != 1 || batch % istride != 0) return TCFFT_NOT_SUPPORTED;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  if (o.precision != TCFFT_PRECISION_PLAIN || o.input_order != TCFFT_ORDER_NATURAL ||
      o.normalization != TCFFT_NORM_NONE)
    return TCFFT_NOT_SUPPORTED;
  const int64_t groups = batch / istride;
  if (many_kind_b(3, n, istride) == kMkKinds || groups > (int64_t)1 << 24 ||
      n * batch > (int64_t(1) << 40))
    return TCFFT_NOT_SUPPORTED;
  std::vector<int32_t> r((size_t)groups, 3);
  std::vector<int64_t> x((size_t)groups, n), y((size_t)groups, istride), off((size_t)groups);
  for (int64_t g = 0; g < groups; ++g) off[g] = g * n * istride;
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 3;
  p->precision = o.precision;
  p->direction = o.direction;
  p->normalize = 0;
  p->batch = groups;
  p->total_elems = n * batch;
  p->span_elems = n * batch;
  p->many_only = true;
  st = alloc_tables(p);
  if (st == TCFFT_SUCCESS && !setup_many_pass(p, groups, r.data(), x.data(), y.data(), off.data()))
    st = TCFFT_NOT_SUPPORTED;
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  p->sched.launches = 1;
  char buf[200];
  snprintf(buf, sizeof buf,
           "strided(plain): %lld transforms of %lld points at stride %lld, one persistent launch of %d "
           "column-FFT items",
           (long long)batch, (long long)n, (long long)istride, p->many_n[0]);
  p->sched.text = buf;
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftPlanMany(tcfftPlan* out, int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                          const int64_t* offsets, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  if (count < 1 || !ranks || !nx || !offsets) return TCFFT_INVALID_VALUE;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  if (o.input_order != TCFFT_ORDER_NATURAL) return TCFFT_INVALID_VALUE;
  const int es = o.precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  std::vector<int64_t> size(count);
  for (int64_t i = 0; i < count; ++i) {
    if (ranks[i] != 1 && ranks[i] != 2) return TCFFT_INVALID_VALUE;
    if (ranks[i] == 2 && !ny) return TCFFT_INVALID_VALUE;
    const int64_t y = ranks[i] == 2 ? ny[i] : 1;
    if (!is_pow2(nx[i]) || !is_pow2(y)) return TCFFT_INVALID_SIZE;
    size[i] = nx[i] * y;
    if (offsets[i] < 0 || (offsets[i] * es) % 128 != 0) return TCFFT_MISALIGNED;
  }
  std::vector<int64_t> order(count);
  for (int64_t i = 0; i < count; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return offsets[a] < offsets[b]; });
  for (int64_t k = 1; k < count; ++k)
    if (offsets[order[k]] < offsets[order[k - 1]] + size[order[k - 1]]) return TCFFT_INVALID_VALUE;  // overlap
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 3;
  p->precision = o.precision;
  p->direction = o.direction;
  p->normalize = o.normalization;
  p->batch = count;
  st = alloc_tables(p);
  tcfftOptions os = o;
  // group by shape (in offset order); a group that is one back-to-back run executes in place,
  // any other group with several members is gathered into `big`, run as one batch, scattered back
  std::map<std::tuple<int, int64_t, int64_t>, std::vector<int64_t>> groups;
  for (int64_t k = 0; k < count; ++k) {
    const int64_t i = order[k];
    groups[std::make_tuple(ranks[i], nx[i], ranks[i] == 2 ? ny[i] : 1)].push_back(i);
  }
  std::map<std::tuple<int, int64_t, int64_t, int64_t>, tcfftPlanImpl*> by_key;
  std::vector<long long> mv_user, mv_big, mv_cum;
  int64_t big_elems = 0;
  long long chunks = 0;
  int launches = 0, nsub = 0;
  for (auto& g : groups) {
    if (st != TCFFT_SUCCESS) break;
    const int r = std::get<0>(g.first);
    const int64_t x = std::get<1>(g.first), y = std::get<2>(g.first), sz = x * y;
    const std::vector<int64_t>& idx = g.second;
    bool contiguous = true;
    for (size_t j = 1; j < idx.size(); ++j) contiguous = contiguous && offsets[idx[j]] == offsets[idx[j - 1]] + sz;
    std::vector<std::pair<int64_t, int64_t>> todo;  // (offset, run length)
    bool in_big = false;
    if (contiguous || idx.size() == 1) {
      todo.push_back({offsets[idx[0]], (int64_t)idx.size()});
    } else {
      in_big = true;
      todo.push_back({big_elems, (int64_t)idx.size()});
      for (size_t j = 0; j < idx.size(); ++j) {
        mv_user.push_back(offsets[idx[j]] * es);
        mv_big.push_back((big_elems + (int64_t)j * sz) * es);
        mv_cum.push_back(chunks);
        chunks += sz * es / 16;
      }
      big_elems += sz * (int64_t)idx.size();
    }
    for (const auto& t : todo) {
      const auto key = std::make_tuple(r, x, y, t.second);
      tcfftPlanImpl* sub = nullptr;
      auto it = by_key.find(key);
      if (it != by_key.end()) {
        sub = it->second;
      } else {
        st = r == 1 ? tcfftPlan1d(&sub, x, t.second, &os) : tcfftPlan2d(&sub, x, y, t.second, &os);
        if (st != TCFFT_SUCCESS) break;
        p->subs.push_back(sub);
        by_key[key] = sub;
        ++nsub;
      }
      p->runs.push_back({sub, t.first, in_big});
      launches += sub->sched.launches;
    }
    p->total_elems += sz * (int64_t)idx.size();
    for (int64_t i : idx) p->span_elems = std::max(p->span_elems, offsets[i] + sz);
  }
  if (st == TCFFT_SUCCESS && !mv_user.empty()) {
    const size_t nb = mv_user.size() * sizeof(long long);
    if (cudaMalloc(&p->big, big_elems * es) != cudaSuccess || cudaMalloc(&p->mv_user, nb) != cudaSuccess ||
        cudaMalloc(&p->mv_big, nb) != cudaSuccess || cudaMalloc(&p->mv_cum, nb) != cudaSuccess)
      st = TCFFT_ALLOC_FAILED;
    else if (cudaMemcpy(p->mv_user, mv_user.data(), nb, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(p->mv_big, mv_big.data(), nb, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(p->mv_cum, mv_cum.data(), nb, cudaMemcpyHostToDevice) != cudaSuccess)
      st = TCFFT_CUDA_ERROR;
    p->mv_n = (int)mv_user.size();
    p->mv_chunks = chunks;
    p->scratch_bytes = big_elems * es;
    launches += 2;
  }
  if (st == TCFFT_SUCCESS && cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
    st = TCFFT_CUDA_ERROR;
  if (st == TCFFT_SUCCESS && cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming) != cudaSuccess)
    st = TCFFT_CUDA_ERROR;
  for (int b = 0; b < tcfftPlanImpl::kBranches && st == TCFFT_SUCCESS; ++b)
    if (cudaStreamCreateWithFlags(&p->branch[b], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->join_ev[b], cudaEventDisableTiming) != cudaSuccess)
      st = TCFFT_CUDA_ERROR;
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  p->sched.launches = launches;
  char buf[200];
  snprintf(buf, sizeof buf, "many(%s): %lld transforms in %d runs (%d gathered), %d sub-plans, %d launches per graph replay",
           prec_name(o.precision), (long long)count, (int)p->runs.size(), p->mv_n,
           nsub, launches);
  p->sched.text = buf;
  if (setup_many_pass(p, count, ranks, nx, ny, offsets)) {
    // the graph stays for normalised executes
    p->sched.launches = 1;
    snprintf(buf, sizeof buf,
             "many(%s): %lld transforms, one persistent many-shape launch of %d work items "
             "(normalised: %d sub-plans in a graph)",
             prec_name(o.precision), (long long)count, p->many_n[0], nsub);
    p->sched.text = buf;
  }
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftExecute(tcfftPlan plan, void* data, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  return exec_plan(plan, data, stream, plan->direction, plan->normalize);
}

tcfftStatus tcfftExecuteOutOfPlace(tcfftPlan plan, const void* in, void* out, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (!in || !out) return TCFFT_INVALID_VALUE;
  return exec_plan(plan, out, stream, plan->direction, plan->normalize, in);
}

tcfftStatus tcfftPlanReal2d(tcfftPlan* out, int64_t nx, int64_t ny, int64_t batch, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  if (o.input_order != TCFFT_ORDER_NATURAL || o.direction != TCFFT_FORWARD) return TCFFT_INVALID_VALUE;
  if (!is_pow2(nx) || !is_pow2(ny) || nx < 16 || ny < 32 || batch < 1 || nx * ny > (int64_t(1) << 40) / batch)
    return TCFFT_INVALID_SIZE;
  const int64_t h = ny / 2 + 1;
  const int es = o.precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 5;
  p->nx = nx;
  p->ny = ny;
  p->n = nx * ny;
  p->batch = batch;
  p->precision = o.precision;
  p->normalize = o.normalization;
  p->total_elems = nx * h * batch;  // complex elements of the half spectrum
  p->sched.kind = Schedule::kNone;
  st = alloc_tables(p);
  // rows: real transforms of ny, carrying the plan's normalisation rule for 1/ny; columns:
  // complex transforms of nx over the h columns of the half spectrum (1/nx on the normalised side)
  tcfftOptions ro = o, co;
  tcfftOptionsDefault(&co);
  co.precision = o.precision;
  co.autotune = o.autotune;
  co.tune_cache_path = o.tune_cache_path;
  tcfftPlan rows = nullptr, cols = nullptr;
  if (st == TCFFT_SUCCESS) st = tcfftPlanReal1d(&rows, ny, nx * batch, &ro);
  if (st == TCFFT_SUCCESS) p->subs.push_back(rows);
  if (st == TCFFT_SUCCESS) st = tcfftPlan1d(&cols, nx, h * batch, &co);
  if (st == TCFFT_SUCCESS) p->subs.push_back(cols);
  // two half-spectrum buffers: [batch][nx][h] and its transpose [batch][h][nx]
  const int64_t half_bytes = ((nx * h * batch * es + 255) / 256) * 256;
  if (st == TCFFT_SUCCESS) {
    p->scratch_bytes = 2 * half_bytes + rows->scratch_bytes + cols->scratch_bytes;
    if (cudaMalloc(&p->big, 2 * half_bytes) != cudaSuccess) st = TCFFT_ALLOC_FAILED;
    p->span_elems = half_bytes;  // byte offset of the second buffer
  }
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  p->sched.launches = rows->sched.launches + cols->sched.launches + 2;
  p->sched.text = "real2d(" + std::string(prec_name(o.precision)) + "): " + std::to_string(nx) + " x " +
                  std::to_string(ny) + ", real rows, transpose, complex columns of " + std::to_string(nx) +
                  ", transpose";
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftPlanReal1d(tcfftPlan* out, int64_t n, int64_t batch, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  tcfftStatus st = validate_opts(opts);
  if (st != TCFFT_SUCCESS) return st;
  tcfftOptions o;
  tcfftOptionsDefault(&o);
  if (opts) o = *opts;
  if (o.input_order != TCFFT_ORDER_NATURAL || o.direction != TCFFT_FORWARD) return TCFFT_INVALID_VALUE;
  if (!is_pow2(n) || n < 32 || n > (int64_t(1) << 27) || batch < 1 || batch > (int64_t(1) << 40) / n)
    return TCFFT_INVALID_SIZE;
  Schedule s;
  st = choose_1d(n / 2, batch, o.precision, s, current_num_sms());  // the half-length complex schedule
  if (st != TCFFT_SUCCESS) return st;
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 4;
  p->n = n;
  p->nx = n;
  p->ny = 1;
  p->batch = batch;
  p->precision = o.precision;
  p->normalize = o.normalization;
  p->total_elems = (n / 2) * batch;  // complex elements of the half-length transforms
  p->sched.kind = Schedule::kNone;
  st = alloc_tables(p);
  if (st == TCFFT_SUCCESS) st = alloc_wn_tables(p, n);
  tcfftOptions so;
  tcfftOptionsDefault(&so);
  so.precision = o.precision;
  so.autotune = o.autotune;
  so.tune_cache_path = o.tune_cache_path;
  tcfftPlan sub = nullptr;
  if (st == TCFFT_SUCCESS) st = tcfftPlan1d(&sub, n / 2, batch, &so);
  if (st == TCFFT_SUCCESS) p->subs.push_back(sub);
  const int es = o.precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  if (st == TCFFT_SUCCESS) {
    p->scratch_bytes = (n / 2) * batch * es + sub->scratch_bytes;
    if (cudaMalloc(&p->big, (n / 2) * batch * es) != cudaSuccess) st = TCFFT_ALLOC_FAILED;
  }
  if (st != TCFFT_SUCCESS) {
    free_tables(p);
    delete p;
    return st;
  }
  p->sched.launches = sub->sched.launches + 1;
  p->sched.text = "real(" + std::string(prec_name(o.precision)) + "): N=" +
                  std::to_string(n) + " as complex " + sub->sched.text.substr(0, 60) + " + Hermitian split pass";
  *out = p;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftExecuteR2C(tcfftPlan plan, const void* in, void* out, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (plan->kind == 5 && in && out) return exec_real2d(plan, in, out, stream, true);
  if (plan->kind != 4 || !in || !out) return TCFFT_INVALID_VALUE;
  if ((reinterpret_cast<uintptr_t>(in) & 127) != 0) return TCFFT_MISALIGNED;
  const int64_t h = plan->n / 2;
  // the real input is the complex sequence x[2m] + i x[2m+1]: its h-point transform into the plan's buffer
  tcfftStatus r = exec_plan(plan->subs[0], plan->big, stream, 0, 0, in);
  if (r != TCFFT_SUCCESS) return r;
  return cuda_status(launch_r2c_post(plan->big, out, plan->batch, h, plan->twlo[0], plan->twhi[0], plan->tw_shift,
                                     plan->normalize ? 1.f / (float)plan->n : 1.f,
                                     plan->precision != TCFFT_PRECISION_PLAIN, plan->num_sms,
                                     reinterpret_cast<cudaStream_t>(stream)),
                     "r2c split pass");
}

tcfftStatus tcfftExecuteC2R(tcfftPlan plan, const void* in, void* out, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (plan->kind == 5 && in && out) return exec_real2d(plan, in, out, stream, false);
  if (plan->kind != 4 || !in || !out) return TCFFT_INVALID_VALUE;
  if ((reinterpret_cast<uintptr_t>(out) & 127) != 0) return TCFFT_MISALIGNED;
  const int64_t h = plan->n / 2;
  // C2R is the inverse of R2C: it carries the 1/n unless R2C does (TCFFT_NORM_BY_N)
  if (cuda_status(launch_c2r_pre(in, out, plan->batch, h, plan->twlo[1], plan->twhi[1], plan->tw_shift,
                                 plan->normalize ? 1.f : 1.f / (float)plan->n,
                                 plan->precision != TCFFT_PRECISION_PLAIN, plan->num_sms,
                                 reinterpret_cast<cudaStream_t>(stream)),
                  "c2r split pass"))
    return TCFFT_CUDA_ERROR;
  return exec_plan(plan->subs[0], out, stream, 1, 0);  // unnormalised inverse of h points
}

tcfftStatus tcfftExecuteHost(tcfftPlan plan, const void* host_in, void* host_out, void* work, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (!host_in || !host_out || !work) return TCFFT_INVALID_VALUE;
  if (plan->kind == 4 || plan->kind == 5) return TCFFT_INVALID_VALUE;  // real plans: R2C / C2R
  if ((reinterpret_cast<uintptr_t>(work) & 127) != 0) return TCFFT_MISALIGNED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int64_t es = plan->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  const int64_t per = plan->kind == 2 ? plan->nx * plan->ny : plan->n;  // elements per transform
  const int64_t total = (plan->kind == 3 ? plan->span_elems : plan->total_elems) * es;
  static const int env_chunks = getenv("TCFFT_HOST_CHUNKS") ? atoi(getenv("TCFFT_HOST_CHUNKS")) : 0;
  const int chunks = env_chunks >= 1 && env_chunks <= tcfftPlanImpl::kHostChunks ? env_chunks : 16;
  const int K = plan->kind == 3 ? 1 : (int)std::min<int64_t>(chunks, plan->batch);
  if (K <= 1) {  // unchunked
    if (cuda_status(cudaMemcpyAsync(work, host_in, total, cudaMemcpyHostToDevice, st), "copy in"))
      return TCFFT_CUDA_ERROR;
    tcfftStatus r = exec_plan(plan, work, stream, plan->direction, plan->normalize);
    if (r != TCFFT_SUCCESS) return r;
    return cuda_status(cudaMemcpyAsync(host_out, work, total, cudaMemcpyDeviceToHost, st), "copy out");
  }
  const int64_t b0 = plan->batch / K, extra = plan->batch % K;  // chunks 0..extra-1 hold b0 + 1
  if (!plan->host_st[0] || plan->host_b0 != b0) {
    for (int i = 0; i < 2; ++i)
      if (plan->host_sub[i]) {
        tcfftDestroy(plan->host_sub[i]);
        plan->host_sub[i] = nullptr;
      }
    tcfftOptions o;
    tcfftOptionsDefault(&o);
    o.precision = plan->precision;
    o.input_order = plan->input_order;
    for (int i = 0; i < 2; ++i) {
      const int64_t b = b0 + i;
      if (b == 0 || (i == 1 && extra == 0)) continue;
      const tcfftStatus r = plan->kind == 2 ? tcfftPlan2d(&plan->host_sub[i], plan->nx, plan->ny, b, &o)
                                            : tcfftPlan1d(&plan->host_sub[i], plan->n, b, &o);
      if (r != TCFFT_SUCCESS) return r;
    }
    plan->host_b0 = b0;
    for (int i = 0; i < 3; ++i)
      if (!plan->host_st[i] && cudaStreamCreateWithFlags(&plan->host_st[i], cudaStreamNonBlocking) != cudaSuccess)
        return TCFFT_CUDA_ERROR;
    for (cudaEvent_t* e : {&plan->host_fork, &plan->host_join[0], &plan->host_join[1]})
      if (!*e && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return TCFFT_CUDA_ERROR;
    for (int c = 0; c < tcfftPlanImpl::kHostChunks; ++c)
      if ((!plan->host_ev_in[c] && cudaEventCreateWithFlags(&plan->host_ev_in[c], cudaEventDisableTiming)) ||
          (!plan->host_ev_fft[c] && cudaEventCreateWithFlags(&plan->host_ev_fft[c], cudaEventDisableTiming)))
        return TCFFT_CUDA_ERROR;
  }
  cudaStream_t sin = plan->host_st[0], sfft = plan->host_st[1], sout = plan->host_st[2];
  if (cuda_status(cudaEventRecord(plan->host_fork, st), "fork")) return TCFFT_CUDA_ERROR;
  for (cudaStream_t x : {sin, sfft, sout})
    if (cuda_status(cudaStreamWaitEvent(x, plan->host_fork, 0), "fork")) return TCFFT_CUDA_ERROR;
  int64_t first = 0;  // first transform of the chunk
  for (int c = 0; c < K; ++c) {
    const int64_t b = b0 + (c < extra ? 1 : 0);
    const int64_t off = first * per * es, bytes = b * per * es;
    unsigned char* dev = static_cast<unsigned char*>(work) + off;
    if (cuda_status(cudaMemcpyAsync(dev, static_cast<const unsigned char*>(host_in) + off, bytes,
                                    cudaMemcpyHostToDevice, sin),
                    "copy in") ||
        cuda_status(cudaEventRecord(plan->host_ev_in[c], sin), "copy in") ||
        cuda_status(cudaStreamWaitEvent(sfft, plan->host_ev_in[c], 0), "copy in"))
      return TCFFT_CUDA_ERROR;
    const tcfftStatus r = exec_plan(plan->host_sub[b == b0 ? 0 : 1], dev, sfft, plan->direction, plan->normalize);
    if (r != TCFFT_SUCCESS) return r;
    if (cuda_status(cudaEventRecord(plan->host_ev_fft[c], sfft), "transform") ||
        cuda_status(cudaStreamWaitEvent(sout, plan->host_ev_fft[c], 0), "transform") ||
        cuda_status(cudaMemcpyAsync(static_cast<unsigned char*>(host_out) + off, dev, bytes, cudaMemcpyDeviceToHost,
                                    sout),
                    "copy out"))
      return TCFFT_CUDA_ERROR;
    first += b;
  }
  // `stream` continues after the last transform and the last copy out
  if (cuda_status(cudaEventRecord(plan->host_join[0], sfft), "join") ||
      cuda_status(cudaEventRecord(plan->host_join[1], sout), "join") ||
      cuda_status(cudaStreamWaitEvent(st, plan->host_join[0], 0), "join") ||
      cuda_status(cudaStreamWaitEvent(st, plan->host_join[1], 0), "join"))
    return TCFFT_CUDA_ERROR;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftExecuteAdjoint(tcfftPlan plan, void* data, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  return exec_plan(plan, data, stream, 1 - plan->direction, plan->normalize);
}

tcfftStatus tcfftExecuteInverse(tcfftPlan plan, void* data, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  return exec_plan(plan, data, stream, 1 - plan->direction, 1 - plan->normalize);
}

tcfftStatus tcfftCheckDevice(tcfftPlan plan, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return TCFFT_CUDA_ERROR;
  return check_errors(plan);
}

tcfftStatus tcfftSetWaitLimit(tcfftPlan plan, int64_t limit_ns) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (limit_ns < 0) return TCFFT_INVALID_VALUE;
  plan->wait_ns = (unsigned long long)limit_ns;
  for (tcfftPlanImpl* sp : plan->subs) tcfftSetWaitLimit(sp, limit_ns);
  for (tcfftPlanImpl* sp : plan->host_sub)
    if (sp) tcfftSetWaitLimit(sp, limit_ns);
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftInjectWaitTimeout(tcfftPlan plan) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  const bool many = plan->kind == 3 && plan->many_ok && plan->many_xf_b >= 0;
  if (plan->sched.kind != Schedule::kFused1d && plan->sched.kind != Schedule::kFused2d && !many)
    return TCFFT_NOT_SUPPORTED;
  plan->inject_timeout = true;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftDestroy(tcfftPlan plan) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  plan->magic = 0;
  free_tables(plan);
  delete plan;
  return TCFFT_SUCCESS;
}

tcfftStatus tcfftGetPlanInfo(tcfftPlan plan, tcfftPlanInfo* info) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (!info) return TCFFT_INVALID_VALUE;
  memset(info, 0, sizeof(*info));
  info->total_elements = plan->total_elems;
  info->element_bytes = plan->precision != TCFFT_PRECISION_PLAIN ? 8 : 4;
  info->launches_per_exec = plan->sched.launches;
  info->scratch_bytes = plan->scratch_bytes;
  info->n_radices = (int)plan->radices_x.size();
  for (int i = 0; i < info->n_radices && i < 16; ++i) info->radices[i] = plan->radices_x[i];
  info->n_radices_y = (int)plan->radices_y.size();
  for (int i = 0; i < info->n_radices_y && i < 16; ++i) info->radices_y[i] = plan->radices_y[i];
  snprintf(info->schedule, sizeof info->schedule, "%s", plan->sched.text.c_str());
  return TCFFT_SUCCESS;
}

}  // extern "C"
