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
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "tcfft_host.h"
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

}  // namespace tcfft

using namespace tcfft;

// ------------------------------------------------------------------ helpers
namespace {

bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

tcfftStatus cuda_status(cudaError_t e) { return e == cudaSuccess ? TCFFT_SUCCESS : TCFFT_CUDA_ERROR; }

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
  p->tables = DeviceTables();
  p->scratch = nullptr;
}

// Host-only schedule selection for a 1D size (no CUDA calls).
tcfftStatus choose_1d(int64_t n, int64_t batch, int precision, Schedule& s) {
  if (!is_pow2(n) || n < 256 || n > (int64_t(1) << 27)) return TCFFT_INVALID_SIZE;
  if (batch < 1 || batch > (int64_t(1) << 40) / n) return TCFFT_INVALID_SIZE;
  const bool split = precision == TCFFT_PRECISION_SPLIT;
  s = Schedule();
  if (n <= 2048 && !(split && n == 2048)) {
    s.kind = Schedule::kSmall;
    s.R = (int)(n / 256);
    s.launches = 1;
    char buf[96];
    snprintf(buf, sizeof buf, "small(R=%d,%s): 1 pass, 2 mma stages + radix-%d", s.R, split ? "split" : "plain", s.R);
    s.text = buf;
    return TCFFT_SUCCESS;
  }
  return TCFFT_NOT_SUPPORTED;
}

tcfftStatus validate_opts(const tcfftOptions* o) {
  if (!o) return TCFFT_SUCCESS;
  if (o->precision != TCFFT_PRECISION_PLAIN && o->precision != TCFFT_PRECISION_SPLIT) return TCFFT_INVALID_VALUE;
  if (o->input_order != TCFFT_ORDER_NATURAL && o->input_order != TCFFT_ORDER_REFERENCE_DIGIT_REVERSED)
    return TCFFT_INVALID_VALUE;
  return TCFFT_SUCCESS;
}

tcfftStatus exec_plan(tcfftPlan plan, void* data, void* stream, int dir) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  if (!data) return TCFFT_INVALID_VALUE;
  if ((reinterpret_cast<uintptr_t>(data) & 127) != 0) return TCFFT_MISALIGNED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const bool split = plan->precision == TCFFT_PRECISION_SPLIT;
  const float2* tw = plan->tables.tw2048[dir];
  const float dsign = dir == 0 ? 1.f : -1.f;
  const Schedule& s = plan->sched;
  if (s.kind == Schedule::kSmall) {
    // 2D view of the whole batch: rows of 128 bytes
    const int es = split ? 8 : 4, er = 128 / es;
    const uint64_t rows = (uint64_t)plan->total_elems / er;
    if (plan->tmap_ptr != data || plan->tmap_dir_kind != 0) {
      uint64_t dims[2] = {(uint64_t)er, rows};
      uint64_t strides[1] = {128};
      uint32_t box[2] = {(uint32_t)er, 256};
      CUresult r = encode_tmap(&plan->tmap0, split ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32,
                               2, data, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
      if (r != CUDA_SUCCESS) return TCFFT_CUDA_ERROR;
      plan->tmap_ptr = data;
      plan->tmap_dir_kind = 0;
    }
    int launches = 0;
    return cuda_status(launch_small(s.R, split, plan->tmap0, plan->total_elems, tw, dsign, plan->tables.err,
                                    plan->num_sms, st, &launches));
  }
  return TCFFT_NOT_SUPPORTED;
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
  if (precision != TCFFT_PRECISION_PLAIN && precision != TCFFT_PRECISION_SPLIT) return TCFFT_INVALID_VALUE;
  Schedule s;
  tcfftStatus st = choose_1d(n, batch, precision, s);
  if (st != TCFFT_SUCCESS) return st;
  snprintf(buf, len, "%s", s.text.c_str());
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
  st = choose_1d(n, batch, o.precision, s);
  if (st != TCFFT_SUCCESS) return st;
  if (o.input_order == TCFFT_ORDER_REFERENCE_DIGIT_REVERSED) return TCFFT_NOT_SUPPORTED;
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return TCFFT_ALLOC_FAILED;
  p->kind = 1;
  p->n = n;
  p->nx = n;
  p->ny = 1;
  p->batch = batch;
  p->precision = o.precision;
  p->input_order = o.input_order;
  p->total_elems = n * batch;
  p->sched = s;
  st = alloc_tables(p);
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
  (void)nx;
  (void)ny;
  (void)batch;
  (void)opts;
  return TCFFT_NOT_SUPPORTED;
}

tcfftStatus tcfftPlanMany(tcfftPlan* out, int64_t count, const int32_t* ranks, const int64_t* nx, const int64_t* ny,
                          const int64_t* offsets, const tcfftOptions* opts) {
  if (!out) return TCFFT_INVALID_VALUE;
  *out = nullptr;
  (void)count;
  (void)ranks;
  (void)nx;
  (void)ny;
  (void)offsets;
  (void)opts;
  return TCFFT_NOT_SUPPORTED;
}

tcfftStatus tcfftExecute(tcfftPlan plan, void* data, void* stream) { return exec_plan(plan, data, stream, 0); }

tcfftStatus tcfftExecuteAdjoint(tcfftPlan plan, void* data, void* stream) {
  return exec_plan(plan, data, stream, 1);
}

tcfftStatus tcfftCheckDevice(tcfftPlan plan, void* stream) {
  if (!plan || plan->magic != tcfftPlanImpl::kMagic) return TCFFT_INVALID_PLAN;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return TCFFT_CUDA_ERROR;
  int e = 0;
  if (cudaMemcpy(&e, plan->tables.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return TCFFT_CUDA_ERROR;
  if (e != 0) {
    cudaMemset(plan->tables.err, 0, sizeof(int));
    return TCFFT_TIMEOUT;
  }
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
  info->element_bytes = plan->precision == TCFFT_PRECISION_SPLIT ? 8 : 4;
  info->launches_per_exec = plan->sched.launches;
  info->scratch_bytes = plan->scratch_bytes;
  snprintf(info->schedule, sizeof info->schedule, "%s", plan->sched.text.c_str());
  return TCFFT_SUCCESS;
}

}  // extern "C"
