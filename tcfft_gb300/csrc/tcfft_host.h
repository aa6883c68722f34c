// tcfft_host.h -- internal host-side declarations shared by the C-ABI
// implementation (tcfft_api.cu) and the per-kernel launch translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tcfft_gb300.h"

namespace tcfft {

// cuTensorMapEncodeTiled, fetched through the runtime's driver entry point
// (no link-time dependency on libcuda).
CUresult encode_tmap(CUtensorMap* map, CUtensorMapDataType dtype, int rank, void* addr, const uint64_t* dims,
                     const uint64_t* strides_bytes /* rank-1 entries */, const uint32_t* box,
                     CUtensorMapSwizzle swizzle);

struct DeviceTables {
  int device = -1;
  float2* tw2048[2] = {nullptr, nullptr};  // W_2048^j: [0] forward, [1] adjoint
  int* err = nullptr;                      // device error word
};

struct FusedMaps;
struct FusedParams;
// Identifies one instantiation of the two-phase executor (fft_fused.cuh).
struct FusedKey {
  int role0 = 0, R0 = 1, C0 = 16, role1 = 0, R1 = 1, C1 = 16;
  bool split = false;  // 8-byte (float2) elements
  bool io32 = false;   // with split: one fp16 product per stage (fp32 I/O mode) instead of three
  int item_kb = 64;    // work-item size target (KiB): 64 (rings of <= 4 stages) or 32 (<= 8 stages)
};
// kModePlain / kModeSplit / kModeIo32 of a key (fft_common.cuh)
inline int fused_mode(const FusedKey& k) { return k.split ? (k.io32 ? 2 : 1) : 0; }
// Ring shape of one instantiation: stages, tiles per work item in each phase, dynamic shared memory.
struct FusedShape {
  int stages = 0, sub0 = 1, sub1 = 1, smem = 0;
};
int fused_cols(int R, bool split, int max_tile_bytes = 64 * 1024);
cudaError_t launch_fused(const FusedKey& k, const FusedMaps& maps, const FusedParams& p, int num_sms,
                         cudaStream_t st, int* grid_out);
// false if `k` names no compiled instantiation
bool fused_shape(const FusedKey& k, FusedShape* out);
// Tensor maps of the 1D two-phase executor (N = n1 * n2; S scratch slots of N elements);
// phase 0 loads from `in` (nullptr: data), phase 1 stores to data.
CUresult encode_fused1d_maps(FusedMaps* maps, const FusedKey& k, void* data, void* scratch, int64_t n1, int64_t n2,
                             int64_t batch, int S, const void* in = nullptr);

// Short 1D transforms N = 16..128 (fft_tiny.cu); N = 128 is plain only.  mode: kModePlain,
// kModeSplit, kModeIo32 (fft_common.cuh).
bool tiny_supported(int64_t n, int mode);
// oscale: output scale of a launch (a power of two; 1/N for a normalised transform).
// in: the input when out of place (nullptr: in place on data)
cudaError_t launch_tiny(int64_t n, int mode, void* data, int64_t batch, const float2* tw, float dsign, int num_sms,
                        cudaStream_t st, float oscale = 1.f, const void* in = nullptr);
// Batched out-of-place transpose [B][R][C] -> [B][C][R] of es-byte elements (tcfft_transpose.cu).
cudaError_t launch_transpose(const void* in, void* out, int64_t B, int64_t R, int64_t C, int es, int num_sms,
                             cudaStream_t st);

// Copies nblocks variable-size blocks (byte offsets, 16-byte aligned) in one launch (tcfft_gather.cu).
cudaError_t launch_move_blocks(const void* src, void* dst, const long long* src_off, const long long* dst_off,
                               const long long* cum, int nblocks, long long total_chunks, int num_sms,
                               cudaStream_t st);

// Column-tile tensor maps (tcfft_api.cu): rows of `ncols` elements, blocks of 256R rows.
CUresult encode_col_load(CUtensorMap* m, CUtensorMapDataType dt, void* base, int64_t ncols, int64_t nblk, int es,
                         int C, int R);
CUresult encode_col_store(CUtensorMap* m, CUtensorMapDataType dt, void* base, int64_t ncols, int64_t nblk, int es,
                          int C, int R);
// Whole-transform-in-shared-memory kernel, N = 4096, 8192, 16384 plain, 4096 and 8192 split (fft_resident.cu).
bool resident_supported(int64_t n, bool split);
cudaError_t launch_resident(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                            const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st,
                            CUtensorMap* lm, CUtensorMap* sm, bool encode, float oscale = 1.f,
                            const void* in = nullptr);
// fp32 data (8-byte elements): split products, or with io32 one fp16 product per stage
cudaError_t launch_resident_split(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                                  const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st,
                                  CUtensorMap* lm, CUtensorMap* sm, bool encode, float oscale = 1.f,
                                  const void* in = nullptr, bool io32 = false);
bool resident_tout_supported(int64_t n, int64_t batch, int64_t rows);
cudaError_t launch_resident_tout(int64_t n, const void* in, void* out, int64_t batch, int64_t rows,
                                 const float2* tw2048, const float2* twlo, const float2* twhi, float dsign, int* err,
                                 int num_sms, cudaStream_t st, CUtensorMap* lm, CUtensorMap* sm, bool encode,
                                 float oscale = 1.f);

// One transform per thread-block cluster, N = 2^15..2^18 plain (fft_cluster.cu).
bool cluster_supported(int64_t n, bool split, int num_sms, int* active_clusters = nullptr);
cudaError_t launch_cluster(int64_t n, void* data, int64_t batch, const float2* tw2048, const float2* twlo,
                           const float2* twhi, float dsign, int* err, int num_sms, cudaStream_t st, CUtensorMap* lm,
                           CUtensorMap* sm, bool encode, float oscale = 1.f, const void* in = nullptr);

// Launch entry points implemented in the kernel translation units. Each
// returns cudaSuccess or the launch error.
// tmap: tiles loaded; omap: tiles stored (the same map for an in-place transform)
cudaError_t launch_small(int R, int mode, const CUtensorMap& tmap, const CUtensorMap& omap, int64_t total_elems,
                         const float2* tw, float dsign, int* err, int num_sms, cudaStream_t stream, int* launches,
                         float oscale = 1.f);
int small_tile_elems(int R, int mode);

// Real transforms of N = 2h points through complex transforms of h points (tcfft_real.cu):
// Z [batch][h] -> Hermitian half X [batch][h + 1], and back; lo/hi: two-level W_N tables.
cudaError_t launch_r2c_post(const void* z, void* x, int64_t batch, int64_t h, const float2* lo, const float2* hi,
                            int shift, float scale, bool split, int num_sms, cudaStream_t st);
cudaError_t launch_c2r_pre(const void* x, void* z, int64_t batch, int64_t h, const float2* lo, const float2* hi,
                           int shift, float scale, bool split, int num_sms, cudaStream_t st);

// ---------------------------------------------------------------- many-shape executor (fft_many.cu)
// Kinds of work item of the plain-precision executor of tcfftPlanMany: each is one
// tile of one transform's pass (or, for kMkRow* with kMkList, up to C whole 1D
// transforms of 256R points listed in the row list).  Pass A: rows / 1D column
// phase; pass B: 1D row phase / 2D columns, started once the transform's pass-A
// items are complete (one launch, per-transform counters).  Per transform, four tensor maps:
// [0] pass-A load (and in-place store), [1] pass-A store to scratch (1D),
// [2] pass-B load, [3] pass-B store.
enum ManyKind : int {
  kMkRow1 = 0, kMkRow2, kMkRow4, kMkRow8,    // rows of 256R in place, C = 32, 32, 16, 8 rows per item
  kMkColWn1x16, kMkColWn1x32, kMkColWn2x32,  // 1D phase 0: columns of 256R times W_N, to scratch
  kMkRowT1,                                  // 1D phase 1: 32 rows of 256 from scratch, written transposed
  kMkRow16T1, kMkRow16T2, kMkRow16T4,        // 1D phase 1: 128 rows of 16R from scratch, written transposed
  kMkCol1, kMkCol2, kMkCol4, kMkCol8,        // 2D columns of 256R in place, C = 32, 32, 16, 8
  kMkRow128, kMkCol128,                      // 2D axes of 128: 128 rows / 128 columns per item, in place
  kMkKinds
};
constexpr int kMkList = 0x100;  // kind flag: the item's rows are whole transforms from the row list
constexpr int kMkB = 0x200;     // kind flag: a pass-B item; waits until done[xf] reaches `count`
constexpr int kMkRelease = 0x400;  // kind flag: a pass-A item of a transform with a pass B (adds 1 to done[xf])
// kind -> R (points / 256, or / 16 for the 16R kinds), C (rows or columns per item)
__host__ __device__ constexpr int many_r(int kind) {
  return kind == kMkRow1 || kind == kMkColWn1x16 || kind == kMkColWn1x32 || kind == kMkRowT1 ||
                 kind == kMkRow16T1 || kind == kMkCol1
             ? 1
             : kind == kMkRow2 || kind == kMkColWn2x32 || kind == kMkRow16T2 || kind == kMkCol2
                   ? 2
                   : kind == kMkRow4 || kind == kMkRow16T4 || kind == kMkCol4 ? 4 : 8;
}
__host__ __device__ constexpr int many_c(int kind) {
  return kind == kMkRow1 || kind == kMkRow2 || kind == kMkColWn1x32 || kind == kMkColWn2x32 || kind == kMkRowT1 ||
                 kind == kMkCol1 || kind == kMkCol2
             ? 32
             : kind == kMkRow4 || kind == kMkColWn1x16 || kind == kMkCol4
                   ? 16
                   : kind == kMkRow8 || kind == kMkCol8 ? 8 : 128;
}
// elements one item moves
__host__ __device__ constexpr int many_item_elems(int kind) {
  return kind == kMkRow16T1 || kind == kMkRow16T2 || kind == kMkRow16T4 ? 128 * 16 * many_r(kind)
         : kind == kMkRow128 || kind == kMkCol128                       ? 128 * 128
                                                                        : many_c(kind) * 256 * many_r(kind);
}
struct ManyItem {
  int kind;   // ManyKind | kMkList / kMkB / kMkRelease
  int xf;     // transform (maps at 4 xf); listed rows: first row-list entry
  int tile;   // first tile of the transform's pass
  int count;  // listed rows: transforms in the item; kMkB: pass-A items of xf
  int nsub;   // consecutive tiles in the item (one stage holds them side by side)
  int wn;     // kMkColWn*: N - 1 of the transform (its W_N factors come from W_65536)
  int pad[2];
};
struct ManyParams {
  const CUtensorMap* maps;  // [4 per transform], 64-byte aligned, global memory
  const ManyItem* items;
  int n_items;
  int* claim;               // items are claimed in order from this counter (zero at launch)
  int* done;                // per transform: completed pass-A items (zero at launch)
  const int* row_list;      // listed rows: each transform's offset in 128-byte rows of the buffer
  int n_xf;                 // transforms; maps[4 n_xf + i] view the whole buffer as rows of 8 << i rows
                            // of 128 bytes (the listed transforms of 256 << i points)
  const float2* tw2048;     // W_2048^j of the direction
  const float2* fold8_t[2]; // T part of the R = 8 fold table, per direction (many_fold8_init)
  const float2* wn3[2];     // per direction: W_65536^(1024 i) (i < 64), W_65536^(32 i), W_65536^i (i < 32)
  int dir;
  float dsign;
  int* err;
  unsigned long long wait_ns;
};
// One launch over `n_items` work items (grid: one CTA per SM at most).
cudaError_t launch_many(const ManyParams& p, int num_sms, cudaStream_t st);
// Stages of the executor's ring (the host's lag between a transform's two passes).
int many_stages();
// The R = 8 fold table (A and T parts, many_fold8_bytes()) of W_2048 table `tw2048` into
// global memory `out`; the T part starts many_fold8_t_offset() bytes in.
int many_fold8_bytes();
int many_fold8_t_offset();
cudaError_t many_fold8_init(unsigned char* out, const float2* tw2048, cudaStream_t st);

// Reference input-order contract (tcfft_permute.cu).
std::vector<int> reference_radices_1d(int64_t n);
std::vector<int> reference_radices_2d_axis(int64_t n);
std::vector<int> digit_reversal(int64_t n, const std::vector<int>& radices);
cudaError_t to_natural_order(void* data, void* tmp, const int* rev_x, const int* rev_y, int64_t nx, int64_t ny,
                             int64_t batch, int es, int num_sms, cudaStream_t st);
int small_smem_bytes(int R, bool split);

}  // namespace tcfft
