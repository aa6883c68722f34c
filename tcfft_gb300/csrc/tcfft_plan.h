// tcfft_plan.h -- the opaque plan object behind `tcfftPlan`.
#pragma once
#include <string>

#include "tcfft_host.h"

namespace tcfft {

// Execution schedule chosen at plan time.
struct Schedule {
  enum Kind { kNone = 0, kSmall = 1 } kind = kNone;
  int R = 1;          // small: radix of the tail (N = 256 R)
  int launches = 0;   // kernel launches per execute
  std::string text;   // human-readable description
};

}  // namespace tcfft

struct tcfftPlanImpl {
  static constexpr uint32_t kMagic = 0x7cff7600u;
  uint32_t magic = kMagic;
  int kind = 0;  // 1: 1D, 2: 2D, 3: many
  int64_t n = 0, nx = 0, ny = 0, batch = 0;
  int precision = 0, input_order = 0;
  int device = -1, num_sms = 0;
  int64_t total_elems = 0;
  tcfft::Schedule sched;
  tcfft::DeviceTables tables;
  void* scratch = nullptr;
  int64_t scratch_bytes = 0;
  // tensor maps encoded for the last data pointer
  void* tmap_ptr = nullptr;
  int tmap_dir_kind = -1;
  CUtensorMap tmap0;
};
