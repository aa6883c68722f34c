// gb300_doit_half.cpp -- the reference's benchmark seam (doit.h:2-4: setup /
// doit / finalize) implemented on this library through the compat header
// include/tcfft_half.h, so that the reference's drivers (speed.cpp, accuracy.cpp)
// run unchanged against it:
//
//   g++ -I <repo>/include speed.cpp gb300_doit_half.cpp -L <repo>/tcfft_gb300 \
//       -ltcfft_gb300 -lcudart
//
// In place of the reference's tcfft_doit_half.cpp.  setup plans the transform,
// converts the caller's double data to half2 in the input order the handle
// reports (natural order by default; the reference's digit reversal when built
// with -DTCFFT_REFERENCE_INPUT_ORDER, which the library undoes on the GPU) and
// copies it to the device; doit runs tcfftExec `iter` times and synchronises;
// finalize copies the natural-order result back into doubles.  doit.h itself is
// not included: it defines generate_data, which the driver already compiles.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "doit_order.h"
#include "tcfft_half.h"

void setup(double* data, int n, int n_batch);
void doit(int iter);
void finalize(double* result);

namespace {
tcfftHandle g_plan;
half* g_host = nullptr;
half* g_dev = nullptr;
size_t g_elems = 0;
bool g_ok = true;

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "gb300_doit_half: %s: %s\n", what, cudaGetErrorString(e));
    g_ok = false;
  }
}
}  // namespace

// Status of the last setup / doit / finalize sequence: false after a failed CUDA
// call or plan creation (the reference's interface returns nothing).
bool gb300_doit_ok() { return g_ok && g_plan.impl != nullptr; }

void gb300_doit_release() {
  tcfftDestroy(&g_plan);
  if (g_dev) cudaFree(g_dev);
  free(g_host);
  g_dev = nullptr;
  g_host = nullptr;
}

void setup(double* data, int n, int n_batch) {
  gb300_doit_release();
  g_ok = true;
  g_elems = (size_t)n * n_batch;
  tcfftCreate(&g_plan, n, n_batch);
  if (!g_plan.impl) {
    g_ok = false;
    return;
  }
  std::vector<int> rev;
  tcfft_input_permutation(n, g_plan.radices, g_plan.n_radices, rev);
  g_host = (half*)malloc(sizeof(half) * 2 * g_elems);
  for (int b = 0; b < n_batch; ++b)
    for (int i = 0; i < n; ++i) {
      const size_t dst = (size_t)b * n + i, src = (size_t)b * n + rev[i];
      g_host[2 * dst] = __double2half(data[2 * src]);
      g_host[2 * dst + 1] = __double2half(data[2 * src + 1]);
    }
  check(cudaMalloc(&g_dev, sizeof(half) * 2 * g_elems), "cudaMalloc");
  if (g_ok) check(cudaMemcpy(g_dev, g_host, sizeof(half) * 2 * g_elems, cudaMemcpyHostToDevice), "copy in");
}

void doit(int iter) {
  if (!gb300_doit_ok()) return;
  for (int t = 0; t < iter; ++t) tcfftExec(g_plan, g_dev);
  check(cudaDeviceSynchronize(), "doit");
}

void finalize(double* result) {
  if (!gb300_doit_ok()) return;
  check(cudaMemcpy(g_host, g_dev, sizeof(half) * 2 * g_elems, cudaMemcpyDeviceToHost), "copy out");
  for (size_t i = 0; i < 2 * g_elems; ++i) result[i] = __half2float(g_host[i]);
}
