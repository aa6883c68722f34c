// gb300_doit_half_2d.cpp -- the reference's 2D benchmark seam (doit_2d.h:2-4:
// setup_2d / doit_2d / finalize_2d) implemented on this library through the
// compat header include/tcfft_half_2d.h, in place of the reference's
// tcfft_doit_half_2d.cpp, so that speed_2d.cpp / accuracy_2d.cpp run unchanged:
//
//   g++ -I <repo>/include speed_2d.cpp gb300_doit_half_2d.cpp \
//       -L <repo>/tcfft_gb300 -ltcfft_gb300 -lcudart
//
// Data are [batch][nx][ny] complex; each axis is put in the input order its
// radix chain names (natural by default, the reference's digit reversal with
// -DTCFFT_REFERENCE_INPUT_ORDER).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "doit_order.h"
#include "tcfft_half_2d.h"

void setup_2d(double* data, int nx, int ny, int n_batch);
void doit_2d(int iter);
void finalize_2d(double* result);

namespace {
tcfftHandle g_plan;
half* g_host = nullptr;
half* g_dev = nullptr;
size_t g_elems = 0;
bool g_ok = true;

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "gb300_doit_half_2d: %s: %s\n", what, cudaGetErrorString(e));
    g_ok = false;
  }
}
}  // namespace

bool gb300_doit_2d_ok() { return g_ok && g_plan.impl != nullptr; }

void gb300_doit_2d_release() {
  tcfftDestroy(&g_plan);
  if (g_dev) cudaFree(g_dev);
  free(g_host);
  g_dev = nullptr;
  g_host = nullptr;
}

void setup_2d(double* data, int nx, int ny, int n_batch) {
  gb300_doit_2d_release();
  g_ok = true;
  g_elems = (size_t)nx * ny * n_batch;
  tcfftCreate(&g_plan, nx, ny, n_batch);
  if (!g_plan.impl) {
    g_ok = false;
    return;
  }
  std::vector<int> rx, ry;
  tcfft_input_permutation(nx, g_plan.radices_x, g_plan.n_radices_x, rx);
  tcfft_input_permutation(ny, g_plan.radices_y, g_plan.n_radices_y, ry);
  g_host = (half*)malloc(sizeof(half) * 2 * g_elems);
  for (int b = 0; b < n_batch; ++b)
    for (int x = 0; x < nx; ++x)
      for (int y = 0; y < ny; ++y) {
        const size_t dst = ((size_t)b * nx + x) * ny + y, src = ((size_t)b * nx + rx[x]) * ny + ry[y];
        g_host[2 * dst] = __double2half(data[2 * src]);
        g_host[2 * dst + 1] = __double2half(data[2 * src + 1]);
      }
  check(cudaMalloc(&g_dev, sizeof(half) * 2 * g_elems), "cudaMalloc");
  if (g_ok) check(cudaMemcpy(g_dev, g_host, sizeof(half) * 2 * g_elems, cudaMemcpyHostToDevice), "copy in");
}

void doit_2d(int iter) {
  if (!gb300_doit_2d_ok()) return;
  for (int t = 0; t < iter; ++t) tcfftExec(g_plan, g_dev);
  check(cudaDeviceSynchronize(), "doit_2d");
}

void finalize_2d(double* result) {
  if (!gb300_doit_2d_ok()) return;
  check(cudaMemcpy(g_host, g_dev, sizeof(half) * 2 * g_elems, cudaMemcpyDeviceToHost), "copy out");
  for (size_t i = 0; i < 2 * g_elems; ++i) result[i] = __half2float(g_host[i]);
}
