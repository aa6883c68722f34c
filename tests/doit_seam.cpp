// Test wrapper around the shipped harness seam tcfft_gb300/doit/gb300_doit_half.cpp
// (or, with SEAM_2D, gb300_doit_half_2d.cpp): one setup / doit(iters) / finalize
// sequence, called the way the reference's speed.cpp:45-64 calls it, behind an
// extern "C" entry point for the Python test; plus the radix chain the compat
// handle reports and the driver's input permutation, for host-side checks.
// Compiled by tests/test_doit_seam.py together with the seam source.
#ifdef SEAM_2D
#include "tcfft_half_2d.h"
void setup_2d(double* data, int nx, int ny, int n_batch);
void doit_2d(int iter);
void finalize_2d(double* result);
bool gb300_doit_2d_ok();
void gb300_doit_2d_release();
#else
#include "tcfft_half.h"
void setup(double* data, int n, int n_batch);
void doit(int iter);
void finalize(double* result);
bool gb300_doit_ok();
void gb300_doit_release();
#endif
#include "doit_order.h"

extern "C" {

// Returns 0 on success, 1 if the sequence failed (plan creation or a CUDA call).
int seam_run(double* data, int nx, int ny, int batch, int iters, double* result) {
#ifdef SEAM_2D
  setup_2d(data, nx, ny, batch);
  doit_2d(iters);
  finalize_2d(result);
  const bool ok = gb300_doit_2d_ok();
  gb300_doit_2d_release();
#else
  (void)ny;
  setup(data, nx, batch);
  doit(iters);
  finalize(result);
  const bool ok = gb300_doit_ok();
  gb300_doit_release();
#endif
  return ok ? 0 : 1;
}

// The radix chain the compat handle reports (x chain then y chain in 2D).
int seam_radices(int nx, int ny, int batch, int* out, int cap) {
  tcfftHandle h;
  int k = 0;
#ifdef SEAM_2D
  tcfftCreate(&h, nx, ny, batch);
  for (int i = 0; i < h.n_radices_x && k < cap; ++i) out[k++] = h.radices_x[i];
  for (int i = 0; i < h.n_radices_y && k < cap; ++i) out[k++] = h.radices_y[i];
#else
  (void)ny;
  tcfftCreate(&h, nx, batch);
  for (int i = 0; i < h.n_radices && k < cap; ++i) out[k++] = h.radices[i];
#endif
  tcfftDestroy(&h);
  return k;
}

// The seam's input permutation of a radix chain.
void seam_permutation(int n, const int* radices, int m, int* rev) {
  std::vector<int> r;
  tcfft_input_permutation(n, radices, m, r);
  for (int i = 0; i < n; ++i) rev[i] = r[i];
}

}  // extern "C"
