/*
 * tcfft_half_2d.h -- source-compatible replacement for the reference's 2D
 * header (rox906/tcFFT tcfft_half_2d.h:7-21) on the C ABI of tcfft_gb300.h:
 *
 *   tcfftHandle plan;  tcfftCreate(&plan, nx, ny, n_batch);  tcfftExec(plan, data);
 *
 * data is [n_batch][nx][ny] interleaved half complex on the device.  Natural
 * input order (radices_x = {nx}, radices_y = {ny} make the reference's
 * gen_rev the identity) unless TCFFT_REFERENCE_INPUT_ORDER is defined; all
 * power-of-two axes 256..2048 work (the reference breaks for nx = 1024,
 * tcfft_half_2d.cu:1178-1182).  Mutually exclusive with tcfft_half.h.
 */
#ifndef TCFFT_HALF_2D_COMPAT_H
#define TCFFT_HALF_2D_COMPAT_H

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <utility>

#include "tcfft_gb300.h"

struct tcfftHandle {
  int Nx, Ny, N_batch;
  int radices_x[3] = {16, 16, 2};
  int radices_y[3] = {16, 16, 2};
  int n_radices_x, n_radices_y;
  int mergings[2] = {0, 0};
  tcfftPlan impl = nullptr;
};

inline void tcfftCreate(tcfftHandle* plan, int nx, int ny, int n_batch) {
  tcfftOptions o;
  tcfftOptionsDefault(&o);
#ifdef TCFFT_REFERENCE_INPUT_ORDER
  o.input_order = TCFFT_ORDER_REFERENCE_DIGIT_REVERSED;
#endif
  plan->Nx = nx;
  plan->Ny = ny;
  plan->N_batch = n_batch;
  plan->impl = nullptr;
  tcfftStatus s = tcfftPlan2d(&plan->impl, nx, ny, n_batch, &o);
  if (s != TCFFT_SUCCESS) {
    fprintf(stderr, "tcfftCreate(nx=%d, ny=%d, batch=%d): %s\n", nx, ny, n_batch, tcfftGetErrorString(s));
    plan->n_radices_x = plan->n_radices_y = 0;
    return;
  }
  tcfftPlanInfo info;
  tcfftGetPlanInfo(plan->impl, &info);
  plan->n_radices_x = info.n_radices > 3 ? 3 : info.n_radices;
  for (int i = 0; i < plan->n_radices_x; ++i) plan->radices_x[i] = info.radices[i];
  plan->n_radices_y = info.n_radices_y > 3 ? 3 : info.n_radices_y;
  for (int i = 0; i < plan->n_radices_y; ++i) plan->radices_y[i] = info.radices_y[i];
}

inline void tcfftExec(tcfftHandle plan, half* data) {
  tcfftStatus s = tcfftExecute(plan.impl, data, nullptr);
  if (s != TCFFT_SUCCESS) fprintf(stderr, "tcfftExec: %s\n", tcfftGetErrorString(s));
}

inline void tcfftDestroy(tcfftHandle* plan) {
  if (plan->impl) tcfftDestroy(plan->impl);
  plan->impl = nullptr;
}

#endif /* TCFFT_HALF_2D_COMPAT_H */
