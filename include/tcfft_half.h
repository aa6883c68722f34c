/*
 * tcfft_half.h -- source-compatible replacement for the reference's 1D header
 * (rox906/tcFFT tcfft_half.h:7-21), implemented on the C ABI of
 * tcfft_gb300.h.  Code written against the reference (e.g. its harness
 * tcfft_doit_half.cpp) compiles unchanged:
 *
 *   tcfftHandle plan;  tcfftCreate(&plan, n, n_batch);  tcfftExec(plan, data);
 *
 * Differences, all on the safe side:
 *   - input is in natural order; the handle reports n_radices = 1 and
 *     radices[0] = N, which makes the reference's gen_rev (tcfft_doit_half.cpp:
 *     6-29) the identity, so its host-side permutation becomes a no-op;
 *     define TCFFT_REFERENCE_INPUT_ORDER before including this header to get
 *     the reference's digit-reversed contract and radix chain instead;
 *   - every power of two 16 <= n <= 2^27 works, with batch x n up to 2^40
 *     elements (the reference supports ten sizes from 256 to 2^27 and leaves
 *     others undefined); failures print a message;
 *   - tcfftDestroy releases the plan (the reference leaks it).
 * Like the reference, this header and tcfft_half_2d.h define the same
 * `tcfftHandle` name and cannot be included in one translation unit.
 */
#ifndef TCFFT_HALF_COMPAT_H
#define TCFFT_HALF_COMPAT_H

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <utility>

#include "tcfft_gb300.h"

struct tcfftHandle {
  int N, N_batch;
  int radices[9] = {16, 16, 16, 16, 16, 16, 16, 16, 16};
  int n_radices;
  int mergings[3] = {0, 0, 0};
  int n_mergings;
  tcfftPlan impl = nullptr;
};

inline void tcfftCreate(tcfftHandle* plan, int n, int n_batch) {
  tcfftOptions o;
  tcfftOptionsDefault(&o);
#ifdef TCFFT_REFERENCE_INPUT_ORDER
  o.input_order = TCFFT_ORDER_REFERENCE_DIGIT_REVERSED;
#endif
  plan->N = n;
  plan->N_batch = n_batch;
  plan->impl = nullptr;
  tcfftStatus s = tcfftPlan1d(&plan->impl, n, n_batch, &o);
  if (s != TCFFT_SUCCESS) {
    fprintf(stderr, "tcfftCreate(n=%d, batch=%d): %s\n", n, n_batch, tcfftGetErrorString(s));
    plan->n_radices = 0;
    plan->n_mergings = 0;
    return;
  }
  tcfftPlanInfo info;
  tcfftGetPlanInfo(plan->impl, &info);
  plan->n_radices = info.n_radices > 9 ? 9 : info.n_radices;
  for (int i = 0; i < plan->n_radices; ++i) plan->radices[i] = info.radices[i];
  plan->n_mergings = info.launches_per_exec;
}

inline void tcfftExec(tcfftHandle plan, half* data) {
  tcfftStatus s = tcfftExecute(plan.impl, data, nullptr);
  if (s != TCFFT_SUCCESS) fprintf(stderr, "tcfftExec: %s\n", tcfftGetErrorString(s));
}

inline void tcfftDestroy(tcfftHandle* plan) {
  if (plan->impl) tcfftDestroy(plan->impl);
  plan->impl = nullptr;
}

#endif /* TCFFT_HALF_COMPAT_H */
