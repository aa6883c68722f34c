// doit_order.h -- input-order permutation used by the setup() of the
// gb300_doit_half*.cpp harness implementations.
#pragma once
#include <vector>

// Input-order permutation of a mixed-radix chain (the reference's input contract,
// tcfft_doit_half.cpp:6-29): position p of the device buffer holds data index
// rev[p].  The chain's last radix splits the whole transform into its residue
// classes first (digit k of p, most significant, becomes the least significant
// digit of the index), the next one each class, and so on down to radices[0].
// A chain of one radix N is the identity (natural order).
inline void tcfft_input_permutation(int n, const int* radices, int m, std::vector<int>& rev) {
  rev.assign(n, 0);
  for (int p = 0; p < n; ++p) {
    int rest = p, block = n, index = 0, stride = 1;
    for (int i = m - 1; i >= 0; --i) {
      const int r = radices[i], sub = block / r;
      index += (rest / sub) * stride;
      rest %= sub;
      stride *= r;
      block = sub;
    }
    rev[p] = index + rest * stride;
  }
}
