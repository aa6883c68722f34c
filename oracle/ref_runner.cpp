// oracle/ref_runner.cpp -- runs the reference's own GPU kernels on this GPU.
//
// TEST INFRASTRUCTURE ONLY (the parity comparator, never the product).  The
// reference kernels are compiled for sm_103a from the reference's sources into
// oracle/_ref/tcfft_half_ref.cubin and tcfft_half_2d_ref.cubin by
// oracle/build.py (device code only; the cubins carry no host code); this file
// loads them with the driver API and restates the reference's host logic:
//   - the size -> radix/merging table and the 16x16 DFT matrix of tcfftCreate
//     (tcfft_half.cu:1250-1344; 2D tcfft_half_2d.cu:1167-1220), with F in fp16
//     rounded from cosf/-sinf of 2*pi*i*j/16 exactly as the reference computes it;
//   - the launch sequence of tcfftExec (tcfft_half.cu:1177-1233; 2D
//     tcfft_half_2d.cu:1128-1149): block (32, 8), dynamic shared memory
//     RADIX * 4 * n_cont bytes, n_cont = {32, 16, 8} for RADIX {256, 512, 1024}.
// Kernel family 0 is what tcfftCreate binds (the Volta fragment-map kernels,
// tcfft_half.cu:1244-1248); family 1 is the sm_80 fragment-map "_A100" twins
// (instantiated by oracle/ref_kernels.cu), launched with the same geometry.
// Input must already be in the reference's digit-reversed order.
#include <cuda.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

namespace {

struct Module {
  CUmodule mod = nullptr;
  CUfunction l0f[2][3] = {};
  CUfunction l1f[2][2] = {};
  CUfunction* l0 = l0f[0];  // the family in use
  CUfunction* l1 = l1f[0];
  CUdeviceptr F_real = 0, F_imag = 0;
};
std::map<std::string, Module> g_mods;

bool find_kernel(const std::vector<std::string>& names, const char* key, std::string& out) {
  for (const auto& n : names)
    if (n.find(key) != std::string::npos) {
      out = n;
      return true;
    }
  return false;
}

int load(const char* cubin, const char* names_path, Module& m) {
  if (cuInit(0) != CUDA_SUCCESS) return 1;
  CUcontext ctx = nullptr;
  if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || ctx == nullptr) {
    CUdevice dev;
    if (cuDeviceGet(&dev, 0) != CUDA_SUCCESS) return 2;
    if (cuDevicePrimaryCtxRetain(&ctx, dev) != CUDA_SUCCESS) return 3;
    if (cuCtxSetCurrent(ctx) != CUDA_SUCCESS) return 4;
  }
  if (cuModuleLoad(&m.mod, cubin) != CUDA_SUCCESS) return 5;
  std::vector<std::string> names;
  std::ifstream f(names_path);
  for (std::string line; std::getline(f, line);)
    if (!line.empty()) names.push_back(line);
  const char* k0[2][3] = {{"11layer_256_0ILi32ELi8E", "11layer_512_0ILi16ELi8E", "12layer_1024_0ILi8ELi8E"},
                           {"16layer_256_0_A100ILi32ELi8E", "16layer_512_0_A100ILi16ELi8E",
                            "17layer_1024_0_A100ILi8ELi8E"}};
  const char* k1[2][2] = {{"11layer_256_1ILi32ELi8E", "11layer_512_1ILi16ELi8E"},
                          {"16layer_256_1_A100ILi32ELi8E", "16layer_512_1_A100ILi16ELi8E"}};
  for (int f = 0; f < 2; ++f) {
    for (int i = 0; i < 3; ++i) {
      std::string n;
      if (!find_kernel(names, k0[f][i], n) || cuModuleGetFunction(&m.l0f[f][i], m.mod, n.c_str()) != CUDA_SUCCESS)
        return 6;
    }
    for (int i = 0; i < 2; ++i) {
      std::string n;
      if (!find_kernel(names, k1[f][i], n) || cuModuleGetFunction(&m.l1f[f][i], m.mod, n.c_str()) != CUDA_SUCCESS)
        return 7;
    }
  }
  // 16x16 DFT matrix as the reference builds it (tcfft_half.cu:1332-1340)
  std::vector<__half> fr(256), fi(256);
  for (int i = 0; i < 16; ++i)
    for (int j = 0; j < 16; ++j) {
      fr[16 * i + j] = __float2half(cosf(2 * M_PI * i * j / 16));
      fi[16 * i + j] = __float2half(-sinf(2 * M_PI * i * j / 16));
    }
  if (cuMemAlloc(&m.F_real, 512) != CUDA_SUCCESS || cuMemAlloc(&m.F_imag, 512) != CUDA_SUCCESS) return 8;
  if (cuMemcpyHtoD(m.F_real, fr.data(), 512) != CUDA_SUCCESS || cuMemcpyHtoD(m.F_imag, fi.data(), 512) != CUDA_SUCCESS)
    return 9;
  const int n_cont[3] = {32, 16, 8};
  for (int f = 0; f < 2; ++f) {
    for (int i = 0; i < 3; ++i)
      cuFuncSetAttribute(m.l0f[f][i], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (256 << i) * 4 * n_cont[i]);
    for (int i = 0; i < 2; ++i)
      cuFuncSetAttribute(m.l1f[f][i], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (256 << i) * 4 * n_cont[i]);
  }
  return 0;
}

Module* get(const char* cubin, const char* names, int family, int* err) {
  if (family < 0 || family > 1) {
    *err = 10;
    return nullptr;
  }
  Module* m;
  auto it = g_mods.find(cubin);
  if (it != g_mods.end()) {
    m = &it->second;
  } else {
    Module fresh;
    *err = load(cubin, names, fresh);
    if (*err) return nullptr;
    m = &(g_mods[cubin] = fresh);
  }
  m->l0 = m->l0f[family];
  m->l1 = m->l1f[family];
  return m;
}

int launch0(Module& m, int merging, CUdeviceptr data, long long blocks) {
  const int n_cont[3] = {32, 16, 8};
  const int radix = 256 << merging;
  void* args[3] = {&data, &m.F_real, &m.F_imag};
  return cuLaunchKernel(m.l0[merging], (unsigned)blocks, 1, 1, 32, 8, 1, radix * 4 * n_cont[merging], nullptr, args,
                        nullptr) == CUDA_SUCCESS
             ? 0
             : 20;
}
int launch1(Module& m, int merging, int step, CUdeviceptr data, long long bx, long long by) {
  const int n_cont[3] = {32, 16, 8};
  const int radix = 256 << merging;
  if (merging > 1) return 21;  // layer_1[2] is never bound by the reference (tcfft_half.cu:1247-1248)
  void* args[4] = {&step, &data, &m.F_real, &m.F_imag};
  return cuLaunchKernel(m.l1[merging], (unsigned)bx, (unsigned)by, 1, 32, 8, 1, radix * 4 * n_cont[merging], nullptr,
                        args, nullptr) == CUDA_SUCCESS
             ? 0
             : 22;
}

// tcfft_half.cu:1250-1330 (mergings; 0/1/2 = 256/512/1024-point kernels)
bool mergings_1d(int n, std::vector<int>& mg) {
  switch (n) {
    case 256: mg = {0}; return true;
    case 512: mg = {1}; return true;
    case 1024: mg = {2}; return true;
    case 131072: mg = {1, 0}; return true;
    case 262144: mg = {1, 1}; return true;
    case 524288: mg = {2, 1}; return true;
    case 16777216: mg = {0, 0, 0}; return true;
    case 33554432: mg = {1, 0, 0}; return true;
    case 67108864: mg = {1, 1, 0}; return true;
    case 134217728: mg = {1, 1, 1}; return true;
    default: return false;
  }
}

}  // namespace

extern "C" {

// In-place reference FFT of `batch` digit-reversed transforms of length n in
// device memory `data` (half2).  Returns 0 on success.
// sync = 0 leaves the launches queued on the legacy default stream (for timing
// with events); otherwise the call waits for them and reports a fault.
int ref_exec_1d(const char* cubin, const char* names, unsigned long long data, int n, int batch, int family,
                int sync) {
  int err = 0;
  Module* m = get(cubin, names, family, &err);
  if (!m) return 100 + err;
  std::vector<int> mg;
  if (!mergings_1d(n, mg)) return 30;
  const int n_cont[3] = {32, 16, 8};
  long long step = 1;
  int radix = 256 << mg[0];
  if ((long long)n * batch % ((long long)n_cont[mg[0]] * radix) != 0) return 31;  // grid must cover the data
  int r = launch0(*m, mg[0], (CUdeviceptr)data, (long long)n * batch / n_cont[mg[0]] / radix);
  if (r) return r;
  step *= radix;
  for (size_t i = 1; i < mg.size(); ++i) {
    radix = 256 << mg[i];
    r = launch1(*m, mg[i], (int)step, (CUdeviceptr)data, step / n_cont[mg[i]], (long long)batch * n / step / radix);
    if (r) return r;
    step *= radix;
  }
  if (!sync) return 0;
  return cuCtxSynchronize() == CUDA_SUCCESS ? 0 : 40;
}

// 2D reference FFT (tcfft_half_2d.cu:1128-1149): rows of ny, then columns of nx.
int ref_exec_2d(const char* cubin, const char* names, unsigned long long data, int nx, int ny, int batch,
                int family, int sync) {
  int err = 0;
  Module* m = get(cubin, names, family, &err);
  if (!m) return 100 + err;
  auto merging = [](int v) { return v == 256 ? 0 : v == 512 ? 1 : v == 1024 ? 2 : -1; };
  const int m0 = merging(ny), m1 = merging(nx);
  if (m0 < 0 || m1 < 0 || m1 > 1) return 30;  // nx = 1024 needs the unbound layer_1[2]
  const int n_cont[3] = {32, 16, 8};
  if ((long long)nx * ny * batch % ((long long)n_cont[m0] * ny) != 0) return 31;
  int r = launch0(*m, m0, (CUdeviceptr)data, (long long)nx * ny * batch / n_cont[m0] / ny);
  if (r) return r;
  r = launch1(*m, m1, ny, (CUdeviceptr)data, ny / n_cont[m1], (long long)batch * nx * ny / ny / nx);
  if (r) return r;
  if (!sync) return 0;
  return cuCtxSynchronize() == CUDA_SUCCESS ? 0 : 40;
}

}  // extern "C"
