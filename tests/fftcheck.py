"""Shared helpers for the parity tests: seeded inputs, running the CUDA path
through the C ABI, and comparing with the FP64 oracle."""
import numpy as np

import oracle

# Tolerances (rel-L2 against the FP64 oracle evaluated on the same rounded
# inputs the kernel sees).  Plain: fp16 operands/storage with fp32 accumulate
# gives ~3e-4 per rounding step; split: hi/lo fp16 products, fp32 storage.
TOL_PLAIN = 2.5e-3
TOL_SPLIT = 1e-5


def uniform_input(shape, seed):
    """real, imag iid uniform[-1, 1) in float64 (numpy PCG64, the benchmark workloads' distribution)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, tuple(shape) + (2,))


def to_complex(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def quantize(x, precision):
    """The values the kernel actually receives."""
    dt = np.float16 if precision == "plain" else np.float32
    return np.asarray(x).astype(dt).astype(np.float64)


def run_gpu(plan, x, precision, adjoint=False, device="cuda:0"):
    """Copy float64 [..., 2] input to the device in the plan's precision, run
    in place through the C ABI, return complex128 result."""
    import torch
    dt = torch.float16 if precision == "plain" else torch.float32
    t = torch.from_numpy(np.ascontiguousarray(x)).to(dtype=dt).to(device)
    plan.exec(t, adjoint=adjoint)
    plan.check_device()
    return to_complex(t.float().cpu().numpy())


def oracle_1d(xq, adjoint=False):
    return oracle.fft_1d(to_complex(xq), sign=+1 if adjoint else -1)


def oracle_2d(xq, adjoint=False):
    return oracle.fft_2d(to_complex(xq), sign=+1 if adjoint else -1)
