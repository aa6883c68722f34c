"""Shared helpers for the parity tests: seeded inputs, running the CUDA path
through the C ABI, and comparing with the FP64 oracle."""
import numpy as np

import oracle

# Tolerances: rel-L2 against the FP64 oracle, per transform size (log2 of the
# elements of one transform, 1D n or 2D nx*ny), 1.5x the largest value
# measured on GB300 at that size over two seeds, forward and adjoint, on the
# rounded and the unrounded inputs (1D and 2D shapes).  Plain: fp16 operands
# and storage with fp32 accumulation (2.4e-4 at N = 16 up to 7.9e-4 at 2^22);
# split: hi/lo fp16 products with fp32 storage (1.2e-7 .. 6.6e-7).  The
# spec bound for the split mode, 1e-5, is far above every entry.
_PLAIN_BOUND = {4: 4.5e-4, 5: 5.4e-4, 6: 5.5e-4, 7: 5.5e-4, 8: 5.6e-4, 9: 6.6e-4, 10: 7.5e-4, 11: 8.6e-4,
                12: 6.7e-4, 13: 7.5e-4, 14: 8.2e-4, 15: 8.9e-4, 16: 7.8e-4, 17: 8.8e-4, 18: 9.0e-4, 19: 9.6e-4,
                20: 1.02e-3, 21: 1.11e-3, 22: 1.19e-3, 23: 1.08e-3, 24: 1.12e-3}
_SPLIT_BOUND = {4: 1.9e-7, 5: 2.2e-7, 6: 2.3e-7, 8: 3.6e-7, 9: 3.7e-7, 10: 3.8e-7, 11: 4.0e-7, 12: 5.3e-7,
                13: 5.4e-7, 14: 5.3e-7, 15: 5.4e-7, 16: 6.7e-7, 17: 6.8e-7, 18: 6.8e-7, 19: 6.8e-7,
                20: 8.3e-7, 21: 8.4e-7, 22: 8.5e-7, 23: 8.6e-7, 24: 9.9e-7}
# sizes beyond the calibration (2^25 .. 2^27): the largest calibrated bound x 1.1
_PLAIN_BEYOND, _SPLIT_BEYOND = 1.3e-3, 1.1e-6
# the bounds the tests used before per-size calibration (kept for mixed-size checks)
TOL_PLAIN = 2.5e-3
TOL_SPLIT = 1e-5


def _lg(size):
    size = int(size)
    assert size > 0 and size & (size - 1) == 0, size
    return size.bit_length() - 1


def tol_plain(size):
    """Plain-precision rel-L2 bound for transforms of `size` elements."""
    return _PLAIN_BOUND.get(_lg(size), _PLAIN_BEYOND)


def tol_split(size):
    """Split-precision rel-L2 bound for transforms of `size` elements."""
    return _SPLIT_BOUND.get(_lg(size), _SPLIT_BEYOND)


def tol(precision, size):
    return tol_plain(size) if precision == "plain" else tol_split(size)


def tol_mixed(precision, sizes):
    """Bound for a batch of mixed sizes: the loosest of their bounds."""
    return max(tol(precision, s) for s in sizes)


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


def run_gpu(plan, x, precision, adjoint=False, device="cuda:0", inverse=False):
    """Copy float64 [..., 2] input to the device in the plan's precision, run
    in place through the C ABI, return complex128 result."""
    import torch
    dt = torch.float16 if precision == "plain" else torch.float32
    t = torch.from_numpy(np.ascontiguousarray(x)).to(dtype=dt).to(device)
    plan.exec(t, adjoint=adjoint, inverse=inverse)
    plan.check_device()
    return to_complex(t.float().cpu().numpy())


def oracle_1d(xq, adjoint=False):
    return oracle.fft_1d(to_complex(xq), sign=+1 if adjoint else -1)


def oracle_2d(xq, adjoint=False):
    return oracle.fft_2d(to_complex(xq), sign=+1 if adjoint else -1)


def tone_input(n, count, seed=0):
    """Three unit-amplitude complex tones (bins and phases from default_rng(seed + 100)) over
    N(0, 1e-3) noise, float64 [count, n, 2]: the size sweep's tone variant; |X_k| ~ n at the
    tone bins, so fp16 output overflows from n ~ 2^16."""
    rng = np.random.default_rng(seed + 100)
    bins = rng.integers(0, n, 3)
    phases = rng.uniform(0, 2 * np.pi, 3)
    idx = np.arange(n)
    z = sum(np.exp(1j * (2 * np.pi * ((int(k) * idx) % n) / n + ph)) for k, ph in zip(bins, phases))
    x = np.empty((count, n, 2))
    noise = rng.normal(0.0, 1e-3, (count, n, 2))
    x[..., 0] = z.real + noise[..., 0]
    x[..., 1] = z.imag + noise[..., 1]
    return x
