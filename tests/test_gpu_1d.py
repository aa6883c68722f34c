"""GPU parity: 1D batched FFT through the C ABI vs the FP64 oracle
(the reference's accuracy procedure, accuracy.cpp:43-81, with our oracle in
place of FFTW)."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, quantize, run_gpu, tol_plain, tol_split, uniform_input

pytestmark = pytest.mark.gpu

SMALL = [256, 512, 1024, 2048]


@pytest.mark.parametrize("n", SMALL)
@pytest.mark.parametrize("batch", [1, 3, 64, 257])
def test_plain_small(cuda_device, n, batch):
    x = uniform_input((batch, n), seed=n + batch)
    xq = quantize(x, "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain")
    ref = oracle_1d(xq)
    err = oracle.rel_l2(y, ref)
    assert np.isfinite(y).all()
    assert err < tol_plain(n), "n=%d batch=%d rel-L2 %.3e" % (n, batch, err)
    # per-transform error stays uniform (no transform left untouched, cf. the
    # reference's integer grid division tcfft_half.cu:1206)
    per = np.linalg.norm(y - ref, axis=-1) / np.linalg.norm(ref, axis=-1)
    assert per.max() < 3 * tol_plain(n)


@pytest.mark.parametrize("n", [256, 512, 1024])
@pytest.mark.parametrize("batch", [1, 5, 64])
def test_split_small(cuda_device, n, batch):
    x = uniform_input((batch, n), seed=7 * n + batch)
    xq = quantize(x, "split")
    with tc.Plan(n=n, batch=batch, precision="split") as p:
        y = run_gpu(p, xq, "split")
    err = oracle.rel_l2(y, oracle_1d(xq))
    assert err < tol_split(n), "n=%d batch=%d rel-L2 %.3e" % (n, batch, err)


@pytest.mark.parametrize("n", SMALL)
def test_adjoint_small(cuda_device, n):
    batch = 16
    x = uniform_input((batch, n), seed=3 * n)
    xq = quantize(x, "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain", adjoint=True)
    err = oracle.rel_l2(y, oracle_1d(xq, adjoint=True))
    assert err < tol_plain(n)


@pytest.mark.parametrize("n", SMALL)
def test_known_answers(cuda_device, n):
    """impulse -> all ones; DC -> N * delta_0; single tone -> N * delta_k."""
    batch = 3
    x = np.zeros((batch, n, 2))
    x[0, 0, 0] = 1.0               # impulse
    x[1, :, 0] = 1.0 / 16          # DC (scaled to stay in fp16 range)
    k0 = n // 3
    ang = 2 * np.pi * k0 * np.arange(n) / n
    x[2, :, 0] = np.cos(ang) / 16  # tone at bin k0
    x[2, :, 1] = np.sin(ang) / 16
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, quantize(x, "plain"), "plain")
    assert np.allclose(y[0], 1.0, atol=2e-3)
    dc = np.zeros(n, complex)
    dc[0] = n / 16
    assert np.abs(y[1] - dc).max() < 2e-3 * n / 16
    tone = np.zeros(n, complex)
    tone[k0] = n / 16
    assert np.abs(y[2] - tone).max() < 4e-3 * n / 16


def test_linearity_and_parseval(cuda_device):
    n, batch = 1024, 8
    a = quantize(uniform_input((batch, n), 11) * 0.5, "split")
    b = quantize(uniform_input((batch, n), 12) * 0.5, "split")
    with tc.Plan(n=n, batch=batch, precision="split") as p:
        fa = run_gpu(p, a, "split")
        fb = run_gpu(p, b, "split")
        fab = run_gpu(p, a + b, "split")
    assert oracle.rel_l2(fab, fa + fb) < 1e-5
    ta = a[..., 0] + 1j * a[..., 1]
    assert abs(np.sum(np.abs(fa) ** 2) / (n * np.sum(np.abs(ta) ** 2)) - 1) < 1e-5


LARGE = [1 << 12, 1 << 13, 1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 19, 1 << 20, 1 << 21, 1 << 22]


@pytest.mark.parametrize("n", LARGE)
@pytest.mark.parametrize("batch", [1, 3])
def test_plain_large(cuda_device, n, batch):
    x = uniform_input((batch, n), seed=n % 1000 + batch)
    xq = quantize(x, "plain")
    with tc.Plan(n=n, batch=batch) as p:
        sched = p.info["schedule"]
        assert sched.startswith("resident" if 4096 <= n <= 32768 else "fused1d"), sched
        y = run_gpu(p, xq, "plain")
    ref = oracle_1d(xq)
    assert np.isfinite(y).all()
    err = oracle.rel_l2(y, ref)
    assert err < tol_plain(n), "n=%d batch=%d rel-L2 %.3e" % (n, batch, err)


@pytest.mark.parametrize("n", [1 << 12, 1 << 14, 1 << 16, 1 << 18, 1 << 20])
def test_split_large(cuda_device, n):
    batch = 2
    x = uniform_input((batch, n), seed=n % 997)
    xq = quantize(x, "split")
    with tc.Plan(n=n, batch=batch, precision="split") as p:
        y = run_gpu(p, xq, "split")
    err = oracle.rel_l2(y, oracle_1d(xq))
    assert err < tol_split(n), "n=%d rel-L2 %.3e" % (n, err)


@pytest.mark.parametrize("n", [1 << 16, 1 << 20])
def test_adjoint_large(cuda_device, n):
    batch = 2
    xq = quantize(uniform_input((batch, n), seed=5), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, oracle_1d(xq, adjoint=True)) < tol_plain(n)


def test_large_batch_many_waves(cuda_device):
    """More transforms than scratch slots: the slot ring is reused many times."""
    n, batch = 1 << 16, 100
    xq = quantize(uniform_input((batch, n), seed=77), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain")
    ref = oracle_1d(xq)
    per = np.linalg.norm(y - ref, axis=-1) / np.linalg.norm(ref, axis=-1)
    assert per.max() < 1.5 * tol_plain(n)


def test_config1_n4096_batch64(cuda_device):
    """N=4096 (16^3), batch 64, seed 0: the reference's CPU-runnable configuration."""
    n, batch = 4096, 64
    x = uniform_input((batch, n), seed=0)
    xq = quantize(x, "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain")
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_plain(n)
    # error against the unrounded FP64 inputs includes fp16 input quantisation
    assert oracle.rel_l2(y, oracle_1d(x)) < tol_plain(n)
