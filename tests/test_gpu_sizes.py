"""GPU parity for the sizes outside the single-pass and fused ranges:

* 1D N = 16..128 (tiny kernel; batches that leave a partial group of 16);
* 1D N = 2^23..2^27 (column pass + row sub-plan + transpose; 2^24..2^27 are
  sizes the reference supports, tcfft_half.cu:1310-1326);
* 2D shapes outside 256..2048 per axis (row plans and transposes; an axis of
  4096 as the resident kernel with transposed output): the 128 x 128 ..
  1024 x 1024 mix of the uneven-batch workload and 4096 x 4096.

Checked against the FP64 oracle on the rounded inputs; at 2^27, where a full
FP64 reference is costly, through size-independent properties (linearity,
Parseval) and exact DFT values at sampled bins."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, to_complex, tol_plain, tol_split, uniform_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 32, 64, 128])
@pytest.mark.parametrize("batch", [1, 37, 1000])
def test_tiny_plain(cuda_device, n, batch):
    xq = quantize(uniform_input((batch, n), seed=n + batch), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        y = run_gpu(p, xq, "plain")
        ya = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_plain(n)
    assert oracle.rel_l2(ya, oracle_1d(xq, adjoint=True)) < tol_plain(n)


@pytest.mark.parametrize("n", [16, 32, 64])
def test_tiny_split(cuda_device, n):
    batch = 53
    xq = quantize(uniform_input((batch, n), seed=5 * n), "split")
    with tc.Plan(n=n, batch=batch, precision="split") as p:
        y = run_gpu(p, xq, "split")
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_split(n)


def test_tiny_split_128_reports_not_supported(cuda_device):
    with pytest.raises(tc.TcfftError, match="NOT_SUPPORTED"):
        tc.Plan(n=128, batch=4, precision="split")


@pytest.mark.parametrize("n,batch", [(1 << 23, 2), (1 << 24, 1)])
def test_large_plain(cuda_device, n, batch):
    xq = quantize(uniform_input((batch, n), seed=11), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        assert "large1d" in p.info["schedule"]
        y = run_gpu(p, xq, "plain")
    err = oracle.rel_l2(y, oracle_1d(xq))
    assert np.isfinite(y).all()
    assert err < tol_plain(n), "n=%d rel-L2 %.3e" % (n, err)


@pytest.mark.parametrize("n", [1 << 21, 1 << 23])
def test_large_split_and_adjoint(cuda_device, n):
    xq = quantize(uniform_input((1, n), seed=12), "split")
    with tc.Plan(n=n, batch=1, precision="split") as p:
        y = run_gpu(p, xq, "split")
        ya = run_gpu(p, xq, "split", adjoint=True)
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_split(n)
    assert oracle.rel_l2(ya, oracle_1d(xq, adjoint=True)) < tol_split(n)


def test_largest_size_properties(cuda_device):
    """N = 2^27 (the reference's largest size): linearity, Parseval and exact
    DFT values at 4 sampled bins."""
    import torch
    n = 1 << 27
    rng = np.random.default_rng(27)
    a = torch.empty(n, 2, dtype=torch.float16, device="cuda").uniform_(-1, 1)
    b = torch.empty(n, 2, dtype=torch.float16, device="cuda").uniform_(-1, 1)
    a *= 0.25
    b *= 0.25
    s = (a.float() + b.float()).half()
    with tc.Plan(n=n, batch=1) as p:
        xa = a.double().cpu().numpy()
        fa, fb, fs = a.clone(), b.clone(), s.clone()
        for t in (fa, fb, fs):
            p.exec(t)
        p.check_device()
    ya, yb, ys = (to_complex(t.double().cpu().numpy()) for t in (fa, fb, fs))
    # linearity: F(a + b) vs F(a) + F(b) (the inputs of the sum rounded to fp16)
    lin = np.linalg.norm(ys - (ya + yb)) / np.linalg.norm(ys)
    assert lin < 3 * tol_plain(n), lin
    # Parseval on a: sum |X|^2 = N sum |x|^2
    xc = to_complex(xa)
    par = abs(np.sum(np.abs(ya) ** 2) / (n * np.sum(np.abs(xc) ** 2)) - 1)
    assert par < 5e-3, par
    # exact DFT at sampled bins (phase index n k mod N in exact integers)
    idx = np.arange(n, dtype=np.int64)
    scale = np.sqrt(np.sum(np.abs(xc) ** 2))  # RMS of |X|
    for k in rng.integers(0, n, size=4):
        ref = np.sum(xc * np.exp(-2j * np.pi * ((idx * int(k)) % n) / n))
        assert abs(ya[k] - ref) < 0.02 * scale, (k, ya[k], ref)


@pytest.mark.parametrize("nx,ny,batch", [(128, 128, 8), (128, 1024, 2), (512, 128, 3), (64, 256, 4),
                                         (1024, 4096, 1), (4096, 256, 2), (4096, 4096, 1)])
def test_generic_2d_plain(cuda_device, nx, ny, batch):
    xq = quantize(uniform_input((batch, nx, ny), seed=nx + ny), "plain")
    with tc.Plan(nx=nx, ny=ny, batch=batch) as p:
        assert "generic2d" in p.info["schedule"]
        y = run_gpu(p, xq, "plain")
        ya = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, oracle_2d(xq)) < tol_plain(nx * ny)
    assert oracle.rel_l2(ya, oracle_2d(xq, adjoint=True)) < tol_plain(nx * ny)


def test_generic_2d_4096_square(cuda_device):
    """4096 x 4096, batch 1 (the 2D configuration the reference cannot plan)."""
    xq = quantize(uniform_input((1, 4096, 4096), seed=1), "plain")
    with tc.Plan(nx=4096, ny=4096, batch=1) as p:
        y = run_gpu(p, xq, "plain")
    err = oracle.rel_l2(y, oracle_2d(xq))
    assert np.isfinite(y).all() and err < tol_plain(4096 * 4096), err


@pytest.mark.parametrize("nx,ny", [(64, 256), (32, 64)])
def test_generic_2d_split(cuda_device, nx, ny):
    xq = quantize(uniform_input((2, nx, ny), seed=3), "split")
    with tc.Plan(nx=nx, ny=ny, batch=2, precision="split") as p:
        y = run_gpu(p, xq, "split")
    assert oracle.rel_l2(y, oracle_2d(xq)) < tol_split(nx * ny)


@pytest.mark.parametrize("n", [2048, 32768])
def test_split_2048_and_short_rows(cuda_device, n):
    """Split precision at N = 2048 (single-pass kernel with two warps per transform,
    each taking four of the eight radix-8 sub-transforms) and 2^15 (512 x 64
    two-phase kernel with radix-4 short rows)."""
    xq = quantize(uniform_input((5, n), seed=21), "split")
    with tc.Plan(n=n, batch=5, precision="split") as p:
        assert ("small(R=8" if n == 2048 else "fused1d") in p.info["schedule"]
        y = run_gpu(p, xq, "split")
        ya = run_gpu(p, xq, "split", adjoint=True)
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_split(n)
    assert oracle.rel_l2(ya, oracle_1d(xq, adjoint=True)) < tol_split(n)
    if n != 2048:
        return
    x2 = quantize(uniform_input((1, 256, 2048), seed=22), "split")
    with tc.Plan(nx=256, ny=2048, batch=1, precision="split") as p:
        y2 = run_gpu(p, x2, "split")
    assert oracle.rel_l2(y2, oracle_2d(x2)) < tol_split(256 * 2048)


@pytest.mark.parametrize("batch", [3, 400])
def test_resident_32768(cuda_device, batch):
    """N = 2^15 plain held whole in one CTA's shared memory (a transform in two
    stages, the output written and stored in two halves): forward and adjoint
    against FP64, with up to three transforms per CTA at batch 400."""
    n = 1 << 15
    xq = quantize(uniform_input((batch, n), seed=batch + 15), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        assert p.info["schedule"].startswith("resident(plain)"), p.info["schedule"]
        y = run_gpu(p, xq, "plain")
        ya = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_plain(n)
    assert oracle.rel_l2(ya, oracle_1d(xq, adjoint=True)) < tol_plain(n)


@pytest.mark.parametrize("many", [False, True])
@pytest.mark.parametrize("n", [1 << 15, 1 << 16, 1 << 17, 1 << 18])
def test_cluster_opt_in(cuda_device, monkeypatch, n, many):
    """The thread-block-cluster kernel (one transform per cluster of N / 2^14
    CTAs, phases exchanged through distributed shared memory), selected with
    TCFFT_CLUSTER=1 where the device can co-schedule the cluster.  `many`: at
    least four transforms per cluster, so that both stages, the receive buffer
    and every per-transform barrier are reused (parities 0 and 1)."""
    monkeypatch.setenv("TCFFT_CLUSTER", "1")
    monkeypatch.setenv("TCFFT_NO_RESIDENT", "1")  # 2^15 plain is resident by default
    cl = n >> 14
    batch = 4 * (152 // cl) + 3 if many else 5
    xq = quantize(uniform_input((batch, n), seed=n % 97 + batch), "plain")
    with tc.Plan(n=n, batch=batch) as p:
        sched = p.info["schedule"]
        y = run_gpu(p, xq, "plain")
        ya = run_gpu(p, xq, "plain", adjoint=True)
    if not sched.startswith("cluster"):
        pytest.skip("cluster of %d CTAs not schedulable here: %s" % (n >> 14, sched))
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_plain(n)
    assert oracle.rel_l2(ya, oracle_1d(xq, adjoint=True)) < tol_plain(n)
