"""GPU: differentiation through the adjoint kernel (torch.autograd.Function)
for loss = sum_k w_k |FFT(x)_k|^2 (w ~ U[0,1), seed 3), checked against the
FP64 analytic gradient 2 F^H (w * F x) (numpy pocketfft stands in for FFTW)
and against central finite differences of the GPU loss.

The plain precision stores the gradient in fp16, whose range ends at 65504:
its weights are scaled by 1/N (N = points per transform), which keeps the
gradient near |x| instead of near N |x|."""
import numpy as np
import pytest
import torch

from fftcheck import quantize, uniform_input
import tcfft_gb300.autograd as ag

pytestmark = pytest.mark.gpu


def loss_fn(y, w):
    yf = y.float()
    return (w * (yf[..., 0] ** 2 + yf[..., 1] ** 2)).sum()


def fp64_grad(xq, w, ndim):
    x = xq[..., 0] + 1j * xq[..., 1]
    if ndim == 1:
        X = np.fft.fft(x, axis=-1)
        g = np.fft.ifft(2 * w * X, axis=-1) * x.shape[-1]
    else:
        X = np.fft.fft2(x)
        g = np.fft.ifft2(2 * w * X) * (x.shape[-1] * x.shape[-2])
    return np.stack([g.real, g.imag], axis=-1)


@pytest.mark.parametrize("precision,batch,n,tol", [("split", 256, 16384, 1e-5), ("plain", 64, 16384, 3e-3),
                                                   ("split", 8, 4096, 1e-5)])
def test_grad_1d(cuda_device, precision, batch, n, tol):
    xq = quantize(uniform_input((batch, n), seed=5), precision)
    w = np.random.default_rng(3).uniform(0, 1, (batch, n))
    if precision == "plain":
        w /= n
    dt = torch.float16 if precision == "plain" else torch.float32
    x = torch.from_numpy(xq).to(dt).to(cuda_device).requires_grad_(True)
    wt = torch.from_numpy(w).float().to(cuda_device)
    loss = loss_fn(ag.fft(x, precision), wt)
    loss.backward()
    g = x.grad.double().cpu().numpy()
    ref = fp64_grad(xq, w, 1)
    err = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    assert err < tol, "rel-L2 %.3e" % err


@pytest.mark.parametrize("precision,tol", [("split", 1e-5), ("plain", 3e-3)])
def test_grad_2d(cuda_device, precision, tol):
    batch, nx, ny = 32, 512, 512
    xq = quantize(uniform_input((batch, nx, ny), seed=6), precision)
    w = np.random.default_rng(3).uniform(0, 1, (batch, nx, ny))
    if precision == "plain":
        w /= nx * ny
    dt = torch.float16 if precision == "plain" else torch.float32
    x = torch.from_numpy(xq).to(dt).to(cuda_device).requires_grad_(True)
    loss = loss_fn(ag.fft2(x, precision), torch.from_numpy(w).float().to(cuda_device))
    loss.backward()
    g = x.grad.double().cpu().numpy()
    ref = fp64_grad(xq, w, 2)
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < tol


def test_grad_vs_finite_differences(cuda_device):
    """Central differences of the GPU loss (split precision, fp32 data) on 64
    random coordinates agree with the adjoint-kernel gradient."""
    batch, n = 2, 1024
    xq = quantize(uniform_input((batch, n), seed=7), "split")
    w = np.random.default_rng(3).uniform(0, 1, (batch, n))
    wt = torch.from_numpy(w).float().to(cuda_device)
    x = torch.from_numpy(xq).float().to(cuda_device).requires_grad_(True)
    loss_fn(ag.fft(x, "split"), wt).backward()
    g = x.grad.double().cpu().numpy()
    rng = np.random.default_rng(11)
    h = 0.1  # the loss is quadratic: central differences are exact up to rounding
    for _ in range(64):
        b, i, c = rng.integers(batch), rng.integers(n), rng.integers(2)
        xp = xq.copy()
        xp[b, i, c] += h
        xm = xq.copy()
        xm[b, i, c] -= h
        with torch.no_grad():
            yp = ag.fft(torch.from_numpy(xp).float().to(cuda_device), "split").double()
            ym = ag.fft(torch.from_numpy(xm).float().to(cuda_device), "split").double()
            lp = (wt.double() * (yp[..., 0] ** 2 + yp[..., 1] ** 2)).sum().item()
            lm = (wt.double() * (ym[..., 0] ** 2 + ym[..., 1] ** 2)).sum().item()
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[b, i, c]) <= 2e-3 * max(1.0, abs(g[b, i, c])) + 0.5, (b, i, c, fd, g[b, i, c])


def test_grad_on_two_streams_and_input_untouched(cuda_device):
    """Two streams differentiating the same shape at once get plans of their own
    (the scratch ring of a plan is not shared by concurrent transforms), and the
    out-of-place passes leave x unmodified."""
    batch, n = 16, 1 << 16
    xs = [quantize(uniform_input((batch, n), seed=20 + k), "plain") for k in range(2)]
    w = np.random.default_rng(3).uniform(0, 1, (batch, n)) / n
    wt = torch.from_numpy(w).float().to(cuda_device)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    xt = [torch.from_numpy(x).half().to(cuda_device).requires_grad_(True) for x in xs]
    keep = [t.detach().clone() for t in xt]
    torch.cuda.synchronize()
    for s, t in zip(streams, xt):
        with torch.cuda.stream(s):
            loss_fn(ag.fft(t, "plain"), wt).backward()
    torch.cuda.synchronize()
    for t, k, x in zip(xt, keep, xs):
        assert torch.equal(t.detach(), k), "the forward pass modified its input"
        g = t.grad.double().cpu().numpy()
        ref = fp64_grad(x, w, 1)
        assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 3e-3
    keys = [k for k in ag._CACHE if k[1] == n]
    assert len({k[-1] for k in keys}) >= 2, "both streams used one plan"
