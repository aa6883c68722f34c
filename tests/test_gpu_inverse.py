"""GPU: the inverse transform and the direction / normalisation options
(tcfftExecuteInverse, tcfftOptions.direction and .normalization), on every
schedule kind: tiny, single-pass, resident, two-phase 1D, composite 1D, fused
2D, composite 2D, split precision and uneven batches.

The reference has no inverse (only the exp(-2 pi i jk/N) twiddles,
tcfft_half.cu:1339); the checks are against the FP64 oracle's inverse DFT
(sign +1, scaled by 1/N) on the same rounded inputs, and round trips
inverse(forward(x)) = x.  The normalised inverse keeps fp16 in range where the
unnormalised adjoint of a spectrum would overflow (N x at N >= 2^16)."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, to_complex, tol, uniform_input

pytestmark = pytest.mark.gpu

CASES_1D = [(16, 37, "plain"), (64, 9, "split"), (128, 5, "plain"), (256, 7, "plain"), (1024, 6, "split"),
            (2048, 3, "plain"), (4096, 5, "plain"), (8192, 2, "split"), (16384, 3, "plain"), (1 << 15, 3, "plain"),
            (1 << 16, 3, "plain"), (1 << 18, 2, "split"), (1 << 20, 2, "plain"), (1 << 23, 1, "plain"),
            (2048, 2, "split")]
CASES_2D = [(256, 512, 3, "plain"), (1024, 1024, 2, "plain"), (512, 256, 2, "split"), (128, 128, 4, "plain"),
            (64, 256, 3, "split"), (4096, 4096, 1, "plain")]


def _inverse_ref(xq, two_d):
    z = to_complex(xq)
    n = z.shape[-1] * (z.shape[-2] if two_d else 1)
    return (oracle.fft_2d(z, sign=+1) if two_d else oracle.fft_1d(z, sign=+1)) / n


@pytest.mark.parametrize("n,batch,precision", CASES_1D)
def test_inverse_1d(cuda_device, n, batch, precision):
    # a spectrum-like input (the forward transform of uniform data, rescaled to its
    # typical magnitude sqrt(N)) so that the unnormalised result would be N times larger
    xq = quantize(uniform_input((batch, n), seed=n % 89 + batch) * np.sqrt(n) / 2, precision)
    with tc.Plan(n=n, batch=batch, precision=precision) as p:
        y = run_gpu(p, xq, precision, inverse=True)
    assert np.isfinite(y).all()
    err = oracle.rel_l2(y, _inverse_ref(xq, False))
    assert err < tol(precision, n), "n=%d %s: rel-L2 %.3e" % (n, precision, err)


@pytest.mark.parametrize("nx,ny,batch,precision", CASES_2D)
def test_inverse_2d(cuda_device, nx, ny, batch, precision):
    xq = quantize(uniform_input((batch, nx, ny), seed=nx + ny) * np.sqrt(nx * ny) / 2, precision)
    with tc.Plan(nx=nx, ny=ny, batch=batch, precision=precision) as p:
        y = run_gpu(p, xq, precision, inverse=True)
    assert np.isfinite(y).all()
    err = oracle.rel_l2(y, _inverse_ref(xq, True))
    assert err < tol(precision, nx * ny), "%dx%d %s: rel-L2 %.3e" % (nx, ny, precision, err)


@pytest.mark.parametrize("n,precision", [(1024, "plain"), (1 << 16, "plain"), (1 << 20, "plain"),
                                         (4096, "split"), (1 << 20, "split")])
def test_round_trip(cuda_device, n, precision):
    """inverse(forward(x)) = x within twice the per-size bound (two transforms);
    at N >= 2^16 the adjoint of the forward result would overflow fp16."""
    import torch
    batch = 2
    xq = quantize(uniform_input((batch, n), seed=3), precision)
    dt = torch.float16 if precision == "plain" else torch.float32
    t = torch.from_numpy(xq).to(dt).to(cuda_device)
    with tc.Plan(n=n, batch=batch, precision=precision) as p:
        p.exec(t)
        p.exec(t, inverse=True)
        p.check_device()
    y = to_complex(t.double().cpu().numpy())
    assert np.isfinite(y).all()
    assert oracle.rel_l2(y, to_complex(xq)) < 2 * tol(precision, n)


@pytest.mark.parametrize("shape", [dict(n=512, batch=4), dict(n=1 << 16, batch=2), dict(nx=256, ny=256, batch=2)],
                         ids=["512", "65536", "256x256"])
def test_plan_options_direction_and_normalization(cuda_device, shape):
    """direction = TCFFT_INVERSE gives the sign +1 transform; normalization =
    TCFFT_NORM_BY_N scales by 1/N; the adjoint keeps the plan's scale and the
    inverse undoes tcfftExecute."""
    import torch
    two_d = "nx" in shape
    dims = (shape["batch"], shape["nx"], shape["ny"]) if two_d else (shape["batch"], shape["n"])
    size = int(np.prod(dims[1:]))
    xq = quantize(uniform_input(dims, seed=size % 53), "plain")
    fwd = (lambda z, s: oracle.fft_2d(z, sign=s)) if two_d else (lambda z, s: oracle.fft_1d(z, sign=s))
    z = to_complex(xq)
    bound = tol("plain", size)
    # inverse direction, unnormalised: sum x exp(+2 pi i nk/N)
    with tc.Plan(direction=tc.INVERSE, **shape) as p:
        y = run_gpu(p, xq, "plain")
        ya = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, fwd(z, +1)) < bound
    assert oracle.rel_l2(ya, fwd(z, -1)) < bound
    # forward, normalised by 1/N; its inverse is the unnormalised conjugate transform
    with tc.Plan(normalize=True, **shape) as p:
        y = run_gpu(p, xq, "plain")
        assert oracle.rel_l2(y, fwd(z, -1) / size) < bound
        t = torch.from_numpy(xq).half().to(cuda_device)
        p.exec(t)
        p.exec(t, inverse=True)
        p.check_device()
    assert oracle.rel_l2(to_complex(t.double().cpu().numpy()), z) < 2 * bound


def test_inverse_uneven_batch(cuda_device):
    """tcfftPlanMany: each transform is scaled by 1/(its own size)."""
    import torch
    shapes = [(256,), (4096,), (128, 256), (1 << 16,), (64,)]
    rng = np.random.default_rng(5)
    parts = [quantize(rng.uniform(-1, 1, tuple(s) + (2,)), "plain") for s in shapes]
    flat = np.concatenate([p.reshape(-1, 2) for p in parts])
    buf = torch.from_numpy(flat).half().to(cuda_device)
    with tc.Plan.many(shapes) as p:
        p.exec(buf, inverse=True)
        p.check_device()
    got = buf.double().cpu().numpy()
    off = 0
    for s, x in zip(shapes, parts):
        size = int(np.prod(s))
        y = to_complex(got[off:off + size].reshape(tuple(s) + (2,)))
        off += size
        err = oracle.rel_l2(y, _inverse_ref(x[None], len(s) == 2)[0])
        assert err < tol("plain", size), (s, err)


@pytest.mark.parametrize("n,precision", [(1 << 16, "plain"), (1 << 20, "plain"), (1 << 23, "plain"),
                                         (1 << 20, "fp32io"), (1 << 21, "fp32io"), (1 << 23, "fp32io"),
                                         (1 << 21, "split")])
def test_inverse_of_unit_sized_data(cuda_device, n, precision):
    """The 1/N of a normalised multi-pass transform is split between the passes
    (1/N1, then 1/N2), so intermediates of O(1) inputs stay far from fp16's
    subnormal range (a single 1/N in the first pass would leave them near 1e-5)."""
    x = quantize(uniform_input((1, n), seed=17), "plain" if precision == "plain" else "split")
    with tc.Plan(n=n, batch=1, precision=precision) as p:
        y = run_gpu(p, x, "plain" if precision == "plain" else "split", inverse=True)
    err = oracle.rel_l2(y, _inverse_ref(x, False))
    assert np.isfinite(y).all() and err < tol("plain" if precision != "split" else "split", n), err
