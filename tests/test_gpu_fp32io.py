"""GPU: the fp32-I/O precision (TCFFT_PRECISION_FP32_IO): complex64 data in
and out, fp16 tensor-core operands converted from fp32 as the kernels read
shared memory, fp32 accumulation, fp32 between passes and at the output.

Every schedule kind is checked against the FP64 oracle on the fp32 inputs
the kernel receives, within the plain fp16 bound of the size (the operands
are fp16; the storage, unlike the plain mode's, is not), and against the
plain mode on the same fp16-representable inputs, where the fp32 mode must be
at least as accurate."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, to_complex, tol_plain, uniform_input

pytestmark = pytest.mark.gpu

SIZES_1D = [(16, 33), (64, 9), (256, 7), (1024, 5), (2048, 3), (4096, 4), (8192, 3), (16384, 2), (1 << 15, 2),
            (1 << 16, 2), (1 << 18, 2), (1 << 20, 2), (1 << 21, 1), (1 << 23, 1)]
SIZES_2D = [(256, 256, 3), (512, 1024, 2), (1024, 1024, 2), (4096, 256, 1), (64, 256, 3)]


@pytest.mark.parametrize("n,batch", SIZES_1D)
def test_fp32io_1d(cuda_device, n, batch):
    x = quantize(uniform_input((batch, n), seed=n % 71 + batch), "split")  # fp32 values
    with tc.Plan(n=n, batch=batch, precision="fp32io") as p:
        sched = p.info["schedule"]
        assert "fp32io" in sched, sched
        y = run_gpu(p, x, "split")
        ya = run_gpu(p, x, "split", adjoint=True)
        yi = run_gpu(p, x, "split", inverse=True)
    ref = oracle_1d(x)
    err = oracle.rel_l2(y, ref)
    assert np.isfinite(y).all() and err < tol_plain(n), "n=%d (%s): rel-L2 %.3e" % (n, sched, err)
    err = oracle.rel_l2(ya, oracle_1d(x, adjoint=True))
    assert err < tol_plain(n), "n=%d adjoint: rel-L2 %.3e" % (n, err)
    err = oracle.rel_l2(yi, oracle_1d(x, adjoint=True) / n)
    assert err < tol_plain(n), "n=%d inverse: rel-L2 %.3e" % (n, err)
    # on fp16-representable inputs the fp32 mode is no less accurate than the plain one
    xh = quantize(x, "plain")
    with tc.Plan(n=n, batch=batch, precision="fp32io") as p:
        e32 = oracle.rel_l2(run_gpu(p, xh, "split"), oracle_1d(xh))
    with tc.Plan(n=n, batch=batch) as p:
        e16 = oracle.rel_l2(run_gpu(p, xh, "plain"), oracle_1d(xh))
    assert e32 <= 1.05 * e16, "n=%d: fp32io %.3e vs plain %.3e" % (n, e32, e16)


@pytest.mark.parametrize("nx,ny,batch", SIZES_2D)
def test_fp32io_2d(cuda_device, nx, ny, batch):
    x = quantize(uniform_input((batch, nx, ny), seed=nx + 3 * ny), "split")
    with tc.Plan(nx=nx, ny=ny, batch=batch, precision="fp32io") as p:
        y = run_gpu(p, x, "split")
        yi = run_gpu(p, x, "split", inverse=True)
    assert oracle.rel_l2(y, oracle_2d(x)) < tol_plain(nx * ny)
    assert oracle.rel_l2(yi, oracle_2d(x, adjoint=True) / (nx * ny)) < tol_plain(nx * ny)


def test_fp32io_out_of_place_and_real(cuda_device):
    import torch
    n, batch = 1 << 16, 3
    x = quantize(uniform_input((batch, n), seed=9), "split")
    src = torch.from_numpy(x).float().to(cuda_device)
    keep = src.clone()
    with tc.Plan(n=n, batch=batch, precision="fp32io") as p:
        ref = src.clone()
        p.exec(ref)
        out = torch.empty_like(src)
        p.exec_out(src, out)
        p.check_device()
    assert torch.equal(src, keep) and torch.equal(out, ref)
    r = np.random.default_rng(4).uniform(-1, 1, (2, 4096)).astype(np.float32)
    rt = torch.from_numpy(r).to(cuda_device)
    spec = torch.empty((2, 2049, 2), dtype=torch.float32, device=cuda_device)
    back = torch.empty_like(rt)
    with tc.RealPlan(4096, 2, precision="fp32io") as p:
        p.r2c(rt, spec)
        p.c2r(spec, back)
        p.check_device()
    X = to_complex(spec.double().cpu().numpy())
    assert oracle.rel_l2(X, oracle.fft_1d(r.astype(np.float64) + 0j)[:, :2049]) < tol_plain(4096)
    assert oracle.rel_l2(back.double().cpu().numpy(), r.astype(np.float64)) < 2 * tol_plain(4096)
