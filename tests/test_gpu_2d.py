"""GPU parity: batched 2D FFT (row pass + column pass, one fused launch)
through the C ABI vs the FP64 oracle (accuracy_2d.cpp's procedure)."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_2d, quantize, run_gpu, tol_plain, tol_split, uniform_input

pytestmark = pytest.mark.gpu

SHAPES = [(256, 256), (256, 512), (512, 256), (512, 512), (256, 1024), (512, 1024), (1024, 1024),
          (2048, 256), (256, 2048), (1024, 2048), (2048, 2048)]


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_plain_2d(cuda_device, nx, ny):
    batch = 2 if nx * ny <= (1 << 20) else 1
    xq = quantize(uniform_input((batch, nx, ny), seed=1), "plain")
    with tc.Plan(nx=nx, ny=ny, batch=batch) as p:
        assert "fused2d" in p.info["schedule"]
        y = run_gpu(p, xq, "plain")
    ref = oracle_2d(xq)
    assert np.isfinite(y).all()
    err = oracle.rel_l2(y, ref)
    assert err < tol_plain(nx * ny), "%dx%d rel-L2 %.3e" % (nx, ny, err)


@pytest.mark.parametrize("nx,ny", [(256, 256), (512, 1024), (1024, 1024)])
def test_split_2d(cuda_device, nx, ny):
    xq = quantize(uniform_input((2, nx, ny), seed=1), "split")
    with tc.Plan(nx=nx, ny=ny, batch=2, precision="split") as p:
        y = run_gpu(p, xq, "split")
    err = oracle.rel_l2(y, oracle_2d(xq))
    assert err < tol_split(nx * ny), "%dx%d rel-L2 %.3e" % (nx, ny, err)


def test_adjoint_2d(cuda_device):
    nx, ny = 512, 256
    xq = quantize(uniform_input((3, nx, ny), seed=4), "plain")
    with tc.Plan(nx=nx, ny=ny, batch=3) as p:
        y = run_gpu(p, xq, "plain", adjoint=True)
    assert oracle.rel_l2(y, oracle_2d(xq, adjoint=True)) < tol_plain(nx * ny)


def test_2d_many_transforms(cuda_device):
    """config: 256x256 batch 1024 (2D sweep case) on a subset: 64 transforms."""
    nx = ny = 256
    batch = 64
    xq = quantize(uniform_input((batch, nx, ny), seed=1), "plain")
    with tc.Plan(nx=nx, ny=ny, batch=batch) as p:
        y = run_gpu(p, xq, "plain")
    ref = oracle_2d(xq)
    per = np.linalg.norm((y - ref).reshape(batch, -1), axis=1) / np.linalg.norm(ref.reshape(batch, -1), axis=1)
    assert per.max() < 1.5 * tol_plain(nx * ny)
