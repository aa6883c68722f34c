"""GPU: the reference's input-order contract (TCFFT_ORDER_REFERENCE_DIGIT_REVERSED).

Input is permuted the way the reference harness does it (gen_rev with the
reference's radix chain, tcfft_doit_half.cpp:38-46 / _2d.cpp:40-50), the
output must be the natural-order DFT of the unpermuted data."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, to_complex, tol_plain, uniform_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [256, 512, 1024, 131072, 262144, 524288])
def test_reference_order_1d(cuda_device, n):
    batch = 3
    xq = quantize(uniform_input((batch, n), seed=n % 313), "plain")
    radices = oracle.reference_radices(n)
    xr = oracle.reference_input_order_1d(xq[..., 0] + 1j * xq[..., 1], radices)
    xin = np.stack([xr.real, xr.imag], axis=-1)
    with tc.Plan(n=n, batch=batch, input_order=tc.ORDER_REFERENCE_DIGIT_REVERSED) as p:
        assert p.info["radices"] == radices
        y = run_gpu(p, xin, "plain")
    assert oracle.rel_l2(y, oracle_1d(xq)) < tol_plain(n)


@pytest.mark.parametrize("nx,ny", [(256, 256), (256, 1024), (512, 512), (1024, 1024)])
def test_reference_order_2d(cuda_device, nx, ny):
    xq = quantize(uniform_input((2, nx, ny), seed=1), "plain")
    rx, ry = oracle.reference_radices_2d_axis(nx), oracle.reference_radices_2d_axis(ny)
    xr = oracle.reference_input_order_2d(xq[..., 0] + 1j * xq[..., 1], rx, ry)
    xin = np.stack([xr.real, xr.imag], axis=-1)
    with tc.Plan(nx=nx, ny=ny, batch=2, input_order=tc.ORDER_REFERENCE_DIGIT_REVERSED) as p:
        assert p.info["radices"] == rx and p.info["radices_y"] == ry
        y = run_gpu(p, xin, "plain")
    assert oracle.rel_l2(y, oracle_2d(xq)) < tol_plain(nx * ny)


def test_natural_order_reports_identity_chain(cuda_device):
    with tc.Plan(n=4096, batch=1) as p:
        assert p.info["radices"] == [4096]   # makes the reference's gen_rev the identity
    with tc.Plan(nx=256, ny=512, batch=1) as p:
        assert p.info["radices"] == [256] and p.info["radices_y"] == [512]


def test_reference_order_rejects_unsupported_sizes(cuda_device):
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan(n=4096, batch=1, input_order=tc.ORDER_REFERENCE_DIGIT_REVERSED)
    assert e.value.status == 2
