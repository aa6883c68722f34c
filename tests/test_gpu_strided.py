"""GPU: strided 1D layouts (tcfftPlanStrided).

* Batch stride (istride 1, idist > n): transforms of n contiguous points idist
  elements apart; the gaps between them are left untouched.
* Element stride (istride > 1, idist 1): istride transforms interleaved point by
  point, i.e. the FFT along the middle axis of a [groups][n][istride] array, run
  as one launch of column FFTs.

Every transform is checked against the FP64 oracle; unsupported layouts report
TCFFT_NOT_SUPPORTED instead of running."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import quantize, to_complex, tol_plain, uniform_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,batch,pad", [(1024, 7, 64), (256, 33, 32), (1 << 16, 3, 32), (2048, 5, 2048)])
def test_batch_stride(cuda_device, n, batch, pad):
    import torch
    idist = n + pad
    xq = quantize(uniform_input((batch, n), seed=n % 89 + batch), "plain")
    buf = torch.full((batch * idist, 2), 5.0, dtype=torch.float16, device=cuda_device)
    view = buf.view(batch, idist, 2)
    view[:, :n] = torch.from_numpy(xq).half()
    with tc.Plan.strided(n, batch, istride=1, idist=idist) as p:
        assert "strided" in p.info["schedule"], p.info["schedule"]
        p.exec(buf)
        p.check_device()
    got = view.double().cpu().numpy()
    err = oracle.rel_l2(to_complex(got[:, :n]), oracle.fft_1d(to_complex(xq)))
    assert err < tol_plain(n), "rel-L2 %.3e" % err
    assert (got[:, n:] == 5.0).all(), "a gap between transforms was written"


@pytest.mark.parametrize("n,istride,groups", [(256, 32, 2), (512, 96, 1), (1024, 48, 2), (2048, 8, 3),
                                              (128, 256, 1), (1024, 16, 1), (256, 1024, 1)])
@pytest.mark.parametrize("adjoint", [False, True])
def test_element_stride(cuda_device, n, istride, groups, adjoint):
    import torch
    rng = np.random.default_rng(n + istride + groups)
    x = quantize(rng.uniform(-1, 1, (groups, n, istride, 2)), "plain")
    t = torch.from_numpy(x).half().to(cuda_device)
    with tc.Plan.strided(n, groups * istride, istride=istride, idist=1) as p:
        assert "stride" in p.info["schedule"], p.info["schedule"]
        assert p.info["launches_per_exec"] == 1
        p.exec(t, adjoint=adjoint)
        p.check_device()
    got = to_complex(t.double().cpu().numpy())
    xc = to_complex(x)
    # the transforms run along axis 1: move it last for the oracle and back
    ref = oracle.fft_1d(np.ascontiguousarray(xc.transpose(0, 2, 1)), +1 if adjoint else -1).transpose(0, 2, 1)
    err = oracle.rel_l2(got, ref)
    assert err < tol_plain(n), "rel-L2 %.3e" % err


def test_unsupported_strided_layouts(cuda_device):
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan.strided(256, 48, istride=48, idist=1)  # not whole 32-column tiles
    assert e.value.status == 7
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan.strided(4096, 32, istride=32, idist=1)  # columns longer than 2048
    assert e.value.status == 7
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan.strided(512, 64, istride=32, idist=1, precision="split")
    assert e.value.status == 7
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan.strided(512, 64, istride=32, idist=1, normalize=True)
    assert e.value.status == 7
    with pytest.raises(tc.TcfftError):
        tc.Plan.strided(1024, 4, istride=1, idist=512)  # transforms would overlap
    with tc.Plan.strided(512, 64, istride=32, idist=1) as p:
        import torch
        t = torch.zeros((2, 512, 32, 2), dtype=torch.float16, device="cuda")
        with pytest.raises(tc.TcfftError) as e:
            p.exec(t, inverse=True)  # the normalised inverse needs the per-shape graph
        assert e.value.status == 7
