"""tcfftExecuteHost: host buffers in and out, the batch pipelined in chunks
(copy in / transform / copy out on three streams).  The chunked result must be
bit-identical to tcfftExecute on the same data (every kernel computes each
transform independently of its batch), and match the FP64 oracle."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, to_complex, tol, tol_plain, uniform_input

pytestmark = pytest.mark.gpu


def _host_pair(xq, precision):
    import torch
    dt = torch.float16 if precision == "plain" else torch.float32
    h_in = torch.from_numpy(np.ascontiguousarray(xq)).to(dt).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    return h_in, h_out


@pytest.mark.parametrize("shape,batch,precision", [((1 << 20,), 9, "plain"), ((4096,), 1000, "split"),
                                                   ((256,), 3, "plain"), ((1024, 1024), 5, "plain"),
                                                   ((1 << 16,), 1, "plain")])
def test_execute_host_matches_device(cuda_device, shape, batch, precision):
    import torch
    xq = quantize(uniform_input((batch,) + shape, seed=sum(shape) + batch), precision)
    h_in, h_out = _host_pair(xq, precision)
    kw = {"n": shape[0]} if len(shape) == 1 else {"nx": shape[0], "ny": shape[1]}
    with tc.Plan(batch=batch, precision=precision, **kw) as p:
        work = h_in.cuda()
        p.exec_host(h_in, h_out, work)
        dev = h_in.cuda()
        p.exec(dev)
        torch.cuda.synchronize()
        p.check_device()
    assert torch.equal(h_out, dev.cpu()), "chunked host execution differs from the device execution"
    y = to_complex(h_out.double().numpy())
    ref = oracle_1d(xq) if len(shape) == 1 else oracle_2d(xq)
    sub = slice(0, min(batch, 16))
    assert oracle.rel_l2(y[sub], ref[sub]) < tol(precision, int(np.prod(shape)))


def test_execute_host_in_place_host_buffer(cuda_device):
    """host_out may be host_in."""
    import torch
    xq = quantize(uniform_input((6, 8192), seed=3), "plain")
    h, _ = _host_pair(xq, "plain")
    with tc.Plan(n=8192, batch=6) as p:
        work = torch.empty_like(h, device="cuda")
        p.exec_host(h, h, work)
        torch.cuda.synchronize()
    assert oracle.rel_l2(to_complex(h.double().numpy()), oracle_1d(xq)) < tol_plain(8192)


def test_execute_host_many(cuda_device):
    """Uneven-batch plans run unchunked."""
    import torch
    shapes = [(512,), (128, 256), (4096,)]
    total = sum(int(np.prod(s)) for s in shapes)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, size=(total, 2)).astype(np.float16)
    h_in = torch.from_numpy(x).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    with tc.Plan.many(shapes) as p:
        work = torch.empty_like(h_in, device="cuda")
        p.exec_host(h_in, h_out, work)
        dev = h_in.cuda()
        p.exec(dev)
        torch.cuda.synchronize()
    assert torch.equal(h_out, dev.cpu())
