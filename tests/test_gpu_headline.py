"""GPU: parity of the exact plan the benchmark times -- 1D N = 2^20, batch 256,
plain fp16 (2^28 elements per call, the headline workload).

That plan runs the two-phase kernel with a ring of scratch slots that wraps
many times over the batch; transforms 0, 1 (first lag window), 127, 128
(mid-batch, after the ring wrapped) and 254, 255 (the last lag window, whose
phase 1 runs after every phase 0 has finished) are checked against the FP64
oracle, and every transform of the batch through Parseval's identity (each
transform's energy, computed on the device in fp32), so a transform left
untouched or written to the wrong place fails."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, quantize, to_complex, tol_plain, uniform_input

pytestmark = pytest.mark.gpu

CHECK = [0, 1, 127, 128, 254, 255]


def test_headline_plan_matches_oracle(cuda_device):
    import torch
    n, batch = 1 << 20, 256
    gen = torch.Generator(device=cuda_device)
    gen.manual_seed(20)
    t = torch.empty((batch, n, 2), dtype=torch.float16, device=cuda_device).uniform_(-1, 1, generator=gen)
    xq = {}
    for b in CHECK:
        xq[b] = quantize(uniform_input((n,), seed=1000 + b), "plain")
        t[b] = torch.from_numpy(xq[b]).to(torch.float16).to(cuda_device)
    energy_in = t.float().pow(2).sum(dim=(1, 2)).double().cpu().numpy()
    with tc.Plan(n=n, batch=batch) as p:
        sched = p.info["schedule"]
        assert sched.startswith("fused1d"), sched
        p.exec(t)
        p.check_device()
    assert torch.isfinite(t).all().item()
    energy_out = t.float().pow(2).sum(dim=(1, 2)).double().cpu().numpy()
    ratio = energy_out / (n * energy_in)
    assert np.abs(ratio - 1).max() < 1e-2, "Parseval ratio range %.4f..%.4f" % (ratio.min(), ratio.max())
    xs = np.stack([xq[b] for b in CHECK])
    ref = oracle_1d(xs)
    y = to_complex(t[CHECK].double().cpu().numpy())
    for i, b in enumerate(CHECK):
        err = oracle.rel_l2(y[i], ref[i])
        assert err < tol_plain(n), "transform %d: rel-L2 %.3e (%s)" % (b, err, sched)
