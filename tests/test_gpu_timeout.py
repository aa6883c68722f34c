"""GPU: the bounded-wait timeout path of the two-phase kernels.

Every cross-CTA wait of the two-phase kernels is bounded; when one runs out
the kernel stops early, raises a device flag and tcfftCheckDevice returns
TCFFT_TIMEOUT.  The failure is made on the host (tcfftInjectWaitTimeout
presets one completion counter to a value that no number of completed tiles
reaches, before the launch) with a 1 ms wait limit, so nothing faults or
hangs: the waits on that counter run out, the kernel's warps leave their
loops, and the same plan must then run a normal execute correctly."""
import time

import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, tol_plain, uniform_input

pytestmark = pytest.mark.gpu

SHAPES = [dict(n=1 << 15, batch=3),      # short-row two-phase schedule (512 x 64, resident kernel off)
          dict(n=1 << 16, batch=8),
          dict(n=1 << 20, batch=3),
          dict(nx=512, ny=512, batch=4)]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(str(v) for v in s.values()))
def test_wait_timeout_is_reported_and_plan_recovers(cuda_device, monkeypatch, shape):
    import torch
    if shape.get("n") == 1 << 15:
        monkeypatch.setenv("TCFFT_NO_RESIDENT", "1")  # plain 2^15 is resident by default
    size = shape["n"] if "n" in shape else shape["nx"] * shape["ny"]
    dims = (shape["batch"], shape["n"]) if "n" in shape else (shape["batch"], shape["nx"], shape["ny"])
    xq = quantize(uniform_input(dims, seed=size % 101), "plain")
    with tc.Plan(**shape) as p:
        if not p.info["schedule"].startswith(("fused1d", "fused2d")):
            pytest.skip("schedule without cross-CTA waits: " + p.info["schedule"])
        p.set_wait_limit(1_000_000)  # 1 ms
        p.inject_wait_timeout()
        t = torch.from_numpy(xq).to(torch.float16).to(cuda_device)
        t0 = time.perf_counter()
        p.exec(t)
        with pytest.raises(tc.TcfftError) as e:
            p.check_device()
        elapsed = time.perf_counter() - t0
        assert e.value.status == 6, e.value  # TCFFT_TIMEOUT
        assert elapsed < 10.0, "the stalled execute took %.1f s" % elapsed
        # the flag was cleared by the check; the next execute is unaffected
        p.set_wait_limit(0)
        y = run_gpu(p, xq, "plain")
        p.check_device()
    ref = oracle_1d(xq) if "n" in shape else oracle_2d(xq)
    assert oracle.rel_l2(y, ref) < tol_plain(size)


def test_inject_on_single_pass_schedule_is_not_supported(cuda_device):
    with tc.Plan(n=1024, batch=4) as p:
        with pytest.raises(tc.TcfftError) as e:
            p.inject_wait_timeout()
        assert e.value.status == 7


def test_noalloc_check_reports_clean_state(cuda_device):
    import torch
    n, batch = 1 << 16, 2
    xq = quantize(uniform_input((batch, n), seed=3), "plain")
    t = torch.from_numpy(xq).to(torch.float16).to(cuda_device)
    tc.execute_1d_noalloc(t, n, batch)
    tc.check_device_noalloc()
    y = t.double().cpu().numpy()
    assert oracle.rel_l2(y[..., 0] + 1j * y[..., 1], oracle_1d(xq)) < tol_plain(n)
    assert np.isfinite(y).all()


def test_many_plan_wait_timeout_and_recovery(cuda_device):
    """The one-launch uneven-batch plan: one transform's completion counter is preset so
    that its pass-B items never become ready; their bounded waits run out (1 ms), the
    launch ends early with TCFFT_TIMEOUT, and the next execute is correct."""
    import torch
    from fftcheck import to_complex
    shapes = [(1024,), (512, 256), (1 << 16,), (256, 256), (4096,), (2048,)]
    rng = np.random.default_rng(4)
    parts = [quantize(rng.uniform(-1, 1, tuple(s) + (2,)), "plain") for s in shapes]
    flat = np.concatenate([p.reshape(-1, 2) for p in parts])
    with tc.Plan.many(shapes) as p:
        assert "persistent" in p.info["schedule"], p.info["schedule"]
        p.set_wait_limit(1_000_000)
        p.inject_wait_timeout()
        buf = torch.from_numpy(flat).half().cuda()
        t0 = time.perf_counter()
        p.exec(buf)
        with pytest.raises(tc.TcfftError) as e:
            p.check_device()
        assert e.value.status == 6, e.value
        assert time.perf_counter() - t0 < 10.0
        p.set_wait_limit(0)
        buf = torch.from_numpy(flat).half().cuda()
        p.exec(buf)
        p.check_device()
        got = buf.double().cpu().numpy()
    off = 0
    for x, s in zip(parts, shapes):
        n = int(np.prod(s))
        y = got[off:off + n].reshape(tuple(s) + (2,))
        ref = oracle.fft_1d(to_complex(x)) if len(s) == 1 else oracle.fft_2d(to_complex(x))
        assert oracle.rel_l2(to_complex(y), ref) < tol_plain(n), s
        off += n


def test_many_plan_without_pass_b_has_no_hook(cuda_device):
    with tc.Plan.many([(256,), (1024,)]) as p:
        with pytest.raises(tc.TcfftError) as e:
            p.inject_wait_timeout()
        assert e.value.status == 7
