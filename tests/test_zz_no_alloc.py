"""GPU: the allocation-free entry point (tcfftExecute1dNoAlloc), called
through the C ABI, against the plan-based entry point.

Some callers cannot allocate device memory when they run an FFT (stream
capture without allocation nodes, hosts that own all device memory); the
no-alloc entry point serves them from fixed static device arrays.  This file
is collected last so that a run stopping at the first failure has already run
every other test; it passes alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

import tcfft_gb300 as tc
from fftcheck import oracle_1d, quantize, to_complex, tol, uniform_input

pytestmark = pytest.mark.gpu

CASES = [(1 << 12, 5, "plain"), (1 << 15, 3, "plain"), (1 << 16, 3, "plain"), (1 << 20, 2, "plain"),
         (1 << 21, 1, "plain"), (1 << 14, 4, "split"), (1 << 15, 2, "split"), (1 << 18, 2, "split")]


def _noalloc(t, n, batch, precision, direction):
    import torch
    prec = 0 if precision == "plain" else 1
    st = tc.lib().tcfftExecute1dNoAlloc(ctypes.c_void_p(t.data_ptr()), n, batch, prec, direction,
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st


@pytest.mark.parametrize("n,batch,precision", CASES)
def test_noalloc_matches_plan_two_calls(cuda_device, monkeypatch, n, batch, precision):
    """Two calls in a row through the C ABI: each agrees with the plan-based
    entry point (the same two-phase kernel: the plan is made with the resident
    kernel turned off; twiddle tables computed on the device in FP64 rather than
    on the host, so agreement is near-exact, well inside the tolerance) and with
    the FP64 oracle within the per-size tolerance."""
    import torch
    monkeypatch.setenv("TCFFT_NO_RESIDENT", "1")
    dt = torch.float16 if precision == "plain" else torch.float32
    bound = tol(precision, n)
    x = quantize(uniform_input((batch, n), seed=n % 991 + batch), precision)
    for direction in (0, 1):
        ref_t = torch.from_numpy(x).to(dt).to(cuda_device)
        with tc.Plan(n=n, batch=batch, precision=precision) as p:
            p.exec(ref_t, adjoint=direction == 1)
            p.check_device()
        ref = to_complex(ref_t.double().cpu().numpy())
        exact = oracle_1d(x, adjoint=direction == 1)
        for call in range(2):  # two calls in a row share the static scratch
            t = torch.from_numpy(x).to(dt).to(cuda_device)
            assert _noalloc(t, n, batch, precision, direction) == 0
            assert tc.lib().tcfftCheckDeviceNoAlloc(None) == 0
            y = to_complex(t.double().cpu().numpy())
            assert np.isfinite(y).all()
            err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
            assert err < 0.25 * bound, "n=%d call %d direction %d: rel-L2 %.3e vs plan" % (n, call, direction, err)
            err = np.linalg.norm(y - exact) / np.linalg.norm(exact)
            assert err < bound, "n=%d call %d direction %d: rel-L2 %.3e vs FP64" % (n, call, direction, err)


@pytest.mark.parametrize("n,batch,precision", [(1 << 16, 3, "plain"), (1 << 14, 2, "split")])
def test_noalloc_stream_capture(cuda_device, tmp_path, n, batch, precision):
    """A call captured into a CUDA graph, after one warm-up call has set up the
    static arrays, replays correctly.  The capture runs in the global capture
    mode, which fails any allocation call made during it; the graph holds the
    table kernel, the counter memset and the transform, and no allocation node."""
    import torch
    dt = torch.float16 if precision == "plain" else torch.float32
    prec = 0 if precision == "plain" else 1
    x = quantize(uniform_input((batch, n), seed=n % 37 + 5), precision)
    xt = torch.from_numpy(x).to(dt).to(cuda_device)
    t = xt.clone()
    assert _noalloc(t.clone(), n, batch, precision, 0) == 0  # warm-up: set-up outside the capture
    g = torch.cuda.CUDAGraph()
    dump = hasattr(g, "enable_debug_mode") and hasattr(g, "debug_dump")
    if dump:
        g.enable_debug_mode()
    with torch.cuda.graph(g, capture_error_mode="global"):
        st = tc.lib().tcfftExecute1dNoAlloc(ctypes.c_void_p(t.data_ptr()), n, batch, prec, 0,
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    exact = oracle_1d(x)
    for rep in range(2):
        t.copy_(xt)
        g.replay()
        torch.cuda.synchronize()
        assert tc.lib().tcfftCheckDeviceNoAlloc(None) == 0
        y = to_complex(t.double().cpu().numpy())
        err = np.linalg.norm(y - exact) / np.linalg.norm(exact)
        assert err < tol(precision, n), "replay %d: rel-L2 %.3e" % (rep, err)
    if dump:
        # some torch builds accept the call without writing the file; the global capture mode
        # above already fails any allocation call made during the capture
        path = tmp_path / "noalloc_graph.dot"
        g.debug_dump(str(path))
        if path.exists():
            text = path.read_text().lower()
            assert "mem_alloc" not in text and "memalloc" not in text, "allocation node in the captured graph"


def test_noalloc_rejects_sizes_beyond_limit(cuda_device):
    import torch
    t = torch.zeros((1, 1 << 22, 2), dtype=torch.float16, device=cuda_device)
    assert _noalloc(t, 1 << 22, 1, "plain", 0) == 2      # beyond the static scratch
    assert _noalloc(t, 1 << 21, 1, "split", 0) == 2      # split limit is 2^20
    assert _noalloc(t, 2048, 1, "plain", 0) == 2          # no scratch below 2^12: use a plan
    assert _noalloc(t, 3000, 1, "plain", 0) == 2
    u = torch.zeros((1 << 13,), dtype=torch.float16, device=cuda_device)
    st = tc.lib().tcfftExecute1dNoAlloc(ctypes.c_void_p(u.data_ptr() + 4), 4096, 1, 0, 0, None)
    assert st == 3                                        # misaligned
