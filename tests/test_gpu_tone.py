"""GPU: the size sweep's tone variant (three unit-amplitude tones over
N(0, 1e-3) noise).  The spectrum has bins of magnitude ~N: the split mode
(fp32 output) keeps rel-L2 <= 1e-5 against FP64; the plain fp16 mode
overflows at large N and must report it as non-finite outputs, not crash, its
finite outputs within fp16 accuracy of the peak; the
fp32-I/O mode (fp32 output) stays within the plain error bound."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, quantize, run_gpu, tol_plain, tone_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1 << 12, 1 << 16, 1 << 20])
def test_tone_split_and_fp32io(cuda_device, n):
    x = quantize(tone_input(n, 2, seed=n.bit_length()), "split")
    ref = oracle_1d(x)
    with tc.Plan(n=n, batch=2, precision="split") as p:
        y = run_gpu(p, x, "split")
    assert np.isfinite(y).all()
    err = oracle.rel_l2(y, ref)
    assert err <= 1e-5, "split n=%d: rel-L2 %.3e" % (n, err)
    with tc.Plan(n=n, batch=2, precision="fp32io") as p:
        y = run_gpu(p, x, "split")
    assert np.isfinite(y).all() and oracle.rel_l2(y, ref) < tol_plain(n)


@pytest.mark.parametrize("n", [1 << 12, 1 << 16, 1 << 20])
def test_tone_plain_reports_overflow(cuda_device, n):
    x = quantize(tone_input(n, 2, seed=n.bit_length()), "plain")
    with tc.Plan(n=n, batch=2) as p:
        y = run_gpu(p, x, "plain")  # check_device inside: no device error
    bad = int((~np.isfinite(y)).sum())
    peak = np.abs(oracle_1d(x)).max()
    if peak < 32768:  # every output component fits fp16 comfortably
        assert bad == 0
        assert oracle.rel_l2(y, oracle_1d(x)) < tol_plain(n)
    if n >= 1 << 20:  # |X_k| ~ 2^20 > 65504: the tone bins overflow fp16
        assert bad > 0
    # the finite outputs are still the DFT to fp16 accuracy relative to the spectrum's
    # peak (measured: 1.3e-4 x peak at 2^16, where the largest bins are near 65504)
    ref = oracle_1d(x)
    finite = np.isfinite(y)
    assert finite.sum() > y.size // 2
    assert np.abs(y[finite] - ref[finite]).max() < 2e-3 * peak
