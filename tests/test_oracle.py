"""CPU: pin the FP64 oracle against the committed golden vectors (numpy
pocketfft outputs and the reference's own gen_rev / tcfftCreate results) and
against an O(N^2) long-double DFT."""
import os

import numpy as np
import pytest

import oracle

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048])
def test_fft1d_matches_golden(n):
    x = GOLDEN["fft1d_in_%d" % n]
    y = oracle.fft_1d(x)
    assert oracle.rel_l2(y, GOLDEN["fft1d_out_%d" % n]) < 1e-14


def test_fft2d_matches_golden():
    y = oracle.fft_2d(GOLDEN["fft2d_in"])
    assert oracle.rel_l2(y, GOLDEN["fft2d_out"]) < 1e-14


@pytest.mark.parametrize("n", [1, 2, 8, 64, 512])
def test_fft_vs_naive_longdouble(n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    for sign in (-1, 1):
        assert oracle.rel_l2(oracle.fft_1d(x[None], sign)[0], oracle.dft_naive(x, sign)) < 1e-14


def test_adjoint_is_conjugate_direction():
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (3, 256)) + 1j * rng.uniform(-1, 1, (3, 256))
    assert oracle.rel_l2(oracle.fft_1d(x, +1), 256 * np.fft.ifft(x, axis=-1)) < 1e-14
    # forward o adjoint = N * I
    assert oracle.rel_l2(oracle.fft_1d(oracle.fft_1d(x, -1), +1), 256 * x) < 1e-14


def test_known_answers():
    n = 64
    imp = np.zeros((1, n), complex)
    imp[0, 0] = 1
    assert np.allclose(oracle.fft_1d(imp), 1.0)
    tone = np.exp(2j * np.pi * 5 * np.arange(n) / n)[None]
    expect = np.zeros((1, n), complex)
    expect[0, 5] = n
    assert np.abs(oracle.fft_1d(tone) - expect).max() < 1e-12


def test_clipped_metric_golden():
    v = oracle.clipped_error(GOLDEN["metric_tested"], GOLDEN["metric_standard"])
    assert abs(v - float(GOLDEN["metric_value"])) < 1e-15


@pytest.mark.parametrize("key", [k for k in GOLDEN.files if k.startswith("ref_gen_rev_")])
def test_gen_rev_matches_reference(key):
    _, _, _, n, rad = key.split("_")
    radices = [int(r) for r in rad.split("x")]
    got = oracle.gen_rev(int(n), radices)
    assert np.array_equal(got, GOLDEN[key].astype(np.int64))


@pytest.mark.parametrize("key", [k for k in GOLDEN.files if k.startswith("ref_table_")])
def test_reference_size_table(key):
    n = int(key.split("_")[-1])
    tab = GOLDEN[key]
    nr = int(tab[0])
    assert oracle.reference_radices(n) == [int(v) for v in tab[1:1 + nr]]


def test_gen_rev_is_permutation_and_inverse_order():
    rev = oracle.gen_rev(4096, [16, 16, 16])
    assert sorted(rev.tolist()) == list(range(4096))
    # base-16 digit reversal for a uniform chain
    i = 0x123
    assert rev[i] == 0x321


def test_reference_input_order_roundtrip():
    """DIT on digit-reversed input (the reference's contract) equals the DFT."""
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, (2, 512)) + 1j * rng.uniform(-1, 1, (2, 512))
    xr = oracle.reference_input_order_1d(x, [16, 16, 2])
    rev = oracle.gen_rev(512, [16, 16, 2])
    assert np.array_equal(xr[:, 0], x[:, rev[0]])
    assert np.array_equal(xr[:, 1], x[:, rev[1]])


def test_bad_arguments():
    with pytest.raises(ValueError):
        oracle.fft_1d(np.zeros((1, 12)))
    with pytest.raises(ValueError):
        oracle.gen_rev(256, [16, 8])
