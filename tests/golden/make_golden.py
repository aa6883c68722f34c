"""Generate the committed golden fixtures in tests/golden/.

Run on the build container (needs the reference sources for the ``ref_*``
entries; everything else needs only numpy):

    python tests/golden/make_golden.py

Writes ``tests/golden/golden.npz`` with:

* ``fft1d_in_<n>`` / ``fft1d_out_<n>``: seeded uniform[-1,1) complex inputs
  (numpy PCG64, seed 1000+n) and their forward DFT from numpy.fft (pocketfft,
  FP64) -- an FFT implementation independent of the oracle's own.
* ``fft2d_in`` / ``fft2d_out``: the same for a 2x16x32 2D case (numpy.fft.fft2).
* ``ref_gen_rev_<n>_<radices>``: the permutation computed by the
  reference's own ``gen_rev`` (tcfft_doit_half.cpp:6-29), compiled from its
  source into oracle/_ref.
* ``ref_table_<n>``: radices and mergings that the reference's own
  ``tcfftCreate`` (tcfft_half.cu:1235-1330) sets for each supported size.
* ``metric_*``: a hand-checked example of the reference's clipped error
  metric (accuracy.cpp:25-41).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

REF_SIZES_1D = [256, 512, 1024, 131072, 262144, 524288, 1 << 24, 1 << 25, 1 << 26, 1 << 27]
GEN_REV_CASES = [(256, [16, 16]), (512, [16, 16, 2]), (1024, [16, 16, 4]),
                 (4096, [16, 16, 16]), (8192, [16, 16, 2, 16]), (64, [4, 2, 8])]


class _RefHandle(ctypes.Structure):
    """Memory layout of struct tcfftHandle (tcfft_half.h:7-18)."""
    _fields_ = [("N", ctypes.c_int), ("N_batch", ctypes.c_int), ("radices", ctypes.c_int * 9),
                ("n_radices", ctypes.c_int), ("mergings", ctypes.c_int * 3), ("n_mergings", ctypes.c_int),
                ("layer_0", ctypes.c_void_p * 3), ("layer_1", ctypes.c_void_p * 3),
                ("F_real", ctypes.c_void_p), ("F_imag", ctypes.c_void_p),
                ("F_real_tmp", ctypes.c_void_p), ("F_imag_tmp", ctypes.c_void_p)]


def main():
    out = {}
    for n in (16, 32, 64, 128, 256, 512, 1024, 2048):
        rng = np.random.default_rng(1000 + n)
        x = rng.uniform(-1, 1, (2, n)) + 1j * rng.uniform(-1, 1, (2, n))
        out["fft1d_in_%d" % n] = x
        out["fft1d_out_%d" % n] = np.fft.fft(x, axis=-1)
    rng = np.random.default_rng(2000)
    x = rng.uniform(-1, 1, (2, 16, 32)) + 1j * rng.uniform(-1, 1, (2, 16, 32))
    out["fft2d_in"] = x
    out["fft2d_out"] = np.fft.fft2(x)

    # metric: tested/standard chosen so each component's term is known
    std = np.array([1.0 + 2.0j, -4.0 + 0.5j, 0.0 + 1.0j])
    tst = np.array([1.1 + 2.0j, -4.0 + 2.0j, 1.0 + 1.5j])
    # terms: re 0.1, im 0; re 0, im min(1,3)=1; re min(1,|1/0|)=1, im 0.5
    out["metric_tested"] = tst
    out["metric_standard"] = std
    out["metric_value"] = np.array((0.1 + 0.0 + 0.0 + 1.0 + 1.0 + 0.5) / 3.0)

    ref_so = os.path.join(ROOT, "oracle", "_ref", "libtcfft_ref_host.so")
    if not os.path.exists(ref_so):
        from oracle import build as ob
        ob.build_ref()
    lib = ctypes.CDLL(ref_so)
    gen_rev = getattr(lib, "_Z7gen_reviPiS_i")
    for n, rad in GEN_REV_CASES:
        rev = (ctypes.c_int * n)()
        rr = (ctypes.c_int * len(rad))(*rad)
        gen_rev(n, rev, rr, len(rad))
        out["ref_gen_rev_%d_%s" % (n, "x".join(map(str, rad)))] = np.array(rev[:], dtype=np.int32)
    create = getattr(lib, "_Z11tcfftCreateP11tcfftHandleii")
    for n in REF_SIZES_1D:
        h = _RefHandle()
        h.radices[:] = [16] * 9  # default member initialisers, tcfft_half.h:10,12
        h.mergings[:] = [0, 0, 0]
        create(ctypes.byref(h), n, 1)
        out["ref_table_%d" % n] = np.array(
            [h.n_radices] + list(h.radices[:h.n_radices]) + [h.n_mergings] + list(h.mergings[:h.n_mergings]),
            dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote %d arrays" % len(out))


if __name__ == "__main__":
    main()
