"""CPU FP64 oracle for the batched half-precision FFT -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker or the timed CPU
baseline.  The tcfft_gb300 product never imports it.

Contents (each cites the reference behaviour it restates; reference =
rox906/tcFFT):

* :func:`fft_1d` / :func:`fft_2d` -- FP64 DFT, sign -1, unnormalised, per batch
  item, on the unrounded doubles: the reference's accuracy oracle
  (accuracy.cpp:11-23, accuracy_2d.cpp:11-23, FFTW_FORWARD).  Computed by
  ``fft64.c`` (own radix-2 FFT; FFTW itself is not available).
* :func:`gen_rev` -- the reference's host digit-reversal permutation
  (tcfft_doit_half.cpp:6-29).
* :func:`clipped_error` -- the reference's metric (accuracy.cpp:25-41).
* :func:`rel_l2`, :func:`max_abs` -- rel-L2 / max-abs error measures.
* :func:`reference_radices` -- the reference's size -> radix table
  (tcfft_half.cu:1250-1330, 2D: tcfft_half_2d.cu:1167-1206), restated.

Parity pin: the reference ships no golden vectors and its oracle (FFTW 3.3.8)
is not installed, so this oracle is pinned against numpy.fft (pocketfft, an
independent FP64 FFT), an O(N^2) long-double DFT, known-answer identities,
and the reference's own ``gen_rev``/``tcfftCreate`` host code compiled from
its sources (``oracle/_ref``, build container only); the pinned values are
committed under ``tests/golden``.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            from . import build as _b
            _b.build()
        lib = ctypes.CDLL(path)
        i64, dp = ctypes.c_int64, ctypes.POINTER(ctypes.c_double)
        lib.oracle_fft_1d.argtypes = [dp, i64, i64, ctypes.c_int]
        lib.oracle_fft_1d.restype = ctypes.c_int
        lib.oracle_fft_2d.argtypes = [dp, i64, i64, i64, ctypes.c_int]
        lib.oracle_fft_2d.restype = ctypes.c_int
        lib.oracle_dft_naive.argtypes = [dp, dp, i64, ctypes.c_int]
        lib.oracle_dft_naive.restype = ctypes.c_int
        lib.oracle_gen_rev.argtypes = [i64, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int64)]
        lib.oracle_gen_rev.restype = ctypes.c_int
        lib.oracle_clipped_error.argtypes = [dp, dp, i64]
        lib.oracle_clipped_error.restype = ctypes.c_double
        lib.oracle_num_threads.restype = ctypes.c_int
        lib.oracle_set_num_threads.argtypes = [ctypes.c_int]
        _LIB = lib
    return _LIB


def _as_c128(x):
    x = np.asarray(x)
    if x.dtype != np.complex128 or not x.flags.c_contiguous:
        x = np.ascontiguousarray(x, dtype=np.complex128)
    return x


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def num_threads():
    return _lib().oracle_num_threads()


def set_num_threads(t):
    _lib().oracle_set_num_threads(int(t))


def fft_1d(x, sign=-1):
    """FP64 DFT along the last axis (power-of-two length), returns a new array.

    sign=-1 is the forward transform (accuracy.cpp:14), sign=+1 the
    conjugate-direction (unnormalised inverse) transform."""
    a = _as_c128(x).copy()
    n = a.shape[-1]
    batch = a.size // n if n else 0
    if _lib().oracle_fft_1d(_dptr(a), n, batch, int(sign)) != 0:
        raise ValueError("oracle_fft_1d: unsupported n=%d" % n)
    return a


def fft_2d(x, sign=-1):
    """FP64 2D DFT over the last two axes ([..., nx, ny] row-major)."""
    a = _as_c128(x).copy()
    nx, ny = a.shape[-2], a.shape[-1]
    batch = a.size // (nx * ny) if nx * ny else 0
    if _lib().oracle_fft_2d(_dptr(a), nx, ny, batch, int(sign)) != 0:
        raise ValueError("oracle_fft_2d: unsupported shape %dx%d" % (nx, ny))
    return a


def dft_naive(x, sign=-1):
    """O(N^2) long-double DFT of a 1D vector (any length)."""
    a = _as_c128(x).reshape(-1)
    out = np.empty_like(a)
    if _lib().oracle_dft_naive(_dptr(a), _dptr(out), a.size, int(sign)) != 0:
        raise ValueError("bad arguments")
    return out


def gen_rev(n, radices):
    """Digit-reversal permutation of tcfft_doit_half.cpp:6-29 (int64 array)."""
    r = (ctypes.c_int * len(radices))(*[int(v) for v in radices])
    out = np.empty(int(n), dtype=np.int64)
    if _lib().oracle_gen_rev(int(n), r, len(radices),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))) != 0:
        raise ValueError("radices %s do not multiply to %d" % (list(radices), n))
    return out


def clipped_error(tested, standard):
    """mean over components of min(1, |(t-s)/s|) * 2 (accuracy.cpp:25-41)."""
    t = _as_c128(tested)
    s = _as_c128(standard)
    if t.shape != s.shape:
        raise ValueError("shape mismatch")
    return _lib().oracle_clipped_error(_dptr(t), _dptr(s), t.size)


def rel_l2(y, ref):
    y = np.asarray(y, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    return float(np.linalg.norm((y - ref).ravel()) / np.linalg.norm(ref.ravel()))


def max_abs(y, ref):
    return float(np.max(np.abs(np.asarray(y, dtype=np.complex128) - np.asarray(ref, dtype=np.complex128))))


# The reference's size -> radix table, restated from tcfftCreate
# (tcfft_half.cu:1250-1330): radices default to 16 (tcfft_half.h:10); only
# these sizes are set; any other size leaves n_radices uninitialised.
_REF_RADICES_1D = {
    256: [16, 16],
    512: [16, 16, 2],
    1024: [16, 16, 4],
    131072: [16, 16, 2, 16, 16],
    262144: [16, 16, 2, 16, 16, 2],
    524288: [16, 16, 4, 16, 16, 2],
    16777216: [16] * 6,
    33554432: [16, 16, 2, 16, 16, 16, 16],
    67108864: [16, 16, 2, 16, 16, 2, 16, 16],
    134217728: [16, 16, 2, 16, 16, 2, 16, 16, 2],
}
# 2D (tcfft_half_2d.cu:1167-1206): radices_{x,y} default {16, 16, 2}
# (tcfft_half_2d.h:10-11); n_radices set per axis for 256/512/1024.
_REF_RADICES_AXIS_2D = {256: [16, 16], 512: [16, 16, 2], 1024: [16, 16, 4]}


def reference_radices(n):
    """Radix chain the reference's tcfftCreate picks for a 1D size, or None."""
    r = _REF_RADICES_1D.get(int(n))
    return list(r) if r is not None else None


def reference_radices_2d_axis(n):
    r = _REF_RADICES_AXIS_2D.get(int(n))
    return list(r) if r is not None else None


def reference_input_order_1d(x, radices):
    """Reorder natural-order input the way the reference harness does before
    tcfftExec (tcfft_doit_half.cpp:38-46): position i gets x[rev[i]]."""
    rev = gen_rev(x.shape[-1], radices)
    return np.ascontiguousarray(x[..., rev])


def reference_input_order_2d(x, radices_x, radices_y):
    """tcfft_doit_half_2d.cpp:40-50: position (j, k) gets x[rev_x[j], rev_y[k]]."""
    rx = gen_rev(x.shape[-2], radices_x)
    ry = gen_rev(x.shape[-1], radices_y)
    return np.ascontiguousarray(x[..., rx, :][..., :, ry])


# ---------------------------------------------------------------- reference kernels on the GPU
REF_DIR = os.path.join(HERE, "_ref")


def reference_gpu_available():
    return (os.path.exists(os.path.join(REF_DIR, "tcfft_half_ref.cubin"))
            and os.path.exists(os.path.join(HERE, "_build", "libref_runner.so")))


_RUNNER = None


def _runner():
    global _RUNNER
    if _RUNNER is None:
        lib = ctypes.CDLL(os.path.join(HERE, "_build", "libref_runner.so"))
        c = ctypes
        lib.ref_exec_1d.argtypes = [c.c_char_p, c.c_char_p, c.c_ulonglong, c.c_int, c.c_int, c.c_int, c.c_int]
        lib.ref_exec_2d.argtypes = [c.c_char_p, c.c_char_p, c.c_ulonglong, c.c_int, c.c_int, c.c_int, c.c_int,
                                    c.c_int]
        _RUNNER = lib
    return _RUNNER


# Kernel families of the reference: "volta" is what tcfftCreate binds
# (tcfft_half.cu:1244-1248); "a100" the sm_80 fragment-map twins it never binds.
REFERENCE_FAMILIES = {"volta": 0, "a100": 1}


def reference_gpu_fft_1d(dev_ptr, n, batch, family="volta", sync=True):
    """Run the reference's own kernels (compiled from its sources for sm_103a)
    in place on digit-reversed half2 data at device address `dev_ptr`."""
    r = _runner().ref_exec_1d(os.path.join(REF_DIR, "tcfft_half_ref.cubin").encode(),
                              os.path.join(REF_DIR, "tcfft_half_kernels.txt").encode(), dev_ptr, n, batch,
                              REFERENCE_FAMILIES[family], int(bool(sync)))
    if r != 0:
        raise RuntimeError("reference 1D kernels failed: code %d" % r)


def reference_gpu_fft_2d(dev_ptr, nx, ny, batch, family="volta", sync=True):
    r = _runner().ref_exec_2d(os.path.join(REF_DIR, "tcfft_half_2d_ref.cubin").encode(),
                              os.path.join(REF_DIR, "tcfft_half_2d_kernels.txt").encode(), dev_ptr, nx, ny, batch,
                              REFERENCE_FAMILIES[family], int(bool(sync)))
    if r != 0:
        raise RuntimeError("reference 2D kernels failed: code %d" % r)
