"""The reference's benchmark seam -- setup / doit / finalize (doit.h:2-4,
doit_2d.h:2-4, implemented in the reference by tcfft_doit_half.cpp:31-67 and its
2D twin) -- as shipped here: tcfft_gb300/doit/gb300_doit_half.cpp and
gb300_doit_half_2d.cpp, over the compat headers include/tcfft_half.h /
tcfft_half_2d.h.

tests/doit_seam.cpp drives that seam the way the reference's speed.cpp:45-64 does
(the reference's drivers are not shipped; test_compat_headers.py links them with
the seam and this library where their sources are present).  Each is built here
into a shared library, once per header and per input order: natural order (the
handle reports radices = {N}, the permutation is the identity) and
TCFFT_REFERENCE_INPUT_ORDER (the handle reports the reference's radix chain, the
seam digit-reverses on the host as the reference's harness does, and the library
undoes it on the GPU).

CPU: the seam's input permutation equals the oracle's restatement of the
reference's gen_rev (tcfft_doit_half.cpp:6-29) for every reference radix chain.
GPU: finalize's output equals the FP64 oracle's DFT of the fp16-rounded data,
for data drawn like the reference's generate_data (uniform [0, 1e-4),
doit.h:5-17) and for unit-scale data; doit(2) gives N x[-k]."""
import ctypes
import functools
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from fftcheck import tol_plain

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "tcfft_gb300")
CUDA = "/usr/local/cuda"
_TMP = tempfile.mkdtemp(prefix="tcfft_seam_")


@functools.lru_cache(maxsize=None)
def seam_lib(two_d, reference_order):
    if not os.path.exists(os.path.join(LIBDIR, "libtcfft_gb300.so")):
        pytest.skip("libtcfft_gb300.so not built")
    out = os.path.join(_TMP, "seam_%d_%d.so" % (two_d, reference_order))
    seam = os.path.join(ROOT, "tcfft_gb300", "doit", "gb300_doit_half_2d.cpp" if two_d else "gb300_doit_half.cpp")
    cmd = ["g++", "-std=c++14", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "tcfft_gb300", "doit"), "-I", CUDA + "/include", seam,
           os.path.join(ROOT, "tests", "doit_seam.cpp"), "-o", out,
           "-L", LIBDIR, "-ltcfft_gb300", "-Wl,-rpath," + LIBDIR, "-L", CUDA + "/lib64", "-lcudart",
           "-Wl,-rpath," + CUDA + "/lib64"]
    if two_d:
        cmd.insert(1, "-DSEAM_2D")
    if reference_order:
        cmd.insert(1, "-DTCFFT_REFERENCE_INPUT_ORDER")
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    lib = ctypes.CDLL(out)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    lib.seam_run.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    lib.seam_radices.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ctypes.c_int]
    lib.seam_permutation.argtypes = [ctypes.c_int, ip, ctypes.c_int, ip]
    return lib


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


@pytest.mark.parametrize("n", [256, 512, 1024, 1 << 17, 1 << 18, 1 << 19, 1 << 24])
def test_seam_permutation_matches_reference_gen_rev(n):
    lib = seam_lib(False, False)
    chain = oracle.reference_radices(n)
    rad = np.array(chain, dtype=np.int32)
    rev = np.empty(n, dtype=np.int32)
    lib.seam_permutation(n, _ptr(rad, ctypes.c_int), len(chain), _ptr(rev, ctypes.c_int))
    assert np.array_equal(rev, oracle.gen_rev(n, chain))


def harness_data(shape, seed):
    """Values like the reference's generate_data: real and imaginary parts uniform in [0, 1e-4)."""
    return np.random.default_rng(seed).uniform(0, 1e-4, tuple(shape) + (2,))


def unit_data(shape, seed):
    return np.random.default_rng(seed).uniform(-1, 1, tuple(shape) + (2,))


def run_seam(data, two_d, reference_order, iters=1):
    lib = seam_lib(two_d, reference_order)
    data = np.ascontiguousarray(data, dtype=np.float64)
    out = np.zeros_like(data)
    if two_d:
        batch, nx, ny = data.shape[:3]
    else:
        (batch, nx), ny = data.shape[:2], 1
    st = lib.seam_run(_ptr(data, ctypes.c_double), nx, ny, batch, iters, _ptr(out, ctypes.c_double))
    assert st == 0, "seam_run failed (status %d)" % st
    return out


def _c(a):
    return a[..., 0] + 1j * a[..., 1]


# harness-scale data reaches fp16's subnormal range (< 6.1e-5) on input: relative error grows
_SCALES = {"harness": (harness_data, 4.0), "unit": (unit_data, 1.0)}

SHAPES_1D = [(256, 64), (1024, 16), (4096, 8), (1 << 17, 2), (1 << 20, 2), (1 << 24, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("reference_order", [False, True], ids=["natural", "reference-order"])
@pytest.mark.parametrize("scale", sorted(_SCALES))
@pytest.mark.parametrize("n,batch", SHAPES_1D)
def test_seam_1d(cuda_device, n, batch, scale, reference_order):
    gen, slack = _SCALES[scale]
    x = gen((batch, n), seed=n % 97 + batch)
    if reference_order:
        want = oracle.reference_radices(n)
        if want is None:
            # the reference's input order exists only for its own sizes: plan creation fails,
            # the seam reports it instead of transforming
            lib = seam_lib(False, True)
            data = np.ascontiguousarray(x)
            out = np.zeros_like(data)
            assert lib.seam_run(_ptr(data, ctypes.c_double), n, 1, batch, 1, _ptr(out, ctypes.c_double)) == 1
            return
        rad = np.zeros(16, dtype=np.int32)
        k = seam_lib(False, True).seam_radices(n, 1, batch, _ptr(rad, ctypes.c_int), 16)
        assert list(rad[:k]) == want
    else:
        rad = np.zeros(16, dtype=np.int32)
        k = seam_lib(False, False).seam_radices(n, 1, batch, _ptr(rad, ctypes.c_int), 16)
        assert list(rad[:k]) == [n]
    y = run_seam(x, False, reference_order)
    xq = x.astype(np.float16).astype(np.float64)
    ref = oracle.fft_1d(_c(xq))
    err = oracle.rel_l2(_c(y), ref)
    assert np.isfinite(y).all() and err < slack * tol_plain(n), "rel-L2 %.3e" % err


SHAPES_2D = [(256, 256, 8), (512, 512, 4), (256, 1024, 2), (1024, 1024, 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("reference_order", [False, True], ids=["natural", "reference-order"])
@pytest.mark.parametrize("nx,ny,batch", SHAPES_2D)
def test_seam_2d(cuda_device, nx, ny, batch, reference_order):
    x = harness_data((batch, nx, ny), seed=nx + ny + batch)
    if reference_order:
        want = (oracle.reference_radices_2d_axis(nx) or []) + (oracle.reference_radices_2d_axis(ny) or [])
        rad = np.zeros(16, dtype=np.int32)
        k = seam_lib(True, True).seam_radices(nx, ny, batch, _ptr(rad, ctypes.c_int), 16)
        assert list(rad[:k]) == want
    y = run_seam(x, True, reference_order)
    xq = x.astype(np.float16).astype(np.float64)
    ref = oracle.fft_2d(_c(xq))
    err = oracle.rel_l2(_c(y), ref)
    assert np.isfinite(y).all() and err < 4.0 * tol_plain(nx * ny), "rel-L2 %.3e" % err


@pytest.mark.gpu
def test_seam_doit_twice(cuda_device):
    """doit(2) applies the forward transform twice: F F x = N x[(-k) mod N] (natural
    order; in the reference's order every execute reads its input digit-reversed, so
    the second one permutes the first one's output, as in the reference)."""
    n, batch = 4096, 4
    x = unit_data((batch, n), seed=12) / 64
    y = run_seam(x, False, False, iters=2)
    xq = x.astype(np.float16).astype(np.float64)
    want = n * _c(xq)[:, (-np.arange(n)) % n]
    err = oracle.rel_l2(_c(y), want)
    assert np.isfinite(y).all() and err < 2 * tol_plain(n), "rel-L2 %.3e" % err
