"""CPU: drop-in compatibility at the source level.

* include/tcfft_gb300.h is valid C (the C ABI).
* The reference's own harness (tcfft_doit_half.cpp, speed.cpp and their 2D
  twins) compiles unchanged against include/tcfft_half.h /
  include/tcfft_half_2d.h.  The reference sources are read from where they
  lie (copied to a temporary directory outside the repository only so that
  their `#include "tcfft_half.h"` resolves to this library's header); the test
  is skipped where the reference is not present.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
CUDA_INC = "/usr/local/cuda/include"
from oracle.build import REFERENCE  # noqa: E402 - the reference source directory (TCFFT_REFERENCE_DIR)


def _gxx(args, cwd):
    return subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I", INC, "-I", CUDA_INC] + args, cwd=cwd,
                          stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


def test_c_abi_header_is_c():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write('#include "tcfft_gb300.h"\nint main(void){ tcfftOptions o; tcfftOptionsDefault(&o);'
                    ' tcfftPlan p = 0; (void)p; return (int)TCFFT_SUCCESS; }\n')
        r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-I", INC, src], stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout


@pytest.mark.skipif(not os.path.isdir(REFERENCE), reason="reference sources not present")
@pytest.mark.parametrize("files", [["tcfft_doit_half.cpp", "speed.cpp", "doit.h"],
                                   ["tcfft_doit_half_2d.cpp", "speed_2d.cpp", "doit_2d.h"]])
def test_reference_harness_compiles_against_shims(files):
    with tempfile.TemporaryDirectory() as d:
        for f in files:
            shutil.copy(os.path.join(REFERENCE, f), d)
        for f in files:
            if f.endswith(".cpp"):
                r = _gxx([f], d)
                assert r.returncode == 0, r.stdout


@pytest.mark.skipif(not os.path.isdir(REFERENCE), reason="reference sources not present")
@pytest.mark.parametrize("reference_order", [False, True], ids=["natural", "reference-order"])
@pytest.mark.parametrize("seam", ["reference", "gb300"])
@pytest.mark.parametrize("files", [["tcfft_doit_half.cpp", "speed.cpp", "doit.h"],
                                   ["tcfft_doit_half_2d.cpp", "speed_2d.cpp", "doit_2d.h"]])
def test_reference_harness_links_against_library(files, seam, reference_order):
    """The reference's speed programs (speed.cpp / speed_2d.cpp, main over the
    setup/doit/finalize seam) build into executables linked with libtcfft_gb300.so,
    in both input orders, with either the reference's own seam (tcfft_doit_half*.cpp
    over the compat headers) or the one shipped here (tcfft_gb300/doit/
    gb300_doit_half*.cpp).  They need a GPU to run; tests/test_doit_seam.py runs
    the shipped seam on one.  accuracy.cpp needs FFTW, absent here."""
    lib = os.path.join(ROOT, "tcfft_gb300", "libtcfft_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("libtcfft_gb300.so not built")
    doit_dir = os.path.join(ROOT, "tcfft_gb300", "doit")
    with tempfile.TemporaryDirectory() as d:
        for f in files:
            shutil.copy(os.path.join(REFERENCE, f), d)
        sources = [f for f in files if f.endswith(".cpp")]
        if seam == "gb300":
            two_d = "2d" in files[0]
            sources[0] = os.path.join(doit_dir, "gb300_doit_half_2d.cpp" if two_d else "gb300_doit_half.cpp")
        objs = []
        for k, f in enumerate(sources):
            o = "obj%d.o" % k
            args = ["g++", "-std=c++14", "-O1", "-c", "-I", INC, "-I", doit_dir, "-I", CUDA_INC, f, "-o", o]
            if reference_order:
                args.insert(1, "-DTCFFT_REFERENCE_INPUT_ORDER")
            r = subprocess.run(args, cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            assert r.returncode == 0, r.stdout
            objs.append(o)
        r = subprocess.run(["g++"] + objs + ["-o", "harness", "-L", os.path.dirname(lib), "-ltcfft_gb300",
                                             "-L", "/usr/local/cuda/lib64", "-lcudart", "-lm"],
                           cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout
        assert os.path.getsize(os.path.join(d, "harness")) > 0
