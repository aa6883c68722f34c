"""CPU: the C-ABI library loads, exports every symbol include/*.h declares,
and its host-only entry points behave (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

import tcfft_gb300 as tc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if not fname.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fname)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        in_c = "extern \"C\"" in src or fname == "tcfft_gb300.h"
        if not in_c:
            continue
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s+\*?(tcfft[A-Za-z0-9_]*)\s*\(",
                             src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = tc.lib()
    decl = declared_symbols()
    assert len(decl) >= 12
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) <= set(tc.exported_symbols()) | set(decl)


def test_bindings_cover_header():
    assert set(declared_symbols()) == set(tc.exported_symbols())


def test_error_strings_and_version():
    lib = tc.lib()
    for s in range(9):
        assert lib.tcfftGetErrorString(s)
    assert b"sm_103a" in lib.tcfftVersion()


@pytest.mark.parametrize("n", [256, 512, 1024, 2048])
def test_describe_small(n):
    assert "small" in tc.describe_1d(n, 4)


@pytest.mark.parametrize("n", [4096, 1 << 15, 1 << 16, 1 << 20, 1 << 22])
def test_describe_fused(n):
    assert "fused1d" in tc.describe_1d(n, 4)


@pytest.mark.parametrize("n,batch", [(100, 1), (8, 1), (0, 1), (256, 0), (1 << 28, 1)])
def test_describe_rejects_bad_sizes(n, batch):
    with pytest.raises(tc.TcfftError) as e:
        tc.describe_1d(n, batch)
    assert e.value.status == 2


def test_describe_rejects_bad_precision():
    with pytest.raises(tc.TcfftError) as e:
        tc.describe_1d(256, 1, precision=7)
    assert e.value.status == 1


def test_null_arguments():
    lib = tc.lib()
    assert lib.tcfftPlan1d(None, 256, 1, None) == 1
    assert lib.tcfftExecute(None, None, None) == 8
    assert lib.tcfftDestroy(None) == 8
    assert lib.tcfftOptionsDefault(None) == 1
