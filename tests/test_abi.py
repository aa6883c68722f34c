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
    assert ("resident" if n in (4096, 1 << 15) else "fused1d") in tc.describe_1d(n, 4)


@pytest.mark.parametrize("n,precision,expect", [
    (4096, 1, "resident(split)"), (8192, 1, "resident(split)"), (16384, 0, "resident(plain)"),
    (1 << 15, 0, "resident(plain): N=256 x 128"), (1 << 15, 1, "N=512 x 64"), (2048, 1, "small(R=8,split)"),
    (1 << 21, 0, "N=1024 x 2048"), (1 << 21, 1, "large1d(split): N=512 x 4096"),
    (1 << 23, 0, "large1d(plain): N=2048 x 4096"), (1 << 20, 0, "N=1024 x 1024")])
def test_describe_schedule_choice(n, precision, expect):
    """The planner's size -> schedule table (host logic only, no device work)."""
    assert expect in tc.describe_1d(n, 4, precision=precision)


@pytest.mark.parametrize("nx,ny,precision,expect", [
    (1024, 1024, 0, "fused2d(plain): 1024 x 1024"), (256, 2048, 0, "fused2d(plain): 256 x 2048"),
    (2048, 2048, 0, "fused2d(plain)"), (512, 512, 1, "fused2d(split)"), (1024, 1024, 2, "fused2d(fp32io)"),
    (2048, 256, 1, "generic2d(split): rows of 256, transpose, rows of 2048"),
    (128, 128, 0, "generic2d(plain): rows of 128"), (4096, 4096, 0, "generic2d(plain): rows of 4096"),
    (64, 4096, 0, "generic2d(plain): rows of 4096, transpose, rows of 64")])
def test_describe_2d_schedule_choice(nx, ny, precision, expect):
    """The 2D planner (host logic only): the fused kernel for axes of 256..2048 (8-byte
    elements: up to 1024), 1D plans and transposes otherwise."""
    assert expect in tc.describe_2d(nx, ny, 4, precision=precision)


@pytest.mark.parametrize("nx,ny,batch", [(100, 256, 1), (256, 3000, 1), (256, 256, 0), (1 << 28, 2, 1)])
def test_describe_2d_rejects_bad_shapes(nx, ny, batch):
    with pytest.raises(tc.TcfftError) as e:
        tc.describe_2d(nx, ny, batch)
    assert e.value.status == 2


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
    assert lib.tcfftExecuteHost(None, None, None, None, None) == 8
    assert lib.tcfftDestroy(None) == 8
    assert lib.tcfftOptionsDefault(None) == 1


def test_plan_many_rejects_bad_layouts():
    """Argument checks of tcfftPlanMany happen before any device work."""
    import ctypes
    lib = tc.lib()

    def call(shapes, offsets):
        n = len(shapes)
        ranks = (ctypes.c_int32 * max(n, 1))(*[len(s) for s in shapes])
        nx = (ctypes.c_int64 * max(n, 1))(*[s[0] for s in shapes])
        ny = (ctypes.c_int64 * max(n, 1))(*[s[1] if len(s) > 1 else 1 for s in shapes])
        off = (ctypes.c_int64 * max(n, 1))(*offsets)
        h = ctypes.c_void_p(None)
        return lib.tcfftPlanMany(ctypes.byref(h), n, ranks, nx, ny, off, None)

    assert call([], []) == 1                              # TCFFT_INVALID_VALUE: empty
    assert call([(256,)], [3]) == 3                       # TCFFT_MISALIGNED: 12-byte offset
    assert call([(256,), (256,)], [0, 128]) == 1          # overlapping transforms
    assert call([(100,)], [0]) == 2                       # TCFFT_INVALID_SIZE


@pytest.mark.parametrize("field,value", [("direction", 2), ("direction", -1), ("normalization", 3),
                                         ("precision", 5), ("input_order", 7)])
def test_plan_rejects_bad_options_before_touching_the_gpu(field, value):
    """Option validation is host logic: bad values return TCFFT_INVALID_VALUE."""
    lib = tc.lib()
    opts = tc.Options()
    assert lib.tcfftOptionsDefault(ctypes.byref(opts)) == 0
    assert opts.direction == tc.FORWARD and opts.normalization == tc.NORM_NONE
    setattr(opts, field, value)
    h = ctypes.c_void_p(None)
    assert lib.tcfftPlan1d(ctypes.byref(h), 1024, 4, ctypes.byref(opts)) == 1
    assert lib.tcfftPlan2d(ctypes.byref(h), 256, 256, 4, ctypes.byref(opts)) == 1
    assert not h.value


def test_options_struct_layout_matches_header():
    """The ctypes mirror of tcfftOptions has the header's size (pointer-aligned)."""
    assert ctypes.sizeof(tc.Options) == 32


@pytest.mark.parametrize("n,batch,istride,idist,kw,status", [
    (256, 48, 48, 1, {}, 7),                        # not whole 32-column tiles
    (4096, 32, 32, 1, {}, 7),                       # columns longer than 2048
    (512, 64, 32, 1, {"precision": "split"}, 7),   # element strides: plain precision only
    (512, 64, 32, 1, {"normalize": True}, 7),      # normalised inverse needs the per-shape graph
    (512, 65, 32, 1, {}, 7),                        # batch not a multiple of the stride
    (512, 64, 32, 2, {}, 7),                        # both strides
    (1024, 4, 1, 512, {}, 1),                       # transforms would overlap
    (1000, 4, 1, 1000, {}, 2),                      # not a power of two
    (1024, 0, 1, 1024, {}, 1)])                     # empty batch
def test_strided_layouts_refused_before_touching_the_gpu(n, batch, istride, idist, kw, status):
    """tcfftPlanStrided's layout checks are host logic: they run before any device call."""
    with pytest.raises(tc.TcfftError) as e:
        tc.Plan.strided(n, batch, istride=istride, idist=idist, **kw)
    assert e.value.status == status


@pytest.mark.parametrize("n", [1 << 12, 1 << 15, 1 << 16, 1 << 18, 1 << 20, 1 << 22])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_two_phase_ring_sizing(n, precision):
    """Two-phase schedules keep a scratch ring of S = 2 D + 2 slots for a lag of D transforms
    between a transform's phase 0 and phase 1, 1 <= D <= batch, D not shrinking as the batch
    grows (host logic; the kernels' cross-CTA waits rely on it)."""
    import re
    last = 0
    for batch in [1, 2, 3, 5, 8, 64, 256, 4096]:
        if n * batch > 1 << 31:
            break
        text = tc.describe_1d(n, batch, precision=precision)
        m = re.search(r"lag (\d+), (\d+) slots", text)
        if not m:  # resident, composite or single-pass schedules have no ring
            assert "fused1d" not in text, text
            continue
        d, slots = int(m.group(1)), int(m.group(2))
        assert slots == 2 * d + 2 and 1 <= d <= batch, text
        assert d >= last, "lag shrank with a larger batch: " + text
        last = d


# The planner's 1D schedule by log2 N, plain and 8-byte-element precisions (split and fp32 I/O
# share their schedules); "-" is TCFFT_NOT_SUPPORTED (no 128-point split / fp32-I/O path).
SUPPORT_1D = {
    "plain": ["tiny"] * 4 + ["small"] * 4 + ["resident"] * 4 + ["fused1d"] * 7 + ["large1d"] * 5,
    "8-byte": ["tiny"] * 3 + ["-"] + ["small"] * 4 + ["resident"] * 2 + ["fused1d"] * 7 + ["large1d"] * 7,
}


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_1d_support_matrix(precision):
    """Every power of two 16..2^27 in plain precision, and all but 128 in split / fp32 I/O."""
    expect = SUPPORT_1D["plain" if precision == 0 else "8-byte"]
    for lg in range(4, 28):
        want = expect[lg - 4]
        if want == "-":
            with pytest.raises(tc.TcfftError) as e:
                tc.describe_1d(1 << lg, 1, precision=precision)
            assert e.value.status == 7
        else:
            assert tc.describe_1d(1 << lg, 1, precision=precision).startswith(want), (lg, want)
    for bad in (8, 1 << 28, 3 << 10):
        with pytest.raises(tc.TcfftError) as e:
            tc.describe_1d(bad, 1, precision=precision)
        assert e.value.status == 2


def test_reference_order_sizes_match_the_oracle_table():
    """Plans in the reference's digit-reversed input order exist exactly for the sizes the
    reference's planner defines (the oracle's table, pinned against the reference's host code):
    other sizes are refused with TCFFT_INVALID_SIZE before any device work."""
    import oracle
    lib = tc.lib()
    opts = tc.Options()
    assert lib.tcfftOptionsDefault(ctypes.byref(opts)) == 0
    opts.input_order = 1  # TCFFT_ORDER_REFERENCE_DIGIT_REVERSED
    for lg in range(4, 28):
        h = ctypes.c_void_p(None)
        st = lib.tcfftPlan1d(ctypes.byref(h), 1 << lg, 1, ctypes.byref(opts))
        if st == 0:
            lib.tcfftDestroy(h)
        assert (st == 2) == (oracle.reference_radices(1 << lg) is None), (lg, st)
    for ax in range(7, 12):
        for ay in range(7, 12):
            h = ctypes.c_void_p(None)
            st = lib.tcfftPlan2d(ctypes.byref(h), 1 << ax, 1 << ay, 1, ctypes.byref(opts))
            if st == 0:
                lib.tcfftDestroy(h)
            ok = oracle.reference_radices_2d_axis(1 << ax) is not None and \
                oracle.reference_radices_2d_axis(1 << ay) is not None
            assert (st == 2) == (not ok), (ax, ay, st)
