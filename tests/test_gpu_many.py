"""GPU: uneven batches in one plan (tcfftPlanMany) -- the mixed 1D/2D
workload of 512 1D transforms of 2^8..2^16 points and 64 2D transforms of
128..1024 per axis (seed 2), packed back to back in one device buffer, run
through a CUDA graph replayed on every execute -- and the plan-time
autotuner.  No reference counterpart (the reference plans one size per
handle)."""
import numpy as np
import pytest
import torch

import oracle
import tcfft_gb300 as tc
from fftcheck import quantize, to_complex, tol, tol_plain

pytestmark = pytest.mark.gpu


def mixed_shapes(seed=2):
    rng = np.random.default_rng(seed)
    shapes = [(1 << int(e),) for e in rng.integers(8, 17, size=512)]
    shapes += [(1 << int(a), 1 << int(b)) for a, b in rng.integers(7, 11, size=(64, 2))]
    order = rng.permutation(len(shapes))
    return [shapes[i] for i in order]


def pack(shapes, seed, precision):
    rng = np.random.default_rng(seed)
    parts = [quantize(rng.uniform(-1, 1, tuple(s) + (2,)), precision) for s in shapes]
    flat = np.concatenate([p.reshape(-1, 2) for p in parts])
    return parts, flat


def unpack(flat, shapes):
    out, off = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(flat[off:off + n].reshape(tuple(s) + (2,)))
        off += n
    return out


def check(parts, ys, precision, adjoint=False):
    """Every transform within the bound of its own size."""
    sign = +1 if adjoint else -1
    worst = 0.0
    for x, y in zip(parts, ys):
        ref = oracle.fft_1d(to_complex(x), sign) if x.ndim == 2 else oracle.fft_2d(to_complex(x), sign)
        err = oracle.rel_l2(to_complex(y), ref)
        bound = tol(precision, int(np.prod(x.shape[:-1])))
        assert err < bound, "shape %s: rel-L2 %.3e >= %.3e" % (x.shape[:-1], err, bound)
        worst = max(worst, err / bound)
    return worst


@pytest.mark.parametrize("precision", ["plain", "split"])
def test_mixed_batch(cuda_device, precision):
    shapes = mixed_shapes()
    if precision == "split":  # the split mode stops at 64 points below 256: keep axes >= 256
        shapes = [s for s in shapes if all(v >= 256 for v in s)]
    parts, flat = pack(shapes, 5, precision)
    dt = torch.float16 if precision == "plain" else torch.float32
    p = tc.Plan.many(shapes, precision=precision)
    try:
        assert "many" in p.info["schedule"]
        base = torch.from_numpy(flat).to(dt).cuda()
        for _ in range(2):  # first call captures the graph, the second replays it
            buf = base.clone()
            p.exec(buf)
            p.check_device()
            check(parts, unpack(buf.double().cpu().numpy(), shapes), precision)
        buf = base.clone()
        p.exec(buf, adjoint=True)
        p.check_device()
        check(parts, unpack(buf.double().cpu().numpy(), shapes), precision, adjoint=True)
        other = torch.zeros(flat.shape[0] + 64, 2, dtype=dt, device="cuda")[64:]  # another pointer
        other.copy_(base)
        p.exec(other)
        p.check_device()
        check(parts, unpack(other.double().cpu().numpy(), shapes), precision)
    finally:
        p.destroy()


def test_contiguous_runs_share_one_launch(cuda_device):
    shapes = [(256,)] * 10 + [(1024,)] * 5 + [(64, 128)] * 3
    parts, flat = pack(shapes, 9, "plain")
    with tc.Plan.many(shapes) as p:
        assert "in 3 runs" in p.info["schedule"], p.info["schedule"]
        buf = torch.from_numpy(flat).half().cuda()
        p.exec(buf)
        p.check_device()
    check(parts, unpack(buf.double().cpu().numpy(), shapes), "plain")


def test_gapped_offsets(cuda_device):
    shapes = [(512,), (512,), (2048,)]
    offsets = [0, 1024, 4096]  # a gap between every transform: three runs
    parts, _ = pack(shapes, 4, "plain")
    buf = torch.full((8192, 2), 7.0, dtype=torch.float16, device="cuda")
    for x, o in zip(parts, offsets):
        buf[o:o + x.shape[0]] = torch.from_numpy(x).half()
    with tc.Plan.many(shapes, offsets=offsets) as p:
        p.exec(buf)
        p.check_device()
    got = buf.double().cpu().numpy()
    ys = [got[o:o + x.shape[0]] for x, o in zip(parts, offsets)]
    check(parts, ys, "plain")
    assert (got[512:1024] == 7.0).all() and (got[2048:4096] == 7.0).all()  # gaps untouched


def test_autotune(cuda_device, tmp_path):
    cache = str(tmp_path / "tune.txt")
    n, batch = 1 << 16, 64
    rng = np.random.default_rng(3)
    xq = quantize(rng.uniform(-1, 1, (batch, n, 2)), "plain")
    with tc.Plan(n=n, batch=batch, autotune=True, tune_cache_path=cache) as p:
        assert "tuned" in p.info["schedule"]
        t = torch.from_numpy(xq).half().cuda()
        p.exec(t)
        p.check_device()
    err = oracle.rel_l2(to_complex(t.double().cpu().numpy()), oracle.fft_1d(to_complex(xq)))
    assert err < tol_plain(n)
    with open(cache) as f:
        assert "|" in f.read()


def test_autotune_decomposition(cuda_device, tmp_path):
    """The tuner times the 1D decompositions N1 x N2 and item sizes, then the lag; the
    choice is cached as "key|lag|N1|item KiB" and reused by a later plan."""
    cache = str(tmp_path / "tune.txt")
    n, batch = 1 << 20, 6
    rng = np.random.default_rng(5)
    xq = quantize(rng.uniform(-1, 1, (batch, n, 2)), "plain")
    with tc.Plan(n=n, batch=batch, autotune=True, tune_cache_path=cache) as p:
        text = p.info["schedule"]
        assert "tuned: N1=" in text, text
        t = torch.from_numpy(xq).half().cuda()
        p.exec(t)
        p.check_device()
    err = oracle.rel_l2(to_complex(t.double().cpu().numpy()), oracle.fft_1d(to_complex(xq)))
    assert err < tol_plain(n)
    with open(cache) as f:
        fields = f.read().strip().split("|")
    assert len(fields) == 4 and int(fields[2]) in (512, 1024, 2048) and int(fields[3]) in (32, 64), fields
    with tc.Plan(n=n, batch=batch, autotune=True, tune_cache_path=cache) as p2:
        assert p2.info["schedule"] == text  # served from the cache


def test_autotune_cache_file_forms(cuda_device, tmp_path):
    """Older "key|lag" lines still load; a cached decomposition the build cannot run
    (N1 = 4096 leaves N2 = 128) falls back to the built-in schedule."""
    n = 1 << 19
    cache = tmp_path / "tune.txt"
    cache.write_text("1 %d 1 3 0|1.600\n1 %d 1 5 0|1.000|4096|64\n" % (n, n))
    rng = np.random.default_rng(9)
    for batch, expect in ((3, "lag x1.6"), (5, "lag x1]")):
        xq = quantize(rng.uniform(-1, 1, (batch, n, 2)), "plain")
        with tc.Plan(n=n, batch=batch, autotune=True, tune_cache_path=str(cache)) as p:
            assert expect in p.info["schedule"], p.info["schedule"]
            t = torch.from_numpy(xq).half().cuda()
            p.exec(t)
            p.check_device()
        err = oracle.rel_l2(to_complex(t.double().cpu().numpy()), oracle.fft_1d(to_complex(xq)))
        assert err < tol_plain(n)


# Shapes of every work-item kind of the persistent many-shape passes (fft_many.cu):
# 1D 256..2048 listed rows, 4096..16384 / 2^15 / 2^16 column + row phases, 2D rows and
# columns of 128..2048 (128: the 16-per-warp kinds).
PASS_SHAPES = [(256,), (512,), (1024,), (2048,), (4096,), (8192,), (16384,), (1 << 15,), (1 << 16,),
               (128, 128), (128, 256), (256, 128), (512, 1024), (1024, 512), (2048, 256), (256, 2048),
               (128, 2048), (2048, 128), (256,), (2048,), (4096,), (1 << 16,)]


@pytest.mark.parametrize("adjoint", [False, True])
def test_many_pass_every_kind(cuda_device, adjoint):
    """One plan over every kind, at gapped offsets (gaps untouched), forward and
    adjoint, each transform against FP64; at most two launches per execute."""
    shapes = PASS_SHAPES
    parts, _ = pack(shapes, 21, "plain")
    offsets, at = [], 0
    for s in shapes:
        offsets.append(at)
        at += int(np.prod(s)) + 96  # a 384-byte gap after every transform
    buf = torch.full((at, 2), 5.0, dtype=torch.float16, device="cuda")
    for x, o in zip(parts, offsets):
        buf[o:o + x.reshape(-1, 2).shape[0]] = torch.from_numpy(x.reshape(-1, 2)).half()
    with tc.Plan.many(shapes, offsets=offsets) as p:
        assert "persistent" in p.info["schedule"], p.info["schedule"]
        assert p.info["launches_per_exec"] <= 2
        p.exec(buf, adjoint=adjoint)
        p.check_device()
    got = buf.double().cpu().numpy()
    ys = [got[o:o + int(np.prod(s))].reshape(tuple(s) + (2,)) for s, o in zip(shapes, offsets)]
    check(parts, ys, "plain", adjoint=adjoint)
    for s, o in zip(shapes, offsets):
        e = o + int(np.prod(s))
        assert (got[e:e + 96] == 5.0).all(), "gap after %s written" % (s,)


def test_many_pass_agrees_with_graph(cuda_device, monkeypatch):
    """The persistent passes and the per-shape graph (TCFFT_MANY_GRAPH=1) both meet
    each transform's bound on the uneven-batch workload; the normalised execute of a
    pass plan takes the graph."""
    shapes = mixed_shapes()
    parts, flat = pack(shapes, 7, "plain")
    base = torch.from_numpy(flat).half().cuda()
    outs = {}
    for mode in ("pass", "graph"):
        if mode == "graph":
            monkeypatch.setenv("TCFFT_MANY_GRAPH", "1")
        with tc.Plan.many(shapes) as p:
            assert ("persistent" in p.info["schedule"]) == (mode == "pass"), p.info["schedule"]
            buf = base.clone()
            p.exec(buf)
            p.check_device()
            outs[mode] = buf.double().cpu().numpy()
            check(parts, unpack(outs[mode], shapes), "plain")
    monkeypatch.delenv("TCFFT_MANY_GRAPH")
    with tc.Plan.many(shapes, normalize=True) as p:
        buf = base.clone()
        p.exec(buf)
        p.check_device()
        ys = unpack(buf.double().cpu().numpy(), shapes)
    for x, y in zip(parts, ys):
        n = int(np.prod(x.shape[:-1]))
        ref = (oracle.fft_1d(to_complex(x)) if x.ndim == 2 else oracle.fft_2d(to_complex(x))) / n
        assert oracle.rel_l2(to_complex(y), ref) < tol_plain(n)


def test_many_pass_out_of_place_and_host(cuda_device):
    """Out of place (the input copied into the output buffer, then the one launch) equals
    in place, leaves the input untouched, and so does the host-buffer execute."""
    shapes = [(2048,), (1 << 15,), (128, 512), (1024, 256), (4096,)]
    parts, flat = pack(shapes, 13, "plain")
    with tc.Plan.many(shapes) as p:
        src = torch.from_numpy(flat).half().cuda()
        keep = src.clone()
        ref = src.clone()
        p.exec(ref)
        out = torch.zeros_like(src)
        p.exec_out(src, out)
        p.check_device()
        assert torch.equal(src, keep)
        assert torch.equal(out, ref)
        h_in = torch.from_numpy(flat).half().pin_memory()
        h_out = torch.empty_like(h_in).pin_memory()
        work = torch.empty_like(src)
        p.exec_host(h_in, h_out, work)
        torch.cuda.synchronize()
        p.check_device()
        assert torch.equal(h_out, ref.cpu())
    check(parts, unpack(out.double().cpu().numpy(), shapes), "plain")


@pytest.mark.parametrize("seed", [31, 32, 33])
def test_many_pass_random_batches(cuda_device, seed):
    """Random uneven batches over every shape the one-launch executor takes (1D 2^8..2^16,
    2D axes 2^7..2^11), random 128-byte-aligned gaps, both directions, each transform
    against FP64 and every gap untouched."""
    rng = np.random.default_rng(seed)
    count = int(rng.integers(20, 60))
    shapes = []
    for _ in range(count):
        if rng.random() < 0.6:
            shapes.append((1 << int(rng.integers(8, 17)),))
        else:
            shapes.append((1 << int(rng.integers(7, 12)), 1 << int(rng.integers(7, 12))))
    shapes = [s for s in shapes if int(np.prod(s)) <= 1 << 20]
    parts, _ = pack(shapes, seed, "plain")
    offsets, at = [], 0
    for s in shapes:
        at += 32 * int(rng.integers(0, 4))  # 0..3 gaps of 128 bytes
        offsets.append(at)
        at += int(np.prod(s))
    buf = torch.full((at + 64, 2), 3.0, dtype=torch.float16, device="cuda")
    for x, o in zip(parts, offsets):
        buf[o:o + x.reshape(-1, 2).shape[0]] = torch.from_numpy(x.reshape(-1, 2)).half()
    adjoint = bool(seed % 2)
    with tc.Plan.many(shapes, offsets=offsets) as p:
        assert "persistent" in p.info["schedule"], p.info["schedule"]
        p.exec(buf, adjoint=adjoint)
        p.check_device()
    got = buf.double().cpu().numpy()
    ys = [got[o:o + int(np.prod(s))].reshape(tuple(s) + (2,)) for s, o in zip(shapes, offsets)]
    check(parts, ys, "plain", adjoint=adjoint)
    covered = np.zeros(got.shape[0], dtype=bool)
    for s, o in zip(shapes, offsets):
        covered[o:o + int(np.prod(s))] = True
    assert (got[~covered] == 3.0).all(), "a gap was written"
