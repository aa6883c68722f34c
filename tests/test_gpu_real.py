"""GPU: out-of-place execution (tcfftExecuteOutOfPlace) and real transforms
(tcfftPlanReal1d, tcfftExecuteR2C / tcfftExecuteC2R) through the C ABI.

Out of place must give exactly the in-place result (the same kernels, the
input read through another tensor map) and leave the input untouched, on
every schedule kind.  Real transforms are checked against the FP64 oracle:
R2C against the first n/2 + 1 bins of the complex DFT of the real input, C2R
against 1/n times the sign +1 transform of the full Hermitian spectrum
(imaginary parts of X[0] and X[n/2] ignored), and round trips
c2r(r2c(x)) = x with the 1/n on either side."""
import numpy as np
import pytest

import oracle
import tcfft_gb300 as tc
from fftcheck import quantize, to_complex, tol, tol_plain, uniform_input

pytestmark = pytest.mark.gpu

OOP = [dict(n=64, batch=37), dict(n=1024, batch=9), dict(n=4096, batch=5), dict(n=8192, batch=3, precision="split"),
       dict(n=1 << 15, batch=3), dict(n=1 << 16, batch=3), dict(n=1 << 18, batch=2, precision="split"),
       dict(n=1 << 20, batch=2), dict(n=1 << 23, batch=1), dict(nx=512, ny=512, batch=2),
       dict(nx=128, ny=128, batch=3), dict(n=2048, batch=3, precision="split")]


@pytest.mark.parametrize("shape", OOP, ids=lambda d: "-".join(str(v) for v in d.values()))
def test_out_of_place_equals_in_place(cuda_device, shape):
    import torch
    prec = shape.get("precision", "plain")
    kw = {k: v for k, v in shape.items() if k != "precision"}
    dims = (kw["batch"], kw["n"]) if "n" in kw else (kw["batch"], kw["nx"], kw["ny"])
    xq = quantize(uniform_input(dims, seed=sum(dims) % 97), prec)
    dt = torch.float16 if prec == "plain" else torch.float32
    src = torch.from_numpy(xq).to(dt).to(cuda_device)
    keep = src.clone()
    with tc.Plan(precision=prec, **kw) as p:
        ref = src.clone()
        p.exec(ref)
        out = torch.full_like(src, 3.0)
        p.exec_out(src, out)
        p.check_device()
        assert torch.equal(src, keep), "the input was modified"
        assert torch.equal(out, ref), "out of place differs from in place (%s)" % p.info["schedule"]
        # a second call with another output buffer (tensor maps re-encoded)
        out2 = torch.zeros_like(src)
        p.exec_out(src, out2)
        p.check_device()
        assert torch.equal(out2, ref)


REAL = [(32, 5, "plain"), (256, 6, "plain"), (1024, 4, "split"), (4096, 3, "plain"), (8192, 3, "split"),
        (1 << 16, 2, "plain"), (1 << 17, 2, "split"), (1 << 20, 2, "plain"), (1 << 22, 1, "plain"),
        (64, 7, "split")]


def _full_spectrum(X, n):
    """Hermitian extension of X[0..n/2] to n bins (imaginary parts of X[0], X[n/2] dropped)."""
    Xh = X.copy()
    Xh[..., 0] = Xh[..., 0].real
    Xh[..., n // 2] = Xh[..., n // 2].real
    return np.concatenate([Xh, np.conj(Xh[..., n // 2 - 1:0:-1])], axis=-1)


@pytest.mark.parametrize("n,batch,precision", REAL)
def test_r2c_c2r(cuda_device, n, batch, precision):
    import torch
    rng = np.random.default_rng(n % 101 + batch)
    dt_np = np.float16 if precision == "plain" else np.float32
    dt = torch.float16 if precision == "plain" else torch.float32
    x = rng.uniform(-1, 1, (batch, n)).astype(dt_np)
    xt = torch.from_numpy(x).to(cuda_device)
    keep = xt.clone()
    spec = torch.empty((batch, n // 2 + 1, 2), dtype=dt, device=cuda_device)
    with tc.RealPlan(n, batch, precision=precision) as p:
        p.r2c(xt, spec)
        p.check_device()
        assert torch.equal(xt, keep), "R2C modified its input"
        X = to_complex(spec.double().cpu().numpy())
        ref = oracle.fft_1d(x.astype(np.float64) + 0j)[:, : n // 2 + 1]
        err = oracle.rel_l2(X, ref)
        assert np.isfinite(X).all() and err < tol(precision, n), "R2C n=%d: rel-L2 %.3e" % (n, err)
        # C2R of a Hermitian half (with junk imaginary parts at bins 0 and n/2, ignored)
        # spectrum-sized values (|X| ~ sqrt(n)), so that the 1/n output is O(1)
        Xin = quantize(uniform_input((batch, n // 2 + 1), seed=n % 89) * np.sqrt(n) / 2, precision)
        Xin[:, 0, 1] = 0.5
        Xin[:, -1, 1] = -0.25
        st = torch.from_numpy(Xin).to(dt).to(cuda_device)
        skeep = st.clone()
        y = torch.empty((batch, n), dtype=dt, device=cuda_device)
        p.c2r(st, y)
        p.check_device()
        assert torch.equal(st, skeep), "C2R modified its input"
    yr = y.double().cpu().numpy()
    full = _full_spectrum(to_complex(Xin), n)
    ref = oracle.fft_1d(full, sign=+1) / n  # the default C2R carries the 1/n
    assert np.abs(ref.imag).max() < 1e-9 * np.abs(ref.real).max()
    err = oracle.rel_l2(yr, ref.real)
    assert np.isfinite(yr).all() and err < tol(precision, n), "C2R n=%d: rel-L2 %.3e" % (n, err)


@pytest.mark.parametrize("n,precision", [(256, "plain"), (1 << 16, "plain"), (1 << 20, "split")])
@pytest.mark.parametrize("normalize", [False, True])
def test_real_round_trip(cuda_device, n, precision, normalize):
    """C2R is the inverse of R2C: c2r(r2c(x)) = x with the 1/n on either side."""
    import torch
    dt = torch.float16 if precision == "plain" else torch.float32
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, (2, n)).astype(np.float16 if precision == "plain" else np.float32)
    xt = torch.from_numpy(x).to(cuda_device)
    spec = torch.empty((2, n // 2 + 1, 2), dtype=dt, device=cuda_device)
    y = torch.empty_like(xt)
    with tc.RealPlan(n, 2, precision=precision, normalize=normalize) as p:
        p.r2c(xt, spec)
        p.c2r(spec, y)
        p.check_device()
    got = y.double().cpu().numpy()
    assert np.isfinite(got).all()
    assert oracle.rel_l2(got, x.astype(np.float64)) < 2 * tol(precision, n)
    X = to_complex(spec.double().cpu().numpy())
    ref = oracle.fft_1d(x.astype(np.float64) + 0j)[:, : n // 2 + 1] / (n if normalize else 1)
    assert oracle.rel_l2(X, ref) < tol(precision, n)


def test_real_plan_rejects_bad_use(cuda_device):
    import torch
    with pytest.raises(tc.TcfftError):
        tc.RealPlan(48, 1)          # not a power of two
    with pytest.raises(tc.TcfftError):
        tc.RealPlan(16, 1)          # below 32 points
    with tc.RealPlan(1024, 1) as p:
        t = torch.zeros((1, 1024), dtype=torch.float16, device="cuda")
        with pytest.raises(tc.TcfftError):
            p.exec(t)               # a real plan has no complex execute


REAL2D = [(64, 128, 3, "plain"), (256, 256, 2, "plain"), (1024, 512, 2, "plain"), (16, 64, 5, "plain"),
          (256, 2048, 1, "split"), (512, 64, 2, "split"), (64, 512, 3, "split"), (256, 1024, 2, "fp32io")]


@pytest.mark.parametrize("nx,ny,batch,precision", REAL2D)
def test_real_2d(cuda_device, nx, ny, batch, precision):
    """R2C 2D against the FP64 2D DFT's first ny/2 + 1 columns; C2R 2D against
    numpy's FP64 irfft2 of the same half spectrum; the round trip returns x."""
    import torch
    h = ny // 2 + 1
    bound = tol_plain(nx * ny) if precision == "fp32io" else tol(precision, nx * ny)  # fp16 arithmetic
    rng = np.random.default_rng(nx + ny + batch)
    dt_np = np.float16 if precision == "plain" else np.float32
    dt = torch.float16 if precision == "plain" else torch.float32
    x = rng.uniform(-1, 1, (batch, nx, ny)).astype(dt_np)
    xt = torch.from_numpy(x).to(cuda_device)
    spec = torch.empty((batch, nx, h, 2), dtype=dt, device=cuda_device)
    y = torch.empty_like(xt)
    with tc.RealPlan(nx=nx, ny=ny, batch=batch, precision=precision) as p:
        assert "real2d" in p.info["schedule"], p.info["schedule"]
        p.r2c(xt, spec)
        p.check_device()
        X = to_complex(spec.double().cpu().numpy())
        ref = oracle.fft_2d(x.astype(np.float64) + 0j)[..., :h]
        err = oracle.rel_l2(X, ref)
        assert np.isfinite(X).all() and err < bound, "R2C %dx%d: rel-L2 %.3e" % (nx, ny, err)
        p.c2r(spec, y)
        p.check_device()
        back = y.double().cpu().numpy()
        assert oracle.rel_l2(back, x.astype(np.float64)) < 2 * bound
        # C2R of a spectrum with arbitrary values (numpy's irfft2 semantics)
        Xin = quantize(uniform_input((batch, nx, h), seed=nx % 37) * np.sqrt(nx * ny) / 2, precision)
        st = torch.from_numpy(Xin).to(dt).to(cuda_device)
        keep = st.clone()
        p.c2r(st, y)
        p.check_device()
        assert torch.equal(st, keep), "C2R modified its input"
    want = np.fft.irfft2(to_complex(Xin), s=(nx, ny))
    got = y.double().cpu().numpy()
    err = oracle.rel_l2(got, want)
    assert np.isfinite(got).all() and err < bound, "C2R %dx%d: rel-L2 %.3e" % (nx, ny, err)
