"""GPU: the parity bar -- on the same seeded inputs, the rel-L2 error of this
library's plain path against the FP64 oracle is no worse than that of the
reference's own tcFFT kernels compiled from its sources for sm_103a and run on
the same GPU (oracle/ref_runner.cpp restates tcfftExec's launch sequence).

Both kernel families of the reference run: "volta", the kernels tcfftCreate
binds (tcfft_half.cu:1244-1248), whose hard-coded Volta WMMA fragment map
does not hold on sm_103a (their output is unrelated to the DFT: rel-L2 ~1.4),
and "a100", the sm_80 fragment-map twins the reference ships but never binds.
The bar is the better of the two.

Inputs: the benchmark workloads' uniform[-1,1) and the reference generator's own
distribution (uniform[0, 1e-4), doit.h:7-19, drawn with numpy).  Sizes: the
reference's supported sizes (test.sh:26-65)."""
import json
import os

import numpy as np
import pytest
import torch

import oracle
import tcfft_gb300 as tc
from fftcheck import oracle_1d, oracle_2d, quantize, run_gpu, to_complex

pytestmark = pytest.mark.gpu

RESULTS = []


def _inputs(shape, kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        return rng.uniform(-1, 1, tuple(shape) + (2,))
    return rng.uniform(0, 1e-4, tuple(shape) + (2,))


def _ref_run_1d(xq, n, batch, family):
    xr = oracle.reference_input_order_1d(xq[..., 0] + 1j * xq[..., 1], oracle.reference_radices(n))
    t = torch.from_numpy(np.stack([xr.real, xr.imag], -1)).half().cuda()
    torch.cuda.synchronize()
    oracle.reference_gpu_fft_1d(t.data_ptr(), n, batch, family)
    return to_complex(t.double().cpu().numpy())


def _ref_run_2d(xq, nx, ny, family):
    rx, ry = oracle.reference_radices_2d_axis(nx), oracle.reference_radices_2d_axis(ny)
    xr = oracle.reference_input_order_2d(xq[..., 0] + 1j * xq[..., 1], rx, ry)
    t = torch.from_numpy(np.stack([xr.real, xr.imag], -1)).half().cuda()
    torch.cuda.synchronize()
    oracle.reference_gpu_fft_2d(t.data_ptr(), nx, ny, xq.shape[0], family)
    return to_complex(t.double().cpu().numpy())


def _finite_rel_l2(y, ref):
    return oracle.rel_l2(y, ref) if np.isfinite(y).all() else float("inf")


@pytest.fixture(scope="module", autouse=True)
def _require_reference():
    if not oracle.reference_gpu_available():
        pytest.skip("reference cubin not built (oracle/_ref)")
    yield
    out_dir = os.environ.get("TCFFT_PARITY_OUT")  # optional: directory for the per-size table
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        with open(os.path.join(out_dir, "reference_parity.json"), "w") as f:
            json.dump(RESULTS, f, indent=1)


@pytest.mark.parametrize("kind", ["uniform", "reference_generator"])
@pytest.mark.parametrize("n,batch", [(256, 32), (512, 32), (1024, 32), (131072, 1), (262144, 1), (524288, 1),
                                     (1 << 24, 1)])
def test_no_worse_than_reference_1d(cuda_device, n, batch, kind):
    x = _inputs((batch, n), kind, seed=42)
    xq = quantize(x, "plain")
    ref64 = oracle.fft_1d(x[..., 0] + 1j * x[..., 1])  # FP64 on the unrounded doubles (accuracy.cpp:71-72)
    rec = {"n": n, "batch": batch, "input": kind}
    for fam in ("volta", "a100"):
        y_ref = _ref_run_1d(xq, n, batch, fam)
        rec["rel_l2_reference_" + fam] = _finite_rel_l2(y_ref, ref64)
        rec["clipped_reference_" + fam] = oracle.clipped_error(y_ref, ref64)
    with tc.Plan(n=n, batch=batch) as p:
        y_ours = run_gpu(p, xq, "plain")
    e_ours = oracle.rel_l2(y_ours, ref64)
    rec.update(rel_l2_ours=e_ours, clipped_ours=oracle.clipped_error(y_ours, ref64))
    RESULTS.append(rec)
    e_ref = min(rec["rel_l2_reference_volta"], rec["rel_l2_reference_a100"])
    assert np.isfinite(y_ours).all()
    assert e_ours <= e_ref * 1.05 + 1e-7, "ours %.3e vs reference %.3e" % (e_ours, e_ref)


@pytest.mark.parametrize("nx,ny", [(256, 256), (256, 512), (512, 512), (256, 1024), (512, 1024)])
def test_no_worse_than_reference_2d(cuda_device, nx, ny):
    x = _inputs((1, nx, ny), "uniform", seed=1)
    xq = quantize(x, "plain")
    ref64 = oracle.fft_2d(x[..., 0] + 1j * x[..., 1])
    rec = {"nx": nx, "ny": ny, "input": "uniform"}
    for fam in ("volta", "a100"):
        rec["rel_l2_reference_" + fam] = _finite_rel_l2(_ref_run_2d(xq, nx, ny, fam), ref64)
    with tc.Plan(nx=nx, ny=ny, batch=1) as p:
        y_ours = run_gpu(p, xq, "plain")
    e_ours = oracle.rel_l2(y_ours, ref64)
    rec["rel_l2_ours"] = e_ours
    RESULTS.append(rec)
    e_ref = min(rec["rel_l2_reference_volta"], rec["rel_l2_reference_a100"])
    assert e_ours <= e_ref * 1.05 + 1e-7, "ours %.3e vs reference %.3e" % (e_ours, e_ref)
