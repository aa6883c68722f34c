"""Benchmark: batched half-precision FFT throughput on GB300.

Workload (default): 1D complex-to-complex forward FFT, N = 2^20, batch 256,
so one call transforms 2^28 complex fp16 elements (1 GiB, larger than the
126 MB L2); real/imag iid uniform[-1, 1) (numpy PCG64, seed 0), generated
synthetically (no dataset).  Metric: GFLOP/s = 5 N log2(N) batch / t.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n N] [--batch B]
                  [--precision plain|split] [--impl ours|reference] [--no-sweep]

One JSON line is printed by rank 0.  Under torchrun (N > 1) every rank runs
an independent replica on its own GPU (the path shards by transform, no
collective), timing is max over ranks and `value` is the whole-job
aggregate ("scaling": "weak").

Keys beyond the base contract: `roofline` (dominant kernel vs the measured
HBM copy bandwidth), `cpu_baseline` (the FP64 CPU FFT of oracle/ on the host
cores, bounded sample), `e2e` (host buffers through the public API, copies
inside the timed region), `clocks` (nvidia-smi sampled during the timed
region), `sweep` (N = 2^8 .. 2^24 at 2^28 elements per call, with rel-L2 vs
FP64 per N on the timed plans, uniform inputs and the tone variant) and
`accuracy` (rel-L2 vs numpy's FP64 FFT: a separate sample, plain and split, and
the timed plan itself on sampled transforms).

With --impl reference it times the reference's CPU path (FFTW in the
reference, absent here: the oracle's FP64 port) for exactly the steps it
reports, one bounded sample of the workload per step.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001 - file optional
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(workload_key):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/traffic.txt: '<workload> <bytes_per_launch>')."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == workload_key:
                    return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.device_index = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def flops_per_call(size, batch):
    return 5.0 * size * math.log2(size) * batch


def make_plan(tc, args, size_args, batch):
    return tc.Plan(batch=batch, precision=args.precision, **size_args)


def time_device(torch, plan, x, steps, warmup, dist=None):
    """W warm-up calls, then K calls timed with CUDA events on the current stream."""
    for _ in range(warmup):
        plan.exec(x)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        plan.exec(x)
    e1.record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    plan.check_device()
    return e0.elapsed_time(e1) / 1000.0  # seconds for K calls


def rel_l2_numpy(y, ref):
    import numpy as np
    return float(np.linalg.norm((y - ref).ravel()) / np.linalg.norm(ref.ravel()))


def accuracy_sample(torch, tc, size_args, precision, seed=0, count=2):
    """rel-L2 against numpy's FP64 FFT on `count` transforms of the workload."""
    import numpy as np
    n = size_args.get("n")
    shape = (count, n) if n else (count, size_args["nx"], size_args["ny"])
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.0, 1.0, shape + (2,))
    dt = np.float16 if precision == "plain" else np.float32
    t = torch.from_numpy(x.astype(dt)).cuda()
    with tc.Plan(batch=count, precision=precision, **size_args) as p:
        p.exec(t)
        p.check_device()
    return compare_fp64(t.double().cpu().numpy(), x, precision, two_d=not n)


def compare_fp64(y, x, precision, two_d=False):
    """rel-L2 of the result y against numpy's FP64 FFT of the inputs x (float64
    [..., 2]) as given (unrounded) and as the kernel saw them (rounded)."""
    import numpy as np
    dt = np.float16 if precision == "plain" else np.float32
    xq = x.astype(dt).astype(np.float64)
    yc = y[..., 0] + 1j * y[..., 1]
    fft = np.fft.fft2 if two_d else (lambda a: np.fft.fft(a, axis=-1))
    ref = fft(xq[..., 0] + 1j * xq[..., 1])
    refu = fft(x[..., 0] + 1j * x[..., 1])
    finite = np.isfinite(yc)
    out = {"rel_l2_vs_fp64_on_rounded_inputs": rel_l2_numpy(np.where(finite, yc, 0), ref),
           "rel_l2_vs_fp64_on_unrounded_inputs": rel_l2_numpy(np.where(finite, yc, 0), refu),
           "nonfinite": int((~finite).sum()), "transforms": int(np.prod(y.shape[:-2 if not two_d else -3]))}
    return out


def tone_input(n, count, seed=0):
    """Three unit-amplitude complex tones (bins and phases from default_rng(seed + 100))
    over N(0, 1e-3) noise, float64 [count, n, 2]: |X_k| ~ n at the tone bins."""
    import numpy as np
    rng = np.random.default_rng(seed + 100)
    bins = rng.integers(0, n, 3)
    phases = rng.uniform(0, 2 * np.pi, 3)
    idx = np.arange(n)
    z = sum(np.exp(1j * (2 * np.pi * ((int(k) * idx) % n) / n + ph)) for k, ph in zip(bins, phases))
    x = np.empty((count, n, 2))
    noise = rng.normal(0.0, 1e-3, (count, n, 2))
    x[..., 0] = z.real + noise[..., 0]
    x[..., 1] = z.imag + noise[..., 1]
    return x


def sample_rows(batch, count):
    """Transforms checked in a batch: the first two, two in the middle, the last two."""
    rows = sorted({0, 1, batch // 2 - 1, batch // 2, batch - 2, batch - 1})
    return [r for r in rows if 0 <= r < batch][:count]


def plan_accuracy(torch, plan, x_dev, precision, n, batch, kind="uniform", seed=0):
    """Run `plan` (the timed one) once on its own buffer after writing seeded inputs
    into sampled transforms (first, middle, last); returns rel-L2 against FP64 on them."""
    import numpy as np
    rows = sample_rows(batch, 6)
    max_elems = 1 << 22
    while len(rows) > 1 and len(rows) * n > max_elems:
        rows = rows[::2]
    if kind == "tone":
        x = tone_input(n, len(rows), seed)
    else:
        x = np.random.default_rng(seed).uniform(-1.0, 1.0, (len(rows), n, 2))
    dt = np.float16 if precision == "plain" else np.float32
    for i, r in enumerate(rows):
        x_dev[r].copy_(torch.from_numpy(x[i].astype(dt)))
    plan.exec(x_dev)
    plan.check_device()
    y = torch.stack([x_dev[r] for r in rows]).double().cpu().numpy()
    out = compare_fp64(y, x, precision)
    out["rows"] = rows
    return out


def cpu_baseline(size_args, budget_s=10.0):
    """The oracle's FP64 CPU FFT (oracle/fft64.c, OpenMP) on the host cores,
    timed on a bounded sample of the workload's transforms; scipy.fft
    (pocketfft, all host threads) on the same sample is reported beside it."""
    import numpy as np
    import oracle
    n = size_args.get("n")
    size = n if n else size_args["nx"] * size_args["ny"]
    threads = oracle.num_threads()
    rng = np.random.default_rng(0)
    per = max(1, threads)
    x = rng.uniform(-1, 1, (per, size)) + 1j * rng.uniform(-1, 1, (per, size))
    if n:
        run = lambda: oracle.fft_1d(x)  # noqa: E731
    else:
        xx = x.reshape(per, size_args["nx"], size_args["ny"])
        run = lambda: oracle.fft_2d(xx)  # noqa: E731
    run()  # warm
    done, t0 = 0, time.perf_counter()
    while True:
        run()
        done += per
        el = time.perf_counter() - t0
        if el > budget_s or done >= 4096:
            break
    gflops = flops_per_call(size, done) / el / 1e9
    out = {"value": gflops, "unit": "GFLOP/s", "cores": threads, "kind": "port",
           "sample": "%d transforms of the workload size (FP64, oracle/fft64.c, %d OpenMP threads), %.1f s"
                     % (done, threads, el)}
    try:
        out["scipy"] = scipy_baseline(size_args, x, budget_s=min(budget_s, 5.0))
    except Exception as e:  # noqa: BLE001 - informational
        out["scipy_error"] = str(e)[:200]
    return out


def scipy_baseline(size_args, x, budget_s=5.0):
    """scipy.fft (pocketfft) complex128 and complex64 with workers = all host threads."""
    import numpy as np
    import scipy.fft as sf
    n = size_args.get("n")
    size = x.shape[-1]
    workers = os.cpu_count() or 1
    res = {"cores": workers, "what": "scipy.fft %s, workers=%d" % ("fft" if n else "fft2", workers)}
    for name, dt in (("complex128", np.complex128), ("complex64", np.complex64)):
        xx = x.astype(dt) if n else x.astype(dt).reshape(x.shape[0], size_args["nx"], size_args["ny"])
        f = (lambda a: sf.fft(a, axis=-1, workers=workers)) if n else (lambda a: sf.fft2(a, workers=workers))
        f(xx)
        done, t0 = 0, time.perf_counter()
        while True:
            f(xx)
            done += x.shape[0]
            el = time.perf_counter() - t0
            if el > budget_s / 2 or done >= 4096:
                break
        res[name + "_gflops"] = round(flops_per_call(size, done) / el / 1e9, 2)
    return res


def sweep(torch, tc, precision, lgs=range(8, 25), total=1 << 28, accuracy=True):
    """1D sizes at `total` elements per call (the size-sweep workload): time per
    call, and -- on the timed plan, after timing -- rel-L2 against FP64 on sampled
    transforms for uniform inputs and for the tone variant, with non-finite counts."""
    out = []
    peak, _ = measured_peak()
    es = 4 if precision == "plain" else 8
    for lg in lgs:
        n = 1 << lg
        batch = max(1, total // n)
        dt = torch.float16 if precision == "plain" else torch.float32
        x = torch.empty((batch, n, 2), dtype=dt, device="cuda").uniform_(-1, 1)
        with tc.Plan(n=n, batch=batch, precision=precision) as p:
            sec = time_device(torch, p, x, 5, 3) / 5
            row = {"n": n, "batch": batch, "us": round(sec * 1e6, 1),
                   "gflops": round(flops_per_call(n, batch) / sec / 1e9, 1),
                   "hbm_frac_of_measured": round(2 * es * n * batch / sec / 1e9 / peak, 3)}
            if accuracy:
                u = plan_accuracy(torch, p, x, precision, n, batch, "uniform", seed=lg)
                tn = plan_accuracy(torch, p, x, precision, n, batch, "tone", seed=lg)
                row["rel_l2"] = float("%.3e" % u["rel_l2_vs_fp64_on_rounded_inputs"])
                row["rel_l2_unrounded"] = float("%.3e" % u["rel_l2_vs_fp64_on_unrounded_inputs"])
                row["tone_rel_l2"] = float("%.3e" % tn["rel_l2_vs_fp64_on_unrounded_inputs"])
                row["tone_nonfinite"] = tn["nonfinite"]
                row["checked_transforms"] = len(u["rows"])
        out.append(row)
        del x
        torch.cuda.empty_cache()
    return out


def flops_2d(nx, ny, batch):
    return 5.0 * nx * ny * math.log2(nx * ny) * batch


def sweep_2d(torch, tc):
    """The 2D workloads: 1024^2 x 16, 4096^2 x 1, 256^2 x 1024 (plain; 1024^2 also split)."""
    out = []
    peak, _ = measured_peak()
    for nx, ny, batch, prec in ((1024, 1024, 16, "plain"), (4096, 4096, 1, "plain"), (256, 256, 1024, "plain"),
                                (1024, 1024, 16, "split")):
        es = 4 if prec == "plain" else 8
        dt = torch.float16 if prec == "plain" else torch.float32
        x = torch.empty((batch, nx, ny, 2), dtype=dt, device="cuda").uniform_(-1, 1)
        with tc.Plan(nx=nx, ny=ny, batch=batch, precision=prec) as p:
            sec = time_device(torch, p, x, 10, 3) / 10
            sched = p.info["schedule"]
        out.append({"nx": nx, "ny": ny, "batch": batch, "precision": prec, "us": round(sec * 1e6, 1),
                    "gflops": round(flops_2d(nx, ny, batch) / sec / 1e9, 1),
                    "hbm_frac_of_measured": round(2 * es * nx * ny * batch / sec / 1e9 / peak, 3),
                    "schedule": sched.split(":")[0]})
        del x
        torch.cuda.empty_cache()
    return out


def uneven_shapes():
    """The uneven-batch workload's shapes: 512 1D transforms of 2^8..2^16 and 64 2D transforms
    of 2^7..2^10 per axis (seed 2), shuffled."""
    import numpy as np
    rng = np.random.default_rng(2)
    shapes = [(1 << int(e),) for e in rng.integers(8, 17, size=512)]
    shapes += [(1 << int(a), 1 << int(b)) for a, b in rng.integers(7, 11, size=(64, 2))]
    return [shapes[i] for i in rng.permutation(len(shapes))]


def uneven_batch(torch, tc, graph=False):
    """The uneven-batch workload (uneven_shapes), back to back in one buffer, one plan: the
    persistent many-shape passes, or (graph=True) the per-shape sub-plans replayed as one CUDA
    graph."""
    import numpy as np
    shapes = uneven_shapes()
    elems = sum(int(np.prod(sh)) for sh in shapes)
    flops = sum(5.0 * int(np.prod(sh)) * math.log2(int(np.prod(sh))) for sh in shapes)
    x = torch.empty((elems, 2), dtype=torch.float16, device="cuda").uniform_(-1, 1)
    peak, _ = measured_peak()
    if graph:
        os.environ["TCFFT_MANY_GRAPH"] = "1"
    try:
        with tc.Plan.many(shapes) as p:
            sec = time_device(torch, p, x, 20, 3) / 20
            info = p.info
    finally:
        os.environ.pop("TCFFT_MANY_GRAPH", None)
    return {"transforms": len(shapes), "elements": elems, "us": round(sec * 1e6, 1),
            "gflops": round(flops / sec / 1e9, 1), "hbm_frac_of_measured": round(8 * elems / sec / 1e9 / peak, 3),
            "launches_per_replay": info["launches_per_exec"], "schedule": info["schedule"]}


def cufft_fp16(torch, size_args, batch):
    """cuFFT half precision (through torch.fft on complex32) on the same workload: a reported
    GPU baseline (out of place), not the reference."""
    n = size_args.get("n")
    if not n:
        return None
    x = torch.empty((batch, n, 2), dtype=torch.float16, device="cuda").uniform_(-1, 1)
    xc = torch.view_as_complex(x)
    for _ in range(3):
        y = torch.fft.fft(xc)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        y = torch.fft.fft(xc)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000.0 / 10
    del y, xc, x
    torch.cuda.empty_cache()
    return {"gflops": round(flops_per_call(n, batch) / sec / 1e9, 1), "us": round(sec * 1e6, 1),
            "what": "torch.fft.fft on complex32 (cuFFT fp16), out of place"}


def reference_arm(size_args, size, args, config, metric, world):
    """The reference's CPU path is FFTW fp64 (accuracy.cpp:11-23), absent here; its
    restatement in oracle/ (fft64.c, OpenMP over transforms) runs on the host cores
    with all threads.  Every step is one bounded sample of the workload -- one
    transform per host thread -- and exactly the W + K steps the line reports are
    run, K of them timed."""
    import numpy as np
    import oracle
    threads = oracle.num_threads()
    per = max(1, threads)
    n = size_args.get("n")
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (per, size)) + 1j * rng.uniform(-1, 1, (per, size))
    if n:
        run = lambda: oracle.fft_1d(x)  # noqa: E731
    else:
        xx = x.reshape(per, size_args["nx"], size_args["ny"])
        run = lambda: oracle.fft_2d(xx)  # noqa: E731
    for _ in range(args.warmup):
        run()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run()
    el = time.perf_counter() - t0
    value = flops_per_call(size, per) * args.steps / el / 1e9
    try:  # informational, outside the timed CPU steps
        ref_gpu = reference_gpu_timings()
    except Exception as e:  # noqa: BLE001
        ref_gpu = {"error": str(e)[:200]}
    sample = ("%d transforms of the workload size per step (one per host thread; FP64, oracle/fft64.c, "
              "%d OpenMP threads), %d timed steps in %.2f s" % (per, threads, args.steps, el))
    return {"impl": "reference", "metric": metric, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic uniform[-1,1)", "config": config,
            "cpu_baseline": {"value": round(value, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu": ref_gpu}


def reference_gpu_timings(total=1 << 28, reps=5):
    """Informational: the reference's own GPU kernels (compiled from its sources for sm_103a,
    driven by oracle/ref_runner.cpp, which restates tcfftExec's launch sequence) timed with
    CUDA events at its supported sizes, 2^28 elements per call.  "a100" are the kernels that
    compute the DFT on this GPU; "volta" the ones tcfftCreate binds (wrong output on sm_103a)."""
    import torch
    import oracle
    if not torch.cuda.is_available() or not oracle.reference_gpu_available():
        return {"unavailable": "no GPU or reference kernels not built"}
    peak, _ = measured_peak()
    out = []
    buf = torch.zeros((total, 2), dtype=torch.float16, device="cuda")
    cases = [((n,), total // n) for n in (256, 512, 1024, 1 << 17, 1 << 18, 1 << 19, 1 << 24)]
    cases += [((256, 256), total // 65536), ((512, 512), total // 262144), ((256, 1024), total // 262144)]
    for shape, batch in cases:
        for fam in ("a100", "volta"):
            run = ((lambda: oracle.reference_gpu_fft_1d(buf.data_ptr(), shape[0], batch, fam, sync=False))
                   if len(shape) == 1 else
                   (lambda: oracle.reference_gpu_fft_2d(buf.data_ptr(), shape[0], shape[1], batch, fam, sync=False)))
            try:
                for _ in range(2):
                    run()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    run()
                e1.record()
                torch.cuda.synchronize()
                sec = e0.elapsed_time(e1) / 1000.0 / reps
                size = int(math.prod(shape))
                out.append({"shape": list(shape), "batch": batch, "family": fam, "us": round(sec * 1e6, 1),
                            "gflops": round(flops_per_call(size, batch) / sec / 1e9, 1),
                            "hbm_frac_of_measured": round(8 * total / sec / 1e9 / peak, 3)})
            except Exception as e:  # noqa: BLE001 - informational
                out.append({"shape": list(shape), "family": fam, "error": str(e)[:120]})
    del buf
    torch.cuda.empty_cache()
    return out


def copy_ceiling(torch, host_in, host_out, dev_a, dev_b, reps=5):
    """Pinned host<->device copies of one step's bytes: H2D alone, D2H alone, and
    both at once on two streams (the bound of a pipelined host-buffer call)."""
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    out = {}
    for name, what in (("h2d", "in"), ("d2h", "out"), ("both", "both")):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        cur = torch.cuda.current_stream()
        for _ in range(reps):
            s_in.wait_stream(cur)
            s_out.wait_stream(cur)
            if what in ("in", "both"):
                with torch.cuda.stream(s_in):
                    dev_a.copy_(host_in, non_blocking=True)
            if what in ("out", "both"):
                with torch.cuda.stream(s_out):
                    host_out.copy_(dev_b, non_blocking=True)
            cur.wait_stream(s_in)
            cur.wait_stream(s_out)
        e1.record()
        torch.cuda.synchronize()
        out[name + "_ms"] = round(e0.elapsed_time(e1) / reps, 3)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--nx", type=int, default=0)
    ap.add_argument("--ny", type=int, default=0)
    ap.add_argument("--batch", type=int, default=0, help="default: 2^28 elements per call")
    ap.add_argument("--precision", default="plain", choices=["plain", "split"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--profile", action="store_true",
                    help="only the warm-up and timed calls (for ncu captures); prints the time per call")
    ap.add_argument("--uneven", action="store_true",
                    help="with --profile: the uneven-batch plan (tcfftPlanMany of the bench's 576 shapes)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.nx and args.ny:
        size_args = {"nx": args.nx, "ny": args.ny}
        size = args.nx * args.ny
        wl = "2D C2C forward FFT %dx%d" % (args.nx, args.ny)
    else:
        size_args = {"n": args.n}
        size = args.n
        wl = "1D C2C forward FFT N=2^%d" % int(math.log2(args.n))
    batch = args.batch or max(1, (1 << 28) // size)
    es = 4 if args.precision == "plain" else 8
    metric = "FFT GFLOP/s (5Nlog2N/t)"
    config = {"workload": "%s, batch %d (%d complex elements per call), %s, interleaved %s"
                          % (wl, batch, batch * size, args.precision,
                             "half2" if args.precision == "plain" else "float2 (hi/lo fp16 products)"),
              "n": size_args.get("n"), "nx": size_args.get("nx"), "ny": size_args.get("ny"),
              "batch": batch, "precision": args.precision,
              "l2": "inputs larger than L2 (%d MiB per call vs 126 MB L2), no flush" % (batch * size * es >> 20),
              "parallelism": "replicas x%d" % world}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(size_args, size, args, config, metric, world)), flush=True)
        return

    import torch
    import tcfft_gb300 as tc
    from tcfft_gb300.replicas import max_over_ranks

    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
        dist = tdist
    else:
        torch.cuda.set_device(0)
    dev_index = torch.cuda.current_device()

    if args.profile and args.uneven:
        import numpy as np
        shapes = uneven_shapes()
        elems = sum(int(np.prod(sh)) for sh in shapes)
        xu = torch.empty((elems, 2), dtype=torch.float16, device="cuda").uniform_(-1, 1)
        with tc.Plan.many(shapes) as p:
            secs = time_device(torch, p, xu, args.steps, args.warmup)
            print(json.dumps({"profile_run": p.info["schedule"], "ms_per_call": secs / args.steps * 1e3}), flush=True)
        return

    dt = torch.float16 if args.precision == "plain" else torch.float32
    gen = torch.Generator(device="cuda")
    gen.manual_seed(rank)
    shape = (batch, size, 2)
    x = torch.empty(shape, dtype=dt, device="cuda").uniform_(-1, 1, generator=gen)
    plan = make_plan(tc, args, size_args, batch)
    info = plan.info
    if args.profile:
        secs = time_device(torch, plan, x, args.steps, args.warmup, dist)
        if rank == 0:
            print(json.dumps({"profile_run": info["schedule"], "ms_per_call": secs / args.steps * 1e3}), flush=True)
        plan.destroy()
        return

    # ---------------- device-resident timing (value) + clocks
    sampler = ClockSampler(dev_index)
    sampler.start()
    time.sleep(0.3)  # let nvidia-smi start sampling before the timed region
    secs = time_device(torch, plan, x, args.steps, args.warmup, dist)
    clocks = sampler.stop()
    secs = max_over_ranks(secs, dist, device="cuda")
    per_call = secs / args.steps
    value = flops_per_call(size, batch) * world / per_call / 1e9

    # ---------------- roofline of the dominant (only) kernel per call
    peak, peak_kind = measured_peak()
    alg_bytes = 2 * es * size * batch
    achieved = alg_bytes / per_call / 1e9
    wkey = "%s_%s_%d" % (args.precision, "x".join(str(v) for v in ([args.nx, args.ny] if args.nx else [args.n])),
                         batch)
    traffic = profile_traffic(wkey)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes_per_launch": alg_bytes,
                "kernel": info["schedule"]}

    # ---------------- e2e through the public API with host buffers
    host_in = torch.empty(shape, dtype=dt, pin_memory=True)
    host_in.uniform_(-1, 1)
    host_out = torch.empty_like(host_in, pin_memory=True)
    # tcfftExecuteHost: copy in, transform and copy out pipelined over chunks of the batch
    stream = torch.cuda.current_stream()
    for _ in range(2):
        plan.exec_host(host_in, host_out, x, stream=stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2e_steps = max(10, args.steps // 4)
    e0.record()
    for _ in range(e2e_steps):
        plan.exec_host(host_in, host_out, x, stream=stream)
    e1.record()
    torch.cuda.synchronize()
    e2e_s = e0.elapsed_time(e1) / 1000.0 / e2e_steps
    e2e_s = max_over_ranks(e2e_s, dist, device="cuda")
    e2e = {"value": round(flops_per_call(size, batch) * world / e2e_s / 1e9, 1), "unit": "GFLOP/s",
           "h2d_bytes_per_step": host_in.numel() * host_in.element_size(),
           "d2h_bytes_per_step": host_out.numel() * host_out.element_size(),
           "ms_per_step": round(e2e_s * 1e3, 3), "steps": e2e_steps}
    try:  # the host-link bound of the same bytes
        dev_b = torch.empty_like(x)
        ceil = copy_ceiling(torch, host_in, host_out, x, dev_b)
        del dev_b
        ceil["e2e_frac_of_copy_bound"] = round(ceil["both_ms"] / (e2e_s * 1e3), 3)
        e2e["copy_ceiling"] = ceil
    except Exception as e:  # noqa: BLE001 - informational
        e2e["copy_ceiling_error"] = str(e)[:200]
    del host_in, host_out

    extra = {}
    if rank == 0:
        extra["accuracy"] = {p: accuracy_sample(torch, tc, size_args, p) for p in ("plain", "split")}
        if "n" in size_args:  # the timed plan itself, on its own buffer, after the timed loop
            for kind in ("uniform", "tone"):
                extra["accuracy"]["timed_plan" + ("" if kind == "uniform" else "_tone")] = plan_accuracy(
                    torch, plan, x, args.precision, size, batch, kind)
        if not args.no_sweep and "n" in size_args:
            for key, fn in (("sweep", lambda: sweep(torch, tc, args.precision)),
                            ("sweep_split", lambda: sweep(torch, tc, "split", lgs=(10, 11, 12, 14, 16, 18, 20, 22))),
                            ("sweep_fp32io", lambda: sweep(torch, tc, "fp32io", lgs=(10, 11, 12, 14, 16, 18, 20, 22))),
                            ("sweep_2d", lambda: sweep_2d(torch, tc)),
                            ("uneven_batch", lambda: uneven_batch(torch, tc)),
                            ("uneven_batch_graph", lambda: uneven_batch(torch, tc, graph=True)),
                            ("cufft_fp16", lambda: cufft_fp16(torch, size_args, batch))):
                try:  # informational
                    extra[key] = fn()
                except Exception as e:  # noqa: BLE001
                    extra[key + "_error"] = str(e)[:200]
                torch.cuda.empty_cache()
    plan.destroy()
    del x
    torch.cuda.empty_cache()

    if rank == 0:
        base = cpu_baseline(size_args, budget_s=args.cpu_budget)
        line = {"metric": metric, "value": round(value, 1), "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(per_call * 1e3, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp16" if args.precision == "plain" else "fp16x3",
                "data": "synthetic: uniform[-1,1) real/imag generated on device",
                "config": config, "roofline": roofline, "cpu_baseline": base, "e2e": e2e,
                "gpu_launches": info["launches_per_exec"] * args.steps, "clocks": clocks}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
