"""Build recipe for the CPU oracle (test infrastructure only).

``build()`` compiles ``oracle/fft64.c`` into ``oracle/_build/liboracle.so``
with gcc (OpenMP when available).  When the reference sources are present
(they are only present on the build container, never on the GPU machine),
``build_ref()`` additionally compiles, from the reference's own files where
they lie, the pieces used to pin the oracle:

* ``oracle/_ref/libtcfft_ref_host.so`` -- ``tcfft_doit_half.cpp`` +
  ``tcfft_half.cu`` (host code), so the tests can call the reference's own
  ``gen_rev`` (tcfft_doit_half.cpp:6-29) and ``tcfftCreate`` size table
  (tcfft_half.cu:1235-1330) on the CPU.
* ``oracle/_ref/tcfft_half_ref.cubin`` / ``tcfft_half_2d_ref.cubin`` -- the
  reference kernels compiled for sm_103a (device code only), plus
  ``*_kernels.txt`` with their mangled names, so the GPU tests can run the
  reference kernels on the same inputs through ``oracle/ref_runner.cpp``.

Outputs go only to ``oracle/_build`` and ``oracle/_ref`` (both git-ignored).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# where the reference sources lie (only on the build container); TCFFT_REFERENCE_DIR overrides
REFERENCE = os.environ.get("TCFFT_REFERENCE_DIR", "/root/reference")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(force=False):
    """Compile liboracle.so (and the ref-runner when nvcc is available)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "fft64.c")
    out = os.path.join(BUILD, "liboracle.so")
    if force or not _newer(out, [src]):
        _run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", out, src, "-lm"])
    runner_src = os.path.join(HERE, "ref_runner.cpp")
    runner_out = os.path.join(BUILD, "libref_runner.so")
    if os.path.exists(runner_src) and os.path.exists(NVCC):
        if force or not _newer(runner_out, [runner_src]):
            _run([NVCC, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", runner_out,
                  runner_src, "-lcuda"])
    if os.path.isdir(REFERENCE):
        build_ref(force=force)
    return out


def build_ref(force=False):
    """Compile the reference's own sources (only where they exist)."""
    if not os.path.isdir(REFERENCE):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    srcs_1d = [os.path.join(REFERENCE, f) for f in ("tcfft_doit_half.cpp", "tcfft_half.cu")]
    host_so = os.path.join(REF_OUT, "libtcfft_ref_host.so")
    if force or not _newer(host_so, srcs_1d):
        _run([NVCC, "-O2", "-std=c++14", "-Xcompiler", "-fPIC,-fopenmp", "-shared", "-I", REFERENCE,
              *ARCH, "-o", host_so, *srcs_1d, "-lgomp"])
    wrapper = os.path.join(HERE, "ref_kernels.cu")  # includes the reference source, adds the _A100 kernels
    for two_d, stem in ((0, "tcfft_half"), (1, "tcfft_half_2d")):
        src = os.path.join(REFERENCE, stem + ".cu")
        cubin = os.path.join(REF_OUT, stem + "_ref.cubin")
        names = os.path.join(REF_OUT, stem + "_kernels.txt")
        flags = ["-std=c++14", "-I", REFERENCE, "-DTCFFT_REF_2D=%d" % two_d, *ARCH]
        if force or not (_newer(cubin, [src, wrapper]) and _newer(names, [src, wrapper])):
            _run([NVCC, "-cubin", "-O3", *flags, "-o", cubin, wrapper])
            # kernel symbol names, read from a host object of the same source
            obj = os.path.join(REF_OUT, stem + "_host.o")
            _run([NVCC, "-c", "-O0", *flags, "-o", obj, wrapper])
            syms = _run(["nm", "--defined-only", obj])
            kern = sorted({m.group(1) for m in re.finditer(r"\s(_Z\d+layer_\w+)$", syms, re.M)})
            with open(names, "w") as f:
                f.write("\n".join(kern) + "\n")
            os.remove(obj)
    return REF_OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built")
