"""tcfft_gb300 -- GB300-native (sm_103a) half-precision FFT library, host side.

The compute path is the CUDA library ``libtcfft_gb300.so`` built from
``tcfft_gb300/csrc`` (see ``tcfft_gb300/build.py``); this module binds its
C ABI (``include/tcfft_gb300.h``) with ctypes and mirrors the reference's plan
API (rox906/tcFFT, tcfft_half.h:20-21 / tcfft_half_2d.h:20-21):

    plan = tcfftCreate(n, n_batch)            # 1D   (tcfft_half.h:21)
    plan = tcfftCreate(nx, ny, n_batch)       # 2D   (tcfft_half_2d.h:21)
    tcfftExec(plan, data)                     # in place, forward (tcfft_half.h:20)
    tcfftDestroy(plan)                        # new: the reference never frees

``data`` is a CUDA torch tensor holding interleaved complex values: fp16
``[..., 2]`` / ``torch.complex32`` for the plain path (the reference's
``half*``), fp32 ``[..., 2]`` / ``torch.complex64`` for split precision.
Unlike the reference, input is in natural order by default, errors raise
:class:`TcfftError`, and execution goes on the current torch stream.

There is no CPU fallback: if the CUDA library is missing, importing works but
every plan/execute call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtcfft_gb300.so")

PRECISION_PLAIN = 0
PRECISION_SPLIT = 1
PRECISION_FP32_IO = 2
ORDER_NATURAL = 0
ORDER_REFERENCE_DIGIT_REVERSED = 1
FORWARD = 0        # sign -1 (the reference's transform)
INVERSE = 1        # sign +1
NORM_NONE = 0
NORM_BY_N = 1

_STATUS = {
    0: "TCFFT_SUCCESS", 1: "TCFFT_INVALID_VALUE", 2: "TCFFT_INVALID_SIZE", 3: "TCFFT_MISALIGNED",
    4: "TCFFT_ALLOC_FAILED", 5: "TCFFT_CUDA_ERROR", 6: "TCFFT_TIMEOUT", 7: "TCFFT_NOT_SUPPORTED",
    8: "TCFFT_INVALID_PLAN",
}


class TcfftError(RuntimeError):
    """A tcfft C-ABI call returned a non-success status."""

    def __init__(self, status, what=""):
        self.status = int(status)
        name = _STATUS.get(self.status, "status %d" % self.status)
        msg = "%s: %s" % (what, name) if what else name
        try:
            msg += " (%s)" % lib().tcfftGetErrorString(self.status).decode()
        except Exception:  # noqa: BLE001 - message decoration only
            pass
        super().__init__(msg)


class Options(ctypes.Structure):
    """struct tcfftOptions (include/tcfft_gb300.h)."""
    _fields_ = [("precision", ctypes.c_int32), ("input_order", ctypes.c_int32),
                ("autotune", ctypes.c_int32), ("direction", ctypes.c_int32),
                ("tune_cache_path", ctypes.c_char_p), ("normalization", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class PlanInfo(ctypes.Structure):
    """struct tcfftPlanInfo (include/tcfft_gb300.h)."""
    _fields_ = [("total_elements", ctypes.c_int64), ("element_bytes", ctypes.c_int32),
                ("launches_per_exec", ctypes.c_int32), ("scratch_bytes", ctypes.c_int64),
                ("n_radices", ctypes.c_int32), ("radices", ctypes.c_int32 * 16),
                ("n_radices_y", ctypes.c_int32), ("radices_y", ctypes.c_int32 * 16),
                ("schedule", ctypes.c_char * 128)]


_LIB = None

# Every entry point declared in include/tcfft_gb300.h, with its ctypes signature.
_SIGNATURES = {
    "tcfftOptionsDefault": ([ctypes.POINTER(Options)], ctypes.c_int),
    "tcfftPlan1d": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(Options)],
                    ctypes.c_int),
    "tcfftPlan2d": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                     ctypes.POINTER(Options)], ctypes.c_int),
    "tcfftPlanStrided": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                          ctypes.c_int64, ctypes.POINTER(Options)], ctypes.c_int),
    "tcfftPlanMany": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(Options)], ctypes.c_int),
    "tcfftExecute": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftExecuteAdjoint": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftExecuteInverse": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftExecuteOutOfPlace": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftPlanReal2d": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                         ctypes.POINTER(Options)], ctypes.c_int),
    "tcfftPlanReal1d": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(Options)],
                        ctypes.c_int),
    "tcfftExecuteR2C": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftExecuteC2R": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftExecuteHost": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                         ctypes.c_int),
    "tcfftCheckDevice": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "tcfftDestroy": ([ctypes.c_void_p], ctypes.c_int),
    "tcfftGetErrorString": ([ctypes.c_int], ctypes.c_char_p),
    "tcfftGetPlanInfo": ([ctypes.c_void_p, ctypes.POINTER(PlanInfo)], ctypes.c_int),
    "tcfftDescribe1d": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t],
                        ctypes.c_int),
    "tcfftDescribe2d": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_char_p,
                         ctypes.c_size_t], ctypes.c_int),
    "tcfftDescribeManyItems": ([ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)],
                               ctypes.c_int),
    "tcfftVersion": ([], ctypes.c_char_p),
    "tcfftExecute1dNoAlloc": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                               ctypes.c_void_p], ctypes.c_int),
    "tcfftCheckDeviceNoAlloc": ([ctypes.c_void_p], ctypes.c_int),
    "tcfftSetWaitLimit": ([ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "tcfftInjectWaitTimeout": ([ctypes.c_void_p], ctypes.c_int),
}


def exported_symbols():
    """Names of the C-ABI entry points this module binds."""
    return sorted(_SIGNATURES)


def lib():
    """Load (once) and return the CUDA library; raises if it was not built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("tcfft_gb300: %s is missing; build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        handle = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = handle
    return _LIB


def _check(status, what):
    if status != 0:
        raise TcfftError(status, what)


def describe_1d(n, batch=1, precision=PRECISION_PLAIN):
    """Host-only schedule description for a 1D size (no GPU needed)."""
    buf = ctypes.create_string_buffer(256)
    _check(lib().tcfftDescribe1d(int(n), int(batch), int(precision), buf, 256), "tcfftDescribe1d")
    return buf.value.decode()


def describe_many_items(shapes, num_sms=152, offsets=None):
    """Host-only diagnostics: the one-launch many-shape executor's work items for ``shapes``
    (as in ``Plan.many``), in launch order, as a list of (kind, xf, tile, count, tiles, elements) tuples
    (tcfftDescribeManyItems); raises TcfftError (status 7) when the executor does not run them."""
    count = len(shapes)
    ranks = (ctypes.c_int32 * count)(*[len(s) for s in shapes])
    nxs = (ctypes.c_int64 * count)(*[int(s[0]) for s in shapes])
    nys = (ctypes.c_int64 * count)(*[int(s[1]) if len(s) > 1 else 1 for s in shapes])
    if offsets is None:
        offsets, acc = [], 0
        for s in shapes:
            offsets.append(acc)
            acc += int(s[0]) * (int(s[1]) if len(s) > 1 else 1)
    offa = (ctypes.c_int64 * count)(*[int(o) for o in offsets])
    n = ctypes.c_int64(0)
    _check(lib().tcfftDescribeManyItems(count, ranks, nxs, nys, offa, int(num_sms), None, 0, ctypes.byref(n)),
           "tcfftDescribeManyItems")
    buf = (ctypes.c_int32 * (6 * max(n.value, 1)))()
    _check(lib().tcfftDescribeManyItems(count, ranks, nxs, nys, offa, int(num_sms), buf, n.value, ctypes.byref(n)),
           "tcfftDescribeManyItems")
    return [tuple(buf[6 * i:6 * i + 6]) for i in range(n.value)]


def describe_2d(nx, ny, batch=1, precision=PRECISION_PLAIN):
    """Host-only schedule description for a 2D shape [batch][nx][ny] (no GPU needed)."""
    buf = ctypes.create_string_buffer(256)
    _check(lib().tcfftDescribe2d(int(nx), int(ny), int(batch), _precision_of(precision), buf, 256),
           "tcfftDescribe2d")
    return buf.value.decode()


def _precision_of(p):
    if p in (PRECISION_PLAIN, "plain", "fp16", None):
        return PRECISION_PLAIN
    if p in (PRECISION_SPLIT, "split"):
        return PRECISION_SPLIT
    if p in (PRECISION_FP32_IO, "fp32io"):
        return PRECISION_FP32_IO
    raise ValueError("precision must be 'plain', 'split' or 'fp32io', got %r" % (p,))


def _stream_handle(stream):
    if stream is None:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def _device_ptr(data, precision):
    """Device address of `data` after checking it matches the precision."""
    if isinstance(data, int):
        return data
    import torch
    if not isinstance(data, torch.Tensor):
        raise TypeError("data must be a CUDA torch tensor or a device pointer (int)")
    if not data.is_cuda:
        raise ValueError("tcfft executes on device memory; got a CPU tensor")
    if not data.is_contiguous():
        raise ValueError("data must be contiguous")
    want = (torch.float16, torch.complex32) if precision == PRECISION_PLAIN else (torch.float32, torch.complex64)
    if data.dtype not in want:
        raise TypeError("precision %s expects %s, got %s" % (
            {0: "plain", 1: "split", 2: "fp32io"}[precision], want, data.dtype))
    return data.data_ptr()


class Plan:
    """An FFT plan (owns its device tables; call :meth:`destroy` or use ``with``).

    1D: ``Plan(n=N, batch=B)``; 2D: ``Plan(nx=NX, ny=NY, batch=B)``;
    uneven batch: ``Plan.many([...shapes...])``.
    """

    def __init__(self, n=None, batch=1, nx=None, ny=None, precision="plain", input_order=ORDER_NATURAL,
                 autotune=False, tune_cache_path=None, direction=FORWARD, normalize=False, _handle=None,
                 _shapes=None):
        self._handle = ctypes.c_void_p(None)
        self.precision = _precision_of(precision)
        self.input_order = int(input_order)
        if _handle is not None:
            self._handle = _handle
            self.shapes = _shapes
            self.n = self.nx = self.ny = None
            self.batch = None
            return
        opts = Options()
        lib().tcfftOptionsDefault(ctypes.byref(opts))
        opts.precision = self.precision
        opts.input_order = self.input_order
        opts.autotune = 1 if autotune else 0
        opts.tune_cache_path = tune_cache_path.encode() if tune_cache_path else None
        opts.direction = int(direction)
        opts.normalization = NORM_BY_N if normalize else NORM_NONE
        self._opts = opts
        if n is not None:
            self.n, self.nx, self.ny, self.batch = int(n), None, None, int(batch)
            _check(lib().tcfftPlan1d(ctypes.byref(self._handle), self.n, self.batch, ctypes.byref(opts)),
                   "tcfftPlan1d(n=%d, batch=%d)" % (self.n, self.batch))
        elif nx is not None and ny is not None:
            self.n, self.nx, self.ny, self.batch = None, int(nx), int(ny), int(batch)
            _check(lib().tcfftPlan2d(ctypes.byref(self._handle), self.nx, self.ny, self.batch, ctypes.byref(opts)),
                   "tcfftPlan2d(nx=%d, ny=%d, batch=%d)" % (self.nx, self.ny, self.batch))
        else:
            raise ValueError("give n (1D) or nx and ny (2D)")

    @classmethod
    def many(cls, shapes, offsets=None, precision="plain", autotune=False, direction=FORWARD, normalize=False):
        """Uneven batch: ``shapes`` is a list of ``(n,)`` or ``(nx, ny)`` tuples,
        transforms packed back to back (or at ``offsets``, in elements)."""
        count = len(shapes)
        ranks = (ctypes.c_int32 * count)(*[len(s) for s in shapes])
        nxs = (ctypes.c_int64 * count)(*[int(s[0]) for s in shapes])
        nys = (ctypes.c_int64 * count)(*[int(s[1]) if len(s) > 1 else 1 for s in shapes])
        if offsets is None:
            offs, acc = [], 0
            for s in shapes:
                offs.append(acc)
                acc += int(s[0]) * (int(s[1]) if len(s) > 1 else 1)
            offsets = offs
        offa = (ctypes.c_int64 * count)(*[int(o) for o in offsets])
        opts = Options()
        lib().tcfftOptionsDefault(ctypes.byref(opts))
        opts.precision = _precision_of(precision)
        opts.autotune = 1 if autotune else 0
        opts.direction = int(direction)
        opts.normalization = NORM_BY_N if normalize else NORM_NONE
        h = ctypes.c_void_p(None)
        _check(lib().tcfftPlanMany(ctypes.byref(h), count, ranks, nxs, nys, offa, ctypes.byref(opts)),
               "tcfftPlanMany(count=%d)" % count)
        p = cls(precision=precision, _handle=h, _shapes=[tuple(s) for s in shapes])
        p.offsets = list(offsets)
        return p

    @classmethod
    def strided(cls, n, batch, istride=1, idist=None, precision="plain", direction=FORWARD, normalize=False):
        """Strided 1D layout (tcfftPlanStrided): point j of transform b at element
        ``b * idist + j`` (``istride == 1``), or, with ``istride > 1`` (``idist`` 1),
        ``(b // istride) * n * istride + j * istride + b % istride``: the FFT along
        the middle axis of a ``[batch // istride][n][istride]`` array."""
        if idist is None:
            idist = n if istride == 1 else 1
        opts = Options()
        lib().tcfftOptionsDefault(ctypes.byref(opts))
        opts.precision = _precision_of(precision)
        opts.direction = int(direction)
        opts.normalization = NORM_BY_N if normalize else NORM_NONE
        h = ctypes.c_void_p(None)
        _check(lib().tcfftPlanStrided(ctypes.byref(h), int(n), int(batch), int(istride), int(idist),
                                      ctypes.byref(opts)),
               "tcfftPlanStrided(n=%d, batch=%d, istride=%d, idist=%d)" % (n, batch, istride, idist))
        return cls(precision=precision, _handle=h)

    # -- execution -------------------------------------------------------
    def _ptr(self, data):
        return _device_ptr(data, self.precision)

    def exec(self, data, stream=None, adjoint=False, inverse=False):
        """Transform ``data`` in place: the plan's transform, its adjoint
        (``adjoint=True``) or its inverse (``inverse=True``, so that
        ``exec(exec(x), inverse=True) == x`` up to rounding)."""
        if not self._handle:
            raise TcfftError(8, "exec on destroyed plan")
        if adjoint and inverse:
            raise ValueError("adjoint and inverse are exclusive")
        name = "tcfftExecuteAdjoint" if adjoint else ("tcfftExecuteInverse" if inverse else "tcfftExecute")
        _check(getattr(lib(), name)(self._handle, ctypes.c_void_p(self._ptr(data)), _stream_handle(stream)), name)
        return data

    def exec_out(self, data, out, stream=None):
        """The plan's transform of ``data`` written to ``out`` (``data`` is not modified)."""
        if not self._handle:
            raise TcfftError(8, "exec on destroyed plan")
        _check(lib().tcfftExecuteOutOfPlace(self._handle, ctypes.c_void_p(self._ptr(data)),
                                            ctypes.c_void_p(self._ptr(out)), _stream_handle(stream)),
               "tcfftExecuteOutOfPlace")
        return out

    def exec_host(self, host_in, host_out, work, stream=None):
        """Forward transform of a host batch: ``host_in`` is copied into the device
        buffer ``work``, transformed and copied to ``host_out`` (pinned CPU tensors of
        the plan's size), pipelined over chunks of the batch (tcfftExecuteHost)."""
        if not self._handle:
            raise TcfftError(8, "exec on destroyed plan")
        inf = self.info
        if getattr(self, "shapes", None) is not None:  # uneven batch: up to the end of the last transform
            span = max(int(o) + int(s[0]) * (int(s[1]) if len(s) > 1 else 1) for o, s in zip(self.offsets, self.shapes))
            nbytes = span * inf["element_bytes"]
        else:
            nbytes = inf["total_elements"] * inf["element_bytes"]
        for t in (host_in, host_out):
            if t.is_cuda or not t.is_contiguous():
                raise ValueError("host buffers must be contiguous CPU tensors")
            if t.numel() * t.element_size() != nbytes:
                raise ValueError("host buffers must hold the plan's %d bytes" % nbytes)
        _check(lib().tcfftExecuteHost(self._handle, ctypes.c_void_p(host_in.data_ptr()),
                                      ctypes.c_void_p(host_out.data_ptr()), ctypes.c_void_p(self._ptr(work)),
                                      _stream_handle(stream)),
               "tcfftExecuteHost")
        return host_out

    def check_device(self, stream=None):
        """Synchronise and raise TcfftError(TCFFT_TIMEOUT) if a bounded wait expired."""
        _check(lib().tcfftCheckDevice(self._handle, _stream_handle(stream)), "tcfftCheckDevice")

    def set_wait_limit(self, limit_ns):
        """Limit of the two-phase kernels' bounded device-side waits (ns; 0 = the 2 s default)."""
        _check(lib().tcfftSetWaitLimit(self._handle, int(limit_ns)), "tcfftSetWaitLimit")

    def inject_wait_timeout(self):
        """Test hook: make the next execute's bounded waits run out (tcfftInjectWaitTimeout)."""
        _check(lib().tcfftInjectWaitTimeout(self._handle), "tcfftInjectWaitTimeout")

    @property
    def info(self):
        inf = PlanInfo()
        _check(lib().tcfftGetPlanInfo(self._handle, ctypes.byref(inf)), "tcfftGetPlanInfo")
        return {
            "total_elements": inf.total_elements, "element_bytes": inf.element_bytes,
            "launches_per_exec": inf.launches_per_exec, "scratch_bytes": inf.scratch_bytes,
            "radices": list(inf.radices[:inf.n_radices]), "radices_y": list(inf.radices_y[:inf.n_radices_y]),
            "schedule": inf.schedule.decode(),
        }

    def destroy(self):
        if self._handle:
            _check(lib().tcfftDestroy(self._handle), "tcfftDestroy")
            self._handle = ctypes.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            if self._handle and _LIB is not None:
                _LIB.tcfftDestroy(self._handle)
                self._handle = ctypes.c_void_p(None)
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class RealPlan(Plan):
    """Real transforms (tcfftPlanReal1d / tcfftPlanReal2d).  1D, ``RealPlan(n, batch)``:
    ``r2c(x, out)`` maps real ``[batch, n]`` (fp16 plain / fp32 split) to the
    Hermitian half ``[batch, n // 2 + 1, 2]``.  2D, ``RealPlan(nx=, ny=, batch=)``:
    real ``[batch, nx, ny]`` to ``[batch, nx, ny // 2 + 1, 2]`` (numpy's rfft2
    layout).  ``c2r(X, out)`` is the inverse (c2r(r2c(x)) = x: the 1/N on c2r, or
    on r2c with ``normalize=True``)."""

    def __init__(self, n=None, batch=1, precision="plain", normalize=False, autotune=False, nx=None, ny=None):
        self._handle = ctypes.c_void_p(None)
        self.precision = _precision_of(precision)
        self.n, self.batch = (int(n) if n else None), int(batch)
        self.nx, self.ny = (int(nx) if nx else None), (int(ny) if ny else None)
        opts = Options()
        lib().tcfftOptionsDefault(ctypes.byref(opts))
        opts.precision = self.precision
        opts.normalization = NORM_BY_N if normalize else NORM_NONE
        opts.autotune = 1 if autotune else 0
        if self.nx:
            _check(lib().tcfftPlanReal2d(ctypes.byref(self._handle), self.nx, self.ny, self.batch,
                                         ctypes.byref(opts)),
                   "tcfftPlanReal2d(nx=%d, ny=%d, batch=%d)" % (self.nx, self.ny, self.batch))
        else:
            _check(lib().tcfftPlanReal1d(ctypes.byref(self._handle), self.n, self.batch, ctypes.byref(opts)),
                   "tcfftPlanReal1d(n=%d, batch=%d)" % (self.n, self.batch))

    def _real_ptr(self, t):
        import torch
        want = torch.float16 if self.precision == PRECISION_PLAIN else torch.float32
        if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous() or t.dtype != want:
            raise TypeError("expected a contiguous CUDA %s tensor" % want)
        return t.data_ptr()

    def r2c(self, x, out, stream=None):
        _check(lib().tcfftExecuteR2C(self._handle, ctypes.c_void_p(self._real_ptr(x)),
                                     ctypes.c_void_p(self._real_ptr(out)), _stream_handle(stream)), "tcfftExecuteR2C")
        return out

    def c2r(self, spec, out, stream=None):
        _check(lib().tcfftExecuteC2R(self._handle, ctypes.c_void_p(self._real_ptr(spec)),
                                     ctypes.c_void_p(self._real_ptr(out)), _stream_handle(stream)), "tcfftExecuteC2R")
        return out


# ---------------------------------------------------------------- reference-named API
def tcfftCreate(*args, precision="plain", input_order=ORDER_NATURAL):
    """Mirror of the reference's ``tcfftCreate`` (tcfft_half.h:21 / tcfft_half_2d.h:21):
    ``tcfftCreate(n, n_batch)`` or ``tcfftCreate(nx, ny, n_batch)``; returns a :class:`Plan`."""
    if len(args) == 2:
        return Plan(n=args[0], batch=args[1], precision=precision, input_order=input_order)
    if len(args) == 3:
        return Plan(nx=args[0], ny=args[1], batch=args[2], precision=precision, input_order=input_order)
    raise TypeError("tcfftCreate(n, n_batch) or tcfftCreate(nx, ny, n_batch)")


def tcfftExec(plan, data, stream=None):
    """Mirror of ``tcfftExec(tcfftHandle, half*)`` (tcfft_half.h:20): forward, in place."""
    return plan.exec(data, stream=stream)


def tcfftDestroy(plan):
    plan.destroy()


def version():
    return lib().tcfftVersion().decode()


def execute_1d_noalloc(data, n, batch, precision="plain", adjoint=False, stream=None):
    """Allocation-free in-place 1D FFT (tcfftExecute1dNoAlloc): for callers
    that cannot allocate device memory when they run a transform.  Uses the
    library's fixed static scratch (n <= 2^21 plain, <= 2^20 split, n >= 2^12);
    calls that overlap on the GPU race on that scratch."""
    prec = _precision_of(precision)
    ptr = _device_ptr(data, prec)
    _check(lib().tcfftExecute1dNoAlloc(ctypes.c_void_p(ptr), int(n), int(batch), prec, 1 if adjoint else 0,
                                       _stream_handle(stream)), "tcfftExecute1dNoAlloc")
    return data


def check_device_noalloc(stream=None):
    """Synchronise and raise TcfftError(TCFFT_TIMEOUT) if a bounded wait of an
    allocation-free call ran out since the last check (tcfftCheckDeviceNoAlloc)."""
    _check(lib().tcfftCheckDeviceNoAlloc(_stream_handle(stream)), "tcfftCheckDeviceNoAlloc")
