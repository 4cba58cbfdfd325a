"""heffte_gb300 — Python host side of the GB300-native fft3d backend.

ctypes over the C ABI of ``libheffte_gb300.so`` (declared in
``include/heffte_gb300.h``), mirroring the reference's own Python binding
(python/heffte.py:116-462: ``box3d``, ``scale``, ``fft3d``, ``fft3d_r2c``,
``forward``/``backward`` and their ``_buffered`` variants, ``size_*``) for one
rank.  Arrays are CUDA tensors (torch is only the device-memory container);
raw device pointers (ints) are accepted by the ``*_ptr`` methods.

There is no CPU fallback: importing the package raises if the library is not
built (``python -m heffte_gb300.build``).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

__all__ = ["box3d", "scale", "kind", "plan_options", "fft3d", "fft3d_r2c", "rtransform", "executor",
           "heffte_input_error", "HeffteError", "lib", "library_path"]


class heffte_input_error(Exception):
    """Invalid input detected on the host, as python/heffte.py:31-36."""


class HeffteError(RuntimeError):
    """A status code returned by the library (message as the reference's runtime_error)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


library_path = _build.LIB
_lib = None


def lib():
    """Loads libheffte_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(library_path):
        raise ImportError("libheffte_gb300.so is not built: run `python -m heffte_gb300.build` "
                          "(the package has no CPU fallback)")
    L = ctypes.CDLL(library_path)
    vp, i, ll, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    I3 = ctypes.c_int * 3
    LL3 = ctypes.c_longlong * 3
    L.heffte_gb300_last_error.restype = ctypes.c_char_p
    L.heffte_gb300_convert.argtypes = [vp, i, ll, vp, vp, i]
    L.heffte_gb300_scale_data.argtypes = [vp, i, ll, vp, d]
    L.heffte_gb300_direct_pack.argtypes = [vp, i, ll, ll, ll, ll, ll, vp, vp]
    L.heffte_gb300_direct_unpack.argtypes = [vp, i, ll, ll, ll, ll, ll, vp, vp]
    L.heffte_gb300_transpose_unpack.argtypes = [vp, i, ll, ll, ll, ll, ll, ll, ll, i, i, i, vp, vp]
    L.heffte_gb300_r2r_prepost.argtypes = [vp, i, i, i, i, ll, ll, ll, vp, vp]
    L.heffte_gb300_set_kernel_variant.argtypes = [i]
    L.heffte_gb300_device_status.argtypes = [ctypes.POINTER(ctypes.c_int), i]
    L.heffte_gb300_executor_create.argtypes = [i, LL3, LL3, I3, i, I3, ctypes.POINTER(vp)]
    L.heffte_gb300_executor_destroy.argtypes = [vp]
    for f in ("box_size", "complex_size", "workspace_size"):
        getattr(L, "heffte_gb300_executor_" + f).argtypes = [vp]
        getattr(L, "heffte_gb300_executor_" + f).restype = ll
    L.heffte_gb300_executor_forward.argtypes = [vp, vp, i, vp, vp, vp]
    L.heffte_gb300_executor_backward.argtypes = [vp, vp, i, vp, vp, vp]
    L.heffte_gb300_reshape_create.argtypes = [i, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(vp)]
    L.heffte_gb300_reshape_destroy.argtypes = [vp]
    for f in ("send_size", "recv_size"):
        getattr(L, "heffte_gb300_reshape_" + f).argtypes = [vp]
        getattr(L, "heffte_gb300_reshape_" + f).restype = ll
    llp = ctypes.POINTER(ll)
    L.heffte_gb300_reshape_counts.argtypes = [vp, llp, llp, llp, llp]
    L.heffte_gb300_reshape_pack.argtypes = [vp, vp, i, vp, vp]
    L.heffte_gb300_reshape_unpack.argtypes = [vp, vp, i, vp, vp]
    L.heffte_gb300_set_default_options.argtypes = [ctypes.c_void_p]
    L.heffte_gb300_plan_create.argtypes = [i, I3, I3, I3, I3, I3, I3, i, vp, vp, ctypes.POINTER(vp)]
    L.heffte_gb300_plan_destroy.argtypes = [vp]
    L.heffte_gb300_plan_set_stream.argtypes = [vp, vp]
    for f in ("size_inbox", "size_outbox", "size_workspace"):
        getattr(L, "heffte_gb300_" + f).argtypes = [vp]
        getattr(L, "heffte_gb300_" + f).restype = ll
    L.heffte_gb300_scale_factor.argtypes = [vp, i]
    L.heffte_gb300_scale_factor.restype = d
    L.heffte_gb300_forward.argtypes = [vp, i, vp, vp, vp, i]
    L.heffte_gb300_backward.argtypes = [vp, i, vp, vp, vp, i]
    L.heffte_gb300_convolve_workspace.argtypes = [vp]
    L.heffte_gb300_convolve_workspace.restype = ll
    L.heffte_gb300_convolve.argtypes = [vp, i, vp, vp, vp, vp, i]
    L.heffte_gb300_convolve_route.argtypes = [vp, i, i, ctypes.POINTER(ctypes.c_int)]
    L.heffte_gb300_plan_set_convolution_fusion.argtypes = [vp, i]
    L.heffte_gb300_forward_batch.argtypes = [vp, i, i, vp, vp, vp, i]
    L.heffte_gb300_backward_batch.argtypes = [vp, i, i, vp, vp, vp, i]
    L.heffte_gb300_boxbatch_create.argtypes = [i, i, i, ctypes.POINTER(ctypes.c_int), vp, ctypes.POINTER(vp)]
    L.heffte_gb300_boxbatch_destroy.argtypes = [vp]
    for f in ("input_offset", "output_offset"):
        getattr(L, "heffte_gb300_boxbatch_" + f).argtypes = [vp, i]
        getattr(L, "heffte_gb300_boxbatch_" + f).restype = ll
    for f in ("input_size", "output_size", "workspace_size"):
        getattr(L, "heffte_gb300_boxbatch_" + f).argtypes = [vp]
        getattr(L, "heffte_gb300_boxbatch_" + f).restype = ll
    L.heffte_gb300_set_dependency_wait_budget.argtypes = [ll]
    L.heffte_gb300_dependency_wait_budget.restype = ll
    L.heffte_gb300_boxbatch_hold_dependencies.argtypes = [vp, i]
    ip = ctypes.POINTER(ctypes.c_int)
    L.heffte_gb300_boxbatch_configure.argtypes = [vp, i, i, i, i]
    L.heffte_gb300_boxbatch_config.argtypes = [vp, ip, ip, ip, ip]
    L.heffte_gb300_boxbatch_autotune.argtypes = [vp, vp, vp, vp, vp, i, ip, ip, ip, ip, ctypes.POINTER(ctypes.c_double)]
    L.heffte_gb300_boxbatch_forward.argtypes = [vp, vp, vp, i]
    L.heffte_gb300_boxbatch_backward.argtypes = [vp, vp, vp, vp, i]
    L.heffte_gb300_tune.argtypes = [i, i, ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, vp, ctypes.POINTER(ctypes.c_int)]
    L.heffte_gb300_tune_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.heffte_gb300_tuned_choice.argtypes = [i, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    ip, fp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)
    L.heffte_gb300_plan_set_knobs.argtypes = [vp, i, i, i]
    L.heffte_gb300_plan_set_tensor_cores.argtypes = [vp, i]
    L.heffte_gb300_plan_features.argtypes = [i, i, I3, fp]
    L.heffte_gb300_candidate_options.argtypes = [i, vp, ip, ip, ip]
    L.heffte_gb300_mlp_create.argtypes = [i, i, i, ctypes.c_ulonglong, ctypes.POINTER(vp)]
    L.heffte_gb300_mlp_destroy.argtypes = [vp]
    L.heffte_gb300_mlp_num_params.argtypes = [vp]
    L.heffte_gb300_mlp_num_params.restype = ll
    L.heffte_gb300_mlp_get_params.argtypes = [vp, fp]
    L.heffte_gb300_mlp_set_params.argtypes = [vp, fp]
    L.heffte_gb300_mlp_loss_grad.argtypes = [vp, vp, vp, i, fp, fp]
    L.heffte_gb300_mlp_train.argtypes = [vp, vp, vp, i, i, ctypes.c_float, vp, fp]
    L.heffte_gb300_mlp_predict.argtypes = [vp, vp, vp, i, vp]
    L.heffte_gb300_select.argtypes = [vp, i, i, I3, ip]
    _lib = L
    return L


def check(code):
    if code != 0:
        msg = lib().heffte_gb300_last_error().decode()
        raise HeffteError(code, msg or f"heffte_gb300 error {code}")


class scale:
    """heffte::scale (include/heffte_fft3d.h:140-147)."""
    none = 0
    full = 1
    symmetric = 2


class kind:
    c2c = 0
    r2c = 1
    cos = 2
    sin = 3
    cos1 = 4


class box3d:
    """box3d (include/heffte_geometry.h:67-133): inclusive low/high, order o0 fastest."""

    def __init__(self, clow, chigh, corder=(0, 1, 2)):
        self.low = tuple(int(v) for v in clow)
        self.high = tuple(int(v) for v in chigh)
        self.order = tuple(int(v) for v in corder)
        if len(self.low) != 3 or len(self.high) != 3 or sorted(self.order) != [0, 1, 2]:
            raise heffte_input_error("box3d needs three low, three high indexes and an order permutation")
        self.size = tuple(self.high[i] - self.low[i] + 1 for i in range(3))

    def count(self):
        return 0 if min(self.size) <= 0 else self.size[0] * self.size[1] * self.size[2]

    def r2c(self, dimension):
        hi = list(self.high)
        hi[dimension] = self.low[dimension] + self.size[dimension] // 2
        return box3d(self.low, hi, self.order)

    def osize(self, d):
        return self.size[self.order[d]]

    def __repr__(self):
        return f"box3d({self.low}, {self.high}, {self.order})"


class plan_options(ctypes.Structure):
    """plan_options (include/heffte_plan_logic.h:131-176), C layout of heffte_plan_options."""
    _fields_ = [("use_reorder", ctypes.c_int), ("algorithm", ctypes.c_int),
                ("use_pencils", ctypes.c_int), ("use_gpu_aware", ctypes.c_int)]

    @staticmethod
    def default():
        o = plan_options()
        check(lib().heffte_gb300_set_default_options(ctypes.byref(o)))
        return o


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)  # torch.cuda.Stream


def _ptr(x):
    if isinstance(x, int):
        return x
    if x is None:
        return None
    if not x.is_cuda:
        raise heffte_input_error("arrays must live on the GPU (no CPU fallback)")
    if not x.is_contiguous():
        raise heffte_input_error("arrays must be contiguous")
    return x.data_ptr()


_REAL = {"torch.float32": 0, "torch.float64": 1}
_CPLX = {"torch.complex64": 0, "torch.complex128": 1}


class _plan:
    """A single-rank 3-D transform plan (fft3d / fft3d_r2c / rtransform)."""

    def __init__(self, tkind, inbox, outbox, r2c_direction=0, options=None, stream=None):
        L = lib()
        self.kind = tkind
        self.inbox, self.outbox = inbox, outbox
        self._h = ctypes.c_void_p()
        I3 = ctypes.c_int * 3
        opts = options if options is not None else plan_options.default()
        self.stream = _stream_handle(stream)
        check(L.heffte_gb300_plan_create(tkind, I3(*inbox.low), I3(*inbox.high), I3(*inbox.order),
                                         I3(*outbox.low), I3(*outbox.high), I3(*outbox.order),
                                         r2c_direction, ctypes.byref(opts), self.stream, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.heffte_gb300_plan_destroy(h)
            self._h = None

    def set_stream(self, stream):
        self.stream = _stream_handle(stream)
        check(lib().heffte_gb300_plan_set_stream(self._h, self.stream))

    def set_knobs(self, variant=0, tile_div=1, radix_policy=0):
        """Re-plans with a kernel family (0 pipelined, 1 one-shot), tile divisor (1, 2) and radix order (0, 1)."""
        check(lib().heffte_gb300_plan_set_knobs(self._h, variant, tile_div, radix_policy))

    def set_tensor_cores(self, enable=True):
        """complex<float> radix-16 stages as split-BF16 DFT contractions on the tensor cores (or back to FP32)."""
        check(lib().heffte_gb300_plan_set_tensor_cores(self._h, 1 if enable else 0))

    def size_inbox(self):
        return lib().heffte_gb300_size_inbox(self._h)

    def size_outbox(self):
        return lib().heffte_gb300_size_outbox(self._h)

    def size_workspace(self):
        return lib().heffte_gb300_size_workspace(self._h)

    def get_scale_factor(self, scaling):
        return lib().heffte_gb300_scale_factor(self._h, scaling)

    # -- type checks mirroring python/heffte.py:236-300 --
    def _prec(self, inarray, outarray, forward):
        it, ot = str(inarray.dtype), str(outarray.dtype)
        if self.kind == kind.c2c:
            if it not in _CPLX or it != ot:
                raise heffte_input_error("c2c transforms need complex64 or complex128 arrays of the same type")
            return _CPLX[it]
        if self.kind == kind.r2c:
            rt, ct = (it, ot) if forward else (ot, it)
            if rt not in _REAL or ct not in _CPLX or _REAL[rt] != _CPLX[ct]:
                raise heffte_input_error("r2c transforms need float32/complex64 or float64/complex128 pairs")
            return _REAL[rt]
        if it not in _REAL or it != ot:
            raise heffte_input_error("real-to-real transforms need float32 or float64 arrays of the same type")
        return _REAL[it]

    def _run(self, forward, inarray, outarray, workspace, scaling, batch=1):
        if scaling not in (0, 1, 2):
            raise heffte_input_error("called with invalid scaling")
        nin, nout = (self.size_inbox(), self.size_outbox()) if forward else (self.size_outbox(), self.size_inbox())
        if inarray.numel() < batch * nin or outarray.numel() < batch * nout:
            raise heffte_input_error("called with invalid array size")
        prec = self._prec(inarray, outarray, forward)
        L = lib()
        f = L.heffte_gb300_forward_batch if forward else L.heffte_gb300_backward_batch
        check(f(self._h, batch, prec, _ptr(inarray), _ptr(outarray), _ptr(workspace), scaling))

    def forward(self, inarray, outarray, scaling=scale.none):
        self._run(True, inarray, outarray, None, scaling)

    def backward(self, inarray, outarray, scaling=scale.none):
        self._run(False, inarray, outarray, None, scaling)

    def forward_buffered(self, inarray, outarray, workspace, scaling=scale.none):
        self._run(True, inarray, outarray, workspace, scaling)

    def backward_buffered(self, inarray, outarray, workspace, scaling=scale.none):
        self._run(False, inarray, outarray, workspace, scaling)

    def convolve_workspace(self):
        return lib().heffte_gb300_convolve_workspace(self._h)

    def set_convolution_fusion(self, enable=True):
        """convolve's fused route where it applies (default), or always the unfused sequence."""
        check(lib().heffte_gb300_plan_set_convolution_fusion(self._h, 1 if enable else 0))

    def convolve_route(self, precision=0, two_inputs=False):
        """Dimension of the fused convolution pass for aligned arrays, -1 when unfused."""
        d = ctypes.c_int(-2)
        check(lib().heffte_gb300_convolve_route(self._h, precision, 1 if two_inputs else 0, ctypes.byref(d)))
        return d.value

    def convolve(self, x, y, outarray, scaling=scale.full, workspace=None):
        """outarray = backward(forward(x) .* forward(y)) with the backward scaling
        (scale.full: the circular convolution of x and y); y None: x .* x.
        The step of the reference's benchmarks/convolution.cpp as one call."""
        if scaling not in (0, 1, 2):
            raise heffte_input_error("called with invalid scaling")
        if self.kind not in (kind.c2c, kind.r2c):
            raise heffte_input_error("convolution needs a c2c or r2c plan")
        n = self.size_inbox()
        if x.numel() < n or outarray.numel() < n or (y is not None and y.numel() < n):
            raise heffte_input_error("called with invalid array size")
        if y is not None and y.dtype != x.dtype:
            raise heffte_input_error("x and y must have the same type")
        it, ot = str(x.dtype), str(outarray.dtype)
        table = _CPLX if self.kind == kind.c2c else _REAL
        if it not in table or it != ot:
            raise heffte_input_error("convolution arrays must have the plan's input type")
        check(lib().heffte_gb300_convolve(self._h, table[it], _ptr(x), _ptr(y), _ptr(outarray), _ptr(workspace),
                                          scaling))

    def forward_batch(self, batch, inarray, outarray, scaling=scale.none, workspace=None):
        self._run(True, inarray, outarray, workspace, scaling, batch)

    def backward_batch(self, batch, inarray, outarray, scaling=scale.none, workspace=None):
        self._run(False, inarray, outarray, workspace, scaling, batch)

    # raw-pointer entry points (prec 0 single / 1 double)
    def forward_ptr(self, prec, inp, out, workspace=0, scaling=scale.none, batch=1):
        check(lib().heffte_gb300_forward_batch(self._h, batch, prec, inp, out, workspace or None, scaling))

    def backward_ptr(self, prec, inp, out, workspace=0, scaling=scale.none, batch=1):
        check(lib().heffte_gb300_backward_batch(self._h, batch, prec, inp, out, workspace or None, scaling))


def fft3d(inbox, outbox, options=None, stream=None):
    """heffte::fft3d<backend::gb300> on one rank (include/heffte_fft3d.h:270-297)."""
    return _plan(kind.c2c, inbox, outbox, 0, options, stream)


def fft3d_r2c(inbox, outbox, r2c_direction, options=None, stream=None):
    """heffte::fft3d_r2c<backend::gb300> on one rank (include/heffte_fft3d_r2c.h:76-93)."""
    if r2c_direction not in (0, 1, 2):
        raise heffte_input_error("fft3d_r2c() called with invalid r2c_direction, must use 0, 1, or 2")
    return _plan(kind.r2c, inbox, outbox, r2c_direction, options, stream)


def rtransform(rkind, inbox, outbox, options=None, stream=None):
    """heffte::rtransform<backend::gb300_cos|gb300_sin|gb300_cos1> (include/heffte_fft3d.h:748-749)."""
    if rkind not in (kind.cos, kind.sin, kind.cos1):
        raise heffte_input_error("rtransform kind must be kind.cos, kind.sin or kind.cos1")
    return _plan(rkind, inbox, outbox, 0, options, stream)


class executor:
    """one_dim_backend<gb300>::executor / executor_r2c on one box."""

    def __init__(self, ekind, box, dims):
        L = lib()
        self._h = ctypes.c_void_p()
        dims = list(dims)
        d3 = (ctypes.c_int * 3)(*(dims + [0] * (3 - len(dims))))
        check(L.heffte_gb300_executor_create(ekind, (ctypes.c_longlong * 3)(*box.low),
                                             (ctypes.c_longlong * 3)(*box.high), (ctypes.c_int * 3)(*box.order),
                                             len(dims), d3, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.heffte_gb300_executor_destroy(h)

    def box_size(self):
        return lib().heffte_gb300_executor_box_size(self._h)

    def complex_size(self):
        return lib().heffte_gb300_executor_complex_size(self._h)

    def workspace_size(self):
        return lib().heffte_gb300_executor_workspace_size(self._h)

    def forward(self, prec, inp, out, stream=None, workspace=None):
        """workspace: workspace_size() elements of the data type, or None
        (the executor then keeps a buffer of its own)."""
        check(lib().heffte_gb300_executor_forward(self._h, _stream_handle(stream), prec, _ptr(inp), _ptr(out),
                                                  _ptr(workspace) if workspace is not None else None))

    def backward(self, prec, inp, out, stream=None, workspace=None):
        check(lib().heffte_gb300_executor_backward(self._h, _stream_handle(stream), prec, _ptr(inp), _ptr(out),
                                                   _ptr(workspace) if workspace is not None else None))


class reshape3d:
    """reshape3d_alltoallv (src/heffte_reshape3d.cpp:365-496) of rank `me`:
    moves data from every rank's input box to every rank's output box.
    inboxes / outboxes: the box3d of every rank of the group.  pack() fills a
    send buffer, unpack() empties a receive buffer, both on the device; the
    exchange between them (counts(): elements per rank, rank order) is the
    caller's all-to-all."""

    def __init__(self, inboxes, outboxes, me):
        self.nranks = len(inboxes)
        self.me = me
        flat = lambda bs: (ctypes.c_int * (9 * len(bs)))(*[int(v) for b in bs for v in (*b.low, *b.high, *b.order)])
        self._h = ctypes.c_void_p()
        check(lib().heffte_gb300_reshape_create(self.nranks, me, flat(inboxes), flat(outboxes), ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.heffte_gb300_reshape_destroy(h)

    def send_size(self):
        return lib().heffte_gb300_reshape_send_size(self._h)

    def recv_size(self):
        return lib().heffte_gb300_reshape_recv_size(self._h)

    def counts(self):
        """(send_counts, send_displs, recv_counts, recv_displs), lists of nranks ints."""
        arrs = [(ctypes.c_longlong * self.nranks)() for _ in range(4)]
        check(lib().heffte_gb300_reshape_counts(self._h, *arrs))
        return tuple(list(a) for a in arrs)

    def pack(self, dtype, inp, send_buffer, stream=None):
        check(lib().heffte_gb300_reshape_pack(self._h, _stream_handle(stream), dtype, _ptr(inp), _ptr(send_buffer)))

    def unpack(self, dtype, recv_buffer, out, stream=None):
        check(lib().heffte_gb300_reshape_unpack(self._h, _stream_handle(stream), dtype, _ptr(recv_buffer), _ptr(out)))


# -- location layer ---------------------------------------------------------
def direct_pack(dtype, nfast, nmid, nslow, line_stride, plane_stride, src, dst, stream=None):
    check(lib().heffte_gb300_direct_pack(_stream_handle(stream), dtype, nfast, nmid, nslow, line_stride,
                                         plane_stride, _ptr(src), _ptr(dst)))


def direct_unpack(dtype, nfast, nmid, nslow, line_stride, plane_stride, src, dst, stream=None):
    check(lib().heffte_gb300_direct_unpack(_stream_handle(stream), dtype, nfast, nmid, nslow, line_stride,
                                           plane_stride, _ptr(src), _ptr(dst)))


def transpose_unpack(dtype, nfast, nmid, nslow, line_stride, plane_stride, buff_line_stride, buff_plane_stride,
                     mp, src, dst, stream=None):
    check(lib().heffte_gb300_transpose_unpack(_stream_handle(stream), dtype, nfast, nmid, nslow, line_stride,
                                              plane_stride, buff_line_stride, buff_plane_stride, mp[0], mp[1], mp[2],
                                              _ptr(src), _ptr(dst)))


def scale_data(prec, num_reals, data, factor, stream=None):
    check(lib().heffte_gb300_scale_data(_stream_handle(stream), prec, num_reals, _ptr(data), factor))


def convert(prec, n, src, dst, to_complex, stream=None):
    check(lib().heffte_gb300_convert(_stream_handle(stream), prec, n, _ptr(src), _ptr(dst), int(to_complex)))


def r2r_prepost(prec, rkind, step, length, lines, in_ld, out_ld, src, dst, stream=None):
    """Batched extended-signal pre/post processing (cos 0, sin 1, cos1 2; steps 0..3)."""
    check(lib().heffte_gb300_r2r_prepost(_stream_handle(stream), prec, rkind, step, length, lines, in_ld, out_ld,
                                         _ptr(src), _ptr(dst)))


def set_kernel_variant(variant):
    """0 automatic, 1 generic runtime-radix kernels, 2 pipelined kernels where they
    apply, 3 automatic with the runtime radix plan for every length that is not a
    power of two (no kernels compiled for one length's plan)."""
    check(lib().heffte_gb300_set_kernel_variant(int(variant)))


def device_status(reset=False):
    """Status word of the current device: 0 = no kernel gave up a bounded wait;
    1 a bulk-copy wait, 2 a batch pass-dependency wait, 3 a tensor-core MMA wait."""
    v = ctypes.c_int(-1)
    check(lib().heffte_gb300_device_status(ctypes.byref(v), int(reset)))
    return v.value


DEV_TIMEOUT_BULK_COPY, DEV_TIMEOUT_DEPENDENCY, DEV_TIMEOUT_MMA = 1, 2, 3

FP64, DOUBLE_FLOAT = 0, 1


def set_double_arithmetic(mode):
    """Arithmetic of the power-of-two complex<double> passes: FP64 (FP64
    instructions) or DOUBLE_FLOAT (pairs of floats on the FP32 pipe); returns
    the previous mode."""
    old = lib().heffte_gb300_double_arithmetic()
    check(lib().heffte_gb300_set_double_arithmetic(int(mode)))
    return old



def set_dependency_wait_budget(clocks):
    """Clock budget of the batch kernel's waits for another CTA's pass of the
    same box (default 4e9); returns the previous budget."""
    old = lib().heffte_gb300_dependency_wait_budget()
    check(lib().heffte_gb300_set_dependency_wait_budget(int(clocks)))
    return old


class boxbatch:
    """Many small 3-D boxes of uneven sizes transformed in one persistent,
    graph-replayed launch (kind.r2c or kind.c2c; r2c along dimension 0)."""

    def __init__(self, bkind, sizes, prec=0, stream=None):
        flat = [int(v) for s in sizes for v in s]
        self.sizes = [tuple(s) for s in sizes]
        self.prec = prec
        self._h = ctypes.c_void_p()
        check(lib().heffte_gb300_boxbatch_create(bkind, prec, len(self.sizes), (ctypes.c_int * len(flat))(*flat),
                                                 _stream_handle(stream), ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.heffte_gb300_boxbatch_destroy(h)

    def input_offset(self, box):
        return lib().heffte_gb300_boxbatch_input_offset(self._h, box)

    def output_offset(self, box):
        return lib().heffte_gb300_boxbatch_output_offset(self._h, box)

    def input_size(self):
        return lib().heffte_gb300_boxbatch_input_size(self._h)

    def output_size(self):
        return lib().heffte_gb300_boxbatch_output_size(self._h)

    def workspace_size(self):
        return lib().heffte_gb300_boxbatch_workspace_size(self._h)

    def configure(self, prefetch=0, tile_kb=48, group_mb=0, values=0):
        """Launch shape: prefetch of each CTA's next tile, tile bound in KB,
        queue order (boxes in L2-sized groups of group_mb MB, 0: pass-major),
        complex values per thread (8, 16; 0: 16)."""
        check(lib().heffte_gb300_boxbatch_configure(self._h, int(prefetch), int(tile_kb), int(group_mb), int(values)))

    def config(self):
        """(prefetch, tile_kb, group_mb, values per thread in use)."""
        v = [ctypes.c_int(0) for _ in range(4)]
        check(lib().heffte_gb300_boxbatch_config(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def autotune(self, inarray, outarray, back, workspace, reps=5):
        """Times every launch shape on these buffers (forward in -> out,
        backward out -> back) and keeps the fastest; returns (prefetch,
        tile_kb, group_mb, values, ms per forward + backward)."""
        v = [ctypes.c_int(0) for _ in range(4)]
        ms = ctypes.c_double(0)
        check(lib().heffte_gb300_boxbatch_autotune(self._h, _ptr(inarray), _ptr(outarray), _ptr(back), _ptr(workspace),
                                                   int(reps), *[ctypes.byref(x) for x in v], ctypes.byref(ms)))
        return tuple(x.value for x in v) + (ms.value,)

    def hold_dependencies(self, hold):
        """Test hook: every pass dependency waits for a tile that never comes
        (hold=True), so the waits run out of their budget; False restores."""
        check(lib().heffte_gb300_boxbatch_hold_dependencies(self._h, int(bool(hold))))

    def forward(self, inarray, outarray, scaling=scale.none):
        check(lib().heffte_gb300_boxbatch_forward(self._h, _ptr(inarray), _ptr(outarray), scaling))

    def backward(self, inarray, outarray, workspace, scaling=scale.none):
        check(lib().heffte_gb300_boxbatch_backward(self._h, _ptr(inarray), _ptr(outarray), _ptr(workspace), scaling))


def tune(prec, lengths, cache_path=None, stream=None):
    """Autotunes the radix plan / tile size of each length; returns how many were measured."""
    arr = (ctypes.c_int * len(lengths))(*[int(n) for n in lengths])
    m = ctypes.c_int(0)
    check(lib().heffte_gb300_tune(prec, len(lengths), arr, cache_path.encode() if cache_path else None,
                                  _stream_handle(stream), ctypes.byref(m)))
    return m.value


def tune_load(cache_path):
    n = ctypes.c_int(0)
    check(lib().heffte_gb300_tune_load(cache_path.encode(), ctypes.byref(n)))
    return n.value


def tune_clear():
    check(lib().heffte_gb300_tune_clear())


def tuned_choice(prec, length):
    rad = (ctypes.c_int * 16)()
    nr, tpb, us = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
    check(lib().heffte_gb300_tuned_choice(prec, length, rad, ctypes.byref(nr), ctypes.byref(tpb), ctypes.byref(us)))
    return list(rad[:nr.value]), tpb.value, us.value
