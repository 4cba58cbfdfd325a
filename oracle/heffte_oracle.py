"""CPU oracle for heFFTe's fft3d hot path (numpy, float64).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the
checker: the product path (``heffte_gb300``) never imports it.

It restates, vectorised over lines with numpy, what the reference computes on
a single rank:

* box layout: an array for a box with ``order = (o0, o1, o2)`` is stored with
  ``o0`` fastest (``include/heffte_geometry.h:34-60``);
* ``fft3d::forward/backward`` with ``scale::none|full|symmetric``
  (``include/heffte_fft3d.h:140-147, 353-547``): forward uses exp(-2 pi i k n / N),
  backward exp(+...) unnormalised;
* ``fft3d_r2c`` (``include/heffte_fft3d_r2c.h:146-292``) with the output box
  ``box3d::r2c(dir)`` (``include/heffte_geometry.h:85-93``);
* ``rtransform`` DCT/DST via the extended-signal pre/post processors of
  ``include/heffte_r2r_executor.h:43-180`` and the scale table of
  ``include/heffte_fft3d.h:635-650`` (stock/cuFFT tags: 1/(64 N), DCT-I:
  1/(64 prod(n-1)));
* ``direct_packer`` / ``transpose_packer<tag::cpu>`` and ``data_scaling``
  (``include/heffte_pack3d.h:83-233``);
* the step of the convolution benchmark (``benchmarks/convolution.cpp:89-95``:
  forward, pointwise product, backward) and the circular convolution it
  builds on (``convolve``, ``convolution_benchmark_step``).

The FFTs themselves are pocketfft in float64 (scipy.fft with all host
threads, else numpy.fft: an FP64 oracle); the
restated parts are the conventions, layouts and pre/post processing above.
Parity of this module is pinned against the reference's own outputs by the
golden fixtures in ``tests/golden`` (generated by compiling the reference's
stock backend, see ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# FP64 FFTs: pocketfft, through scipy.fft with all host threads where scipy is
# installed (the full-size checks of 512^3 and 1024x1024x512 boxes), else
# numpy.fft (the same algorithm, one thread).
try:
    import scipy.fft as _sfft
    _WORKERS = os.cpu_count() or 1

    def _call(name, *a, **k):
        return getattr(_sfft, name)(*a, workers=_WORKERS, **k)
except ImportError:  # pragma: no cover - scipy is present where the tests run
    def _call(name, *a, **k):
        return getattr(np.fft, name)(*a, **k)


def fftn(a, axes=None):
    return _call("fftn", a, axes=axes)


def ifftn(a, axes=None):
    return _call("ifftn", a, axes=axes)


def fft(a, axis=-1):
    return _call("fft", a, axis=axis)


def ifft(a, axis=-1):
    return _call("ifft", a, axis=axis)


def rfft(a, axis=-1):
    return _call("rfft", a, axis=axis)


def irfft(a, n=None, axis=-1):
    return _call("irfft", a, n=n, axis=axis)

SCALE_NONE, SCALE_FULL, SCALE_SYMMETRIC = 0, 1, 2
COS, SIN, COS1 = 0, 1, 2


# --------------------------------------------------------------------------
# box layout helpers (heffte_geometry.h:67-133)
# --------------------------------------------------------------------------
def box_size(lo, hi):
    return tuple(int(hi[i]) - int(lo[i]) + 1 for i in range(3))


def to_canonical(flat, size, order):
    """Flat array of a box in ``order`` -> ndarray indexed [k][j][i] (dim 2, 1, 0)."""
    o0, o1, o2 = order
    a = np.asarray(flat).reshape(size[o2], size[o1], size[o0])
    # axis a of `a` holds dim (o2, o1, o0)[a]; canonical axis c holds dim 2 - c
    dims_of_axes = (o2, o1, o0)
    perm = [dims_of_axes.index(2 - c) for c in range(3)]
    return np.transpose(a, perm)


def from_canonical(arr, order):
    """ndarray indexed [k][j][i] -> flat array of the box in ``order``."""
    o0, o1, o2 = order
    perm = [2 - o2, 2 - o1, 2 - o0]
    return np.ascontiguousarray(np.transpose(arr, perm)).ravel()


def axis_of(dim):
    return 2 - dim


def scale_factor(scaling, count):
    if scaling == SCALE_NONE:
        return 1.0
    f = 1.0 / float(count)
    return f if scaling == SCALE_FULL else np.sqrt(f)


# --------------------------------------------------------------------------
# transforms
# --------------------------------------------------------------------------
def fft3d_c2c(x, size, in_order=(0, 1, 2), out_order=(0, 1, 2), direction=0, scaling=SCALE_NONE):
    """fft3d<...>::forward (direction 0) / backward (1), complex128 result."""
    c = to_canonical(np.asarray(x, dtype=np.complex128), size, in_order)
    n = int(np.prod(size))
    if direction == 0:
        y = fftn(c)
    else:
        y = ifftn(c) * n
    y = y * scale_factor(scaling, n)
    return from_canonical(y, out_order)


def r2c_size(size, r2c_dir):
    s = list(size)
    s[r2c_dir] = size[r2c_dir] // 2 + 1
    return tuple(s)


def fft3d_r2c(x, size, r2c_dir, in_order=(0, 1, 2), out_order=(0, 1, 2), scaling=SCALE_NONE):
    """fft3d_r2c::forward: real box -> complex box.r2c(r2c_dir)."""
    c = to_canonical(np.asarray(x, dtype=np.float64), size, in_order)
    n = int(np.prod(size))
    y = fftn(c)
    ax = axis_of(r2c_dir)
    y = np.take(y, np.arange(size[r2c_dir] // 2 + 1), axis=ax)
    y = y * scale_factor(scaling, n)
    return from_canonical(y, out_order)


def fft3d_c2r(x, size, r2c_dir, in_order=(0, 1, 2), out_order=(0, 1, 2), scaling=SCALE_NONE):
    """fft3d_r2c::backward: complex box.r2c(r2c_dir) -> real box (unnormalised)."""
    csize = r2c_size(size, r2c_dir)
    c = to_canonical(np.asarray(x, dtype=np.complex128), csize, in_order)
    n = int(np.prod(size))
    ax = axis_of(r2c_dir)
    others = [a for a in range(3) if a != ax]
    y = ifftn(c, axes=others) * (size[2 - others[0]] * size[2 - others[1]])
    y = irfft(y, n=size[r2c_dir], axis=ax) * size[r2c_dir]
    y = y * scale_factor(scaling, n)
    return from_canonical(y, out_order)


def convolve(x, y, size, r2c_dir=None, order=(0, 1, 2), scaling=SCALE_FULL):
    """backward(forward(x) .* forward(y)) with the backward scaling: the step of
    benchmarks/convolution.cpp:89-95 (forward, pointwise product, backward)
    with both forward transforms unscaled.  y None: x .* x.  r2c_dir None:
    complex arrays through fft3d; else real arrays through fft3d_r2c (the
    product on the half spectrum)."""
    n = int(np.prod(size))
    if r2c_dir is None:
        fx = fft3d_c2c(x, size, order, order)
        fy = fx if y is None else fft3d_c2c(y, size, order, order)
        return fft3d_c2c(fx * fy, size, order, order, direction=1, scaling=scaling)
    fx = fft3d_r2c(x, size, r2c_dir, order, order)
    fy = fx if y is None else fft3d_r2c(y, size, r2c_dir, order, order)
    return fft3d_c2r(fx * fy, size, r2c_dir, order, order, scaling=scaling)


def convolution_benchmark_step(x, size):
    """The in-place step timed by benchmarks/convolution.cpp:89-95:
    forward with scale::full, X .* X, backward unscaled."""
    f = fft3d_c2c(x, size, scaling=SCALE_FULL)
    return fft3d_c2c(f * f, size, direction=1)


def _r2r_forward_1d(kind, x):
    """Forward r2r along the last axis through the extended signal
    (cpu_*_pre_pos_processor::pre_forward/post_forward)."""
    N = x.shape[-1]
    lead = x.shape[:-1]
    if kind == COS:
        M = 4 * N
        sig = np.zeros(lead + (M + 1,))
        sig[..., 1:2 * N:2] = x
        sig[..., 4 * N - np.arange(2 * N)] = sig[..., :2 * N]
        f = rfft(sig[..., :M], axis=-1)
        return f[..., :N].real
    if kind == SIN:
        M = 4 * N
        sig = np.zeros(lead + (M + 1,))
        sig[..., 1:2 * N:2] = x
        i = np.arange(N)
        sig[..., 4 * N - 2 * i - 1] = -x
        f = rfft(sig[..., :M], axis=-1)
        return -f[..., 1:N + 1].imag
    # COS1
    M = 4 * (N - 1)
    sig = np.zeros(lead + (M,))
    i = np.arange(N - 1)
    sig[..., 2 * i] = x[..., :N - 1]
    i = np.arange(1, N)
    sig[..., 4 * (N - 1) - 2 * i] = x[..., 1:]
    f = rfft(sig, axis=-1)
    return f[..., :N].real


def _r2r_backward_1d(kind, x):
    """Backward r2r along the last axis (pre_backward, c2r, post_backward)."""
    N = x.shape[-1]
    lead = x.shape[:-1]
    M = 4 * (N - 1) if kind == COS1 else 4 * N
    H = M // 2 + 1
    cs = np.zeros(lead + (H,), dtype=np.complex128)
    if kind == COS:
        cs[..., :N] = x
        cs[..., N + 1:2 * N + 1] = -x[..., ::-1]
    elif kind == SIN:
        cs[..., 1:N + 1] = -1j * x
        cs[..., N + 1:2 * N] = -1j * x[..., N - 2::-1]
    else:
        cs[..., :N] = x
        cs[..., N:2 * N - 1] = x[..., N - 2::-1]
    r = irfft(cs, n=M, axis=-1) * M
    if kind == COS1:
        return r[..., 0:2 * N:2]
    return r[..., 1:2 * N:2]


def rtransform(kind, x, size, in_order=(0, 1, 2), out_order=(0, 1, 2), direction=0, scaling=SCALE_NONE):
    """rtransform<*_cos|*_sin|*_cos1>::forward/backward, float64 result."""
    c = to_canonical(np.asarray(x, dtype=np.float64), size, in_order)
    fn = _r2r_forward_1d if direction == 0 else _r2r_backward_1d
    for dim in range(3):
        ax = axis_of(dim)
        c = np.moveaxis(fn(kind, np.moveaxis(c, ax, -1)), -1, ax)
    if scaling != SCALE_NONE:
        if kind == COS1:
            f = 1.0 / (64.0 * np.prod([s - 1 for s in size]))
        else:
            f = 1.0 / (64.0 * np.prod(size))
        c = c * (f if scaling == SCALE_FULL else np.sqrt(f))
    return from_canonical(c, out_order)


def executor_c2c(x, size, order, dimension, direction=0):
    """One executor stage: the batch of 1-D transforms along `dimension`."""
    c = to_canonical(np.asarray(x, dtype=np.complex128), size, order)
    ax = axis_of(dimension)
    y = fft(c, axis=ax) if direction == 0 else ifft(c, axis=ax) * size[dimension]
    return from_canonical(y, order)


# --------------------------------------------------------------------------
# pack / unpack / transpose (heffte_pack3d.h:83-197) — bit-exact index maps
# --------------------------------------------------------------------------
def _strided_view_index(size, line_stride, plane_stride):
    k, j, i = np.meshgrid(np.arange(size[2]), np.arange(size[1]), np.arange(size[0]), indexing="ij")
    return (k * plane_stride + j * line_stride + i).ravel()


def direct_pack(src, size, line_stride, plane_stride):
    """buffer[(slow*nmid + mid)*nfast + fast] = data[slow*plane + mid*line + fast]."""
    return np.asarray(src)[_strided_view_index(size, line_stride, plane_stride)].copy()


def direct_unpack(buf, dst, size, line_stride, plane_stride):
    out = np.array(dst, copy=True)
    out[_strided_view_index(size, line_stride, plane_stride)] = np.asarray(buf)[:int(np.prod(size))]
    return out


def transpose_source_index(size, buff_line_stride, buff_plane_stride, mp):
    """Source offsets for transpose_packer<tag::cpu>::unpack, in destination
    order (slow k, mid j, fast i) — the six map cases of heffte_pack3d.h:139-196."""
    k, j, i = np.meshgrid(np.arange(size[2]), np.arange(size[1]), np.arange(size[0]), indexing="ij")
    bl, bp = buff_line_stride, buff_plane_stride
    m0, m1 = mp[0], mp[1]
    if m0 == 0 and m1 == 1:
        s = k * bp + j * bl + i
    elif m0 == 0 and m1 == 2:
        s = j * bp + k * bl + i
    elif m0 == 1 and m1 == 0:
        s = k * bp + i * bl + j
    elif m0 == 1 and m1 == 2:
        s = i * bp + k * bl + j
    elif m0 == 2 and m1 == 0:
        s = j * bp + i * bl + k
    else:
        s = i * bp + j * bl + k
    return s.ravel()


def transpose_unpack(buf, dst, size, line_stride, plane_stride, buff_line_stride, buff_plane_stride, mp):
    out = np.array(dst, copy=True)
    didx = _strided_view_index(size, line_stride, plane_stride)
    sidx = transpose_source_index(size, buff_line_stride, buff_plane_stride, mp)
    out[didx] = np.asarray(buf)[sidx]
    return out


# --------------------------------------------------------------------------
# multi-rank reshape (reshape3d_alltoallv, src/heffte_reshape3d.cpp:147-233,
# 365-496): boxes are (low, high, order) triples
# --------------------------------------------------------------------------
def _osize(box, d):
    lo, hi, order = box
    return hi[order[d]] - lo[order[d]] + 1


def box_count(box):
    lo, hi, _ = box
    return max(0, int(np.prod([hi[d] - lo[d] + 1 for d in range(3)]))) if all(hi[d] >= lo[d] for d in range(3)) else 0


def collide(a, b):
    """box3d::collide: the intersection in the order of `a` (None if empty)."""
    lo = tuple(max(a[0][d], b[0][d]) for d in range(3))
    hi = tuple(min(a[1][d], b[1][d]) for d in range(3))
    return None if any(hi[d] < lo[d] for d in range(3)) else (lo, hi, tuple(a[2]))


def reshape_counts(me, inboxes, outboxes):
    """Elements rank `me` sends to / receives from every rank (rank order)."""
    n = len(inboxes)
    send = [0] * n
    recv = [0] * n
    for r in range(n):
        o = collide(inboxes[me], outboxes[r]) if box_count(inboxes[me]) and box_count(outboxes[r]) else None
        send[r] = box_count(o) if o else 0
        o = collide(outboxes[me], inboxes[r]) if box_count(outboxes[me]) and box_count(inboxes[r]) else None
        recv[r] = box_count(o) if o else 0
    return send, recv


def _offset_in(box, ov):
    lo, _, order = box
    return ((ov[0][order[2]] - lo[order[2]]) * _osize(box, 0) * _osize(box, 1) +
            (ov[0][order[1]] - lo[order[1]]) * _osize(box, 0) + (ov[0][order[0]] - lo[order[0]]))


def reshape_pack(me, inboxes, outboxes, data):
    """The send buffer of rank `me`: the overlap of its input box with each
    rank's output box, in rank order, each packed in the input box's order
    (direct_pack, compute_overlap_map_direct_pack :147-167)."""
    box = inboxes[me]
    parts = []
    for r in range(len(inboxes)):
        o = collide(box, outboxes[r]) if box_count(box) and box_count(outboxes[r]) else None
        if o is None:
            continue
        size = tuple(_osize(o, d) for d in range(3))
        off = _offset_in(box, o)
        parts.append(direct_pack(np.asarray(data)[off:], size, _osize(box, 0), _osize(box, 0) * _osize(box, 1)))
    return np.concatenate(parts) if parts else np.zeros(0, np.asarray(data).dtype)


def reshape_unpack(me, inboxes, outboxes, recv, out):
    """Scatters rank `me`'s receive buffer (chunks in rank order, each in the
    sender's input order) into its output box (transpose_unpack with the map
    of compute_overlap_map_transpose_pack :197-222)."""
    box = outboxes[me]
    out = np.array(out, copy=True)
    pos = 0
    for r in range(len(inboxes)):
        src = inboxes[r]
        o = collide(box, src) if box_count(box) and box_count(src) else None
        if o is None:
            continue
        size = tuple(_osize(o, d) for d in range(3))
        mp = [0, 0, 0]
        for j in range(3):
            for k in range(3):
                if box[2][k] == src[2][j]:
                    mp[j] = k
        n = box_count(o)
        ext = [o[1][d] - o[0][d] + 1 for d in range(3)]
        bls, bps = ext[src[2][0]], ext[src[2][0]] * ext[src[2][1]]
        off = _offset_in(box, o)
        view = out[off:]
        view = transpose_unpack(recv[pos:pos + n], view, size, _osize(box, 0), _osize(box, 0) * _osize(box, 1),
                                bls, bps, tuple(mp))
        out[off:] = view
        pos += n
    return out


def box_slice(global_canonical, box):
    """The values of `box` (in its order) from an array indexed [k][j][i]."""
    lo, hi, order = box
    sub = global_canonical[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
    return from_canonical(sub, order)


def scale_data(x, factor, dtype):
    """data_scaling::apply: x *= (scalar)factor in the working precision."""
    x = np.asarray(x)
    if np.iscomplexobj(x):
        r = x.view(dtype)
        return (r * dtype(factor)).view(x.dtype)
    return x * dtype(factor)


# --------------------------------------------------------------------------
# compiled checkers: the C port (any host) and the reference build (here)
# --------------------------------------------------------------------------
PORT_LIB = os.path.join(HERE, "_build", "libheffte_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libheffte_ref.so")

_port = None
_ref = None


def load_port():
    """ctypes handle of the C restatement (oracle/port), or None if unbuilt."""
    global _port
    if _port is None and os.path.exists(PORT_LIB):
        lib = ctypes.CDLL(PORT_LIB)
        LL3 = ctypes.c_longlong * 3
        vp, i, ll, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
        lib.port_fft3d_c2c.argtypes = [i, LL3, i, i, vp, vp, i]
        lib.port_fft3d_r2c.argtypes = [i, LL3, i, i, i, vp, vp, i]
        lib.port_rtransform.argtypes = [i, i, LL3, i, i, vp, vp, i]
        lib.port_pack.argtypes = [i, i, LL3, ll, ll, ll, ll, ctypes.c_int * 3, vp, vp]
        lib.port_scale.argtypes = [i, ll, vp, d, i]
        _port = lib
    return _port


def load_ref():
    """ctypes handle of the compiled reference (oracle/_ref), or None."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        lib = ctypes.CDLL(REF_LIB)
        I3 = ctypes.c_int * 3
        LL3 = ctypes.c_longlong * 3
        vp, i, ll, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
        lib.ref_fft3d_c2c.argtypes = [i, I3, I3, I3, I3, i, i, i, i, vp, vp]
        lib.ref_fft3d_r2c.argtypes = [i, I3, I3, I3, I3, i, i, i, i, i, vp, vp]
        lib.ref_rtransform.argtypes = [i, i, I3, I3, I3, I3, i, i, i, i, vp, vp]
        lib.ref_executor_c2c.argtypes = [i, I3, I3, I3, i, i, vp]
        lib.ref_pack.argtypes = [i, i, LL3, ll, ll, ll, ll, I3, vp, vp]
        lib.ref_scale.argtypes = [i, ll, vp, d]
        _ref = lib
    return _ref


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def port_fft3d_c2c(x, size, direction=0, scaling=SCALE_NONE, threads=1):
    lib = load_port()
    prec = 0 if x.dtype == np.complex64 else 1
    out = np.empty_like(x)
    lib.port_fft3d_c2c(prec, (ctypes.c_longlong * 3)(*size), direction, scaling, _ptr(x), _ptr(out), threads)
    return out


def port_fft3d_r2c(x, size, r2c_dir, direction=0, scaling=SCALE_NONE, threads=1):
    lib = load_port()
    if direction == 0:
        prec = 0 if x.dtype == np.float32 else 1
        out = np.empty(int(np.prod(r2c_size(size, r2c_dir))), dtype=np.complex64 if prec == 0 else np.complex128)
    else:
        prec = 0 if x.dtype == np.complex64 else 1
        out = np.empty(int(np.prod(size)), dtype=np.float32 if prec == 0 else np.float64)
    lib.port_fft3d_r2c(prec, (ctypes.c_longlong * 3)(*size), r2c_dir, direction, scaling, _ptr(x), _ptr(out), threads)
    return out


def port_rtransform(kind, x, size, direction=0, scaling=SCALE_NONE, threads=1):
    lib = load_port()
    prec = 0 if x.dtype == np.float32 else 1
    out = np.empty_like(x)
    lib.port_rtransform(kind, prec, (ctypes.c_longlong * 3)(*size), direction, scaling, _ptr(x), _ptr(out), threads)
    return out


def port_pack(op, src, dst, size, ls, ps, bls=0, bps=0, mp=(0, 1, 2)):
    lib = load_port()
    out = np.array(dst, copy=True)
    lib.port_pack(op, src.itemsize, (ctypes.c_longlong * 3)(*size), ls, ps, bls, bps, (ctypes.c_int * 3)(*mp),
                  _ptr(src), _ptr(out))
    return out


def rel_l2(a, b, chunk=1 << 24):
    """||a - b|| / ||b|| in float64, in chunks (full-size boxes hold 2^29
    values), both scaled by the largest |b| so that squares of magnitudes near
    the float64 limits neither overflow nor underflow."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    assert a.size == b.size, (a.size, b.size)
    dt = np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64
    m = 0.0
    for i in range(0, b.size, chunk):
        m = max(m, float(np.max(np.abs(b[i:i + chunk].astype(dt)))) if b[i:i + chunk].size else 0.0)
    m = m if m > 0 and np.isfinite(m) else 1.0
    num = den = 0.0
    for i in range(0, a.size, chunk):
        ai = a[i:i + chunk].astype(dt) / m
        bi = b[i:i + chunk].astype(dt) / m
        num += float(np.sum(np.abs(ai - bi) ** 2))
        den += float(np.sum(np.abs(bi) ** 2))
    return float(np.sqrt(num) / (np.sqrt(den) if den > 0 else 1.0))


def prepost_line(kind, step, x, N):
    """One line of cpu_{cos,sin,cos1}_pre_pos_processor (heffte_r2r_executor.h:43-180),
    restated loop by loop.  step 0 pre_forward, 1 post_forward, 2 pre_backward,
    3 post_backward.  Returns the output line (pre_forward: the M entries of the
    extended signal, without the extra entry 4N the reference also zeroes)."""
    M = 4 * (N - 1) if kind == COS1 else 4 * N
    if step == 0:
        sig = np.zeros(M + 1, dtype=x.dtype)
        if kind == COS:
            for i in range(N):
                sig[2 * i] = 0
                sig[2 * i + 1] = x[i]
            sig[2 * N] = 0
            for i in range(2 * N):
                sig[4 * N - i] = sig[i]
        elif kind == SIN:
            for i in range(N):
                sig[2 * i] = 0
                sig[2 * i + 1] = x[i]
            sig[2 * N] = 0
            for i in range(N):
                sig[4 * N - 2 * i] = 0
                sig[4 * N - 2 * i - 1] = -x[i]
        else:
            for i in range(N - 1):
                sig[2 * i] = x[i]
                sig[2 * i + 1] = 0
            for i in range(1, N):
                sig[4 * (N - 1) - 2 * i] = x[i]
                sig[4 * (N - 1) - 2 * i + 1] = 0
        return sig[:M]
    if step == 1:
        if kind == SIN:
            return np.array([-x[i + 1].imag for i in range(N)], dtype=x.real.dtype)
        return np.array([x[i].real for i in range(N)], dtype=x.real.dtype)
    if step == 2:
        H = M // 2 + 1
        cdt = np.complex64 if x.dtype == np.float32 else np.complex128
        sig = np.zeros(H, dtype=cdt)
        if kind == COS:
            for i in range(N):
                sig[i] = x[i]
            sig[N] = 0
            idx = N - 1
            for i in range(N + 1, 2 * N + 1):
                sig[i] = -x[idx]
                idx -= 1
        elif kind == SIN:
            sig[0] = 0
            for i in range(N):
                sig[i + 1] = -1j * x[i]
            sig[2 * N] = 0
            for i in range(N - 1):
                sig[N + i + 1] = -1j * x[N - i - 2]
        else:
            for i in range(N):
                sig[i] = x[i]
            idx = N - 2
            for i in range(N, 2 * N - 1):
                sig[i] = x[idx]
                idx -= 1
        return sig
    if kind == COS1:
        return np.array([x[2 * i] for i in range(N)], dtype=x.dtype)
    return np.array([x[2 * i + 1] for i in range(N)], dtype=x.dtype)
