"""Learned plan selection for heffte_gb300 plans.

* ``sample_shapes`` draws the selector workload: box sides 32..768, 80% with
  only factors 2, 3, 5 and 20% with a factor 7 or 11, a mix of c2c / r2c /
  DCT-II and float / double; volumes are capped (``max_elems``) so that every
  candidate of every shape can be timed.
* ``measure`` is the exhaustive autotuner: it times every candidate plan (the
  16 combinations of use_reorder x kernel family x tile size x radix order,
  ``heffte_gb300_candidate_options``) of every shape with CUDA events and
  appends the timings to an ``.npz`` dataset after each chunk, so an
  interrupted measurement resumes where it stopped.
* ``train`` fits the 3-layer MLP (``heffte_gb300_mlp_*``: forward, backward
  and Adam are this library's CUDA kernels) to predict, per candidate, the
  log2 slow-down against the best candidate of the shape.
* ``regret`` compares the chosen candidate's time with the exhaustive best.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import HeffteError, box3d, check, fft3d, fft3d_r2c, kind, lib, plan_options, rtransform, scale

N_FEATURES = 18
N_CANDIDATES = 16
KINDS = (kind.c2c, kind.r2c, kind.cos)


def _sides(lo=32, hi=768):
    smooth = sorted({2 ** a * 3 ** b * 5 ** c for a in range(11) for b in range(7) for c in range(5)
                     if lo <= 2 ** a * 3 ** b * 5 ** c <= hi})
    rough = sorted({n for n in range(lo, hi + 1) if (n % 7 == 0 or n % 11 == 0) and _only(n, (2, 3, 5, 7, 11))})
    return smooth, rough


def _only(n, primes):
    for p in primes:
        while n % p == 0:
            n //= p
    return n == 1


def sample_shapes(n, seed=2000, max_elems=1 << 26):
    """n shapes (size, kind, prec): sides 32..768, 80% 5-smooth, 20% with a 7 or 11."""
    rng = np.random.default_rng(seed)
    smooth, rough = _sides()
    out = []
    while len(out) < n:
        use_rough = rng.random() < 0.2
        size = [int(rng.choice(smooth)) for _ in range(3)]
        if use_rough:
            size[int(rng.integers(0, 3))] = int(rng.choice(rough))
        if size[0] * size[1] * size[2] > max_elems:
            continue
        out.append((tuple(size), int(rng.choice(KINDS)), int(rng.integers(0, 2))))
    return out


def features(size, tkind, prec):
    f = (ctypes.c_float * N_FEATURES)()
    check(lib().heffte_gb300_plan_features(tkind, prec, (ctypes.c_int * 3)(*size), f))
    return np.array(f[:], dtype=np.float32)


def candidate(c):
    L = lib()
    opts = plan_options()
    v, t, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(L.heffte_gb300_candidate_options(c, ctypes.byref(opts), ctypes.byref(v), ctypes.byref(t), ctypes.byref(r)))
    return opts, v.value, t.value, r.value


def make_plan(size, tkind, prec, c, stream=None):
    opts, v, t, r = candidate(c)
    box = box3d((0, 0, 0), [s - 1 for s in size])
    if tkind == kind.c2c:
        p = fft3d(box, box, opts, stream)
    elif tkind == kind.r2c:
        p = fft3d_r2c(box, box.r2c(0), 0, opts, stream)
    else:
        p = rtransform(tkind, box, box, opts, stream)
    p.set_knobs(v, t, r)
    return p


def measure(shapes, path=None, reps=3, chunk=50, log=None):
    """Times every candidate of every shape; returns (X features, T seconds [n x 16]).

    A candidate the library refuses for a shape is recorded as NaN."""
    import torch
    done_X, done_T, start = [], [], 0
    if path and os.path.exists(path):
        d = np.load(path)
        done_X, done_T = list(d["X"]), list(d["T"])
        start = len(done_X)
    if start >= len(shapes):
        return np.array(done_X[:len(shapes)]), np.array(done_T[:len(shapes)])
    stream = torch.cuda.current_stream()
    max_elems = max(s[0] * s[1] * s[2] for s, _, _ in shapes)
    # input, output: one complex128 per element (+ the r2c half-line padding); workspace: four
    bufs = [torch.zeros(n * max_elems + (1 << 16), dtype=torch.complex128, device="cuda") for n in (2, 2, 4)]
    work_bytes = bufs[2].numel() * 16
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(start, len(shapes)):
        size, tkind, prec = shapes[i]
        times = np.full(N_CANDIDATES, np.nan)
        for c in range(N_CANDIDATES):
            try:
                p = make_plan(size, tkind, prec, c, stream)
            except HeffteError:
                continue
            es = 16 if prec == 1 else 8
            if p.size_workspace() * es > work_bytes:
                raise RuntimeError(f"workspace of {size} exceeds the measurement buffer")
            args = (prec, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), scale.none)
            p.forward_ptr(*args)
            ts = []
            for _ in range(reps):
                e0.record(stream)
                p.forward_ptr(*args)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1) * 1e-3)
            times[c] = float(np.median(ts))
            del p
        done_X.append(features(size, tkind, prec))
        done_T.append(times)
        if path and ((i + 1) % chunk == 0 or i + 1 == len(shapes)):
            np.savez(path, X=np.array(done_X), T=np.array(done_T))
            if log:
                log(f"measured {i + 1}/{len(shapes)}")
    return np.array(done_X), np.array(done_T)


def filled(T):
    """Times with refused candidates (NaN) replaced by four times the slowest measured one."""
    T = np.array(T, dtype=np.float64)
    worst = np.nanmax(T, axis=1, keepdims=True)
    return np.where(np.isnan(T), 4.0 * worst, T)


def targets(T):
    """log2 slow-down of each candidate against the best one of its shape."""
    T = filled(T)
    return np.log2(T / T.min(axis=1, keepdims=True)).astype(np.float32)


class Selector:
    """The MLP (18 -> 64 -> 64 -> 16) on the GPU."""

    def __init__(self, hidden=64, seed=1):
        self._h = ctypes.c_void_p()
        check(lib().heffte_gb300_mlp_create(N_FEATURES, hidden, N_CANDIDATES, seed, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().heffte_gb300_mlp_destroy(h)

    def num_params(self):
        return lib().heffte_gb300_mlp_num_params(self._h)

    def params(self):
        out = np.empty(self.num_params(), dtype=np.float32)
        check(lib().heffte_gb300_mlp_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().heffte_gb300_mlp_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def loss_grad(self, X, T):
        import torch
        Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        Td = torch.from_numpy(np.ascontiguousarray(T, dtype=np.float32)).cuda()
        loss = ctypes.c_float()
        g = np.empty(self.num_params(), dtype=np.float32)
        check(lib().heffte_gb300_mlp_loss_grad(self._h, Xd.data_ptr(), Td.data_ptr(), len(X), ctypes.byref(loss),
                                               g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return loss.value, g

    def train(self, X, T, steps=3000, lr=3e-3):
        import torch
        Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        Td = torch.from_numpy(np.ascontiguousarray(T, dtype=np.float32)).cuda()
        loss = ctypes.c_float()
        check(lib().heffte_gb300_mlp_train(self._h, Xd.data_ptr(), Td.data_ptr(), len(X), steps, ctypes.c_float(lr),
                                           None, ctypes.byref(loss)))
        return loss.value

    def predict(self, X):
        import torch
        Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        Yd = torch.empty((len(X), N_CANDIDATES), dtype=torch.float32, device="cuda")
        check(lib().heffte_gb300_mlp_predict(self._h, Xd.data_ptr(), Yd.data_ptr(), len(X), None))
        torch.cuda.synchronize()
        return Yd.cpu().numpy()

    def choose(self, X):
        return self.predict(X).argmin(axis=1)

    def select(self, size, tkind, prec):
        c = ctypes.c_int()
        check(lib().heffte_gb300_select(self._h, tkind, prec, (ctypes.c_int * 3)(*size), ctypes.byref(c)))
        return c.value


def regret(T, choice):
    """Mean relative slow-down of the chosen candidates against the exhaustive best."""
    T = filled(T)
    t = T[np.arange(len(T)), choice]
    return float(np.mean(t / T.min(axis=1) - 1.0))


def best_candidate(size, tkind, prec, net=None, reps=3):
    """The candidate plan of one shape: the network's pick, or, without a
    network (the fallback), the fastest of all 16 by exhaustive timing."""
    if net is not None:
        return net.select(tuple(size), tkind, prec)
    _, T = measure([(tuple(size), tkind, prec)], reps=reps)
    return int(np.nanargmin(T[0]))


def plan_for(size, tkind, prec, net=None, stream=None):
    """A plan of the shape built with the chosen candidate's options and knobs."""
    return make_plan(tuple(size), tkind, prec, best_candidate(size, tkind, prec, net), stream)
