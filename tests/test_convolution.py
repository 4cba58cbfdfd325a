"""Convolution through the plan's transforms (the step of the reference's
benchmarks/convolution.cpp:89-95: forward, pointwise product, backward).

CPU: the oracle's restatement against a direct circular-convolution sum and
against the reference's own outputs (tests/golden/convolution.npz); the C ABI
validates its arguments.  GPU: plan.convolve (fused route: forward FFT along
one dimension, product, backward FFT along it in one kernel; unfused route:
two forward transforms, a product kernel, a backward transform) against the
golden fixtures and the FP64 oracle, rel-L2 <= 1e-6 (float) / 1e-12 (double).
"""
import numpy as np
import pytest

from oracle import heffte_oracle as O

TOL = {0: 1e-6, 1: 1e-12}
# the reference's float transforms (stock<float>, twiddles by recurrence)
# carry more rounding than this library's; their convolution results are
# compared with this bar
REF_FLOAT_TOL = 5e-6


def direct_circular(x, y, size):
    X = O.to_canonical(x, size, (0, 1, 2))
    Y = O.to_canonical(y, size, (0, 1, 2))
    D = np.zeros(X.shape, dtype=np.complex128)
    for k in range(X.shape[0]):
        for j in range(X.shape[1]):
            for i in range(X.shape[2]):
                D += X[k, j, i] * np.roll(Y, (k, j, i), axis=(0, 1, 2))
    return O.from_canonical(D, (0, 1, 2))


def test_oracle_convolution_is_the_circular_sum():
    rng = np.random.default_rng(1)
    size = (6, 5, 4)
    n = int(np.prod(size))
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert O.rel_l2(O.convolve(x, y, size), direct_circular(x, y, size)) < 1e-13
    # real inputs through the r2c form (product on the half spectrum)
    xr, yr = rng.standard_normal(n), rng.standard_normal(n)
    for d in range(3):
        assert O.rel_l2(O.convolve(xr, yr, size, r2c_dir=d), direct_circular(xr, yr, size).real) < 1e-13
    # the benchmark step is the self-convolution over N (forward scale::full, X .* X, backward unscaled)
    assert O.rel_l2(O.convolution_benchmark_step(x, size), O.convolve(x, None, size) / n) < 1e-13


def test_oracle_convolution_against_reference(golden):
    g = golden["convolution"]
    for tag in ("f", "d", "d2"):
        size = tuple(int(s) for s in g[tag + "_size"])
        x, y = g[tag + "_x"], g[tag + "_y"]
        tol = 1e-12 if x.dtype == np.complex128 else REF_FLOAT_TOL
        assert O.rel_l2(O.convolution_benchmark_step(x, size), g[tag + "_step"]) < tol, tag
        assert O.rel_l2(O.convolve(x, y, size), g[tag + "_conv"]) < tol, tag
    # real data through fft3d_r2c
    for tag in ("rf", "rd", "rd2", "rf3", "rd3"):
        size = tuple(int(s) for s in g[tag + "_size"])
        x, y = g[tag + "_x"], g[tag + "_y"]
        tol = 1e-12 if x.dtype == np.float64 else REF_FLOAT_TOL
        assert O.rel_l2(O.convolve(x, y, size, r2c_dir=int(g[tag + "_dir"])), g[tag + "_conv"]) < tol, tag


def test_convolve_abi_validates(gb):
    import ctypes
    L = gb.lib()
    p = gb.fft3d(gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 7)))
    assert p.convolve_workspace() >= 2 * 512 + p.size_workspace()
    assert L.heffte_gb300_convolve(p._h, 0, None, None, None, None, 1) == 1          # null arrays
    assert L.heffte_gb300_convolve(p._h, 2, 16, None, 16, None, 1) == 1              # precision
    assert L.heffte_gb300_convolve(p._h, 0, 16, None, 16, None, 3) == 1              # scaling
    assert L.heffte_gb300_convolve(None, 0, 16, None, 16, None, 1) == 1              # plan
    c = gb.rtransform(gb.kind.cos, gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 7)))
    assert L.heffte_gb300_convolve(c._h, 0, 16, None, 16, None, 1) == 3              # no r2r convolution
    assert b"c2c or r2c" in L.heffte_gb300_last_error()
    d = ctypes.c_int(0)
    assert L.heffte_gb300_convolve_route(None, 0, 0, ctypes.byref(d)) == 1


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _rand_c(rng, n, prec):
    dt = np.complex64 if prec == 0 else np.complex128
    return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)


def _c2c_plan(gb, size, order=(0, 1, 2)):
    b = gb.box3d((0, 0, 0), [s - 1 for s in size], order)
    return gb.fft3d(b, b)


@pytest.mark.gpu
def test_gpu_convolution_against_reference(gb, golden):
    import torch
    g = golden["convolution"]
    for tag in ("f", "d", "d2"):
        size = tuple(int(s) for s in g[tag + "_size"])
        x, y = g[tag + "_x"], g[tag + "_y"]
        prec = 0 if x.dtype == np.complex64 else 1
        n = int(np.prod(size))
        p = _c2c_plan(gb, size)
        xd, yd = _dev(x), _dev(y)
        out = torch.empty_like(xd)
        p.convolve(xd, yd, out, gb.scale.full)
        conv = _host(out)
        # the benchmark's in-place self-convolution: out = x .* x over N, in place
        z = xd.clone()
        p.convolve(z, None, z, gb.scale.full)
        step = _host(z) / n
        oracle_conv = O.convolve(x, y, size)
        oracle_step = O.convolution_benchmark_step(x, size)
        assert O.rel_l2(conv, oracle_conv) < TOL[prec], tag
        assert O.rel_l2(step, oracle_step) < TOL[prec], tag
        ref_tol = 1e-12 if prec == 1 else REF_FLOAT_TOL
        assert O.rel_l2(conv, g[tag + "_conv"]) < ref_tol, tag
        assert O.rel_l2(step, g[tag + "_step"]) < ref_tol, tag


@pytest.mark.gpu
def test_gpu_r2c_convolution_against_reference(gb, golden):
    """Both routes of an r2c plan against the reference's own r2c convolution
    (the 16x16x16 cases take the fused route when it is allowed)."""
    import torch
    g = golden["convolution"]
    for tag in ("rf", "rd", "rd2", "rf3", "rd3"):
        size = tuple(int(s) for s in g[tag + "_size"])
        rd = int(g[tag + "_dir"])
        x, y = g[tag + "_x"], g[tag + "_y"]
        prec = 0 if x.dtype == np.float32 else 1
        ib = gb.box3d((0, 0, 0), [s - 1 for s in size])
        for fused in (True, False):
            p = gb.fft3d_r2c(ib, ib.r2c(rd), rd)
            p.set_convolution_fusion(fused)
            if tag.endswith("3"):
                assert p.convolve_route(prec, True) == (2 if fused else -1)
            xd, yd = _dev(x), _dev(y)
            out = torch.empty_like(xd)
            p.convolve(xd, yd, out, gb.scale.full)
            got = _host(out)
            assert O.rel_l2(got, O.convolve(x, y, size, r2c_dir=rd)) < TOL[prec], (tag, fused)
            assert O.rel_l2(got, g[tag + "_conv"]) < (1e-12 if prec == 1 else REF_FLOAT_TOL), (tag, fused)


# (size, order, fused dimension expected for aligned arrays)
FUSED_CASES = [
    ((32, 16, 64), (0, 1, 2), 2),
    ((64, 64, 512), (0, 1, 2), 2),
    # 4096-point columns of two operands do not fit shared memory double
    # buffered in 16-byte aligned tiles: the 32-point middle dimension is fused
    ((16, 32, 4096), (0, 1, 2), {(0, False): 2, (0, True): 1, (1, False): 2, (1, True): 1}),
    ((32, 64, 12), (0, 1, 2), 1),       # 12 has no pipelined kernel: the middle dimension is fused
    ((64, 16, 32), (2, 0, 1), 1),       # order (2, 0, 1): the slowest dimension is 1
    ((24, 20, 12), (0, 1, 2), -1),      # no power-of-two column dimension: unfused
]


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("case", FUSED_CASES, ids=lambda c: "x".join(map(str, c[0])) + "_o" + "".join(map(str, c[1])))
@pytest.mark.parametrize("two", [False, True], ids=["self", "xy"])
def test_gpu_convolution_routes(gb, prec, case, two):
    import torch
    size, order, fused = case
    if isinstance(fused, dict):
        fused = fused[(prec, two)]
    rng = np.random.default_rng(7)
    n = int(np.prod(size))
    x = _rand_c(rng, n, prec)
    y = _rand_c(rng, n, prec) if two else None
    p = _c2c_plan(gb, size, order)
    assert p.convolve_route(prec, two) == fused
    xd = _dev(x)
    yd = _dev(y) if two else None
    out = torch.empty_like(xd)
    p.convolve(xd, yd, out, gb.scale.full)
    got = _host(out)
    # oracle in the box's own order
    want = O.convolve(x, y, size, order=order)
    assert O.rel_l2(got, want) < TOL[prec]
    assert np.array_equal(_host(xd), x), "input modified"
    assert gb.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_convolution_aliasing_and_scaling(gb, prec):
    import torch
    size = (32, 32, 64)
    n = int(np.prod(size))
    rng = np.random.default_rng(11)
    x, y = _rand_c(rng, n, prec), _rand_c(rng, n, prec)
    p = _c2c_plan(gb, size)
    want = O.convolve(x, y, size, scaling=O.SCALE_NONE)
    for scaling, f in ((gb.scale.none, 1.0), (gb.scale.full, 1.0 / n), (gb.scale.symmetric, n ** -0.5)):
        # in place on x
        xd, yd = _dev(x), _dev(y)
        p.convolve(xd, yd, xd, scaling)
        assert O.rel_l2(_host(xd), want * f) < TOL[prec]
        # in place on y
        xd, yd = _dev(x), _dev(y)
        p.convolve(xd, yd, yd, scaling)
        assert O.rel_l2(_host(yd), want * f) < TOL[prec]
    # a caller-owned workspace
    xd, yd = _dev(x), _dev(y)
    w = torch.empty(p.convolve_workspace(), dtype=xd.dtype, device="cuda")
    out = torch.empty_like(xd)
    p.convolve(xd, yd, out, gb.scale.full, workspace=w)
    assert O.rel_l2(_host(out), want / n) < TOL[prec]


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_convolution_reorder_and_orders(gb, prec):
    """use_reorder plans and plans whose input and output orders differ take
    the unfused route; the result is in the input box's order."""
    import torch
    size = (32, 16, 64)
    n = int(np.prod(size))
    rng = np.random.default_rng(29)
    x, y = _rand_c(rng, n, prec), _rand_c(rng, n, prec)
    cases = [((0, 1, 2), (0, 1, 2), True), ((1, 2, 0), (1, 2, 0), True), ((0, 1, 2), (2, 1, 0), False)]
    for io, oo, reorder in cases:
        opts = gb.plan_options.default()
        opts.use_reorder = reorder
        p = gb.fft3d(gb.box3d((0, 0, 0), [s - 1 for s in size], io), gb.box3d((0, 0, 0), [s - 1 for s in size], oo),
                     opts)
        assert p.convolve_route(prec, True) == -1
        xd, yd = _dev(x), _dev(y)
        out = torch.empty_like(xd)
        p.convolve(xd, yd, out, gb.scale.full)
        assert O.rel_l2(_host(out), O.convolve(x, y, size, order=io)) < TOL[prec], (io, oo, reorder)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("r2c_dir", [0, 1, 2])
def test_gpu_convolution_r2c(gb, prec, r2c_dir):
    import torch
    size = (64, 24, 32)
    n = int(np.prod(size))
    rng = np.random.default_rng(13 + r2c_dir)
    dt = np.float32 if prec == 0 else np.float64
    x, y = rng.standard_normal(n).astype(dt), rng.standard_normal(n).astype(dt)
    ib = gb.box3d((0, 0, 0), [s - 1 for s in size])
    want_xy = O.convolve(x, y, size, r2c_dir=r2c_dir)
    want_xx = O.convolve(x, None, size, r2c_dir=r2c_dir)
    for fused in (True, False):
        p = gb.fft3d_r2c(ib, ib.r2c(r2c_dir), r2c_dir)
        p.set_convolution_fusion(fused)
        # the fused route takes r2c along the fastest dimension; the
        # 32-point slowest dimension is the fused one
        route = 2 if (fused and r2c_dir == 0) else -1
        assert p.convolve_route(prec, True) == route and p.convolve_route(prec, False) == route
        xd, yd = _dev(x), _dev(y)
        out = torch.empty_like(xd)
        p.convolve(xd, yd, out, gb.scale.full)
        assert O.rel_l2(_host(out), want_xy) < TOL[prec]
        p.convolve(xd, None, out, gb.scale.full)
        assert O.rel_l2(_host(out), want_xx) < TOL[prec]
        # in place on x
        p.convolve(xd, None, xd, gb.scale.full)
        assert O.rel_l2(_host(xd), want_xx) < TOL[prec]
        assert gb.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("size", [(512, 64, 32), (256, 16, 128), (96, 64, 64)], ids=lambda s: "x".join(map(str, s)))
def test_gpu_convolution_r2c_fused_sizes(gb, prec, size):
    """The fused r2c route on half spectra of padded width (257, 129) and an
    even one (49): r2c along x, a c2c pass, the fused pass, c2r."""
    import torch
    n = int(np.prod(size))
    rng = np.random.default_rng(23)
    dt = np.float32 if prec == 0 else np.float64
    x, y = rng.standard_normal(n).astype(dt), rng.standard_normal(n).astype(dt)
    ib = gb.box3d((0, 0, 0), [s - 1 for s in size])
    p = gb.fft3d_r2c(ib, ib.r2c(0), 0)
    assert p.convolve_route(prec, True) == 2
    xd, yd = _dev(x), _dev(y)
    out = torch.empty_like(xd)
    p.convolve(xd, yd, out, gb.scale.full)
    assert O.rel_l2(_host(out), O.convolve(x, y, size, r2c_dir=0)) < TOL[prec]
    p.convolve(xd, None, out, gb.scale.full)
    assert O.rel_l2(_host(out), O.convolve(x, None, size, r2c_dir=0)) < TOL[prec]


@pytest.mark.gpu
def test_gpu_convolution_knobs_take_the_unfused_route(gb):
    import torch
    size = (64, 32, 128)
    n = int(np.prod(size))
    rng = np.random.default_rng(17)
    x, y = _rand_c(rng, n, 0), _rand_c(rng, n, 0)
    want = O.convolve(x, y, size)
    for setter in (lambda p: p.set_tensor_cores(True), lambda p: p.set_knobs(variant=1),
                   lambda p: p.set_convolution_fusion(False)):
        p = _c2c_plan(gb, size)
        setter(p)
        assert p.convolve_route(0, True) == -1
        xd, yd = _dev(x), _dev(y)
        out = torch.empty_like(xd)
        p.convolve(xd, yd, out, gb.scale.full)
        assert O.rel_l2(_host(out), want) < 1e-6
