"""complex<double> power-of-two c2c passes in double-float arithmetic (pairs of
floats on the FP32 pipe, each tile scaled by a power of two into the float
exponent range): against the FP64 oracle at rel-L2 <= 1e-12, over line and
column passes, orders, reorder on / off, and inputs far outside the float
exponent range (the per-tile scaling), and against the FP64-instruction path.
"""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture
def double_float(gb):
    old = gb.set_double_arithmetic(gb.DOUBLE_FLOAT)
    yield gb
    gb.set_double_arithmetic(old)


def _run(gb, x, size, io=(0, 1, 2), oo=(0, 1, 2), reorder=0):
    opts = gb.plan_options.default()
    opts.use_reorder = reorder
    p = gb.fft3d(gb.box3d((0, 0, 0), [s - 1 for s in size], io), gb.box3d((0, 0, 0), [s - 1 for s in size], oo), opts)
    xin = torch.from_numpy(x).cuda()
    y = torch.empty_like(xin)
    p.forward(xin, y)
    z = torch.empty_like(xin)
    p.backward(y, z, gb.scale.full)
    torch.cuda.synchronize()
    return y.cpu().numpy(), z.cpu().numpy()


@pytest.mark.parametrize("size", [(16, 32, 64), (64, 16, 128), (128, 256, 32), (2048, 16, 8), (512, 8, 1024),
                                  (4096, 4, 2), (2, 4, 8), (8, 1024, 4), (32, 512, 6)])
def test_double_float_against_fp64(double_float, size):
    gb = double_float
    rng = np.random.default_rng(sum(size))
    n = int(np.prod(size))
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    for io, oo, reorder in (((0, 1, 2), (0, 1, 2), 0), ((2, 0, 1), (1, 2, 0), 0), ((0, 1, 2), (2, 1, 0), 1)):
        xi = O.from_canonical(O.to_canonical(x, size, (0, 1, 2)), io)
        y, z = _run(gb, xi, size, io, oo, reorder)
        e_f = O.rel_l2(y, O.fft3d_c2c(xi, size, io, oo))
        e_b = O.rel_l2(z, xi)
        assert e_f < TOL and e_b < TOL, (io, oo, reorder, e_f, e_b)
    assert gb.device_status() == 0


@pytest.mark.parametrize("mag", [1e-300, 1e-40, 1e40, 1e290])
def test_double_float_exponent_range(double_float, mag):
    """Inputs whose magnitudes the float exponent range cannot hold directly
    (each tile is scaled by a power of two), and a box mixing magnitudes 2^40
    apart across tiles."""
    gb = double_float
    size = (64, 32, 32)
    n = int(np.prod(size))
    rng = np.random.default_rng(5)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)) * mag
    y, z = _run(gb, x, size)
    assert np.all(np.isfinite(y)) and np.all(np.isfinite(z))
    assert O.rel_l2(y, O.fft3d_c2c(x, size)) < TOL
    assert O.rel_l2(z, x) < TOL
    # planes 2^40 apart: every tile of the passes carries its own scale
    w = x / mag * np.repeat(2.0 ** (40 * (np.arange(size[2]) % 2)), size[0] * size[1])
    y, z = _run(gb, w, size)
    assert O.rel_l2(y, O.fft3d_c2c(w, size)) < TOL and O.rel_l2(z, w) < TOL


def test_double_float_matches_fp64_instructions(gb):
    """The same transform in both arithmetic forms: the two results agree to
    the accuracy of the double-float one."""
    size = (256, 128, 64)
    n = int(np.prod(size))
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    old = gb.set_double_arithmetic(gb.FP64)
    try:
        y64, _ = _run(gb, x, size)
        gb.set_double_arithmetic(gb.DOUBLE_FLOAT)
        ydf, _ = _run(gb, x, size)
    finally:
        gb.set_double_arithmetic(old)
    ref = O.fft3d_c2c(x, size)
    assert O.rel_l2(y64, ref) < TOL and O.rel_l2(ydf, ref) < TOL
    assert O.rel_l2(ydf, y64) < TOL


def test_double_float_partial_last_tile(double_float):
    """Line tiles whose last tile is partial: its lines alone are copied into
    the tile buffer, and the rows past them still hold an earlier tile's values
    (here 2^300 larger), which must not set the last tile's scale.  The 1-D
    executor along dimension 0 of 64 x 255 x 129 (32895 lines: several tiles
    per CTA, a partial last one), the first 16384 lines (whole tiles of any
    power-of-two width) 2^300 larger; every other line against the FP64
    oracle, each on its own scale.  And a single line (a one-line tile), as Bluestein's chirp
    spectrum is computed."""
    gb = double_float
    size = (64, 255, 129)
    lines = size[1] * size[2]
    rng = np.random.default_rng(77)
    x = rng.uniform(-1, 1, (lines, size[0])) + 1j * rng.uniform(-1, 1, (lines, size[0]))
    x[:16384] *= 2.0 ** 300
    ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), [s - 1 for s in size]), [0])
    xin = torch.from_numpy(x.reshape(-1)).cuda()
    y = torch.empty_like(xin)
    ex.forward(1, xin, y)
    torch.cuda.synchronize()
    got = y.cpu().numpy().reshape(lines, size[0])[16384:]
    want = np.fft.fft(x[16384:], axis=1)
    err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert err.max() < TOL, (int(err.argmax()), err.max())
    one = rng.uniform(-1, 1, 64) + 1j * rng.uniform(-1, 1, 64)
    e1 = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), (63, 0, 0)), [0])
    xin = torch.from_numpy(one).cuda()
    y = torch.empty_like(xin)
    e1.forward(1, xin, y)
    torch.cuda.synchronize()
    assert O.rel_l2(y.cpu().numpy(), np.fft.fft(one)) < TOL
    assert gb.device_status() == 0
