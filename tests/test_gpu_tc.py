"""GPU parity of the tensor-core form (split-BF16 tcgen05 radix-16 stages) of
the complex<float> transforms against the FP64 oracle: rel-L2 <= 1e-6, the
same bar as the plain FP32 kernels, for every layout the plans produce."""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _c2c(gb, x, size, io, oo, direction, scaling, tc, reorder=0):
    opts = gb.plan_options.default()
    opts.use_reorder = reorder
    ib = gb.box3d((0, 0, 0), [s - 1 for s in size], io)
    ob = gb.box3d((0, 0, 0), [s - 1 for s in size], oo)
    p = gb.fft3d(ib, ob, opts)
    if tc:
        p.set_tensor_cores(True)
    xin = _dev(x)
    y = torch.empty_like(xin)
    (p.forward if direction == 0 else p.backward)(xin, y, scaling)
    return _host(y)


def _status_ok(gb):
    assert gb.device_status(reset=True) == 0


@pytest.mark.parametrize("size,io,oo,reorder", [
    ((64, 128, 256), (0, 1, 2), (0, 1, 2), 0),
    ((256, 64, 128), (0, 1, 2), (2, 1, 0), 0),
    ((512, 64, 64), (1, 0, 2), (0, 1, 2), 1),
    ((1024, 32, 64), (0, 1, 2), (0, 1, 2), 0),
    ((64, 2048, 16), (0, 1, 2), (0, 1, 2), 0),
    ((4096, 8, 16), (0, 1, 2), (0, 1, 2), 1),
    ((128, 96, 80), (0, 1, 2), (0, 1, 2), 0),      # 96 and 80 keep the FP32 kernels
])
@pytest.mark.parametrize("direction", [0, 1])
def test_tc_c2c_matches_oracle(gb, size, io, oo, reorder, direction):
    rng = np.random.default_rng(sum(size) + direction)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    out = _c2c(gb, x, size, io, oo, direction, gb.scale.none, tc=True, reorder=reorder)
    # backward reads the outbox order and writes the inbox order
    src, dst = (io, oo) if direction == 0 else (oo, io)
    ref = O.fft3d_c2c(x, size, src, dst, direction, O.SCALE_NONE)
    err = O.rel_l2(out, ref)
    print(f"tensor-core c2c {size} dir {direction}: rel-L2 {err:.2e}")
    assert err <= 1e-6
    _status_ok(gb)


@pytest.mark.parametrize("scaling", [1, 2])
def test_tc_round_trip_with_scaling(gb, scaling):
    size = (256, 128, 64)
    rng = np.random.default_rng(5)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    y = _c2c(gb, x, size, (0, 1, 2), (0, 1, 2), 0, scaling, tc=True)
    ref = O.fft3d_c2c(x, size, (0, 1, 2), (0, 1, 2), 0, scaling)
    assert O.rel_l2(y, ref) <= 1e-6
    # full: scaled forward, unscaled backward; symmetric: both scaled
    z = _c2c(gb, y, size, (0, 1, 2), (0, 1, 2), 1, 0 if scaling == 1 else 2, tc=True)
    assert O.rel_l2(z, x) <= 1e-6
    _status_ok(gb)


def test_tc_in_place(gb):
    size = (512, 16, 32)
    rng = np.random.default_rng(7)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    p = gb.fft3d(box, box)
    p.set_tensor_cores(True)
    buf = _dev(x)
    p.forward(buf, buf)
    assert O.rel_l2(_host(buf), O.fft3d_c2c(x, size)) <= 1e-6
    _status_ok(gb)


def test_tc_and_fp32_forms_agree(gb):
    """Both forms of the same plan are within 1e-6 of the oracle and of each other."""
    size = (1024, 64, 32)
    rng = np.random.default_rng(9)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    ref = O.fft3d_c2c(x, size)
    a = _c2c(gb, x, size, (0, 1, 2), (0, 1, 2), 0, gb.scale.none, tc=False)
    b = _c2c(gb, x, size, (0, 1, 2), (0, 1, 2), 0, gb.scale.none, tc=True)
    ea, eb = O.rel_l2(a, ref), O.rel_l2(b, ref)
    print(f"rel-L2 vs FP64: plain FP32 {ea:.2e}, split-BF16 tensor cores {eb:.2e}")
    assert ea <= 1e-6 and eb <= 1e-6
    assert O.rel_l2(b, a) <= 2e-6


def test_tc_double_plans_are_unaffected(gb):
    size = (64, 64, 64)
    rng = np.random.default_rng(11)
    n = int(np.prod(size))
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    p = gb.fft3d(box, box)
    p.set_tensor_cores(True)
    xin = _dev(x)
    y = torch.empty_like(xin)
    p.forward(xin, y)
    assert O.rel_l2(_host(y), O.fft3d_c2c(x, size)) <= 1e-12
