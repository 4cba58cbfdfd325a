"""User streams, impulse responses and 64-bit indexing on the GPU — the
reference's test_streams.cpp, the impulse case of test_units_stock.cpp and
test_longlong.cpp, restated for this backend."""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _box(size):
    import heffte_gb300 as gb
    return gb.box3d((0, 0, 0), [s - 1 for s in size])


def test_plans_run_on_the_user_stream(gb):
    """Work queued on the plan's stream after a long producer on the same
    stream sees the producer's data (no implicit default-stream sync)."""
    size = (64, 48, 40)
    n = int(np.prod(size))
    s = torch.cuda.Stream()
    rng = np.random.default_rng(3)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    p = gb.fft3d(_box(size), _box(size), stream=s)
    with torch.cuda.stream(s):
        src = torch.from_numpy(x).to("cuda", non_blocking=False)
        xin = torch.empty_like(src)
        big = torch.empty(1 << 26, device="cuda")
        for _ in range(20):
            big.mul_(1.0001)          # keeps the stream busy before the copy
        xin.copy_(src)
        y = torch.empty_like(xin)
        p.forward(xin, y)
        z = torch.empty_like(xin)
        p.backward(y, z, gb.scale.full)
    s.synchronize()
    assert O.rel_l2(y.cpu().numpy(), O.fft3d_c2c(x, size)) <= 1e-6
    assert O.rel_l2(z.cpu().numpy(), x) <= 1e-6
    # set_stream moves the plan to another stream
    s2 = torch.cuda.Stream()
    p.set_stream(s2)
    with torch.cuda.stream(s2):
        y2 = torch.empty_like(xin)
        p.forward(xin, y2)
    s2.synchronize()
    assert torch.equal(y2, y)


@pytest.mark.parametrize("prec", [0, 1])
def test_impulse_gives_all_ones(gb, prec):
    size = (30, 32, 27)
    n = int(np.prod(size))
    cdt = torch.complex64 if prec == 0 else torch.complex128
    rdt = torch.float32 if prec == 0 else torch.float64
    tol = 1e-6 if prec == 0 else 1e-14
    x = torch.zeros(n, dtype=cdt, device="cuda")
    x[0] = 1
    y = torch.empty_like(x)
    gb.fft3d(_box(size), _box(size)).forward(x, y)
    assert float((y - 1).abs().max()) <= tol
    xr = torch.zeros(n, dtype=rdt, device="cuda")
    xr[0] = 1
    box = _box(size)
    p = gb.fft3d_r2c(box, box.r2c(0), 0)
    yr = torch.empty(p.size_outbox(), dtype=cdt, device="cuda")
    p.forward(xr, yr)
    assert float((yr - 1).abs().max()) <= tol


def test_64bit_indexing(gb):
    """A complex<float> box of more than 2^31 elements: an impulse beyond
    element 2^31 has the analytic spectrum at sampled frequencies (also
    beyond 2^31), and the round trip returns it."""
    size = (1024, 1024, 2100)
    n = int(np.prod(size))
    assert n > 2 ** 31
    free, _ = torch.cuda.mem_get_info()
    if free < 48 * 2 ** 30:
        pytest.skip("needs 48 GiB of free device memory")
    p0 = (5, 777, 2099)                              # linear index > 2^31
    lin = p0[0] + size[0] * (p0[1] + size[1] * p0[2])
    assert lin > 2 ** 31
    x = torch.zeros(n, dtype=torch.complex64, device="cuda")
    x[lin] = 1
    y = torch.empty_like(x)
    p = gb.fft3d(_box(size), _box(size))
    p.forward(x, y)
    rng = np.random.default_rng(64)
    ks = [(0, 0, 0), (1023, 1023, 2099), (3, 900, 1500)] + \
         [tuple(int(rng.integers(0, s)) for s in size) for _ in range(29)]
    idx = torch.tensor([k[0] + size[0] * (k[1] + size[1] * k[2]) for k in ks], device="cuda")
    got = y[idx].cpu().numpy()
    want = np.array([np.exp(-2j * np.pi * sum(k[d] * p0[d] / size[d] for d in range(3))) for k in ks])
    assert np.max(np.abs(got - want)) <= 2e-5
    assert any(int(i) > 2 ** 31 for i in idx)
    # round trip in place (backward with scale::full) gives the impulse back
    p.backward(y, y, gb.scale.full)
    torch.cuda.synchronize()
    assert abs(complex(y[lin].item()) - 1) <= 1e-5
    y[lin] = 0
    assert float(y.abs().max()) <= 1e-5
