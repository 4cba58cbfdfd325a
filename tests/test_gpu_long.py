"""Transform lengths outside the radix kernels: prime factors above 13
(Bluestein's algorithm) and lengths above 8192 (four-step), which the
cufft_executor role accepts (include/heffte_backend_cuda.h:346-422) and the
reference's stock backend computes with Rader's algorithm for large primes
(include/stock_fft/heffte_stock_algos.h:328-).  Every kind (c2c, r2c / c2r,
DCT / DST, DCT-I) and both precisions against the FP64 oracle: rel-L2 <= 1e-6
(float), <= 1e-12 (double).
"""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {0: 1e-6, 1: 1e-12}


def cdt(prec):
    return np.complex64 if prec == 0 else np.complex128


def rdt(prec):
    return np.float32 if prec == 0 else np.float64


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def box_of(size, order=(0, 1, 2)):
    import heffte_gb300 as gb
    return gb.box3d((0, 0, 0), [s - 1 for s in size], order)


@pytest.mark.parametrize("size", [(17, 8, 6), (19, 12, 5), (97, 4, 3), (127, 3, 2), (8, 17, 10), (6, 9, 97),
                                  (17, 23, 29)])
@pytest.mark.parametrize("prec", [0, 1])
def test_c2c_prime_lengths(gb, size, prec, report):
    rng = np.random.default_rng(sum(size) + prec)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(cdt(prec))
    worst = 0.0
    for reorder in (0, 1):
        opts = gb.plan_options.default()
        opts.use_reorder = reorder
        for io, oo in (((0, 1, 2), (0, 1, 2)), ((2, 0, 1), (1, 2, 0))):
            p = gb.fft3d(box_of(size, io), box_of(size, oo), opts)
            assert p.size_workspace() > 0
            xin = dev(O.from_canonical(O.to_canonical(x, size, (0, 1, 2)), io))
            y = torch.empty_like(xin)
            p.forward(xin, y)
            want = O.fft3d_c2c(host(xin), size, io, oo)
            e_f = O.rel_l2(host(y), want)
            z = torch.empty_like(xin)
            p.backward(y, z, gb.scale.full)
            e_b = O.rel_l2(host(z), host(xin))
            worst = max(worst, e_f, e_b)
            assert e_f < TOL[prec] and e_b < TOL[prec], (reorder, io, oo, e_f, e_b)
    report.append(f"c2c {size} prec={prec} (Bluestein): worst rel-L2 {worst:.2e}")
    assert gb.device_status() == 0


@pytest.mark.parametrize("n,dims", [(8191, (8191, 3, 2)), (16384, (16384, 2, 3)), (16384, (3, 16384, 2)),
                                    (10007, (2, 3, 10007)), (24576, (24576, 1, 2))])
@pytest.mark.parametrize("prec", [0, 1])
def test_long_lengths_executor_and_plan(gb, n, dims, prec, report):
    """8191 (prime: Bluestein through a 16384-point four-step), 16384
    (four-step 128 x 128) along the fastest and a strided dimension, 10007
    (prime above 8192: Bluestein through 32768 = 128 x 256), 24576 = 3 x 8192
    (four-step); the 1-D executor along that dimension with a caller
    workspace, and the whole 3-D plan."""
    rng = np.random.default_rng(n + prec)
    size = dims
    total = int(np.prod(size))
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(cdt(prec))
    d = size.index(n)
    ex = gb.executor(gb.kind.c2c, box_of(size), [d])
    w = torch.empty(max(ex.workspace_size(), 1), dtype=torch.complex64 if prec == 0 else torch.complex128,
                    device="cuda")
    assert ex.workspace_size() > 0
    t = dev(x)
    ex.forward(prec, t, t, workspace=w)
    e_x = O.rel_l2(host(t), O.executor_c2c(x, size, (0, 1, 2), d))
    p = gb.fft3d(box_of(size), box_of(size))
    xin = dev(x)
    y = torch.empty_like(xin)
    p.forward(xin, y)
    e_f = O.rel_l2(host(y), O.fft3d_c2c(x, size))
    z = torch.empty_like(xin)
    p.backward(y, z, gb.scale.full)
    e_b = O.rel_l2(host(z), x)
    report.append(f"length {n} {size} prec={prec}: executor {e_x:.2e}, forward {e_f:.2e}, round trip {e_b:.2e}")
    assert e_x < TOL[prec] and e_f < TOL[prec] and e_b < TOL[prec], (e_x, e_f, e_b)
    assert gb.device_status() == 0


@pytest.mark.parametrize("size,r2c_dir", [((34, 6, 5), 0), ((17, 6, 5), 0), ((6, 19, 4), 1), ((8, 6, 38), 2),
                                          ((16384, 2, 2), 0), ((3, 8191, 2), 1)])
@pytest.mark.parametrize("prec", [0, 1])
def test_r2c_composite_lengths(gb, size, r2c_dir, prec):
    rng = np.random.default_rng(sum(size) + 7 * prec)
    n = int(np.prod(size))
    x = rng.standard_normal(n).astype(rdt(prec))
    for reorder in (0, 1):
        opts = gb.plan_options.default()
        opts.use_reorder = reorder
        b = box_of(size)
        p = gb.fft3d_r2c(b, b.r2c(r2c_dir), r2c_dir, opts)
        xin = dev(x)
        y = torch.empty(p.size_outbox(), dtype=torch.complex64 if prec == 0 else torch.complex128, device="cuda")
        p.forward(xin, y)
        yh = host(y)
        e_f = O.rel_l2(yh, O.fft3d_r2c(x, size, r2c_dir))
        z = torch.empty_like(xin)
        y_before = y.clone()
        p.backward(y, z, gb.scale.full)
        assert torch.equal(y, y_before), "c2r modified its input"
        e_b = O.rel_l2(host(z), x)
        assert e_f < TOL[prec] and e_b < TOL[prec], (reorder, e_f, e_b)
    assert gb.device_status() == 0


@pytest.mark.parametrize("rkind", ["cos", "sin", "cos1"])
@pytest.mark.parametrize("prec", [0, 1])
def test_r2r_composite_lengths(gb, rkind, prec):
    """DCT-II/III and DST-II/III of 17 and 19 points (Bluestein on the
    N-point Makhoul transform), DCT-I of 18 points (an FFT of 34 = 2 x 17)."""
    rng = np.random.default_rng(3 + prec)
    size = (18, 6, 5) if rkind == "cos1" else (17, 6, 19)
    n = int(np.prod(size))
    x = rng.standard_normal(n).astype(rdt(prec))
    k = {"cos": O.COS, "sin": O.SIN, "cos1": O.COS1}[rkind]
    p = gb.rtransform(getattr(gb.kind, rkind), box_of(size), box_of(size))
    xin = dev(x)
    y = torch.empty_like(xin)
    p.forward(xin, y)
    e_f = O.rel_l2(host(y), O.rtransform(k, x, size))
    z = torch.empty_like(xin)
    p.backward(y, z, gb.scale.full)
    e_b = O.rel_l2(host(z), x)
    assert e_f < TOL[prec] and e_b < TOL[prec], (e_f, e_b)
    # the 1-D r2r executor along the Bluestein dimension, with its own workspace
    ex = gb.executor(getattr(gb.kind, rkind), box_of(size), [0])
    t = dev(x)
    ex.forward(prec, t, t)
    c = O.to_canonical(x, size, (0, 1, 2))
    c = np.moveaxis(O._r2r_forward_1d(k, np.moveaxis(c, O.axis_of(0), -1)), -1, O.axis_of(0))
    assert O.rel_l2(host(t), O.from_canonical(c, (0, 1, 2))) < TOL[prec]
    assert gb.device_status() == 0
