"""GPU parity of the CUDA path (through the C ABI) against the oracle.

Bars: bit-exact for pack / unpack / transpose; rel-L2 <= 1e-6 (float) and
<= 1e-12 (double) against the FP64 oracle for every transform; the reference's
own float outputs (golden fixtures, stock<float>) within 5e-6 rel-L2.
"""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {0: 1e-6, 1: 1e-12}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def cdt(prec):
    return np.complex64 if prec == 0 else np.complex128


def rdt(prec):
    return np.float32 if prec == 0 else np.float64


def rand_c(rng, n, prec):
    return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(cdt(prec))


def run_c2c(gb, x, size, io, oo, direction, scaling, prec, reorder=0, workspace=False):
    opts = gb.plan_options.default()
    opts.use_reorder = reorder
    ib = gb.box3d((0, 0, 0), [s - 1 for s in size], io)
    ob = gb.box3d((0, 0, 0), [s - 1 for s in size], oo)
    p = gb.fft3d(ib, ob, opts)
    xin = dev(x)
    y = torch.empty_like(xin)
    if workspace:
        w = torch.empty(max(p.size_workspace(), 1), dtype=xin.dtype, device="cuda")
        (p.forward_buffered if direction == 0 else p.backward_buffered)(xin, y, w, scaling)
    else:
        (p.forward if direction == 0 else p.backward)(xin, y, scaling)
    out = host(y)
    assert np.array_equal(host(xin), x), "input modified"
    return out


# ---------------------------------------------------------------------------
# location layer
# ---------------------------------------------------------------------------
def test_packers_bit_exact(gb, golden):
    g = golden["packers"]
    dtype_of = {4: 0, 8: 2, 16: 3}   # float, complex<float>, complex<double> words
    for m in g["meta"]:
        idx = int(m["idx"])
        es = int(m["esize"])
        src, dst, want = g[f"t{idx}_src"], g[f"t{idx}_dst"], g[f"t{idx}_out"]
        s, d = dev(src), dev(dst)
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        dt = dtype_of[es]
        if m["op"] == "pack":
            gb.direct_pack(dt, *size, int(m["ls"]), int(m["ps"]), s, d)
        elif m["op"] == "unpack":
            gb.direct_unpack(dt, *size, int(m["ls"]), int(m["ps"]), s, d)
        else:
            gb.transpose_unpack(dt, *size, int(m["ls"]), int(m["ps"]), int(m["bls"]), int(m["bps"]),
                                (int(m["m0"]), int(m["m1"]), int(m["m2"])), s, d)
        assert host(d).tobytes() == want.tobytes(), (str(m["op"]), idx, es)


@pytest.mark.parametrize("mp", [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)])
@pytest.mark.parametrize("dtype,np_t", [(0, np.float32), (2, np.complex64), (3, np.complex128)])
def test_transpose_large_tiles_bit_exact(gb, mp, dtype, np_t):
    """Transposes larger than one 32x32 tile, ragged edges, all six maps."""
    rng = np.random.default_rng(5)
    size = (67, 45, 33)
    src_dims = [size[mp[a]] for a in range(3)]
    bls, bps = src_dims[0], src_dims[0] * src_dims[1]
    ls, ps = size[0] + 3, (size[0] + 3) * (size[1] + 2)
    nsrc = int(np.prod(src_dims))
    src = rng.standard_normal(nsrc * (2 if np.iscomplexobj(np.zeros(1, np_t)) else 1)).astype(
        np.float32 if np_t in (np.float32, np.complex64) else np.float64).view(np_t)
    dst = np.zeros(ps * size[2], np_t)
    want = O.transpose_unpack(src, dst, size, ls, ps, bls, bps, mp)
    s, d = dev(src), dev(dst)
    gb.transpose_unpack(dtype, *size, ls, ps, bls, bps, mp, s, d)
    assert host(d).tobytes() == want.tobytes()


def test_direct_pack_unpack_roundtrip_bit_exact(gb):
    rng = np.random.default_rng(9)
    box = rng.standard_normal(40 * 30 * 20).astype(np.float64).view(np.complex128)  # 40*30*10 complex
    size, ls, ps = (17, 13, 7), 40, 40 * 30
    packed = O.direct_pack(box, size, ls, ps)
    s = dev(box)
    buf = torch.empty(int(np.prod(size)), dtype=torch.complex128, device="cuda")
    gb.direct_pack(3, *size, ls, ps, s, buf)
    assert host(buf).tobytes() == packed.tobytes()
    back = torch.zeros_like(s)
    gb.direct_unpack(3, *size, ls, ps, buf, back)
    assert host(back).tobytes() == O.direct_unpack(packed, np.zeros_like(box), size, ls, ps).tobytes()


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n", [1, 7, 1000, 1 << 20])
def test_scale_and_convert(gb, prec, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n).astype(rdt(prec))
    t = dev(x)
    gb.scale_data(prec, n, t, 0.125)
    assert np.array_equal(host(t), O.scale_data(x, 0.125, rdt(prec)))
    c = torch.empty(2 * n, dtype=t.dtype, device="cuda")
    gb.convert(prec, n, dev(x), c, True)
    hc = host(c)
    assert np.array_equal(hc[0::2], x) and not hc[1::2].any()
    r = torch.empty(n, dtype=t.dtype, device="cuda")
    gb.convert(prec, n, c, r, False)
    assert np.array_equal(host(r), x)


# ---------------------------------------------------------------------------
# executors (the cufft_executor role)
# ---------------------------------------------------------------------------
def test_executor_known_answers(gb, golden):
    ka = golden["known_answers"]
    x = ka["input"].astype(np.complex128)
    for d in range(3):
        ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), (1, 2, 3)), [d])
        t = dev(x)
        ex.forward(1, t, t)
        assert np.allclose(host(t), ka[f"exec_dim{d}"], atol=1e-12)
        ex.backward(1, t, t)
        assert np.allclose(host(t), x * (2, 3, 4)[d], atol=1e-12)
    for d in range(3):
        ex = gb.executor(gb.kind.r2c, gb.box3d((0, 0, 0), (1, 2, 3)), [d])
        r = dev(ka["input"])
        c = torch.empty(ex.complex_size(), dtype=torch.complex128, device="cuda")
        ex.forward(1, r, c)
        want = O.from_canonical(np.take(np.fft.fft(O.to_canonical(ka["input"], (2, 3, 4), (0, 1, 2)), axis=2 - d),
                                        np.arange((2, 3, 4)[d] // 2 + 1), axis=2 - d), (0, 1, 2))
        assert np.allclose(host(c), want, atol=1e-12)


@pytest.mark.parametrize("order", [(0, 1, 2), (2, 0, 1), (1, 2, 0)])
@pytest.mark.parametrize("prec", [0, 1])
def test_executor_each_dimension(gb, order, prec):
    rng = np.random.default_rng(3)
    size = (48, 20, 36)
    n = int(np.prod(size))
    x = rand_c(rng, n, prec)
    for d in range(3):
        ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), [s - 1 for s in size], order), [d])
        t = dev(x)
        ex.forward(prec, t, t)
        assert O.rel_l2(host(t), O.executor_c2c(x, size, order, d)) < TOL[prec]
    ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), [s - 1 for s in size], order), [0, 1, 2])
    t = dev(x)
    ex.forward(prec, t, t)
    assert O.rel_l2(host(t), O.fft3d_c2c(x, size, order, order)) < TOL[prec]


@pytest.mark.parametrize("order", [(0, 1, 2), (2, 0, 1), (1, 2, 0)])
@pytest.mark.parametrize("prec", [0, 1])
def test_executor_two_dimensions(gb, order, prec):
    """The 2-D executor (the cufft_executor (d1, d2) constructor,
    include/heffte_backend_cuda.h:459-481) on every pair of dimensions,
    including (0, 2), the pair that needs the reference's embedded layout, and
    the pair given in reverse order; forward and backward against the oracle
    (two 1-D executor stages), in place and out of place."""
    rng = np.random.default_rng(11)
    size = (40, 24, 18)
    n = int(np.prod(size))
    box = gb.box3d((0, 0, 0), [s - 1 for s in size], order)
    x = rand_c(rng, n, prec)
    for dims in ([0, 1], [1, 2], [0, 2], [2, 0]):
        ex = gb.executor(gb.kind.c2c, box, dims)
        want = O.executor_c2c(O.executor_c2c(x, size, order, dims[0]), size, order, dims[1])
        t = dev(x)
        ex.forward(prec, t, t)
        assert O.rel_l2(host(t), want) < TOL[prec], (dims, "forward")
        o = torch.empty_like(t)
        ex.backward(prec, t, o)
        back = O.executor_c2c(O.executor_c2c(want, size, order, dims[0], 1), size, order, dims[1], 1)
        assert O.rel_l2(host(o), back) < TOL[prec], (dims, "backward")
        assert O.rel_l2(host(o), x * size[dims[0]] * size[dims[1]]) < 3 * TOL[prec], (dims, "round trip")
    # a 2-D real-to-real executor (DCT-II along dimensions 0 and 2)
    xr = rng.standard_normal(n).astype(rdt(prec))
    ex = gb.executor(gb.kind.cos, box, [0, 2])
    t = dev(xr)
    ex.forward(prec, t, t)
    c = O.to_canonical(xr, size, order)
    for d in (0, 2):
        c = np.moveaxis(O._r2r_forward_1d(O.COS, np.moveaxis(c, O.axis_of(d), -1)), -1, O.axis_of(d))
    assert O.rel_l2(host(t), O.from_canonical(c, order)) < TOL[prec]


# ---------------------------------------------------------------------------
# fft3d / fft3d_r2c / rtransform against the reference fixtures and the oracle
# ---------------------------------------------------------------------------
def test_known_answers_3d(gb, golden):
    ka = golden["known_answers"]
    x = ka["input"]
    y = run_c2c(gb, x.astype(np.complex128), (2, 3, 4), (0, 1, 2), (0, 1, 2), 0, 0, 1)
    assert np.allclose(y, ka["c2c_fwd"], atol=1e-11)
    for kind, name in ((gb.kind.cos, "cos"), (gb.kind.sin, "sin"), (gb.kind.cos1, "cos1")):
        p = gb.rtransform(kind, gb.box3d((0, 0, 0), (1, 2, 3)), gb.box3d((0, 0, 0), (1, 2, 3)))
        t = dev(x)
        o = torch.empty_like(t)
        p.forward(t, o)
        assert np.allclose(host(o), ka[f"{name}_fwd"], atol=1e-10), name


@pytest.mark.parametrize("reorder", [0, 1])
def test_seeded_against_reference(gb, golden, reorder):
    g = golden["seeded"]
    for m in g["meta"]:
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        io = (int(m["io0"]), int(m["io1"]), int(m["io2"]))
        oo = (int(m["oo0"]), int(m["oo1"]), int(m["oo2"]))
        prec = int(m["prec"])
        key = str(m["key"])
        x, fwd_ref, bwd_ref = g[key + "_in"], g[key + "_fwd"], g[key + "_bwd"]
        opts = gb.plan_options.default()
        opts.use_reorder = reorder
        ib = gb.box3d((0, 0, 0), [s - 1 for s in size], io)
        if m["kind"] == "c2c":
            ob = gb.box3d((0, 0, 0), [s - 1 for s in size], oo)
            p = gb.fft3d(ib, ob, opts)
            want_f = O.fft3d_c2c(x, size, io, oo, 0)
        elif m["kind"] == "r2c":
            rd = int(m["r2c_dir"])
            cb = ib.r2c(rd)
            ob = gb.box3d(cb.low, cb.high, oo)
            p = gb.fft3d_r2c(ib, ob, rd, opts)
            want_f = O.fft3d_r2c(x, size, rd, io, oo)
        else:
            k = int(m["r2r_kind"])
            ob = gb.box3d((0, 0, 0), [s - 1 for s in size], oo)
            p = gb.rtransform((gb.kind.cos, gb.kind.sin, gb.kind.cos1)[k], ib, ob, opts)
            want_f = O.rtransform(k, x, size, io, oo)
        xin = dev(x)
        y = torch.empty(p.size_outbox(), dtype=torch.from_numpy(fwd_ref[:1]).dtype, device="cuda")
        p.forward(xin, y)
        yf = host(y)
        assert O.rel_l2(yf, want_f) < TOL[prec], (key, "fwd vs FP64", O.rel_l2(yf, want_f))
        assert O.rel_l2(yf, fwd_ref) < (5e-6 if prec == 0 else 1e-12), (key, "fwd vs reference")
        z = torch.empty(p.size_inbox(), dtype=xin.dtype, device="cuda")
        p.backward(dev(fwd_ref), z, gb.scale.full)
        zb = host(z)
        assert O.rel_l2(zb, bwd_ref) < (5e-6 if prec == 0 else 1e-12), (key, "bwd vs reference")
        assert np.array_equal(host(xin), x)


SIZES = [(8, 8, 8), (16, 12, 10), (27, 25, 7), (11, 13, 6), (64, 1, 9), (1, 1, 32), (5, 1, 1), (1, 1, 1),
         (96, 80, 48), (49, 22, 26), (120, 33, 2)]


@pytest.mark.parametrize("size", SIZES)
@pytest.mark.parametrize("prec", [0, 1])
def test_c2c_sizes_against_fp64(gb, size, prec):
    rng = np.random.default_rng(sum(size))
    n = int(np.prod(size))
    x = rand_c(rng, n, prec)
    for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 1, 0), (1, 0, 2))]:
        y = run_c2c(gb, x, size, io, oo, 0, 0, prec)
        assert O.rel_l2(y, O.fft3d_c2c(x, size, io, oo)) < TOL[prec], (io, oo)
        z = run_c2c(gb, y, size, io, oo, 1, 1, prec)
        assert O.rel_l2(z, O.fft3d_c2c(y, size, oo, io, 1, 1)) < TOL[prec]
        assert O.rel_l2(z, x) < 3 * TOL[prec]


@pytest.mark.parametrize("size", [(10, 9, 8), (7, 6, 5), (16, 16, 16), (2, 3, 4), (33, 10, 1), (128, 20, 12)])
@pytest.mark.parametrize("prec", [0, 1])
def test_r2c_sizes_against_fp64(gb, size, prec):
    rng = np.random.default_rng(7 + sum(size))
    n = int(np.prod(size))
    x = rng.standard_normal(n).astype(rdt(prec))
    for rd in range(3):
        for io, oo in [((0, 1, 2), (0, 1, 2)), ((1, 2, 0), (0, 2, 1))]:
            for reorder in (0, 1):
                opts = gb.plan_options.default()
                opts.use_reorder = reorder
                ib = gb.box3d((0, 0, 0), [s - 1 for s in size], io)
                cb = ib.r2c(rd)
                p = gb.fft3d_r2c(ib, gb.box3d(cb.low, cb.high, oo), rd, opts)
                xin = dev(x)
                y = torch.empty(p.size_outbox(), dtype=torch.complex64 if prec == 0 else torch.complex128,
                                device="cuda")
                p.forward(xin, y)
                yh = host(y)
                assert O.rel_l2(yh, O.fft3d_r2c(x, size, rd, io, oo)) < TOL[prec], (rd, io, oo, reorder)
                z = torch.empty_like(xin)
                p.backward(y, z, gb.scale.full)
                assert O.rel_l2(host(z), x) < 3 * TOL[prec]
                assert np.array_equal(host(y), yh), "c2r modified its input"


@pytest.mark.parametrize("size", [(8, 8, 8), (7, 6, 5), (16, 9, 4), (1, 5, 3), (32, 24, 20), (33, 25, 17),
                                  (65, 9, 2), (257, 129, 65)])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("rkind", [2, 3, 4])
def test_r2r_sizes_against_fp64(gb, size, prec, rkind):
    # every length runs (lengths with a prime factor above 13 through
    # Bluestein's algorithm); DCT-I of n values needs n >= 2
    if rkind == 4 and min(size) < 2:
        with pytest.raises(gb.HeffteError):
            gb.rtransform(rkind, gb.box3d((0, 0, 0), [s - 1 for s in size]),
                          gb.box3d((0, 0, 0), [s - 1 for s in size]))
        return
    rng = np.random.default_rng(11 + sum(size))
    n = int(np.prod(size))
    x = rng.standard_normal(n).astype(rdt(prec))
    ok = {2: O.COS, 3: O.SIN, 4: O.COS1}[rkind]
    for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 0, 1), (1, 2, 0))]:
        for reorder in (0, 1):
            opts = gb.plan_options.default()
            opts.use_reorder = reorder
            p = gb.rtransform(rkind, gb.box3d((0, 0, 0), [s - 1 for s in size], io),
                              gb.box3d((0, 0, 0), [s - 1 for s in size], oo), opts)
            xin = dev(x)
            y = torch.empty_like(xin)
            p.forward(xin, y)
            assert O.rel_l2(host(y), O.rtransform(ok, x, size, io, oo)) < TOL[prec], (io, oo, reorder)
            z = torch.empty_like(xin)
            p.backward(y, z, gb.scale.full)
            assert O.rel_l2(host(z), O.rtransform(ok, host(y), size, oo, io, 1, 1)) < TOL[prec]
            assert O.rel_l2(host(z), x) < 3 * TOL[prec]


def test_scaling_modes_and_workspace(gb):
    rng = np.random.default_rng(2)
    size = (24, 18, 10)
    x = rand_c(rng, int(np.prod(size)), 1)
    for sc in (0, 1, 2):
        for ws in (False, True):
            y = run_c2c(gb, x, size, (0, 1, 2), (0, 1, 2), 0, sc, 1, workspace=ws)
            assert O.rel_l2(y, O.fft3d_c2c(x, size, scaling=sc)) < 1e-12


def test_in_place_c2c_and_r2c(gb):
    rng = np.random.default_rng(4)
    size = (32, 16, 12)
    n = int(np.prod(size))
    x = rand_c(rng, n, 0)
    p = gb.fft3d(gb.box3d((0, 0, 0), (31, 15, 11)), gb.box3d((0, 0, 0), (31, 15, 11)))
    t = dev(x)
    p.forward(t, t)
    assert O.rel_l2(host(t), O.fft3d_c2c(x, size)) < 1e-6
    # r2c "in place": real input stored in the complex output buffer
    xr = rng.standard_normal(n).astype(np.float32)
    pr = gb.fft3d_r2c(gb.box3d((0, 0, 0), (31, 15, 11)), gb.box3d((0, 0, 0), (16, 15, 11)), 0)
    buf = torch.zeros(pr.size_outbox(), dtype=torch.complex64, device="cuda")
    buf.view(torch.float32)[:n] = dev(xr)
    pr.forward(buf.view(torch.float32)[:n], buf)
    assert O.rel_l2(host(buf), O.fft3d_r2c(xr, size, 0)) < 1e-6


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_api(gb, prec):
    rng = np.random.default_rng(6)
    size, batch = (12, 10, 9), 5   # test/test_fft3d.h:505-572 uses batch 5 on small boxes
    n = int(np.prod(size))
    x = rand_c(rng, n * batch, prec)
    p = gb.fft3d(gb.box3d((0, 0, 0), (11, 9, 8)), gb.box3d((0, 0, 0), (11, 9, 8)))
    xin = dev(x)
    y = torch.empty_like(xin)
    p.forward_batch(batch, xin, y, gb.scale.symmetric)
    yh = host(y)
    for b in range(batch):
        assert O.rel_l2(yh[b * n:(b + 1) * n], O.fft3d_c2c(x[b * n:(b + 1) * n], size, scaling=2)) < TOL[prec]


def test_c2c64_double_configuration(gb, golden):
    """64^3 complex<double> forward + backward(scale::full) against the reference."""
    g = golden["c2c64"]
    rng = np.random.default_rng(64)
    n = 64 ** 3
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    y = run_c2c(gb, x, (64, 64, 64), (0, 1, 2), (0, 1, 2), 0, 0, 1)
    assert O.rel_l2(y, O.fft3d_c2c(x, (64, 64, 64))) < 1e-12
    pos = g["pos"]
    assert np.abs(y[pos] - g["fwd_sample"]).max() / np.abs(g["fwd_sample"]).max() < 1e-12
    z = run_c2c(gb, y, (64, 64, 64), (0, 1, 2), (0, 1, 2), 1, 1, 1)
    assert O.rel_l2(z, x) < 1e-12
    assert np.abs(z - x).max() < 1e-12


def test_errors_on_gpu(gb):
    p = gb.fft3d(gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 7)))
    a = torch.zeros(512, dtype=torch.complex64, device="cuda")
    b = torch.zeros(512, dtype=torch.complex128, device="cuda")
    with pytest.raises(gb.heffte_input_error):
        p.forward(a, b)
    with pytest.raises(gb.heffte_input_error):
        p.forward(a[:100], a)
    with pytest.raises(gb.heffte_input_error):
        p.forward(a.cpu(), a)


@pytest.mark.parametrize("rkind", [0, 1, 2])
@pytest.mark.parametrize("prec", [0, 1])
def test_r2r_prepost_location_layer_bit_exact(gb, rkind, prec):
    """Batched pre/post processors against the restated CPU processors (data moves and negations only)."""
    rng = np.random.default_rng(rkind * 10 + prec)
    N, lines = 13, 7
    M = 4 * (N - 1) if rkind == 2 else 4 * N
    H = M // 2 + 1
    real = rdt(prec)
    x = rng.standard_normal(lines * N).astype(real)
    ext = rng.standard_normal(lines * M).astype(real)
    cext = rand_c(rng, lines * H, prec)
    cases = [(0, x, N, M, real), (1, cext, H, N, real), (2, x, N, H, cdt(prec)), (3, ext, M, N, real)]
    for step, inp, in_ld, out_ld, odt in cases:
        want = np.concatenate([O.prepost_line(rkind, step, inp[b * in_ld:(b + 1) * in_ld], N)
                               for b in range(lines)]).astype(odt)
        out = torch.zeros(lines * out_ld, dtype=torch.from_numpy(np.zeros(1, odt)).dtype, device="cuda")
        gb.r2r_prepost(prec, rkind, step, N, lines, in_ld, out_ld, dev(inp), out)
        assert host(out).tobytes() == want.tobytes(), (rkind, step)


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("prec", [0, 1])
def test_power_of_two_kernel_variants(gb, variant, prec):
    """Every kernel family (0: the default pipelined kernels with tensor-map
    column tiles; 1, 2: generic runtime-radix, pipelined bulk-copy) on the
    power-of-two lengths, line and column layouts (partial wide column tiles
    of 512, 2048 and 4096 points), in and out of place."""
    gb.set_kernel_variant(variant)
    try:
        rng = np.random.default_rng(variant + 2 * prec)
        for size in [(2, 4, 8), (16, 32, 64), (128, 16, 32), (256, 8, 16), (512, 16, 32), (32, 1024, 2),
                     (2048, 2, 16), (4096, 2, 4), (64, 64, 64), (50, 512, 2), (14, 2048, 2), (6, 4096, 2)]:
            n = int(np.prod(size))
            x = rand_c(rng, n, prec)
            for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 1, 0), (2, 1, 0)), ((1, 0, 2), (0, 2, 1))]:
                y = run_c2c(gb, x, size, io, oo, 0, 1, prec)
                assert O.rel_l2(y, O.fft3d_c2c(x, size, io, oo, 0, 1)) < TOL[prec], (size, io, oo)
                z = run_c2c(gb, y, size, io, oo, 1, 0, prec)
                assert O.rel_l2(z, x) < 3 * TOL[prec]
            p = gb.fft3d(gb.box3d((0, 0, 0), [s - 1 for s in size]), gb.box3d((0, 0, 0), [s - 1 for s in size]))
            t = dev(x)
            p.forward(t, t)
            assert O.rel_l2(host(t), O.fft3d_c2c(x, size)) < TOL[prec]
        assert gb.device_status() == 0
    finally:
        gb.set_kernel_variant(0)


@pytest.mark.parametrize("variant", [0, 3])
def test_compiled_plan_lengths(gb, variant):
    """The float lengths with kernels compiled for their radix plan (96 ...
    960; variant 0) and the same lengths on the runtime radix plan (variant
    3): the length along each dimension (line tiles, column tiles), partial
    tiles, three orders, forward and backward."""
    gb.set_kernel_variant(variant)
    try:
        rng = np.random.default_rng(70 + variant)
        for N in (96, 160, 192, 240, 288, 320, 384, 448, 480, 576, 640, 720, 768, 960):
            for size in [(N, 13, 3), (5, N, 7), (3, 11, N)]:
                n = int(np.prod(size))
                x = rand_c(rng, n, 0)
                for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 1, 0), (2, 1, 0)), ((1, 0, 2), (0, 2, 1))]:
                    y = run_c2c(gb, x, size, io, oo, 0, 1, 0)
                    assert O.rel_l2(y, O.fft3d_c2c(x, size, io, oo, 0, 1)) < TOL[0], (N, size, io, oo)
                    z = run_c2c(gb, y, size, io, oo, 1, 0, 0)
                    assert O.rel_l2(z, x) < 3 * TOL[0], (N, size, io, oo, "backward")
        assert gb.device_status() == 0
    finally:
        gb.set_kernel_variant(0)


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("prec", [0, 1])
def test_power_of_two_real_kernel_variants(gb, variant, prec):
    """r2c / c2r and DCT / DST through both kernel families: line tiles, column
    tiles with TMA tensor maps and cp.async (odd half-spectrum widths, partial
    tiles), every r2c direction, two orders."""
    gb.set_kernel_variant(variant)
    try:
        rng = np.random.default_rng(40 + variant + 2 * prec)
        for size in [(64, 32, 16), (32, 128, 16), (256, 16, 32), (16, 16, 512)]:
            n = int(np.prod(size))
            x = rng.standard_normal(n).astype(rdt(prec))
            for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 0, 1), (2, 0, 1))]:
                ib = gb.box3d((0, 0, 0), [s - 1 for s in size], io)
                for rd in range(3):
                    cb = ib.r2c(rd)
                    p = gb.fft3d_r2c(ib, gb.box3d(cb.low, cb.high, oo), rd)
                    xin = dev(x)
                    y = torch.empty(p.size_outbox(), dtype=torch.complex64 if prec == 0 else torch.complex128,
                                    device="cuda")
                    p.forward(xin, y, gb.scale.full)
                    assert O.rel_l2(host(y), O.fft3d_r2c(x, size, rd, io, oo, 1)) < TOL[prec], (size, rd, io)
                    z = torch.empty_like(xin)
                    p.backward(y, z)
                    assert O.rel_l2(host(z), x) < 3 * TOL[prec], (size, rd, io, "c2r")
                for rk, ok in ((gb.kind.cos, O.COS), (gb.kind.sin, O.SIN)):
                    p = gb.rtransform(rk, ib, gb.box3d((0, 0, 0), [s - 1 for s in size], oo))
                    xin = dev(x)
                    y = torch.empty_like(xin)
                    p.forward(xin, y)
                    assert O.rel_l2(host(y), O.rtransform(ok, x, size, io, oo)) < TOL[prec], (size, rk, io)
                    z = torch.empty_like(xin)
                    p.backward(y, z, gb.scale.full)
                    assert O.rel_l2(host(z), x) < 3 * TOL[prec], (size, rk, io, "bwd")
        assert gb.device_status() == 0
    finally:
        gb.set_kernel_variant(0)
