"""Batches of uneven boxes in one persistent graph-replayed launch, and the
autotuner that picks their radix plans.  Each box is checked against the FP64
oracle of its own fft3d_r2c (rel-L2 <= 1e-6 float, <= 1e-12 double)."""
import os
import tempfile

import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIDES = [16, 24, 32, 40, 48, 64, 80, 96, 128]
TOL = {0: 1e-6, 1: 1e-12}


def _sizes(rng, nboxes, sides):
    return [tuple(int(v) for v in rng.choice(sides, 3)) for _ in range(nboxes)]


@pytest.mark.parametrize("prec", [0, 1])
def test_r2c_batch_against_oracle(gb, prec):
    rng = np.random.default_rng(256 + prec)
    sizes = _sizes(rng, 40, SIDES[:6])
    b = gb.boxbatch(gb.kind.r2c, sizes, prec)
    rdt, cdt = (np.float32, torch.complex64) if prec == 0 else (np.float64, torch.complex128)
    x = rng.standard_normal(b.input_size()).astype(rdt)
    xin = torch.from_numpy(x).cuda()
    y = torch.empty(b.output_size(), dtype=cdt, device="cuda")
    for sc in (gb.scale.none, gb.scale.full):
        b.forward(xin, y, sc)
        yh = y.cpu().numpy()
        for i, s in enumerate(sizes):
            n = int(np.prod(s))
            nc = (s[0] // 2 + 1) * s[1] * s[2]
            xi = x[b.input_offset(i):b.input_offset(i) + n]
            yi = yh[b.output_offset(i):b.output_offset(i) + nc]
            assert O.rel_l2(yi, O.fft3d_r2c(xi, s, 0, scaling=sc)) < TOL[prec], (i, s, sc)
    # backward: input untouched, round trip
    w = torch.empty(b.workspace_size(), dtype=cdt, device="cuda")
    z = torch.empty_like(xin)
    y_before = y.clone()
    b.backward(y, z, w, gb.scale.none)
    torch.cuda.synchronize()
    assert torch.equal(y, y_before)
    assert O.rel_l2(z.cpu().numpy(), x) < 3 * TOL[prec]
    assert gb.device_status() == 0


def test_c2c_batch_and_repeated_replay(gb):
    rng = np.random.default_rng(7)
    sizes = _sizes(rng, 17, SIDES[:7])
    b = gb.boxbatch(gb.kind.c2c, sizes, 0)
    n = b.input_size()
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    for rep in range(3):          # the graph is replayed with new buffers each time
        xin = torch.from_numpy(x).cuda()
        y = torch.empty_like(xin)
        b.forward(xin, y, gb.scale.symmetric)
        yh = y.cpu().numpy()
        for i, s in enumerate(sizes):
            m = int(np.prod(s))
            o = b.input_offset(i)
            assert O.rel_l2(yh[o:o + m], O.fft3d_c2c(x[o:o + m], s, scaling=2)) < 1e-6
        x = np.roll(x, 1)
    assert gb.device_status() == 0


def test_tuner_resumes_from_cache_and_batch_uses_tuned_plans(gb):
    gb.tune_clear()
    with tempfile.TemporaryDirectory() as tmp:
        cache = os.path.join(tmp, "tune.tsv")
        assert gb.tune(0, [24, 48], cache) == 2
        assert gb.tune(0, [24, 48, 80], cache) == 1          # only 80 is new
        rad48, tpb48, us48 = gb.tuned_choice(0, 48)
        assert int(np.prod(rad48)) == 48 and tpb48 > 0 and us48 > 0
        gb.tune_clear()
        assert gb.tuned_choice(0, 48)[0] == []
        assert gb.tune_load(cache) == 3                        # resume: read back, nothing re-measured
        assert gb.tune(0, [24, 48, 80], cache) == 0
        assert gb.tuned_choice(0, 48)[0] == rad48
    rng = np.random.default_rng(3)
    sizes = [(24, 48, 80), (48, 24, 24), (80, 80, 48)]
    b = gb.boxbatch(gb.kind.r2c, sizes, 0)
    x = rng.standard_normal(b.input_size()).astype(np.float32)
    y = torch.empty(b.output_size(), dtype=torch.complex64, device="cuda")
    b.forward(torch.from_numpy(x).cuda(), y)
    yh = y.cpu().numpy()
    for i, s in enumerate(sizes):
        n = int(np.prod(s))
        nc = (s[0] // 2 + 1) * s[1] * s[2]
        xi = x[b.input_offset(i):b.input_offset(i) + n]
        assert O.rel_l2(yh[b.output_offset(i):b.output_offset(i) + nc], O.fft3d_r2c(xi, s, 0)) < 1e-6
    gb.tune_clear()


def test_dependency_wait_gives_up_and_the_next_call_is_correct(gb):
    """The give-up path of the batch kernel's bounded pass-dependency wait.

    With the dependencies held (each waits for one tile more than its pass
    has, a count no CTA reaches) and a 2e6-clock budget (about a millisecond),
    every waiting CTA must give up, record status 2, and return; the launch
    then ends by itself.  After the status is read and cleared, the budget
    restored and the hold lifted, the same batch must run correctly."""
    rng = np.random.default_rng(99)
    sizes = _sizes(rng, 24, SIDES[:6])
    b = gb.boxbatch(gb.kind.r2c, sizes, 0)
    x = rng.standard_normal(b.input_size()).astype(np.float32)
    xin = torch.from_numpy(x).cuda()
    y = torch.zeros(b.output_size(), dtype=torch.complex64, device="cuda")
    assert gb.device_status(reset=True) == 0
    old = gb.set_dependency_wait_budget(2_000_000)
    try:
        b.hold_dependencies(True)
        b.forward(xin, y)
        torch.cuda.synchronize()
        assert gb.device_status(reset=True) == gb.DEV_TIMEOUT_DEPENDENCY
    finally:
        gb.set_dependency_wait_budget(old)
        b.hold_dependencies(False)
    assert old == 4_000_000_000
    assert gb.device_status() == 0
    b.forward(xin, y)
    yh = y.cpu().numpy()
    for i, s in enumerate(sizes):
        n = int(np.prod(s))
        nc = (s[0] // 2 + 1) * s[1] * s[2]
        xi = x[b.input_offset(i):b.input_offset(i) + n]
        yi = yh[b.output_offset(i):b.output_offset(i) + nc]
        assert O.rel_l2(yi, O.fft3d_r2c(xi, s, 0)) < TOL[0], (i, s)
    assert gb.device_status() == 0


@pytest.mark.parametrize("prefetch,tile_kb,group_mb,values", [(1, 48, 0, 16), (0, 48, 0, 16), (1, 24, 0, 16),
                                                             (1, 32, 0, 8), (0, 24, 0, 8), (0, 48, 1, 8),
                                                             (1, 32, 2, 16), (0, 24, 16, 8), (1, 48, 0, 8)])
def test_batch_launch_shapes_give_the_same_result(gb, prefetch, tile_kb, group_mb, values):
    """Every launch shape (the next tile copied ahead into shared memory or
    not; tile bounds that change the CTAs per SM; pass-major queue or boxes in
    groups, 1 and 2 MB groups making many groups of a few boxes; 16 or 8
    values per thread) against the oracle, r2c forward and the backward round
    trip, float and double sides."""
    rng = np.random.default_rng(31 + tile_kb + group_mb + values)
    sizes = _sizes(rng, 30, SIDES)
    for prec in (0, 1):
        b = gb.boxbatch(gb.kind.r2c, sizes, prec)
        b.configure(prefetch, tile_kb, group_mb, values)
        assert b.config() == (prefetch, tile_kb, group_mb, values)
        rdt, cdt = (np.float32, torch.complex64) if prec == 0 else (np.float64, torch.complex128)
        x = rng.standard_normal(b.input_size()).astype(rdt)
        xin = torch.from_numpy(x).cuda()
        y = torch.empty(b.output_size(), dtype=cdt, device="cuda")
        b.forward(xin, y)
        yh = y.cpu().numpy()
        for i, s in enumerate(sizes):
            n = int(np.prod(s))
            nc = (s[0] // 2 + 1) * s[1] * s[2]
            xi = x[b.input_offset(i):b.input_offset(i) + n]
            yi = yh[b.output_offset(i):b.output_offset(i) + nc]
            assert O.rel_l2(yi, O.fft3d_r2c(xi, s, 0)) < TOL[prec], (prec, i, s)
        w = torch.empty(b.workspace_size(), dtype=cdt, device="cuda")
        z = torch.empty_like(xin)
        b.backward(y, z, w, gb.scale.full)
        assert O.rel_l2(z.cpu().numpy(), x) < 3 * TOL[prec]
    assert gb.device_status() == 0


def test_batch_autotune_keeps_a_correct_shape(gb):
    rng = np.random.default_rng(64)
    sizes = _sizes(rng, 40, SIDES)
    b = gb.boxbatch(gb.kind.c2c, sizes, 0)
    n = b.input_size()
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    xin = torch.from_numpy(x).cuda()
    y = torch.empty_like(xin)
    z = torch.empty_like(xin)
    w = torch.empty(b.workspace_size(), dtype=torch.complex64, device="cuda")
    pf, kb, gm, vals, ms = b.autotune(xin, y, z, w, reps=2)
    assert (pf, kb, gm, vals) == b.config() and pf in (0, 1) and kb in (24, 32, 48) and gm in (0, 16)
    assert vals in (8, 16) and ms > 0
    assert torch.equal(xin.cpu(), torch.from_numpy(x))      # the input is left as it was
    b.forward(xin, y)
    yh = y.cpu().numpy()
    for i, s in enumerate(sizes):
        m = int(np.prod(s))
        xi = x[b.input_offset(i):b.input_offset(i) + m]
        yi = yh[b.output_offset(i):b.output_offset(i) + m]
        assert O.rel_l2(yi, O.fft3d_c2c(xi, s)) < TOL[0], (i, s)


@pytest.mark.parametrize("prec", [0, 1])
def test_r2c_batch_with_sides_of_prime_factors_7_11_13(gb, prec):
    """Sides with factors 7, 11 and 13 (the kernels with every radix stage)
    beside 5-smooth ones (the kernels without the radix-7/11/13 stages run
    only batches whose plans are all 5-smooth), forward and round trip."""
    rng = np.random.default_rng(77 + prec)
    sizes = _sizes(rng, 12, [56, 44, 52, 28, 112, 16, 40])
    b = gb.boxbatch(gb.kind.r2c, sizes, prec)
    rdt, cdt = (np.float32, torch.complex64) if prec == 0 else (np.float64, torch.complex128)
    x = rng.standard_normal(b.input_size()).astype(rdt)
    xin = torch.from_numpy(x).cuda()
    y = torch.empty(b.output_size(), dtype=cdt, device="cuda")
    b.forward(xin, y)
    yh = y.cpu().numpy()
    for i, s in enumerate(sizes):
        n = int(np.prod(s))
        nc = (s[0] // 2 + 1) * s[1] * s[2]
        xi = x[b.input_offset(i):b.input_offset(i) + n]
        yi = yh[b.output_offset(i):b.output_offset(i) + nc]
        assert O.rel_l2(yi, O.fft3d_r2c(xi, s, 0)) < TOL[prec], (i, s)
    w = torch.empty(b.workspace_size(), dtype=cdt, device="cuda")
    z = torch.empty_like(xin)
    b.backward(y, z, w, gb.scale.full)
    assert O.rel_l2(z.cpu().numpy(), x) < 3 * TOL[prec]
    assert gb.device_status() == 0
