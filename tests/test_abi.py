"""CPU checks of the C ABI: the library loads, exports every declared symbol,
and rejects bad input with the documented status codes and messages (plan and
executor creation touch no GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "heffte_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(heffte_gb300_\w+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("heffte_gb300_transpose_unpack", "heffte_gb300_direct_pack", "heffte_gb300_direct_unpack",
              "heffte_gb300_scale_data", "heffte_gb300_convert", "heffte_gb300_executor_create",
              "heffte_gb300_plan_create", "heffte_gb300_forward", "heffte_gb300_backward"):
        assert n in names


def test_library_exports_every_declared_symbol(gb):
    L = gb.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def _box(lo, hi, o=(0, 1, 2)):
    I3 = ctypes.c_int * 3
    return I3(*lo), I3(*hi), I3(*o)


def test_plan_create_and_sizes(gb):
    p = gb.fft3d(gb.box3d((0, 0, 0), (63, 31, 15)), gb.box3d((0, 0, 0), (63, 31, 15)))
    assert p.size_inbox() == 64 * 32 * 16 and p.size_outbox() == 64 * 32 * 16
    assert p.get_scale_factor(gb.scale.full) == pytest.approx(1.0 / (64 * 32 * 16))
    r = gb.fft3d_r2c(gb.box3d((0, 0, 0), (63, 31, 15)), gb.box3d((0, 0, 0), (32, 31, 15)), 0)
    assert r.size_outbox() == 33 * 32 * 16
    c = gb.rtransform(gb.kind.cos, gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 7)))
    # rtransform scale: 1 / (64 N) for the cuFFT-style cos/sin conventions (heffte_fft3d.h:635-650)
    assert c.get_scale_factor(gb.scale.full) == pytest.approx(1.0 / (64 * 512))
    assert c.get_scale_factor(gb.scale.symmetric) == pytest.approx((1.0 / (64 * 512)) ** 0.5)


def test_plan_rejects_bad_geometry(gb):
    with pytest.raises(gb.HeffteError) as e:
        gb.fft3d(gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 6)))
    assert e.value.code == 1 and "same indexes" in str(e.value)
    with pytest.raises(gb.HeffteError) as e:
        gb.fft3d_r2c(gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (7, 7, 7)), 0)
    assert e.value.code == 1
    with pytest.raises(gb.heffte_input_error):
        gb.fft3d_r2c(gb.box3d((0, 0, 0), (7, 7, 7)), gb.box3d((0, 0, 0), (4, 7, 7)), 3)
    with pytest.raises(gb.heffte_input_error):
        gb.box3d((0, 0, 0), (7, 7, 7), (0, 0, 1))


def test_plan_rejects_unsupported_length(gb):
    n = (1 << 25) + 1                           # above the longest transform, 2^25
    with pytest.raises(gb.HeffteError) as e:
        gb.fft3d(gb.box3d((0, 0, 0), (n - 1, 0, 0)), gb.box3d((0, 0, 0), (n - 1, 0, 0)))
    assert e.value.code == 3 and str(n) in str(e.value)


def test_composite_lengths_plan_with_a_workspace(gb):
    """Lengths with a prime factor above 13 (Bluestein) and above 8192
    (four-step) are planned like any other; their scratch is part of the
    plan's workspace, and the executors report theirs (no GPU needed)."""
    for size in ((17, 8, 6), (17, 23, 29), (16384, 2, 2), (8191, 1, 2)):
        b = gb.box3d((0, 0, 0), [s - 1 for s in size])
        p = gb.fft3d(b, b)
        assert p.size_workspace() > 0, size
        r = gb.fft3d_r2c(b, b.r2c(0), 0)
        assert r.size_workspace() > 0, size
    b = gb.box3d((0, 0, 0), (63, 31, 15))
    assert gb.fft3d(b, b).size_workspace() == 0          # direct lengths, no reshapes: none
    ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), (96, 3, 2)), [0])
    assert ex.workspace_size() >= 2 * 97 * 12            # two copies of the lines, plus Bluestein's
    ex = gb.executor(gb.kind.cos, gb.box3d((0, 0, 0), (96, 3, 2)), [0])
    assert ex.workspace_size() % 2 == 0 and ex.workspace_size() > 0   # real elements
    with pytest.raises(gb.HeffteError) as e:
        gb.boxbatch(gb.kind.r2c, [(17, 16, 16)])       # the batch kernel takes direct lengths only
    assert e.value.code == 3


def test_dct1_plans_and_scale(gb):
    """rtransform<cos1>: lengths n >= 2, scale 1/(64 prod(n_i - 1))
    (include/heffte_fft3d.h:643-647)."""
    b = gb.box3d((0, 0, 0), (32, 24, 16))           # 33 x 25 x 17: FFTs of 64, 48, 32
    p = gb.rtransform(gb.kind.cos1, b, b)
    assert p.size_inbox() == 33 * 25 * 17
    assert p.get_scale_factor(gb.scale.full) == pytest.approx(1.0 / (64 * 32 * 24 * 16))
    b = gb.box3d((0, 0, 0), (31, 7, 7))              # 2 * 31 = 62: Bluestein's FFT
    assert gb.rtransform(gb.kind.cos1, b, b).size_workspace() > 0
    for bad in ((0, 7, 7), ((1 << 24) + 1, 7, 7)):    # n = 1; 2(n - 1) above 2^25
        with pytest.raises(gb.HeffteError) as e:
            bb = gb.box3d((0, 0, 0), bad)
            gb.rtransform(gb.kind.cos1, bb, bb)
        assert e.value.code == 3 and "DCT-I" in str(e.value)


def test_plan_option_setters_validate(gb):
    b = gb.box3d((0, 0, 0), (63, 31, 15))
    p = gb.fft3d(b, b)
    p.set_tensor_cores(True)
    p.set_tensor_cores(False)
    p.set_knobs(1, 2, 1)
    p.set_knobs(0, 1, 0)
    L = gb.lib()
    assert L.heffte_gb300_plan_set_tensor_cores(p._h, 2) == 1
    for args in ((2, 1, 0), (0, 3, 0), (0, 1, 2), (-1, 1, 0)):
        assert L.heffte_gb300_plan_set_knobs(p._h, *args) == 1
    assert L.heffte_gb300_plan_set_tensor_cores(None, 1) == 1
    assert p.size_inbox() == 64 * 32 * 16          # the plan survives rejected settings
    # process-wide kernel family: 0 automatic, 1 generic, 2 pipelined, 3 automatic
    # with runtime radix plans only; anything else is rejected and changes nothing
    for v in (3, 2, 1, 0):
        assert L.heffte_gb300_set_kernel_variant(v) == 0
    for v in (-1, 4):
        assert L.heffte_gb300_set_kernel_variant(v) == 1
        assert b"variant" in L.heffte_gb300_last_error()


def test_raw_abi_status_codes(gb):
    L = gb.lib()
    h = ctypes.c_void_p()
    lo, hi, o = _box((0, 0, 0), (3, 3, 3))
    bad = (ctypes.c_int * 3)(0, 0, 0)
    assert L.heffte_gb300_plan_create(0, lo, hi, bad, lo, hi, o, 0, None, None, ctypes.byref(h)) == 1
    assert b"permutation" in L.heffte_gb300_last_error()
    assert L.heffte_gb300_plan_create(9, lo, hi, o, lo, hi, o, 0, None, None, ctypes.byref(h)) == 1
    assert L.heffte_gb300_plan_create(0, lo, hi, o, lo, hi, o, 0, None, None, None) == 1
    assert L.heffte_gb300_plan_create(0, lo, hi, o, lo, hi, o, 0, None, None, ctypes.byref(h)) == 0
    assert L.heffte_gb300_last_error() == b""
    assert L.heffte_gb300_size_workspace(h) >= 0
    # null data pointers are rejected before any device work
    assert L.heffte_gb300_forward(h, 0, None, None, None, 0) == 1
    assert L.heffte_gb300_forward(h, 5, None, None, None, 0) == 1
    assert L.heffte_gb300_plan_destroy(h) == 0
    # location layer argument checks
    assert L.heffte_gb300_transpose_unpack(None, 2, 4, 4, 4, 4, 16, 4, 16, 0, 0, 1, None, None) == 1
    assert L.heffte_gb300_direct_pack(None, 7, 4, 4, 4, 4, 16, None, None) == 1
    assert L.heffte_gb300_scale_data(None, 0, 0, None, 2.0) == 0  # empty box: no-op
    assert L.heffte_gb300_scale_data(None, 0, -1, None, 2.0) == 1


def test_executor_abi(gb):
    ex = gb.executor(gb.kind.c2c, gb.box3d((0, 0, 0), (7, 5, 3)), [1])
    assert ex.box_size() == 8 * 6 * 4 and ex.workspace_size() == 0
    r = gb.executor(gb.kind.r2c, gb.box3d((0, 0, 0), (7, 5, 3)), [0])
    assert r.complex_size() == 5 * 6 * 4
    with pytest.raises(gb.HeffteError):
        gb.executor(gb.kind.r2c, gb.box3d((0, 0, 0), (7, 5, 3)), [0, 1])


def test_fast_division_parameters():
    """The magic-number division used for the Stockham index split is exact
    for every divisor/numerator the kernels can see (numerators < 2^20)."""
    import numpy as np
    divisors = sorted({a * b for a in (1, 2, 3, 4, 5, 7, 8, 11, 13, 16) for b in (1, 2, 4, 8, 16, 32, 64, 128, 256,
                                                                                    512, 1024, 3, 9, 27, 81, 5, 25)})
    j = np.arange(1 << 20, dtype=np.uint64)
    for d in divisors:
        l = 0
        while (1 << l) < d:
            l += 1
        m = ((1 << 32) * ((1 << l) - d)) // d + 1
        m &= 0xFFFFFFFF
        q = (((j * np.uint64(m)) >> np.uint64(32)) + j) >> np.uint64(l)
        assert np.array_equal(q, j // np.uint64(d)), d
