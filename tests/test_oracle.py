"""Pins the CPU oracles (numpy restatement and the C port) to the reference's
own outputs (golden fixtures produced by the compiled reference) and to the
known answers of the reference's unit tests.  CPU only."""
import numpy as np
import pytest

from oracle import heffte_oracle as O

SIZE_KA = (2, 3, 4)


def test_known_answer_dct_ii_reference_unit_test():
    # test/test_units_nompi.cpp:311 — DCT-II of [1,2,3,4] (FFTW REDFT10 convention)
    y = O._r2r_forward_1d(O.COS, np.array([[1.0, 2.0, 3.0, 4.0]]))[0]
    assert np.allclose(y, [20.0, -6.308644059797899, 0.0, -0.44834152916796777], atol=1e-12)


def test_known_answer_dft_impulse():
    # impulse -> all ones (test/test_units_stock.cpp:179-226)
    x = np.zeros(11, complex)
    x[0] = 1
    y = O.fft3d_c2c(x, (11, 1, 1))
    assert np.allclose(y, 1.0)


def test_numpy_oracle_known_answers(golden):
    ka = golden["known_answers"]
    x = ka["input"]
    assert np.allclose(O.fft3d_c2c(x.astype(complex), SIZE_KA), ka["c2c_fwd"], atol=1e-12)
    for d in range(3):
        assert np.allclose(O.executor_c2c(x.astype(complex), SIZE_KA, (0, 1, 2), d), ka[f"exec_dim{d}"], atol=1e-12)
        assert np.allclose(O.fft3d_r2c(x, SIZE_KA, d), ka[f"r2c_dir{d}"], atol=1e-12)
    for kind, name in ((O.COS, "cos"), (O.SIN, "sin"), (O.COS1, "cos1")):
        assert np.allclose(O.rtransform(kind, x, SIZE_KA), ka[f"{name}_fwd"], atol=1e-10)


def _cases(golden, kind):
    meta = golden["seeded"]["meta"]
    return [m for m in meta if m["kind"] == kind]


def _tol(prec):
    return 1e-5 if prec == 0 else 1e-12


def test_numpy_oracle_seeded(golden):
    g = golden["seeded"]
    for m in g["meta"]:
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        io = (int(m["io0"]), int(m["io1"]), int(m["io2"]))
        oo = (int(m["oo0"]), int(m["oo1"]), int(m["oo2"]))
        key = str(m["key"])
        x, fwd, bwd = g[key + "_in"], g[key + "_fwd"], g[key + "_bwd"]
        tol = _tol(int(m["prec"]))
        if m["kind"] == "c2c":
            assert O.rel_l2(O.fft3d_c2c(x, size, io, oo, 0), fwd) < tol, key
            assert O.rel_l2(O.fft3d_c2c(fwd, size, oo, io, 1, O.SCALE_FULL), bwd) < tol, key
        elif m["kind"] == "r2c":
            rd = int(m["r2c_dir"])
            assert O.rel_l2(O.fft3d_r2c(x, size, rd, io, oo), fwd) < tol, key
            assert O.rel_l2(O.fft3d_c2r(fwd, size, rd, oo, io, O.SCALE_FULL), bwd) < tol, key
        else:
            k = int(m["r2r_kind"])
            assert O.rel_l2(O.rtransform(k, x, size), fwd) < tol, key
            assert O.rel_l2(O.rtransform(k, fwd, size, direction=1, scaling=O.SCALE_FULL), bwd) < tol, key


def test_numpy_oracle_packers_bit_exact(golden):
    g = golden["packers"]
    for m in g["meta"]:
        idx = int(m["idx"])
        es = int(m["esize"])
        dt = {4: np.uint32, 8: np.uint64, 16: np.dtype((np.void, 16))}[es]
        src = g[f"t{idx}_src"].view(dt)
        dst = g[f"t{idx}_dst"].view(dt)
        want = g[f"t{idx}_out"].view(dt)
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        if m["op"] == "pack":
            got = dst.copy()
            got[:int(np.prod(size))] = O.direct_pack(src, size, int(m["ls"]), int(m["ps"]))
        elif m["op"] == "unpack":
            got = O.direct_unpack(src, dst, size, int(m["ls"]), int(m["ps"]))
        else:
            got = O.transpose_unpack(src, dst, size, int(m["ls"]), int(m["ps"]), int(m["bls"]), int(m["bps"]),
                                     (int(m["m0"]), int(m["m1"]), int(m["m2"])))
        assert got.tobytes() == want.tobytes(), (m["op"], idx)


def test_port_seeded(golden, port_lib):
    """The C port reproduces the reference within the reference's own tolerances."""
    g = golden["seeded"]
    for m in g["meta"]:
        io = (int(m["io0"]), int(m["io1"]), int(m["io2"]))
        oo = (int(m["oo0"]), int(m["oo1"]), int(m["oo2"]))
        if io != (0, 1, 2) or oo != (0, 1, 2):
            continue  # the port runs the order (0,1,2) plan
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        key = str(m["key"])
        x, fwd, bwd = g[key + "_in"], g[key + "_fwd"], g[key + "_bwd"]
        tol = 5e-6 if int(m["prec"]) == 0 else 1e-12
        if m["kind"] == "c2c":
            assert O.rel_l2(O.port_fft3d_c2c(x, size, 0), fwd) < tol, key
            assert O.rel_l2(O.port_fft3d_c2c(fwd, size, 1, O.SCALE_FULL), bwd) < tol, key
        elif m["kind"] == "r2c":
            rd = int(m["r2c_dir"])
            assert O.rel_l2(O.port_fft3d_r2c(x, size, rd, 0), fwd) < tol, key
            assert O.rel_l2(O.port_fft3d_r2c(fwd, size, rd, 1, O.SCALE_FULL), bwd) < tol, key
        else:
            k = int(m["r2r_kind"])
            assert O.rel_l2(O.port_rtransform(k, x, size, 0), fwd) < tol, key
            assert O.rel_l2(O.port_rtransform(k, fwd, size, 1, O.SCALE_FULL), bwd) < tol, key


def test_port_packers_bit_exact(golden, port_lib):
    g = golden["packers"]
    for m in g["meta"]:
        idx = int(m["idx"])
        es = int(m["esize"])
        src, dst, want = g[f"t{idx}_src"], g[f"t{idx}_dst"], g[f"t{idx}_out"]
        size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
        op = {"pack": 0, "unpack": 1, "transpose": 2}[str(m["op"])]
        # the port moves esize-byte elements; view the byte buffers accordingly
        dt = {4: np.float32, 8: np.float64, 16: np.complex128}[es]
        got = O.port_pack(op, src.view(dt), dst.view(dt), size, int(m["ls"]), int(m["ps"]), int(m["bls"]),
                          int(m["bps"]), (int(m["m0"]), int(m["m1"]), int(m["m2"])))
        assert got.view(np.uint8).tobytes() == want.tobytes(), (m["op"], idx)


def test_c2c64_golden_against_oracle(golden):
    """Configuration 64^3 complex<double>: the numpy oracle against the reference samples."""
    import sys
    sys.path.insert(0, O.HERE)
    g = golden["c2c64"]
    rng = np.random.default_rng(64)
    n = 64 ** 3
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    y = O.fft3d_c2c(x, (64, 64, 64))
    pos = g["pos"]
    assert np.abs(y[pos] - g["fwd_sample"]).max() / np.abs(g["fwd_sample"]).max() < 1e-12
    assert abs(np.linalg.norm(y) - float(g["fwd_norm"])) / float(g["fwd_norm"]) < 1e-12


@pytest.mark.skipif(O.load_ref() is None, reason="reference build (oracle/_ref) not present")
def test_numpy_oracle_against_reference_random():
    """Extra random geometries straight against the compiled reference."""
    import ctypes
    lib = O.load_ref()
    I3 = ctypes.c_int * 3
    rng = np.random.default_rng(11)
    for size in [(3, 5, 7), (9, 4, 11), (16, 1, 6), (1, 1, 13)]:
        for io, oo in [((0, 1, 2), (0, 1, 2)), ((2, 0, 1), (1, 2, 0))]:
            for reorder in (0, 1):
                n = int(np.prod(size))
                x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
                y = np.empty_like(x)
                assert lib.ref_fft3d_c2c(1, I3(0, 0, 0), I3(*[s - 1 for s in size]), I3(*io), I3(*oo), reorder, 1, 0,
                                         0, O._ptr(x), O._ptr(y)) == 0
                assert O.rel_l2(O.fft3d_c2c(x, size, io, oo), y) < 1e-13
