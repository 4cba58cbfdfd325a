"""Generate the golden fixtures in this directory from the heFFTe reference.

The fixtures are produced by the reference's own stock backend, compiled from
the reference sources by ``oracle/ref/Makefile`` into
``oracle/_ref/libheffte_ref.so`` (a container with the reference tree is
needed to regenerate them; the GPU tests only read the committed ``.npz``).

Cases:
* ``known_answers.npz`` — the 2x3x4 box holding 1..24 used by the reference's
  unit tests (test/test_units_nompi.cpp:92-202, test/test_cos.cpp:36-54):
  3-D c2c, the per-dimension executor stages, r2c along each dimension and
  the three real-to-real kinds, computed by the reference;
* ``seeded.npz`` — seeded random boxes (numpy PCG64) in several orders,
  forward and backward, float and double, c2c / r2c / r2r;
* ``packers.npz`` — pack, unpack and all six transpose maps on random bytes
  (bit-exact cases) for 4, 8 and 16 byte elements;
* ``c2c64.npz`` — the 64x64x64 complex<double> forward+backward case with
  re/im uniform [-1, 1) from seed 64: the output sampled at 4096 seeded
  positions plus its L2 norm (the full arrays are regenerated from the seed);
* ``convolution.npz`` — the convolution benchmark's step (forward scale::full,
  X .* X, backward) and a two-input circular convolution, complex<float> and
  complex<double>, and two-input convolutions of real data through
  fft3d_r2c, computed by the reference's transforms.

Run:  python tests/golden/make_golden.py [fixture ...]
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import heffte_oracle as O  # noqa: E402

I3 = ctypes.c_int * 3
LL3 = ctypes.c_longlong * 3


def ref():
    lib = O.load_ref()
    if lib is None:
        raise SystemExit("build oracle/_ref first: make -C oracle/ref")
    return lib


def hi_of(size):
    return I3(*[s - 1 for s in size])


def ref_c2c(x, size, io, oo, direction, scaling, reorder=0):
    lib = ref()
    prec = 0 if x.dtype == np.complex64 else 1
    y = np.empty_like(x)
    assert lib.ref_fft3d_c2c(prec, I3(0, 0, 0), hi_of(size), I3(*io), I3(*oo), reorder, 1, direction, scaling,
                             O._ptr(x), O._ptr(y)) == 0
    return y


def ref_r2c(x, size, rd, io, oo, direction, scaling, reorder=0):
    lib = ref()
    if direction == 0:
        prec = 0 if x.dtype == np.float32 else 1
        y = np.empty(int(np.prod(O.r2c_size(size, rd))), np.complex64 if prec == 0 else np.complex128)
    else:
        prec = 0 if x.dtype == np.complex64 else 1
        y = np.empty(int(np.prod(size)), np.float32 if prec == 0 else np.float64)
    assert lib.ref_fft3d_r2c(prec, I3(0, 0, 0), hi_of(size), I3(*io), I3(*oo), rd, reorder, 1, direction, scaling,
                             O._ptr(x), O._ptr(y)) == 0
    return y


def ref_r2r(kind, x, size, direction, scaling, io=(0, 1, 2), oo=(0, 1, 2)):
    lib = ref()
    prec = 0 if x.dtype == np.float32 else 1
    y = np.empty_like(x)
    assert lib.ref_rtransform(kind, prec, I3(0, 0, 0), hi_of(size), I3(*io), I3(*oo), 1, 1, direction, scaling,
                              O._ptr(x), O._ptr(y)) == 0
    return y


def ref_exec(x, size, order, dim, direction):
    lib = ref()
    prec = 0 if x.dtype == np.complex64 else 1
    y = np.array(x, copy=True)
    assert lib.ref_executor_c2c(prec, I3(0, 0, 0), hi_of(size), I3(*order), dim, direction, O._ptr(y)) == 0
    return y


def known_answers():
    size = (2, 3, 4)
    x = (np.arange(24) + 1).astype(np.float64)
    xc = x.astype(np.complex128)
    out = {"input": x}
    out["c2c_fwd"] = ref_c2c(xc, size, (0, 1, 2), (0, 1, 2), 0, 0)
    for d in range(3):
        out[f"exec_dim{d}"] = ref_exec(xc, size, (0, 1, 2), d, 0)
        out[f"r2c_dir{d}"] = ref_r2c(x, size, d, (0, 1, 2), (0, 1, 2), 0, 0)
    for kind, name in ((0, "cos"), (1, "sin"), (2, "cos1")):
        out[f"{name}_fwd"] = ref_r2r(kind, x, size, 0, 0)
    return out


ORDERS = [((0, 1, 2), (0, 1, 2)), ((2, 1, 0), (0, 1, 2)), ((1, 2, 0), (2, 0, 1))]


def seeded():
    rng = np.random.default_rng(4242)
    out = {}
    cases = []
    for ci, (size, prec) in enumerate([((5, 6, 7), 1), ((8, 9, 10), 0), ((16, 12, 15), 0), ((12, 10, 9), 1)]):
        for oi, (io, oo) in enumerate(ORDERS):
            n = int(np.prod(size))
            x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n))
            x = x.astype(np.complex64 if prec == 0 else np.complex128)
            key = f"c2c_{ci}_{oi}"
            out[key + "_in"] = x
            out[key + "_fwd"] = ref_c2c(x, size, io, oo, 0, 0)
            out[key + "_bwd"] = ref_c2c(out[key + "_fwd"], size, io, oo, 1, 1)
            cases.append(("c2c", key, size, prec, io, oo, -1, -1))
    for ci, (size, prec) in enumerate([((6, 5, 4), 1), ((8, 9, 10), 0), ((7, 6, 5), 0)]):
        for rd in range(3):
            for oi, (io, oo) in enumerate(ORDERS[:2]):
                n = int(np.prod(size))
                x = rng.standard_normal(n).astype(np.float32 if prec == 0 else np.float64)
                key = f"r2c_{ci}_{rd}_{oi}"
                out[key + "_in"] = x
                out[key + "_fwd"] = ref_r2c(x, size, rd, io, oo, 0, 0)
                out[key + "_bwd"] = ref_r2c(out[key + "_fwd"], size, rd, io, oo, 1, 1)
                cases.append(("r2c", key, size, prec, io, oo, rd, -1))
    for kind in range(3):
        for ci, (size, prec) in enumerate([((6, 5, 4), 1), ((8, 7, 9), 0)]):
            n = int(np.prod(size))
            x = rng.standard_normal(n).astype(np.float32 if prec == 0 else np.float64)
            key = f"r2r{kind}_{ci}"
            out[key + "_in"] = x
            out[key + "_fwd"] = ref_r2r(kind, x, size, 0, 0)
            out[key + "_bwd"] = ref_r2r(kind, out[key + "_fwd"], size, 1, 1)
            cases.append(("r2r", key, size, prec, (0, 1, 2), (0, 1, 2), -1, kind))
    meta = np.array([(c[0], c[1], *c[2], c[3], *c[4], *c[5], c[6], c[7]) for c in cases],
                    dtype=[("kind", "U4"), ("key", "U16"), ("n0", "i4"), ("n1", "i4"), ("n2", "i4"), ("prec", "i4"),
                           ("io0", "i4"), ("io1", "i4"), ("io2", "i4"), ("oo0", "i4"), ("oo1", "i4"), ("oo2", "i4"),
                           ("r2c_dir", "i4"), ("r2r_kind", "i4")])
    out["meta"] = meta
    return out


def packers():
    lib = ref()
    rng = np.random.default_rng(7)
    out = {}
    rows = []
    idx = 0
    for esize in (4, 8, 16):
        for mp in [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]:
            size = tuple(int(v) for v in rng.integers(2, 9, 3))
            ls = size[0] + int(rng.integers(0, 3))
            ps = ls * (size[1] + int(rng.integers(0, 3)))
            # the buffer holds the source box: its a-th (fast, mid, slow) dimension is
            # the destination dimension map[a] (transpose_unpacker, src/heffte_backend_cuda.cu:90-133)
            src_dims = [size[mp[a]] for a in range(3)]
            bls = src_dims[0]
            bps = src_dims[0] * src_dims[1]
            nsrc = int(np.prod(src_dims))
            ndst = ps * size[2]
            src = rng.integers(0, 256, nsrc * esize, dtype=np.uint8)
            dst = rng.integers(0, 256, ndst * esize, dtype=np.uint8)
            y = dst.copy()
            assert lib.ref_pack(2, esize, LL3(*size), ls, ps, bls, bps, I3(*mp), O._ptr(src), O._ptr(y)) == 0
            out[f"t{idx}_src"], out[f"t{idx}_dst"], out[f"t{idx}_out"] = src, dst, y
            rows.append(("transpose", idx, esize, *size, ls, ps, bls, bps, *mp))
            idx += 1
        for op in (0, 1):
            size = tuple(int(v) for v in rng.integers(2, 9, 3))
            ls = size[0] + int(rng.integers(0, 4))
            ps = ls * (size[1] + int(rng.integers(0, 4)))
            nbox = ps * size[2]
            nbuf = int(np.prod(size))
            if op == 0:
                src = rng.integers(0, 256, nbox * esize, dtype=np.uint8)
                dst = rng.integers(0, 256, nbuf * esize, dtype=np.uint8)
            else:
                src = rng.integers(0, 256, nbuf * esize, dtype=np.uint8)
                dst = rng.integers(0, 256, nbox * esize, dtype=np.uint8)
            y = dst.copy()
            assert lib.ref_pack(op, esize, LL3(*size), ls, ps, 0, 0, I3(0, 1, 2), O._ptr(src), O._ptr(y)) == 0
            out[f"t{idx}_src"], out[f"t{idx}_dst"], out[f"t{idx}_out"] = src, dst, y
            rows.append(("pack" if op == 0 else "unpack", idx, esize, *size, ls, ps, 0, 0, 0, 1, 2))
            idx += 1
    out["meta"] = np.array(rows, dtype=[("op", "U9"), ("idx", "i4"), ("esize", "i4"), ("n0", "i8"), ("n1", "i8"),
                                        ("n2", "i8"), ("ls", "i8"), ("ps", "i8"), ("bls", "i8"), ("bps", "i8"),
                                        ("m0", "i4"), ("m1", "i4"), ("m2", "i4")])
    return out


def c2c64_input():
    """64^3 complex<double>, re/im i.i.d. uniform [-1, 1) from seed 64."""
    rng = np.random.default_rng(64)
    n = 64 ** 3
    re = rng.uniform(-1, 1, n)
    im = rng.uniform(-1, 1, n)
    return re + 1j * im


def c2c64():
    size = (64, 64, 64)
    x = c2c64_input()
    y = ref_c2c(x, size, (0, 1, 2), (0, 1, 2), 0, 0)
    z = ref_c2c(y, size, (0, 1, 2), (0, 1, 2), 1, 1)
    pos = np.random.default_rng(65).choice(x.size, 4096, replace=False)
    return {"pos": pos, "fwd_sample": y[pos], "fwd_norm": np.array(np.linalg.norm(y)),
            "bwd_sample": z[pos], "roundtrip_err": np.array(np.abs(z - x).max())}


def convolution():
    """The step of benchmarks/convolution.cpp:89-95 run through the reference:
    forward with scale::full, the product X .* X (the benchmark's host loop,
    restated here with numpy), backward unscaled; and the two-input form
    with both forward transforms unscaled and the backward one scale::full."""
    out = {}
    rng = np.random.default_rng(95)
    for tag, size, dt in (("f", (16, 12, 10), np.complex64), ("d", (16, 12, 10), np.complex128),
                          ("d2", (32, 8, 6), np.complex128)):
        n = int(np.prod(size))
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)
        y = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)
        fx = ref_c2c(x, size, (0, 1, 2), (0, 1, 2), 0, 1)
        step = ref_c2c((fx * fx).astype(dt), size, (0, 1, 2), (0, 1, 2), 1, 0)
        gx = ref_c2c(x, size, (0, 1, 2), (0, 1, 2), 0, 0)
        gy = ref_c2c(y, size, (0, 1, 2), (0, 1, 2), 0, 0)
        conv = ref_c2c((gx * gy).astype(dt), size, (0, 1, 2), (0, 1, 2), 1, 1)
        out.update({tag + "_size": np.array(size), tag + "_x": x, tag + "_y": y, tag + "_step": step,
                    tag + "_conv": conv})
    # real data through fft3d_r2c (the product on the half spectrum), r2c
    # along dimension 0 and along dimension 2
    for tag, size, dt, rd in (("rf", (16, 12, 10), np.float32, 0), ("rd", (16, 12, 10), np.float64, 0),
                              ("rd2", (12, 10, 16), np.float64, 2), ("rf3", (16, 16, 16), np.float32, 0),
                              ("rd3", (16, 16, 16), np.float64, 0)):
        n = int(np.prod(size))
        x = rng.standard_normal(n).astype(dt)
        y = rng.standard_normal(n).astype(dt)
        gx = ref_r2c(x, size, rd, (0, 1, 2), (0, 1, 2), 0, 0)
        gy = ref_r2c(y, size, rd, (0, 1, 2), (0, 1, 2), 0, 0)
        conv = ref_r2c((gx * gy).astype(gx.dtype), size, rd, (0, 1, 2), (0, 1, 2), 1, 1)
        out.update({tag + "_size": np.array(size), tag + "_dir": np.array(rd), tag + "_x": x, tag + "_y": y,
                    tag + "_conv": conv})
    return out


FIXTURES = {"known_answers": known_answers, "seeded": seeded, "packers": packers, "c2c64": c2c64,
            "convolution": convolution}


def main():
    names = sys.argv[1:] or list(FIXTURES)
    for name in names:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **FIXTURES[name]())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
