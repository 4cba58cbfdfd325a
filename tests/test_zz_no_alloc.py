"""The in-place transpose entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (device memory owned by an
arena, real-time loops that must not allocate after start-up, callers at the
memory limit).  Its output must equal the allocating path: the ordinary
transpose_unpack entry point reading from a separate copy of the source.
The case runs two calls in a row, so that the scratch array the entry point
reuses between calls cannot leak one call's data into the next.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ESIZE = {0: 4, 1: 8, 2: 8, 3: 16}


def _bind(L):
    vp, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
    L.heffte_gb300_transpose_unpack_inplace_noalloc.argtypes = [vp, i, ll, ll, ll, ll, ll, ll, ll, i, i, i, vp]
    L.heffte_gb300_transpose_unpack.argtypes = [vp, i, ll, ll, ll, ll, ll, ll, ll, i, i, i, vp, vp]
    L.heffte_gb300_last_error.restype = ctypes.c_char_p
    return L


def _case(L, rng, dtype, size, mp, pad=(0, 0)):
    """pad = extra elements per source line and per source plane (a padded
    buffer layout, whose span differs from its element count)."""
    nf, nm, ns = size
    src_dims = [size[mp[a]] for a in range(3)]
    bls = src_dims[0] + pad[0]
    bps = bls * src_dims[1] + pad[1]
    ls, ps = nf, nf * nm
    es = ESIZE[dtype]
    src_span = (src_dims[2] - 1) * bps + (src_dims[1] - 1) * bls + src_dims[0]
    n = max(src_span, ns * ps)
    host = rng.integers(0, 256, n * es, dtype=np.uint8)
    data = torch.from_numpy(host).cuda()
    src_copy = data.clone()
    expected = data.clone()
    # the allocating path: separate source buffer
    assert L.heffte_gb300_transpose_unpack(None, dtype, nf, nm, ns, ls, ps, bls, bps, mp[0], mp[1], mp[2],
                                           src_copy.data_ptr(), expected.data_ptr()) == 0
    # the no-allocation path: in place
    assert L.heffte_gb300_transpose_unpack_inplace_noalloc(None, dtype, nf, nm, ns, ls, ps, bls, bps,
                                                           mp[0], mp[1], mp[2], data.data_ptr()) == 0, \
        L.heffte_gb300_last_error()
    torch.cuda.synchronize()
    return data.cpu().numpy(), expected.cpu().numpy()


def test_noalloc_inplace_transpose_matches_allocating_path(gb):
    L = _bind(gb.lib())
    rng = np.random.default_rng(2024)
    # two calls in a row, different shapes, maps and element types
    for dtype, size, mp, pad in [(2, (67, 45, 33), (2, 0, 1), (0, 0)), (3, (40, 28, 19), (1, 2, 0), (0, 0)),
                                 (0, (129, 31, 17), (2, 1, 0), (0, 0)),
                                 # map0 == 0: the row-copy branch (source rows stay rows)
                                 (1, (70, 23, 41), (0, 2, 1), (0, 0)),
                                 # padded source lines and planes
                                 (2, (37, 52, 29), (1, 0, 2), (5, 17)), (3, (33, 18, 27), (0, 2, 1), (3, 0))]:
        got, want = _case(L, rng, dtype, size, mp, pad)
        assert got.tobytes() == want.tobytes(), (dtype, size, mp, pad)


def test_noalloc_rejects_oversized_source(gb):
    L = _bind(gb.lib())
    t = torch.zeros(16, dtype=torch.float32, device="cuda")
    # 1024^3 complex<float> words = 8 GiB, above the 32 MiB scratch
    rc = L.heffte_gb300_transpose_unpack_inplace_noalloc(None, 2, 1024, 1024, 1024, 1024, 1 << 20, 1024, 1 << 20,
                                                         1, 0, 2, t.data_ptr())
    assert rc == 1
    assert b"MiB scratch" in L.heffte_gb300_last_error()


def test_noalloc_rejects_inconsistent_strides(gb):
    """Negative, overlapping or overflowing strides are refused before any copy
    (a wrapped span could otherwise pass the scratch-size check)."""
    L = _bind(gb.lib())
    t = torch.zeros(64, dtype=torch.float32, device="cuda")
    bad = [
        (8, 4, 2, 8, 32, -8, 32),           # negative source line stride
        (8, 4, 2, 8, 32, 8, -32),           # negative source plane stride
        (8, 4, 2, 8, 32, 3, 32),            # source lines overlap
        (8, 4, 2, 4, 32, 8, 32),            # destination lines overlap
        (8, 4, 3, 8, 32, 8, 1 << 62),       # span (2 x 2^62 + ...) overflows 63 bits
    ]
    for nf, nm, ns, ls, ps, bls, bps in bad:
        rc = L.heffte_gb300_transpose_unpack_inplace_noalloc(None, 0, nf, nm, ns, ls, ps, bls, bps, 0, 1, 2,
                                                             t.data_ptr())
        assert rc == 1, (nf, nm, ns, ls, ps, bls, bps)
        assert b"layout" in L.heffte_gb300_last_error()
