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


def _case(L, rng, dtype, size, mp):
    nf, nm, ns = size
    src_dims = [size[mp[a]] for a in range(3)]
    bls, bps = src_dims[0], src_dims[0] * src_dims[1]
    ls, ps = nf, nf * nm
    es = ESIZE[dtype]
    n = max(int(np.prod(src_dims)), ns * ps)
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
    for dtype, size, mp in [(2, (67, 45, 33), (2, 0, 1)), (3, (40, 28, 19), (1, 2, 0)),
                            (0, (129, 31, 17), (2, 1, 0))]:
        got, want = _case(L, rng, dtype, size, mp)
        assert got.tobytes() == want.tobytes(), (dtype, size, mp)


def test_noalloc_rejects_oversized_source(gb):
    L = _bind(gb.lib())
    t = torch.zeros(16, dtype=torch.float32, device="cuda")
    # 1024^3 complex<float> words = 8 GiB, above the 32 MiB scratch
    rc = L.heffte_gb300_transpose_unpack_inplace_noalloc(None, 2, 1024, 1024, 1024, 1024, 1 << 20, 1024, 1 << 20,
                                                         1, 0, 2, t.data_ptr())
    assert rc == 1
    assert b"MiB scratch" in L.heffte_gb300_last_error()
