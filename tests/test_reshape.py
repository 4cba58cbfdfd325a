"""Reshapes between the box decompositions of a group of ranks (the device side
of reshape3d_alltoallv, src/heffte_reshape3d.cpp:365-496) and the distributed
fft3d over them (heffte_gb300.distributed: the slab decomposition of
plan_slab_reshapes, src/heffte_plan_logic.cpp:273-422).

CPU (no GPU): the plan's per-rank counts against the oracle's overlap maps,
and the exchange protocol on a world-size-2 gloo group (the oracle packs and
unpacks on the host with the plan's counts).  GPU: pack / unpack of every
rank of a 4-rank group, bit-exact against the global array; the distributed
fft3d on two gloo ranks sharing the GPU (host-staged all-to-all) against the
FP64 oracle.  Unmeasured on more than one GPU: every call here uses one.
"""
import os
import socket

import numpy as np
import pytest

from oracle import heffte_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORLD = (12, 10, 9)
# four ranks: input pencils along dimension 0 (order 0,1,2), output pencils
# along dimension 2 in another order, so every chunk crosses a transpose
INBOXES = [((0, 0, 0), (11, 4, 4), (0, 1, 2)), ((0, 5, 0), (11, 9, 4), (0, 1, 2)),
           ((0, 0, 5), (11, 4, 8), (0, 1, 2)), ((0, 5, 5), (11, 9, 8), (0, 1, 2))]
OUTBOXES = [((0, 0, 0), (5, 4, 8), (2, 0, 1)), ((6, 0, 0), (11, 4, 8), (2, 1, 0)),
            ((0, 5, 0), (5, 9, 8), (1, 2, 0)), ((6, 5, 0), (11, 9, 8), (2, 0, 1))]


def _box(gb, b):
    return gb.box3d(b[0], b[1], b[2])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reshape_counts_match_the_overlap_maps(gb):
    for me in range(4):
        r = gb.reshape3d([_box(gb, b) for b in INBOXES], [_box(gb, b) for b in OUTBOXES], me)
        sc, sd, rc, rd = r.counts()
        osend, orecv = O.reshape_counts(me, INBOXES, OUTBOXES)
        assert sc == osend and rc == orecv
        assert sd == list(np.cumsum([0] + sc[:-1])) and rd == list(np.cumsum([0] + rc[:-1]))
        assert r.send_size() == O.box_count(INBOXES[me]) and r.recv_size() == O.box_count(OUTBOXES[me])
    # a rank whose boxes match moves everything to itself
    same = [_box(gb, b) for b in INBOXES]
    r = gb.reshape3d(same, same, 2)
    assert r.counts()[0] == [0, 0, O.box_count(INBOXES[2]), 0]
    with pytest.raises(gb.HeffteError):
        gb.reshape3d(same, same, 4)


def _gloo_exchange_worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import heffte_gb300 as gb
    from oracle import heffte_oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    inb = [((0, 0, 0), (6, 5, 1), (0, 1, 2)), ((0, 0, 2), (6, 5, 4), (2, 0, 1))]
    outb = [((0, 0, 0), (3, 5, 4), (1, 2, 0)), ((4, 0, 0), (6, 5, 4), (0, 2, 1))]
    g = np.random.default_rng(3).standard_normal((5, 6, 7))        # world 7 x 6 x 5, [k][j][i]
    plan = gb.reshape3d([gb.box3d(*b) for b in inb], [gb.box3d(*b) for b in outb], rank)
    sc, sd, rc, rd = plan.counts()
    send = torch.from_numpy(O.reshape_pack(rank, inb, outb, O.box_slice(g, inb[rank])))
    recv = torch.empty(plan.recv_size(), dtype=send.dtype)
    dist.all_to_all_single(recv, send, rc, sc)
    got = O.reshape_unpack(rank, inb, outb, recv.numpy(), np.zeros(plan.recv_size()))
    out[rank] = bool(np.array_equal(got, O.box_slice(g, outb[rank])))
    dist.destroy_process_group()


def test_reshape_exchange_on_two_gloo_ranks():
    """The plan's counts drive a world-size-2 all-to-all (gloo, CPU); the
    buffers packed and unpacked by the oracle in the plan's layout rebuild
    every output box exactly."""
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_gloo_exchange_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(180)
            assert p.exitcode == 0
        assert dict(out) == {0: True, 1: True}


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,npdt", [(0, np.float32), (2, np.complex64), (3, np.complex128)])
def test_reshape_pack_unpack_bit_exact(gb, dtype, npdt):
    """Every rank of the 4-rank group packs on the GPU, the chunks are
    exchanged on the host, every rank unpacks on the GPU: each output box is
    the global array's values, bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(dtype)
    g = rng.standard_normal((WORLD[2], WORLD[1], WORLD[0]))
    if np.iscomplexobj(npdt(0)):
        g = g + 1j * rng.standard_normal(g.shape)
    g = g.astype(npdt)
    plans = [gb.reshape3d([_box(gb, b) for b in INBOXES], [_box(gb, b) for b in OUTBOXES], me) for me in range(4)]
    sends = []
    for me in range(4):
        x = torch.from_numpy(O.box_slice(g, INBOXES[me])).cuda()
        s = torch.empty(plans[me].send_size(), dtype=x.dtype, device="cuda")
        plans[me].pack(dtype, x, s)
        torch.cuda.synchronize()
        sends.append(s.cpu().numpy())
        # the device packing equals the oracle's
        assert sends[-1].tobytes() == O.reshape_pack(me, INBOXES, OUTBOXES, x.cpu().numpy()).tobytes()
    for me in range(4):
        cnt = [plans[r].counts() for r in range(4)]
        recv = np.concatenate([sends[r][cnt[r][1][me]:cnt[r][1][me] + cnt[r][0][me]] for r in range(4)])
        y = torch.zeros(O.box_count(OUTBOXES[me]), dtype=torch.from_numpy(recv).dtype, device="cuda")
        plans[me].unpack(dtype, torch.from_numpy(recv).cuda(), y)
        torch.cuda.synchronize()
        assert y.cpu().numpy().tobytes() == O.box_slice(g, OUTBOXES[me]).tobytes(), me


def _dist_fft_worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import heffte_gb300 as gb
    from heffte_gb300 import distributed as D
    from oracle import heffte_oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    size = (24, 20, 18)
    rng = np.random.default_rng(41)
    g = rng.uniform(-1, 1, size[::-1]) + 1j * rng.uniform(-1, 1, size[::-1])
    # input pencils split along dimension 1, output split along dimension 0 in another order
    inb = [((0, 0, 0), (23, 9, 17), (0, 1, 2)), ((0, 10, 0), (23, 19, 17), (0, 1, 2))]
    outb = [((0, 0, 0), (11, 19, 17), (2, 1, 0)), ((12, 0, 0), (23, 19, 17), (2, 1, 0))]
    ref = O.fft3d_c2c(O.from_canonical(g, (0, 1, 2)), size)
    G = O.to_canonical(ref, size, (0, 1, 2))
    res = {}
    for prec in (0, 1):
        cdt = torch.complex64 if prec == 0 else torch.complex128
        f = D.fft3d(gb.box3d(*inb[rank]), gb.box3d(*outb[rank]), prec=prec)
        x = torch.from_numpy(O.box_slice(g, inb[rank])).to(cdt).cuda()
        x0 = x.clone()
        y = torch.empty(f.size_outbox(), dtype=cdt, device="cuda")
        f.forward(x, y)
        e_f = O.rel_l2(y.cpu().numpy(), O.box_slice(G, outb[rank]))
        z = torch.empty_like(x)
        f.backward(y, z, gb.scale.full)
        e_b = O.rel_l2(z.cpu().numpy(), x0.cpu().numpy())
        res[prec] = (e_f, e_b, bool(torch.equal(x, x0)))
    out[rank] = res
    dist.destroy_process_group()


@pytest.mark.gpu
def test_distributed_fft3d_on_two_ranks(gb, report):
    """Two ranks (processes on the one GPU, gloo, host-staged all-to-all):
    forward against the FP64 oracle's transform restricted to each rank's
    output box, backward (scale::full) back to the input."""
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_dist_fft_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        res = dict(out)
    tol = {0: 1e-6, 1: 1e-12}
    for rank in range(2):
        for prec in (0, 1):
            e_f, e_b, kept = res[rank][prec]
            assert e_f < tol[prec] and e_b < tol[prec] and kept, (rank, prec, e_f, e_b)
    report.append("distributed fft3d, 2 ranks: forward rel-L2 float "
                  f"{max(res[r][0][0] for r in range(2)):.2e}, double {max(res[r][1][0] for r in range(2)):.2e}")
