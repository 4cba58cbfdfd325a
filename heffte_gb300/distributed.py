"""heffte::fft3d on a group of ranks, one GPU per rank.

The multi-rank path of the reference: fft3d on a communicator of several
ranks plans reshapes between box decompositions (include/heffte_fft3d.h:599-651)
and moves data with reshape3d_alltoallv (src/heffte_reshape3d.cpp:365-443).
Here the decomposition is heFFTe's slab one (plan_slab_reshapes,
src/heffte_plan_logic.cpp:273-422, use_pencils = false):

  input boxes --reshape--> slabs split along dimension 2 (2-D executor over
  dimensions 0 and 1) --reshape--> slabs split along dimension 1 (1-D
  executor over dimension 2) --reshape--> output boxes

and backward the same in reverse.  Packing and unpacking run on the device
(heffte_gb300.reshape3d); the exchange between them is an all-to-all over a
torch.distributed process group: on device buffers when the group's backend
is NCCL, staged through host memory otherwise (gloo).  A reshape whose boxes
already match skips the exchange.
"""
from __future__ import annotations

import heffte_gb300 as gb

_DTYPE_CODE = {"complex64": 2, "complex128": 3}


def split_world(world, dim, nranks):
    """The world box cut along `dim` into nranks contiguous slabs whose
    extents differ by at most one (the larger ones first)."""
    n = world.size[dim]
    base, extra = divmod(n, nranks)
    boxes, lo = [], world.low[dim]
    for r in range(nranks):
        ext = base + (1 if r < extra else 0)
        low, high = list(world.low), list(world.high)
        low[dim], high[dim] = lo, lo + ext - 1
        boxes.append(gb.box3d(low, high, world.order))
        lo += ext
    return boxes


def _same(a, b):
    return a.low == b.low and a.high == b.high and a.order == b.order


class fft3d:
    """Distributed complex-to-complex fft3d: every rank passes its own input
    and output boxes (the union of the input boxes and of the output boxes is
    the same world box) and its process group; arrays are this rank's device
    tensors of its boxes.  prec 0 = complex<float>, 1 = complex<double>."""

    def __init__(self, inbox, outbox, group=None, prec=0):
        import torch
        import torch.distributed as dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.nranks = dist.get_world_size(group)
        self.prec = prec
        self.dtype = torch.complex64 if prec == 0 else torch.complex128
        self.code = _DTYPE_CODE[str(self.dtype).split(".")[-1]]
        # mpi::gather_boxes (include/heffte_geometry.h:707-718)
        mine = (inbox.low, inbox.high, inbox.order, outbox.low, outbox.high, outbox.order)
        every = [None] * self.nranks
        dist.all_gather_object(every, mine, group=group)
        self.inboxes = [gb.box3d(e[0], e[1], e[2]) for e in every]
        self.outboxes = [gb.box3d(e[3], e[4], e[5]) for e in every]
        lo = [min(b.low[d] for b in self.inboxes) for d in range(3)]
        hi = [max(b.high[d] for b in self.inboxes) for d in range(3)]
        self.world = gb.box3d(lo, hi)
        total = sum(b.count() for b in self.inboxes)
        if total != self.world.count() or sum(b.count() for b in self.outboxes) != self.world.count():
            raise gb.heffte_input_error("the input (and output) boxes of the ranks must tile the world box")
        self.slabs_a = split_world(self.world, 2, self.nranks)
        self.slabs_b = split_world(self.world, 1, self.nranks)
        a, b = self.slabs_a[self.rank], self.slabs_b[self.rank]
        self.box_a, self.box_b = a, b
        mk = lambda src, dst: None if all(_same(x, y) for x, y in zip(src, dst)) else gb.reshape3d(src, dst, self.rank)
        self.fwd_reshapes = [mk(self.inboxes, self.slabs_a), mk(self.slabs_a, self.slabs_b),
                             mk(self.slabs_b, self.outboxes)]
        self.bwd_reshapes = [mk(self.outboxes, self.slabs_b), mk(self.slabs_b, self.slabs_a),
                             mk(self.slabs_a, self.inboxes)]
        self.ex_a = gb.executor(gb.kind.c2c, a, [0, 1]) if a.count() > 0 else None
        self.ex_b = gb.executor(gb.kind.c2c, b, [2]) if b.count() > 0 else None
        self.nccl = dist.get_backend(group) == "nccl"

    def size_inbox(self):
        return self.inboxes[self.rank].count()

    def size_outbox(self):
        return self.outboxes[self.rank].count()

    def _exchange(self, r, send):
        """The reference's MPI_Alltoallv between the packed buffers."""
        import torch
        import torch.distributed as dist
        sc, _, rc, _ = r.counts()
        recv = torch.empty(max(r.recv_size(), 1), dtype=self.dtype, device="cuda")
        if self.nccl:
            dist.all_to_all_single(recv[:r.recv_size()], send[:r.send_size()], rc, sc, group=self.group)
            return recv
        # host staging: complex values as pairs of reals
        torch.cuda.current_stream().synchronize()
        hs = torch.view_as_real(send[:r.send_size()].cpu()).reshape(-1)
        hr = torch.empty(2 * r.recv_size(), dtype=hs.dtype)
        dist.all_to_all_single(hr, hs, [2 * c for c in rc], [2 * c for c in sc], group=self.group)
        recv[:r.recv_size()].copy_(torch.view_as_complex(hr.reshape(-1, 2)))
        return recv

    def _reshape(self, r, src, dst_count, out=None):
        import torch
        if r is None:
            if out is not None and out.data_ptr() != src.data_ptr():
                out.copy_(src[:dst_count])
                return out
            return src
        send = torch.empty(max(r.send_size(), 1), dtype=self.dtype, device="cuda")
        r.pack(self.code, src, send)
        recv = self._exchange(r, send)
        dst = out if out is not None else torch.empty(max(dst_count, 1), dtype=self.dtype, device="cuda")
        r.unpack(self.code, recv, dst)
        return dst

    def _run(self, forward, x, y, scaling):
        import torch
        rs = self.fwd_reshapes if forward else self.bwd_reshapes
        first, second = (self.box_a, self.box_b) if forward else (self.box_b, self.box_a)
        ex1, ex2 = (self.ex_a, self.ex_b) if forward else (self.ex_b, self.ex_a)
        t = self._reshape(rs[0], x, first.count())
        if t is x:
            t = x.clone()       # the input is never modified
        if ex1 is not None:
            (ex1.forward if forward else ex1.backward)(self.prec, t, t)
        t = self._reshape(rs[1], t, second.count())
        if ex2 is not None:
            (ex2.forward if forward else ex2.backward)(self.prec, t, t)
        out = self._reshape(rs[2], t, y.numel(), out=y)
        if scaling != gb.scale.none and y.numel() > 0:
            n = self.world.count()
            f = 1.0 / n if scaling == gb.scale.full else n ** -0.5
            gb.scale_data(self.prec, 2 * y.numel(), y, f)
        del out
        torch.cuda.current_stream().synchronize()

    def forward(self, x, y, scaling=gb.scale.none):
        self._run(True, x, y, scaling)

    def backward(self, x, y, scaling=gb.scale.none):
        self._run(False, x, y, scaling)
