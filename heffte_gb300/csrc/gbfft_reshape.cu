// Reshape between two box decompositions of a group of ranks: the device
// side of heFFTe's reshape3d_alltoallv (src/heffte_reshape3d.cpp:365-443,
// built by make_reshape3d_alltoallv, :445-496).
//
// Each rank holds one input box and one output box; the plan of rank `me`
// lists, for every rank r, the overlap of its input box with r's output box
// (what it sends) and the overlap of its output box with r's input box (what
// it receives), as compute_overlap_map_direct_pack / _transpose_pack do
// (src/heffte_reshape3d.cpp:147-233).  pack() copies every outgoing overlap
// into one contiguous send buffer (direct_pack, the input box's order),
// unpack() copies every incoming chunk into the output box, transposing when
// the sender's box order differs (transpose_unpack).  The exchange between
// the two - the reference's MPI_Alltoallv - is the caller's: the send and
// receive counts and displacements are per rank in rank order, so the buffers
// go straight to MPI_Alltoallv, NCCL send / recv or an all-to-all of any other
// library.  One GPU per rank; nothing here touches another rank's memory.
#include "gbfft_plan.h"

namespace gbfft {

namespace {

// box3d::collide (include/heffte_geometry.h): the intersection, in the order of `a`
Box3 collide(Box3 const &a, Box3 const &b){
    std::array<long long, 3> lo, hi;
    for (int d = 0; d < 3; d++){
        lo[d] = std::max(a.lo[d], b.lo[d]);
        hi[d] = std::min(a.hi[d], b.hi[d]);
    }
    return Box3(lo, hi, a.order);
}

// offset of the overlap's first element inside `box` (box order, dense)
long long offset_in(Box3 const &box, Box3 const &overlap){
    return (overlap.lo[box.order[2]] - box.lo[box.order[2]]) * box.osize(0) * box.osize(1) +
           (overlap.lo[box.order[1]] - box.lo[box.order[1]]) * box.osize(0) +
           (overlap.lo[box.order[0]] - box.lo[box.order[0]]);
}

} // namespace

std::unique_ptr<Reshape> make_reshape(int nranks, int me, std::vector<Box3> const &inboxes,
                                      std::vector<Box3> const &outboxes){
    if (nranks < 1 || me < 0 || me >= nranks || (int)inboxes.size() != nranks || (int)outboxes.size() != nranks)
        throw Error(ST_INVALID, "a reshape needs one input and one output box per rank and 0 <= me < nranks");
    for (int r = 0; r < nranks; r++)
        if (!valid_order(inboxes[r].order) || !valid_order(outboxes[r].order))
            throw Error(ST_INVALID, "invalid box order");
    auto R = std::make_unique<Reshape>();
    R->nranks = nranks;
    R->me = me;
    R->inbox = inboxes[me];
    R->outbox = outboxes[me];
    R->send_counts.assign(nranks, 0);
    R->send_displs.assign(nranks, 0);
    R->recv_counts.assign(nranks, 0);
    R->recv_displs.assign(nranks, 0);
    Box3 const &in = R->inbox, &out = R->outbox;
    for (int r = 0; r < nranks; r++){
        if (!in.empty() && !outboxes[r].empty()){
            Box3 ov = collide(in, outboxes[r]);
            if (!ov.empty()){
                Reshape::Chunk c;
                c.rank = r;
                c.box_offset = offset_in(in, ov);
                c.size = {ov.osize(0), ov.osize(1), ov.osize(2)};
                c.line_stride = in.osize(0);
                c.plane_stride = in.osize(0) * in.osize(1);
                R->send.push_back(c);
                R->send_counts[r] = ov.count();
            }
        }
        if (!out.empty() && !inboxes[r].empty()){
            Box3 ov = collide(out, inboxes[r]);
            if (!ov.empty()){
                Reshape::Chunk c;
                c.rank = r;
                c.box_offset = offset_in(out, ov);
                c.size = {ov.osize(0), ov.osize(1), ov.osize(2)};
                c.line_stride = out.osize(0);
                c.plane_stride = out.osize(0) * out.osize(1);
                // the received chunk is the overlap packed in the sender's
                // order: its fast / mid / slow dimensions map to the
                // receiver's as in compute_overlap_map_transpose_pack (:197-222)
                Box3 const &src = inboxes[r];
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++)
                        if (out.order[k] == src.order[j]) c.map[j] = k;
                c.buff_line_stride = ov.size[src.order[0]];
                c.buff_plane_stride = ov.size[src.order[0]] * ov.size[src.order[1]];
                R->recv.push_back(c);
                R->recv_counts[r] = ov.count();
            }
        }
    }
    long long s = 0, q = 0;
    for (int r = 0; r < nranks; r++){
        R->send_displs[r] = s; s += R->send_counts[r];
        R->recv_displs[r] = q; q += R->recv_counts[r];
    }
    R->send_total = s;
    R->recv_total = q;
    return R;
}

void Reshape::pack(cudaStream_t st, int dtype, void const *input, void *send_buffer) const{
    size_t es = elem_size(dtype);
    for (auto const &c : send){
        void const *src = static_cast<char const*>(input) + (size_t)c.box_offset * es;
        void *dst = static_cast<char*>(send_buffer) + (size_t)send_displs[c.rank] * es;
        launch_direct_pack(st, dtype, c.size[0], c.size[1], c.size[2], c.line_stride, c.plane_stride, src, dst, true);
    }
}

void Reshape::unpack(cudaStream_t st, int dtype, void const *recv_buffer, void *output) const{
    size_t es = elem_size(dtype);
    for (auto const &c : recv){
        void const *src = static_cast<char const*>(recv_buffer) + (size_t)recv_displs[c.rank] * es;
        void *dst = static_cast<char*>(output) + (size_t)c.box_offset * es;
        if (c.map[0] == 0 && c.map[1] == 1)
            launch_direct_pack(st, dtype, c.size[0], c.size[1], c.size[2], c.line_stride, c.plane_stride, src, dst, false);
        else
            launch_transpose_unpack(st, dtype, c.size[0], c.size[1], c.size[2], c.line_stride, c.plane_stride,
                                    c.buff_line_stride, c.buff_plane_stride, c.map[0], c.map[1], src, dst);
    }
}

} // namespace gbfft
