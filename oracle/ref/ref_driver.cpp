/*
 * Thin extern "C" driver over the heFFTe reference's own stock backend.
 * Test infrastructure: compiled from the reference sources where they lie
 * (include paths only, nothing copied) into oracle/_ref/libheffte_ref.so, and
 * used to pin the CPU oracles and to generate golden fixtures.
 *
 * Every entry point runs the reference's public API:
 *   heffte::fft3d<backend::stock>      include/heffte_fft3d.h:239-692
 *   heffte::fft3d_r2c<backend::stock>  include/heffte_fft3d_r2c.h:45-380
 *   heffte::rtransform<stock_cos|sin|cos1> include/heffte_fft3d.h:748-749
 *   direct_packer/transpose_packer<tag::cpu>, data_scaling::apply
 *                                      include/heffte_pack3d.h:83-233
 * on a single rank (the MPI stand-in in this directory has one process).
 */
#include "heffte.h"
#include <chrono>
#include <random>

using namespace heffte;

namespace {

box3d<int> make_box(const int lo[3], const int hi[3], const int order[3]){
    return box3d<int>({lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}, {order[0], order[1], order[2]});
}

scale to_scale(int s){
    return (s == 1) ? scale::full : ((s == 2) ? scale::symmetric : scale::none);
}

plan_options make_options(int use_reorder, int use_pencils){
    plan_options opts = default_options<backend::stock>();
    opts.use_reorder = (use_reorder != 0);
    opts.use_pencils = (use_pencils != 0);
    return opts;
}

template<typename T>
int guarded(T &&fn){
    try{ fn(); return 0; }
    catch(std::exception const &e){ fprintf(stderr, "heffte reference: %s\n", e.what()); return 1; }
}

} // namespace

/* Pack / unpack / transpose-unpack through the reference CPU packers.
 * esize selects the element type: 4 float, 8 double or complex<float>
 * (moved as one 8-byte unit), 16 complex<double>. */
template<typename T>
static void pack_impl(int op, const long long size[3], long long ls, long long ps, long long bls, long long bps,
                      const int map[3], const void *src, void *dst){
    pack_plan_3d<long long> plan{{size[0], size[1], size[2]}, ls, ps, bls, bps, {map[0], map[1], map[2]}};
    auto *s = reinterpret_cast<T const*>(src);
    auto *d = reinterpret_cast<T*>(dst);
    if (op == 0) direct_packer<tag::cpu>().pack(nullptr, plan, s, d);
    else if (op == 1) direct_packer<tag::cpu>().unpack(nullptr, plan, s, d);
    else transpose_packer<tag::cpu>().unpack(nullptr, plan, s, d);
}

extern "C" {

/* 3-D complex-to-complex transform; prec 0 = complex<float>, 1 = complex<double>;
 * direction 0 = forward, 1 = backward. */
int ref_fft3d_c2c(int prec, const int lo[3], const int hi[3], const int in_order[3], const int out_order[3],
                  int use_reorder, int use_pencils, int direction, int scaling, const void *in, void *out){
    return guarded([&]{
        fft3d<backend::stock> fft(make_box(lo, hi, in_order), make_box(lo, hi, out_order), MPI_COMM_SELF,
                                  make_options(use_reorder, use_pencils));
        if (prec == 0){
            auto *i = reinterpret_cast<std::complex<float> const*>(in);
            auto *o = reinterpret_cast<std::complex<float>*>(out);
            if (direction == 0) fft.forward(i, o, to_scale(scaling)); else fft.backward(i, o, to_scale(scaling));
        }else{
            auto *i = reinterpret_cast<std::complex<double> const*>(in);
            auto *o = reinterpret_cast<std::complex<double>*>(out);
            if (direction == 0) fft.forward(i, o, to_scale(scaling)); else fft.backward(i, o, to_scale(scaling));
        }
    });
}

/* Sizes of the r2c in/out boxes (the outbox is the r2c-reduced world box). */
long long ref_r2c_outbox_count(const int lo[3], const int hi[3], int r2c_direction){
    box3d<int> b({lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]});
    return b.r2c(r2c_direction).count();
}

/* 3-D real-to-complex (direction 0) / complex-to-real (direction 1). The
 * outbox is world.r2c(r2c_direction), with its own order. */
int ref_fft3d_r2c(int prec, const int lo[3], const int hi[3], const int in_order[3], const int out_order[3],
                  int r2c_direction, int use_reorder, int use_pencils, int direction, int scaling,
                  const void *in, void *out){
    return guarded([&]{
        box3d<int> world = make_box(lo, hi, in_order);
        box3d<int> cbox  = world.r2c(r2c_direction);
        box3d<int> outbox(cbox.low, cbox.high, {out_order[0], out_order[1], out_order[2]});
        fft3d_r2c<backend::stock> fft(world, outbox, r2c_direction, MPI_COMM_SELF,
                                      make_options(use_reorder, use_pencils));
        if (prec == 0){
            if (direction == 0) fft.forward(reinterpret_cast<float const*>(in), reinterpret_cast<std::complex<float>*>(out), to_scale(scaling));
            else fft.backward(reinterpret_cast<std::complex<float> const*>(in), reinterpret_cast<float*>(out), to_scale(scaling));
        }else{
            if (direction == 0) fft.forward(reinterpret_cast<double const*>(in), reinterpret_cast<std::complex<double>*>(out), to_scale(scaling));
            else fft.backward(reinterpret_cast<std::complex<double> const*>(in), reinterpret_cast<double*>(out), to_scale(scaling));
        }
    });
}

/* 3-D real-to-real transform; kind 0 = cos (DCT-II/III), 1 = sin (DST-II/III), 2 = cos1 (DCT-I). */
int ref_rtransform(int kind, int prec, const int lo[3], const int hi[3], const int in_order[3], const int out_order[3],
                   int use_reorder, int use_pencils, int direction, int scaling, const void *in, void *out){
    auto run = [&](auto &fft){
        if (prec == 0){
            if (direction == 0) fft.forward(reinterpret_cast<float const*>(in), reinterpret_cast<float*>(out), to_scale(scaling));
            else fft.backward(reinterpret_cast<float const*>(in), reinterpret_cast<float*>(out), to_scale(scaling));
        }else{
            if (direction == 0) fft.forward(reinterpret_cast<double const*>(in), reinterpret_cast<double*>(out), to_scale(scaling));
            else fft.backward(reinterpret_cast<double const*>(in), reinterpret_cast<double*>(out), to_scale(scaling));
        }
    };
    return guarded([&]{
        box3d<int> ib = make_box(lo, hi, in_order), ob = make_box(lo, hi, out_order);
        plan_options opts = make_options(use_reorder, use_pencils);
        if (kind == 0){ rtransform<backend::stock_cos> f(ib, ob, MPI_COMM_SELF, opts); run(f); }
        else if (kind == 1){ rtransform<backend::stock_sin> f(ib, ob, MPI_COMM_SELF, opts); run(f); }
        else { rtransform<backend::stock_cos1> f(ib, ob, MPI_COMM_SELF, opts); run(f); }
    });
}

/* One batch of 1-D transforms along `dimension` of a box, through the stock
 * executor (the executor role the GPU backend replaces). */
int ref_executor_c2c(int prec, const int lo[3], const int hi[3], const int order[3], int dimension,
                     int direction, void *data){
    return guarded([&]{
        stock_fft_executor ex(nullptr, make_box(lo, hi, order), dimension);
        if (prec == 0){
            auto *d = reinterpret_cast<std::complex<float>*>(data);
            if (direction == 0) ex.forward(d, nullptr); else ex.backward(d, nullptr);
        }else{
            auto *d = reinterpret_cast<std::complex<double>*>(data);
            if (direction == 0) ex.forward(d, nullptr); else ex.backward(d, nullptr);
        }
    });
}

int ref_pack(int op, int esize, const long long size[3], long long line_stride, long long plane_stride,
             long long buff_line_stride, long long buff_plane_stride, const int map[3], const void *src, void *dst){
    return guarded([&]{
        if (esize == 4) pack_impl<float>(op, size, line_stride, plane_stride, buff_line_stride, buff_plane_stride, map, src, dst);
        else if (esize == 8) pack_impl<double>(op, size, line_stride, plane_stride, buff_line_stride, buff_plane_stride, map, src, dst);
        else pack_impl<std::complex<double>>(op, size, line_stride, plane_stride, buff_line_stride, buff_plane_stride, map, src, dst);
    });
}

/* data_scaling::apply on prec 0 float / 1 double reals, complex as 2n reals. */
int ref_scale(int prec, long long n, void *data, double factor){
    return guarded([&]{
        if (prec == 0) data_scaling::apply(nullptr, n, reinterpret_cast<float*>(data), factor);
        else data_scaling::apply(nullptr, n, reinterpret_cast<double*>(data), factor);
    });
}

} // extern "C"
