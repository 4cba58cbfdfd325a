// Instantiation of the batched transform kernels for one precision.
// Included by gbfft_fft_f32.cu (GB_T = float) and gbfft_fft_f64.cu (GB_T = double)
// so that the two precisions compile in parallel.
#include "gbfft_internal.h"
#include "gbfft_kernels.cuh"
#include <atomic>

namespace gbfft {

namespace {

// Opt every instantiation into the full shared-memory carve-out, once per
// device (the attribute is per device context).
template<auto Kfn>
void prepare(){
    static std::atomic<unsigned long long> mask{0};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    unsigned long long bit = 1ull << (dev & 63);
    if (!(mask.load() & bit)){
        check_cuda(cudaFuncSetAttribute(Kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024),
                   "cudaFuncSetAttribute(max dynamic shared memory)");
        mask.fetch_or(bit);
    }
}

template<bool COLS>
void dispatch(cudaStream_t s, int kind, KernelArgs const &a){
    using T = GB_T;
    using C = c_t<T>;
    dim3 grid((unsigned)a.blocks), block((unsigned)a.threads);
    T sc = (T)a.scale;
    switch (kind){
        case K_C2C_F: {
            auto k = k_c2c<T, kEmax, true, COLS>; prepare<k_c2c<T, kEmax, true, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (C const*)a.in, (C*)a.out, (C const*)a.tw, a.G, a.tpb, sc, a.do_scale);
            break;
        }
        case K_C2C_B: {
            auto k = k_c2c<T, kEmax, false, COLS>; prepare<k_c2c<T, kEmax, false, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (C const*)a.in, (C*)a.out, (C const*)a.tw, a.G, a.tpb, sc, a.do_scale);
            break;
        }
        case K_R2C: {
            auto k = k_r2c<T, kEmax, COLS>; prepare<k_r2c<T, kEmax, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (T const*)a.in, (C*)a.out, (C const*)a.tw, a.G, a.tpb, sc, a.do_scale);
            break;
        }
        case K_C2R: {
            auto k = k_c2r<T, kEmax, COLS>; prepare<k_c2r<T, kEmax, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (C const*)a.in, (T*)a.out, (C const*)a.tw, a.G, a.tpb, sc, a.do_scale);
            break;
        }
        case K_R2R_F: {
            auto k = k_r2r<T, kEmax, true, COLS>; prepare<k_r2r<T, kEmax, true, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (T const*)a.in, (T*)a.out, (C const*)a.tw, (C const*)a.rtw,
                                          a.G, a.tpb, a.sine, sc, a.do_scale);
            break;
        }
        case K_R2R_B: {
            auto k = k_r2r<T, kEmax, false, COLS>; prepare<k_r2r<T, kEmax, false, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.Li, a.Lo, (T const*)a.in, (T*)a.out, (C const*)a.tw, (C const*)a.rtw,
                                          a.G, a.tpb, a.sine, sc, a.do_scale);
            break;
        }
        case K_DCT1: {
            auto k = k_dct1<T, kEmax, COLS>; prepare<k_dct1<T, kEmax, COLS>>();
            k<<<grid, block, a.smem, s>>>(*a.plan, a.ndata, a.Li, a.Lo, (T const*)a.in, (T*)a.out, (C const*)a.tw,
                                          a.G, a.tpb, sc, a.do_scale);
            break;
        }
        default: throw Error(ST_INVALID, "unknown kernel kind");
    }
    check_cuda(cudaPeekAtLastError(), "fft kernel launch");
}

} // namespace

void GB_LAUNCH_NAME(cudaStream_t s, int kind, bool cols, KernelArgs const &a){
    if (cols) dispatch<true>(s, kind, a); else dispatch<false>(s, kind, a);
}

} // namespace gbfft
