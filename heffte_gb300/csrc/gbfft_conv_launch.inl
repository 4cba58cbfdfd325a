// Host dispatch of the fused convolution pass (gbfft_conv.cuh) for one
// precision.  Included by gbfft_conv_f32.cu / gbfft_conv_f64.cu with
//   GB_T          float or double
//   GB_CONV_NAME  the exported dispatcher
#include "gbfft_internal.h"
#include "gbfft_conv.cuh"
#include <atomic>
#include <cstring>

namespace gbfft {

namespace {

template<int N, bool TWO>
bool run_conv(cudaStream_t s, ConvLaunch const &a, bool dry_run){
    using T = GB_T;
    using C = c_t<T>;
    constexpr int SMEM = conv_smem(N, (int)sizeof(C), TWO);
    if constexpr (SMEM > 227 * 1024){
        return false;   // (complex<double> of 4096 points with two operands)
    } else {
        constexpr int TPB = conv_tpb(N, (int)sizeof(C), TWO);
        constexpr int THREADS = conv_threads(N, (int)sizeof(C), TWO);
        Layout const &L = a.L;
        if (a.G <= 0) return true;
        if (L.dist != 1 || a.G % L.count != 0) return false;
        if ((reinterpret_cast<uintptr_t>(a.x) & 15) || (TWO && (reinterpret_cast<uintptr_t>(a.y) & 15)) ||
            (TPB * sizeof(C)) % 16 != 0)
            return false;
        long long blocks = a.G / L.count;
        CUtensorMap tmx, tmy;
        std::memset(&tmx, 0, sizeof(tmx));
        std::memset(&tmy, 0, sizeof(tmy));
        int swap = 0, swap_y = 0;
        int boxr = N < 256 ? N : 256;
        if (!encode_column_tmap(&tmx, a.x, (int)sizeof(C), L.count, N, blocks, L.estride, L.bstride, TPB, boxr, &swap))
            return false;
        if (TWO){
            if (!encode_column_tmap(&tmy, a.y, (int)sizeof(C), L.count, N, blocks, L.estride, L.bstride, TPB, boxr,
                                    &swap_y) || swap_y != swap)
                return false;
        } else {
            tmy = tmx;
        }
        if (dry_run) return true;
        auto kern = k_conv_cols<T, N, TWO>;
        static std::atomic<unsigned long long> ready{0};
        static int blocks_per_sm[64] = {0};
        int dev = 0;
        check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        unsigned long long bit = 1ull << (dev & 63);
        if (!(ready.load() & bit)){
            check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM),
                       "cudaFuncSetAttribute(convolution pass)");
            int nb = 0;
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, THREADS, SMEM), "occupancy query");
            blocks_per_sm[dev & 63] = std::max(nb, 1);
            ready.fetch_or(bit);
        }
        ConvParams P{};
        P.L = L; P.x = a.x; P.y = a.y; P.tw = a.tw;
        P.tiles_per_block = (L.count + TPB - 1) / TPB;
        P.ntiles = blocks * P.tiles_per_block;
        P.tswap = swap; P.scale = a.scale; P.status = a.status;
        long long grid = std::min<long long>(P.ntiles, (long long)num_sms() * blocks_per_sm[dev & 63]);
        kern<<<(unsigned)grid, THREADS, SMEM, s>>>(P, tmx, tmy);
        check_cuda(cudaPeekAtLastError(), "convolution pass launch");
        return true;
    }
}

template<int N>
bool run_n(cudaStream_t s, ConvLaunch const &a, bool dry_run){
    return a.y ? run_conv<N, true>(s, a, dry_run) : run_conv<N, false>(s, a, dry_run);
}

} // namespace

bool GB_CONV_NAME(cudaStream_t s, int N, ConvLaunch const &a, bool dry_run){
    switch (N){
        case 16: return run_n<16>(s, a, dry_run);
        case 32: return run_n<32>(s, a, dry_run);
        case 64: return run_n<64>(s, a, dry_run);
        case 128: return run_n<128>(s, a, dry_run);
        case 256: return run_n<256>(s, a, dry_run);
        case 512: return run_n<512>(s, a, dry_run);
        case 1024: return run_n<1024>(s, a, dry_run);
        case 2048: return run_n<2048>(s, a, dry_run);
        case 4096: return run_n<4096>(s, a, dry_run);
        default: return false;
    }
}

} // namespace gbfft
