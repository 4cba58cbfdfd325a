// Host dispatch of the pipelined power-of-two kernels for one precision.
// Included by gbfft_pipe_f32.cu (GB_T = float) and gbfft_pipe_f64.cu (GB_T = double).
#include "gbfft_internal.h"
#include "gbfft_pipe.cuh"
#include <atomic>
#include <cstring>

namespace gbfft {

namespace {

template<int N, bool FWD, bool COLS>
bool run_pipe(cudaStream_t s, PipeArgs const &a){
    using T = GB_T;
    using C = c_t<T>;
    constexpr int TPB = pipe_tpb(N, sizeof(C), COLS);
    constexpr int SMEM = pipe_smem(N, sizeof(C), COLS);
    constexpr int THREADS = TPB * pipe_tt(N);
    auto kern = k_c2c_pipe<T, N, FWD, COLS>;
    // applicability: whole tiles, contiguous tile rows / lines, 16-byte aligned copies
    if (a.G % TPB != 0) return false;
    if ((reinterpret_cast<uintptr_t>(a.in) & 15) != 0) return false;
    if (COLS){
        if (a.Li.dist != 1 || a.Li.count % TPB != 0) return false;
        if (((long long)a.Li.estride * (long long)sizeof(C)) % 16 != 0) return false;
        if (((long long)a.Li.bstride * (long long)sizeof(C)) % 16 != 0) return false;
        if ((TPB * sizeof(C)) % 16 != 0) return false;
    } else {
        if (a.Li.dist != N) return false;
        if (a.Li.count % TPB != 0 && a.Li.bstride != a.Li.count * N) return false;
        if (((long long)a.Li.bstride * (long long)sizeof(C)) % 16 != 0) return false;
        if ((N * sizeof(C)) % 16 != 0) return false;
    }
    static std::atomic<unsigned long long> ready{0};
    static int blocks_per_sm[64] = {0};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    unsigned long long bit = 1ull << (dev & 63);
    if (!(ready.load() & bit)){
        check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM),
                   "cudaFuncSetAttribute(pipelined kernel)");
        int nb = 0;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, THREADS, SMEM), "occupancy query");
        blocks_per_sm[dev & 63] = std::max(nb, 1);
        ready.fetch_or(bit);
    }
    long long ntiles = a.G / TPB;
    long long grid = std::min<long long>(ntiles, (long long)num_sms() * blocks_per_sm[dev & 63]);
    if (grid <= 0) return true;
    CUtensorMap tmap;
    std::memset(&tmap, 0, sizeof(tmap));
    int tswap = 0;
    if (COLS){
        long long blocks = a.G / a.Li.count;
        if (!encode_column_tmap(&tmap, a.in, (int)sizeof(C), a.Li.count, N, blocks, a.Li.estride, a.Li.bstride,
                                TPB, std::min(N, 256), &tswap))
            return false;
    }
    kern<<<(unsigned)grid, THREADS, SMEM, s>>>(a.Li, a.Lo, (C const*)a.in, (C*)a.out, (C const*)a.tw, ntiles,
                                              (T)a.scale, a.do_scale, a.status, tmap, tswap);
    check_cuda(cudaPeekAtLastError(), "pipelined fft kernel launch");
    return true;
}

template<bool FWD, bool COLS>
bool dispatch_n(cudaStream_t s, int N, PipeArgs const &a){
    switch (N){
        case 2: return run_pipe<2, FWD, COLS>(s, a);
        case 4: return run_pipe<4, FWD, COLS>(s, a);
        case 8: return run_pipe<8, FWD, COLS>(s, a);
        case 16: return run_pipe<16, FWD, COLS>(s, a);
        case 32: return run_pipe<32, FWD, COLS>(s, a);
        case 64: return run_pipe<64, FWD, COLS>(s, a);
        case 128: return run_pipe<128, FWD, COLS>(s, a);
        case 256: return run_pipe<256, FWD, COLS>(s, a);
        case 512: return run_pipe<512, FWD, COLS>(s, a);
        case 1024: return run_pipe<1024, FWD, COLS>(s, a);
        case 2048: return run_pipe<2048, FWD, COLS>(s, a);
        case 4096: return run_pipe<4096, FWD, COLS>(s, a);
        default: return false;
    }
}

} // namespace

bool GB_PIPE_NAME(cudaStream_t s, int N, bool fwd, bool cols, PipeArgs const &a){
    if (cols) return fwd ? dispatch_n<true, true>(s, N, a) : dispatch_n<false, true>(s, N, a);
    return fwd ? dispatch_n<true, false>(s, N, a) : dispatch_n<false, false>(s, N, a);
}

} // namespace gbfft
