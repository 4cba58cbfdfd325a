// Host dispatch of the pipelined power-of-two kernels for one precision and
// one group of kinds.  Included by the gbfft_pipe_*.cu units with
//   GB_T          float or double
//   GB_PIPE_NAME  the exported dispatcher
//   GB_GROUP      0: c2c (forward, backward), 1: r2c + c2r, 2: r2r forward + backward
//   GB_DF         1: complex<double> in double-float arithmetic (c2c group; default 0)
// so that the instantiations compile in parallel.
#ifndef GB_DF
#define GB_DF 0
#endif
#include "gbfft_internal.h"
#include "gbfft_pipe.cuh"
#include <atomic>
#include <cstring>

namespace gbfft {

namespace {

template<int N, int KIND, bool COLS, int LOADER>
bool run_pipe(cudaStream_t s, PipeLaunch const &a){
    using T = GB_T;
    using C = c_t<T>;
    constexpr bool PAIRED = pipe_paired(KIND);
    constexpr bool DF = GB_DF != 0;
    constexpr int TPB = pipe_tpb(N, sizeof(C), COLS, DF);
    constexpr int SMEM = pipe_smem(N, sizeof(C), COLS, KIND, LOADER, DF);
    static_assert(SMEM <= 227 * 1024, "pipelined tile exceeds the shared memory of a CTA");
    constexpr int THREADS = pipe_threads(N, sizeof(C), COLS, DF);
    constexpr int IN_ES = (KIND == PK_R2C_FWD || KIND == PK_R2R_FWD || KIND == PK_R2R_BWD) ? (int)sizeof(T) : (int)sizeof(C);
    constexpr int ROWS = (KIND == PK_C2R_BWD) ? N / 2 + 1 : N;
    constexpr int WIDTH = PAIRED ? 2 * TPB : TPB;
    constexpr int LINE_LEN = ROWS;
    constexpr int UNITS = PAIRED ? 2 : 1;
    Layout const &Li = a.Li;
    uintptr_t base = reinterpret_cast<uintptr_t>(a.in);
    if (a.G <= 0) return true;
    if (a.G % Li.count != 0) return false;
    long long blocks = a.G / Li.count;
    PipeParams P{};
    CUtensorMap tmap;
    std::memset(&tmap, 0, sizeof(tmap));
    if constexpr (LOADER == LD_TENSOR){
        if (Li.dist != 1 || (base & 15) || ((WIDTH * IN_ES) % 16) != 0) return false;
        int swap = 0;
        if (!encode_column_tmap(&tmap, a.in, IN_ES, Li.count, ROWS, blocks, Li.estride, Li.bstride, WIDTH,
                                ROWS < 256 ? ROWS : 256, &swap))
            return false;
        P.tswap = swap;
    } else if constexpr (LOADER == LD_BULK){
        // lines back to back, or (c2r) at the padded pitch of a workspace
        long long pitch = LINE_LEN;
        if (Li.dist != LINE_LEN){
            if (KIND != PK_C2R_BWD || Li.dist != pipe_c2r_pitch(N)) return false;
            pitch = Li.dist;
        }
        if (blocks > 1 && Li.bstride != Li.count * pitch) return false;
        if ((base & 15) || ((long long)a.G * pitch * IN_ES) % 16 != 0 ||
            ((long long)TPB * UNITS * pitch * IN_ES) % 16 != 0)
            return false;
        P.line_pitch = (int)pitch;
        // c2c line tiles whose output lines are back to back: one bulk store per tile
        Layout const &Lo = a.Lo;
        uintptr_t obase = reinterpret_cast<uintptr_t>(a.out);
        if ((KIND == PK_C2C_FWD || KIND == PK_C2C_BWD) && N >= 32 && Lo.estride == 1 && Lo.dist == N &&
            (a.G <= Lo.count || Lo.bstride == Lo.count * N) && (obase & 15) == 0)
            P.bulk_store = 1;
        // r2c: complex output lines (N/2+1, or the padded pitch) back to back;
        // c2r: real output lines back to back; every tile's bytes a multiple of 16
        constexpr int H2 = N / 2 + 1;
        if (KIND == PK_R2C_FWD && N >= 32 && Lo.estride == 1 && (Lo.dist == H2 || Lo.dist == pipe_c2r_pitch(N)) &&
            (a.G <= Lo.count || Lo.bstride == Lo.count * Lo.dist) && (obase & 15) == 0 &&
            (a.G % 2 == 0 || Lo.dist % 2 == 0))
            P.bulk_store = 1;
        if ((KIND == PK_C2R_BWD || KIND == PK_R2R_FWD || KIND == PK_R2R_BWD) && N >= 32 && Lo.estride == 1 &&
            Lo.dist == N && (a.G <= Lo.count || Lo.bstride == Lo.count * N) && (obase & 15) == 0)
            P.bulk_store = 1;
    } else {
        if (Li.dist != 1 || (IN_ES != 8 && IN_ES != 16) || (base % IN_ES)) return false;
    }
    auto kern = []{
        if constexpr (DF) return k_pipe_df<T, N, KIND, COLS, LOADER>;
        else return k_pipe<T, N, KIND, COLS, LOADER>;
    }();
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
    P.Li = a.Li; P.Lo = a.Lo; P.in = a.in; P.out = a.out; P.tw = a.tw; P.rtw = a.rtw;
    P.G = a.G; P.scale = a.scale; P.do_scale = (a.scale != 1.0); P.sine = a.sine; P.status = a.status;
    P.out_split = a.out_split;
    if (COLS){
        P.tiles_per_block = (Li.count + WIDTH - 1) / WIDTH;
        P.ntiles = blocks * P.tiles_per_block;
    } else {
        P.tiles_per_block = 0;
        P.ntiles = (a.G + (long long)TPB * UNITS - 1) / ((long long)TPB * UNITS);
    }
    long long grid = std::min<long long>(P.ntiles, (long long)num_sms() * blocks_per_sm[dev & 63]);
    kern<<<(unsigned)grid, THREADS, SMEM, s>>>(P, tmap);
    check_cuda(cudaPeekAtLastError(), "pipelined fft kernel launch");
    return true;
}

template<int N, int KIND>
bool run_kind(cudaStream_t s, bool cols, PipeLaunch const &a){
    constexpr bool REAL_IN = (KIND == PK_R2C_FWD || KIND == PK_R2R_FWD || KIND == PK_R2R_BWD);
    if (!cols) return run_pipe<N, KIND, false, LD_BULK>(s, a);
    if constexpr (KIND != PK_C2R_BWD){
        if (run_pipe<N, KIND, true, LD_TENSOR>(s, a)) return true;
    }
    if constexpr (!REAL_IN){
        return run_pipe<N, KIND, true, LD_CPASYNC>(s, a);
    }
    return false;
}

template<int N>
bool run_group(cudaStream_t s, int kind, bool cols, PipeLaunch const &a){
#if GB_GROUP == 0
    if (kind == PK_C2C_FWD) return run_kind<N, PK_C2C_FWD>(s, cols, a);
    if (kind == PK_C2C_BWD) return run_kind<N, PK_C2C_BWD>(s, cols, a);
#elif GB_GROUP == 1
    if (kind == PK_R2C_FWD) return run_kind<N, PK_R2C_FWD>(s, cols, a);
    if (kind == PK_C2R_BWD) return run_kind<N, PK_C2R_BWD>(s, cols, a);
#else
    if (kind == PK_R2R_FWD) return run_kind<N, PK_R2R_FWD>(s, cols, a);
    if (kind == PK_R2R_BWD) return run_kind<N, PK_R2R_BWD>(s, cols, a);
#endif
    return false;
}

} // namespace

bool GB_PIPE_NAME(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a){
    constexpr bool DBL = sizeof(GB_T) == 8;
    switch (N){
        case 16: return run_group<16>(s, kind, cols, a);
        case 32: return run_group<32>(s, kind, cols, a);
        case 64: return run_group<64>(s, kind, cols, a);
        case 128: return run_group<128>(s, kind, cols, a);
        case 256: return run_group<256>(s, kind, cols, a);
        case 512: return run_group<512>(s, kind, cols, a);
        case 1024: return run_group<1024>(s, kind, cols, a);
        case 2048: return run_group<2048>(s, kind, cols, a);
        case 4096: if constexpr (!DBL) return run_group<4096>(s, kind, cols, a); else return false;
        default: return false;
    }
}

} // namespace gbfft
