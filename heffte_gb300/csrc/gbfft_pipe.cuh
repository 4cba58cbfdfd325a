// Pipelined batched transforms for power-of-two lengths (sm_103a).
//
// Persistent CTAs walk over tiles of TPB "units" (one complex transform, or a
// pair of real transforms packed into one complex FFT).  Each tile is
// streamed from HBM into shared memory while the previous tile is being
// transformed (double buffering), by one of three loaders:
//   TENSOR  column tiles through a 3-D TMA tensor map (x = column, rows,
//           blocks), one TMA op per 256 rows; out-of-range columns are filled
//           with zeros by the TMA unit;
//   BULK    line tiles (transform along the fastest dimension, lines
//           contiguous) as one 1-D bulk copy;
//   CPASYNC column tiles element by element with cp.async (any alignment,
//           e.g. the odd row stride of an r2c half-spectrum box).
// TMA copies complete on mbarriers whose waits are bounded (a device status
// word reports a wait that gave up); cp.async copies complete on commit
// groups.  Transform length, radix plan and tile shape are compile-time
// constants; the radix-stage exchange happens in shared memory and the last
// stage (or the fused post-processing of r2c / DCT) stores straight to HBM.
#pragma once
#include <cuda.h>
#include <type_traits>
#include "gbfft_common.cuh"
#include "gbfft_ptx.cuh"

namespace gbfft {

// kinds (same numbering as the host-side kernel kinds)
enum { PK_C2C_FWD = 0, PK_C2C_BWD = 1, PK_R2C_FWD = 2, PK_C2R_BWD = 3, PK_R2R_FWD = 4, PK_R2R_BWD = 5 };
// loaders
enum { LD_TENSOR = 0, LD_BULK = 1, LD_CPASYNC = 2 };

// Radix plan of the pipelined kernels: at most 16 values per thread.  The
// double-float kernels (df) use radices up to 8 (8 values per thread):
// radix-8 stages, the rest as 4 or 4 x 4.
__host__ __device__ constexpr int pipe_df_radix(int N, int s){
    switch (N){
        case 2: return 2;
        case 4: return 4;
        case 8: return 8;
        case 16: return 4;
        case 32: return (s == 0) ? 8 : 4;
        case 64: return 8;
        case 128: return (s == 0) ? 8 : 4;
        case 256: return (s < 2) ? 8 : 4;
        case 512: return 8;
        case 1024: return (s < 2) ? 8 : 4;
        case 2048: return (s < 3) ? 8 : 4;
        case 4096: return 8;
        default: return 0;
    }
}
__host__ __device__ constexpr int pipe_nstages(int N, bool df = false){
    if (df) return (N <= 8) ? 1 : ((N <= 64) ? 2 : ((N <= 512) ? 3 : 4));
    return (N <= 16) ? 1 : ((N <= 256) ? 2 : 3);
}
__host__ __device__ constexpr int pipe_radix(int N, int s, bool df = false){
    if (df) return pipe_df_radix(N, s);
    switch (N){
        case 2: return 2;
        case 4: return 4;
        case 8: return 8;
        case 16: return 16;
        case 32: return (s == 0) ? 8 : 4;
        case 64: return 8;
        case 128: return (s == 0) ? 16 : 8;
        case 256: return 16;
        case 512: return 8;
        case 1024: return (s == 0) ? 16 : 8;
        case 2048: return (s == 2) ? 8 : 16;
        case 4096: return 16;
        default: return 0;
    }
}
__host__ __device__ constexpr int pipe_ns(int N, int s, bool df = false){
    int p = 1;
    for (int i = 0; i < s; i++) p *= pipe_radix(N, i, df);
    return p;
}
__host__ __device__ constexpr int pipe_twoff(int N, int s, bool df = false){
    int off = 0;
    for (int i = 1; i < s; i++) off += pipe_ns(N, i, df) * (pipe_radix(N, i, df) - 1);
    return off;
}
__host__ __device__ constexpr int cilog2(int v){
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}
// values per thread: 16, or 8 for the double-float kernels (their plans
// have no radix above 8: half the registers and half the unrolled code per
// stage of 16 values, twice the threads)
__host__ __device__ constexpr int pipe_pe(int N, bool df = false){
    return df ? ((N < 8) ? N : 8) : ((N < 16) ? N : 16);
}
__host__ __device__ constexpr int pipe_tt(int N, bool df = false){ return N / pipe_pe(N, df); }   // threads per unit
__host__ __device__ constexpr int pipe_padn(int N){ return N + N / 16 + 1; }
__host__ __device__ constexpr bool pipe_paired(int kind){ return kind >= PK_R2C_FWD; }
// units (complex transforms or real pairs) per tile.  df: the double-float
// complex<double> kernels, which are bound by the latency of their FP32
// dependency chains rather than by memory: CTAs of about 256 threads with
// one tile slot and no separate exchange buffer (line tiles exchange in the
// tile buffer, swizzled), so that shared memory holds several CTAs per SM and
// their warps hide that latency (one slot: 21.7 against 29.0 ms with two
// slots for a 512^3 complex<double> forward + backward).
__host__ __device__ constexpr int pipe_tpb(int N, int csize, bool cols, bool df = false){
    if (df){
        int const tt = pipe_tt(N, true), target = 256;
        int tpb = (target / tt > 1) ? target / tt : 1;
        while (tpb > 1 && (N + 4) * tpb * csize > 64 * 1024) tpb /= 2;
        return tpb;
    }
    int tt = pipe_tt(N);
    if (cols && csize == 8 && N >= 512){
        // complex<float> columns of 512 points and more: as many columns as
        // two tile slots of ~100 KB hold (an even count: 16-byte rows), at
        // most 1024 threads; wider row pieces read HBM better (512^3 c2c:
        // 24 columns 2.160 ms per forward + backward, 16 columns with three
        // slots 2.205, 8 columns 2.68-2.70)
        int w = (100 * 1024) / (N * csize);
        w -= w & 1;
        int const wmax = (1024 / tt) - ((1024 / tt) & 1);
        w = (w < wmax) ? w : wmax;
        return (w >= 2) ? w : 2;
    }
    int tpb = cols ? ((csize == 8) ? 16 : 8) : 1;
    if (cols){ while (tpb * tt < 256 && tpb < 256) tpb *= 2; }
    else { while (tpb * tt < 256) tpb *= 2; }
    while (tpb > 1 && tpb * tt > 512) tpb /= 2;
    while (tpb > 1 && 2 * (N + 2) * tpb * csize > 160 * 1024) tpb /= 2;
    // and within the 227 KB of a CTA: two tile buffers (c2r lines at an even
    // pitch: 2 (N/2+1) rounded up <= N + 4 values per unit) + the line exchange buffer
    while (tpb > 1 && 2 * (N + 4) * tpb * csize + (cols ? 0 : tpb * pipe_padn(N) * csize) > 227 * 1024) tpb /= 2;
    return tpb;
}
// complex elements of one tile buffer (the c2r input tile holds N/2+1 rows of 2*TPB values)
// (line tiles of the c2r kind keep their lines at a pitch of N/2+1, or at
// the padded pitch of a workspace whose rows are padded_pitch(N/2+1))
__host__ __device__ constexpr int pipe_c2r_pitch(int N){ return (int)padded_pitch(N / 2 + 1); }
// (an r2c tile buffer also stages the tile's complex output lines at that pitch)
__host__ __device__ constexpr int pipe_tile_elems(int N, int tpb, int kind){
    return (kind == PK_C2R_BWD || kind == PK_R2C_FWD)
           ? ((pipe_c2r_pitch(N) * 2 * tpb > N * tpb) ? pipe_c2r_pitch(N) * 2 * tpb : N * tpb) : N * tpb;
}
// Tile buffers: three (two tiles in flight while one is transformed) for c2c
// column tiles of the tensor-map loader whose two buffers already take more
// than half of an SM's shared memory (one CTA per SM, so a deeper prefetch is
// what keeps more copies in flight), two otherwise.
#ifndef GBFFT_DF_SLOTS
#define GBFFT_DF_SLOTS 1
#endif
__host__ __device__ constexpr int pipe_nbuf(int N, int csize, bool cols, int kind, int loader, bool df = false){
    if (df && loader != LD_CPASYNC) return GBFFT_DF_SLOTS;
    return (!df && cols && loader == LD_TENSOR && (kind == PK_C2C_FWD || kind == PK_C2C_BWD) &&
            2 * pipe_tile_elems(N, pipe_tpb(N, csize, cols), kind) * csize > 114 * 1024 &&
            3 * pipe_tile_elems(N, pipe_tpb(N, csize, cols), kind) * csize <= 200 * 1024) ? 3 : 2;
}
__host__ __device__ constexpr int pipe_smem(int N, int csize, bool cols, int kind, int loader, bool df = false){
    int tpb = pipe_tpb(N, csize, cols, df);
    return pipe_nbuf(N, csize, cols, kind, loader, df) * pipe_tile_elems(N, tpb, kind) * csize +
           ((cols || df) ? 0 : tpb * pipe_padn(N) * csize);
}

struct PipeParams {
    Layout Li, Lo;          // per transform (real or complex elements of each array)
    void const *in;
    void *out;
    void const *tw;         // Stockham twiddles
    void const *rtw;        // exp(-i pi k / 2N) (r2r)
    long long G;            // transforms
    long long ntiles;
    long long tiles_per_block;  // column tiles: tiles covering one block of `count` columns
    double scale;
    int do_scale;
    int sine;
    int tswap;
    int line_pitch;         // line tiles: input elements per line (the line length, or padded for c2r)
    int bulk_store;         // c2c line tiles: results staged in the tile buffer, one bulk store per tile
    int out_split;          // column tiles: the input's blocks are merged into one, the output's are not
    int *status;
};

// Position of element p within a line of the swizzled exchange: the low three
// bits XORed with the three-bit groups above them, so that the eight 16-byte
// accesses of a quarter warp at any power-of-two stride (1 .. 256 elements)
// fall on distinct bank groups; a permutation within each aligned 8 elements.
__host__ __device__ constexpr int pipe_swz(int p){
    return p ^ (((p >> 3) ^ (p >> 6) ^ (p >> 9)) & 7);
}

// One radix stage; S == 0 reads through ld0, the last stage writes through st
// (or to the exchange buffer when POST is set).  Stages S .. SEND-1 run
// (SEND below the stage count stops early, the last run stage writing the
// exchange buffer).
// SWZ: line tiles exchanged in the tile buffer itself (pitch N), element p of
// a line at pipe_swz(p) (no padding, the bank spread of an XOR swizzle).
template<typename T, int N, int TPB, int S, bool FWD, bool COLS, bool POST,
         int SEND = pipe_nstages(N, std::is_same<T, df>::value), bool SWZ = false, class LD, class ST>
__device__ __forceinline__ void pstage(int t, int loc, c_t<T> *xch, c_t<T> const *__restrict__ tw,
                                       c_t<T> (&v)[16], LD &ld0, ST &st){
    using C = c_t<T>;
    constexpr bool DFT = std::is_same<T, df>::value;
    constexpr int NS = pipe_nstages(N, DFT);
    if constexpr (S < SEND){
        constexpr int R = pipe_radix(N, S, DFT), Ns = pipe_ns(N, S, DFT), TWO = pipe_twoff(N, S, DFT);
        constexpr int NR = N / R, TT = pipe_tt(N, DFT), M = pipe_pe(N, DFT) / R, PADN = pipe_padn(N);
        constexpr bool LAST = (S == NS - 1);
        constexpr bool TO_XCH = !LAST || POST;
        constexpr int LNS = cilog2(Ns), LNSR = cilog2(Ns * R);
        auto xi = [&](int p) -> int {
            if constexpr (COLS) return p * TPB + loc;
            else if constexpr (SWZ) return loc * N + pipe_swz(p);
            else return loc * PADN + p + (p >> 4);
        };
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            #pragma unroll
            for (int q = 0; q < R; q++){
                int p = j + q * NR;
                if constexpr (S == 0) v[m * R + q] = ld0(p);
                else v[m * R + q] = xch[xi(p)];
            }
        }
        // the exchange buffer is rewritten below: everyone must have read it
        if (TO_XCH) __syncthreads();
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            int k = j & (Ns - 1);
            if constexpr (S > 0){
                C const *w = tw + TWO + k * (R - 1);
                #pragma unroll
                for (int q = 1; q < R; q++){
                    C wq = ldg_c(w + q - 1);
                    v[m * R + q] = FWD ? cmul(v[m * R + q], wq) : cmulc(v[m * R + q], wq);
                }
            }
            bfly<R, FWD, C, T>(&v[m * R]);
            int ob = ((j >> LNS) << LNSR) + k;
            #pragma unroll
            for (int q = 0; q < R; q++){
                int p = ob + q * Ns;
                if constexpr (TO_XCH) xch[xi(p)] = v[m * R + q];
                else st(p, v[m * R + q]);
            }
        }
        if (TO_XCH) __syncthreads();
        pstage<T, N, TPB, S + 1, FWD, COLS, POST, SEND, SWZ>(t, loc, xch, tw, v, ld0, st);
    }
}

__device__ __forceinline__ long long base_of_fast(Layout const &L, long long g){ return base_of(L, g); }

__device__ __forceinline__ void cp_async_8(void *dst, void const *src, bool valid){
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" :: "r"(smem_u32(dst)), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_16(void *dst, void const *src, bool valid){
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" :: "r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit(){ asm volatile("cp.async.commit_group;" ::: "memory"); }
template<int NG> __device__ __forceinline__ void cp_async_wait(){ asm volatile("cp.async.wait_group %0;" :: "n"(NG) : "memory"); }

__host__ __device__ constexpr int pipe_threads(int N, int csize, bool cols, bool df = false){
    return pipe_tpb(N, csize, cols, df) * pipe_tt(N, df);
}

// DF: complex<double> tiles transformed in double-float arithmetic (c2c kinds).
// CTAs per SM the double-float kernels are compiled for (their register
// budget): 1024 threads per SM, 64 registers a thread, which 8 values per
// thread fit without spilling (512^3 Z2Z forward + backward 16.4 ms; compiled
// for 3 or 5 CTAs of 256 threads: 17.2, 16.7 ms).  With 16 values per thread
// (the earlier plans with radix-16 stages) the best budgets were 128 registers
// (512^3: 20.0 ms; 168 unbounded: 35.7) and 80 for 256 points.
#ifndef GBFFT_DF_MIN_CTAS
#define GBFFT_DF_MIN_CTAS 0
#endif
__host__ __device__ constexpr int pipe_df_min_ctas(int N, int threads){
    return GBFFT_DF_MIN_CTAS > 0 ? GBFFT_DF_MIN_CTAS : ((threads >= 1024) ? 1 : 1024 / threads);
}
// The body of the pipelined kernels; k_pipe (bounded by its thread count
// alone: the compiler's own register choice) and k_pipe_df (also by the CTAs
// per SM above) are its two entry points.
template<typename T, int N, int KIND, bool COLS, int LOADER, bool DF>
__device__ __forceinline__ void pipe_body(PipeParams const &P, CUtensorMap const &tmap){
    using C = c_t<T>;
    static_assert(!DF || ((KIND == PK_C2C_FWD || KIND == PK_C2C_BWD) && sizeof(T) == 8),
                  "double-float arithmetic serves the complex<double> c2c kinds");
    constexpr bool PAIRED = pipe_paired(KIND);
    constexpr int TPB = pipe_tpb(N, sizeof(C), COLS, DF);
    constexpr int TT = pipe_tt(N, DF);
    constexpr int NT = TPB * TT;
    constexpr int TILE = pipe_tile_elems(N, TPB, KIND);   // complex elements per buffer
    constexpr int H = N / 2 + 1;
    // input of one tile: rows x width (columns) or lines x line_len, in input elements
    constexpr int IN_ES = (KIND == PK_R2C_FWD || KIND == PK_R2R_FWD || KIND == PK_R2R_BWD) ? (int)sizeof(T) : (int)sizeof(C);
    constexpr int ROWS = (KIND == PK_C2R_BWD) ? H : N;
    constexpr int WIDTH = PAIRED ? 2 * TPB : TPB;           // input elements per tile row (columns)
    constexpr bool FWD = (KIND == PK_C2C_FWD || KIND == PK_R2C_FWD || KIND == PK_R2R_FWD);
    constexpr int PADN = pipe_padn(N);
    constexpr int NBUF = pipe_nbuf(N, (int)sizeof(C), COLS, KIND, LOADER, DF);
    static_assert(LOADER != LD_CPASYNC || NBUF == 2, "cp.async tiles are double buffered");

    extern __shared__ __align__(128) unsigned char smraw[];
    C *tiles = reinterpret_cast<C*>(smraw);
    C *xline = tiles + NBUF * TILE;  // line tiles: padded exchange buffer
    __shared__ __align__(8) uint64_t bar[NBUF];
    __shared__ unsigned s_emax[DF ? NT / 32 : 1];   // per-warp largest exponent of a tile (DF)

    int tid = threadIdx.x;
    int loc, t;
    if (COLS){ loc = tid % TPB; t = tid / TPB; } else { loc = tid / TT; t = tid % TT; }
    int lane = tid & 31, warp = tid >> 5;
    Layout const Li = P.Li, Lo = P.Lo;
    int units_per = PAIRED ? 2 : 1;

    if (LOADER != LD_CPASYNC && tid == 0){
        #pragma unroll
        for (int i = 0; i < NBUF; i++) mbar_init(&bar[i], 1);
        fence_mbar_init();
    }
    if (LOADER == LD_TENSOR && tid == 0) prefetch_tmap(&tmap);
    __syncthreads();

    // tile -> (block, first column) for column tiles, first line for line tiles
    auto tile_origin = [&](long long tile, long long &blk, long long &c0){
        if (COLS){
            if (tile < 0x7fffffffLL && P.tiles_per_block < 0x7fffffffLL){
                unsigned q = (unsigned)tile / (unsigned)P.tiles_per_block;
                blk = q;
                c0 = (long long)((unsigned)tile - q * (unsigned)P.tiles_per_block) * WIDTH;
            } else {
                blk = tile / P.tiles_per_block;
                c0 = (tile - blk * P.tiles_per_block) * WIDTH;
            }
        } else {
            blk = 0;
            c0 = tile * (long long)TPB * units_per;   // first line
        }
    };

    auto issue = [&](long long tile, int b){
        long long blk, c0;
        tile_origin(tile, blk, c0);
        unsigned char *dst = reinterpret_cast<unsigned char*>(tiles + b * TILE);
        if constexpr (LOADER == LD_TENSOR){
            if (warp == 0 && lane == 0){
                constexpr int BOXR = (ROWS < 256) ? ROWS : 256;
                constexpr int WPE = (IN_ES >= 8) ? IN_ES / 8 : 1;      // tensor words per input element
                mbar_arrive_expect_tx(&bar[b], (uint32_t)(ROWS * WIDTH * IN_ES));
                #pragma unroll
                for (int r0 = 0; r0 < ROWS; r0 += BOXR){
                    int x = (int)(c0 * WPE);
                    if (P.tswap) tma_load_3d(dst + (size_t)r0 * WIDTH * IN_ES, &tmap, x, (int)blk, r0, &bar[b]);
                    else tma_load_3d(dst + (size_t)r0 * WIDTH * IN_ES, &tmap, x, r0, (int)blk, &bar[b]);
                }
            }
        } else if constexpr (LOADER == LD_BULK){
            if (warp == 0 && lane == 0){
                // the buffer's previous tile may still be read by its bulk store
                if (P.bulk_store) bulk_wait_read<0>();
                long long lines = ((long long)TPB * units_per < P.G - c0) ? (long long)TPB * units_per : (P.G - c0);
                uint32_t bytes = (uint32_t)(lines * P.line_pitch * IN_ES);
                long long base = base_of_fast(Li, c0);
                mbar_arrive_expect_tx(&bar[b], bytes);
                bulk_g2s(dst, reinterpret_cast<unsigned char const*>(P.in) + base * IN_ES, bytes, &bar[b]);
            }
        } else {
            // cp.async, element by element (8- or 16-byte elements), zero fill out
            // of range; each thread keeps one column (NT is a multiple of WIDTH)
            long long rstride = Li.estride * IN_ES;
            if constexpr (NT % WIDTH == 0){
                constexpr int RSTEP = NT / WIDTH;
                int c = tid % WIDTH, r = tid / WIDTH;
                bool valid = (c0 + c) < Li.count;
                long long col = valid ? blk * Li.bstride + (c0 + c) * Li.dist : 0;
                unsigned char const *src = reinterpret_cast<unsigned char const*>(P.in) + col * IN_ES;
                #pragma unroll 4
                for (; r < ROWS; r += RSTEP){
                    int e = r * WIDTH + c;
                    if constexpr (IN_ES == 16) cp_async_16(dst + (size_t)e * 16, src + (valid ? r * rstride : 0), valid);
                    else cp_async_8(dst + (size_t)e * 8, src + (valid ? r * rstride : 0), valid);
                }
            } else {
                for (int e = tid; e < ROWS * WIDTH; e += NT){
                    int r = e / WIDTH, c = e - r * WIDTH;
                    bool valid = (c0 + c) < Li.count;
                    long long off = valid ? (blk * Li.bstride + (c0 + c) * Li.dist) * IN_ES + r * rstride : 0;
                    unsigned char const *src = reinterpret_cast<unsigned char const*>(P.in) + off;
                    if constexpr (IN_ES == 16) cp_async_16(dst + (size_t)e * 16, src, valid);
                    else cp_async_8(dst + (size_t)e * 8, src, valid);
                }
            }
            cp_async_commit();
        }
    };

    uint32_t phase = 0;              // bit b: parity of the next wait on bar[b]
    long long tile = blockIdx.x;
    // the first NBUF - 1 tiles of this CTA
    #pragma unroll
    for (int i = 0; i < NBUF - 1; i++){
        long long tl = tile + (long long)i * gridDim.x;
        if (tl < P.ntiles) issue(tl, i);
    }
    T sc = (T)P.scale;
    // the plan's scale as a float pair (double-float tiles)
    df scale_df;
    if constexpr (DF) scale_df = df_from(P.scale);
    for (int it = 0; tile < P.ntiles; tile += gridDim.x, it++){
        int b = it % NBUF;
        // the tile NBUF - 1 ahead goes into the buffer consumed last iteration
        long long nxt = tile + (long long)(NBUF - 1) * gridDim.x;
        if (nxt < P.ntiles){
            if (LOADER != LD_CPASYNC && warp == 0) fence_proxy_async_smem();
            issue(nxt, (it + NBUF - 1) % NBUF);
        }
        if constexpr (LOADER == LD_CPASYNC){
            if (nxt < P.ntiles) cp_async_wait<1>(); else cp_async_wait<0>();
            __syncthreads();
        } else {
            bool ok = mbar_wait_bounded(&bar[b], (phase >> b) & 1u, P.status);
            if (__syncthreads_or(!ok)){
                if (P.bulk_store && tid == 0) bulk_wait<0>();
                return;
            }
            phase ^= 1u << b;
        }

        C *tb = tiles + b * TILE;
        C *xch = (COLS || DF) ? tb : xline;
        long long blk, c0;
        tile_origin(tile, blk, c0);
        // transforms of this thread's unit
        bool va, vb;
        long long oa = 0, obb = 0;
        if (COLS){
            // column ca of block blk: the output offset needs no division
            long long ca = c0 + (long long)loc * units_per;
            va = ca < Li.count;
            vb = PAIRED ? (ca + 1 < Li.count) : false;
            if (P.out_split){
                // ca counts columns over all blocks of the output
                if (va) oa = base_of_fast(Lo, ca);
                if (vb) obb = base_of_fast(Lo, ca + 1);
            } else {
                oa = blk * Lo.bstride + ca * Lo.dist;
                obb = oa + Lo.dist;
            }
        } else {
            long long ga = c0 + (long long)loc * units_per, gb = ga + 1;
            va = ga < P.G;
            vb = PAIRED ? (gb < P.G) : false;
            if (va) oa = base_of_fast(Lo, ga);
            if (vb) obb = base_of_fast(Lo, gb);
        }
        long long oes = Lo.estride;
        T const *tr = reinterpret_cast<T const*>(tb);
        int sine = P.sine;
        C v[16];

        if constexpr (DF){
            // double-float: the tile is scaled by 2^-sh so that its largest
            // magnitude lies in [1, 2) (the float exponent range then holds
            // everything above 2^-126 of it; smaller values contribute less
            // than 2^-126 of the tile's norm), transformed as float pairs, and
            // scaled back by 2^sh (with the plan's scale) on the store
            using D = c_t<df>;
            uint4 const *words = reinterpret_cast<uint4 const*>(tb);
            unsigned e = 0;
            // only the tile's own lines: the line loader copies the last,
            // partial tile's lines alone, and the rows past them still hold
            // an older tile (column tiles are zero-filled past the edge)
            int const scan = COLS ? TILE : (int)min((long long)TILE, (P.G - c0) * N);
            for (int i = tid; i < scan; i += NT){
                uint4 w = words[i];
                e = max(e, max((w.y >> 20) & 0x7ffu, (w.w >> 20) & 0x7ffu));
            }
            e = __reduce_max_sync(0xffffffffu, e);
            if (lane == 0) s_emax[warp] = e;
            __syncthreads();
            unsigned em = 0;
            #pragma unroll
            for (int w = 0; w < NT / 32; w++) em = max(em, s_emax[w]);
            int sh = (em == 0) ? -1022 : (int)em - 1023;
            sh = min(max(sh, -1022), 1022);
            // the conversions use integer and FP32 instructions (one FP64
            // addition per value on the way back), see df_from_scaled
            auto ld0 = [&](int p) -> D {
                C v = COLS ? tb[p * TPB + loc] : tb[loc * N + p];
                D r; r.x = df_from_scaled(v.x, sh); r.y = df_from_scaled(v.y, sh);
                return r;
            };
            auto back = [&](D x) -> C {
                if (P.do_scale){ x.x = x.x * scale_df; x.y = x.y * scale_df; }
                C r; r.x = df_to_scaled(x.x, sh); r.y = df_to_scaled(x.y, sh);
                return r;
            };
            D *xd = reinterpret_cast<D*>(xch);
            D const *twd = reinterpret_cast<D const*>(P.tw);
            D vd[16];
            C *out = reinterpret_cast<C*>(P.out);
            // the exchange is the tile buffer (swizzled for line tiles), so
            // the last stage stores straight to global memory
            auto st = [&](int p, D x){ if (va) out[oa + p * oes] = back(x); };
            pstage<df, N, TPB, 0, FWD, COLS, false, pipe_nstages(N, true), !COLS>(t, loc, xd, twd, vd, ld0, st);
            (void)v;
        } else if constexpr (KIND == PK_C2C_FWD || KIND == PK_C2C_BWD){
            auto ld0 = [&](int p) -> C { return COLS ? tb[p * TPB + loc] : tb[loc * N + p]; };
            C *out = reinterpret_cast<C*>(P.out);
            if (!COLS && LOADER == LD_BULK && P.bulk_store){
                // the last stage writes the tile buffer (read only by stage 0),
                // one thread stores the whole tile with a bulk copy
                auto st = [&](int p, C x){ tb[loc * N + p] = P.do_scale ? cscale(x, sc) : x; };
                pstage<T, N, TPB, 0, FWD, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
                fence_proxy_async_smem();
                __syncthreads();
                if (tid == 0){
                    long long lines = ((long long)TPB < P.G - c0) ? (long long)TPB : (P.G - c0);
                    bulk_s2g(out + base_of_fast(Lo, c0), tb, (uint32_t)(lines * N * sizeof(C)));
                    bulk_commit();
                }
            } else {
                auto st = [&](int p, C x){ if (va) out[oa + p * oes] = P.do_scale ? cscale(x, sc) : x; };
                pstage<T, N, TPB, 0, FWD, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
            }
        } else if constexpr (KIND == PK_R2C_FWD || KIND == PK_R2R_FWD){
            auto ld0 = [&](int p) -> C {
                int n = p;
                T sg = (T)1;
                if constexpr (KIND == PK_R2R_FWD){
                    n = (2 * p < N) ? 2 * p : 2 * (N - 1 - p) + 1;   // Makhoul reordering
                    if (sine && (n & 1)) sg = (T)-1;
                }
                C z;
                if (COLS){ z = tb[n * TPB + loc]; }
                else { z.x = tr[(2 * loc) * N + n]; z.y = tr[(2 * loc + 1) * N + n]; }
                z.x *= sg; z.y *= sg;
                return z;
            };
            auto st = [&](int, C){};
            pstage<T, N, TPB, 0, true, COLS, true>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
            auto xi = [&](int p) -> int { return COLS ? (p * TPB + loc) : (loc * PADN + p + (p >> 4)); };
            if constexpr (KIND == PK_R2C_FWD){
                C *out = reinterpret_cast<C*>(P.out);
                T h = (T)0.5 * (P.do_scale ? sc : (T)1);
                if (!COLS && LOADER == LD_BULK && P.bulk_store){
                    // output lines staged in the tile buffer (its real input was
                    // read by stage 0) at the output pitch, one bulk store
                    long long const SP = Lo.dist;
                    for (int k = t; k <= N / 2; k += TT){
                        C zk = xch[xi(k)], zn = xch[xi((k == 0) ? 0 : N - k)];
                        C xa; xa.x = h * (zk.x + zn.x); xa.y = h * (zk.y - zn.y);
                        C xb; xb.x = h * (zk.y + zn.y); xb.y = -h * (zk.x - zn.x);
                        tb[(2 * loc) * SP + k] = xa;
                        tb[(2 * loc + 1) * SP + k] = xb;
                    }
                    fence_proxy_async_smem();
                    __syncthreads();
                    if (tid == 0){
                        long long lines = ((long long)TPB * 2 < P.G - c0) ? (long long)TPB * 2 : (P.G - c0);
                        bulk_s2g(out + base_of_fast(Lo, c0), tb, (uint32_t)(lines * SP * sizeof(C)));
                        bulk_commit();
                    }
                } else {
                    for (int k = t; k <= N / 2; k += TT){
                        C zk = xch[xi(k)], zn = xch[xi((k == 0) ? 0 : N - k)];
                        C xa; xa.x = h * (zk.x + zn.x); xa.y = h * (zk.y - zn.y);
                        C xb; xb.x = h * (zk.y + zn.y); xb.y = -h * (zk.x - zn.x);
                        if (va) out[oa + k * oes] = xa;
                        if (vb) out[obb + k * oes] = xb;
                    }
                }
            } else {
                T *out = reinterpret_cast<T*>(P.out);
                C const *rtw = reinterpret_cast<C const*>(P.rtw);
                T s = P.do_scale ? sc : (T)1;
                // bulk store: the real output lines staged in the tile buffer
                // (its real input was read by stage 0)
                bool const stage = !COLS && LOADER == LD_BULK && P.bulk_store;
                T *stg = reinterpret_cast<T*>(tb);
                for (int k = t; k < N; k += TT){
                    C zk = xch[xi(k)], zn = xch[xi((k == 0) ? 0 : N - k)];
                    C w = __ldg(rtw + k);
                    T ax = zk.x + zn.x, ay = zk.y - zn.y;
                    T bx = zk.y + zn.y, by = -(zk.x - zn.x);
                    int ko = sine ? (N - 1 - k) : k;
                    T ya = (w.x * ax - w.y * ay) * s, yb = (w.x * bx - w.y * by) * s;
                    if (stage){
                        stg[(2 * loc) * N + ko] = ya;
                        stg[(2 * loc + 1) * N + ko] = yb;
                    } else {
                        if (va) out[oa + ko * oes] = ya;
                        if (vb) out[obb + ko * oes] = yb;
                    }
                }
                if (stage){
                    fence_proxy_async_smem();
                    __syncthreads();
                    if (tid == 0){
                        long long lines = ((long long)TPB * 2 < P.G - c0) ? (long long)TPB * 2 : (P.G - c0);
                        bulk_s2g(out + base_of_fast(Lo, c0), stg, (uint32_t)(lines * N * sizeof(T)));
                        bulk_commit();
                    }
                }
            }
        } else if constexpr (KIND == PK_C2R_BWD){
            auto ld0 = [&](int p) -> C {
                int pp = (2 * p <= N) ? p : N - p;
                bool cj = (2 * p > N);
                bool real_only = (pp == 0) || (2 * pp == N);
                C xa, xb;
                if (COLS){ xa = tb[pp * (2 * TPB) + 2 * loc]; xb = tb[pp * (2 * TPB) + 2 * loc + 1]; }
                else { xa = tb[(2 * loc) * P.line_pitch + pp]; xb = tb[(2 * loc + 1) * P.line_pitch + pp]; }
                if (real_only){ xa.y = 0; xb.y = 0; }
                if (cj){ xa.y = -xa.y; xb.y = -xb.y; }
                C z; z.x = xa.x - xb.y; z.y = xa.y + xb.x;
                return z;
            };
            T *out = reinterpret_cast<T*>(P.out);
            T s = P.do_scale ? sc : (T)1;
            if (!COLS && LOADER == LD_BULK && P.bulk_store){
                // the real output lines staged in the tile buffer (its complex
                // input was read by stage 0), one bulk store
                T *stg = reinterpret_cast<T*>(tb);
                auto st = [&](int p, C x){
                    stg[(2 * loc) * N + p] = x.x * s;
                    stg[(2 * loc + 1) * N + p] = x.y * s;
                };
                pstage<T, N, TPB, 0, false, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
                fence_proxy_async_smem();
                __syncthreads();
                if (tid == 0){
                    long long lines = ((long long)TPB * 2 < P.G - c0) ? (long long)TPB * 2 : (P.G - c0);
                    bulk_s2g(out + base_of_fast(Lo, c0), stg, (uint32_t)(lines * N * sizeof(T)));
                    bulk_commit();
                }
            } else {
                auto st = [&](int p, C x){
                    if (va) out[oa + p * oes] = x.x * s;
                    if (vb) out[obb + p * oes] = x.y * s;
                };
                pstage<T, N, TPB, 0, false, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
            }
        } else {
            // PK_R2R_BWD: V[k] = 2 exp(i pi k / 2N) (Y[k] - i Y[N-k]), two lines per FFT
            C const *rtw = reinterpret_cast<C const*>(P.rtw);
            auto yv = [&](int which, int k) -> T {
                if (k >= N) return (T)0;
                int kk = sine ? (N - 1 - k) : k;
                if (COLS){ C z = tb[kk * TPB + loc]; return which ? z.y : z.x; }
                return tr[(2 * loc + which) * N + kk];
            };
            auto ld0 = [&](int p) -> C {
                C w = __ldg(rtw + p); w.y = -w.y;
                T a0 = yv(0, p), a1 = (p == 0) ? (T)0 : yv(0, N - p);
                T b0 = yv(1, p), b1 = (p == 0) ? (T)0 : yv(1, N - p);
                C va_, vb_;
                va_.x = 2 * (w.x * a0 + w.y * a1); va_.y = 2 * (w.y * a0 - w.x * a1);
                vb_.x = 2 * (w.x * b0 + w.y * b1); vb_.y = 2 * (w.y * b0 - w.x * b1);
                C z; z.x = va_.x - vb_.y; z.y = va_.y + vb_.x;
                return z;
            };
            T *out = reinterpret_cast<T*>(P.out);
            T s = P.do_scale ? sc : (T)1;
            if (!COLS && LOADER == LD_BULK && P.bulk_store){
                // the real output lines staged in the tile buffer (its real
                // input was read by stage 0), one bulk store
                T *stg = reinterpret_cast<T*>(tb);
                auto st = [&](int n, C x){
                    int m = (2 * n < N) ? 2 * n : 2 * (N - 1 - n) + 1;
                    T sg = (sine && (m & 1)) ? -s : s;
                    stg[(2 * loc) * N + m] = x.x * sg;
                    stg[(2 * loc + 1) * N + m] = x.y * sg;
                };
                pstage<T, N, TPB, 0, false, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
                fence_proxy_async_smem();
                __syncthreads();
                if (tid == 0){
                    long long lines = ((long long)TPB * 2 < P.G - c0) ? (long long)TPB * 2 : (P.G - c0);
                    bulk_s2g(out + base_of_fast(Lo, c0), stg, (uint32_t)(lines * N * sizeof(T)));
                    bulk_commit();
                }
            } else {
                auto st = [&](int n, C x){
                    int m = (2 * n < N) ? 2 * n : 2 * (N - 1 - n) + 1;
                    T sg = (sine && (m & 1)) ? -s : s;
                    if (va) out[oa + m * oes] = x.x * sg;
                    if (vb) out[obb + m * oes] = x.y * sg;
                };
                pstage<T, N, TPB, 0, false, COLS, false>(t, loc, xch, reinterpret_cast<C const*>(P.tw), v, ld0, st);
            }
        }
        __syncthreads();
    }
    // the last bulk stores must be complete before the CTA's shared memory goes
    if (LOADER == LD_BULK && P.bulk_store && tid == 0) bulk_wait<0>();
}

template<typename T, int N, int KIND, bool COLS, int LOADER>
__global__ void __launch_bounds__(pipe_threads(N, sizeof(c_t<T>), COLS))
k_pipe(PipeParams P, const __grid_constant__ CUtensorMap tmap){
    pipe_body<T, N, KIND, COLS, LOADER, false>(P, tmap);
}

template<typename T, int N, int KIND, bool COLS, int LOADER>
__global__ void __launch_bounds__(pipe_threads(N, sizeof(c_t<T>), COLS, true),
                                  pipe_df_min_ctas(N, pipe_threads(N, sizeof(c_t<T>), COLS, true)))
k_pipe_df(PipeParams P, const __grid_constant__ CUtensorMap tmap){
    pipe_body<T, N, KIND, COLS, LOADER, true>(P, tmap);
}

} // namespace gbfft
