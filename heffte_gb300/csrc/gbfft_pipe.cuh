// Pipelined batched transforms for power-of-two lengths (sm_103a).
//
// Persistent CTAs walk over tiles of TPB transforms.  Each tile is streamed
// from HBM into shared memory by 1-D bulk copies (the TMA engine) that
// complete on an mbarrier, double-buffered: while the CTA transforms tile i,
// tile i+1 is already in flight.  Transform length, radix sequence and tile
// shape are compile-time constants, so index arithmetic folds to shifts and
// the butterflies are straight-line code; the result leaves the registers of
// the last radix stage directly for HBM.
//
//   column tiles (transform along a strided dimension): TPB adjacent columns
//     x N rows; row p of the tile is one bulk copy of TPB*sizeof(C) bytes;
//     the radix stages exchange through the tile buffer itself.
//   line tiles (transform along the fastest dimension): TPB contiguous lines,
//     one bulk copy; the stages exchange through a padded buffer.
#pragma once
#include <cuda.h>
#include "gbfft_common.cuh"
#include "gbfft_ptx.cuh"

namespace gbfft {

// Radix plan of the pipelined kernels: at most 16 values per thread.
__host__ __device__ constexpr int pipe_nstages(int N){
    return (N <= 16) ? 1 : ((N <= 256) ? 2 : 3);
}
__host__ __device__ constexpr int pipe_radix(int N, int s){
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
__host__ __device__ constexpr int pipe_ns(int N, int s){
    int p = 1;
    for (int i = 0; i < s; i++) p *= pipe_radix(N, i);
    return p;
}
__host__ __device__ constexpr int pipe_twoff(int N, int s){
    int off = 0;
    for (int i = 1; i < s; i++) off += pipe_ns(N, i) * (pipe_radix(N, i) - 1);
    return off;
}
__host__ __device__ constexpr int cilog2(int v){
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}
__host__ __device__ constexpr int pipe_pe(int N){ return (N < 16) ? N : 16; }     // values per thread
__host__ __device__ constexpr int pipe_tt(int N){ return N / pipe_pe(N); }        // threads per transform
__host__ __device__ constexpr int pipe_padn(int N){ return N + N / 16 + 1; }
// transforms per tile
__host__ __device__ constexpr int pipe_tpb(int N, int csize, bool cols){
    int tt = pipe_tt(N);
    int tpb = cols ? ((csize == 8) ? 16 : 8) : 1;
    if (cols){ while (tpb * tt < 256 && tpb < 256) tpb *= 2; }
    else { while (tpb * tt < 256) tpb *= 2; }
    while (tpb > 1 && tpb * tt > 512) tpb /= 2;
    while (tpb > 1 && 2 * N * tpb * csize > 160 * 1024) tpb /= 2;
    return tpb;
}
__host__ __device__ constexpr int pipe_smem(int N, int csize, bool cols){
    int tpb = pipe_tpb(N, csize, cols);
    return 2 * N * tpb * csize + (cols ? 0 : tpb * pipe_padn(N) * csize);
}

template<typename T, int N, int TPB, int S, bool FWD, bool COLS, class ST>
__device__ __forceinline__ void pipe_stage(int t, int loc, c_t<T> *tile, c_t<T> *xch, c_t<T> const *__restrict__ tw,
                                           c_t<T> (&v)[16], ST &st){
    using C = c_t<T>;
    constexpr int NS = pipe_nstages(N);
    if constexpr (S < NS){
        constexpr int R = pipe_radix(N, S), Ns = pipe_ns(N, S), TWO = pipe_twoff(N, S);
        constexpr int NR = N / R, TT = pipe_tt(N), M = pipe_pe(N) / R, PADN = pipe_padn(N);
        constexpr bool LAST = (S == NS - 1);
        constexpr int LNS = cilog2(Ns), LNSR = cilog2(Ns * R);
        C const *src = (COLS || S == 0) ? tile : xch;
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            #pragma unroll
            for (int q = 0; q < R; q++){
                int p = j + q * NR;
                int ix = COLS ? (p * TPB + loc) : ((S == 0) ? (loc * N + p) : (loc * PADN + p + (p >> 4)));
                v[m * R + q] = src[ix];
            }
        }
        // the next writes go to the buffer just read (column tiles, later stages)
        if (!LAST && (COLS || S > 0)) __syncthreads();
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            int k = j & (Ns - 1);
            if constexpr (S > 0){
                C const *w = tw + TWO + k * (R - 1);
                #pragma unroll
                for (int q = 1; q < R; q++){
                    C wq = __ldg(w + q - 1);
                    v[m * R + q] = FWD ? cmul(v[m * R + q], wq) : cmulc(v[m * R + q], wq);
                }
            }
            bfly<R, FWD, C, T>(&v[m * R]);
            int ob = ((j >> LNS) << LNSR) + k;
            #pragma unroll
            for (int q = 0; q < R; q++){
                int p = ob + q * Ns;
                if constexpr (LAST) st(p, v[m * R + q]);
                else {
                    int ix = COLS ? (p * TPB + loc) : (loc * PADN + p + (p >> 4));
                    (COLS ? tile : xch)[ix] = v[m * R + q];
                }
            }
        }
        if (!LAST) __syncthreads();
        pipe_stage<T, N, TPB, S + 1, FWD, COLS>(t, loc, tile, xch, tw, v, st);
    }
}

__device__ __forceinline__ long long base_of_fast(Layout const &L, long long g){
    if (g < 0x7fffffffLL && L.count < 0x7fffffffLL){
        unsigned gg = (unsigned)g, c = (unsigned)L.count;
        unsigned q = gg / c;
        return (long long)q * L.bstride + (long long)(gg - q * c) * L.dist;
    }
    return (g / L.count) * L.bstride + (g % L.count) * L.dist;
}

// Column tiles are loaded with a 3-D tensor map over the input batch:
// (x = column in 8-byte words, y = row p of the transform, z = block), box
// (TPB columns, min(N, 256) rows, 1); one TMA op per 256 rows of a tile.
template<typename T, int N, bool FWD, bool COLS>
__global__ void __launch_bounds__(pipe_tpb(N, sizeof(c_t<T>), COLS) * pipe_tt(N))
k_c2c_pipe(Layout Li, Layout Lo, c_t<T> const *in, c_t<T> *out, c_t<T> const *__restrict__ tw,
           long long ntiles, T scale, int do_scale, int *status, const __grid_constant__ CUtensorMap tmap,
           int tswap){
    using C = c_t<T>;
    constexpr int TPB = pipe_tpb(N, sizeof(C), COLS);
    constexpr int TT = pipe_tt(N);
    constexpr int TILE = N * TPB;
    constexpr uint32_t TILE_BYTES = (uint32_t)(TILE * sizeof(C));
    extern __shared__ __align__(128) unsigned char smraw[];
    C *tiles = reinterpret_cast<C*>(smraw);
    C *xch = tiles + 2 * TILE;
    __shared__ __align__(8) uint64_t bar[2];
    int tid = threadIdx.x;
    int loc, t;
    if (COLS){ loc = tid % TPB; t = tid / TPB; } else { loc = tid / TT; t = tid % TT; }
    int warp = tid >> 5, lane = tid & 31;
    if (tid == 0){
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    if (COLS && tid == 0) prefetch_tmap(&tmap);
    auto issue = [&](long long tile, int b){
        C *dst = tiles + b * TILE;
        if (COLS){
            if (lane == 0){
                constexpr int BOXR = (N < 256) ? N : 256;
                constexpr int WPC = (int)(sizeof(C) / 8);       // 8-byte words per complex value
                long long g0 = tile * TPB;
                int blk = (int)(g0 / Li.count), c0 = (int)(g0 - (long long)blk * Li.count);
                mbar_arrive_expect_tx(&bar[b], TILE_BYTES);
                #pragma unroll
                for (int r0 = 0; r0 < N; r0 += BOXR){
                    // tswap: the map lists the block dimension before the rows (strides ascending)
                    if (tswap) tma_load_3d(dst + r0 * TPB, &tmap, c0 * WPC, blk, r0, &bar[b]);
                    else tma_load_3d(dst + r0 * TPB, &tmap, c0 * WPC, r0, blk, &bar[b]);
                }
            }
        } else if (lane == 0){
            long long base = base_of_fast(Li, tile * TPB);
            mbar_arrive_expect_tx(&bar[b], TILE_BYTES);
            bulk_g2s(dst, in + base, TILE_BYTES, &bar[b]);
        }
    };

    uint32_t phase0 = 0, phase1 = 0;
    long long tile = blockIdx.x;
    if (tile < ntiles && warp == 0) issue(tile, 0);
    for (int it = 0; tile < ntiles; tile += gridDim.x, it++){
        int b = it & 1;
        long long nxt = tile + gridDim.x;
        if (nxt < ntiles && warp == 0){
            // the buffer was last read in the previous iteration (ended by a barrier)
            fence_proxy_async_smem();
            issue(nxt, b ^ 1);
        }
        uint32_t ph = b ? phase1 : phase0;
        // every wait is bounded; if any thread gave up, the whole CTA leaves
        bool ok = mbar_wait_bounded(&bar[b], ph, status);
        if (__syncthreads_or(!ok)) return;
        if (b) phase1 ^= 1; else phase0 ^= 1;

        long long ob = base_of_fast(Lo, tile * TPB + loc);
        long long oes = Lo.estride;
        auto st = [&](int p, C v){ out[ob + p * oes] = do_scale ? cscale(v, scale) : v; };
        C v[16];
        pipe_stage<T, N, TPB, 0, FWD, COLS>(t, loc, tiles + b * TILE, xch, tw, v, st);
        __syncthreads();
    }
}

} // namespace gbfft
