// Fused middle pass of a 3-D circular convolution,
//   out = IFFT( FFT(x) .* FFT(y) )      (benchmarks/convolution.cpp: FFT, pointwise product, IFFT)
// The two other dimensions of x (and y) are transformed by the ordinary
// forward passes; this pass then takes one dimension of columns through
//   forward FFT  ->  pointwise product with y's spectrum (or x's own: X .* X)
//   ->  scale  ->  backward FFT
// without leaving shared memory, so the spectrum is never written to HBM and
// the product costs no pass of its own.  Column tiles come in by 3-D
// tensor-map copies (one map per operand, both completing on the tile's
// mbarrier, bounded waits) into two or three slots as in the pipelined
// transforms; every radix stage runs in place in the tile.
#pragma once
#include <cuda.h>
#include "gbfft_pipe.cuh"

namespace gbfft {

struct ConvParams {
    Layout L;                  // columns of the pass (same layout for x, y and the result)
    void *x;                   // x, transformed along the other dimensions; overwritten by the result
    void const *y;             // y, transformed along the other dimensions (null: self-convolution)
    void const *tw;            // Stockham twiddles of the pipelined radix plan of length N
    long long ntiles;
    long long tiles_per_block; // column tiles covering one block of `count` columns
    int tswap;
    double scale;
    int *status;
};

// columns per tile: the column tile of the pipelined transforms, halved until
// two tile slots of every operand fit in shared memory and a tile
// row is at most 256 tensor words (the box limit of a tensor-map copy)
__host__ __device__ constexpr int conv_tpb(int N, int csize, bool two){
    int tpb = pipe_tpb(N, csize, true);
    int bufs = two ? 4 : 2;
    while (tpb > 1 && bufs * N * tpb * csize > 200 * 1024) tpb /= 2;
    while (tpb > 1 && tpb * (csize / 8) > 256) tpb /= 2;
    return tpb;
}
__host__ __device__ constexpr int conv_threads(int N, int csize, bool two){ return conv_tpb(N, csize, two) * pipe_tt(N); }
// tile slots per operand: three (two tiles in flight while one is
// transformed) for a self-convolution whose two slots already take more than
// half of an SM's shared memory, two otherwise
__host__ __device__ constexpr int conv_nbuf(int N, int csize, bool two){
    return (!two && 2 * N * conv_tpb(N, csize, two) * csize > 114 * 1024 &&
            3 * N * conv_tpb(N, csize, two) * csize <= 200 * 1024) ? 3 : 2;
}
__host__ __device__ constexpr int conv_smem(int N, int csize, bool two){
    return (two ? 2 : 1) * conv_nbuf(N, csize, two) * N * conv_tpb(N, csize, two) * csize;
}

// The last forward stage L of the pipelined radix plan of one column, in
// registers: reads the positions j + q N/R stage L reads (the tile itself
// when L = 0), applies its twiddles and butterflies; the results sit at the
// positions stage L writes (natural frequency order).
template<typename T, int N, int TPB>
__device__ __forceinline__ void conv_last_forward(int t, int loc, c_t<T> const *tile, c_t<T> const *__restrict__ tw,
                                                  c_t<T> (&v)[16]){
    using C = c_t<T>;
    constexpr int L = pipe_nstages(N) - 1;
    constexpr int R = pipe_radix(N, L), Ns = pipe_ns(N, L), TWO_ = pipe_twoff(N, L);
    constexpr int NR = N / R, TT = pipe_tt(N), M = pipe_pe(N) / R;
    #pragma unroll
    for (int m = 0; m < M; m++){
        int j = t + m * TT;
        #pragma unroll
        for (int q = 0; q < R; q++) v[m * R + q] = tile[(j + q * NR) * TPB + loc];
        if constexpr (L > 0){
            int k = j & (Ns - 1);
            C const *w = tw + TWO_ + k * (R - 1);
            #pragma unroll
            for (int q = 1; q < R; q++) v[m * R + q] = cmul(v[m * R + q], __ldg(w + q - 1));
        }
        bfly<R, true, C, T>(&v[m * R]);
    }
}

// Adjoint (conjugate transpose) of forward stage S, in place in a column
// tile: reads the positions stage S writes, inverse butterflies, conjugate
// twiddles, writes the positions stage S reads (S == 0: through st, to HBM).
// Run for S = L-1 .. 0 after the adjoint of stage L, the adjoints give the
// unnormalised backward transform (F^H = N F^-1).
template<typename T, int N, int TPB, int S, class ST>
__device__ __forceinline__ void conv_adjoint(int t, int loc, c_t<T> *tile, c_t<T> const *__restrict__ tw,
                                             c_t<T> (&v)[16], ST &st){
    using C = c_t<T>;
    if constexpr (S >= 0){
        constexpr int R = pipe_radix(N, S), Ns = pipe_ns(N, S), TWO_ = pipe_twoff(N, S);
        constexpr int NR = N / R, TT = pipe_tt(N), M = pipe_pe(N) / R;
        constexpr int LNS = cilog2(Ns), LNSR = cilog2(Ns * R);
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            int k = j & (Ns - 1);
            int ob = ((j >> LNS) << LNSR) + k;
            #pragma unroll
            for (int q = 0; q < R; q++) v[m * R + q] = tile[(ob + q * Ns) * TPB + loc];
        }
        if constexpr (S > 0) __syncthreads();       // everyone has read before the tile is rewritten
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * TT;
            bfly<R, false, C, T>(&v[m * R]);
            if constexpr (S > 0){
                int k = j & (Ns - 1);
                C const *w = tw + TWO_ + k * (R - 1);
                #pragma unroll
                for (int q = 1; q < R; q++) v[m * R + q] = cmulc(v[m * R + q], __ldg(w + q - 1));
            }
            #pragma unroll
            for (int q = 0; q < R; q++){
                int p = j + q * NR;
                if constexpr (S == 0) st(p, v[m * R + q]);
                else tile[p * TPB + loc] = v[m * R + q];
            }
        }
        if constexpr (S > 0) __syncthreads();
        conv_adjoint<T, N, TPB, S - 1>(t, loc, tile, tw, v, st);
    }
}

template<typename T, int N, bool TWO>
__global__ void __launch_bounds__(conv_threads(N, sizeof(c_t<T>), TWO))
k_conv_cols(ConvParams P, const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmy){
    using C = c_t<T>;
    constexpr int TPB = conv_tpb(N, sizeof(C), TWO);
    constexpr int TILE = N * TPB;                       // complex values per tile buffer
    constexpr int BOXR = (N < 256) ? N : 256;           // rows per tensor-map copy
    constexpr int WPE = (int)sizeof(C) / 8;             // 8-byte tensor words per value
    constexpr int NBUF = conv_nbuf(N, (int)sizeof(C), TWO);
    extern __shared__ __align__(128) unsigned char smraw[];
    C *tiles = reinterpret_cast<C*>(smraw);             // x tiles [0, NBUF), y tiles [NBUF, 2 NBUF)
    __shared__ __align__(8) uint64_t bar[NBUF];
    int const tid = threadIdx.x, warp = tid >> 5;
    int const loc = tid % TPB, t = tid / TPB;
    Layout const L = P.L;

    if (tid == 0){
        #pragma unroll
        for (int i = 0; i < NBUF; i++) mbar_init(&bar[i], 1);
        fence_mbar_init();
        prefetch_tmap(&tmx);
        if (TWO) prefetch_tmap(&tmy);
    }
    __syncthreads();

    auto tile_origin = [&](long long tile, long long &blk, long long &c0){
        blk = tile / P.tiles_per_block;
        c0 = (tile - blk * P.tiles_per_block) * TPB;
    };
    auto load = [&](CUtensorMap const *m, C *dst, long long blk, long long c0, uint64_t *b){
        int x = (int)(c0 * WPE);
        #pragma unroll
        for (int r0 = 0; r0 < N; r0 += BOXR){
            unsigned char *d = reinterpret_cast<unsigned char*>(dst + (size_t)r0 * TPB);
            if (P.tswap) tma_load_3d(d, m, x, (int)blk, r0, b);
            else tma_load_3d(d, m, x, r0, (int)blk, b);
        }
    };
    auto issue = [&](long long tile, int b){
        if (tid != 0) return;
        long long blk, c0;
        tile_origin(tile, blk, c0);
        // out-of-range columns are zero-filled and still count as transferred bytes
        mbar_arrive_expect_tx(&bar[b], (uint32_t)((TWO ? 2 : 1) * TILE * sizeof(C)));
        load(&tmx, tiles + b * TILE, blk, c0, &bar[b]);
        if (TWO) load(&tmy, tiles + (NBUF + b) * TILE, blk, c0, &bar[b]);
    };

    uint32_t phase = 0;                                 // bit b: parity of the next wait on bar[b]
    long long tile = blockIdx.x;
    #pragma unroll
    for (int i = 0; i < NBUF - 1; i++){
        long long tl = tile + (long long)i * gridDim.x;
        if (tl < P.ntiles) issue(tl, i);
    }
    T const sc = (T)P.scale;
    C const *tw = reinterpret_cast<C const*>(P.tw);
    C *out = reinterpret_cast<C*>(P.x);
    for (int it = 0; tile < P.ntiles; tile += gridDim.x, it++){
        int b = it % NBUF;
        // the tile NBUF - 1 ahead goes into the slot consumed last iteration
        long long nxt = tile + (long long)(NBUF - 1) * gridDim.x;
        if (nxt < P.ntiles){
            if (warp == 0) fence_proxy_async_smem();
            issue(nxt, (it + NBUF - 1) % NBUF);
        }
        bool ok = mbar_wait_bounded(&bar[b], (phase >> b) & 1u, P.status);
        if (__syncthreads_or(!ok)) return;
        phase ^= 1u << b;

        C *tx = tiles + b * TILE;
        C *ty = tiles + (NBUF + b) * TILE;
        long long blk, c0;
        tile_origin(tile, blk, c0);
        long long const ca = c0 + loc;
        bool const valid = ca < L.count;
        long long const oa = blk * L.bstride + ca * L.dist;
        constexpr int NS = pipe_nstages(N);
        constexpr int LR = pipe_radix(N, NS - 1), LNR = N / LR, LM = pipe_pe(N) / LR, TT = pipe_tt(N);
        C v[16], vy[16];
        auto none = [&](int, C){};
        auto st = [&](int p, C z){ if (valid) out[oa + (long long)p * L.estride] = z; };
        // forward stages but the last of the column(s), in place in the tiles
        if constexpr (TWO){
            auto ldy = [&](int p) -> C { return ty[p * TPB + loc]; };
            pstage<T, N, TPB, 0, true, true, false, NS - 1>(t, loc, ty, tw, v, ldy, none);
            conv_last_forward<T, N, TPB>(t, loc, ty, tw, vy);
        }
        auto ldx = [&](int p) -> C { return tx[p * TPB + loc]; };
        pstage<T, N, TPB, 0, true, true, false, NS - 1>(t, loc, tx, tw, v, ldx, none);
        // the last forward stage, the scaled pointwise product and the adjoint
        // of that stage in registers: the thread writes back the very
        // positions it read, so no exchange is needed
        conv_last_forward<T, N, TPB>(t, loc, tx, tw, v);
        #pragma unroll
        for (int i = 0; i < 16; i++){
            if (i < pipe_pe(N)) v[i] = cscale(cmul(v[i], TWO ? vy[i] : v[i]), sc);
        }
        {
            constexpr int S = NS - 1, Ns = pipe_ns(N, S), TWO_ = pipe_twoff(N, S);
            #pragma unroll
            for (int m = 0; m < LM; m++){
                int j = t + m * TT;
                bfly<LR, false, C, T>(&v[m * LR]);
                if constexpr (S > 0){
                    int k = j & (Ns - 1);
                    C const *w = tw + TWO_ + k * (LR - 1);
                    #pragma unroll
                    for (int q = 1; q < LR; q++) v[m * LR + q] = cmulc(v[m * LR + q], __ldg(w + q - 1));
                }
                #pragma unroll
                for (int q = 0; q < LR; q++){
                    int p = j + q * LNR;
                    if constexpr (S == 0) st(p, v[m * LR + q]);
                    else tx[p * TPB + loc] = v[m * LR + q];
                }
            }
            if constexpr (S > 0) __syncthreads();
        }
        // the adjoints of the earlier stages: the backward transform, last one to HBM
        conv_adjoint<T, N, TPB, NS - 2>(t, loc, tx, tw, v, st);
        __syncthreads();
    }
}

} // namespace gbfft
