// Pipelined complex transforms of any supported length (runtime radix plan):
// the persistent tile pipeline of the power-of-two kernels
// (lines by 1-D bulk copies, columns by 3-D tensor-map copies, both
// completing on mbarriers with bounded waits) around the runtime Stockham
// stages of the generic kernels (radices 2, 3, 4, 5, 7, 8, 11, 13, 16).
//
//   * line tiles: TPB whole lines land in shared memory unpadded; stage 0
//     reads them there and the later stages exchange through a padded
//     buffer; the last stage stores to global memory;
//   * column tiles: TPB adjacent columns land as a [row][column] tile, which
//     is the stages' exchange layout, so every stage (stage 0 included) runs
//     in place in the tile.
// With two tile slots the next tile is copied in while this one is
// transformed; with one slot (float line tiles, and float column tiles when
// no two-CTA form of two slots fits an SM's shared memory) the CTAs on an SM
// overlap each other's copies.
//
// Float lengths of a fixed list (GBFFT_RT_CT_LENGTHS) also have kernels
// compiled for their default plan (NC = N): the same pipeline with every
// radix, butterfly count, division and trip count a constant, and the
// twiddle table copied once per CTA into shared memory, transposed per stage
// (TWS).  The host picks the slots, the tile width and TWS per launch.
#pragma once
#include <cuda.h>
#include "gbfft_kernels.cuh"
#include "gbfft_ptx.cuh"
#include "gbfft_internal.h"

namespace gbfft {

enum { RT_LD_BULK = 0, RT_LD_TENSOR = 1 };

// All stages of one tile; sm_x: exchange buffer (line tiles), or the tile
// itself (column tiles).
template<int EMAX, bool FWD, bool COLS, typename T, class LD, class ST>
__device__ __forceinline__ void rt_stages(Plan1D const &P, int t, bool active, c_t<T> *sm_x, int loc, int TPB,
                                          int padn, c_t<T> const *__restrict__ tw, LD &ld, ST &st){
    Regs<T, EMAX> r;
    for (int s = 0; s < P.nstages; s++){
        Stage const S = P.st[s];
        // line tiles read stage 0 from the unpadded tile (ld); column tiles
        // read every stage from the tile in place (read, barrier, write)
        bool first = !COLS && (s == 0);
        bool tg = (s == P.nstages - 1);
        switch (S.R){
            case 16: if constexpr (EMAX >= 16) fft_stage<16, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 13: if constexpr (EMAX >= 13) fft_stage<13, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 11: if constexpr (EMAX >= 11) fft_stage<11, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 8: fft_stage<8, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 7: fft_stage<7, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 5: fft_stage<5, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 4: fft_stage<4, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            case 3: fft_stage<3, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
            default: fft_stage<2, EMAX, FWD, COLS, T>(S, t, P.T, active, first, tg, sm_x, loc, TPB, padn, tw, r, ld, st); break;
        }
    }
}

// Compile-time radix plan of one length, built by the rule of the host's
// plan builder for lengths that are not powers of two (radix-16 stages first,
// the rest of the power of two as 8x4, 8, 4 or 2, then the odd primes 13,
// 11, 7, 5, 3; twiddle offsets of the Stockham table; threads per transform
// the most that any stage needs at `emax` values per thread).  The host runs
// a compile-time kernel only when its runtime plan equals this one
// (ct_plan_matches).
struct CtPlan {
    int N, T, nstages;
    int R[kMaxStages], Ns[kMaxStages], NR[kMaxStages], tw[kMaxStages];
};

__host__ __device__ constexpr CtPlan ct_plan(int N, int emax){
    CtPlan p{};
    p.N = N; p.T = 1; p.nstages = 0;
    if (N <= 1) return p;
    int odd[kMaxStages] = {};
    int nodd = 0, n = N;
    int const primes[5] = {13, 11, 7, 5, 3};
    for (int i = 0; i < 5; i++)
        while (n % primes[i] == 0){ odd[nodd++] = primes[i]; n /= primes[i]; }
    int a = 0;
    while (n % 2 == 0){ n /= 2; a++; }
    if (n != 1) return p;                     // a prime factor without a butterfly: no plan
    int rad[kMaxStages] = {};
    int ns = 0, q = a / 4, rem = a % 4;
    int tail[2] = {0, 0}, ntail = 0;
    if (rem == 1 && q >= 1){ q -= 1; tail[0] = 8; tail[1] = 4; ntail = 2; }
    else if (rem == 1){ tail[0] = 2; ntail = 1; }
    else if (rem == 2){ tail[0] = 4; ntail = 1; }
    else if (rem == 3){ tail[0] = 8; ntail = 1; }
    for (int i = 0; i < q; i++) rad[ns++] = 16;
    for (int i = 0; i < ntail; i++) rad[ns++] = tail[i];
    for (int i = 0; i < nodd; i++) rad[ns++] = odd[i];
    int Ns = 1, off = 0, T = 1;
    for (int s = 0; s < ns; s++){
        int R = rad[s];
        p.R[s] = R; p.Ns[s] = Ns; p.NR[s] = N / R; p.tw[s] = off;
        if (s > 0) off += Ns * (R - 1);
        int per = emax / R;
        int need = (N / R + per - 1) / per;
        if (need > T) T = need;
        Ns *= R;
    }
    p.nstages = ns;
    p.T = T;
    return p;
}

// Twiddles of the compile-time plan of N (complex values): stage s > 0 holds
// Ns * (R - 1) of them.
__host__ __device__ constexpr int ct_twiddles(int N, int emax){
    CtPlan const p = ct_plan(N, emax);
    int n = 0;
    for (int s = 1; s < p.nstages; s++) n += p.Ns[s] * (p.R[s] - 1);
    return n;
}

// Whether the runtime plan of a transform is the compile-time plan of NC.
template<int NC>
inline bool ct_plan_matches(Plan1D const &P){
    constexpr CtPlan c = ct_plan(NC, kEmax);
    if (c.nstages == 0 || P.N != NC || P.nstages != c.nstages || P.T != c.T) return false;
    for (int s = 0; s < c.nstages; s++)
        if (P.st[s].R != c.R[s] || P.st[s].Ns != c.Ns[s] || P.st[s].NR != c.NR[s] || P.st[s].tw != c.tw[s])
            return false;
    return true;
}

// One Stockham stage with every size a constant: radix R, NS = product of
// the previous radices, NR = N / R butterflies, TWO = the stage's twiddle
// offset, TT threads per transform (each owns butterflies t, t + TT, ...).
// FIRST: stage 0 of line tiles, read from the unpadded tile by `ld`; TG: the
// last stage, stored to global memory by `st`.  Otherwise the exchange of
// fft_stage (gbfft_kernels.cuh).  TWS: tw is the twiddle table in shared
// memory, each stage's block transposed to [q - 1][k] (twiddle q of
// butterfly column k at TWO + (q - 1) * NS + k), so that a warp's threads,
// which hold consecutive k, read consecutive entries; else the Stockham
// table in global memory ([k][q - 1]).
template<int R, int NS, int NR, int TWO, int TT, int EMAX, bool FWD, bool COLS, bool FIRST, bool TG, bool TWS,
         typename T, class LD, class ST>
__device__ __forceinline__ void fft_stage_ct(int t, bool active, c_t<T> *sm, int loc, int TPB, int padn,
                                             c_t<T> const *tw, Regs<T, EMAX> &r, LD &ld, ST &st){
    using C = c_t<T>;
    constexpr int MU = (NR + TT - 1) / TT;            // butterflies per thread, at most
    static_assert(MU * R <= EMAX, "stage does not fit the register file");
    #pragma unroll
    for (int m = 0; m < MU; m++){
        int j = t + m * TT;
        if (active && ((m + 1) * TT <= NR || j < NR)){
            #pragma unroll
            for (int q = 0; q < R; q++){
                if constexpr (FIRST) r.v[m * R + q] = ld(j + q * NR);
                else r.v[m * R + q] = sm[sm_index<COLS>(j + q * NR, loc, TPB, padn)];
            }
        }
    }
    if constexpr (!FIRST) __syncthreads();
    #pragma unroll
    for (int m = 0; m < MU; m++){
        int j = t + m * TT;
        if (active && ((m + 1) * TT <= NR || j < NR)){
            int hi = j / NS;
            int k = j - hi * NS;
            if constexpr (NS > 1){
                if (k != 0){
                    #pragma unroll
                    for (int q = 1; q < R; q++){
                        C wq = TWS ? tw[TWO + (q - 1) * NS + k] : __ldg(tw + TWO + k * (R - 1) + q - 1);
                        r.v[m * R + q] = FWD ? cmul(r.v[m * R + q], wq) : cmulc(r.v[m * R + q], wq);
                    }
                }
            }
            bfly<R, FWD, C, T>(&r.v[m * R]);
            int ob = hi * NS * R + k;
            #pragma unroll
            for (int q = 0; q < R; q++){
                if constexpr (TG) st(ob + q * NS, r.v[m * R + q]);
                else sm[sm_index<COLS>(ob + q * NS, loc, TPB, padn)] = r.v[m * R + q];
            }
        }
    }
    if constexpr (!TG) __syncthreads();
}

// Stages S.. of the compile-time plan of NC.
template<int NC, int S, int EMAX, bool FWD, bool COLS, bool TWS, typename T, class LD, class ST>
__device__ __forceinline__ void rt_stages_ct(int t, bool active, c_t<T> *sm_x, int loc, int TPB, int padn,
                                             c_t<T> const *tw, Regs<T, EMAX> &r, LD &ld, ST &st){
    constexpr CtPlan P = ct_plan(NC, EMAX);
    if constexpr (S < P.nstages){
        fft_stage_ct<P.R[S], P.Ns[S], P.NR[S], P.tw[S], P.T, EMAX, FWD, COLS, !COLS && S == 0, S == P.nstages - 1, TWS,
                     T>(t, active, sm_x, loc, TPB, padn, tw, r, ld, st);
        rt_stages_ct<NC, S + 1, EMAX, FWD, COLS, TWS, T>(t, active, sm_x, loc, TPB, padn, tw, r, ld, st);
    }
}

// Copies the twiddles of stages S.. of the compile-time plan of NC from the
// Stockham table (stage block [k][q - 1]) to shared memory ([q - 1][k]).
template<int NC, int S, int EMAX, typename C>
__device__ __forceinline__ void ct_copy_twiddles(C *tws, C const *__restrict__ tw){
    constexpr CtPlan P = ct_plan(NC, EMAX);
    if constexpr (S < P.nstages){
        constexpr int R1 = P.R[S] - 1, NS = P.Ns[S], TWO = P.tw[S];
        for (int i = threadIdx.x; i < NS * R1; i += blockDim.x){
            int k = i / R1, q1 = i - k * R1;
            tws[TWO + q1 * NS + k] = __ldg(tw + TWO + i);
        }
        ct_copy_twiddles<NC, S + 1, EMAX>(tws, tw);
    }
}

// float: compiled for two 512-thread CTAs per SM (64 registers, no spills);
// the line tiles of a compiled plan (at most 256 threads, three CTAs per SM
// by shared memory) for three 256-thread CTAs (85 registers).
// NC: 0 for the runtime plan, else the length whose compile-time plan the
// stages run (constant sizes, divisions and trip counts); TWS (NC != 0): its
// twiddles copied to shared memory (the host adds their bytes), else read
// from the global table.
template<typename T, bool FWD, bool COLS, int LOADER, int NC, bool TWS>
__global__ void __launch_bounds__((NC != 0 && !COLS) ? 256 : 512,
                                  (NC != 0 && !COLS) ? 3 : (sizeof(T) == 4 ? 2 : 1))
k_pipe_rt(PipeRtParams const __grid_constant__ P, const __grid_constant__ CUtensorMap tmap){
    using C = c_t<T>;
    constexpr int EMAX = kEmax;
    constexpr int TC = ct_plan(NC, EMAX).T;
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar[2];
    int const N = NC ? NC : P.plan.N, TPB = P.tpb;
    int const Tt = NC ? TC : P.plan.T;
    int const padn = padded_len(N);
    long long const TILE = (long long)TPB * N;             // complex values per tile buffer
    C *tiles = reinterpret_cast<C*>(smraw);
    int const nbuf = P.nbuf;
    C *xline = tiles + nbuf * TILE;                        // line tiles: padded exchange buffer
    int const tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int loc, t;
    thread_map<COLS>(TPB, Tt, loc, t);
    Layout const Li = P.Li, Lo = P.Lo;

    if (tid == 0){
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        if (LOADER == RT_LD_TENSOR) prefetch_tmap(&tmap);
    }
    // compile-time plans: the twiddle table, transposed per stage, after the
    // tile slots (and the exchange buffer of line tiles)
    C *tws = tiles + nbuf * TILE + (COLS ? 0 : (long long)TPB * padn);
    if constexpr (NC != 0 && TWS) ct_copy_twiddles<NC, 1, EMAX>(tws, reinterpret_cast<C const*>(P.tw));
    __syncthreads();

    auto tile_origin = [&](long long tile, long long &blk, long long &c0){
        if (COLS){ blk = tile / P.tiles_per_block; c0 = (tile - blk * P.tiles_per_block) * TPB; }
        else { blk = 0; c0 = tile * (long long)TPB; }
    };
    auto issue = [&](long long tile, int b){
        if (warp != 0 || lane != 0) return;
        long long blk, c0;
        tile_origin(tile, blk, c0);
        unsigned char *dst = reinterpret_cast<unsigned char*>(tiles + b * TILE);
        if constexpr (LOADER == RT_LD_TENSOR){
            constexpr int WPE = (sizeof(C) >= 8) ? (int)sizeof(C) / 8 : 1;
            mbar_arrive_expect_tx(&bar[b], (uint32_t)((long long)N * TPB * sizeof(C)));
            int x = (int)(c0 * WPE);
            for (int r0 = 0; r0 < N; r0 += P.boxr){
                unsigned char *d = dst + (size_t)r0 * TPB * sizeof(C);
                if (P.tswap) tma_load_3d(d, &tmap, x, (int)blk, r0, &bar[b]);
                else tma_load_3d(d, &tmap, x, r0, (int)blk, &bar[b]);
            }
        } else {
            long long lines = ((long long)TPB < P.G - c0) ? (long long)TPB : (P.G - c0);
            uint32_t bytes = (uint32_t)(lines * N * sizeof(C));
            mbar_arrive_expect_tx(&bar[b], bytes);
            bulk_g2s(dst, reinterpret_cast<C const*>(P.in) + base_of(Li, c0), bytes, &bar[b]);
        }
    };

    uint32_t ph0 = 0, ph1 = 0;
    long long tile = blockIdx.x;
    if (nbuf == 2 && tile < P.ntiles) issue(tile, 0);
    T const sc = (T)P.scale;
    C const *tw = reinterpret_cast<C const*>(P.tw);
    for (int it = 0; tile < P.ntiles; tile += gridDim.x, it++){
        int b = (nbuf == 2) ? (it & 1) : 0;
        if (nbuf == 2){
            long long nxt = tile + gridDim.x;
            if (nxt < P.ntiles){
                if (warp == 0) fence_proxy_async_smem();
                issue(nxt, b ^ 1);
            }
        } else {
            // one slot: this tile's copy, after the last iteration's barrier
            if (warp == 0) fence_proxy_async_smem();
            issue(tile, 0);
        }
        bool ok = mbar_wait_bounded(&bar[b], b ? ph1 : ph0, P.status);
        if (__syncthreads_or(!ok)) return;
        if (b) ph1 ^= 1; else ph0 ^= 1;

        C *tb = tiles + b * TILE;
        long long blk, c0;
        tile_origin(tile, blk, c0);
        bool active, valid;
        long long oa = 0;
        if (COLS){
            long long ca = c0 + loc;
            valid = ca < Li.count;
            oa = blk * Lo.bstride + ca * Lo.dist;
        } else {
            long long g = c0 + loc;
            valid = g < P.G;
            if (valid) oa = base_of(Lo, g);
        }
        active = valid && (t < Tt) && (loc < TPB);
        C *out = reinterpret_cast<C*>(P.out);
        long long const oes = Lo.estride;
        auto ld = [&](int p) -> C { return tb[(long long)loc * N + p]; };
        auto st = [&](int p, C x){ out[oa + p * oes] = P.do_scale ? cscale(x, sc) : x; };
        if constexpr (NC != 0){
            Regs<T, EMAX> r;
            rt_stages_ct<NC, 0, EMAX, FWD, COLS, TWS, T>(t, active, COLS ? tb : xline, loc, TPB, padn,
                                                         TWS ? tws : tw, r, ld, st);
        } else {
            rt_stages<EMAX, FWD, COLS, T>(P.plan, t, active, COLS ? tb : xline, loc, TPB, padn, tw, ld, st);
        }
        __syncthreads();
    }
}

} // namespace gbfft
