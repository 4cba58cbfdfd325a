// The persistent batch kernel (k_batch) and the unit table it walks; the
// kernel template is instantiated for 16 and for 8 values per thread in
// gbfft_batch_e16.cu / gbfft_batch_e8.cu, the host side is gbfft_batch.cu.
#pragma once
#include "gbfft_batch.h"
#include "gbfft_kernels.cuh"
#include "gbfft_ptx.cuh"

namespace gbfft {


struct BatchUnit {
    int kind;            // K_R2C, K_C2R, K_C2C_F, K_C2C_B
    int cols;            // column layout (1) or lines (0)
    int plan;            // index into the plan table
    int tpb;             // transforms (or pairs) per tile
    int src, dst;        // buffers: 0 input, 1 output, 2 workspace
    int dep;             // unit that must complete first (-1: none)
    int dep_extra;       // tiles awaited beyond the dependency's own (0; 1 only under hold_dependencies)
    int last;            // carries the scale
    long long G;         // transforms of this pass
    long long tiles, tile0;
    long long in_off, out_off;   // element offsets into the source / destination buffer
    Layout Li, Lo;
    double scale;
    int pf;              // the input of a tile can be copied ahead into shared memory (lines back to back, or adjacent columns)
};

// Copy of a tile's input into shared memory: `rows` rows of `rowbytes`
// contiguous bytes, srcstride apart in global memory and dststride apart in
// shared memory (every figure a multiple of 16 bytes).
struct TileCopy {
    unsigned char const *src;
    long long srcstride;
    int rows, rowbytes, dststride;
};

// The copy plan of tile lt of unit U, or false when the tile does not meet
// the 16-byte granularity of the asynchronous copy (or spans two blocks).
// Shared-memory layout: lines back to back (what tile_r2c / tile_c2r /
// tile_c2c read for line tiles), or one row of TPB columns per element
// position (column tiles).
template<typename T>
__device__ __forceinline__ bool tile_copy_plan(BatchUnit const &U, Plan1D const &P, BatchBufs const &bufs, long long lt,
                                               TileCopy &tc){
    using C = c_t<T>;
    if (!U.pf) return false;
    unsigned char const *srcb = reinterpret_cast<unsigned char const*>(U.src == 0 ? bufs.in : (U.src == 1 ? bufs.out : bufs.work));
    int const N = P.N;
    if (!U.cols){
        int const per = (U.kind == K_R2C || U.kind == K_C2R) ? 2 : 1;
        int const len = (U.kind == K_C2R) ? N / 2 + 1 : N;
        long long const es = (U.kind == K_R2C) ? (long long)sizeof(T) : (long long)sizeof(C);
        long long const first = lt * (long long)U.tpb * per;
        long long const lines = min((long long)U.tpb * per, U.G - first);
        unsigned char const *src = srcb + (U.in_off + first * len) * es;
        long long const bytes = lines * len * es;
        if ((reinterpret_cast<uintptr_t>(src) & 15) || (bytes & 15)) return false;
        tc.src = src; tc.srcstride = 0; tc.rows = 1; tc.rowbytes = (int)bytes; tc.dststride = 0;
        return true;
    }
    long long const es = sizeof(C);
    long long const g0 = lt * (long long)U.tpb;
    long long const W = min((long long)U.tpb, U.G - g0);
    long long const blk = g0 / U.Li.count, c0 = g0 - blk * U.Li.count;
    if (c0 + W > U.Li.count) return false;
    unsigned char const *src = srcb + (U.in_off + blk * U.Li.bstride + c0) * es;
    // both sides of every 16-byte copy aligned: the source start and row
    // stride, the row length, and the shared-memory row stride (TPB columns)
    if ((reinterpret_cast<uintptr_t>(src) & 15) || ((W * es) & 15) || ((U.Li.estride * es) & 15) ||
        (((long long)U.tpb * es) & 15))
        return false;
    tc.src = src; tc.srcstride = U.Li.estride * es; tc.rows = N; tc.rowbytes = (int)(W * es);
    tc.dststride = (int)(U.tpb * es);
    return true;
}

// 16-byte asynchronous copy global -> shared through L2 only (.cg): the
// data was written by other CTAs of the same launch, so this SM's L1 may
// hold stale lines of it
__device__ __forceinline__ void cp_async_cg16(void *dst, void const *src){
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(smem_u32(dst)), "l"(src) : "memory");
}

// CTAs per SM the batch kernels are compiled for (registers per thread
// <= 65536 / (256 x this)); float measured best at 4, double kept at 2
template<typename T, int EMAX = 16, bool R2C = false> constexpr int batch_ctas_per_sm(){
    // the float kernels with 16 values per thread: three CTAs (80 registers,
    // about 1 KB of spill code) beat four (64 registers, 3-5 KB): 1.15
    // against 1.22 ms per step of 256 r2c boxes (five: 1.42-1.51), 1.87
    // against 2.19 ms for the same boxes as c2c
    return sizeof(T) == 4 ? ((EMAX == 16) ? 3 : 4) : 2;
}

// scaling: 0 none, 1 full (1/N of each box), 2 symmetric.  One kernel per
// direction: the forward one holds the r2c and forward c2c tile paths, the
// backward one the backward c2c and c2r paths (fewer paths, fewer
// registers), compiled for several CTAs per SM: the stage-0 loads of small
// tiles are latency-bound, and more warps per SM hide them better than the
// few spills cost (256 uneven r2c float boxes, ms per step: 2.09 at one CTA
// per SM, 1.54 at two, 1.46 at three, 1.38 at four, 1.64-1.80 at five to
// eight).
// the stage-0 hook of the batch kernel: on only when the batch prefetches
template<class F> struct PrefetchHook {
    F const &f;
    bool on;
    __device__ __forceinline__ bool enabled() const { return on; }
    __device__ __forceinline__ void operator()() const { f(); }
};

// R2C: the kernel of r2c batches, whose r2c / c2r units are x passes (line
// tiles) and whose c2c units are y / z passes (column tiles): it compiles
// those paths alone (fewer registers and less spill code); without it, the
// kernel of c2c batches (c2c line and column tiles)
// S5: every radix plan of the batch is 5-smooth (radices 2, 3, 4, 5, 8, 16):
// the stages of radix 7, 11 and 13 are not compiled (fewer registers)
// TWT: every CTA first copies the twiddle tables of all nplans plans into
// shared memory at byte offset tw_off (at most kBatchTwPlans plans), each
// stage's block transposed to [q - 1][k] so that a warp reads consecutive
// entries; the stages read them there instead of from global memory
constexpr int kBatchTwPlans = 64;
template<typename T, bool FWD, int EMAX, bool R2C, bool S5, bool TWT = false>
__global__ void __launch_bounds__(256, batch_ctas_per_sm<T, EMAX, R2C>())
k_batch(BatchUnit const *__restrict__ units, int nunits, Plan1D const *__restrict__ plans,
        c_t<T> const *const *__restrict__ tws, BatchBufs bufs, unsigned long long *work_counter, int *done,
        long long total_tiles, int *status, int scaling, long long dep_budget, int pf_offset, int nplans,
        int tw_off){
    using C = c_t<T>;
    using Opts = StageOpts<S5, TWT>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C*>(smraw);
    // the twiddle tables in shared memory (TWT): table of plan p at s_twoff[p]
    __shared__ int s_twoff[TWT ? kBatchTwPlans : 1];
    C *smtw = reinterpret_cast<C*>(smraw + (tw_off > 0 ? tw_off : 0));
    if constexpr (TWT){
        if (threadIdx.x == 0){
            int o = 0;
            for (int p = 0; p < nplans && p < kBatchTwPlans; p++){
                s_twoff[p] = o;
                for (int s = 1; s < plans[p].nstages; s++) o += plans[p].st[s].Ns * (plans[p].st[s].R - 1);
            }
        }
        __syncthreads();
        for (int p = 0; p < nplans && p < kBatchTwPlans; p++){
            C const *g = tws[p];
            C *d = smtw + s_twoff[p];
            for (int s = 1; s < plans[p].nstages; s++){
                Stage const S = plans[p].st[s];
                int const R1 = S.R - 1;
                for (int i = threadIdx.x; i < S.Ns * R1; i += blockDim.x){
                    int k = i / R1, q1 = i - k * R1;
                    d[S.tw + q1 * S.Ns + k] = __ldg(g + S.tw + i);
                }
            }
        }
    }
    // prefetch buffer after the exchange buffer (pf_offset < 0: no prefetch)
    unsigned char *pfbuf = smraw + (pf_offset > 0 ? pf_offset : 0);
    __shared__ long long s_tile, s_next;
    __shared__ int s_unit, s_next_unit, s_pf_cur, s_pf_next;
    __shared__ TileCopy s_copy;
    // first tile of every unit, for the tile -> unit search (shared memory
    // when it fits, else the unit table itself)
    constexpr int kUnitsInSmem = 1024;
    __shared__ long long s_tile0[kUnitsInSmem];
    int tid = threadIdx.x;
    bool const smem_units = nunits <= kUnitsInSmem;
    if (smem_units)
        for (int i = tid; i < nunits; i += blockDim.x) s_tile0[i] = units[i].tile0;
    __syncthreads();
    auto find_unit = [&](long long t) -> int {      // last unit with tile0 <= t
        int lo = 0, hi = nunits - 1;
        while (lo < hi){
            int mid = (lo + hi + 1) >> 1;
            long long t0 = smem_units ? s_tile0[mid] : units[mid].tile0;
            if (t0 <= t) lo = mid; else hi = mid - 1;
        }
        return lo;
    };
    // the next tile is claimed (and its unit found) while the current one is
    // processed, so the queue atomic's latency is hidden; the smallest
    // unfinished tile is always some CTA's current tile and depends only on
    // smaller ones, so claiming ahead cannot stall the queue
    if (tid == 0){
        s_next = (long long)atomicAdd(work_counter, 1ull);
        s_next_unit = (s_next < total_tiles) ? find_unit(s_next) : 0;
        s_pf_next = 0;
    }
    __syncthreads();
    while (true){
        // thread 0 takes the claimed tile, claims the next one and waits for
        // the taken tile's pass dependency; one barrier hands all of it to the CTA
        bool ok = true;
        if (tid == 0){
            s_tile = s_next;
            s_unit = s_next_unit;
            s_pf_cur = s_pf_next;
            s_pf_next = 0;
            if (s_tile < total_tiles){
                long long nx = (long long)atomicAdd(work_counter, 1ull);
                s_next = nx;
                s_next_unit = (nx < total_tiles) ? find_unit(nx) : 0;
                BatchUnit const &W = units[s_unit];
                // a prefetched tile's dependency was met before its copy was issued
                if (W.dep >= 0 && !s_pf_cur){
                    long long need = units[W.dep].tiles + W.dep_extra;
                    volatile int *d = done + W.dep;
                    if (*d < need){
                        long long t0 = clock64();
                        while (*d < need){
                            if (clock64() - t0 > dep_budget){ atomicExch(status, DEV_TIMEOUT_DEPENDENCY); ok = false; break; }
                        }
                    }
                    __threadfence();
                }
            }
        }
        if (__syncthreads_or(!ok)) return;
        long long gt = s_tile;
        int u = s_unit;
        bool const pfcur = s_pf_cur != 0;
        if (gt >= total_tiles) return;
        BatchUnit const &U = units[u];
        if (pfcur){
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();
        }
        // once stage 0 has read this tile's inputs, the claimed next tile's
        // input goes into the prefetch buffer if its dependency is met
        auto prefetch_next = [&](){
            if (tid == 0){
                int go = 0;
                if (pf_offset > 0 && s_next < total_tiles){
                    BatchUnit const &V = units[s_next_unit];
                    bool met = true;
                    if (V.dep >= 0){
                        volatile int *d = done + V.dep;
                        met = *d >= units[V.dep].tiles + V.dep_extra;
                    }
                    TileCopy tc;
                    if (met && tile_copy_plan<T>(V, plans[V.plan], bufs, s_next - V.tile0, tc)){
                        __threadfence();
                        s_copy = tc;
                        go = 1;
                    }
                }
                s_pf_next = go;
            }
            __syncthreads();
            if (s_pf_next){
                TileCopy const tc = s_copy;
                // 16-byte chunk c = r * cpr + k of the tile, this thread's
                // chunks tid, tid + blockDim, ...: (r, k) stepped without a
                // division per chunk
                int const cpr = tc.rowbytes >> 4, nt = (int)blockDim.x;
                int const step_r = nt / cpr, step_k = nt - step_r * cpr;
                int r = tid / cpr, k = tid - (tid / cpr) * cpr;
                for (; r < tc.rows; ){
                    cp_async_cg16(pfbuf + (long long)r * tc.dststride + 16 * k, tc.src + r * tc.srcstride + 16 * k);
                    r += step_r;
                    k += step_k;
                    if (k >= cpr){ k -= cpr; r++; }
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            }
        };
        PrefetchHook<decltype(prefetch_next)> const hook{prefetch_next, pf_offset > 0};
        long long lt = gt - U.tile0;
        Plan1D const &P = plans[U.plan];
        C const *tw = TWT ? static_cast<C const*>(smtw + s_twoff[U.plan]) : tws[U.plan];
        unsigned char const *srcb = reinterpret_cast<unsigned char const*>(U.src == 0 ? bufs.in : (U.src == 1 ? bufs.out : bufs.work));
        unsigned char *dstb = reinterpret_cast<unsigned char*>(U.dst == 1 ? bufs.out : bufs.work);
        double f = (scaling == 0) ? 1.0 : ((scaling == 1) ? U.scale : sqrt(U.scale));
        T sc = (T)f;
        int dsc = U.last && scaling != 0;
        C const *pfc = pfcur ? reinterpret_cast<C const*>(pfbuf) : nullptr;
        if constexpr (FWD){
            // (R2C false: the kernel of c2c batches, which have no r2c unit)
            if (R2C && U.kind == K_R2C){
                T const *in = reinterpret_cast<T const*>(srcb) + U.in_off;
                C *out = reinterpret_cast<C*>(dstb) + U.out_off;
                T const *pfr = pfcur ? reinterpret_cast<T const*>(pfbuf) : nullptr;
                // the r2c pass of a batch runs along x, the fastest dimension:
                // line tiles (the 8-value kernel compiles that path alone: it
                // then spills less, 1.44 against 1.61 ms per step of 256
                // boxes; the 16-value kernel keeps both paths, which measured
                // faster for it, 1.41 against 1.48 ms)
                if constexpr (EMAX == 8 || R2C)
                    tile_r2c<T, EMAX, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfr, hook, Opts{});
                else if (U.cols) tile_r2c<T, EMAX, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfr, hook, Opts{});
                else tile_r2c<T, EMAX, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfr, hook, Opts{});
            } else {
                C const *in = reinterpret_cast<C const*>(srcb) + U.in_off;
                C *out = reinterpret_cast<C*>(dstb) + U.out_off;
                if constexpr (R2C) tile_c2c<T, EMAX, true, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else if (U.cols) tile_c2c<T, EMAX, true, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else tile_c2c<T, EMAX, true, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
            }
        } else {
            if (R2C && U.kind == K_C2R){
                C const *in = reinterpret_cast<C const*>(srcb) + U.in_off;
                T *out = reinterpret_cast<T*>(dstb) + U.out_off;
                // the c2r pass runs along x: line tiles (as for r2c above)
                if constexpr (EMAX == 8 || R2C)
                    tile_c2r<T, EMAX, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else if (U.cols) tile_c2r<T, EMAX, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else tile_c2r<T, EMAX, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
            } else {
                C const *in = reinterpret_cast<C const*>(srcb) + U.in_off;
                C *out = reinterpret_cast<C*>(dstb) + U.out_off;
                if constexpr (R2C) tile_c2c<T, EMAX, false, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else if (U.cols) tile_c2c<T, EMAX, false, true>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
                else tile_c2c<T, EMAX, false, false>(P, U.Li, U.Lo, in, out, tw, U.G, U.tpb, sc, dsc, lt, sm, pfc, hook, Opts{});
            }
        }
        // publish completion of this tile
        __syncthreads();
        if (tid == 0){
            __threadfence();
            atomicAdd(done + u, 1);
        }
    }
}

// k_batch<T, FWD, EMAX, R2C> for EMAX = 16 (any radix plan, radices up to 16)
// and EMAX = 8 (radices up to 8: fewer registers per thread); cast to a pointer
void const *batch_kernel_e16_any(int prec, bool fwd);
void const *batch_kernel_e16_r2c(int prec, bool fwd);
void const *batch_kernel_e16_r2c5(int prec, bool fwd);
// the same (float) with the twiddle tables in shared memory
void const *batch_kernel_e16_r2c5_tw(bool fwd);
void const *batch_kernel_e8(int prec, bool fwd, bool r2c, bool s5);

} // namespace gbfft
