// Tensor-core form of the complex<float> 1-D transforms: the radix-16
// butterflies of a Stockham FFT are evaluated as dense 16-point DFT
// contractions on the 5th-generation tensor cores (tcgen05.mma, BF16 inputs,
// FP32 accumulation in tensor memory), with the operands split in three BF16
// terms so that the result keeps FP32 accuracy.
//
// The split is fixed-point per butterfly row (the scheme of Ozaki et al. for
// exact products on low-precision units): with 2^e above the largest |re|,
// |im| of the row's 16 twiddled inputs, every real x of the row is
//     x = 2^(e-8) (a0 + a1 / 512 + a2 / 512^2) + r,   |r| <= 2^(e-27),
// with integers |a0|, |a1|, |a2| <= 256 (exact in BF16), and every entry w of
// the 16-point DFT matrix likewise  w = 2^-8 (b0 + b1 / 512 + b2 / 512^2) + r'.
// The products of equal order o = s + t of the slices a_s, b_t are summed by
// the tensor cores into their own FP32 accumulator:
//     G_o = sum_k sum_{s+t=o} a_s b_t,   |G_o| <= 3 * 32 * 2^16 < 2^24,
// so each G_o is an exactly represented integer whatever rounding the tensor
// core applies inside the accumulation, and the only rounding left is the FP32
// (round-to-nearest) combination on the CUDA cores
//     y = 2^(e-16) (G_0 + 2^-9 (G_1 + 2^-9 G_2)).
// The order-3 and order-4 products are below 2^-27 relative and dropped.
//
// For one radix-16 stage of a tile of 4096 complex values (256 butterflies):
//   * each thread gathers the 16 inputs of its butterfly rows from the FP32
//     tile in shared memory, applies the stage twiddles in FP32 (FP64-built
//     table) and slices the row; the slices form the A operand (128 rows x
//     96 BF16 per MMA batch, [a0 | a1 | a2] x 32 reals) in the K-major
//     no-swizzle core-matrix layout;
//   * B is the real 32x32 form of the 16-point DFT matrix (three 32x32 BF16
//     slices, built once per direction on the host and copied in by each CTA);
//   * one thread issues the six slice products (two K=16 steps each) into
//     three 128x32 FP32 accumulators in TMEM and commits them to an mbarrier;
//   * each warp reads its 32 TMEM lanes back (tcgen05.ld 32x32b), combines the
//     three accumulators and writes the 16 outputs of its rows to the tile (or,
//     after the last stage, to global memory with the plan's scale).
// Lengths are 16^s * r0 with r0 in {1, 2, 4, 8}; the r0 stage runs first on
// the CUDA cores, fused with the global load.
//
// Every wait on the MMA barrier is bounded; a wait that gives up records
// DEV_TIMEOUT_MMA in the device status word, the CTA waits once more (bounded)
// for its MMAs, frees its tensor memory and returns.
#include "gbfft_common.cuh"
#include "gbfft_ptx.cuh"
#include "gbfft_internal.h"
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

namespace gbfft {

namespace {

// ---------------------------------------------------------------------------
// tcgen05 helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols){
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(slot)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish(){
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols){
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before(){ asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after(){ asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (BF16 inputs, FP32 accumulator)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate){
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
// arrive on the barrier once every MMA issued so far by this thread completed
__device__ __forceinline__ void mma_commit(uint64_t *bar){
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(bar)) : "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]){
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                   "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr) : "memory");
}
__device__ __forceinline__ void tmem_wait_ld(){ asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d){
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" :: "r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices of
// 8 rows x 16 bytes; lbo = byte distance of core matrices adjacent in K,
// sbo = byte distance of core matrices adjacent in M (or N).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo){
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 32, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

// Exponent e of a butterfly row: 2^e is above its largest |value|
// (clamped so that the scale factors stay normal floats).
__device__ __forceinline__ int row_exponent(float mx){
    int e = (mx > 0.f) ? (int)((__float_as_uint(mx) >> 23) & 0xFF) - 126 : 0;
    return max(e, -100);
}
__device__ __forceinline__ float pow2f(int k){ return __uint_as_float((uint32_t)(127 + k) << 23); }

// Three integer slices of re and im of x (already scaled by 2^(8-e)), packed
// as BF16 pairs (re in the low half).
__device__ __forceinline__ void slice3(float2 x, uint32_t &s0, uint32_t &s1, uint32_t &s2){
    float a0r = rintf(x.x), a0i = rintf(x.y);
    float rr = (x.x - a0r) * 512.f, ri = (x.y - a0i) * 512.f;
    float a1r = rintf(rr), a1i = rintf(ri);
    float a2r = rintf((rr - a1r) * 512.f), a2i = rintf((ri - a1i) * 512.f);
    __nv_bfloat162 b0 = __floats2bfloat162_rn(a0r, a0i);
    __nv_bfloat162 b1 = __floats2bfloat162_rn(a1r, a1i);
    __nv_bfloat162 b2 = __floats2bfloat162_rn(a2r, a2i);
    s0 = *reinterpret_cast<uint32_t*>(&b0);
    s1 = *reinterpret_cast<uint32_t*>(&b1);
    s2 = *reinterpret_cast<uint32_t*>(&b2);
}

// ---------------------------------------------------------------------------
// tile geometry
// ---------------------------------------------------------------------------
constexpr int kThreads = 256;      // two warpgroups, one per MMA batch: warp w reads TMEM lanes 32(w%4)..+31
constexpr int kTile = 4096;        // complex values per tile
constexpr int kRows = kTile / 16;  // radix-16 butterflies per stage and tile
constexpr int kBatches = kRows / 128;
constexpr int kAbytes = 128 * 96 * 2;   // one MMA batch: 128 rows x (3 terms x 32 reals) BF16
constexpr int kBbytes = 3 * 32 * 32 * 2;
constexpr int kChunk = 128 * 16;        // one K chunk (8 BF16) of all 128 rows = LBO of A
constexpr int kBatchCols = 128;         // TMEM columns of one batch: accumulators G_0, G_1, G_2 (32 each)
constexpr uint32_t kTmemCols = kBatchCols * kBatches;
static_assert(kBatches * 128 == kRows, "tile must hold whole MMA batches");
static_assert(kThreads == kRows, "one thread per butterfly row, one warpgroup per MMA batch");
static_assert(kTmemCols >= 32 && (kTmemCols & (kTmemCols - 1)) == 0, "TMEM allocation is a power of two >= 32");

template<int N> struct TcShape {
    static constexpr int LT = kTile / N;            // lines per tile
    static constexpr int NR16 = N / 16;             // radix-16 butterflies per line
    static constexpr int PADN = N + N / 16 + 1;     // padded line in the tile (bank spread)
    static constexpr int S16 = (N >= 4096) ? 3 : (N >= 256) ? 2 : 1;
    static constexpr int R0 = N / ((S16 == 3) ? 4096 : (S16 == 2) ? 256 : 16);
    static constexpr int DATA_BYTES = LT * PADN * 8;
    static constexpr int SMEM = kBbytes + kBatches * kAbytes + ((DATA_BYTES + 15) / 16) * 16 + 8 * kBatches + 16;
    static_assert(R0 == 1 || R0 == 2 || R0 == 4 || R0 == 8, "length must be 16^s * {1, 2, 4, 8}");
    static_assert(LT >= 1 && LT * N == kTile, "length must divide the tile");
};

// The (A slice, B slice) products kept, in order groups 0 | 1, 1 | 2, 2, 2.
__device__ __forceinline__ constexpr int term_a(int pr){ return (pr == 2 || pr == 4) ? 1 : (pr == 5) ? 2 : 0; }
__device__ __forceinline__ constexpr int term_b(int pr){ return (pr == 1 || pr == 4) ? 1 : (pr == 3) ? 2 : 0; }
__device__ __forceinline__ constexpr int group_of(int pr){ return term_a(pr) + term_b(pr); }
__device__ __forceinline__ constexpr bool group_first(int pr){ return pr == 0 || pr == 1 || pr == 3; }

__device__ __forceinline__ int sidx(int padn, int l, int p){ return l * padn + p + (p >> 4); }

struct TcArgs {
    Plan1D plan;               // radices: [r0,] 16, 16, ...
    Layout Li, Lo;
    float2 const *in;
    float2 *out;
    float2 const *tw;
    uint4 const *bmat;         // B operand image (kBbytes), built once per direction and device
    long long G, ntiles;
    float scale;
    int do_scale;
    int *status;
};

__device__ __forceinline__ bool mma_wait(uint64_t *bar, uint32_t parity, int *status){
    if (mbar_try_wait(bar, parity)) return true;
    long long t0 = clock64();
    while (true){
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > kWaitBudgetClocks){
            if (status) atomicExch(status, DEV_TIMEOUT_MMA);
            return false;
        }
    }
}

template<int N, bool FWD, bool COLS>
__global__ void __launch_bounds__(kThreads, 2) k_tc_c2c(TcArgs const a){
    using Sh = TcShape<N>;
    constexpr int LT = Sh::LT, NR16 = Sh::NR16, PADN = Sh::PADN, R0 = Sh::R0;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *Bs = smem;
    unsigned char *As = smem + kBbytes;
    float2 *D = reinterpret_cast<float2*>(smem + kBbytes + kBatches * kAbytes);
    uint64_t *bar = reinterpret_cast<uint64_t*>(smem + kBbytes + kBatches * kAbytes + ((Sh::DATA_BYTES + 15) / 16) * 16);
    uint32_t *slot = reinterpret_cast<uint32_t*>(bar + kBatches);
    int const tid = threadIdx.x, warp = tid >> 5;

    if (warp == 0){ tmem_alloc(slot, kTmemCols); tmem_relinquish(); }
    // B operand: the three DFT slices, already in the shared-memory layout
    for (int i = tid; i < kBbytes / 16; i += kThreads)
        reinterpret_cast<uint4*>(Bs)[i] = __ldg(a.bmat + i);
    if (tid == 0){
        for (int bb = 0; bb < kBatches; bb++) mbar_init(&bar[bb], 1);
        fence_mbar_init();
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t const tbase = *slot;
    uint32_t const a_base = smem_u32(As), b_base = smem_u32(Bs);

    Plan1D const &P = a.plan;
    int const first16 = (R0 > 1) ? 1 : 0;
    uint32_t phase = 0;
    bool fail = false;
    // The raw values of a tile, kPer per thread, are loaded into registers one
    // tile ahead: the loads of tile t+1 are in flight while the tensor-core
    // stages of tile t run.  Value i of a thread is element e = tid + 256 i of
    // the tile (r0 = 1), or input q of butterfly b = tid + 256 (i / r0) of
    // the leading radix-r0 stage (i % r0 = q).
    constexpr int kPer = kTile / kThreads;
    constexpr int NRr = N / R0;
    float2 pre[kPer];
    auto issue_loads = [&](long long tile){
        long long const g0 = tile * LT;
        #pragma unroll
        for (int i = 0; i < kPer / R0; i++){
            int b = tid + kThreads * i;
            int l, p0, step;
            if constexpr (R0 == 1){ l = COLS ? b % LT : b / N; p0 = COLS ? b / LT : b % N; step = 0; }
            else { l = COLS ? b % LT : b / NRr; p0 = COLS ? b / LT : b % NRr; step = NRr; }
            long long g = g0 + l;
            bool ok = g < a.G;
            long long base = ok ? base_of(a.Li, g) : 0;
            #pragma unroll
            for (int q = 0; q < R0; q++)
                pre[i * R0 + q] = ok ? __ldcs(a.in + base + (long long)(p0 + q * step) * a.Li.estride) : make_float2(0.f, 0.f);
        }
    };
    if ((long long)blockIdx.x < a.ntiles) issue_loads(blockIdx.x);
    for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x){
        long long const g0 = tile * LT;
        // ---- the tile into shared memory (through the leading radix-r0 stage)
        #pragma unroll
        for (int i = 0; i < kPer / R0; i++){
            int b = tid + kThreads * i;
            if constexpr (R0 == 1){
                int l = COLS ? b % LT : b / N, p = COLS ? b / LT : b % N;
                D[sidx(PADN, l, p)] = pre[i];
            } else {
                int l = COLS ? b % LT : b / NRr, j = COLS ? b / LT : b % NRr;
                bfly<R0, FWD, float2, float>(&pre[i * R0]);
                #pragma unroll
                for (int q = 0; q < R0; q++) D[sidx(PADN, l, j * R0 + q)] = pre[i * R0 + q];
            }
        }
        __syncthreads();
        if (tile + gridDim.x < a.ntiles) issue_loads(tile + gridDim.x);
        // ---- radix-16 stages on the tensor cores: warpgroup bb builds, and
        // reads back, MMA batch bb (thread tid owns butterfly row tid)
        for (int s = first16; s < P.nstages; s++){
            Stage const S = P.st[s];
            bool const last = (s == P.nstages - 1);
            int const row = tid, bb = tid >> 7, r = tid & 127;
            int const l = COLS ? row % LT : row / NR16, j = COLS ? row / LT : row % NR16;
            int rexp;
            {
                // A row: gather, twiddle, slice
                int k = j & (S.Ns - 1);
                float2 x[16];
                #pragma unroll
                for (int q = 0; q < 16; q++) x[q] = D[sidx(PADN, l, j + q * NR16)];
                if (k != 0){
                    float2 const *w = a.tw + S.tw + k * 15;
                    #pragma unroll
                    for (int q = 1; q < 16; q++){
                        float2 wq = __ldg(w + q - 1);
                        x[q] = FWD ? cmul(x[q], wq) : cmulc(x[q], wq);
                    }
                }
                float mx = 0.f;
                #pragma unroll
                for (int q = 0; q < 16; q++) mx = fmaxf(mx, fmaxf(fabsf(x[q].x), fabsf(x[q].y)));
                rexp = row_exponent(mx);
                float const sc = pow2f(8 - rexp);
                uint32_t rowaddr = a_base + bb * kAbytes + (r >> 3) * 128 + (r & 7) * 16;
                #pragma unroll
                for (int c = 0; c < 4; c++){
                    uint32_t h[4], m[4], lo[4];
                    #pragma unroll
                    for (int i = 0; i < 4; i++) slice3(cscale(x[4 * c + i], sc), h[i], m[i], lo[i]);
                    st_shared_v4(rowaddr + (0 + c) * kChunk, h[0], h[1], h[2], h[3]);
                    st_shared_v4(rowaddr + (4 + c) * kChunk, m[0], m[1], m[2], m[3]);
                    st_shared_v4(rowaddr + (8 + c) * kChunk, lo[0], lo[1], lo[2], lo[3]);
                }
            }
            fence_proxy_async_smem();
            tc_fence_before();
            __syncthreads();
            if (tid == 0){
                tc_fence_after();
                #pragma unroll
                for (int b2 = 0; b2 < kBatches; b2++){
                    #pragma unroll
                    for (int pr = 0; pr < 6; pr++){
                        #pragma unroll
                        for (int ks = 0; ks < 2; ks++){
                            uint64_t ad = smem_desc(a_base + b2 * kAbytes + (4 * term_a(pr) + 2 * ks) * kChunk, kChunk, 128);
                            uint64_t bd = smem_desc(b_base + term_b(pr) * 2048 + 2 * ks * 512, 512, 128);
                            mma_bf16(tbase + b2 * kBatchCols + 32 * group_of(pr), ad, bd, kIdesc,
                                     !(group_first(pr) && ks == 0));
                        }
                    }
                    mma_commit(&bar[b2]);
                }
            }
            // reconverge warp 0 before its other lanes enter the wait
            __syncwarp();
            bool const ok = mma_wait(&bar[bb], phase, a.status);
            phase ^= 1;
            tc_fence_after();
            // D row back from TMEM (every gather of the stage is done, so the
            // tile can be overwritten)
            {
                uint32_t const taddr = tbase + ((uint32_t)((warp & 3) * 32) << 16) + bb * kBatchCols;
                float y[32];
                {
                    uint32_t g1[32], g2[32];
                    tmem_ld32(taddr + 32, g1);
                    tmem_ld32(taddr + 64, g2);
                    tmem_wait_ld();
                    #pragma unroll
                    for (int i = 0; i < 32; i++) y[i] = fmaf(__uint_as_float(g2[i]), 1.f / 512.f, __uint_as_float(g1[i]));
                }
                {
                    uint32_t g0[32];
                    tmem_ld32(taddr, g0);
                    tmem_wait_ld();
                    float const os = pow2f(rexp - 16) * (last && a.do_scale ? a.scale : 1.f);
                    #pragma unroll
                    for (int i = 0; i < 32; i++) y[i] = fmaf(y[i], 1.f / 512.f, __uint_as_float(g0[i])) * os;
                }
                if (last){
                    long long g = g0 + l;
                    if (g < a.G){
                        long long base = base_of(a.Lo, g);
                        #pragma unroll
                        for (int q = 0; q < 16; q++)
                            a.out[base + (long long)(j + q * NR16) * a.Lo.estride] = make_float2(y[2 * q], y[2 * q + 1]);
                    }
                } else {
                    int hi = j >> (__ffs(S.Ns) - 1), k = j & (S.Ns - 1);
                    int ob = hi * S.Ns * 16 + k;
                    #pragma unroll
                    for (int q = 0; q < 16; q++)
                        D[sidx(PADN, l, ob + q * S.Ns)] = make_float2(y[2 * q], y[2 * q + 1]);
                }
            }
            tc_fence_before();
            if (__syncthreads_or(!ok)){ fail = true; break; }
        }
        if (fail) break;
    }
    if (fail){
        // one more bounded wait for the MMAs in flight before the memory is freed
        for (int bb = 0; bb < kBatches; bb++) mma_wait(&bar[bb], phase ^ 1, nullptr);
    }
    __syncthreads();
    if (warp == 0){
        tc_fence_after();
        tmem_dealloc(tbase, kTmemCols);
    }
}

template<auto Kfn, int SMEM>
void launch_kernel(cudaStream_t s, TcArgs const &a){
    static int done_mask = 0;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (!(done_mask & (1 << dev))){
        check_cuda(cudaFuncSetAttribute(Kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM), "smem attribute");
        // the whole unified L1 / shared array as shared memory: two CTAs per SM
        check_cuda(cudaFuncSetAttribute(Kfn, cudaFuncAttributePreferredSharedMemoryCarveout, 100), "carveout attribute");
        done_mask |= 1 << dev;
    }
    // resident CTAs per SM from the device's limits: shared memory (with the
    // per-block reservation), registers, and tensor memory (every resident
    // CTA holds kTmemCols of the SM's 512 columns)
    int smem_sm = 0, smem_rsv = 0, regs_sm = 0;
    check_cuda(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev), "device attribute");
    check_cuda(cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev), "device attribute");
    check_cuda(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev), "device attribute");
    cudaFuncAttributes fa{};
    check_cuda(cudaFuncGetAttributes(&fa, Kfn), "function attributes");
    int regs_cta = ((fa.numRegs * 32 + 255) / 256) * 256 * (kThreads / 32);
    int per_sm = std::min(smem_sm / (SMEM + smem_rsv), regs_sm / std::max(regs_cta, 1));
    per_sm = std::max(1, std::min(per_sm, (int)(512 / kTmemCols)));
    long long grid = std::min<long long>(a.ntiles, (long long)per_sm * num_sms());
    Kfn<<<(unsigned)grid, kThreads, SMEM, s>>>(a);
    check_cuda(cudaPeekAtLastError(), "tensor-core FFT launch");
}

template<int N>
void launch_n(cudaStream_t s, bool fwd, bool cols, TcArgs const &a){
    constexpr int SM = TcShape<N>::SMEM;
    if (fwd){
        if (cols) launch_kernel<k_tc_c2c<N, true, true>, SM>(s, a);
        else      launch_kernel<k_tc_c2c<N, true, false>, SM>(s, a);
    } else {
        if (cols) launch_kernel<k_tc_c2c<N, false, true>, SM>(s, a);
        else      launch_kernel<k_tc_c2c<N, false, false>, SM>(s, a);
    }
}

// The B operand of one direction: rows n = output (2m + re/im), columns
// k = input (2k' + re/im) of the real 32x32 form of the 16-point DFT, each
// entry w = 2^-8 (b0 + b1/512 + b2/512^2) (integers |b| <= 256, exact in
// BF16), three slices of 2048 bytes in the K-major core-matrix layout
// (K chunks of 8 at 512 bytes, row groups of 8 at 128 bytes).
std::vector<uint16_t> dft16_slices(bool fwd){
    std::vector<uint16_t> img(kBbytes / 2, 0);
    double const pi = 3.14159265358979323846;
    for (int n = 0; n < 32; n++){
        for (int k = 0; k < 32; k++){
            int m = n >> 1, kk = k >> 1, ro = n & 1, ri = k & 1;
            double t = pi * (double)((m * kk) & 15) / 8.0;
            double c = std::cos(t), s = std::sin(t);
            double v;
            if (fwd) v = ro == 0 ? (ri == 0 ? c : s) : (ri == 0 ? -s : c);     // exp(-i t)
            else     v = ro == 0 ? (ri == 0 ? c : -s) : (ri == 0 ? s : c);     // exp(+i t)
            double x = v * 256.0, b0 = std::nearbyint(x);
            double r = (x - b0) * 512.0, b1 = std::nearbyint(r);
            double b2 = std::nearbyint((r - b1) * 512.0);
            int off = ((k >> 3) * 512 + (n >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2) / 2;
            double b[3] = {b0, b1, b2};
            for (int u = 0; u < 3; u++){
                float f = (float)b[u];             // an integer of at most 9 bits: exact in BF16
                uint32_t bits;
                std::memcpy(&bits, &f, 4);
                img[u * 1024 + off] = (uint16_t)(bits >> 16);
            }
        }
    }
    return img;
}

uint4 const *dft16_device(bool fwd){
    static std::mutex mu;
    static std::map<int, uint4*> tables[2];
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    auto &t = tables[fwd ? 0 : 1];
    auto it = t.find(dev);
    if (it != t.end()) return it->second;
    std::vector<uint16_t> img = dft16_slices(fwd);
    uint4 *d = nullptr;
    check_cuda(cudaMalloc(&d, kBbytes), "cudaMalloc(DFT slices)");
    check_cuda(cudaMemcpy(d, img.data(), kBbytes, cudaMemcpyHostToDevice), "copy DFT slices");
    t[dev] = d;
    return d;
}

} // namespace

std::vector<int> tc_radices(int N){
    switch (N){
        case 64:   return {4, 16};
        case 128:  return {8, 16};
        case 256:  return {16, 16};
        case 512:  return {2, 16, 16};
        case 1024: return {4, 16, 16};
        case 2048: return {8, 16, 16};
        case 4096: return {16, 16, 16};
        default:   return {};
    }
}

bool tc_supported(int N){ return !tc_radices(N).empty(); }

void launch_tc_c2c(cudaStream_t s, int N, bool fwd, Layout Li, Layout Lo, void const *in, void *out, long long G,
                   double scale){
    if (G <= 0) return;
    std::vector<int> rad = tc_radices(N);
    if (rad.empty()) throw Error(ST_UNSUPPORTED, "tensor-core path: length " + std::to_string(N) + " is not 16^s * {1,2,4,8} in [64, 4096]");
    auto f = get_fft1d(N, rad);
    TcArgs a{};
    a.plan = f->plan;
    a.Li = Li; a.Lo = Lo;
    a.in = static_cast<float2 const*>(in);
    a.out = static_cast<float2*>(out);
    a.tw = static_cast<float2 const*>(f->twiddles(0, s));
    a.bmat = dft16_device(fwd);
    a.G = G;
    int lt = kTile / N;
    a.ntiles = (G + lt - 1) / lt;
    a.scale = (float)scale;
    a.do_scale = (scale != 1.0);
    a.status = device_status();
    bool cols = !(Li.estride == 1 && Lo.estride == 1);
    switch (N){
        case 64:   launch_n<64>(s, fwd, cols, a); break;
        case 128:  launch_n<128>(s, fwd, cols, a); break;
        case 256:  launch_n<256>(s, fwd, cols, a); break;
        case 512:  launch_n<512>(s, fwd, cols, a); break;
        case 1024: launch_n<1024>(s, fwd, cols, a); break;
        case 2048: launch_n<2048>(s, fwd, cols, a); break;
        default:   launch_n<4096>(s, fwd, cols, a); break;
    }
}

} // namespace gbfft
