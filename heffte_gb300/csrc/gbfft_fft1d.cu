// Host side of one transform length: radix plan, FP64-generated twiddle
// tables, launch geometry of the batched kernels.
#include "gbfft_internal.h"
#include "gbfft_pipe.cuh"
#include <atomic>
#include <cstring>
#include <map>
#include <math.h>

namespace gbfft {

int num_sms(){
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    int &c = cached[dev & 63];
    if (c == 0){
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        c = v;
    }
    return c;
}

// ---------------------------------------------------------------------------
// Twiddle tables, computed in FP64 on the device and rounded once.
// ---------------------------------------------------------------------------
template<typename T>
__global__ void k_stockham_twiddles(Plan1D P, c_t<T> *tw){
    for (int s = 1; s < P.nstages; s++){
        Stage S = P.st[s];
        int n = S.Ns * (S.R - 1);
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x){
            int k = idx / (S.R - 1), q = idx % (S.R - 1) + 1;
            double sn, cs;
            // exp(-2 pi i q k / (Ns R)); q k < Ns R so the ratio is exact-ish in FP64
            sincospi(-2.0 * (double)(q * k) / (double)(S.Ns * S.R), &sn, &cs);
            tw[S.tw + idx] = mk<T>((T)cs, (T)sn);
        }
    }
}

// the same table as double-float pairs: each FP64 value split into a
// float and the float nearest to its remainder
__global__ void k_stockham_twiddles_df(Plan1D P, cdf *tw){
    for (int s = 1; s < P.nstages; s++){
        Stage S = P.st[s];
        int n = S.Ns * (S.R - 1);
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x){
            int k = idx / (S.R - 1), q = idx % (S.R - 1) + 1;
            double sn, cs;
            sincospi(-2.0 * (double)(q * k) / (double)(S.Ns * S.R), &sn, &cs);
            cdf w;
            w.x = df_from(cs);
            w.y = df_from(sn);
            tw[S.tw + idx] = w;
        }
    }
}

template<typename T>
__global__ void k_r2r_twiddles(int N, c_t<T> *tw){
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x){
        double sn, cs;
        sincospi(-(double)k / (2.0 * (double)N), &sn, &cs);
        tw[k] = mk<T>((T)cs, (T)sn);
    }
}

Fft1D::~Fft1D(){
    // tables live until process exit in the shared registry; freeing at
    // static destruction time may run after the CUDA runtime is torn down
}

void const *Fft1D::twiddles(int prec, cudaStream_t s){
    std::lock_guard<std::mutex> lk(mu);
    if (!tw[prec]){
        size_t es = (prec == 0) ? sizeof(float2) : sizeof(double2);
        long long cnt = std::max<long long>(tw_count, 1);
        check_cuda(cudaMalloc(&tw[prec], cnt * es), "cudaMalloc(twiddles)");
        if (tw_count > 0){
            int blocks = (int)std::min<long long>((tw_count + 255) / 256, 1024);
            if (prec == 0) k_stockham_twiddles<float><<<blocks, 256, 0, s>>>(plan, (float2*)tw[prec]);
            else k_stockham_twiddles<double><<<blocks, 256, 0, s>>>(plan, (double2*)tw[prec]);
            check_cuda(cudaPeekAtLastError(), "twiddle kernel");
        }
    }
    return tw[prec];
}

void const *Fft1D::twiddles_df(cudaStream_t s){
    std::lock_guard<std::mutex> lk(mu);
    if (!tw_df){
        long long cnt = std::max<long long>(tw_count, 1);
        check_cuda(cudaMalloc(&tw_df, cnt * sizeof(cdf)), "cudaMalloc(double-float twiddles)");
        if (tw_count > 0){
            int blocks = (int)std::min<long long>((tw_count + 255) / 256, 1024);
            k_stockham_twiddles_df<<<blocks, 256, 0, s>>>(plan, reinterpret_cast<cdf*>(tw_df));
            check_cuda(cudaPeekAtLastError(), "twiddle kernel");
        }
    }
    return tw_df;
}

void const *Fft1D::r2r_twiddles(int prec, cudaStream_t s){
    std::lock_guard<std::mutex> lk(mu);
    if (!rtw[prec]){
        size_t es = (prec == 0) ? sizeof(float2) : sizeof(double2);
        check_cuda(cudaMalloc(&rtw[prec], N * es), "cudaMalloc(r2r twiddles)");
        int blocks = std::min((N + 255) / 256, 1024);
        if (prec == 0) k_r2r_twiddles<float><<<blocks, 256, 0, s>>>(N, (float2*)rtw[prec]);
        else k_r2r_twiddles<double><<<blocks, 256, 0, s>>>(N, (double2*)rtw[prec]);
        check_cuda(cudaPeekAtLastError(), "r2r twiddle kernel");
    }
    return rtw[prec];
}

// ---------------------------------------------------------------------------
// Radix plans
// ---------------------------------------------------------------------------
static const int kRadices[] = {16, 13, 11, 8, 7, 5, 4, 3, 2};

int max_length(int){ return kMaxLength; }

std::vector<int> default_radices(int N){
    // powers of two share the radix plan (and twiddle table) of the pipelined kernels
    std::vector<int> pr = pipe_radices(N);
    if (!pr.empty()) return pr;
    std::vector<int> r;
    int n = N;
    for (int p : {13, 11, 7, 5, 3}){
        while (n % p == 0){ r.push_back(p); n /= p; }
    }
    int a = 0;
    while (n % 2 == 0){ n /= 2; a++; }
    if (n != 1) return {};  // a prime factor without a butterfly
    // powers of two: as many radix-16 stages as possible, remainder 8/4 (or 8x4 for 2^1 with a 16 to spare)
    std::vector<int> p2;
    int q = a / 4, rem = a % 4;
    if (rem == 1 && q >= 1){ q -= 1; p2.push_back(8); p2.push_back(4); }
    else if (rem == 1) p2.push_back(2);
    else if (rem == 2) p2.push_back(4);
    else if (rem == 3) p2.push_back(8);
    for (int i = 0; i < q; i++) p2.insert(p2.begin(), 16);
    // radix-16 stages first, odd primes after
    std::vector<int> out = p2;
    out.insert(out.end(), r.begin(), r.end());
    return out;
}

static void fast_div_params(int d, uint32_t &mul, int &shift){
    int l = 0;
    while ((1LL << l) < d) l++;
    unsigned long long m = ((1ULL << 32) * ((1ULL << l) - (unsigned long long)d)) / (unsigned long long)d + 1ULL;
    mul = (uint32_t)m;
    shift = l;
}

static Plan1D build_plan(int N, std::vector<int> const &radices, long long &tw_count){
    Plan1D P{};
    P.N = N;
    P.nstages = (int)radices.size();
    if (P.nstages > kMaxStages) throw Error(ST_UNSUPPORTED, "too many radix stages");
    int Ns = 1, off = 0, T = 1;
    for (int s = 0; s < P.nstages; s++){
        int R = radices[s];
        Stage &S = P.st[s];
        S.R = R; S.Ns = Ns; S.NR = N / R; S.tw = off;
        fast_div_params(Ns, S.mul, S.shift);
        if (s > 0) off += Ns * (R - 1);
        int per = kEmax / R;
        T = std::max(T, (S.NR + per - 1) / per);
        Ns *= R;
    }
    if (Ns != N && N != 1) throw Error(ST_INVALID, "radix plan does not multiply to N");
    P.T = T;
    tw_count = off;
    return P;
}

bool supported_length(int N, int prec){
    return N >= 1 && N <= max_length(prec);
}

bool direct_length(int N){
    if (N == 1) return true;
    return N >= 1 && N <= kMaxDirectLength && !default_radices(N).empty();
}

// Split of a composite length with prime factors <= 13 into two direct
// lengths: powers of two first (their pipelined kernels), then the most
// balanced pair.  False when there is none.
static bool fourstep_split(int N, int &N1, int &N2){
    int best = -1;
    double best_score = -1e30;
    for (int d = std::max(2, (N + kMaxDirectLength - 1) / kMaxDirectLength); d <= kMaxDirectLength; d++){
        if (N % d) continue;
        int e = N / d;
        if (e > kMaxDirectLength || !direct_length(d) || !direct_length(e)) continue;
        auto pow2 = [](int v){ return (v & (v - 1)) == 0 ? 1 : 0; };
        double score = 100.0 * (pow2(d) + pow2(e)) - std::fabs(std::log2((double)d) - std::log2((double)e));
        if (score > best_score){ best_score = score; best = d; }
    }
    if (best < 0) return false;
    N1 = best;
    N2 = N / best;
    return true;
}

std::shared_ptr<Fft1D> get_fft1d(int N, std::vector<int> const &radices){
    // recursive: a composite length registers its factors (or Bluestein's length)
    static std::recursive_mutex mu;
    static std::map<std::pair<int, std::vector<int>>, std::shared_ptr<Fft1D>> reg;
    std::lock_guard<std::recursive_mutex> lk(mu);
    auto key = std::make_pair(N, radices);
    auto it = reg.find(key);
    if (it != reg.end()) return it->second;
    if (N < 1 || N > kMaxLength)
        throw Error(ST_UNSUPPORTED, "transform length " + std::to_string(N) + " is outside [1, " +
                    std::to_string(kMaxLength) + "]");
    if (radices.empty() && !direct_length(N)){
        auto f = std::make_shared<Fft1D>();
        f->N = N;
        int N1 = 0, N2 = 0;
        if (fourstep_split(N, N1, N2)){
            f->algo = ALGO_FOURSTEP;
            f->sub1 = get_fft1d(N1);
            f->sub2 = get_fft1d(N2);
        } else {
            int M = 1;
            while (M < 2 * N - 1) M *= 2;
            f->algo = ALGO_BLUESTEIN;
            f->sub1 = get_fft1d(M);
        }
        reg[key] = f;
        return f;
    }
    std::vector<int> rad = radices.empty() ? default_radices(N) : radices;
    if (N != 1 && rad.empty())
        throw Error(ST_UNSUPPORTED, "transform length " + std::to_string(N) + " has no radix plan");
    long long prod = 1;
    for (int r : rad){
        bool ok = false;
        for (int k : kRadices) ok = ok || (k == r);
        if (!ok) throw Error(ST_INVALID, "unsupported radix " + std::to_string(r));
        prod *= r;
    }
    if (N != 1 && prod != N) throw Error(ST_INVALID, "radix plan does not multiply to N");
    auto f = std::make_shared<Fft1D>();
    f->N = N;
    f->radices = rad;
    if (N == 1) f->radices.clear();
    f->plan = build_plan(N, f->radices, f->tw_count);
    reg[key] = f;
    return f;
}

// ---------------------------------------------------------------------------
// Launch geometry
// ---------------------------------------------------------------------------
static void geometry(Fft1D &f, int prec, bool cols, bool paired, long long G, LaunchCfg cfg, KernelArgs &a){
    int N = f.N, T = f.plan.T;
    size_t ce = (prec == 0) ? sizeof(float2) : sizeof(double2);
    size_t unit = cols ? (size_t)N * ce : (size_t)(N + (N >> 4) + 1) * ce;
    long long units = paired ? (G + 1) / 2 : G;
    int tpb;
    if (cfg.tpb > 0) tpb = cfg.tpb;
    else if (cols) tpb = std::max((prec == 0) ? (paired ? 16 : 16) : 8, (256 + T - 1) / T);
    else tpb = std::max(1, 256 / T);
    tpb = std::min(tpb, std::max(1, 512 / T));
    if (cfg.tpb <= 0 && cfg.tpb_div > 1) tpb = std::max(1, tpb / cfg.tpb_div);
    size_t budget = 100 * 1024;
    while (tpb > 1 && (size_t)tpb * unit > budget) tpb--;
    if ((size_t)tpb * unit > 227 * 1024) throw Error(ST_UNSUPPORTED, "transform length " + std::to_string(N) + " does not fit in shared memory");
    if (units < tpb) tpb = (int)std::max<long long>(units, 1);
    a.tpb = tpb;
    a.threads = tpb * T;
    a.smem = (size_t)tpb * unit;
    a.blocks = (units + tpb - 1) / tpb;
    a.plan = &f.plan;
    a.G = G;
}

static void run(cudaStream_t s, int kind, int prec, bool cols, KernelArgs &a){
    if (a.blocks <= 0) return;
    if (a.blocks > 0x7fffffffLL) throw Error(ST_UNSUPPORTED, "batch too large for one launch");
    if (prec == 0) launch_kernel_f32(s, kind, cols, a); else launch_kernel_f64(s, kind, cols, a);
}

static bool is_cols(Layout const &Li, Layout const &Lo){ return !(Li.estride == 1 && Lo.estride == 1); }

static std::atomic<int> g_variant{0};
int kernel_variant(){ return g_variant.load(); }
bool rt_compiled_plans(){ return g_variant.load() != 3; }
void set_kernel_variant(int v){ g_variant.store(v); }

// double-float by default: 1.45x the FP64-instruction passes on GB300
// (512^3 Z2Z 31.0 against 44.8 ms per forward + backward) at rel-L2 ~1e-14
static std::atomic<int> g_double_arith{DA_DOUBLE_FLOAT};
int double_arithmetic(){ return g_double_arith.load(); }
void set_double_arithmetic(int mode){ g_double_arith.store(mode); }

int *device_status(){
    static int *ptrs[64] = {nullptr};
    static std::mutex mu;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    int *&p = ptrs[dev & 63];
    if (!p){
        check_cuda(cudaMalloc(&p, sizeof(int)), "cudaMalloc(status word)");
        check_cuda(cudaMemset(p, 0, sizeof(int)), "cudaMemset(status word)");
    }
    return p;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, cuuint64_t const *,
                                  cuuint64_t const *, cuuint32_t const *, cuuint32_t const *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn(){
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!tried){
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

bool encode_column_tmap(void *tmap, void const *base, int esize, long long count, long long N, long long blocks,
                        long long estride, long long bstride, int width, int boxr, int *swap){
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    // 4-byte elements map to FLOAT32 words, 8- and 16-byte elements to FLOAT64 words
    long long wpc = (esize >= 8) ? esize / 8 : 1;
    int csize = esize;
    int tpb = width;
    bool sw = estride > bstride && blocks > 1;
    cuuint64_t dims[3], strides[2];
    cuuint32_t box[3], estr[3] = {1, 1, 1};
    dims[0] = (cuuint64_t)(count * wpc);
    box[0] = (cuuint32_t)(tpb * wpc);
    if (!sw){
        dims[1] = (cuuint64_t)N; dims[2] = (cuuint64_t)blocks;
        strides[0] = (cuuint64_t)(estride * csize); strides[1] = (cuuint64_t)(bstride * csize);
        box[1] = (cuuint32_t)boxr; box[2] = 1;
    } else {
        dims[1] = (cuuint64_t)blocks; dims[2] = (cuuint64_t)N;
        strides[0] = (cuuint64_t)(bstride * csize); strides[1] = (cuuint64_t)(estride * csize);
        box[1] = 1; box[2] = (cuuint32_t)boxr;
    }
    if (blocks == 1) strides[sw ? 0 : 1] = strides[sw ? 1 : 0] * (cuuint64_t)(sw ? N : 1) + 16;
    CUtensorMapDataType dt = (esize == 4) ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    CUresult r = fn(reinterpret_cast<CUtensorMap *>(tmap), dt, 3, const_cast<void *>(base),
                    dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *swap = sw ? 1 : 0;
    return true;
}

std::vector<int> pipe_radices(int N, bool df){
    if (N < 2 || N > 4096 || (N & (N - 1))) return {};
    std::vector<int> r;
    for (int s = 0; s < pipe_nstages(N, df); s++) r.push_back(pipe_radix(N, s, df));
    return r;
}

// Pipelined path: power-of-two length, not in place across different layouts.
// Merges the two batch levels of a layout when its blocks are contiguous
// (bstride = count * dist), so that column tiles can span whole planes.
static void merge_blocks(Layout &Li, Layout &Lo, long long G){
    if (Li.bstride == Li.count * Li.dist && Lo.bstride == Lo.count * Lo.dist && Li.count == Lo.count){
        Li.count = G; Li.bstride = G * Li.dist;
        Lo.count = G; Lo.bstride = G * Lo.dist;
    }
}

// Pipelined path: power-of-two length, not in place across different layouts
// (the element type changes for r2c/c2r: never in place).
static bool try_pipe(cudaStream_t s, int kind, Fft1D &f, int prec, Layout Li, Layout Lo, void const *in, void *out,
                     long long G, double scale, int sine, LaunchCfg const &cfg){
    int v = (cfg.variant != 0) ? cfg.variant : kernel_variant();
    if (v == 1) return false;
    std::vector<int> pr = pipe_radices(f.N);
    if (pr.empty() || pr != f.radices || f.N < 16) return false;
    bool same = Li.count == Lo.count && Li.dist == Lo.dist && Li.bstride == Lo.bstride && Li.estride == Lo.estride;
    if (in == out && (!same || kind == K_R2C || kind == K_C2R)) return false;
    bool cols = !(Li.estride == 1 && Lo.estride == 1);
    if (!cols && (Li.estride != 1)) return false;
    merge_blocks(Li, Lo, G);
    // column tiles whose input blocks are contiguous but whose output blocks
    // are not (a padded pitch on one side): merge the input's alone, so that
    // tiles span whole planes and a plane stride that is no multiple of 16
    // bytes does not keep the tensor-map loader out
    int out_split = 0;
    if (cols && Li.count != G && Li.bstride == Li.count * Li.dist && in != out){
        Li.count = G;
        Li.bstride = G * Li.dist;
        out_split = 1;
    }
    PipeLaunch a{};
    a.out_split = out_split;
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    a.rtw = (kind == K_R2R_F || kind == K_R2R_B) ? f.r2r_twiddles(prec, s) : nullptr;
    a.G = G; a.scale = scale; a.sine = sine;
    a.status = device_status();
    bool c2c = (kind == K_C2C_F || kind == K_C2C_B), r2c = (kind == K_R2C || kind == K_C2R);
    if (prec == 0){
        if (c2c) return launch_pipe_f32_c2c(s, kind, f.N, cols, a);
        if (r2c) return launch_pipe_f32_r2c(s, kind, f.N, cols, a);
        return launch_pipe_f32_r2r(s, kind, f.N, cols, a);
    }
    if (c2c && double_arithmetic() == DA_DOUBLE_FLOAT){
        // the double-float kernels run their own plan (radices up to 8)
        a.tw = get_fft1d(f.N, pipe_radices(f.N, true))->twiddles_df(s);
        return launch_pipe_df64_c2c(s, kind, f.N, cols, a);
    }
    if (c2c) return launch_pipe_f64_c2c(s, kind, f.N, cols, a);
    if (r2c) return launch_pipe_f64_r2c(s, kind, f.N, cols, a);
    return launch_pipe_f64_r2r(s, kind, f.N, cols, a);
}

// Whether two CTAs of `smem` dynamic shared-memory bytes are resident on
// one SM of the current device (with the per-block reservation).
static bool two_ctas_fit(size_t smem){
    int dev = 0, smem_sm = 0, smem_rsv = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev), "device attribute");
    check_cuda(cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev), "device attribute");
    return 2 * (smem + (size_t)smem_rsv) <= (size_t)smem_sm;
}

// Pipelined runtime-radix path (c2c of any supported length): line tiles need
// back-to-back lines whose tile bytes are multiples of 16, column tiles a
// tensor map over adjacent columns.  Returns false when the batch does not
// fit either form (the generic kernels run it then).
static bool try_pipe_rt(cudaStream_t s, Fft1D &f, int prec, bool fwd, Layout Li, Layout Lo, void const *in, void *out,
                        long long G, double scale, LaunchCfg const &cfg){
    int v = (cfg.variant != 0) ? cfg.variant : kernel_variant();
    if (v == 1 || f.N < 8 || f.plan.nstages < 1) return false;
    bool same = Li.count == Lo.count && Li.dist == Lo.dist && Li.bstride == Lo.bstride && Li.estride == Lo.estride;
    if (in == out && !same) return false;
    bool cols = !(Li.estride == 1 && Lo.estride == 1);
    if (!cols && Li.estride != 1) return false;
    merge_blocks(Li, Lo, G);
    int N = f.N, T = f.plan.T;
    size_t es = (prec == 0) ? sizeof(float2) : sizeof(double2);
    size_t padn = (size_t)(N + N / 16 + 1);
    uintptr_t base = reinterpret_cast<uintptr_t>(in);
    if (base & 15) return false;
    PipeRtParams P{};
    CUtensorMap tmap;
    std::memset(&tmap, 0, sizeof(tmap));
    int tpb = 1;
    size_t smem = 0;
    // tile slots: two (the copy of the next tile overlaps the transform of
    // this one), or one for float line tiles (the float kernel is compiled
    // for two CTAs per SM, which then overlap each other's copies; measured
    // faster for line tiles at 384-640 points).  Float column tiles keep two
    // slots where two CTAs of them fit in an SM's shared memory: 16 columns;
    // else 16 columns with a compiled kernel's twiddles left in global
    // memory; else 8 columns (even N); else one slot of 16 columns.  `extra`:
    // the twiddle table of a kernel compiled for this plan (float), in shared
    // memory after the tiles (ct 1), or 0 (ct 2: in global memory).
    size_t const ctb = (prec == 0) ? rt_ct_smem(f.plan) : 0;
    size_t extra = ctb;
    int ct = (ctb > 0) ? 1 : 0;
    int nbuf = 2, cap = 16;
    auto shape = [&](int nb){
        if (!cols){
            tpb = std::max(1, 256 / T);
            while (tpb > 1 && tpb * T > 512) tpb /= 2;
            while (tpb > 1 && (nb * (size_t)tpb * N + (size_t)tpb * padn) * es + extra > 200 * 1024) tpb /= 2;
            smem = (nb * (size_t)tpb * N + (size_t)tpb * padn) * es + extra;
        } else {
            tpb = (prec == 0) ? cap : 8;
            while (tpb > 2 && tpb * T > 512) tpb /= 2;
            while (tpb > 2 && nb * (size_t)tpb * N * es + extra > 200 * 1024) tpb /= 2;
            smem = nb * (size_t)tpb * N * es + extra;
        }
    };
    shape(nbuf);
    if (prec == 0 && !cols){
        nbuf = 1;
        shape(nbuf);
    } else if (prec == 0 && !two_ctas_fit(smem)){
        bool fit = false;
        if (ctb > 0){
            extra = 0;
            shape(nbuf);
            fit = two_ctas_fit(smem);
            if (fit) ct = 2; else extra = ctb;
        }
        // 8 columns are 64 bytes per row, so a copy's rows (a divisor of N)
        // must be even for its 128-byte aligned destination: even N only
        if (!fit && N % 2 == 0){
            cap = 8;
            shape(nbuf);
            fit = two_ctas_fit(smem);
        }
        if (!fit){
            nbuf = 1; cap = 16;
            shape(nbuf);
        }
    }
    if (!cols){
        if (Li.dist != N || (G > Li.count && Li.bstride != Li.count * N)) return false;
        long long last = G % tpb;
        if (((size_t)tpb * N * es) % 16 != 0 || ((size_t)last * N * es) % 16 != 0) return false;
        P.ntiles = (G + tpb - 1) / tpb;
        P.tiles_per_block = 0;
    } else {
        if (Li.dist != 1 || G % Li.count != 0) return false;
        if (((size_t)tpb * es) % 16 != 0 || tpb * T > 512) return false;
        // the rows of each tensor copy: a divisor of N up to 256 whose box
        // (and so every box destination) is a multiple of 128 bytes, as is
        // the tile buffer, since a tensor copy's shared-memory destination
        // must be 128-byte aligned
        int boxr = 0;
        for (int d = std::min(N, 256); d >= 1; d--)
            if (N % d == 0 && ((size_t)d * tpb * es) % 128 == 0){ boxr = d; break; }
        if (boxr == 0 || ((size_t)tpb * N * es) % 128 != 0) return false;
        long long blocks = G / Li.count;
        int swap = 0;
        if (!encode_column_tmap(&tmap, in, (int)es, Li.count, N, blocks, Li.estride, Li.bstride, tpb, boxr, &swap))
            return false;
        P.boxr = boxr;
        P.tswap = swap;
        P.tiles_per_block = (Li.count + tpb - 1) / tpb;
        P.ntiles = blocks * P.tiles_per_block;
    }
    if (smem > 226 * 1024) return false;
    P.plan = f.plan;
    P.Li = Li; P.Lo = Lo; P.in = in; P.out = out;
    P.tw = f.twiddles(prec, s);
    P.G = G;
    P.tpb = tpb;
    P.nbuf = nbuf;
    P.ct = ct;
    P.scale = scale;
    P.do_scale = (scale != 1.0);
    P.status = device_status();
    launch_pipe_rt(s, prec, fwd, cols, P, &tmap, smem, tpb * T);
    return true;
}

void launch_c2c(cudaStream_t s, Fft1D &f, int prec, bool fwd, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg){
    if (G <= 0) return;
    if (f.algo != ALGO_DIRECT){
        launch_composite(s, LM_C2C, f, prec, fwd, 0, f.N, Li, Lo, in, out, G, scale, cfg);
        return;
    }
    if (cfg.tc && prec == 0 && tc_supported(f.N)){
        launch_tc_c2c(s, f.N, fwd, Li, Lo, in, out, G, scale);
        return;
    }
    if (try_pipe(s, fwd ? K_C2C_F : K_C2C_B, f, prec, Li, Lo, in, out, G, scale, 0, cfg)) return;
    if (try_pipe_rt(s, f, prec, fwd, Li, Lo, in, out, G, scale, cfg)) return;
    KernelArgs a{};
    bool cols = is_cols(Li, Lo);
    geometry(f, prec, cols, false, G, cfg, a);
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    a.scale = scale; a.do_scale = (scale != 1.0);
    run(s, fwd ? K_C2C_F : K_C2C_B, prec, cols, a);
}

// Fused convolution pass over the columns of x (in place): power-of-two
// lengths of the pipelined radix plan, column layouts (estride != 1) whose
// tiles a tensor map can copy.  Returns false when the pass cannot run.
bool launch_conv_pass(cudaStream_t s, Fft1D &f, int prec, Layout L, void *x, void const *y, long long G,
                      double scale, bool dry_run){
    if (kernel_variant() == 1) return false;
    std::vector<int> pr = pipe_radices(f.N);
    if (pr.empty() || pr != f.radices || f.N < 16 || L.estride == 1) return false;
    Layout Lo = L;
    merge_blocks(L, Lo, G);
    ConvLaunch a{};
    a.L = L; a.x = x; a.y = y; a.G = G; a.scale = scale;
    a.status = device_status();
    a.tw = dry_run ? nullptr : f.twiddles(prec, s);
    return (prec == 0) ? launch_conv_f32(s, f.N, a, dry_run) : launch_conv_f64(s, f.N, a, dry_run);
}

void launch_r2c(cudaStream_t s, Fft1D &f, int prec, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg){
    if (G <= 0) return;
    if (f.algo != ALGO_DIRECT){
        launch_composite(s, LM_R2C, f, prec, true, 0, f.N, Li, Lo, in, out, G, scale, cfg);
        return;
    }
    if (try_pipe(s, K_R2C, f, prec, Li, Lo, in, out, G, scale, 0, cfg)) return;
    KernelArgs a{};
    bool cols = is_cols(Li, Lo);
    geometry(f, prec, cols, true, G, cfg, a);
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    a.scale = scale; a.do_scale = (scale != 1.0);
    run(s, K_R2C, prec, cols, a);
}

void launch_c2r(cudaStream_t s, Fft1D &f, int prec, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg){
    if (G <= 0) return;
    if (f.algo != ALGO_DIRECT){
        launch_composite(s, LM_C2R, f, prec, false, 0, f.N, Li, Lo, in, out, G, scale, cfg);
        return;
    }
    if (try_pipe(s, K_C2R, f, prec, Li, Lo, in, out, G, scale, 0, cfg)) return;
    KernelArgs a{};
    bool cols = is_cols(Li, Lo);
    geometry(f, prec, cols, true, G, cfg, a);
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    a.scale = scale; a.do_scale = (scale != 1.0);
    run(s, K_C2R, prec, cols, a);
}

void launch_dct1(cudaStream_t s, Fft1D &f, int prec, bool fwd, int N, Layout Li, Layout Lo, void const *in, void *out,
                 long long G, double scale, LaunchCfg cfg){
    if (G <= 0) return;
    if (N < 2 || f.N != 2 * (N - 1)) throw Error(ST_INVALID, "DCT-I of N values runs on an FFT of length 2(N-1)");
    if (f.algo != ALGO_DIRECT){
        launch_composite(s, LM_DCT1, f, prec, true, 0, N, Li, Lo, in, out, G, fwd ? scale : 2.0 * scale, cfg);
        return;
    }
    KernelArgs a{};
    bool cols = is_cols(Li, Lo);
    geometry(f, prec, cols, true, G, cfg, a);
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    double sc = fwd ? scale : 2.0 * scale;
    a.scale = sc; a.do_scale = (sc != 1.0);
    a.ndata = N;
    run(s, K_DCT1, prec, cols, a);
}

void launch_r2r(cudaStream_t s, Fft1D &f, int prec, bool fwd, bool sine, Layout Li, Layout Lo, void const *in,
                void *out, long long G, double scale, LaunchCfg cfg){
    if (G <= 0) return;
    if (f.algo != ALGO_DIRECT){
        launch_composite(s, fwd ? LM_R2R_F : LM_R2R_B, f, prec, fwd, sine ? 1 : 0, f.N, Li, Lo, in, out, G, scale, cfg);
        return;
    }
    if (try_pipe(s, fwd ? K_R2R_F : K_R2R_B, f, prec, Li, Lo, in, out, G, scale, sine ? 1 : 0, cfg)) return;
    KernelArgs a{};
    bool cols = is_cols(Li, Lo);
    geometry(f, prec, cols, true, G, cfg, a);
    a.Li = Li; a.Lo = Lo; a.in = in; a.out = out;
    a.tw = f.twiddles(prec, s);
    a.rtw = f.r2r_twiddles(prec, s);
    a.scale = scale; a.do_scale = (scale != 1.0);
    a.sine = sine ? 1 : 0;
    run(s, fwd ? K_R2R_F : K_R2R_B, prec, cols, a);
}

} // namespace gbfft
