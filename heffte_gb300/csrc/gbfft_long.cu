// Transform lengths the radix kernels do not take directly (the
// cufft_executor role takes any length, include/heffte_backend_cuda.h:346-422):
//
//  * four-step, for lengths above 8192 whose prime factors are all <= 13:
//    N = N1 N2 with both factors direct lengths, n = N2 n1 + n2,
//    k = k1 + N1 k2:  the N1-point transforms over n1 (one per n2), a twiddle
//    exp(-+2 pi i n2 k1 / N), then the N2-point transforms over n2 (one per
//    k1), which leave X[k1 + N1 k2] in natural order;
//  * Bluestein's chirp-z algorithm, for lengths with a prime factor above 13
//    (the reference's stock backend uses Rader's algorithm for large primes,
//    include/stock_fft/heffte_stock_algos.h:328-; cuFFT accepts any length):
//    with nk = (n^2 + k^2 - (k - n)^2) / 2 and c_n = exp(-i pi n^2 / N),
//    X_k = c_k sum_n (x_n c_n) conj(c_{k-n}), a circular convolution of length
//    M >= 2N - 1 (a power of two) computed with two length-M transforms and a
//    product with the precomputed spectrum of conj(c) (FP64-generated).
//
// Every transform kind reaches the composite transform the same way: a
// "pre" kernel gathers the batch from the caller's layout into contiguous
// complex lines in scratch (pairing two real lines for r2c / c2r / DCT / DST,
// the extensions of DCT-I, Makhoul's reordering of DCT-II, exactly the data
// the fused direct kernels put through their FFT), the composite transform
// runs line by line in scratch, and a "post" kernel writes the result into
// the caller's layout (r2c split, DCT post-twiddle ...), carrying the scale.
// Lines are processed in chunks so that the scratch stays bounded.
#include "gbfft_internal.h"
#include <cmath>

namespace gbfft {

namespace {

constexpr int kThreads = 256;

int grid_of(long long work){
    long long b = (work + kThreads - 1) / kThreads;
    return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 32));
}

__device__ __forceinline__ int makhoul_index(int p, int N){ return (2 * p < N) ? 2 * p : 2 * (N - 1 - p) + 1; }

// ---------------------------------------------------------------------------
// pre / post kernels between the caller's layout and contiguous lines
// ---------------------------------------------------------------------------
struct LineArgs {
    Layout L;          // the caller's layout (input for pre, output for post)
    long long G;       // lines of the caller's batch
    long long u0;      // first unit (a line, or a pair of lines for the paired modes) of this chunk
    long long units;   // units in this chunk
    int N;             // length of the data lines
    int Lc;            // length of the complex lines in scratch (N; 2(N - 1) for DCT-I)
    int sine;          // DST instead of DCT (r2r modes)
    double scale;
};

template<typename T>
__global__ void __launch_bounds__(kThreads)
k_lines_pre(LineArgs a, int mode, void const *__restrict__ in_, c_t<T> *__restrict__ X,
            c_t<T> const *__restrict__ rtw){
    using C = c_t<T>;
    long long total = a.units * a.Lc;
    int const N = a.N;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long u = idx / a.Lc;
        int p = (int)(idx - u * a.Lc);
        long long gu = a.u0 + u;
        long long es = a.L.estride;
        C z;
        if (mode == LM_C2C){
            C const *in = reinterpret_cast<C const*>(in_);
            z = in[base_of(a.L, gu) + p * es];
        } else {
            long long ga = 2 * gu, gb = 2 * gu + 1;
            bool hasb = gb < a.G;
            long long ia = base_of(a.L, ga), ib = hasb ? base_of(a.L, gb) : 0;
            if (mode == LM_C2R){
                // half spectra X_a, X_b (p <= N/2) extended by conjugate symmetry;
                // the imaginary parts of the DC and Nyquist terms are dropped
                C const *in = reinterpret_cast<C const*>(in_);
                int pp = (2 * p <= N) ? p : N - p;
                bool cj = 2 * p > N;
                bool real_only = (pp == 0) || (2 * pp == N);
                C xa = in[ia + pp * es];
                C xb = hasb ? in[ib + pp * es] : mk<T>(0, 0);
                if (real_only){ xa.y = 0; xb.y = 0; }
                if (cj){ xa.y = -xa.y; xb.y = -xb.y; }
                z.x = xa.x - xb.y; z.y = xa.y + xb.x;
            } else {
                T const *in = reinterpret_cast<T const*>(in_);
                if (mode == LM_R2C){
                    z.x = in[ia + p * es];
                    z.y = hasb ? in[ib + p * es] : (T)0;
                } else if (mode == LM_DCT1){
                    int n = (p < N) ? p : a.Lc - p;       // even extension of length 2(N - 1)
                    z.x = in[ia + n * es];
                    z.y = hasb ? in[ib + n * es] : (T)0;
                } else if (mode == LM_R2R_F){
                    int n = makhoul_index(p, N);
                    T sg = (a.sine && (n & 1)) ? (T)-1 : (T)1;
                    z.x = sg * in[ia + n * es];
                    z.y = hasb ? sg * in[ib + n * es] : (T)0;
                } else {   // LM_R2R_B: V[p] = 2 exp(i pi p / 2N) (Y[p] - i Y[N - p]), Y[N] = 0
                    auto yval = [&](long long base, int k) -> T {
                        if (k >= N) return (T)0;
                        return in[base + (a.sine ? (N - 1 - k) : k) * es];
                    };
                    C w = rtw[p]; w.y = -w.y;
                    T a0 = yval(ia, p), a1 = (p == 0) ? (T)0 : yval(ia, N - p);
                    T b0 = hasb ? yval(ib, p) : (T)0, b1 = (hasb && p != 0) ? yval(ib, N - p) : (T)0;
                    C va, vb;
                    va.x = 2 * (w.x * a0 + w.y * a1); va.y = 2 * (w.y * a0 - w.x * a1);
                    vb.x = 2 * (w.x * b0 + w.y * b1); vb.y = 2 * (w.y * b0 - w.x * b1);
                    z.x = va.x - vb.y; z.y = va.y + vb.x;
                }
            }
        }
        X[u * a.Lc + p] = z;
    }
}

// Number of outputs per unit of the post kernel.
__host__ __device__ __forceinline__ int post_count(int mode, int N){ return (mode == LM_R2C) ? N / 2 + 1 : N; }

template<typename T>
__global__ void __launch_bounds__(kThreads)
k_lines_post(LineArgs a, int mode, c_t<T> const *__restrict__ Y, void *__restrict__ out_,
             c_t<T> const *__restrict__ rtw){
    using C = c_t<T>;
    int const N = a.N;
    int const K = post_count(mode, N);
    long long total = a.units * K;
    T const s = (T)a.scale;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long u = idx / K;
        int k = (int)(idx - u * K);
        long long gu = a.u0 + u;
        long long es = a.L.estride;
        C const *z = Y + u * a.Lc;
        if (mode == LM_C2C){
            C *out = reinterpret_cast<C*>(out_);
            out[base_of(a.L, gu) + k * es] = cscale(z[k], s);
            continue;
        }
        long long ga = 2 * gu, gb = 2 * gu + 1;
        bool hasb = gb < a.G;
        long long oa = base_of(a.L, ga), ob = hasb ? base_of(a.L, gb) : 0;
        if (mode == LM_R2C){
            // X_a[k] = (Z_k + conj Z_{N-k}) / 2, X_b[k] = -i (Z_k - conj Z_{N-k}) / 2
            C *out = reinterpret_cast<C*>(out_);
            C zk = z[k], zn = z[(k == 0) ? 0 : N - k];
            T h = (T)0.5 * s;
            C xa; xa.x = h * (zk.x + zn.x); xa.y = h * (zk.y - zn.y);
            out[oa + k * es] = xa;
            if (hasb){
                C xb; xb.x = h * (zk.y + zn.y); xb.y = -h * (zk.x - zn.x);
                out[ob + k * es] = xb;
            }
            continue;
        }
        T *out = reinterpret_cast<T*>(out_);
        if (mode == LM_C2R || mode == LM_DCT1){
            out[oa + k * es] = z[k].x * s;
            if (hasb) out[ob + k * es] = z[k].y * s;
        } else if (mode == LM_R2R_F){
            // A = Z_k + conj Z_{N-k}, B = -i (Z_k - conj Z_{N-k}); y = Re(w A), Re(w B)
            C zk = z[k], zn = z[(k == 0) ? 0 : N - k];
            C w = rtw[k];
            T ax = zk.x + zn.x, ay = zk.y - zn.y;
            T bx = zk.y + zn.y, by = -(zk.x - zn.x);
            int ko = a.sine ? (N - 1 - k) : k;
            out[oa + ko * es] = (w.x * ax - w.y * ay) * s;
            if (hasb) out[ob + ko * es] = (w.x * bx - w.y * by) * s;
        } else {   // LM_R2R_B
            int m = makhoul_index(k, N);
            T sg = (a.sine && (m & 1)) ? -s : s;
            out[oa + m * es] = z[k].x * sg;
            if (hasb) out[ob + m * es] = z[k].y * sg;
        }
    }
}

// ---------------------------------------------------------------------------
// four-step twiddle and Bluestein chirp kernels on contiguous lines
// ---------------------------------------------------------------------------
// Y[g][n2][k1] *= exp(-+2 pi i n2 k1 / N) (table ftw[m] = exp(-2 pi i m / N))
template<typename T>
__global__ void __launch_bounds__(kThreads)
k_fourstep_twiddle(c_t<T> *Y, long long lines, int N1, int N, c_t<T> const *__restrict__ ftw, int fwd){
    long long total = lines * N;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long r = idx % N;
        long long n2 = r / N1, k1 = r - n2 * N1;
        c_t<T> w = ftw[(n2 * k1) % N];
        Y[idx] = fwd ? cmul(Y[idx], w) : cmulc(Y[idx], w);
    }
}

// P[g][m] = X[g][m] c_m (conj for the backward direction) for m < N, 0 up to M
template<typename T>
__global__ void __launch_bounds__(kThreads)
k_chirp_pre(c_t<T> const *__restrict__ X, c_t<T> *__restrict__ P, long long lines, int N, int M,
            c_t<T> const *__restrict__ ch, int fwd){
    long long total = lines * M;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long g = idx / M;
        int m = (int)(idx - g * M);
        c_t<T> v = mk<T>(0, 0);
        if (m < N){
            c_t<T> x = X[g * N + m];
            v = fwd ? cmul(x, ch[m]) : cmulc(x, ch[m]);
        }
        P[idx] = v;
    }
}

// Q[g][j] *= B[j] (conj B for the backward direction); B is symmetric, B[j] = B[M - j]
template<typename T>
__global__ void __launch_bounds__(kThreads)
k_chirp_mul(c_t<T> *Q, long long lines, int M, c_t<T> const *__restrict__ B, int fwd){
    long long total = lines * M;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        c_t<T> b = B[idx % M];
        Q[idx] = fwd ? cmul(Q[idx], b) : cmulc(Q[idx], b);
    }
}

// Y[g][k] = P[g][k] c_k (conj backward), k < N
template<typename T>
__global__ void __launch_bounds__(kThreads)
k_chirp_post(c_t<T> const *__restrict__ P, c_t<T> *__restrict__ Y, long long lines, int N, int M,
             c_t<T> const *__restrict__ ch, int fwd){
    long long total = lines * N;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long g = idx / N;
        int k = (int)(idx - g * N);
        c_t<T> v = P[g * M + k];
        Y[idx] = fwd ? cmul(v, ch[k]) : cmulc(v, ch[k]);
    }
}

// ---------------------------------------------------------------------------
// tables, generated in FP64
// ---------------------------------------------------------------------------
// c_n = exp(-i pi n^2 / N): the angle from n^2 mod 2N, exact in integers
__global__ void k_chirp_table(int N, double2 *ch){
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x){
        long long q = (n * n) % (2LL * N);
        double sn, cs;
        sincospi(-(double)q / (double)N, &sn, &cs);
        ch[n] = make_double2(cs, sn);
    }
}

// b_m = conj(c_|m|) placed circularly in a length-M line (b_m = b_{M-m}), zero between
__global__ void k_chirp_line(int N, int M, double2 const *ch, double2 *b){
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (long long)gridDim.x * blockDim.x){
        long long j = (m < N) ? m : ((m > M - N) ? M - m : -1);
        b[m] = (j >= 0) ? make_double2(ch[j].x, -ch[j].y) : make_double2(0.0, 0.0);
    }
}

// exp(-2 pi i m / N), m < N
__global__ void k_unit_roots(int N, double2 *t){
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < N; m += (long long)gridDim.x * blockDim.x){
        double sn, cs;
        sincospi(-2.0 * (double)m / (double)N, &sn, &cs);
        t[m] = make_double2(cs, sn);
    }
}

template<typename T>
__global__ void k_round_table(double2 const *src, c_t<T> *dst, long long n, double scale){
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = mk<T>((T)(src[i].x * scale), (T)(src[i].y * scale));
}

size_t csize_of(int prec){ return prec == 0 ? sizeof(float2) : sizeof(double2); }

// Rounds an FP64 table to the working precision (a device copy for double).
void *table_in(int prec, double2 const *d64, long long n, double scale, cudaStream_t s){
    void *t = nullptr;
    check_cuda(cudaMalloc(&t, (size_t)n * csize_of(prec)), "cudaMalloc(composite table)");
    if (prec == 0) k_round_table<float><<<grid_of(n), kThreads, 0, s>>>(d64, reinterpret_cast<float2*>(t), n, scale);
    else k_round_table<double><<<grid_of(n), kThreads, 0, s>>>(d64, reinterpret_cast<double2*>(t), n, scale);
    check_cuda(cudaPeekAtLastError(), "table kernel");
    return t;
}

} // namespace

// ---------------------------------------------------------------------------
// composite transform of contiguous lines: X (lines x N) -> Y (lines x N)
// ---------------------------------------------------------------------------
long long composite_extra_per_line(Fft1D const &f){
    if (f.algo == ALGO_BLUESTEIN) return 2LL * f.sub1->N + composite_extra_per_line(*f.sub1);
    return 0;
}

void const *Fft1D::composite_table(int which, int prec, cudaStream_t s){
    std::lock_guard<std::mutex> lk(mu);
    void *&slot = ctab[which][prec];
    if (slot) return slot;
    if (which == TAB_ROOTS){
        double2 *t64 = nullptr;
        check_cuda(cudaMalloc(&t64, (size_t)N * sizeof(double2)), "cudaMalloc(four-step twiddles)");
        k_unit_roots<<<grid_of(N), kThreads, 0, s>>>(N, t64);
        slot = table_in(prec, t64, N, 1.0, s);
        check_cuda(cudaStreamSynchronize(s), "four-step twiddle table");
        cudaFree(t64);
        return slot;
    }
    // Bluestein: the chirp c_n, and B = FFT_M(b) / M of the circular conj(c)
    double2 *c64 = nullptr;
    check_cuda(cudaMalloc(&c64, (size_t)N * sizeof(double2)), "cudaMalloc(chirp)");
    k_chirp_table<<<grid_of(N), kThreads, 0, s>>>(N, c64);
    check_cuda(cudaPeekAtLastError(), "chirp kernel");
    if (which == TAB_CHIRP){
        slot = table_in(prec, c64, N, 1.0, s);
        check_cuda(cudaStreamSynchronize(s), "chirp table");
        cudaFree(c64);
        return slot;
    }
    int M = sub1->N;
    double2 *b = nullptr, *B = nullptr, *extra = nullptr;
    long long ex = composite_extra_per_line(*sub1);
    check_cuda(cudaMalloc(&b, (size_t)M * sizeof(double2)), "cudaMalloc(chirp line)");
    check_cuda(cudaMalloc(&B, (size_t)M * sizeof(double2)), "cudaMalloc(chirp spectrum)");
    if (ex > 0) check_cuda(cudaMalloc(&extra, (size_t)ex * sizeof(double2)), "cudaMalloc(chirp scratch)");
    k_chirp_line<<<grid_of(M), kThreads, 0, s>>>(N, M, c64, b);
    check_cuda(cudaPeekAtLastError(), "chirp line kernel");
    // the spectrum in FP64 by this library's own double-precision transform
    composite_core(s, *sub1, 1, true, b, B, 1, extra);
    slot = table_in(prec, B, M, 1.0 / (double)M, s);
    check_cuda(cudaStreamSynchronize(s), "chirp spectrum");
    cudaFree(c64); cudaFree(b); cudaFree(B);
    if (extra) cudaFree(extra);
    return slot;
}

void composite_core(cudaStream_t s, Fft1D &f, int prec, bool fwd, void *X, void *Y, long long lines, void *extra){
    if (lines <= 0) return;
    int N = f.N;
    size_t cs = csize_of(prec);
    if (f.algo == ALGO_DIRECT){
        Layout L{lines, N, lines * (long long)N, 1};
        launch_c2c(s, f, prec, fwd, L, L, X, Y, lines, 1.0);
        return;
    }
    if (f.algo == ALGO_FOURSTEP){
        Fft1D &f1 = *f.sub1, &f2 = *f.sub2;
        int N1 = f1.N, N2 = f2.N;
        // N1-point transforms over n1 (stride N2), one per (line, n2), written as Y[g][n2][k1]
        Layout Li{N2, 1, N, N2}, Lo{N2, N1, N, 1};
        launch_c2c(s, f1, prec, fwd, Li, Lo, X, Y, lines * N2, 1.0);
        void const *tw = f.composite_table(TAB_ROOTS, prec, s);
        if (prec == 0)
            k_fourstep_twiddle<float><<<grid_of(lines * N), kThreads, 0, s>>>(reinterpret_cast<float2*>(Y), lines, N1, N,
                                                                             reinterpret_cast<float2 const*>(tw), fwd);
        else
            k_fourstep_twiddle<double><<<grid_of(lines * N), kThreads, 0, s>>>(reinterpret_cast<double2*>(Y), lines, N1, N,
                                                                               reinterpret_cast<double2 const*>(tw), fwd);
        check_cuda(cudaPeekAtLastError(), "four-step twiddle kernel");
        // N2-point transforms over n2 (stride N1), one per (line, k1), in place: X[k1 + N1 k2]
        Layout Lc{N1, 1, N, N1};
        launch_c2c(s, f2, prec, fwd, Lc, Lc, Y, Y, lines * N1, 1.0);
        return;
    }
    // Bluestein through length M: P, Q in the extra scratch
    Fft1D &fm = *f.sub1;
    int M = fm.N;
    char *P = static_cast<char*>(extra);
    char *Q = P + (size_t)lines * M * cs;
    void *inner = Q + (size_t)lines * M * cs;
    void const *ch = f.composite_table(TAB_CHIRP, prec, s);
    void const *B = f.composite_table(TAB_CHIRP_SPECTRUM, prec, s);
    int fw = fwd ? 1 : 0;
    if (prec == 0){
        k_chirp_pre<float><<<grid_of(lines * M), kThreads, 0, s>>>(reinterpret_cast<float2 const*>(X), reinterpret_cast<float2*>(P),
                                                                  lines, N, M, reinterpret_cast<float2 const*>(ch), fw);
    } else {
        k_chirp_pre<double><<<grid_of(lines * M), kThreads, 0, s>>>(reinterpret_cast<double2 const*>(X), reinterpret_cast<double2*>(P),
                                                                   lines, N, M, reinterpret_cast<double2 const*>(ch), fw);
    }
    check_cuda(cudaPeekAtLastError(), "chirp kernel");
    composite_core(s, fm, prec, true, P, Q, lines, inner);
    if (prec == 0)
        k_chirp_mul<float><<<grid_of(lines * M), kThreads, 0, s>>>(reinterpret_cast<float2*>(Q), lines, M,
                                                                  reinterpret_cast<float2 const*>(B), fw);
    else
        k_chirp_mul<double><<<grid_of(lines * M), kThreads, 0, s>>>(reinterpret_cast<double2*>(Q), lines, M,
                                                                   reinterpret_cast<double2 const*>(B), fw);
    check_cuda(cudaPeekAtLastError(), "chirp product kernel");
    composite_core(s, fm, prec, false, Q, P, lines, inner);
    if (prec == 0)
        k_chirp_post<float><<<grid_of(lines * N), kThreads, 0, s>>>(reinterpret_cast<float2 const*>(P), reinterpret_cast<float2*>(Y),
                                                                   lines, N, M, reinterpret_cast<float2 const*>(ch), fw);
    else
        k_chirp_post<double><<<grid_of(lines * N), kThreads, 0, s>>>(reinterpret_cast<double2 const*>(P), reinterpret_cast<double2*>(Y),
                                                                    lines, N, M, reinterpret_cast<double2 const*>(ch), fw);
    check_cuda(cudaPeekAtLastError(), "chirp kernel");
}

// ---------------------------------------------------------------------------
// the batched transform of a composite length in the caller's layouts
// ---------------------------------------------------------------------------
static bool paired_mode(int mode){ return mode != LM_C2C; }

static long long units_of(int mode, long long G){ return paired_mode(mode) ? (G + 1) / 2 : G; }

static long long per_unit_elems(Fft1D const &f){ return 2LL * f.N + composite_extra_per_line(f); }

static long long chunk_units(Fft1D const &f, long long units){
    long long per = per_unit_elems(f);
    long long c = std::max<long long>(1, kCompositeScratchElems / per);
    return std::min(units, c);
}

long long composite_scratch_elems(Fft1D const &f, int mode, long long G){
    if (f.algo == ALGO_DIRECT || G <= 0) return 0;
    return chunk_units(f, units_of(mode, G)) * per_unit_elems(f);
}

void launch_composite(cudaStream_t s, int mode, Fft1D &f, int prec, bool fwd, int sine, int N, Layout Li, Layout Lo,
                      void const *in, void *out, long long G, double scale, LaunchCfg const &cfg){
    long long units = units_of(mode, G);
    size_t cs = csize_of(prec);
    size_t need = (size_t)composite_scratch_elems(f, mode, G) * cs;
    if (!cfg.scratch || cfg.scratch_bytes < need)
        throw Error(ST_INVALID, "transform length " + std::to_string(f.N) + " needs a workspace of " +
                    std::to_string(need) + " bytes for its composite (" +
                    std::string(f.algo == ALGO_FOURSTEP ? "four-step" : "Bluestein") + ") algorithm");
    long long cu = chunk_units(f, units);
    int Lc = f.N;
    char *X = static_cast<char*>(cfg.scratch);
    char *Y = X + (size_t)cu * Lc * cs;
    void *extra = Y + (size_t)cu * Lc * cs;
    void const *rtw = (mode == LM_R2R_F || mode == LM_R2R_B) ? f.r2r_twiddles(prec, s) : nullptr;
    for (long long u0 = 0; u0 < units; u0 += cu){
        long long c = std::min(cu, units - u0);
        LineArgs a{};
        a.L = Li; a.G = G; a.u0 = u0; a.units = c; a.N = N; a.Lc = Lc; a.sine = sine; a.scale = 1.0;
        if (prec == 0)
            k_lines_pre<float><<<grid_of(c * Lc), kThreads, 0, s>>>(a, mode, in, reinterpret_cast<float2*>(X),
                                                                   reinterpret_cast<float2 const*>(rtw));
        else
            k_lines_pre<double><<<grid_of(c * Lc), kThreads, 0, s>>>(a, mode, in, reinterpret_cast<double2*>(X),
                                                                    reinterpret_cast<double2 const*>(rtw));
        check_cuda(cudaPeekAtLastError(), "composite gather kernel");
        composite_core(s, f, prec, fwd, X, Y, c, extra);
        a.L = Lo; a.scale = scale;
        long long nout = c * post_count(mode, N);
        if (prec == 0)
            k_lines_post<float><<<grid_of(nout), kThreads, 0, s>>>(a, mode, reinterpret_cast<float2 const*>(Y), out,
                                                                  reinterpret_cast<float2 const*>(rtw));
        else
            k_lines_post<double><<<grid_of(nout), kThreads, 0, s>>>(a, mode, reinterpret_cast<double2 const*>(Y), out,
                                                                   reinterpret_cast<double2 const*>(rtw));
        check_cuda(cudaPeekAtLastError(), "composite scatter kernel");
    }
}

} // namespace gbfft
