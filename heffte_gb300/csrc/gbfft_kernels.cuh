// Batched 1-D transform kernels for sm_103a (GB300).
//
// One CTA owns TPB transforms (TPB "lines" when the transform runs along the
// fastest dimension, TPB adjacent "columns" when it runs along a strided
// dimension) and T threads per transform.  The transform is a Stockham
// autosort FFT whose radix sequence is a runtime list (radices 2, 3, 4, 5, 7,
// 8, 11, 13, 16); each thread keeps up to EMAX complex values in registers:
//   * stage 0 loads its butterfly inputs straight from HBM (coalesced: the
//     Stockham input positions j + q*N/R are consecutive across threads, and
//     in the column layout adjacent threads own adjacent columns);
//   * middle stages exchange through shared memory (one read, one write);
//   * the last stage stores straight to HBM (again positions j + q*N/R),
//     or to shared memory when a fused post-processing step follows
//     (r2c split, DCT/DST post-twiddle).
// Twiddles come from a per-length table generated in FP64 on the device.
#pragma once
#include <type_traits>
#include "gbfft_common.cuh"

namespace gbfft {

// Register file of one thread: EMAX complex values.
template<typename T, int EMAX> struct Regs { c_t<T> v[EMAX]; };

// Shared-memory index of element p of the local transform `loc`.
template<bool COLS>
__device__ __forceinline__ int sm_index(int p, int loc, int TPB, int padn){
    return COLS ? (p * TPB + loc) : (loc * padn + p + (p >> 4));
}

// Options of fft_run beyond the radix set: S5 (the radices of 5-smooth
// lengths alone, as std::integral_constant<bool, S5>) and TWT (tw is the
// twiddle table in shared memory with each stage's block transposed to
// [q - 1][k]: a warp's threads, which hold consecutive k, read consecutive
// entries).
template<bool S5, bool TWT> struct StageOpts {
    static constexpr bool value = S5;
    static constexpr bool twt = TWT;
};
template<class X, class = void> struct opts_twt : std::false_type {};
template<class X> struct opts_twt<X, std::void_t<decltype(X::twt)>> : std::integral_constant<bool, X::twt> {};

template<int R, int EMAX, bool FWD, bool COLS, typename T, bool TWT = false, class LD, class ST>
__device__ __forceinline__ void fft_stage(Stage const &S, int t, int Tt, bool active, bool first, bool to_global,
                                          c_t<T> *sm, int loc, int TPB, int padn,
                                          c_t<T> const *__restrict__ tw, Regs<T, EMAX> &r, LD &ld, ST &st){
    using C = c_t<T>;
    constexpr int M = EMAX / R;
    if (first){
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * Tt;
            if (active && j < S.NR){
                #pragma unroll
                for (int q = 0; q < R; q++) r.v[m * R + q] = ld(j + q * S.NR);
            }
        }
    } else {
        #pragma unroll
        for (int m = 0; m < M; m++){
            int j = t + m * Tt;
            if (active && j < S.NR){
                #pragma unroll
                for (int q = 0; q < R; q++) r.v[m * R + q] = sm[sm_index<COLS>(j + q * S.NR, loc, TPB, padn)];
            }
        }
        __syncthreads();
    }
    #pragma unroll
    for (int m = 0; m < M; m++){
        int j = t + m * Tt;
        if (active && j < S.NR){
            int hi = fdiv(j, S);
            int k = j - hi * S.Ns;
            if (!first && k != 0){
                #pragma unroll
                for (int q = 1; q < R; q++){
                    C wq = TWT ? tw[S.tw + (q - 1) * S.Ns + k] : __ldg(tw + S.tw + k * (R - 1) + q - 1);
                    r.v[m * R + q] = FWD ? cmul(r.v[m * R + q], wq) : cmulc(r.v[m * R + q], wq);
                }
            }
            bfly<R, FWD, C, T>(&r.v[m * R]);
            int ob = hi * S.Ns * R + k;
            #pragma unroll
            for (int q = 0; q < R; q++){
                if (to_global) st(ob + q * S.Ns, r.v[m * R + q]);
                else sm[sm_index<COLS>(ob + q * S.Ns, loc, TPB, padn)] = r.v[m * R + q];
            }
        }
    }
    if (!to_global) __syncthreads();
}

// Called by every thread once the first stage has read all its inputs, when
// enabled() (uniform over the CTA); the batch kernel starts the copy of its
// next tile into the buffer the first stage read from.
struct NoHook {
    __device__ __forceinline__ bool enabled() const { return false; }
    __device__ __forceinline__ void operator()() const {}
};

// Runs the whole transform. If last_to_global is false the result is left in
// shared memory (natural order) and the CTA is synchronised on return.
// S5T: std::true_type compiles the radices of 5-smooth lengths alone (2, 3,
// 4, 5, 8, 16; the caller guarantees the plan has no other): fewer registers;
// or StageOpts<S5, TWT> (TWT: tw in shared memory, transposed per stage)
template<int EMAX, bool FWD, bool COLS, typename T, class LD, class ST, class AF = NoHook, class S5T = std::false_type>
__device__ __forceinline__ void fft_run(Plan1D const &P, int t, bool active, c_t<T> *sm, int loc, int TPB, int padn,
                                        c_t<T> const *__restrict__ tw, bool last_to_global, LD &ld, ST &st,
                                        AF const &after_first = AF{}, S5T = S5T{}){
    constexpr bool S5 = S5T::value;
    constexpr bool TWT = opts_twt<S5T>::value;
    constexpr bool HOOK = !std::is_same<AF, NoHook>::value;
    Regs<T, EMAX> r;
    if (P.nstages == 0){
        // length-1 transform: identity
        if (active && t == 0){
            c_t<T> x = ld(0);
            if (last_to_global) st(0, x); else sm[sm_index<COLS>(0, loc, TPB, padn)] = x;
        }
        if (!last_to_global) __syncthreads();
        if constexpr (HOOK){
            if (after_first.enabled()){ __syncthreads(); after_first(); }
        }
        return;
    }
    for (int s = 0; s < P.nstages; s++){
        Stage const S = P.st[s];
        bool first = (s == 0);
        bool tg = (s == P.nstages - 1) && last_to_global;
        switch (S.R){
            case 16: if constexpr (EMAX >= 16) fft_stage<16, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 13: if constexpr (EMAX >= 13 && !S5) fft_stage<13, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 11: if constexpr (EMAX >= 11 && !S5) fft_stage<11, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 8: fft_stage<8, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 7: if constexpr (!S5) fft_stage<7, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 5: fft_stage<5, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 4: fft_stage<4, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            case 3: fft_stage<3, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
            default: fft_stage<2, EMAX, FWD, COLS, T, TWT>(S, t, P.T, active, first, tg, sm, loc, TPB, padn, tw, r, ld, st); break;
        }
        if constexpr (HOOK){
            // a stage that ends in shared memory ends with a barrier; one that
            // stores to global memory needs one before the inputs are free
            if (first && after_first.enabled()){
                if (tg) __syncthreads();
                after_first();
            }
        }
    }
}

// Thread -> (local transform, thread-in-transform) mapping.
template<bool COLS>
__device__ __forceinline__ void thread_map(int TPB, int Tt, int &loc, int &t){
    int tid = threadIdx.x;
    if (COLS){ loc = tid % TPB; t = tid / TPB; } else { loc = tid / Tt; t = tid % Tt; }
}

__device__ __forceinline__ int padded_len(int N){ return N + (N >> 4) + 1; }

// ---------------------------------------------------------------------------
// complex-to-complex
// ---------------------------------------------------------------------------
// Each kernel body is a per-tile device function (tile = block of TPB
// transforms) so that the batched multi-box kernel can reuse it; threads
// beyond TPB * T of a larger CTA stay inactive but join every barrier.
// pf (optional): the tile's input already copied into shared memory, lines
// back to back (pf[loc * N + p]) or rows of TPB columns (pf[p * TPB + loc]);
// after_first: see fft_run.
template<typename T, int EMAX, bool FWD, bool COLS, class AF = NoHook, class S5T = std::false_type>
__device__ __forceinline__ void tile_c2c(Plan1D const &P, Layout Li, Layout Lo, c_t<T> const *in, c_t<T> *out,
                                         c_t<T> const *__restrict__ tw, long long G, int TPB, T scale, int do_scale,
                                         long long tile, c_t<T> *sm, c_t<T> const *pf = nullptr,
                                         AF const &after_first = AF{}, S5T s5 = S5T{}){
    using C = c_t<T>;
    int loc, t;
    thread_map<COLS>(TPB, P.T, loc, t);
    long long g = tile * TPB + loc;
    bool active = (g < G) && (t < P.T) && (loc < TPB);
    long long ib = active ? base_of(Li, g) : 0, ob = active ? base_of(Lo, g) : 0;
    long long ies = Li.estride, oes = Lo.estride;
    int const N = P.N;
    // L2-only loads: in the batched kernel the data was written by other CTAs
    // of the same launch, so this SM's L1 may hold stale lines
    auto ld = [&](int p) -> C {
        if (pf) return COLS ? pf[p * TPB + loc] : pf[loc * N + p];
        return __ldcg(in + ib + p * ies);
    };
    auto st = [&](int p, C v){ out[ob + p * oes] = do_scale ? cscale(v, scale) : v; };
    fft_run<EMAX, FWD, COLS, T>(P, t, active, sm, loc, TPB, padded_len(P.N), tw, true, ld, st, after_first, s5);
}

template<typename T, int EMAX, bool FWD, bool COLS>
__global__ void __launch_bounds__(512)
k_c2c(Plan1D P, Layout Li, Layout Lo, c_t<T> const *in, c_t<T> *out, c_t<T> const *__restrict__ tw,
      long long G, int TPB, T scale, int do_scale){
    extern __shared__ __align__(16) unsigned char smraw[];
    tile_c2c<T, EMAX, FWD, COLS>(P, Li, Lo, in, out, tw, G, TPB, scale, do_scale, blockIdx.x,
                                 reinterpret_cast<c_t<T>*>(smraw));
}

// ---------------------------------------------------------------------------
// real-to-complex: two real transforms (a = 2g, b = 2g+1) in one complex FFT,
// z = x_a + i x_b; X_a[k] = (Z_k + conj Z_{N-k})/2, X_b[k] = -i (Z_k - conj Z_{N-k})/2.
// Li is in real elements, Lo in complex elements; outputs k = 0..N/2.
// ---------------------------------------------------------------------------
// pf (optional, line tiles): the tile's real input lines back to back in
// shared memory (line 2 loc + b at pf[(2 loc + b) N + p])
template<typename T, int EMAX, bool COLS, class AF = NoHook, class S5T = std::false_type>
__device__ __forceinline__ void tile_r2c(Plan1D const &P, Layout Li, Layout Lo, T const *in, c_t<T> *out,
                                         c_t<T> const *__restrict__ tw, long long G, int TPB, T scale, int do_scale,
                                         long long tile, c_t<T> *sm, T const *pf = nullptr,
                                         AF const &after_first = AF{}, S5T s5 = S5T{}){
    using C = c_t<T>;
    int loc, t;
    thread_map<COLS>(TPB, P.T, loc, t);
    long long gp = tile * TPB + loc;
    long long ga = 2 * gp, gb = 2 * gp + 1;
    bool active = (ga < G) && (t < P.T) && (loc < TPB);
    bool hasb = gb < G;
    long long ia = active ? base_of(Li, ga) : 0, ibb = (active && hasb) ? base_of(Li, gb) : 0;
    long long ies = Li.estride;
    int const NL = P.N;
    auto ld = [&](int p) -> C {
        C z;
        if (!COLS && pf){
            z.x = pf[(2 * loc) * NL + p]; z.y = hasb ? pf[(2 * loc + 1) * NL + p] : (T)0;
            return z;
        }
        z.x = __ldcg(in + ia + p * ies); z.y = hasb ? __ldcg(in + ibb + p * ies) : (T)0; return z;
    };
    auto st = [&](int, C){};
    int padn = padded_len(P.N);
    fft_run<EMAX, true, COLS, T>(P, t, active, sm, loc, TPB, padn, tw, false, ld, st, after_first, s5);
    if (!active) return;
    int N = P.N;
    long long oa = base_of(Lo, ga), obb = hasb ? base_of(Lo, gb) : 0;
    long long oes = Lo.estride;
    T h = (T)0.5 * (do_scale ? scale : (T)1);
    for (int k = t; k <= N / 2; k += P.T){
        C zk = sm[sm_index<COLS>(k, loc, TPB, padn)];
        int nk = (k == 0) ? 0 : N - k;
        C zn = sm[sm_index<COLS>(nk, loc, TPB, padn)];
        C xa; xa.x = h * (zk.x + zn.x); xa.y = h * (zk.y - zn.y);
        out[oa + k * oes] = xa;
        if (hasb){
            // -i * (zk - conj zn) / 2
            C xb; xb.x = h * (zk.y + zn.y); xb.y = -h * (zk.x - zn.x);
            out[obb + k * oes] = xb;
        }
    }
}

template<typename T, int EMAX, bool COLS>
__global__ void __launch_bounds__(512)
k_r2c(Plan1D P, Layout Li, Layout Lo, T const *in, c_t<T> *out, c_t<T> const *__restrict__ tw,
      long long G, int TPB, T scale, int do_scale){
    extern __shared__ __align__(16) unsigned char smraw[];
    tile_r2c<T, EMAX, COLS>(P, Li, Lo, in, out, tw, G, TPB, scale, do_scale, blockIdx.x,
                            reinterpret_cast<c_t<T>*>(smraw));
}

// ---------------------------------------------------------------------------
// complex-to-real (unnormalised inverse): two half spectra in one complex FFT.
// Z_p = X'_a[p] + i X'_b[p] with X'[p] = X[p] (p <= N/2, imaginary part of
// the DC and Nyquist terms dropped) and conj X[N-p] above N/2.
// ---------------------------------------------------------------------------
// pf (optional, line tiles): the tile's half-spectrum lines back to back in
// shared memory (line 2 loc + b at pf[(2 loc + b) (N/2 + 1) + p])
template<typename T, int EMAX, bool COLS, class AF = NoHook, class S5T = std::false_type>
__device__ __forceinline__ void tile_c2r(Plan1D const &P, Layout Li, Layout Lo, c_t<T> const *in, T *out,
                                         c_t<T> const *__restrict__ tw, long long G, int TPB, T scale, int do_scale,
                                         long long tile, c_t<T> *sm, c_t<T> const *pf = nullptr,
                                         AF const &after_first = AF{}, S5T s5 = S5T{}){
    using C = c_t<T>;
    int loc, t;
    thread_map<COLS>(TPB, P.T, loc, t);
    long long gp = tile * TPB + loc;
    long long ga = 2 * gp, gb = 2 * gp + 1;
    bool active = (ga < G) && (t < P.T) && (loc < TPB);
    bool hasb = gb < G;
    long long ia = active ? base_of(Li, ga) : 0, ibb = (active && hasb) ? base_of(Li, gb) : 0;
    long long oa = active ? base_of(Lo, ga) : 0, obb = (active && hasb) ? base_of(Lo, gb) : 0;
    long long ies = Li.estride, oes = Lo.estride;
    int N = P.N;
    auto ld = [&](int p) -> C {
        int pp = (2 * p <= N) ? p : N - p;
        bool cj = (2 * p > N);
        bool real_only = (pp == 0) || (2 * pp == N);
        C xa, xb;
        if (!COLS && pf){
            int const H = N / 2 + 1;
            xa = pf[(2 * loc) * H + pp];
            xb = hasb ? pf[(2 * loc + 1) * H + pp] : mk<T>(0, 0);
        } else {
            xa = __ldcg(in + ia + pp * ies);
            xb = hasb ? __ldcg(in + ibb + pp * ies) : mk<T>(0, 0);
        }
        if (real_only){ xa.y = 0; xb.y = 0; }
        if (cj){ xa.y = -xa.y; xb.y = -xb.y; }
        C z; z.x = xa.x - xb.y; z.y = xa.y + xb.x; return z;
    };
    auto st = [&](int p, C v){
        T s = do_scale ? scale : (T)1;
        out[oa + p * oes] = v.x * s;
        if (hasb) out[obb + p * oes] = v.y * s;
    };
    fft_run<EMAX, false, COLS, T>(P, t, active, sm, loc, TPB, padded_len(P.N), tw, true, ld, st, after_first, s5);
}

template<typename T, int EMAX, bool COLS>
__global__ void __launch_bounds__(512)
k_c2r(Plan1D P, Layout Li, Layout Lo, c_t<T> const *in, T *out, c_t<T> const *__restrict__ tw,
      long long G, int TPB, T scale, int do_scale){
    extern __shared__ __align__(16) unsigned char smraw[];
    tile_c2r<T, EMAX, COLS>(P, Li, Lo, in, out, tw, G, TPB, scale, do_scale, blockIdx.x,
                            reinterpret_cast<c_t<T>*>(smraw));
}

// ---------------------------------------------------------------------------
// real-to-real: DCT-II (forward, REDFT10) / 2 x DCT-III (backward, 2 x REDFT01)
// by Makhoul's N-point reordering, two lines per complex FFT; the sine kinds
// (RODFT10 / 2 x RODFT01) by the identities
//   DST-II(x)[k]  = DCT-II((-1)^n x_n)[N-1-k]
//   DST-III(y)[n] = (-1)^n DCT-III(y_rev)[n].
// rtw holds exp(-i pi k / 2N), k = 0..N-1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int makhoul_src(int p, int N){ return (2 * p < N) ? 2 * p : 2 * (N - 1 - p) + 1; }

template<typename T, int EMAX, bool FWD, bool COLS>
__global__ void __launch_bounds__(512)
k_r2r(Plan1D P, Layout Li, Layout Lo, T const *in, T *out, c_t<T> const *__restrict__ tw,
      c_t<T> const *__restrict__ rtw, long long G, int TPB, int sine, T scale, int do_scale){
    using C = c_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C*>(smraw);
    int loc, t;
    thread_map<COLS>(TPB, P.T, loc, t);
    long long gp = (long long)blockIdx.x * TPB + loc;
    long long ga = 2 * gp, gb = 2 * gp + 1;
    bool active = (ga < G) && (t < P.T) && (loc < TPB);
    bool hasb = gb < G;
    long long ia = active ? base_of(Li, ga) : 0, ibb = (active && hasb) ? base_of(Li, gb) : 0;
    long long oa = active ? base_of(Lo, ga) : 0, obb = (active && hasb) ? base_of(Lo, gb) : 0;
    long long ies = Li.estride, oes = Lo.estride;
    int N = P.N;
    int padn = padded_len(N);
    T s = do_scale ? scale : (T)1;
    if (FWD){
        auto ld = [&](int p) -> C {
            int n = makhoul_src(p, N);
            T sg = (sine && (n & 1)) ? (T)-1 : (T)1;
            C z; z.x = sg * in[ia + n * ies]; z.y = hasb ? sg * in[ibb + n * ies] : (T)0; return z;
        };
        auto st = [&](int, C){};
        fft_run<EMAX, true, COLS, T>(P, t, active, sm, loc, TPB, padn, tw, false, ld, st);
        if (!active) return;
        for (int k = t; k < N; k += P.T){
            C zk = sm[sm_index<COLS>(k, loc, TPB, padn)];
            C zn = sm[sm_index<COLS>((k == 0) ? 0 : N - k, loc, TPB, padn)];
            C w = __ldg(rtw + k);                       // exp(-i pi k / 2N)
            // A = zk + conj zn, B = -i (zk - conj zn); Y = Re(w * A), Re(w * B)
            T ax = zk.x + zn.x, ay = zk.y - zn.y;
            T bx = zk.y + zn.y, by = -(zk.x - zn.x);
            T ya = (w.x * ax - w.y * ay) * s;
            T yb = (w.x * bx - w.y * by) * s;
            int ko = sine ? (N - 1 - k) : k;
            out[oa + ko * oes] = ya;
            if (hasb) out[obb + ko * oes] = yb;
        }
    } else {
        // V[k] = 2 exp(i pi k / 2N) (Y[k] - i Y[N-k]), Y[N] = 0; Z = V_a + i V_b.
        auto yval = [&](long long base, int k) -> T {
            if (k >= N) return (T)0;
            int kk = sine ? (N - 1 - k) : k;
            return in[base + kk * ies];
        };
        auto ld = [&](int p) -> C {
            C w = __ldg(rtw + p); w.y = -w.y;             // exp(+i pi p / 2N)
            T a0 = yval(ia, p), a1 = (p == 0) ? (T)0 : yval(ia, N - p);
            T b0 = hasb ? yval(ibb, p) : (T)0, b1 = (hasb && p != 0) ? yval(ibb, N - p) : (T)0;
            // V_a = 2 w (a0 - i a1), V_b = 2 w (b0 - i b1)
            C va; va.x = 2 * (w.x * a0 + w.y * a1); va.y = 2 * (w.y * a0 - w.x * a1);
            C vb; vb.x = 2 * (w.x * b0 + w.y * b1); vb.y = 2 * (w.y * b0 - w.x * b1);
            C z; z.x = va.x - vb.y; z.y = va.y + vb.x; return z;
        };
        auto st = [&](int n, C v){
            int m = makhoul_src(n, N);
            T sg = (sine && (m & 1)) ? -s : s;
            out[oa + m * oes] = v.x * sg;
            if (hasb) out[obb + m * oes] = v.y * sg;
        };
        fft_run<EMAX, false, COLS, T>(P, t, active, sm, loc, TPB, padn, tw, true, ld, st);
    }
}

// ---------------------------------------------------------------------------
// DCT-I (REDFT00) of lines of N >= 2 values, the reference's cos1 transform:
//   y_k = x_0 + (-1)^k x_{N-1} + 2 sum_{n=1}^{N-2} x_n cos(pi n k / (N-1)),
// forward = REDFT00, backward = 2 x REDFT00.  The DFT of the even extension
//   e = (x_0, x_1, ..., x_{N-1}, x_{N-2}, ..., x_1)   (length L = 2(N-1))
// is real and equals REDFT00 on k < N, so two lines share one complex FFT of
// length L: z = e_a + i e_b, y_a = Re Z, y_b = Im Z.  P is the plan of length L.
// ---------------------------------------------------------------------------
template<typename T, int EMAX, bool COLS>
__global__ void __launch_bounds__(512)
k_dct1(Plan1D P, int N, Layout Li, Layout Lo, T const *in, T *out, c_t<T> const *__restrict__ tw,
       long long G, int TPB, T scale, int do_scale){
    using C = c_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C*>(smraw);
    int loc, t;
    thread_map<COLS>(TPB, P.T, loc, t);
    long long gp = (long long)blockIdx.x * TPB + loc;
    long long ga = 2 * gp, gb = 2 * gp + 1;
    bool active = (ga < G) && (t < P.T) && (loc < TPB);
    bool hasb = gb < G;
    long long ia = active ? base_of(Li, ga) : 0, ibb = (active && hasb) ? base_of(Li, gb) : 0;
    long long oa = active ? base_of(Lo, ga) : 0, obb = (active && hasb) ? base_of(Lo, gb) : 0;
    long long ies = Li.estride, oes = Lo.estride;
    int const L = P.N;
    T s = do_scale ? scale : (T)1;
    auto ld = [&](int p) -> C {
        int n = (p < N) ? p : L - p;
        C z; z.x = in[ia + n * ies]; z.y = hasb ? in[ibb + n * ies] : (T)0; return z;
    };
    auto st = [&](int k, C v){
        if (k >= N) return;
        out[oa + k * oes] = v.x * s;
        if (hasb) out[obb + k * oes] = v.y * s;
    };
    fft_run<EMAX, true, COLS, T>(P, t, active, sm, loc, TPB, padded_len(L), tw, true, ld, st);
}

} // namespace gbfft
