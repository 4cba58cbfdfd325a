// Shared definitions of the GB300 fft3d backend: complex helpers, the
// device-side plan of one batched 1-D transform, radix butterflies.
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfft {

// ---------------------------------------------------------------------------
// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi) / 2 (about 48 significant bits), computed on
// the FP32 pipe, which on GB300 issues 64 times the FP64 pipe's rate.  Built
// from error-free transformations: Knuth's TwoSum, Dekker's FastTwoSum and
// the FMA form of TwoProduct (Dekker 1971; the double-double operations of
// Hida, Li and Bailey, 2001).  The sum is the normwise form (TwoSum of the
// high parts, low parts added once): its error is bounded by about
// 2^-46 (|a| + |b|), not by the size of the result, which is the bound the
// normwise error analysis of an FFT uses.  The exponent range is the
// float's: callers scale their data into it (the pipelined complex<double>
// kernels scale each tile by a power of two).
// ---------------------------------------------------------------------------
struct __align__(8) df {
    float hi, lo;
    __host__ __device__ constexpr df() : hi(0.f), lo(0.f) {}
    __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
    // constants of the butterflies (folded at compile time)
    __host__ __device__ constexpr df(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

// A rounded product that the compiler may not contract with a later addition
// into one FMA (the error-free transformations need the rounded value).
__host__ __device__ __forceinline__ float mul_rn(float a, float b){
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

__host__ __device__ __forceinline__ df df_two_sum(float a, float b){
    float s = a + b;
    float bb = s - a;
    return df(s, (a - (s - bb)) + (b - bb));
}
// |a| >= |b| (or a == 0)
__host__ __device__ __forceinline__ df df_fast_two_sum(float a, float b){
    float s = a + b;
    return df(s, b - (s - a));
}
__host__ __device__ __forceinline__ df operator+(df a, df b){
    df s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ df operator-(df a){ return df(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ df operator-(df a, df b){ return a + (-b); }
__host__ __device__ __forceinline__ df operator*(df a, df b){
    float p = mul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);          // exact low part of a.hi * b.hi
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return df_fast_two_sum(p, e);
}
// a * b + c * d, renormalised once (the twiddle products of the FFT stages):
// the two head products summed exactly, the low-order terms added once; the
// error is bounded by about 2^-45 (|a b| + |c d|), the normwise bound
__host__ __device__ __forceinline__ df df_dot2(df a, df b, df c, df d){
    float const p1 = mul_rn(a.hi, b.hi), p2 = mul_rn(c.hi, d.hi);
    float const e1 = fmaf(a.hi, b.hi, -p1), e2 = fmaf(c.hi, d.hi, -p2);
    float const s = p1 + p2;
    float const bb = s - p1;
    float e = ((p1 - (s - bb)) + (p2 - bb)) + (e1 + e2);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    e = fmaf(c.hi, d.lo, e);
    e = fmaf(c.lo, d.hi, e);
    float const h = s + e;
    return df(h, e - (h - s));
}
__device__ __forceinline__ df &operator+=(df &a, df b){ a = a + b; return a; }
__device__ __forceinline__ df &operator*=(df &a, df b){ a = a * b; return a; }
// rounding conversions from / to double (FP64 instructions; for tables)
__device__ __forceinline__ df df_from(double x){
    float hi = __double2float_rn(x);
    return df(hi, __double2float_rn(x - (double)hi));
}
__device__ __forceinline__ double df_to(df a){ return (double)a.hi + (double)a.lo; }

// Bit casts usable on host and device (the conversions below are checked
// bit for bit on the host).
__host__ __device__ __forceinline__ uint64_t bits_of(double x){
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b; __builtin_memcpy(&b, &x, 8); return b;
#endif
}
__host__ __device__ __forceinline__ double double_of(uint64_t b){
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x; __builtin_memcpy(&x, &b, 8); return x;
#endif
}
__host__ __device__ __forceinline__ uint32_t bits_of(float x){
#ifdef __CUDA_ARCH__
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t b; __builtin_memcpy(&b, &x, 4); return b;
#endif
}
__host__ __device__ __forceinline__ float float_of(uint32_t b){
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float x; __builtin_memcpy(&x, &b, 4); return x;
#endif
}

// x * 2^-sh as a float pair without FP64 instructions (integer and FP32
// operations only; the FP64 pipe of GB300 issues 1/64 of the FP32 rate).
// The 53-bit significand M is split into its nearest 24-bit head H (hi, exact)
// and the signed remainder M - H 2^29 (|r| <= 2^28, rounded once to a float:
// lo).  Scaled values below the float normal range (2^-126) are returned as
// zero, and so are zeros and subnormal doubles.  sh must make the scaled
// value < 2^128 (the kernels choose it from the tile's largest exponent).
__host__ __device__ __forceinline__ df df_from_scaled(double x, int sh){
    uint64_t b = bits_of(x);
    uint32_t const sign = (uint32_t)(b >> 32) & 0x80000000u;
    int const e = (int)((b >> 52) & 0x7ff);
    int ef = e - sh - 896;                        // float biased exponent of the scaled value
    if (e == 0 || ef <= 0) return df(0.f, 0.f);
    uint64_t const M = (b & 0xfffffffffffffull) | (1ull << 52);
    uint64_t H = (M + (1ull << 28)) >> 29;        // 2^23 <= H <= 2^24
    int const r = (int)((int64_t)M - (int64_t)(H << 29));
    // lo = r 2^(ef - 179), the power split so both factors are normal floats
    float lo = (float)r * float_of((uint32_t)(ef - 79 + 127) << 23) * float_of((uint32_t)(-100 + 127) << 23);
    if (H == (1ull << 24)){ H >>= 1; ef += 1; }
    float const hi = float_of(sign | ((uint32_t)ef << 23) | ((uint32_t)H & 0x7fffffu));
    return df(hi, sign ? -lo : lo);
}

// float -> double bits by widening (exact); 0 for zero, ~0 for a subnormal
// float (the caller takes its slow path then)
__host__ __device__ __forceinline__ uint64_t widen_bits(float f){
    uint32_t const b = bits_of(f);
    uint32_t const e = (b >> 23) & 0xffu;
    if ((b & 0x7fffffffu) == 0) return (uint64_t)(b & 0x80000000u) << 32;
    if (e == 0 || e == 0xffu) return ~0ull;
    return ((uint64_t)(b & 0x80000000u) << 32) | ((uint64_t)(e + 896) << 52) | ((uint64_t)(b & 0x7fffffu) << 29);
}

// (hi + lo) * 2^sh as a double with a single FP64 instruction (the sum of
// the two exactly widened floats); the power of two is an exponent addition,
// or a multiplication where the result would leave the normal range.
__host__ __device__ __forceinline__ double df_to_scaled(df a, int sh){
    uint64_t const h = widen_bits(a.hi), l = widen_bits(a.lo);
    double const p2 = double_of((uint64_t)(1023 + sh) << 52);     // 2^sh, |sh| <= 1022
    if (h == ~0ull || l == ~0ull) return ((double)a.hi + (double)a.lo) * p2;
    double const s = double_of(h) + double_of(l);
    uint64_t const sb = bits_of(s);
    int const E = (int)((sb >> 52) & 0x7ff);
    if (E == 0 || E + sh <= 0 || E + sh >= 2047) return s * p2;
    return double_of(sb + ((uint64_t)(int64_t)sh << 52));
}

struct __align__(16) cdf { df x, y; };

template<typename T> struct cplx;
template<> struct cplx<float>  { using type = float2; };
template<> struct cplx<double> { using type = double2; };
template<> struct cplx<df>     { using type = cdf; };
template<typename T> using c_t = typename cplx<T>::type;

// read-only cached load of a complex value (twiddle tables)
__device__ __forceinline__ float2 ldg_c(float2 const *p){ return __ldg(p); }
__device__ __forceinline__ double2 ldg_c(double2 const *p){ return __ldg(p); }
__device__ __forceinline__ cdf ldg_c(cdf const *p){
    float4 v = __ldg(reinterpret_cast<float4 const*>(p));
    cdf r;
    r.x = df(v.x, v.y);
    r.y = df(v.z, v.w);
    return r;
}

template<typename T> __host__ __device__ __forceinline__ c_t<T> mk(T re, T im){ c_t<T> r; r.x = re; r.y = im; return r; }
template<typename C> __device__ __forceinline__ C cadd(C a, C b){ C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template<typename C> __device__ __forceinline__ C csub(C a, C b){ C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template<typename C> __device__ __forceinline__ C cmul(C a, C b){
    C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template<typename C> __device__ __forceinline__ C cmulc(C a, C b){
    C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
template<typename C> __device__ __forceinline__ C cconj(C a){ C r; r.x = a.x; r.y = -a.y; return r; }
// double-float complex products through the fused dot (one renormalisation per part)
// a * b + c * d without the final renormalisation: the rounded sum of the
// head products and the sum of every lower-order term; the pair represents
// the value as df_dot2's does, its tail not necessarily below half an ulp of
// its head (the butterflies that take it renormalise)
__host__ __device__ __forceinline__ df df_dot2_lazy(df a, df b, df c, df d){
    float const p1 = mul_rn(a.hi, b.hi), p2 = mul_rn(c.hi, d.hi);
    float const e1 = fmaf(a.hi, b.hi, -p1), e2 = fmaf(c.hi, d.hi, -p2);
    float const s = p1 + p2;
    float const bb = s - p1;
    float e = ((p1 - (s - bb)) + (p2 - bb)) + (e1 + e2);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    e = fmaf(c.hi, d.lo, e);
    e = fmaf(c.lo, d.hi, e);
    return df(s, e);
}
// complex products of the twiddle multiplications (outputs not renormalised)
__host__ __device__ __forceinline__ cdf cmul(cdf a, cdf b){
    cdf r; r.x = df_dot2_lazy(a.x, b.x, -a.y, b.y); r.y = df_dot2_lazy(a.x, b.y, a.y, b.x); return r;
}
__host__ __device__ __forceinline__ cdf cmulc(cdf a, cdf b){
    cdf r; r.x = df_dot2_lazy(a.x, b.x, a.y, b.y); r.y = df_dot2_lazy(a.y, b.x, -a.x, b.y); return r;
}
// Double-float butterflies of radix 2, 4 and 8 with one renormalisation per
// output instead of one per addition: inside a butterfly the sums keep the
// exact sum of the heads (TwoSum) and add the tails without renormalising
// (8 FP32 operations instead of 11); a pair whose tail is not below half an
// ulp of its head still represents the value to about 2^-48 of the operand
// magnitudes (the normwise bound an FFT's error analysis uses), and it is
// renormalised (FastTwoSum) before a product and on the way out.
struct dfb {
    __host__ __device__ static __forceinline__ df add(df a, df b){
        df const s = df_two_sum(a.hi, b.hi);
        return df(s.hi, s.lo + (a.lo + b.lo));
    }
    __host__ __device__ static __forceinline__ df sub(df a, df b){ return add(a, -b); }
    __host__ __device__ static __forceinline__ df norm(df a){ return df_fast_two_sum(a.hi, a.lo); }
    __host__ __device__ static __forceinline__ cdf cadd(cdf a, cdf b){ cdf r; r.x = add(a.x, b.x); r.y = add(a.y, b.y); return r; }
    __host__ __device__ static __forceinline__ cdf csub(cdf a, cdf b){ cdf r; r.x = sub(a.x, b.x); r.y = sub(a.y, b.y); return r; }
    __host__ __device__ static __forceinline__ cdf cnorm(cdf a){ cdf r; r.x = norm(a.x); r.y = norm(a.y); return r; }
    template<bool FWD> __host__ __device__ static __forceinline__ cdf rot(cdf a){
        cdf r;
        if (FWD){ r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
        return r;
    }
    // radix 4 in place, outputs not renormalised
    template<bool FWD> __host__ __device__ static __forceinline__ void r4(cdf *v){
        cdf const a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        cdf const c = cadd(v[1], v[3]), d = rot<FWD>(csub(v[1], v[3]));
        v[0] = cadd(a, c); v[2] = csub(a, c);
        v[1] = cadd(b, d); v[3] = csub(b, d);
    }
    template<int R, bool FWD> __host__ __device__ static __forceinline__ void bfly(cdf *v){
        if constexpr (R == 2){
            cdf const a = v[0], b = v[1];
            v[0] = cnorm(cadd(a, b)); v[1] = cnorm(csub(a, b));
        } else if constexpr (R == 4){
            r4<FWD>(v);
            for (int k = 0; k < 4; k++) v[k] = cnorm(v[k]);
        } else {
            static_assert(R == 8, "double-float butterflies of radix 2, 4, 8");
            cdf e[4] = {v[0], v[2], v[4], v[6]};
            cdf o[4] = {v[1], v[3], v[5], v[7]};
            r4<FWD>(e);
            r4<FWD>(o);
            // o[k] *= w8^k; the products take renormalised operands
            df const h(0.70710678118654752440);
            cdf const o1 = o[1], o3 = o[3];
            if (FWD){
                o[1].x = h * norm(add(o1.x, o1.y)); o[1].y = h * norm(sub(o1.y, o1.x));
                o[3].x = h * norm(sub(o3.y, o3.x)); o[3].y = -(h * norm(add(o3.x, o3.y)));
            } else {
                o[1].x = h * norm(sub(o1.x, o1.y)); o[1].y = h * norm(add(o1.y, o1.x));
                o[3].x = -(h * norm(add(o3.x, o3.y))); o[3].y = h * norm(sub(o3.x, o3.y));
            }
            o[2] = rot<FWD>(o[2]);
            for (int k = 0; k < 4; k++){ v[k] = cnorm(cadd(e[k], o[k])); v[k + 4] = cnorm(csub(e[k], o[k])); }
        }
    }
};

// multiply by -i (forward) or +i (backward)
template<bool FWD, typename C> __device__ __forceinline__ C rot90(C a){
    C r;
    if (FWD){ r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
    return r;
}
template<typename C, typename T> __device__ __forceinline__ C cscale(C a, T s){ C r; r.x = a.x * s; r.y = a.y * s; return r; }

// --------------------------------------------------------------------------
// Plan of one batched 1-D transform as seen by the kernels.
// --------------------------------------------------------------------------
constexpr int kMaxStages = 16;

struct Stage {
    int R;          // radix
    int Ns;         // product of the radices of the previous stages
    int NR;         // N / R (butterflies per transform)
    int tw;         // offset of this stage's twiddles in the table
    uint32_t mul;   // j / Ns = (umulhi(j, mul) + j) >> shift
    int shift;
};

struct Plan1D {
    int N;          // transform length
    int T;          // threads per transform
    int nstages;
    Stage st[kMaxStages];
};

// Layout of a batch of G transforms of length N inside an array:
//   element p of transform g sits at  (g / count) * bstride + (g % count) * dist + p * estride.
struct Layout {
    long long count, dist, bstride, estride;
};

// Padded row pitch (in elements) of workspace-resident boxes whose fastest
// extent e is odd: even (16-byte rows for complex<float>), and a multiple of
// 8 (64-byte rows) from 65 elements on, where the c2r line tiles still fit.
__host__ __device__ constexpr long long padded_pitch(long long e){
    return (e >= 65) ? ((e + 7) / 8) * 8 : e + (e & 1);
}

// 32-bit division where g and count allow it (a 64-bit division is a long
// instruction sequence, and the generic kernels take this per thread per tile)
__device__ __forceinline__ long long base_of(Layout const &L, long long g){
    if (g < 0x7fffffffLL && L.count < 0x7fffffffLL){
        unsigned const gg = (unsigned)g, c = (unsigned)L.count;
        unsigned const q = gg / c;
        return (long long)q * L.bstride + (long long)(gg - q * c) * L.dist;
    }
    return (g / L.count) * L.bstride + (g % L.count) * L.dist;
}

__device__ __forceinline__ int fdiv(int j, Stage const &s){
    return (int)((__umulhi((uint32_t)j, s.mul) + (uint32_t)j) >> s.shift);
}

// Radix constants cos/sin(2 pi m / P) for the odd prime radices P (values of
// the mathematical constants, written out in decimal).  Called with
// compile-time arguments after unrolling, so the switch folds away.
__host__ __device__ __forceinline__ constexpr double prime_cs(int P, int m, bool sine){
    switch (P * 100 + m){
        case 301: return sine ? 0.86602540378443864676 : -0.5;
        case 501: return sine ? 0.95105651629515353118 : 0.30901699437494745126;
        case 502: return sine ? 0.58778525229247324813 : -0.80901699437494734024;
        case 701: return sine ? 0.78183148246802980363 : 0.62348980185873359439;
        case 702: return sine ? 0.97492791218182361934 : -0.22252093395631433737;
        case 703: return sine ? 0.43388373911755823142 : -0.90096886790241903498;
        case 1101: return sine ? 0.54064081745559755543 : 0.84125353283118120551;
        case 1102: return sine ? 0.90963199535451833011 : 0.41541501300188643508;
        case 1103: return sine ? 0.98982144188093279524 : -0.14231483827328500480;
        case 1104: return sine ? 0.75574957435425826890 : -0.65486073394528498959;
        case 1105: return sine ? 0.28173255684142967104 : -0.95949297361449736865;
        case 1301: return sine ? 0.46472317204376850652 : 0.88545602565320991051;
        case 1302: return sine ? 0.82298386589365635224 : 0.56806474673115592289;
        case 1303: return sine ? 0.99270887409805397272 : 0.12053668025532300601;
        case 1304: return sine ? 0.93501624268541483342 : -0.35460488704253545489;
        case 1305: return sine ? 0.66312265824079519305 : -0.74851074817110119231;
        case 1306: return sine ? 0.23931566428755768339 : -0.97094181742605201180;
        default: return 0.0;
    }
}

// Odd prime radix P: y_q = sum_r v_r w^(q r), w = exp(-+ 2 pi i / P).
template<int P, bool FWD, typename C, typename T>
__device__ __forceinline__ void bfly_prime(C *v){
    constexpr int H = (P - 1) / 2;
    C a[H], b[H];
    C v0 = v[0];
    C y0 = v0;
    #pragma unroll
    for (int r = 1; r <= H; r++){
        a[r - 1] = cadd(v[r], v[P - r]);
        b[r - 1] = csub(v[r], v[P - r]);
        y0 = cadd(y0, a[r - 1]);
    }
    #pragma unroll
    for (int q = 1; q <= H; q++){
        C re = v0, im; im.x = 0; im.y = 0;
        #pragma unroll
        for (int r = 1; r <= H; r++){
            int m = (q * r) % P;             // angle index in [1, P-1]
            int mm = (m <= H) ? m : P - m;    // cos symmetric, sin antisymmetric
            T c = (T)prime_cs(P, mm, false);
            T s = (m <= H) ? (T)prime_cs(P, mm, true) : -(T)prime_cs(P, mm, true);
            re.x += a[r - 1].x * c; re.y += a[r - 1].y * c;
            im.x += b[r - 1].x * s; im.y += b[r - 1].y * s;
        }
        // forward: y_q = re - i*im, y_{P-q} = re + i*im (backward swaps)
        C t; t.x = im.y; t.y = -im.x;   // -i * im
        if (FWD){ v[q] = cadd(re, t); v[P - q] = csub(re, t); }
        else    { v[q] = csub(re, t); v[P - q] = cadd(re, t); }
    }
    v[0] = y0;
}

template<int R, bool FWD, typename C, typename T>
__device__ __forceinline__ void bfly(C *v){
    if constexpr (std::is_same<C, cdf>::value && (R == 2 || R == 4 || R == 8)){
        dfb::bfly<R, FWD>(v);
    } else if constexpr (R == 1){
        return;
    } else if constexpr (R == 2){
        C a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    } else if constexpr (R == 4){
        C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        C c = cadd(v[1], v[3]), d = rot90<FWD>(csub(v[1], v[3]));
        v[0] = cadd(a, c); v[2] = csub(a, c);
        v[1] = cadd(b, d); v[3] = csub(b, d);
    } else if constexpr (R == 8){
        const T h = (T)0.70710678118654752440;
        // radix-2 split into even/odd radix-4 transforms
        C e[4] = {v[0], v[2], v[4], v[6]};
        C o[4] = {v[1], v[3], v[5], v[7]};
        bfly<4, FWD, C, T>(e);
        bfly<4, FWD, C, T>(o);
        // o[k] *= w8^k
        C o1 = o[1], o3 = o[3];
        if (FWD){
            o[1].x = h * (o1.x + o1.y); o[1].y = h * (o1.y - o1.x);
            o[3].x = h * (o3.y - o3.x); o[3].y = -h * (o3.x + o3.y);
        } else {
            o[1].x = h * (o1.x - o1.y); o[1].y = h * (o1.y + o1.x);
            o[3].x = -h * (o3.x + o3.y); o[3].y = h * (o3.x - o3.y);
        }
        o[2] = rot90<FWD>(o[2]);
        #pragma unroll
        for (int k = 0; k < 4; k++){ v[k] = cadd(e[k], o[k]); v[k + 4] = csub(e[k], o[k]); }
    } else if constexpr (R == 16){
        // 4 x 4: columns, internal twiddles w16^(k1 n2), rows
        const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173, h = (T)0.70710678118654752440;
        C x[16];
        #pragma unroll
        for (int n2 = 0; n2 < 4; n2++){
            C t[4] = {v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]};
            bfly<4, FWD, C, T>(t);
            #pragma unroll
            for (int k1 = 0; k1 < 4; k1++) x[k1 * 4 + n2] = t[k1];
        }
        // twiddles w16^(k1*n2): exponents 0..9
        auto tw = [&](C a, int e) -> C {
            // multiply by exp(-+ 2 pi i e / 16)
            C r;
            T cs, sn;
            switch (e){
                case 1: cs = c1; sn = s1; break;
                case 2: cs = h; sn = h; break;
                case 3: cs = s1; sn = c1; break;
                case 4: cs = 0; sn = 1; break;
                case 6: cs = -h; sn = h; break;
                case 9: cs = -c1; sn = -s1; break;
                default: cs = 1; sn = 0; break;
            }
            if (FWD) sn = -sn;
            r.x = a.x * cs - a.y * sn; r.y = a.x * sn + a.y * cs;
            return r;
        };
        #pragma unroll
        for (int k1 = 1; k1 < 4; k1++){
            #pragma unroll
            for (int n2 = 1; n2 < 4; n2++) x[k1 * 4 + n2] = tw(x[k1 * 4 + n2], k1 * n2);
        }
        #pragma unroll
        for (int k1 = 0; k1 < 4; k1++){
            C t[4] = {x[k1 * 4 + 0], x[k1 * 4 + 1], x[k1 * 4 + 2], x[k1 * 4 + 3]};
            bfly<4, FWD, C, T>(t);
            #pragma unroll
            for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = t[k2];
        }
    } else if constexpr (R == 3){
        bfly_prime<3, FWD, C, T>(v);
    } else if constexpr (R == 5){
        bfly_prime<5, FWD, C, T>(v);
    } else if constexpr (R == 7){
        bfly_prime<7, FWD, C, T>(v);
    } else if constexpr (R == 11){
        bfly_prime<11, FWD, C, T>(v);
    } else if constexpr (R == 13){
        bfly_prime<13, FWD, C, T>(v);
    }
}

} // namespace gbfft
