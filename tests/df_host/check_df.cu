// Host check of the double-float arithmetic of the complex<double> kernels
// (heffte_gb300/csrc/gbfft_common.cuh): the same functions the device runs,
// compiled for the host, against long double arithmetic.  Prints one line
// per check and exits non-zero on the first bound that does not hold.
#include "../../heffte_gb300/csrc/gbfft_common.cuh"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using namespace gbfft;
typedef long double LD;

static LD val(df a){ return (LD)a.hi + (LD)a.lo; }
static df split(LD v){ float h = (float)v; return df(h, (float)(v - (LD)h)); }
static int fails = 0;
static void report(char const *what, double worst, double bound){
    bool ok = worst <= bound;
    printf("%-44s worst %.3e bound %.3e %s\n", what, worst, bound, ok ? "ok" : "FAIL");
    if (!ok) fails++;
}

int main(){
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1, 1);
    std::uniform_int_distribution<int> ex(-1000, 1000);
    double const u45 = std::ldexp(1.0, -45);

    // double -> float pair (scaled by 2^-sh) -> double, with the kernels' choice
    // of sh (the value's exponent, so the scaled value lies in [1, 2)) and a
    // spread below it (values down to 2^-100 of the tile's largest)
    double worst_from = 0, worst_round = 0, worst_lo = 0;
    long long exact_back = 0, checked = 0;
    for (int i = 0; i < 2000000; i++){
        double x = std::ldexp(u(rng), ex(rng));
        if (i % 97 == 0) x = std::nextafter(1.0, 2.0) * std::ldexp(1.0, ex(rng));          // significand edges
        if (i % 101 == 0) x = std::ldexp((double)((1ull << 53) - 1), ex(rng) - 52);       // carry into hi
        if (x == 0) continue;
        int e; std::frexp(x, &e);
        int sh = (e - 1) + ((i % 3 == 0) ? (int)(rng() % 100) : 0);
        sh = std::min(std::max(sh, -1022), 1022);
        df a = df_from_scaled(x, sh);
        LD want = std::ldexp((LD)x, -sh);
        if (std::fabs(want) < std::ldexp(1.0L, -126)) continue;     // dropped by design
        worst_from = std::max(worst_from, (double)(std::fabs(val(a) - want) / std::fabs(want)));
        worst_lo = std::max(worst_lo, (double)(std::fabs((LD)a.lo) / std::fabs((LD)a.hi)));
        double back = df_to_scaled(a, sh);
        checked++;
        worst_round = std::max(worst_round, std::fabs(back - x) / std::fabs(x));
        // the way back is the one rounding of the exact sum hi + lo
        if (back == (double)std::ldexp(val(a), sh)) exact_back++;
    }
    report("double -> float pair, relative", worst_from, std::ldexp(1.0, -48));
    report("float pair lo / hi", worst_lo, std::ldexp(1.0, -23));
    report("double -> float pair -> double, relative", worst_round, std::ldexp(1.0, -47));
    printf("%-44s %lld of %lld %s\n", "way back equals RN(hi + lo) * 2^sh", exact_back, checked,
           exact_back == checked ? "ok" : "FAIL");
    if (exact_back != checked) fails++;

    // sums, products and the twiddle dot product, normwise (the bounds the
    // FFT error analysis uses), with cancellation cases
    double w_add = 0, w_mul = 0, w_dot = 0, w_cmul = 0;
    for (int i = 0; i < 2000000; i++){
        LD A = u(rng), B = u(rng), C = u(rng), D = u(rng);
        if (i % 7 == 0){ C = -A; D = B * (1 + 1e-9L); }
        df a = split(A), b = split(B), c = split(C), d = split(D);
        LD va = val(a), vb = val(b), vc = val(c), vd = val(d);
        w_add = std::max(w_add, (double)(std::fabs(val(a + b) - (va + vb)) / (std::fabs(va) + std::fabs(vb))));
        w_add = std::max(w_add, (double)(std::fabs(val(a - c) - (va - vc)) / (std::fabs(va) + std::fabs(vc))));
        w_mul = std::max(w_mul, (double)(std::fabs(val(a * b) - va * vb) / std::fabs(va * vb)));
        LD dot = va * vb + vc * vd;
        w_dot = std::max(w_dot, (double)(std::fabs(val(df_dot2(a, b, c, d)) - dot) / (std::fabs(va * vb) + std::fabs(vc * vd))));
        cdf z{a, c}, w{b, d};
        cdf r = cmul(z, w);
        LD re = va * vb - vc * vd, im = va * vd + vc * vb;
        LD nz = std::sqrt(va * va + vc * vc), nw = std::sqrt(vb * vb + vd * vd);
        w_cmul = std::max(w_cmul, (double)(std::hypot(val(r.x) - re, val(r.y) - im) / (nz * nw)));
    }
    report("a + b, a - b: |err| / (|a| + |b|)", w_add, std::ldexp(1.0, -46));
    report("a * b, relative", w_mul, std::ldexp(1.0, -45));
    report("a b + c d: |err| / (|a b| + |c d|)", w_dot, u45);
    report("complex product: |err| / (|z| |w|)", w_cmul, 2 * u45);
    return fails ? 1 : 0;
}
