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

    // the butterflies with one renormalisation per output (radix 2, 4, 8,
    // both directions) against the exact DFT in long double, normwise
    // (|error| over the sum of the input magnitudes), with inputs of mixed
    // magnitudes and cancelling pairs
    double w_b[3] = {0, 0, 0};
    bool tails_ok = true;
    for (int i = 0; i < 300000; i++){
        cdf v[8];
        LD xr[8], xi[8];
        for (int k = 0; k < 8; k++){
            LD a = u(rng), b = u(rng);
            if (i % 5 == 0 && k % 2 == 1){ a = -xr[k - 1] * (1 + 1e-7L); b = -xi[k - 1]; }
            if (i % 7 == 0) { a = std::ldexp(a, (int)(rng() % 40) - 20); b = std::ldexp(b, (int)(rng() % 40) - 20); }
            v[k].x = split(a); v[k].y = split(b);
            xr[k] = val(v[k].x); xi[k] = val(v[k].y);
        }
        for (int ri = 0; ri < 3; ri++){
            int const R = ri == 0 ? 2 : (ri == 1 ? 4 : 8);
            bool const fwd = (i & 1) == 0;
            cdf w[8];
            for (int k = 0; k < 8; k++) w[k] = v[k];
            if (R == 2){ if (fwd) dfb::bfly<2, true>(w); else dfb::bfly<2, false>(w); }
            else if (R == 4){ if (fwd) dfb::bfly<4, true>(w); else dfb::bfly<4, false>(w); }
            else { if (fwd) dfb::bfly<8, true>(w); else dfb::bfly<8, false>(w); }
            LD sum = 0;
            for (int k = 0; k < R; k++) sum += std::fabs(xr[k]) + std::fabs(xi[k]);
            for (int q = 0; q < R; q++){
                LD er = 0, ei = 0;
                for (int k = 0; k < R; k++){
                    LD ang = (fwd ? -2 : 2) * 3.14159265358979323846264338327950288L * (LD)(q * k % R) / R;
                    er += xr[k] * std::cos(ang) - xi[k] * std::sin(ang);
                    ei += xr[k] * std::sin(ang) + xi[k] * std::cos(ang);
                }
                double e = (double)(std::hypot(val(w[q].x) - er, val(w[q].y) - ei) / sum);
                if (e > w_b[ri]) w_b[ri] = e;
                // every output renormalised: the tail within half an ulp of the head
                for (df const &d : {w[q].x, w[q].y})
                    if (d.hi != 0 && std::fabs((LD)d.lo) > std::ldexp(std::fabs((LD)d.hi), -23)) tails_ok = false;
            }
        }
    }
    report("radix-2 butterfly, normwise", w_b[0], u45);
    report("radix-4 butterfly, normwise", w_b[1], u45);
    report("radix-8 butterfly, normwise", w_b[2], u45);
    printf("%-44s %s\n", "butterfly outputs renormalised", tails_ok ? "ok" : "FAIL");
    if (!tails_ok) fails++;
    return fails ? 1 : 0;
}
