// Host check of the compile-time tables of the pipelined kernels
// (heffte_gb300/csrc/gbfft_pipe.cuh): every radix plan multiplies to its
// length, the double-float plans have no radix above 8 and hold 8 values per
// thread, each stage's butterflies fill a thread's values exactly, the
// twiddle offsets follow the Stockham layout, and the line-exchange swizzle
// is a permutation within each line that spreads every stage's 16-byte
// accesses of a quarter warp over distinct bank groups.
#include "../../heffte_gb300/csrc/gbfft_pipe.cuh"
#include <cstdio>
#include <vector>

using namespace gbfft;
static int fails = 0;
#define CHECK(c, ...) do { if (!(c)){ printf("FAIL: " __VA_ARGS__); printf("\n"); fails++; } } while (0)

int main(){
    for (int N = 2; N <= 4096; N *= 2){
        for (int df = 0; df < 2; df++){
            int const ns = pipe_nstages(N, df), pe = pipe_pe(N, df), tt = pipe_tt(N, df);
            long long prod = 1;
            int off = 0, Ns = 1;
            for (int s = 0; s < ns; s++){
                int const R = pipe_radix(N, s, df);
                CHECK(R >= 2 && R <= (df ? 8 : 16), "N=%d df=%d stage %d radix %d", N, df, s, R);
                CHECK(pe % R == 0, "N=%d df=%d: radix %d does not divide %d values", N, df, R, pe);
                CHECK(pipe_ns(N, s, df) == Ns, "N=%d df=%d: Ns of stage %d", N, df, s);
                CHECK(pipe_twoff(N, s, df) == off, "N=%d df=%d: twiddle offset of stage %d", N, df, s);
                if (s > 0) off += Ns * (R - 1);
                Ns *= R;
                prod *= R;
            }
            CHECK(prod == N, "N=%d df=%d: radices multiply to %lld", N, df, prod);
            CHECK(tt * pe == N, "N=%d df=%d: %d threads x %d values", N, df, tt, pe);
            CHECK(!df || N < 8 || pe == 8, "N=%d: double-float values per thread %d", N, pe);
        }
        // swizzle: a permutation within each aligned group of 8
        std::vector<int> seen(N, 0);
        for (int p = 0; p < N; p++){
            int const q = pipe_swz(p);
            CHECK(q >= 0 && q < N && (q & ~7) == (p & ~7), "N=%d: swizzle of %d is %d", N, p, q);
            if (q >= 0 && q < N) seen[q]++;
        }
        for (int q = 0; q < N; q++) CHECK(seen[q] == 1, "N=%d: swizzle not a permutation at %d", N, q);
        // conflict-free exchange of the double-float line tiles: each stage's
        // reads (S > 0) and writes (not the last stage), eight lanes at a time
        if (N >= 16){
            int const ns = pipe_nstages(N, true), tt = pipe_tt(N, true), pe = pipe_pe(N, true);
            int Ns = 1;
            for (int s = 0; s < ns; s++){
                int const R = pipe_radix(N, s, true), NR = N / R, M = pe / R;
                int const LNS = cilog2(Ns), LNSR = cilog2(Ns * R);
                for (int m = 0; m < M; m++)
                    for (int q = 0; q < R; q++)
                        for (int l0 = 0; l0 < (tt < 32 ? tt : 32); l0 += 8){
                            int rb[8] = {0}, wb[8] = {0}, lanes = 0;
                            for (int l = l0; l < l0 + 8 && l < tt; l++, lanes++){
                                int const j = l + m * tt, k = j & (Ns - 1);
                                rb[pipe_swz(j + q * NR) & 7]++;
                                wb[pipe_swz(((j >> LNS) << LNSR) + k + q * Ns) & 7]++;
                            }
                            for (int g = 0; g < 8; g++){
                                CHECK(s == 0 || rb[g] <= 1, "N=%d stage %d: %d reads in bank group %d", N, s, rb[g], g);
                                CHECK(s == ns - 1 || wb[g] <= 1, "N=%d stage %d: %d writes in bank group %d", N, s, wb[g], g);
                            }
                        }
                Ns *= R;
            }
        }
    }
    printf("%s\n", fails ? "FAIL" : "plans and swizzle ok");
    return fails ? 1 : 0;
}
