// Host check of the compile-time radix plans of the runtime-radix pipelined
// kernels (ct_plan in heffte_gb300/csrc/gbfft_pipe_rt.cuh) against the plans
// the library builds (get_fft1d): for every length up to 8192 that is not a
// power of two and that the radix kernels take directly, the constexpr plan
// has the library's stages (radix, Ns, N / R, twiddle offset), threads per
// transform and twiddle count, so a kernel compiled for any such length
// would run that length's default plan.  Also checks that the lengths with
// compiled kernels are among them, and that their per-stage transposed
// twiddle copy is read back as the Stockham table.  No GPU call.
#include "../../heffte_gb300/csrc/gbfft_pipe_rt.cuh"
#include "../../heffte_gb300/csrc/gbfft_internal.h"
#include <cstdio>
#include <vector>

using namespace gbfft;

int main(){
    int fails = 0, checked = 0;
    for (int N = 3; N <= 8192; N++){
        if ((N & (N - 1)) == 0 || !direct_length(N)) continue;
        std::shared_ptr<Fft1D> f = get_fft1d(N);
        Plan1D const &P = f->plan;
        CtPlan const c = ct_plan(N, kEmax);
        bool ok = c.nstages == P.nstages && c.T == P.T && c.N == N;
        int tw = 0;
        for (int s = 0; ok && s < P.nstages; s++){
            ok = c.R[s] == P.st[s].R && c.Ns[s] == P.st[s].Ns && c.NR[s] == P.st[s].NR && c.tw[s] == P.st[s].tw;
            if (s > 0) tw += P.st[s].Ns * (P.st[s].R - 1);
        }
        ok = ok && ct_twiddles(N, kEmax) == tw;
        if (!ok){
            printf("FAIL: N=%d compile-time plan differs from the library's\n", N);
            fails++;
        }
        checked++;
    }
    for (int N : {96, 160, 192, 240, 288, 320, 384, 448, 480, 576, 640, 720, 768, 960})
        if (!direct_length(N) || ct_plan(N, kEmax).nstages == 0){
            printf("FAIL: compiled length %d has no direct plan\n", N);
            fails++;
        }
    // the twiddle copy of the compiled kernels (ct_copy_twiddles: global
    // entry TWO + i, i = k (R - 1) + q - 1, to TWO + (q - 1) Ns + k) read back
    // where the stages read it (fft_stage_ct with TWS) gives the Stockham
    // table's entry of butterfly column k and twiddle q, for every stage
    for (int N : {96, 160, 192, 240, 288, 320, 384, 448, 480, 576, 640, 720, 768, 960}){
        CtPlan const c = ct_plan(N, kEmax);
        int const n = ct_twiddles(N, kEmax);
        std::vector<int> g(n), d(n, -1);
        for (int i = 0; i < n; i++) g[i] = i;
        for (int s = 1; s < c.nstages; s++){
            int const R1 = c.R[s] - 1;
            for (int i = 0; i < c.Ns[s] * R1; i++){
                int k = i / R1, q1 = i - k * R1;
                d[c.tw[s] + q1 * c.Ns[s] + k] = g[c.tw[s] + i];
            }
        }
        for (int s = 1; s < c.nstages; s++)
            for (int k = 0; k < c.Ns[s]; k++)
                for (int q = 1; q < c.R[s]; q++)
                    if (d[c.tw[s] + (q - 1) * c.Ns[s] + k] != c.tw[s] + k * (c.R[s] - 1) + q - 1){
                        printf("FAIL: N=%d stage %d k=%d q=%d: transposed twiddle\n", N, s, k, q);
                        fails++;
                    }
    }
    printf("%d lengths checked\n", checked);
    if (fails == 0) printf("compile-time plans ok\n");
    return fails ? 1 : 0;
}
