// Host check of the compile-time radix plans of the runtime-radix pipelined
// kernels (ct_plan in heffte_gb300/csrc/gbfft_pipe_rt.cuh) against the plans
// the library builds (get_fft1d): for every length up to 8192 that is not a
// power of two and that the radix kernels take directly, the constexpr plan
// has the library's stages (radix, Ns, N / R, twiddle offset), threads per
// transform and twiddle count, so a kernel compiled for any such length
// would run that length's default plan.  Also checks that the lengths with
// compiled kernels are among them.  No GPU call.
#include "../../heffte_gb300/csrc/gbfft_pipe_rt.cuh"
#include "../../heffte_gb300/csrc/gbfft_internal.h"
#include <cstdio>

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
    printf("%d lengths checked\n", checked);
    if (fails == 0) printf("compile-time plans ok\n");
    return fails ? 1 : 0;
}
