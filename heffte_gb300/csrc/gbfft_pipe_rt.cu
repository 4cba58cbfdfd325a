// Instantiations and launch of the pipelined runtime-radix complex kernels
// (gbfft_pipe_rt.cuh): float and double, forward and backward, line tiles
// (1-D bulk copies) and column tiles (3-D tensor-map copies).  Float
// transforms of the lengths in GBFFT_RT_CT_LENGTHS run the kernels compiled
// for that length's plan (gbfft_pipe_rt_n*.cu) when the plan is the default one.
#include "gbfft_pipe_rt_launch.inl"

namespace gbfft {

template<int NC>
static size_t ct_smem(Plan1D const &plan){
    return ct_plan_matches<NC>(plan) ? (size_t)ct_twiddles(NC, kEmax) * sizeof(float2) : 0;
}

size_t rt_ct_smem(Plan1D const &plan){
    if (!rt_compiled_plans()) return 0;
    switch (plan.N){
#define GBFFT_CASE(n) case n: return ct_smem<n>(plan);
        GBFFT_RT_CT_LENGTHS(GBFFT_CASE)
#undef GBFFT_CASE
        default: return 0;
    }
}

static bool launch_ct(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, void const *tmap, size_t smem,
                      int threads){
    switch (P.plan.N){
#define GBFFT_CASE(n) case n: return launch_pipe_rt_ct<n>(s, fwd, cols, P, tmap, smem, threads);
        GBFFT_RT_CT_LENGTHS(GBFFT_CASE)
#undef GBFFT_CASE
        default: return false;
    }
}

void launch_pipe_rt(cudaStream_t s, int prec, bool fwd, bool cols, PipeRtParams const &P, void const *tmap,
                    size_t smem, int threads){
    CUtensorMap const &m = *reinterpret_cast<CUtensorMap const*>(tmap);
    if (prec == 0){
        // P.ct: a compiled kernel, with its twiddles in shared memory (1, counted
        // in smem) or in global memory (2)
        if (P.ct && launch_ct(s, fwd, cols, P, tmap, smem, threads)) return;
        dispatch<float, 0, false>(s, fwd, cols, P, m, smem, threads);
    } else {
        dispatch<double, 0, false>(s, fwd, cols, P, m, smem, threads);
    }
}

} // namespace gbfft
