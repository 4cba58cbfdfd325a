// Instantiations and launch of the pipelined runtime-radix complex kernels
// (gbfft_pipe_rt.cuh): float and double, forward and backward, line tiles
// (1-D bulk copies) and column tiles (3-D tensor-map copies).  Float
// transforms of the lengths in kRtCtLengths run the kernels compiled for
// that length's plan (gbfft_pipe_rt_n*.cu) when the plan is the default one.
#include "gbfft_pipe_rt_launch.inl"

namespace gbfft {

static bool launch_ct(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, void const *tmap, size_t smem,
                      int threads){
    switch (P.plan.N){
        case 320: return launch_pipe_rt_ct<320>(s, fwd, cols, P, tmap, smem, threads);
        case 384: return launch_pipe_rt_ct<384>(s, fwd, cols, P, tmap, smem, threads);
        case 448: return launch_pipe_rt_ct<448>(s, fwd, cols, P, tmap, smem, threads);
        case 480: return launch_pipe_rt_ct<480>(s, fwd, cols, P, tmap, smem, threads);
        case 640: return launch_pipe_rt_ct<640>(s, fwd, cols, P, tmap, smem, threads);
        case 768: return launch_pipe_rt_ct<768>(s, fwd, cols, P, tmap, smem, threads);
        default: return false;
    }
}

void launch_pipe_rt(cudaStream_t s, int prec, bool fwd, bool cols, PipeRtParams const &P, void const *tmap,
                    size_t smem, int threads){
    CUtensorMap const &m = *reinterpret_cast<CUtensorMap const*>(tmap);
    if (prec == 0){
        if (rt_compiled_plans() && launch_ct(s, fwd, cols, P, tmap, smem, threads)) return;
        dispatch<float, 0>(s, fwd, cols, P, m, smem, threads);
    } else {
        dispatch<double, 0>(s, fwd, cols, P, m, smem, threads);
    }
}

} // namespace gbfft
