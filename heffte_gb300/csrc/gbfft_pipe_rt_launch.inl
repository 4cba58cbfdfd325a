// Launch of the pipelined runtime-radix complex kernels (gbfft_pipe_rt.cuh),
// shared by gbfft_pipe_rt.cu (runtime plans) and the instantiation units of
// the compile-time plans (gbfft_pipe_rt_n*.cu: #define GBFFT_RT_LEN, then
// include this file).
#include "gbfft_pipe_rt.cuh"
#include <atomic>

namespace gbfft {

namespace {

template<typename T, bool FWD, bool COLS, int LOADER, int NC, bool TWS>
void launch_one(cudaStream_t s, PipeRtParams const &P, CUtensorMap const &tmap, size_t smem, int threads){
    auto kern = k_pipe_rt<T, FWD, COLS, LOADER, NC, TWS>;
    static std::atomic<unsigned long long> ready{0};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    unsigned long long bit = 1ull << (dev & 63);
    if (!(ready.load() & bit)){
        // the opt-in maximum per block less the kernel's static shared memory
        int optin = 0;
        check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "device attribute");
        cudaFuncAttributes fa{};
        check_cuda(cudaFuncGetAttributes(&fa, kern), "function attributes");
        check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes),
                   "cudaFuncSetAttribute(pipelined runtime-radix kernel)");
        ready.fetch_or(bit);
    }
    int nb = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem), "occupancy query");
    long long grid = std::min<long long>(P.ntiles, (long long)num_sms() * std::max(nb, 1));
    kern<<<(unsigned)grid, threads, smem, s>>>(P, tmap);
    check_cuda(cudaPeekAtLastError(), "pipelined runtime-radix kernel launch");
}

template<typename T, int NC, bool TWS>
void dispatch(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, CUtensorMap const &tmap, size_t smem,
              int threads){
    if (cols){
        if (fwd) launch_one<T, true, true, RT_LD_TENSOR, NC, TWS>(s, P, tmap, smem, threads);
        else launch_one<T, false, true, RT_LD_TENSOR, NC, TWS>(s, P, tmap, smem, threads);
    } else {
        if (fwd) launch_one<T, true, false, RT_LD_BULK, NC, TWS>(s, P, tmap, smem, threads);
        else launch_one<T, false, false, RT_LD_BULK, NC, TWS>(s, P, tmap, smem, threads);
    }
}

} // namespace

#ifdef GBFFT_RT_LEN
template<>
bool launch_pipe_rt_ct<GBFFT_RT_LEN>(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, void const *tmap,
                                     size_t smem, int threads){
    if (!ct_plan_matches<GBFFT_RT_LEN>(P.plan)) return false;
    if (!cols && threads > 256) return false;   // compiled line kernels: 256 threads at most
    CUtensorMap const &m = *reinterpret_cast<CUtensorMap const*>(tmap);
    // P.ct: 1 twiddles in shared memory (counted in smem), 2 in global memory
    if (P.ct == 1) dispatch<float, GBFFT_RT_LEN, true>(s, fwd, cols, P, m, smem, threads);
    else dispatch<float, GBFFT_RT_LEN, false>(s, fwd, cols, P, m, smem, threads);
    return true;
}
#endif

} // namespace gbfft
