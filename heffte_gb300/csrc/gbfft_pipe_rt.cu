// Instantiations and launch of the pipelined runtime-radix complex kernels
// (gbfft_pipe_rt.cuh): float and double, forward and backward, line tiles
// (1-D bulk copies) and column tiles (3-D tensor-map copies).
#include "gbfft_pipe_rt.cuh"
#include <atomic>

namespace gbfft {

namespace {

template<typename T, bool FWD, bool COLS, int LOADER>
void launch_one(cudaStream_t s, PipeRtParams const &P, CUtensorMap const &tmap, size_t smem, int threads){
    auto kern = k_pipe_rt<T, FWD, COLS, LOADER>;
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

template<typename T>
void dispatch(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, CUtensorMap const &tmap, size_t smem,
              int threads){
    if (cols){
        if (fwd) launch_one<T, true, true, RT_LD_TENSOR>(s, P, tmap, smem, threads);
        else launch_one<T, false, true, RT_LD_TENSOR>(s, P, tmap, smem, threads);
    } else {
        if (fwd) launch_one<T, true, false, RT_LD_BULK>(s, P, tmap, smem, threads);
        else launch_one<T, false, false, RT_LD_BULK>(s, P, tmap, smem, threads);
    }
}

} // namespace

void launch_pipe_rt(cudaStream_t s, int prec, bool fwd, bool cols, PipeRtParams const &P, void const *tmap,
                    size_t smem, int threads){
    CUtensorMap const &m = *reinterpret_cast<CUtensorMap const*>(tmap);
    if (prec == 0) dispatch<float>(s, fwd, cols, P, m, smem, threads);
    else dispatch<double>(s, fwd, cols, P, m, smem, threads);
}

} // namespace gbfft
