// The batch kernel with 16 values per thread, r2c batches (see gbfft_batch_kernel.cuh;
// one translation unit per form so that they compile in parallel).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e16_r2c(int prec, bool fwd){
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true, false>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 16, true, false>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, true, false>)
               : reinterpret_cast<void const*>(k_batch<double, false, 16, true, false>);
}

} // namespace gbfft
