// The batch kernel with 16 values per thread, any batch (see gbfft_batch_kernel.cuh;
// one translation unit per form so that they compile in parallel).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e16_any(int prec, bool fwd){
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, false, false>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 16, false, false>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, false, false>)
               : reinterpret_cast<void const*>(k_batch<double, false, 16, false, false>);
}

} // namespace gbfft
