// The batch kernel with 16 values per thread, r2c batches of 5-smooth plans (see gbfft_batch_kernel.cuh;
// one translation unit per form so that they compile in parallel).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e16_r2c5(int prec, bool fwd){
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true, true>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 16, true, true>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, true, true>)
               : reinterpret_cast<void const*>(k_batch<double, false, 16, true, true>);
}

void const *batch_kernel_e16_r2c5_tw(bool fwd){
    return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true, true, true>)
               : reinterpret_cast<void const*>(k_batch<float, false, 16, true, true, true>);
}

} // namespace gbfft
