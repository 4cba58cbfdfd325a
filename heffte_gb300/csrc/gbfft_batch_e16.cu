// The batch kernel with 16 values per thread (see gbfft_batch_kernel.cuh).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e16(int prec, bool fwd, bool r2c, bool s5){
    // r2c batches: 5-smooth or any plans; other batches: any plans
    if (r2c && s5){
        if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true, true>)
                                  : reinterpret_cast<void const*>(k_batch<float, false, 16, true, true>);
        return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, true, true>)
                   : reinterpret_cast<void const*>(k_batch<double, false, 16, true, true>);
    }
    if (r2c){
        if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true, false>)
                                  : reinterpret_cast<void const*>(k_batch<float, false, 16, true, false>);
        return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, true, false>)
                   : reinterpret_cast<void const*>(k_batch<double, false, 16, true, false>);
    }
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, false, false>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 16, false, false>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, false, false>)
               : reinterpret_cast<void const*>(k_batch<double, false, 16, false, false>);
}

} // namespace gbfft
