// The batch kernel with 16 values per thread (see gbfft_batch_kernel.cuh).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e16(int prec, bool fwd, bool r2c){
    if (r2c){
        if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, true>)
                                  : reinterpret_cast<void const*>(k_batch<float, false, 16, true>);
        return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, true>)
                   : reinterpret_cast<void const*>(k_batch<double, false, 16, true>);
    }
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 16, false>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 16, false>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 16, false>)
               : reinterpret_cast<void const*>(k_batch<double, false, 16, false>);
}

} // namespace gbfft
