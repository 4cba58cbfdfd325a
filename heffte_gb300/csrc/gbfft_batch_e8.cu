// The batch kernel with 8 values per thread (see gbfft_batch_kernel.cuh).
#include "gbfft_batch_kernel.cuh"

namespace gbfft {

void const *batch_kernel_e8(int prec, bool fwd, bool r2c){
    if (r2c){
        if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 8, true>)
                                  : reinterpret_cast<void const*>(k_batch<float, false, 8, true>);
        return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 8, true>)
                   : reinterpret_cast<void const*>(k_batch<double, false, 8, true>);
    }
    if (prec == 0) return fwd ? reinterpret_cast<void const*>(k_batch<float, true, 8, false>)
                              : reinterpret_cast<void const*>(k_batch<float, false, 8, false>);
    return fwd ? reinterpret_cast<void const*>(k_batch<double, true, 8, false>)
               : reinterpret_cast<void const*>(k_batch<double, false, 8, false>);
}

} // namespace gbfft
