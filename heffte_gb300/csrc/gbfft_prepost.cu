// Location-layer pre/post processors of the extended-signal DCT/DST method,
// the roles of cuda::{cos,sin,cos1}_pre_pos_processor (include/heffte_backend_cuda.h:116-174,
// src/heffte_backend_cuda.cu:149-327), batched over lines (one launch for all
// lines instead of one per line).  Each output entry is a closed formula of
// its index, so every entry of the output line is written exactly once.
//
// Per line (N input values, extended length M = 4N, or 4(N-1) for cos1, H = M/2+1):
//   step 0 pre_forward : real N      -> real M   (symmetric embedding, 0 at even/odd slots)
//   step 1 post_forward: complex H   -> real N   (Re X_k, or -Im X_{k+1} for sin)
//   step 2 pre_backward: real N      -> complex H
//   step 3 post_backward: real M     -> real N   (odd entries, even entries for cos1)
// Also the pointwise spectrum product of the unfused convolution path.
#include "gbfft_internal.h"

namespace gbfft {

template<typename T>
__global__ void __launch_bounds__(256)
k_prepost(int kind, int step, int N, long long lines, long long in_ld, long long out_ld, int out_len,
          void const *inp, void *outp){
    long long total = lines * (long long)out_len;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x){
        long long b = idx / out_len;
        int m = (int)(idx - b * out_len);
        if (step == 0){
            T const *x = reinterpret_cast<T const*>(inp) + b * in_ld;
            T *o = reinterpret_cast<T*>(outp) + b * out_ld;
            T v = 0;
            if (kind == 2){
                if (!(m & 1)){
                    int i = m / 2;
                    v = (i < N - 1) ? x[i] : x[(4 * N - 4 - m) / 2];
                }
            } else if (m & 1){
                if (m < 2 * N) v = x[(m - 1) / 2];
                else v = (kind == 1) ? -x[(4 * N - m - 1) / 2] : x[(4 * N - m - 1) / 2];
            }
            o[m] = v;
        } else if (step == 1){
            c_t<T> const *X = reinterpret_cast<c_t<T> const*>(inp) + b * in_ld;
            T *o = reinterpret_cast<T*>(outp) + b * out_ld;
            o[m] = (kind == 1) ? -X[m + 1].y : X[m].x;
        } else if (step == 2){
            T const *x = reinterpret_cast<T const*>(inp) + b * in_ld;
            c_t<T> *o = reinterpret_cast<c_t<T>*>(outp) + b * out_ld;
            c_t<T> v = mk<T>(0, 0);
            if (kind == 0){
                if (m < N) v.x = x[m];
                else if (m > N) v.x = -x[2 * N - m];
            } else if (kind == 1){
                if (m >= 1 && m <= N) v.y = -x[m - 1];
                else if (m > N && m < 2 * N) v.y = -x[2 * N - m - 1];
            } else {
                v.x = (m < N) ? x[m] : x[2 * N - 2 - m];
            }
            o[m] = v;
        } else {
            T const *r = reinterpret_cast<T const*>(inp) + b * in_ld;
            T *o = reinterpret_cast<T*>(outp) + b * out_ld;
            o[m] = (kind == 2) ? r[2 * m] : r[2 * m + 1];
        }
    }
}

void launch_prepost(cudaStream_t s, int prec, int kind, int step, int N, long long lines, long long in_ld,
                    long long out_ld, void const *in, void *out){
    int M = (kind == 2) ? 4 * (N - 1) : 4 * N;
    int out_len = (step == 0) ? M : ((step == 2) ? M / 2 + 1 : N);
    long long total = lines * (long long)out_len;
    if (total <= 0) return;
    long long blocks = std::min<long long>((total + 255) / 256, (long long)num_sms() * 32);
    if (prec == 0) k_prepost<float><<<(unsigned)blocks, 256, 0, s>>>(kind, step, N, lines, in_ld, out_ld, out_len, in, out);
    else k_prepost<double><<<(unsigned)blocks, 256, 0, s>>>(kind, step, N, lines, in_ld, out_ld, out_len, in, out);
}

} // namespace gbfft

namespace gbfft {

// Pointwise product of two spectra (the middle step of benchmarks/convolution.cpp,
// output_array[i] *= output_array[i] there), scaled: a[i] = a[i] * b[i] * s,
// or a[i]^2 * s when b is null.  Grid-stride over n complex values.
template<typename T>
__global__ void __launch_bounds__(256)
k_pointwise(long long n, c_t<T> *a, c_t<T> const *b, T s){
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x){
        c_t<T> u = a[i];
        c_t<T> v = b ? b[i] : u;
        a[i] = cscale(cmul(u, v), s);
    }
}

void launch_pointwise(cudaStream_t s, int prec, long long n, void *a, void const *b, double scale){
    if (n <= 0) return;
    long long blocks = std::min<long long>((n + 255) / 256, (long long)num_sms() * 16);
    if (prec == 0)
        k_pointwise<float><<<(unsigned)blocks, 256, 0, s>>>(n, static_cast<float2*>(a), static_cast<float2 const*>(b),
                                                           (float)scale);
    else
        k_pointwise<double><<<(unsigned)blocks, 256, 0, s>>>(n, static_cast<double2*>(a),
                                                             static_cast<double2 const*>(b), scale);
    check_cuda(cudaPeekAtLastError(), "pointwise product launch");
}

} // namespace gbfft
