/*
 * Location layer of heFFTe's tag::gpu on libheffte_gb300: a drop-in
 * replacement for the reference's src/heffte_backend_cuda.cu.  Each function
 * keeps the reference signature (include/heffte_backend_cuda.h:67-174) and
 * forwards to the C ABI of include/heffte_gb300.h; a non-zero status is
 * rethrown as std::runtime_error("<call> failed with message: <text>"), the
 * reference's check_error convention (include/heffte_backend_cuda.h:49-60).
 *
 * Compile it in place of src/heffte_backend_cuda.cu in a heFFTe build with
 * Heffte_ENABLE_CUDA, together with include/heffte_backend_gb300.h, and link
 * libheffte_gb300.so.
 */
#include "heffte.h"
#include "heffte_backend_gb300.h"

namespace heffte {

namespace gpu {

void device_set(int active_device){
    if (active_device < 0 or active_device > device_count())
        throw std::runtime_error("device_set() called with invalid cuda device id");
    cuda::check_error(cudaSetDevice(active_device), "cudaSetDevice()");
}

void synchronize_default_stream(){
    cuda::check_error(cudaStreamSynchronize(nullptr), "device sync");
}

int device_count(){
    int count = 0;
    cuda::check_error(cudaGetDeviceCount(&count), "cudaGetDeviceCount()");
    return count;
}

}

namespace cuda {

namespace {
template<typename T> struct code;
template<> struct code<float>{ static constexpr int value = HEFFTE_GB300_FLOAT; };
template<> struct code<double>{ static constexpr int value = HEFFTE_GB300_DOUBLE; };
template<> struct code<std::complex<float>>{ static constexpr int value = HEFFTE_GB300_CFLOAT; };
template<> struct code<std::complex<double>>{ static constexpr int value = HEFFTE_GB300_CDOUBLE; };
template<typename P> constexpr int prec(){ return std::is_same<P, float>::value ? 0 : 1; }
}

template<typename precision_type, typename index>
void convert(cudaStream_t stream, index num_entries, precision_type const source[], std::complex<precision_type> destination[]){
    gb300::check(heffte_gb300_convert(stream, prec<precision_type>(), num_entries, source, destination, 1), "convert()");
}
template<typename precision_type, typename index>
void convert(cudaStream_t stream, index num_entries, std::complex<precision_type> const source[], precision_type destination[]){
    gb300::check(heffte_gb300_convert(stream, prec<precision_type>(), num_entries, source, destination, 0), "convert()");
}

template<typename scalar_type, typename index>
void direct_pack(cudaStream_t stream, index nfast, index nmid, index nslow, index line_stride, index plane_stride,
                 scalar_type const source[], scalar_type destination[]){
    gb300::check(heffte_gb300_direct_pack(stream, code<scalar_type>::value, nfast, nmid, nslow, line_stride, plane_stride,
                                          source, destination), "direct_pack()");
}

template<typename scalar_type, typename index>
void direct_unpack(cudaStream_t stream, index nfast, index nmid, index nslow, index line_stride, index plane_stride,
                   scalar_type const source[], scalar_type destination[]){
    gb300::check(heffte_gb300_direct_unpack(stream, code<scalar_type>::value, nfast, nmid, nslow, line_stride, plane_stride,
                                            source, destination), "direct_unpack()");
}

template<typename scalar_type, typename index>
void transpose_unpack(cudaStream_t stream, index nfast, index nmid, index nslow, index line_stride, index plane_stride,
                      index buff_line_stride, index buff_plane_stride, int map0, int map1, int map2,
                      scalar_type const source[], scalar_type destination[]){
    gb300::check(heffte_gb300_transpose_unpack(stream, code<scalar_type>::value, nfast, nmid, nslow, line_stride,
                                               plane_stride, buff_line_stride, buff_plane_stride, map0, map1, map2,
                                               source, destination), "transpose_unpack()");
}

template<typename scalar_type, typename index>
void scale_data(cudaStream_t stream, index num_entries, scalar_type *data, double scale_factor){
    gb300::check(heffte_gb300_scale_data(stream, prec<scalar_type>(), num_entries, data, scale_factor), "scale_data()");
}

#define gb300_instantiate_convert(precision, index) \
    template void convert<precision, index>(cudaStream_t, index, precision const[], std::complex<precision>[]); \
    template void convert<precision, index>(cudaStream_t, index, std::complex<precision> const[], precision[]);
gb300_instantiate_convert(float, int)
gb300_instantiate_convert(double, int)
gb300_instantiate_convert(float, long long)
gb300_instantiate_convert(double, long long)

#define gb300_instantiate_pack(T, index) \
    template void direct_pack<T, index>(cudaStream_t, index, index, index, index, index, T const[], T[]); \
    template void direct_unpack<T, index>(cudaStream_t, index, index, index, index, index, T const[], T[]); \
    template void transpose_unpack<T, index>(cudaStream_t, index, index, index, index, index, index, index, \
                                             int, int, int, T const[], T[]);
gb300_instantiate_pack(float, int)
gb300_instantiate_pack(double, int)
gb300_instantiate_pack(std::complex<float>, int)
gb300_instantiate_pack(std::complex<double>, int)
gb300_instantiate_pack(float, long long)
gb300_instantiate_pack(double, long long)
gb300_instantiate_pack(std::complex<float>, long long)
gb300_instantiate_pack(std::complex<double>, long long)

template void scale_data<float, int>(cudaStream_t, int, float*, double);
template void scale_data<double, int>(cudaStream_t, int, double*, double);
template void scale_data<float, long long>(cudaStream_t, long long, float*, double);
template void scale_data<double, long long>(cudaStream_t, long long, double*, double);

// pre/post processors of the extended-signal method, one line per call as the
// reference declares them (the batched ABI call with lines = 1)
namespace {
template<typename P>
void prepost(cudaStream_t s, int kind, int step, int length, void const *in, void *out){
    gb300::check(heffte_gb300_r2r_prepost(s, prec<P>(), kind, step, length, 1, 0, 0, in, out), "r2r pre/post");
}
}
#define gb300_define_prepost(NAME, KIND) \
template<typename precision> void NAME::pre_forward(cudaStream_t s, int length, precision const input[], precision fft_signal[]){ \
    prepost<precision>(s, KIND, 0, length, input, fft_signal); } \
template<typename precision> void NAME::post_forward(cudaStream_t s, int length, std::complex<precision> const fft_result[], precision result[]){ \
    prepost<precision>(s, KIND, 1, length, fft_result, result); } \
template<typename precision> void NAME::pre_backward(cudaStream_t s, int length, precision const input[], std::complex<precision> fft_signal[]){ \
    prepost<precision>(s, KIND, 2, length, input, fft_signal); } \
template<typename precision> void NAME::post_backward(cudaStream_t s, int length, precision const fft_result[], precision result[]){ \
    prepost<precision>(s, KIND, 3, length, fft_result, result); } \
template void NAME::pre_forward<float>(cudaStream_t, int, float const[], float[]); \
template void NAME::post_forward<float>(cudaStream_t, int, std::complex<float> const[], float[]); \
template void NAME::pre_backward<float>(cudaStream_t, int, float const[], std::complex<float>[]); \
template void NAME::post_backward<float>(cudaStream_t, int, float const[], float[]); \
template void NAME::pre_forward<double>(cudaStream_t, int, double const[], double[]); \
template void NAME::post_forward<double>(cudaStream_t, int, std::complex<double> const[], double[]); \
template void NAME::pre_backward<double>(cudaStream_t, int, double const[], std::complex<double>[]); \
template void NAME::post_backward<double>(cudaStream_t, int, double const[], double[]);

gb300_define_prepost(cos_pre_pos_processor, 0)
gb300_define_prepost(sin_pre_pos_processor, 1)
gb300_define_prepost(cos1_pre_pos_processor, 2)

} // namespace cuda

} // namespace heffte
