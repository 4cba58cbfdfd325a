/*
 * heffte_backend_gb300.h - the reference-side binding: heFFTe backend tags
 * gb300 / gb300_cos / gb300_sin / gb300_cos1 whose executors call
 * libheffte_gb300 through the C ABI of heffte_gb300.h.
 *
 * Include after heffte.h in a heFFTe build configured with Heffte_ENABLE_CUDA
 * (the tags reuse tag::gpu: device_vector, data_manipulator<tag::gpu>,
 * device_instance<tag::gpu> of include/heffte_backend_cuda.h).  With it,
 *     heffte::fft3d<heffte::backend::gb300> fft(inbox, outbox, MPI_COMM_SELF);
 * runs on the GB300 kernels of this repository.  The traits mirror those of
 * the cuFFT tags (include/heffte_backend_cuda.h:183-326, :759-877).
 */
#ifndef HEFFTE_BACKEND_GB300_H
#define HEFFTE_BACKEND_GB300_H

#include <stdexcept>
#include <string>
#include "heffte_gb300.h"

namespace heffte {

namespace backend {
    //! \brief Type-tag for the GB300 c2c / r2c backend.
    struct gb300{};
    //! \brief Type-tag for the GB300 DCT-II/III (cuFFT-cos conventions).
    struct gb300_cos{};
    //! \brief Type-tag for the GB300 DST-II/III (cuFFT-sin conventions).
    struct gb300_sin{};
    //! \brief Type-tag for the GB300 DCT-I (cuFFT-cos1 conventions).
    struct gb300_cos1{};

    template<> struct is_enabled<gb300> : std::true_type{};
    template<> struct is_enabled<gb300_cos> : std::true_type{};
    template<> struct is_enabled<gb300_sin> : std::true_type{};
    template<> struct is_enabled<gb300_cos1> : std::true_type{};

    template<> struct buffer_traits<gb300>{
        using location = tag::gpu;
        template<typename T> using container = heffte::gpu::device_vector<T, data_manipulator<tag::gpu>>;
    };
    template<> struct buffer_traits<gb300_cos>{
        using location = tag::gpu;
        template<typename T> using container = heffte::gpu::device_vector<T, data_manipulator<tag::gpu>>;
    };
    template<> struct buffer_traits<gb300_sin>{
        using location = tag::gpu;
        template<typename T> using container = heffte::gpu::device_vector<T, data_manipulator<tag::gpu>>;
    };
    template<> struct buffer_traits<gb300_cos1>{
        using location = tag::gpu;
        template<typename T> using container = heffte::gpu::device_vector<T, data_manipulator<tag::gpu>>;
    };

    template<> struct uses_fft_types<gb300_cos> : std::false_type{};
    template<> struct uses_fft_types<gb300_sin> : std::false_type{};
    template<> struct uses_fft_types<gb300_cos1> : std::false_type{};

    template<> inline std::string name<gb300>(){ return "gb300"; }
    template<> inline std::string name<gb300_cos>(){ return "gb300-cos-type-II"; }
    template<> inline std::string name<gb300_sin>(){ return "gb300-sin-type-II"; }
    template<> inline std::string name<gb300_cos1>(){ return "gb300-cos-type-I"; }
}

namespace gb300 {
    //! \brief Throws the reference's runtime_error text for a non-zero status.
    inline void check(int status, char const *what){
        if (status != HEFFTE_GB300_SUCCESS)
            throw std::runtime_error(std::string(what) + " failed with message: " + heffte_gb300_last_error());
    }

    //! \brief Owns one heffte_gb300_executor over a box and a set of dimensions.
    class executor_handle{
    public:
        template<typename index>
        executor_handle(int kind, box3d<index> const box, std::initializer_list<int> dims){
            long long lo[3] = {box.low[0], box.low[1], box.low[2]};
            long long hi[3] = {box.high[0], box.high[1], box.high[2]};
            int order[3] = {box.order[0], box.order[1], box.order[2]};
            int d[3] = {0, 0, 0}, n = 0;
            for (int v : dims) d[n++] = v;
            check(heffte_gb300_executor_create(kind, lo, hi, order, n, d, &handle), "heffte_gb300_executor_create()");
        }
        ~executor_handle(){ if (handle) heffte_gb300_executor_destroy(handle); }
        executor_handle(executor_handle const&) = delete;
        executor_handle& operator =(executor_handle const&) = delete;
        void forward(cudaStream_t s, int prec, void const *in, void *out, void *work) const{
            check(heffte_gb300_executor_forward(handle, s, prec, in, out, work), "heffte_gb300_executor_forward()");
        }
        void backward(cudaStream_t s, int prec, void const *in, void *out, void *work) const{
            check(heffte_gb300_executor_backward(handle, s, prec, in, out, work), "heffte_gb300_executor_backward()");
        }
        long long box_size() const{ return heffte_gb300_executor_box_size(handle); }
        long long complex_size() const{ return heffte_gb300_executor_complex_size(handle); }
        //! \brief Elements of the executor's data type the composite lengths need (executor_base::workspace_size).
        size_t workspace_size() const{ return static_cast<size_t>(heffte_gb300_executor_workspace_size(handle)); }
    private:
        heffte_gb300_executor handle = nullptr;
    };
}

/*!
 * \brief c2c executor: the cufft_executor role (include/heffte_backend_cuda.h:436-572)
 * with the 1-D, 2-D and 3-D constructors the fft3d setup may request.
 */
class gb300_executor : public executor_base{
public:
    using executor_base::forward;
    using executor_base::backward;
    using executor_base::complex_size;
    template<typename index>
    gb300_executor(cudaStream_t s, box3d<index> const box, int dimension)
        : stream(s), total(box.count()), exec(HEFFTE_GB300_C2C, box, {dimension}){}
    template<typename index>
    gb300_executor(cudaStream_t s, box3d<index> const box, int dir1, int dir2)
        : stream(s), total(box.count()), exec(HEFFTE_GB300_C2C, box, {dir1, dir2}){}
    template<typename index>
    gb300_executor(cudaStream_t s, box3d<index> const box)
        : stream(s), total(box.count()), exec(HEFFTE_GB300_C2C, box, {0, 1, 2}){}

    void forward(std::complex<float> data[], std::complex<float> *w) const override{ exec.forward(stream, 0, data, data, w); }
    void backward(std::complex<float> data[], std::complex<float> *w) const override{ exec.backward(stream, 0, data, data, w); }
    void forward(std::complex<double> data[], std::complex<double> *w) const override{ exec.forward(stream, 1, data, data, w); }
    void backward(std::complex<double> data[], std::complex<double> *w) const override{ exec.backward(stream, 1, data, data, w); }
    // real input through the complex transform, as cufft_executor (:527-545)
    void forward(float const indata[], std::complex<float> outdata[], std::complex<float> *w) const override{
        gb300::check(heffte_gb300_convert(stream, 0, total, indata, outdata, 1), "heffte_gb300_convert()");
        forward(outdata, w);
    }
    void backward(std::complex<float> indata[], float outdata[], std::complex<float> *w) const override{
        backward(indata, w);
        gb300::check(heffte_gb300_convert(stream, 0, total, indata, outdata, 0), "heffte_gb300_convert()");
    }
    void forward(double const indata[], std::complex<double> outdata[], std::complex<double> *w) const override{
        gb300::check(heffte_gb300_convert(stream, 1, total, indata, outdata, 1), "heffte_gb300_convert()");
        forward(outdata, w);
    }
    void backward(std::complex<double> indata[], double outdata[], std::complex<double> *w) const override{
        backward(indata, w);
        gb300::check(heffte_gb300_convert(stream, 1, total, indata, outdata, 0), "heffte_gb300_convert()");
    }
    int box_size() const override{ return static_cast<int>(total); }
    size_t workspace_size() const override{ return exec.workspace_size(); }
private:
    cudaStream_t stream;
    long long total;
    gb300::executor_handle exec;
};

/*!
 * \brief r2c / c2r executor: the cufft_executor_r2c role (include/heffte_backend_cuda.h:631-751).
 * Real pointers need only 4-byte alignment and the input of backward() is not modified.
 */
class gb300_executor_r2c : public executor_base{
public:
    using executor_base::forward;
    using executor_base::backward;
    template<typename index>
    gb300_executor_r2c(cudaStream_t s, box3d<index> const box, int dimension)
        : stream(s), exec(HEFFTE_GB300_R2C, box, {dimension}){}
    void forward(float const indata[], std::complex<float> outdata[], std::complex<float> *w) const override{
        exec.forward(stream, 0, indata, outdata, w);
    }
    void backward(std::complex<float> indata[], float outdata[], std::complex<float> *w) const override{
        exec.backward(stream, 0, indata, outdata, w);
    }
    void forward(double const indata[], std::complex<double> outdata[], std::complex<double> *w) const override{
        exec.forward(stream, 1, indata, outdata, w);
    }
    void backward(std::complex<double> indata[], double outdata[], std::complex<double> *w) const override{
        exec.backward(stream, 1, indata, outdata, w);
    }
    int box_size() const override{ return static_cast<int>(exec.box_size()); }
    int complex_size() const override{ return static_cast<int>(exec.complex_size()); }
    size_t workspace_size() const override{ return exec.workspace_size(); }
private:
    cudaStream_t stream;
    gb300::executor_handle exec;
};

/*!
 * \brief Real-to-real executor: the real2real_executor<cufft, cos|sin> role
 * (include/heffte_r2r_executor.h:191-278).  Unlike the reference it accepts
 * any dimension and the 2-D / 3-D constructors, which fft3d's setup requests
 * for tags it does not list (include/heffte_common.h:714-755).
 */
template<int kind>
class gb300_r2r_executor : public executor_base{
public:
    using executor_base::forward;
    using executor_base::backward;
    template<typename index>
    gb300_r2r_executor(cudaStream_t s, box3d<index> const box, int dimension)
        : stream(s), exec(kind, box, {dimension}){}
    template<typename index>
    gb300_r2r_executor(cudaStream_t s, box3d<index> const box, int dir1, int dir2)
        : stream(s), exec(kind, box, {dir1, dir2}){}
    template<typename index>
    gb300_r2r_executor(cudaStream_t s, box3d<index> const box)
        : stream(s), exec(kind, box, {0, 1, 2}){}
    void forward(float data[], float *w) const override{ exec.forward(stream, 0, data, data, w); }
    void forward(double data[], double *w) const override{ exec.forward(stream, 1, data, data, w); }
    void backward(float data[], float *w) const override{ exec.backward(stream, 0, data, data, w); }
    void backward(double data[], double *w) const override{ exec.backward(stream, 1, data, data, w); }
    int box_size() const override{ return static_cast<int>(exec.box_size()); }
    size_t workspace_size() const override{ return exec.workspace_size(); }
private:
    cudaStream_t stream;
    gb300::executor_handle exec;
};

template<> struct one_dim_backend<backend::gb300>{
    using executor = gb300_executor;
    using executor_r2c = gb300_executor_r2c;
};
template<> struct one_dim_backend<backend::gb300_cos>{
    using executor = gb300_r2r_executor<HEFFTE_GB300_COS>;
    using executor_r2c = void;
};
template<> struct one_dim_backend<backend::gb300_sin>{
    using executor = gb300_r2r_executor<HEFFTE_GB300_SIN>;
    using executor_r2c = void;
};
template<> struct one_dim_backend<backend::gb300_cos1>{
    using executor = gb300_r2r_executor<HEFFTE_GB300_COS1>;
    using executor_r2c = void;
};

// No 3-D executor for the gb300 tags: fft3d::setup puts a 3-D executor in the
// first of its three executor slots (include/heffte_fft3d.h:607-608), so the
// backward executor list begins with a null slot, and compute_transform's
// branch for a single active reshape copies the input into its temporary
// buffer only when that first slot is set (src/heffte_compute_transform.cpp:
// 73-80).  Backward transforms with use_reorder = false and different input
// and output orders (the last reshape alone active) then transform an
// uninitialised buffer; the cuFFT tags, for which has_executor3d is also
// true, take the same branch.  The 2-D + 1-D executors fft3d::setup picks
// instead run the same passes and keep the first backward slot set.
template<> constexpr bool has_executor3d<backend::gb300>(){ return false; }
template<> constexpr bool has_executor3d<backend::gb300_cos>(){ return false; }
template<> constexpr bool has_executor3d<backend::gb300_sin>(){ return false; }
template<> constexpr bool has_executor3d<backend::gb300_cos1>(){ return false; }

// strided executors are the fast path: no transposes by default
template<> struct default_plan_options<backend::gb300>{ static const bool use_reorder = false; };
template<> struct default_plan_options<backend::gb300_cos>{ static const bool use_reorder = false; };
template<> struct default_plan_options<backend::gb300_sin>{ static const bool use_reorder = false; };
template<> struct default_plan_options<backend::gb300_cos1>{ static const bool use_reorder = false; };

}

#endif
