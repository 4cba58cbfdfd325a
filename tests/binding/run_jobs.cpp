// Runs heFFTe's own fft3d / fft3d_r2c / rtransform classes with the GB300
// backend tags (include/heffte_backend_gb300.h) on the GPU, through the
// reference's compute_transform (src/heffte_compute_transform.cpp) and
// reshape3d_transpose, for a list of jobs written by
// tests/test_reference_binding.py.
//
// Job line: kind prec reorder n0 n1 n2 io0 io1 io2 oo0 oo1 oo2 r2c_dir api prefix
//   kind : c2c | real (fft3d with real input / output: the executor's real
//          overloads) | r2c | cos | sin | cos1
//   api  : 0 pointer calls with a caller workspace, 1 pointer calls without
//          one (the plan allocates per call), 2 the vector API
//          (gpu::transfer::load, forward(container); not for kind real,
//          whose vector backward is backward_real), 3 in place (c2c), 4 a
//          user stream given to the constructor
// Reads <prefix>_in.bin (forward input) and <prefix>_fin.bin (backward
// input), writes <prefix>_fwd.bin = forward(in, scale::none) and
// <prefix>_bwd.bin = backward(fin, scale::full).
#include "heffte.h"
#include "heffte_backend_gb300.h"
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace heffte;

namespace {

void cuda_ok(cudaError_t e, char const *what){
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template<typename T>
std::vector<T> read_file(std::string const &path, size_t n){
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    if (!f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T))) throw std::runtime_error("cannot read " + path);
    return v;
}

template<typename T>
void write_file(std::string const &path, std::vector<T> const &v){
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<char const*>(v.data()), v.size() * sizeof(T));
}

template<typename T>
T *dev_copy(std::vector<T> const &h){
    T *d = nullptr;
    cuda_ok(cudaMalloc(reinterpret_cast<void**>(&d), std::max<size_t>(h.size(), 1) * sizeof(T)), "cudaMalloc");
    cuda_ok(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "H2D");
    return d;
}

template<typename T>
std::vector<T> host_copy(T const *d, size_t n){
    std::vector<T> h(n);
    cuda_ok(cudaDeviceSynchronize(), "sync");
    cuda_ok(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
    return h;
}

struct Job {
    std::string kind, prefix;
    int prec = 0, reorder = 0, r2c_dir = 0, api = 0;
    int n[3] = {0, 0, 0}, io[3] = {0, 1, 2}, oo[3] = {0, 1, 2};
};

// fwd_in / fwd_out: element types of forward's input and output (backward
// swaps them); the workspace has forward's output type.
template<typename fwd_in, typename fwd_out, typename plan_t>
void run(plan_t &plan, Job const &j){
    size_t nin = plan.size_inbox(), nout = plan.size_outbox(), nw = plan.size_workspace();
    auto hin = read_file<fwd_in>(j.prefix + "_in.bin", nin);
    auto hfin = read_file<fwd_out>(j.prefix + "_fin.bin", nout);
    if (j.api == 2){
        auto x = gpu::transfer::load(hin.data(), nin);
        auto y = plan.forward(x);
        auto f = gpu::transfer::load(hfin.data(), nout);
        auto z = plan.backward(f, scale::full);
        write_file(j.prefix + "_fwd.bin", gpu::transfer::unload(y.data(), y.size()));
        write_file(j.prefix + "_bwd.bin", gpu::transfer::unload(z.data(), z.size()));
        return;
    }
    fwd_in *din = dev_copy(hin);
    fwd_out *dfin = dev_copy(hfin);
    fwd_out *dout = nullptr, *dw = nullptr;
    fwd_in *dback = nullptr;
    cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dout), std::max<size_t>(nout, 1) * sizeof(fwd_out)), "cudaMalloc");
    cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dback), std::max<size_t>(nin, 1) * sizeof(fwd_in)), "cudaMalloc");
    cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dw), std::max<size_t>(nw, 1) * sizeof(fwd_out)), "cudaMalloc");
    if (j.api == 3){
        // in place: the output buffer holds the input (c2c only: same type and size)
        cuda_ok(cudaMemcpy(dout, din, nin * sizeof(fwd_in), cudaMemcpyDeviceToDevice), "D2D");
        plan.forward(reinterpret_cast<fwd_in*>(dout), dout, dw, scale::none);
        cuda_ok(cudaMemcpy(dback, dfin, nout * sizeof(fwd_out), cudaMemcpyDeviceToDevice), "D2D");
        plan.backward(reinterpret_cast<fwd_out*>(dback), dback, reinterpret_cast<fwd_out*>(dw), scale::full);
    } else if (j.api == 1){
        plan.forward(din, dout, scale::none);
        plan.backward(dfin, dback, scale::full);
    } else {
        plan.forward(din, dout, dw, scale::none);
        plan.backward(dfin, dback, dw, scale::full);
    }
    write_file(j.prefix + "_fwd.bin", host_copy(dout, nout));
    write_file(j.prefix + "_bwd.bin", host_copy(dback, nin));
    cudaFree(din); cudaFree(dfin); cudaFree(dout); cudaFree(dback); cudaFree(dw);
}

template<typename real>
void dispatch(Job const &j, cudaStream_t stream){
    using cplx = std::complex<real>;
    box3d<> inbox({0, 0, 0}, {j.n[0] - 1, j.n[1] - 1, j.n[2] - 1}, {j.io[0], j.io[1], j.io[2]});
    plan_options opts = default_options<backend::gb300>();
    opts.use_reorder = (j.reorder != 0);
    if (j.kind == "c2c" || j.kind == "real"){
        box3d<> outbox({0, 0, 0}, {j.n[0] - 1, j.n[1] - 1, j.n[2] - 1}, {j.oo[0], j.oo[1], j.oo[2]});
        fft3d<backend::gb300> plan(stream, inbox, outbox, MPI_COMM_SELF, opts);
        if (j.kind == "c2c") run<cplx, cplx>(plan, j);
        else run<real, cplx>(plan, j);
    } else if (j.kind == "r2c"){
        box3d<> half = inbox.r2c(j.r2c_dir);
        box3d<> outbox(half.low, half.high, {j.oo[0], j.oo[1], j.oo[2]});
        fft3d_r2c<backend::gb300> plan(stream, inbox, outbox, j.r2c_dir, MPI_COMM_SELF, opts);
        run<real, cplx>(plan, j);
    } else {
        box3d<> outbox({0, 0, 0}, {j.n[0] - 1, j.n[1] - 1, j.n[2] - 1}, {j.oo[0], j.oo[1], j.oo[2]});
        if (j.kind == "cos"){
            rtransform<backend::gb300_cos> plan(stream, inbox, outbox, MPI_COMM_SELF, opts);
            run<real, real>(plan, j);
        } else if (j.kind == "sin"){
            rtransform<backend::gb300_sin> plan(stream, inbox, outbox, MPI_COMM_SELF, opts);
            run<real, real>(plan, j);
        } else {
            rtransform<backend::gb300_cos1> plan(stream, inbox, outbox, MPI_COMM_SELF, opts);
            run<real, real>(plan, j);
        }
    }
}

} // namespace

int main(int argc, char **argv){
    if (argc != 2){
        std::fprintf(stderr, "usage: %s <job file>\n", argv[0]);
        return 2;
    }
    std::ifstream jobs(argv[1]);
    std::string line;
    int done = 0;
    try {
        while (std::getline(jobs, line)){
            if (line.empty()) continue;
            std::istringstream is(line);
            Job j;
            is >> j.kind >> j.prec >> j.reorder >> j.n[0] >> j.n[1] >> j.n[2] >> j.io[0] >> j.io[1] >> j.io[2]
               >> j.oo[0] >> j.oo[1] >> j.oo[2] >> j.r2c_dir >> j.api >> j.prefix;
            cudaStream_t stream = nullptr;
            if (j.api == 4) cuda_ok(cudaStreamCreate(&stream), "cudaStreamCreate");
            if (j.prec == 0) dispatch<float>(j, stream); else dispatch<double>(j, stream);
            if (stream){
                cuda_ok(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
                cuda_ok(cudaStreamDestroy(stream), "cudaStreamDestroy");
            }
            done++;
        }
    } catch (std::exception const &e){
        std::fprintf(stderr, "job %d (%s) failed: %s\n", done, line.c_str(), e.what());
        return 1;
    }
    std::printf("%d jobs\n", done);
    return 0;
}
