// Host C++ mirror of heFFTe's single-rank fft3d machinery for the GB300
// backend: box geometry, batched executors and the 3-D plan.
#pragma once
#include "gbfft_internal.h"
#include <array>

namespace gbfft {

// box3d (include/heffte_geometry.h:67-133): inclusive low/high, order o0 fastest.
struct Box3 {
    std::array<long long, 3> lo{0, 0, 0}, hi{-1, -1, -1}, size{0, 0, 0};
    std::array<int, 3> order{0, 1, 2};
    long long pitch0 = 0;   // padded extent of the fastest dimension order[0] (0: dense)
    Box3() = default;
    Box3(std::array<long long, 3> l, std::array<long long, 3> h, std::array<int, 3> o) : lo(l), hi(h), order(o){
        for (int i = 0; i < 3; i++) size[i] = hi[i] - lo[i] + 1;
    }
    bool empty() const { return size[0] <= 0 || size[1] <= 0 || size[2] <= 0; }
    long long count() const { return empty() ? 0 : size[0] * size[1] * size[2]; }
    long long p0() const { return pitch0 > 0 ? pitch0 : size[order[0]]; }
    // elements of the array holding the box (with the padding)
    long long alloc_count() const { return empty() ? 0 : p0() * size[order[1]] * size[order[2]]; }
    long long osize(int d) const { return size[order[d]]; }
    int find_order(int dir) const { return (dir == order[0]) ? 0 : ((dir == order[1]) ? 1 : 2); }
    // box3d::r2c (heffte_geometry.h:85-93)
    Box3 r2c(int dim) const {
        Box3 b = *this;
        b.hi[dim] = lo[dim] + size[dim] / 2;
        b.size[dim] = b.hi[dim] - b.lo[dim] + 1;
        b.pitch0 = 0;
        return b;
    }
    Box3 with_order(std::array<int, 3> o) const { Box3 b = *this; b.order = o; b.pitch0 = 0; return b; }
    std::array<long long, 3> strides() const {
        std::array<long long, 3> s{};
        s[order[0]] = 1;
        s[order[1]] = p0();
        s[order[2]] = p0() * size[order[1]];
        return s;
    }
};

bool valid_order(std::array<int, 3> const &o);

// Layout of the batch of 1-D transforms along `dim` of `box` (the other two
// dimensions enumerate the batch; the faster one of the *reference* order
// varies fastest in g).
Layout pass_layout(Box3 const &box, int dim, std::array<int, 3> const &ref_order);

enum ExecKind { EX_C2C = 0, EX_R2C = 1, EX_COS = 2, EX_SIN = 3, EX_COS1 = 4 };

// One executor: the role of cufft_executor / cufft_executor_r2c /
// real2real_executor (include/heffte_backend_cuda.h:436-751,
// include/heffte_r2r_executor.h:191-278): a batch of 1-D transforms along
// each listed dimension of one box, in place for c2c/r2r, real->complex for r2c.
struct Executor {
    int kind = EX_C2C;
    Box3 box;
    std::vector<int> dims;
    std::vector<std::shared_ptr<Fft1D>> ffts;
    long long scratch_elems = 0;          // complex elements the composite lengths need (0: none)
    mutable void *cached = nullptr;       // used when the caller passes no workspace
    mutable size_t cached_bytes = 0;
    mutable std::mutex cache_mu;
    ~Executor();
    long long box_size() const { return box.count(); }
    long long complex_size() const { return (kind == EX_R2C) ? box.r2c(dims[0]).count() : box.count(); }
    // in elements of the executor's data type: complex for c2c / r2c, real for r2r
    long long workspace_size() const { return (kind == EX_C2C || kind == EX_R2C) ? scratch_elems : 2 * scratch_elems; }
    // work: workspace_size() elements, or null (the executor then keeps a buffer of its own)
    void forward(cudaStream_t s, int prec, void const *in, void *out, void *work = nullptr, double scale = 1.0) const;
    void backward(cudaStream_t s, int prec, void const *in, void *out, void *work = nullptr, double scale = 1.0) const;
private:
    LaunchCfg config(int prec, void *work) const;
};
std::unique_ptr<Executor> make_executor(int kind, Box3 const &box, std::vector<int> const &dims);

// plan_options (include/heffte_plan_logic.h:131-176) fields that apply on one rank.
struct Options {
    bool use_reorder = false;
    int algorithm = 0;
    bool use_pencils = true;
    bool use_gpu_aware = true;
};

enum PlanKind { PK_C2C = 0, PK_R2C = 1, PK_COS = 2, PK_SIN = 3, PK_COS1 = 4 };

// Tuning knobs of a plan (the choices the learned selector makes): kernel
// family (0 pipelined where it applies, 1 generic only), tile of the generic
// kernels (automatic / tile_div), radix order (0 default, 1 ascending); and
// the precision form of the complex<float> passes (tensor_cores = 1: radix-16
// stages as split-BF16 DFT contractions on the tensor cores); whether
// convolve may fuse its middle pass (conv_fused).
struct Knobs {
    int variant = 0;
    int tile_div = 1;
    int radix_policy = 0;
    int tensor_cores = 0;
    int conv_fused = 1;
};
std::shared_ptr<Fft1D> fft_for(int N, int radix_policy);

// One operation of a compiled plan.
struct Op {
    enum Type { FFT, RESHAPE, COPY } type = FFT;
    int kind = 0;          // Kind of kernel for FFT ops (K_*), unused otherwise
    int dim = 0;
    int src = 0, dst = 0;  // buffer ids: 0 input, 1 output, 2 work A, 3 work B
    Box3 sbox, dbox;       // source / destination boxes (sizes + order)
    std::array<int, 3> ref_order{0, 1, 2};
    bool last = false;     // receives the scale factor
    std::shared_ptr<Fft1D> fft;
};

// fft3d / fft3d_r2c / rtransform on a single rank (MPI_COMM_SELF).
struct Plan3D {
    int kind = PK_C2C;
    Box3 inbox, outbox;    // outbox = inbox.r2c(r2c_dir) geometry for PK_R2C
    int r2c_dir = 0;
    Options opts;
    cudaStream_t stream = nullptr;
    std::vector<Op> fwd, fwd_alias, bwd;
    long long work_elems = 0;     // workspace in output-type elements (complex for c2c/r2c)
    long long work_buf_elems = 0; // elements of one of the (up to two) workspace buffers
    long long scratch_elems = 0;  // complex elements of scratch for composite lengths (four-step, Bluestein)
    long long scratch_offset = 0; // where that scratch starts in the workspace (workspace elements)
    double scale_factor = 1.0;    // "full" factor
    void *cached_work = nullptr;  // lazily allocated when the caller passes no workspace
    size_t cached_bytes = 0;
    void *conv_cache = nullptr;   // the same for convolve()
    size_t conv_cache_bytes = 0;
    Knobs knobs;
    ~Plan3D();

    long long size_inbox() const { return inbox.count(); }
    long long size_outbox() const { return outbox.count(); }
    long long size_workspace() const { return work_elems; }
    double get_scale(int scaling) const;
    void execute(bool forward, int prec, int batch, void const *in, void *out, void *work, int scaling);
    // Circular convolution through the plan's transforms (benchmarks/convolution.cpp):
    // out = backward(forward(x) .* forward(y)) with the backward scaling;
    // y null or equal to x: self-convolution.  Workspace in complex elements:
    // the plan's own, then two spectrum boxes.
    long long convolve_workspace() const;
    void convolve(int prec, void const *x, void const *y, void *out, void *work, int scaling);
    // the box the spectra of the fused route live in
    Box3 conv_box() const;
    // the fused route of convolve; false when it does not apply
    bool convolve_fused(int prec, void const *x, void const *y, void *out, void *w1, void *w2, double scale);
    // the dimension the fused route transforms in its fused pass (-1: unfused);
    // only the alignment of the spectrum buffers xb and yb (null: self-
    // convolution) is looked at
    int convolve_fused_dim(int prec, void *xb, void const *yb) const;
};

// reshape3d_alltoallv of one rank of a group (src/heffte_reshape3d.cpp:365-496):
// the overlaps this rank sends and receives, packed / unpacked on the device;
// the exchange between the buffers is the caller's (gbfft_reshape.cu).
struct Reshape {
    struct Chunk {
        int rank = 0;                      // the other rank
        long long box_offset = 0;          // first element of the overlap in this rank's box
        std::array<long long, 3> size{};   // fast, mid, slow extents of the overlap (this rank's order)
        long long line_stride = 0, plane_stride = 0;      // of this rank's box
        std::array<int, 3> map{0, 1, 2};   // received chunks: the sender's fast / mid / slow -> this rank's
        long long buff_line_stride = 0, buff_plane_stride = 0;   // of the received chunk
    };
    int nranks = 1, me = 0;
    Box3 inbox, outbox;
    std::vector<Chunk> send, recv;
    // elements per rank (rank order) of the send / receive buffers
    std::vector<long long> send_counts, send_displs, recv_counts, recv_displs;
    long long send_total = 0, recv_total = 0;
    void pack(cudaStream_t s, int dtype, void const *input, void *send_buffer) const;
    void unpack(cudaStream_t s, int dtype, void const *recv_buffer, void *output) const;
};
std::unique_ptr<Reshape> make_reshape(int nranks, int me, std::vector<Box3> const &inboxes,
                                      std::vector<Box3> const &outboxes);

std::unique_ptr<Plan3D> make_plan(int kind, Box3 const &inbox, Box3 const &outbox, int r2c_dir, Options const &o,
                                  cudaStream_t stream, Knobs const &knobs = Knobs{});

} // namespace gbfft
