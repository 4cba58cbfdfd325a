// Host-side internals shared by the translation units of libheffte_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>
#include "gbfft_common.cuh"

namespace gbfft {

enum DType { DT_FLOAT = 0, DT_DOUBLE = 1, DT_CFLOAT = 2, DT_CDOUBLE = 3 };

// Error raised inside the library; the C-ABI turns it into a status code and
// a message readable through heffte_gb300_last_error().
struct Error : std::runtime_error {
    int code;
    Error(int c, std::string const &m) : std::runtime_error(m), code(c) {}
};
enum { ST_OK = 0, ST_INVALID = 1, ST_CUDA = 2, ST_UNSUPPORTED = 3, ST_ALLOC = 4, ST_TIMEOUT = 5 };

inline void check_cuda(cudaError_t e, char const *what){
    if (e != cudaSuccess) throw Error(ST_CUDA, std::string(what) + " failed with message: " + cudaGetErrorString(e));
}

int num_sms();
int elem_size(int dtype);
// message returned by heffte_gb300_last_error() on the calling thread
void set_last_error(std::string const &msg);

// ---------------------------------------------------------------------------
// 1-D transform length: radix plan, thread count and device twiddle tables.
// ---------------------------------------------------------------------------
constexpr int kEmax = 16;
// Lengths the radix kernels take directly: up to kMaxDirectLength with prime
// factors 2, 3, 5, 7, 11, 13.  Longer lengths and other primes are composite
// (gbfft_long.cu), up to kMaxLength.
constexpr int kMaxDirectLength = 8192;
constexpr int kMaxLength = 1 << 25;
// Scratch bound of one chunk of lines of a composite length (complex elements).
constexpr long long kCompositeScratchElems = 1LL << 26;

// How a length is transformed: by the radix kernels, as N1 x N2 (four-step),
// or by Bluestein's algorithm through a power-of-two length M >= 2N - 1.
enum Algo { ALGO_DIRECT = 0, ALGO_FOURSTEP = 1, ALGO_BLUESTEIN = 2 };
// Device tables of a composite length (per precision).
enum CompositeTable { TAB_ROOTS = 0, TAB_CHIRP = 1, TAB_CHIRP_SPECTRUM = 2 };

struct Fft1D {
    int N = 0;
    Plan1D plan{};
    std::vector<int> radices;
    int algo = ALGO_DIRECT;
    std::shared_ptr<Fft1D> sub1, sub2;    // four-step: N1, N2; Bluestein: M (sub1)
    // device tables, created lazily per precision: [0] float, [1] double
    void *tw[2] = {nullptr, nullptr};     // Stockham twiddles
    void *rtw[2] = {nullptr, nullptr};    // exp(-i pi k / 2N), k < N (r2r)
    void *ctab[3][2] = {};                // composite tables (CompositeTable)
    void *tw_df = nullptr;                // Stockham twiddles as double-float pairs
    long long tw_count = 0;
    std::mutex mu;
    ~Fft1D();
    void const *twiddles(int prec, cudaStream_t s);
    void const *r2r_twiddles(int prec, cudaStream_t s);
    // the Stockham twiddles for double-float arithmetic (FP64-generated, split into float pairs)
    void const *twiddles_df(cudaStream_t s);
    // four-step roots exp(-2 pi i m / N); Bluestein chirp exp(-i pi n^2 / N)
    // and the spectrum of its conjugate on M points divided by M (FP64-generated)
    void const *composite_table(int which, int prec, cudaStream_t s);
};

// Shared registry of lengths (plans are immutable once built; tables lazily).
// `radices` empty = default radix choice.
std::shared_ptr<Fft1D> get_fft1d(int N, std::vector<int> const &radices = {});
std::vector<int> default_radices(int N);
bool supported_length(int N, int prec);
// a length the radix kernels take directly (the batch and tensor-core kernels need one)
bool direct_length(int N);
int max_length(int prec);

// Tuning knobs of one launch (chosen by the planner / autotuner).
struct LaunchCfg {
    int tpb = 0;      // transforms (or transform pairs) per CTA; 0 = automatic
    int variant = 0;  // 0 = process-wide choice, 1 = generic kernels, 2 = pipelined kernels
    int tpb_div = 1;  // divides the automatic tile of the generic kernels
    int tc = 0;       // 1: complex<float> radix-16 stages on the tensor cores (split BF16)
    void *scratch = nullptr;    // workspace of composite lengths (composite_scratch_elems)
    size_t scratch_bytes = 0;
};

// Kinds of the gather / scatter around a composite transform (gbfft_long.cu).
enum LineMode { LM_C2C = 0, LM_R2C = 1, LM_C2R = 2, LM_R2R_F = 3, LM_R2R_B = 4, LM_DCT1 = 5 };
// Complex elements of scratch a batch of G lines of a composite length needs
// (0 for direct lengths): two copies of a chunk of lines plus what
// Bluestein's inner length needs; for the paired modes a unit is two lines.
long long composite_scratch_elems(Fft1D const &f, int mode, long long G);
long long composite_extra_per_line(Fft1D const &f);
// Composite transform of `lines` contiguous lines X -> Y (X is kept; extra:
// composite_extra_per_line(f) * lines complex elements).
void composite_core(cudaStream_t s, Fft1D &f, int prec, bool fwd, void *X, void *Y, long long lines, void *extra);
// The batched transform of a composite length in the caller's layouts (N is
// the data length: the real length for r2c / c2r / r2r, the DCT-I length).
void launch_composite(cudaStream_t s, int mode, Fft1D &f, int prec, bool fwd, int sine, int N, Layout Li, Layout Lo,
                      void const *in, void *out, long long G, double scale, LaunchCfg const &cfg);

// Tensor-core (tcgen05, split-BF16) complex<float> transforms of lengths
// 16^s * {1, 2, 4, 8} in [64, 4096].
bool tc_supported(int N);
std::vector<int> tc_radices(int N);
void launch_tc_c2c(cudaStream_t s, int N, bool fwd, Layout Li, Layout Lo, void const *in, void *out, long long G,
                   double scale);

// Batched 1-D launches (in units of elements of the respective arrays).
void launch_c2c(cudaStream_t s, Fft1D &f, int prec, bool fwd, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg = {});
void launch_r2c(cudaStream_t s, Fft1D &f, int prec, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg = {});
void launch_c2r(cudaStream_t s, Fft1D &f, int prec, Layout Li, Layout Lo, void const *in, void *out,
                long long G, double scale, LaunchCfg cfg = {});
// DCT-I (REDFT00, backward 2 x REDFT00) of lines of N values; f has length 2(N-1).
void launch_dct1(cudaStream_t s, Fft1D &f, int prec, bool fwd, int N, Layout Li, Layout Lo, void const *in, void *out,
                 long long G, double scale, LaunchCfg cfg = {});
void launch_r2r(cudaStream_t s, Fft1D &f, int prec, bool fwd, bool sine, Layout Li, Layout Lo, void const *in,
                void *out, long long G, double scale, LaunchCfg cfg = {});

// Location-layer data movement.
// Validates a strided 3-D layout of n0 x n1 x n2 elements (n0 fastest, line
// stride ls, plane stride ps): strides non-negative, lines and planes that do
// not overlap, and a span that fits in 63 bits.  Returns the number of
// elements the layout spans ((n2-1) ps + (n1-1) ls + n0); throws ST_INVALID
// naming `what` otherwise.  All sizes must be positive.
long long strided_extent(long long n0, long long n1, long long n2, long long ls, long long ps, char const *what);
void launch_direct_pack(cudaStream_t s, int dtype, long long nf, long long nm, long long ns, long long ls,
                        long long ps, void const *src, void *dst, bool pack);
void launch_transpose_unpack(cudaStream_t s, int dtype, long long nf, long long nm, long long ns, long long ls,
                             long long ps, long long bls, long long bps, int m0, int m1, void const *src, void *dst);
void launch_scale(cudaStream_t s, int prec, long long n, void *data, double factor);
void launch_convert(cudaStream_t s, int prec, long long n, void const *src, void *dst, bool to_complex);
void launch_prepost(cudaStream_t s, int prec, int kind, int step, int N, long long lines, long long in_ld,
                    long long out_ld, void const *in, void *out);

// Per-precision kernel launchers (defined in gbfft_fft_f32.cu / _f64.cu).
struct KernelArgs {
    Plan1D const *plan;
    Layout Li, Lo;
    void const *in;
    void *out;
    void const *tw;
    void const *rtw;
    long long G;        // number of transforms (real transforms for the paired kernels)
    int tpb;
    int threads;
    size_t smem;
    long long blocks;
    double scale;
    int do_scale;
    int sine;
    int ndata;          // line length of the DCT-I kernel (the FFT has length 2(ndata - 1))
};
enum Kind { K_C2C_F, K_C2C_B, K_R2C, K_C2R, K_R2R_F, K_R2R_B, K_DCT1 };
void launch_kernel_f32(cudaStream_t s, int kind, bool cols, KernelArgs const &a);
void launch_kernel_f64(cudaStream_t s, int kind, bool cols, KernelArgs const &a);

// Pipelined power-of-two kernels (gbfft_pipe_f32.cu / _f64.cu); return false
// when the batch does not meet their tiling / alignment conditions.
struct PipeLaunch {
    Layout Li, Lo;
    void const *in;
    void *out;
    void const *tw;
    void const *rtw;
    long long G;
    double scale;
    int sine;
    int out_split;      // column tiles: Li's blocks merged into one, Lo's kept (output offsets by division)
    int *status;
};
// Pipelined complex transforms of any supported length (runtime radix plan,
// gbfft_pipe_rt.cuh): the parameters of one launch and its dispatcher.
struct PipeRtParams {
    Plan1D plan;
    Layout Li, Lo;
    void const *in;
    void *out;
    void const *tw;
    long long G;
    long long ntiles;
    long long tiles_per_block;   // column tiles covering one block of `count` columns
    int tpb;                     // transforms per tile
    int nbuf;                    // tile slots: 2 (the next tile copied while one is transformed) or 1
    int ct;                      // float: the kernel compiled for the plan, 1 twiddles in shared memory
                                 // (smem includes them), 2 in global memory; 0 the runtime-plan kernel
    int boxr;                    // rows per tensor-map copy (divides N)
    int tswap;
    double scale;
    int do_scale;
    int *status;
};
void launch_pipe_rt(cudaStream_t s, int prec, bool fwd, bool cols, PipeRtParams const &P, void const *tmap,
                    size_t smem, int threads);
// Float lengths with runtime-radix pipelined kernels compiled for their
// default radix plan (one instantiation unit gbfft_pipe_rt_n<N>.cu each)
#define GBFFT_RT_CT_LENGTHS(X) X(96) X(160) X(192) X(240) X(288) X(320) X(384) X(448) X(480) X(576) \
                               X(640) X(720) X(768) X(960)
// shared-memory bytes that the float kernel compiled for this plan adds to
// the tiles (its twiddle table), 0 when no compiled kernel runs it
size_t rt_ct_smem(Plan1D const &plan);
// float kernels compiled for the plan of length NC (gbfft_pipe_rt_n<NC>.cu);
// false (nothing launched) when P.plan is not that plan
template<int NC>
bool launch_pipe_rt_ct(cudaStream_t s, bool fwd, bool cols, PipeRtParams const &P, void const *tmap, size_t smem,
                       int threads);
// (explicit specializations, one per compiled length, defined in gbfft_pipe_rt_n<N>.cu)
#define GBFFT_RT_CT_DECL(n) \
    template<> bool launch_pipe_rt_ct<n>(cudaStream_t, bool, bool, PipeRtParams const &, void const *, size_t, int);
GBFFT_RT_CT_LENGTHS(GBFFT_RT_CT_DECL)
#undef GBFFT_RT_CT_DECL

// one dispatcher per precision and kind group (c2c / r2c+c2r / r2r), kind = K_*
bool launch_pipe_f32_c2c(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
bool launch_pipe_f32_r2c(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
bool launch_pipe_f32_r2r(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
bool launch_pipe_f64_c2c(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
bool launch_pipe_f64_r2c(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
bool launch_pipe_f64_r2r(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
// complex<double> c2c passes in double-float arithmetic (a.tw: twiddles_df)
bool launch_pipe_df64_c2c(cudaStream_t s, int kind, int N, bool cols, PipeLaunch const &a);
// Fused convolution pass (gbfft_conv.cuh): forward FFT of the columns of x
// (and y), pointwise product, scale, backward FFT, in place in x.
struct ConvLaunch {
    Layout L;
    void *x;
    void const *y;     // null: self-convolution (X .* X)
    void const *tw;
    long long G;
    double scale;
    int *status;
};
// dry_run: only checks that the pass can run (length, alignment, tensor maps)
bool launch_conv_f32(cudaStream_t s, int N, ConvLaunch const &a, bool dry_run);
bool launch_conv_f64(cudaStream_t s, int N, ConvLaunch const &a, bool dry_run);
bool launch_conv_pass(cudaStream_t s, Fft1D &f, int prec, Layout L, void *x, void const *y, long long G,
                      double scale, bool dry_run);
// a[i] = a[i] * b[i] * scale (b null: a[i]^2 * scale) over n complex values
void launch_pointwise(cudaStream_t s, int prec, long long n, void *a, void const *b, double scale);

// Tensor map over a batch of column transforms: x = column (8-byte words),
// then rows and blocks ordered by ascending stride (*swap = 1 when blocks
// come before rows).  Returns false if the driver rejects the geometry.
struct CUtensorMap_st;
bool encode_column_tmap(void *tmap, void const *base, int csize, long long count, long long N, long long blocks,
                        long long estride, long long bstride, int tpb, int boxr, int *swap);
// empty if N has no pipelined kernel; df: the plan of the double-float kernels
std::vector<int> pipe_radices(int N, bool df = false);

// Kernel family selection (process-wide): 0 automatic, 1 generic runtime-radix
// kernels only, 2 pipelined kernels wherever they apply.
int kernel_variant();
// whether float lengths with a compile-time plan kernel use it (variant != 3)
bool rt_compiled_plans();
void set_kernel_variant(int v);
// Arithmetic of the pipelined complex<double> c2c passes (process-wide):
// 0 FP64 instructions, 1 double-float pairs on the FP32 pipe.
enum { DA_FP64 = 0, DA_DOUBLE_FLOAT = 1 };
int double_arithmetic();
void set_double_arithmetic(int mode);

// Per-device status word written by kernels whose bounded waits gave up.
int *device_status();

} // namespace gbfft
