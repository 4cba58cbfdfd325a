/*
 * heffte_gb300.h - C ABI of the GB300-native fft3d backend for heFFTe.
 *
 * A single-GPU, single-rank (MPI_COMM_SELF) drop-in for the device parts of
 * heFFTe's fft3d hot path.  Plain C: opaque handles, raw device pointers,
 * sizes as integers, a cudaStream_t passed as `void*` (NULL = default stream).
 * Every function returns a status code (HEFFTE_GB300_SUCCESS = 0) and never
 * throws; the message of the last failure on the calling thread is returned by
 * heffte_gb300_last_error().  The reference turns every CUDA error into
 * std::runtime_error("<call> failed with message: <text>")
 * (include/heffte_backend_cuda.h:49-60); the reference-side shim in
 * INTEGRATION.md rethrows our status the same way.
 *
 * Three layers, each replacing a reference interface:
 *   1. location layer  -> src/heffte_backend_cuda.cu (cuda::convert, scale_data,
 *                         direct_pack, direct_unpack, transpose_unpack);
 *   2. executors       -> cufft_executor, cufft_executor_r2c and
 *                         real2real_executor<cufft_cos|cufft_sin>;
 *   3. 3-D plans       -> heffte::fft3d / fft3d_r2c / rtransform on one rank,
 *                         shaped after the reference C API (include/heffte_c.h).
 */
#ifndef HEFFTE_GB300_H
#define HEFFTE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define HEFFTE_GB300_SUCCESS 0
#define HEFFTE_GB300_INVALID 1      /* bad geometry, null pointer, bad option   */
#define HEFFTE_GB300_CUDA_ERROR 2   /* a CUDA runtime call or launch failed     */
#define HEFFTE_GB300_UNSUPPORTED 3  /* e.g. a transform length above 2^25           */
#define HEFFTE_GB300_ALLOC_ERROR 4  /* device allocation failed                  */

/* element types: float, double, std::complex<float>, std::complex<double> */
#define HEFFTE_GB300_FLOAT 0
#define HEFFTE_GB300_DOUBLE 1
#define HEFFTE_GB300_CFLOAT 2
#define HEFFTE_GB300_CDOUBLE 3

/* precision of a transform */
#define HEFFTE_GB300_SINGLE 0
#define HEFFTE_GB300_DOUBLE_PREC 1

/* heffte::scale (include/heffte_fft3d.h:140-147), same values as heffte_c_defines.h */
#define HEFFTE_GB300_SCALE_NONE 0
#define HEFFTE_GB300_SCALE_FULL 1
#define HEFFTE_GB300_SCALE_SYMMETRIC 2

/* transform kinds: fft3d (c2c), fft3d_r2c, rtransform<cos> (DCT-II / 2xDCT-III),
 * rtransform<sin> (DST-II / 2xDST-III), rtransform<cos1> (DCT-I / 2xDCT-I,
 * scale 1/(64 prod(n_i - 1)), every n_i >= 2) */
#define HEFFTE_GB300_C2C 0
#define HEFFTE_GB300_R2C 1
#define HEFFTE_GB300_COS 2
#define HEFFTE_GB300_SIN 3
#define HEFFTE_GB300_COS1 4

/* Message of the last failure on this thread ("" after a success). */
const char *heffte_gb300_last_error(void);
/* 10000*major + 100*minor + patch */
int heffte_gb300_version(void);

/* No reference counterpart (tuning / diagnostics of this backend).
 * Kernel family used by all later calls of this process: 0 automatic
 * (pipelined power-of-two kernels where they apply; float lengths 96, 160,
 * 192, 240, 288, 320, 384, 448, 480, 576, 640, 720, 768 and 960 by kernels
 * compiled for their radix plan), 1 generic
 * runtime-radix kernels only, 2 pipelined kernels wherever they apply, 3 as
 * 0 but every length that is not a power of two on the runtime radix plan. */
int heffte_gb300_set_kernel_variant(int variant);

/* No reference counterpart.  Arithmetic of the complex<double> passes of
 * power-of-two lengths (the pipelined kernels) for all later calls of this
 * process: 0 = FP64 instructions; 1 (default) = double-float, each value carried as
 * the unevaluated sum of two floats (about 48 significant bits) on the FP32
 * pipe, every tile scaled by a power of two into the float exponent range
 * (values below 2^-126 of a tile's largest are dropped, which changes the
 * tile's norm by less than 2^-126).  Both hold rel-L2 <= 1e-12 against an
 * FP64 transform; on GB300 the FP64 pipe issues 1/64 of the FP32 rate.
 * Other lengths and kinds always use FP64 instructions. */
int heffte_gb300_set_double_arithmetic(int mode);
int heffte_gb300_double_arithmetic(void);

/* No reference counterpart.  Reads the current device's status word: 0 = no
 * fault; otherwise a bounded device wait gave up and its kernel returned
 * early, so that call's output is invalid: 1 = a wait for a bulk (TMA) copy,
 * 2 = the batch kernel's wait for another CTA's pass of the same box, 3 = a
 * wait for tensor-core MMAs.  Synchronises with the device.  reset != 0
 * clears the word after reading. */
int heffte_gb300_device_status(int *status, int reset);

/* ======================================================================= */
/* 1. Location layer                                                        */
/* ======================================================================= */

/* Replaces cuda::convert (src/heffte_backend_cuda.cu:345-361):
 * to_complex = 1: dst[2i] = src[i], dst[2i+1] = 0 for i < n;
 * to_complex = 0: dst[i] = src[2i].  prec 0 = float, 1 = double. */
int heffte_gb300_convert(void *stream, int prec, long long n, const void *src, void *dst, int to_complex);

/* Replaces cuda::scale_data (src/heffte_backend_cuda.cu:471-483):
 * data[i] *= (scalar) factor for i < num_reals (complex data = 2n reals).
 * num_reals = 0 is a no-op, as in the reference. */
int heffte_gb300_scale_data(void *stream, int prec, long long num_reals, void *data, double factor);

/* Replaces cuda::direct_pack (src/heffte_backend_cuda.cu:385-393), i.e.
 * direct_packer<tag::gpu>::pack (include/heffte_backend_cuda.h:800-806):
 * dst[(slow*nmid + mid)*nfast + fast] = src[slow*plane_stride + mid*line_stride + fast].
 * dtype: HEFFTE_GB300_FLOAT .. HEFFTE_GB300_CDOUBLE.  Bit-exact copy. */
int heffte_gb300_direct_pack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                             long long line_stride, long long plane_stride, const void *src, void *dst);

/* Replaces cuda::direct_unpack (src/heffte_backend_cuda.cu:395-402): the inverse of direct_pack. */
int heffte_gb300_direct_unpack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                               long long line_stride, long long plane_stride, const void *src, void *dst);

/* Replaces cuda::transpose_unpack (src/heffte_backend_cuda.cu:404-441), i.e.
 * transpose_packer<tag::gpu>::unpack (include/heffte_backend_cuda.h:824-828):
 * dst[k*plane_stride + j*line_stride + i] = src[<map case>] for the six
 * (map0, map1, map2) cases of the reference kernel (:90-133). Bit-exact.
 * Strides that are negative or make lines / planes overlap, on either side,
 * are rejected with HEFFTE_GB300_INVALID (also for direct_pack / unpack). */
int heffte_gb300_transpose_unpack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                                  long long line_stride, long long plane_stride,
                                  long long buff_line_stride, long long buff_plane_stride,
                                  int map0, int map1, int map2, const void *src, void *dst);

/* No counterpart in the reference.  transpose_unpack performed in place, for
 * callers that cannot allocate device memory: programs whose device memory is
 * owned by an arena that forbids other allocations, real-time loops that must
 * not allocate after start-up (cudaMalloc can synchronise the device and take
 * unbounded time), and callers at the memory limit.  `data` holds the source
 * in the buffer layout (buff_line_stride, buff_plane_stride) and receives the
 * destination (line_stride, plane_stride); the six maps are those of
 * heffte_gb300_transpose_unpack.  The source is staged in a fixed 32 MiB
 * scratch array inside the library (reserved on every GPU that loads the
 * library until the process exits); a larger source, and strides that are
 * negative, overlap or overflow, are rejected with HEFFTE_GB300_INVALID.  The
 * first call on a device (and the first after a cudaDeviceReset) looks up the
 * array's device address; make it before any stream capture.  All calls share the
 * array, which keeps the last call's contents, so calls that overlap on the
 * GPU (e.g. on two streams) race.  Nothing is allocated. */
int heffte_gb300_transpose_unpack_inplace_noalloc(void *stream, int dtype, long long nfast, long long nmid,
                                                  long long nslow, long long line_stride, long long plane_stride,
                                                  long long buff_line_stride, long long buff_plane_stride,
                                                  int map0, int map1, int map2, void *data);

/* Replaces cuda::{cos,sin,cos1}_pre_pos_processor::{pre,post}_{forward,backward}
 * (include/heffte_backend_cuda.h:116-174, kernels src/heffte_backend_cuda.cu:149-327)
 * and batches them: `lines` lines of length `length` (N) in one launch.
 *   kind: 0 cos (DCT-II/III), 1 sin (DST-II/III), 2 cos1 (DCT-I);
 *   step: 0 pre_forward  (real N  -> real M),    1 post_forward (complex M/2+1 -> real N),
 *         2 pre_backward (real N  -> complex M/2+1), 3 post_backward (real M -> real N);
 *   M = 4N (cos, sin) or 4(N-1) (cos1); in_ld / out_ld: distance between
 *   lines in elements of the input / output type.  Every output entry of a
 *   line is written (the reference's pre_forward also zeroes entry 4N, which
 *   is outside the line and never read). */
int heffte_gb300_r2r_prepost(void *stream, int prec, int kind, int step, int length, long long lines,
                             long long in_ld, long long out_ld, const void *in, void *out);

/* ======================================================================= */
/* 2. Executors (one_dim_backend<tag>::executor / executor_r2c)             */
/* ======================================================================= */

typedef struct heffte_gb300_executor_s *heffte_gb300_executor;

/* Creates a batched executor on the box {low, high, order}:
 *   kind C2C: ndims = 1, 2 or 3 transform dimensions, the roles of the
 *             cufft_executor constructors (include/heffte_backend_cuda.h:445-491);
 *   kind R2C: ndims = 1, cufft_executor_r2c (:631-646);
 *   kind COS / SIN / COS1: ndims = 1, real2real_executor<cufft_cos|cufft_sin|
 *             cufft_cos1> (include/heffte_r2r_executor.h:191-210); unlike the
 *             reference the dimension need not be the fastest one.
 * An empty box gives *out = NULL and HEFFTE_GB300_SUCCESS, as make_executor
 * returns a null pointer for empty boxes (include/heffte_common.h:669-676). */
int heffte_gb300_executor_create(int kind, const long long low[3], const long long high[3], const int order[3],
                                 int ndims, const int dims[3], heffte_gb300_executor *out);
int heffte_gb300_executor_destroy(heffte_gb300_executor e);
/* executor_base::box_size / complex_size / workspace_size (include/heffte_common.h:585-594).
 * The workspace is counted in elements of the executor's data type (complex
 * for C2C / R2C, real for COS / SIN / COS1, of the precision of each call);
 * it is 0 unless a length is transformed by the composite algorithms: lengths
 * above 8192 (four-step, N = N1 N2) and lengths with a prime factor above 13
 * (Bluestein's algorithm), which the cufft_executor role also accepts
 * (include/heffte_backend_cuda.h:346-422). */
long long heffte_gb300_executor_box_size(heffte_gb300_executor e);
long long heffte_gb300_executor_complex_size(heffte_gb300_executor e);
long long heffte_gb300_executor_workspace_size(heffte_gb300_executor e);
/* Forward / backward.  C2C and COS/SIN: in-place when in == out (the
 * reference signature forward(data[], workspace)); R2C forward: real in ->
 * complex out; R2C backward: complex in -> real out (the input is not modified).
 * prec 0 = single, 1 = double.  workspace: workspace_size() elements, or NULL
 * (the executor then allocates one buffer of its own once and keeps it). */
int heffte_gb300_executor_forward(heffte_gb300_executor e, void *stream, int prec, const void *in, void *out,
                                  void *workspace);
int heffte_gb300_executor_backward(heffte_gb300_executor e, void *stream, int prec, const void *in, void *out,
                                   void *workspace);

/* ======================================================================= */
/* 2b. Reshapes between the box decompositions of a group of ranks          */
/* ======================================================================= */

/* Replaces reshape3d_alltoallv (src/heffte_reshape3d.cpp:365-443, built by
 * make_reshape3d_alltoallv, :445-496) on rank `me` of `nranks`, one GPU per
 * rank.  inboxes / outboxes hold 9 ints per rank (low[3], high[3], order[3])
 * for every rank of the group, as mpi::gather_boxes gives them
 * (include/heffte_geometry.h:707-718).  This rank sends the overlap of its
 * input box with each rank's output box and receives the overlap of its
 * output box with each rank's input box.  pack() gathers the outgoing
 * overlaps into one send buffer (send_size() elements, rank r's part at
 * send_displs[r], send_counts[r] elements, in this rank's input order);
 * unpack() scatters a receive buffer laid out the same way (recv_counts,
 * recv_displs) into the output box, transposing chunks whose sender's order
 * differs.  The exchange between the two, the reference's MPI_Alltoallv, is
 * the caller's (MPI_Alltoallv, NCCL send / recv, or a host-staged all-to-all).
 * Bit-exact copies; dtype as for direct_pack. */
typedef struct heffte_gb300_reshape_s *heffte_gb300_reshape;
int heffte_gb300_reshape_create(int nranks, int me, const int *inboxes, const int *outboxes,
                                heffte_gb300_reshape *reshape);
int heffte_gb300_reshape_destroy(heffte_gb300_reshape reshape);
long long heffte_gb300_reshape_send_size(heffte_gb300_reshape reshape);
long long heffte_gb300_reshape_recv_size(heffte_gb300_reshape reshape);
/* nranks entries each (any pointer may be NULL) */
int heffte_gb300_reshape_counts(heffte_gb300_reshape reshape, long long *send_counts, long long *send_displs,
                                long long *recv_counts, long long *recv_displs);
int heffte_gb300_reshape_pack(heffte_gb300_reshape reshape, void *stream, int dtype, const void *input,
                              void *send_buffer);
int heffte_gb300_reshape_unpack(heffte_gb300_reshape reshape, void *stream, int dtype, const void *recv_buffer,
                                void *output);

/* ======================================================================= */
/* 3. 3-D plans: fft3d / fft3d_r2c / rtransform on one rank                 */
/* ======================================================================= */

/* plan_options (include/heffte_plan_logic.h:131-176), laid out as
 * heffte_plan_options (include/heffte_c_defines.h:98-107). On one rank only
 * use_reorder changes the device work: 1 = transpose so that every 1-D pass
 * is contiguous (the reference's reshape3d_transpose), 0 = strided passes. */
typedef struct {
    int use_reorder;
    int algorithm;
    int use_pencils;
    int use_gpu_aware;
} heffte_gb300_plan_options;

typedef struct heffte_gb300_plan_s *heffte_gb300_plan;

/* Defaults of the GB300 tags: use_reorder = 0, alltoallv, pencils, gpu-aware
 * (heffte_set_default_options, include/heffte_c.h:62). */
int heffte_gb300_set_default_options(heffte_gb300_plan_options *options);

/* heffte_plan_create / heffte_plan_create_r2c (include/heffte_c.h:78-105) for
 * one rank: the boxes span the whole index set; *_order may be NULL for
 * (0,1,2).  kind: HEFFTE_GB300_C2C, _R2C (outbox = inbox.r2c(r2c_direction)),
 * _COS, _SIN or _COS1.  stream: the cudaStream_t every call of this plan uses
 * (NULL = default stream, a non-owning handle as in fft3d's constructor). */
int heffte_gb300_plan_create(int kind, const int inbox_low[3], const int inbox_high[3], const int *inbox_order,
                             const int outbox_low[3], const int outbox_high[3], const int *outbox_order,
                             int r2c_direction, const heffte_gb300_plan_options *options, void *stream,
                             heffte_gb300_plan *plan);
int heffte_gb300_plan_destroy(heffte_gb300_plan plan);
int heffte_gb300_plan_set_stream(heffte_gb300_plan plan, void *stream);

/* fft3d::size_inbox / size_outbox / size_workspace (include/heffte_fft3d.h:324-331, :553-555).
 * The workspace is counted in elements of the complex type (c2c, r2c) or of
 * the real type (cos, sin). */
long long heffte_gb300_size_inbox(heffte_gb300_plan plan);
long long heffte_gb300_size_outbox(heffte_gb300_plan plan);
long long heffte_gb300_size_workspace(heffte_gb300_plan plan);
/* fft3d::get_scale_factor (include/heffte_fft3d.h:548-550) */
double heffte_gb300_scale_factor(heffte_gb300_plan plan, int scale);

/* fft3d::forward / backward with and without workspace
 * (include/heffte_fft3d.h:353-542; heffte_forward_*, heffte_backward_*,
 * include/heffte_c.h:140-256).  prec 0 = single, 1 = double.  Input is never
 * modified.  workspace = NULL uses a buffer the plan allocates once and keeps
 * (the reference allocates one per call).  batch > 1 transforms batch
 * contiguous inputs (stride size_inbox) into contiguous outputs. */
int heffte_gb300_forward(heffte_gb300_plan plan, int prec, const void *input, void *output, void *workspace,
                         int scale);
int heffte_gb300_backward(heffte_gb300_plan plan, int prec, const void *input, void *output, void *workspace,
                          int scale);
int heffte_gb300_forward_batch(heffte_gb300_plan plan, int batch, int prec, const void *input, void *output,
                               void *workspace, int scale);
int heffte_gb300_backward_batch(heffte_gb300_plan plan, int batch, int prec, const void *input, void *output,
                                void *workspace, int scale);

/* Circular convolution through the plan's transforms, the step of the
 * reference's convolution benchmark (benchmarks/convolution.cpp:89-95:
 * forward, pointwise product, backward) as one call:
 *     output = backward( forward(x) .* forward(y) ),
 * both forward transforms unscaled, the backward one scaled by `scale`
 * (HEFFTE_GB300_SCALE_FULL gives the circular convolution of x and y).
 * y = NULL or y = x: self-convolution (the benchmark's X .* X).  c2c plans
 * take and return complex inbox arrays, r2c plans real ones (the product
 * runs on the half spectrum).  x, y and output may alias one another.
 * workspace = NULL uses a buffer the plan allocates once, else it holds
 * convolve_workspace() complex elements.  On c2c plans without reshapes the
 * forward transform along one dimension, the product and the backward
 * transform along it run as one fused kernel. */
long long heffte_gb300_convolve_workspace(heffte_gb300_plan plan);
/* The route convolve takes for 16-byte aligned arrays: *fused_dim = the
 * dimension of the fused pass, or -1 for the unfused sequence (two forward
 * transforms, a product kernel, a backward transform). */
int heffte_gb300_convolve_route(heffte_gb300_plan plan, int prec, int two_inputs, int *fused_dim);
int heffte_gb300_convolve(heffte_gb300_plan plan, int prec, const void *x, const void *y, void *output,
                          void *workspace, int scale);

/* ======================================================================= */
/* 4. Batches of many small boxes of uneven sizes, autotuner                */
/* ======================================================================= */

/* No reference counterpart as one call: it replaces a loop over many
 * fft3d_r2c<cufft> (or fft3d<cufft>) objects, one per box, each box on one
 * rank with order (0,1,2), r2c along dimension 0.  All boxes run in ONE
 * persistent kernel launch (a device work queue over the 1-D passes of all
 * boxes, with per-box pass dependencies), replayed as a CUDA graph.  Inputs
 * of all boxes are packed in one array (box i at input_offset(i)), outputs in
 * another (box i at output_offset(i)); offsets count elements of the
 * respective type.  kind: HEFFTE_GB300_R2C or HEFFTE_GB300_C2C; sizes holds
 * nboxes triplets (n0, n1, n2).  The backward transform needs a workspace of
 * workspace_size() complex elements and leaves its input untouched; scaling
 * is per box (1/(n0 n1 n2) for scale::full). */
typedef struct heffte_gb300_boxbatch_s *heffte_gb300_boxbatch;
int heffte_gb300_boxbatch_create(int kind, int prec, int nboxes, const int *sizes, void *stream,
                                 heffte_gb300_boxbatch *batch);
int heffte_gb300_boxbatch_destroy(heffte_gb300_boxbatch batch);
long long heffte_gb300_boxbatch_input_offset(heffte_gb300_boxbatch batch, int box);
long long heffte_gb300_boxbatch_output_offset(heffte_gb300_boxbatch batch, int box);
long long heffte_gb300_boxbatch_input_size(heffte_gb300_boxbatch batch);
long long heffte_gb300_boxbatch_output_size(heffte_gb300_boxbatch batch);
long long heffte_gb300_boxbatch_workspace_size(heffte_gb300_boxbatch batch);
int heffte_gb300_boxbatch_forward(heffte_gb300_boxbatch batch, const void *input, void *output, int scale);
int heffte_gb300_boxbatch_backward(heffte_gb300_boxbatch batch, const void *input, void *output, void *workspace,
                                   int scale);

/* No reference counterpart.  Launch shape of a batch: prefetch = 1 copies
 * each CTA's next tile into shared memory while the CTA transforms the
 * current one (when that tile's pass dependency is already met; default 0);
 * tile_kb (8..96, default 48) bounds one tile's shared exchange buffer, so
 * smaller values give smaller tiles and more CTAs per SM; group_mb (0..4096,
 * default 0) > 0 queues the boxes in groups of about that many MB of
 * spectrum with each group's passes two groups apart, so a box's data stays
 * in L2 from one pass to the next (0: pass 0 of every box, then pass 1, then
 * pass 2); values (0, 8 or 16, default 0) is the number of complex values
 * each thread holds: 8 runs radix plans up to 8 with fewer registers and
 * needs box sides whose prime factors are at most 7, 16 (or 0) runs any plan.  Results agree for every shape (to
 * rounding: the radix plan may differ).  configure() rebuilds the batch with
 * a shape; config() reports it (values: the one in use); autotune() times
 * forward (input -> output) + backward (output -> back, with workspace)
 * `reps` times for every shape (the tuning table's radix plans or the
 * default ones x 16 / 8 values x groups of 0, 16 MB x prefetch on / off x
 * 48, 32, 24 KB), keeps the fastest (the untuned default is a candidate, so
 * tuning never makes a batch slower beyond timing noise), and returns it
 * with its ms per forward + backward; it overwrites output, back and
 * workspace, and leaves input as it was. */
int heffte_gb300_boxbatch_configure(heffte_gb300_boxbatch batch, int prefetch, int tile_kb, int group_mb, int values);
int heffte_gb300_boxbatch_config(heffte_gb300_boxbatch batch, int *prefetch, int *tile_kb, int *group_mb, int *values);
int heffte_gb300_boxbatch_autotune(heffte_gb300_boxbatch batch, const void *input, void *output, void *back,
                                   void *workspace, int reps, int *prefetch, int *tile_kb, int *group_mb,
                                   int *values, double *ms);

/* No reference counterpart.  Clock budget (GPU clocks, >= 0) after which the
 * batch kernel's wait for another CTA's pass of the same box gives up, records
 * status 2 (heffte_gb300_device_status) and returns; read at every batch
 * launch; default 4e9 (about two seconds).  The waits for bulk copies and
 * tensor-core MMAs keep the default: giving up on them early could return
 * while a copy or an MMA still writes the CTA's memory. */
int heffte_gb300_set_dependency_wait_budget(long long clocks);
long long heffte_gb300_dependency_wait_budget(void);
/* No reference counterpart; a test hook for the give-up path.  hold = 1 makes
 * every pass dependency of the batch wait for one tile more than its pass has
 * (a count no CTA reaches), so each such wait runs out of its budget; hold = 0
 * restores the batch.  Nothing faults: the waiting CTAs record status 2 and
 * return. */
int heffte_gb300_boxbatch_hold_dependencies(heffte_gb300_boxbatch batch, int hold);

/* No reference counterpart.  Measures, on the current device, every candidate
 * radix plan and tile size of each length and keeps the fastest for later
 * batches (plans made after the call use it).  With a cache path the results
 * are appended to that file after each length, keyed by the device, and
 * lengths already in the file are not measured again (an interrupted tuning
 * resumes).  *measured (may be NULL) receives the number of lengths timed. */
int heffte_gb300_tune(int prec, int nlengths, const int *lengths, const char *cache_path, void *stream,
                      int *measured);
/* Loads the entries of a tuning cache written for this device. */
int heffte_gb300_tune_load(const char *cache_path, int *entries);
int heffte_gb300_tune_clear(void);
/* The tuned choice of a length (nradices = 0 when it was never measured);
 * radices must hold 16 ints. */
int heffte_gb300_tuned_choice(int prec, int length, int *radices, int *nradices, int *tpb, double *us);

/* ======================================================================= */
/* 5. Plan knobs and the learned plan selector (no reference counterpart)   */
/* ======================================================================= */

/* Re-plans with the given knobs: variant 0 = pipelined kernels where they
 * apply, 1 = generic kernels only; tile_div 1 or 2 divides the automatic tile
 * of the generic kernels; radix_policy 0 = default radix order, 1 = ascending.
 * Results are unchanged (within rounding); only the speed differs. */
int heffte_gb300_plan_set_knobs(heffte_gb300_plan plan, int variant, int tile_div, int radix_policy);
/* Precision form of the plan's complex<float> 1-D passes: enable = 1 evaluates
 * their radix-16 butterflies as 16-point DFT contractions on the tensor cores
 * (tcgen05, operands split into three BF16 terms, FP32 accumulation; lengths
 * 16^s * {1,2,4,8} in [64, 4096], other lengths keep the FP32 kernels);
 * enable = 0 (default) is the plain FP32 form.  No counterpart in the
 * reference, whose GPU backends call cuFFT / rocFFT / oneMKL
 * (src/heffte_backend_cuda.cu). */
int heffte_gb300_plan_set_tensor_cores(heffte_gb300_plan plan, int enable);
/* enable = 1 (default): convolve takes its fused route where it applies;
 * 0: always the unfused sequence (forward transforms, product kernel,
 * backward transform), the reference's order of operations. */
int heffte_gb300_plan_set_convolution_fusion(heffte_gb300_plan plan, int enable);
/* The 18 features the selector reads for a transform of `kind` and `prec`. */
int heffte_gb300_plan_features(int kind, int prec, const int size[3], float *features);
/* Candidate c in [0, 16): use_reorder = c & 1, variant = (c >> 1) & 1,
 * tile_div = 1 + ((c >> 2) & 1), radix_policy = (c >> 3) & 1. */
int heffte_gb300_candidate_options(int candidate, heffte_gb300_plan_options *options, int *variant, int *tile_div,
                                   int *radix_policy);

/* A 3-layer perceptron (nin -> nhidden -> nhidden -> nout, ReLU), trained on
 * the GPU by this library's own forward, backward and Adam kernels (FP32).
 * Parameters are W1, b1, W2, b2, W3, b3 (row-major, W[in][out]).  X and T
 * are device arrays of n rows; the loss is the mean squared error. */
typedef struct heffte_gb300_mlp_s *heffte_gb300_mlp;
int heffte_gb300_mlp_create(int nin, int nhidden, int nout, unsigned long long seed, heffte_gb300_mlp *mlp);
int heffte_gb300_mlp_destroy(heffte_gb300_mlp mlp);
long long heffte_gb300_mlp_num_params(heffte_gb300_mlp mlp);
int heffte_gb300_mlp_get_params(heffte_gb300_mlp mlp, float *host_params);
int heffte_gb300_mlp_set_params(heffte_gb300_mlp mlp, const float *host_params);
/* Loss and gradient of one full batch (host copies; synchronises). */
int heffte_gb300_mlp_loss_grad(heffte_gb300_mlp mlp, const float *X, const float *T, int n, float *loss,
                               float *host_grads);
/* `steps` full-batch Adam steps with learning rate lr; *final_loss = last loss. */
int heffte_gb300_mlp_train(heffte_gb300_mlp mlp, const float *X, const float *T, int n, int steps, float lr,
                           void *stream, float *final_loss);
/* Y[n x nout] = network(X[n x nin]) (device arrays). */
int heffte_gb300_mlp_predict(heffte_gb300_mlp mlp, const float *X, float *Y, int n, void *stream);
/* The candidate the network predicts fastest for one transform (an
 * 18-in / 16-out network); the caller then uses heffte_gb300_candidate_options. */
int heffte_gb300_select(heffte_gb300_mlp mlp, int kind, int prec, const int size[3], int *candidate);

#ifdef __cplusplus
}
#endif

#endif
