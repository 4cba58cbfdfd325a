// extern "C" boundary of libheffte_gb300 (declarations in include/heffte_gb300.h).
#include "gbfft_plan.h"
#include "gbfft_batch.h"
#include "gbfft_mlp.h"
#include "../../include/heffte_gb300.h"
#include <cstring>
#include <new>

using namespace gbfft;

struct heffte_gb300_executor_s { std::unique_ptr<Executor> e; };
struct heffte_gb300_plan_s { std::unique_ptr<Plan3D> p; };

namespace {

thread_local std::string g_last_error;

template<class F>
int guard(F &&fn){
    try {
        fn();
        g_last_error.clear();
        return HEFFTE_GB300_SUCCESS;
    } catch (Error const &e){
        g_last_error = e.what();
        return e.code;
    } catch (std::bad_alloc const &){
        g_last_error = "host allocation failed";
        return HEFFTE_GB300_ALLOC_ERROR;
    } catch (std::exception const &e){
        g_last_error = e.what();
        return HEFFTE_GB300_INVALID;
    }
}

cudaStream_t as_stream(void *s){ return reinterpret_cast<cudaStream_t>(s); }

void check_dtype(int dtype){
    if (dtype < 0 || dtype > 3) throw Error(ST_INVALID, "unknown element type code " + std::to_string(dtype));
}
void check_prec(int prec){
    if (prec != 0 && prec != 1) throw Error(ST_INVALID, "precision must be 0 (single) or 1 (double)");
}
void check_sizes(long long a, long long b, long long c){
    if (a < 0 || b < 0 || c < 0) throw Error(ST_INVALID, "negative size");
}

std::array<int, 3> order_of(int const *o){
    if (!o) return {0, 1, 2};
    std::array<int, 3> r{o[0], o[1], o[2]};
    if (!valid_order(r)) throw Error(ST_INVALID, "order must be a permutation of 0, 1, 2");
    return r;
}

} // namespace

namespace gbfft {
void set_last_error(std::string const &msg){ g_last_error = msg; }
}

extern "C" {

const char *heffte_gb300_last_error(void){ return g_last_error.c_str(); }
int heffte_gb300_version(void){ return 10000; }

int heffte_gb300_set_kernel_variant(int variant){
    return guard([&]{
        if (variant < 0 || variant > 3)
            throw Error(ST_INVALID, "variant must be 0 (auto), 1 (generic), 2 (pipelined) or 3 (auto, runtime plans)");
        set_kernel_variant(variant);
    });
}

int heffte_gb300_set_double_arithmetic(int mode){
    return guard([&]{
        if (mode != DA_FP64 && mode != DA_DOUBLE_FLOAT)
            throw Error(ST_INVALID, "mode must be 0 (FP64 instructions) or 1 (double-float)");
        set_double_arithmetic(mode);
    });
}

int heffte_gb300_double_arithmetic(void){ return double_arithmetic(); }

int heffte_gb300_device_status(int *status, int reset){
    return guard([&]{
        if (!status) throw Error(ST_INVALID, "null pointer");
        int *d = device_status();
        check_cuda(cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost), "read device status");
        if (reset) check_cuda(cudaMemset(d, 0, sizeof(int)), "reset device status");
    });
}

int heffte_gb300_convert(void *stream, int prec, long long n, const void *src, void *dst, int to_complex){
    return guard([&]{
        check_prec(prec);
        if (n < 0) throw Error(ST_INVALID, "negative size");
        if (n == 0) return;
        if (!src || !dst) throw Error(ST_INVALID, "null pointer");
        launch_convert(as_stream(stream), prec, n, src, dst, to_complex != 0);
        check_cuda(cudaPeekAtLastError(), "convert kernel launch");
    });
}

int heffte_gb300_scale_data(void *stream, int prec, long long num_reals, void *data, double factor){
    return guard([&]{
        check_prec(prec);
        if (num_reals < 0) throw Error(ST_INVALID, "negative size");
        if (num_reals == 0) return;   // empty box is allowed (src/heffte_backend_cuda.cu:473)
        if (!data) throw Error(ST_INVALID, "null pointer");
        launch_scale(as_stream(stream), prec, num_reals, data, factor);
        check_cuda(cudaPeekAtLastError(), "scale kernel launch");
    });
}

static int pack_common(void *stream, int dtype, long long nf, long long nm, long long ns, long long ls, long long ps,
                       const void *src, void *dst, bool pack){
    return guard([&]{
        check_dtype(dtype);
        check_sizes(nf, nm, ns);
        if (nf == 0 || nm == 0 || ns == 0) return;
        if (!src || !dst) throw Error(ST_INVALID, "null pointer");
        strided_extent(nf, nm, ns, ls, ps, pack ? "direct_pack source" : "direct_unpack destination");
        launch_direct_pack(as_stream(stream), dtype, nf, nm, ns, ls, ps, src, dst, pack);
        check_cuda(cudaPeekAtLastError(), pack ? "direct_pack kernel launch" : "direct_unpack kernel launch");
    });
}

int heffte_gb300_direct_pack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                             long long line_stride, long long plane_stride, const void *src, void *dst){
    return pack_common(stream, dtype, nfast, nmid, nslow, line_stride, plane_stride, src, dst, true);
}

int heffte_gb300_direct_unpack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                               long long line_stride, long long plane_stride, const void *src, void *dst){
    return pack_common(stream, dtype, nfast, nmid, nslow, line_stride, plane_stride, src, dst, false);
}

int heffte_gb300_transpose_unpack(void *stream, int dtype, long long nfast, long long nmid, long long nslow,
                                  long long line_stride, long long plane_stride,
                                  long long buff_line_stride, long long buff_plane_stride,
                                  int map0, int map1, int map2, const void *src, void *dst){
    return guard([&]{
        check_dtype(dtype);
        check_sizes(nfast, nmid, nslow);
        if (!valid_order({map0, map1, map2})) throw Error(ST_INVALID, "map must be a permutation of 0, 1, 2");
        if (nfast == 0 || nmid == 0 || nslow == 0) return;
        if (!src || !dst) throw Error(ST_INVALID, "null pointer");
        // the source's a-th dimension (fast, mid, slow) is destination dimension map[a]
        long long size[3] = {nfast, nmid, nslow};
        strided_extent(nfast, nmid, nslow, line_stride, plane_stride, "transpose_unpack destination");
        strided_extent(size[map0], size[map1], size[map2], buff_line_stride, buff_plane_stride,
                       "transpose_unpack source");
        launch_transpose_unpack(as_stream(stream), dtype, nfast, nmid, nslow, line_stride, plane_stride,
                                buff_line_stride, buff_plane_stride, map0, map1, src, dst);
        check_cuda(cudaPeekAtLastError(), "transpose_unpack kernel launch");
    });
}

int heffte_gb300_r2r_prepost(void *stream, int prec, int kind, int step, int length, long long lines,
                             long long in_ld, long long out_ld, const void *in, void *out){
    return guard([&]{
        check_prec(prec);
        if (kind < 0 || kind > 2) throw Error(ST_INVALID, "kind must be 0 (cos), 1 (sin) or 2 (cos1)");
        if (step < 0 || step > 3) throw Error(ST_INVALID, "step must be 0..3");
        if (length < 1 || (kind == 2 && length < 2) || lines < 0) throw Error(ST_INVALID, "invalid length");
        if (lines == 0) return;
        if (!in || !out) throw Error(ST_INVALID, "null pointer");
        launch_prepost(as_stream(stream), prec, kind, step, length, lines, in_ld, out_ld, in, out);
        check_cuda(cudaPeekAtLastError(), "r2r pre/post kernel launch");
    });
}

// ---------------------------------------------------------------------------
int heffte_gb300_executor_create(int kind, const long long low[3], const long long high[3], const int order[3],
                                 int ndims, const int dims[3], heffte_gb300_executor *out){
    return guard([&]{
        if (!out || !low || !high || !dims) throw Error(ST_INVALID, "null pointer");
        *out = nullptr;
        if (kind < 0 || kind > 4) throw Error(ST_INVALID, "unknown executor kind");
        if (ndims < 1 || ndims > 3) throw Error(ST_INVALID, "ndims must be 1, 2 or 3");
        Box3 box({low[0], low[1], low[2]}, {high[0], high[1], high[2]}, order_of(order));
        std::vector<int> d(dims, dims + ndims);
        auto e = make_executor(kind, box, d);
        if (!e) return;
        auto *h = new heffte_gb300_executor_s;
        h->e = std::move(e);
        *out = h;
    });
}

int heffte_gb300_executor_destroy(heffte_gb300_executor e){
    return guard([&]{ delete e; });
}

long long heffte_gb300_executor_box_size(heffte_gb300_executor e){ return e ? e->e->box_size() : 0; }
long long heffte_gb300_executor_complex_size(heffte_gb300_executor e){ return e ? e->e->complex_size() : 0; }
long long heffte_gb300_executor_workspace_size(heffte_gb300_executor e){ return e ? e->e->workspace_size() : 0; }

int heffte_gb300_executor_forward(heffte_gb300_executor e, void *stream, int prec, const void *in, void *out,
                                  void *workspace){
    return guard([&]{
        if (!e) throw Error(ST_INVALID, "null executor");
        check_prec(prec);
        if (!in || !out) throw Error(ST_INVALID, "null pointer");
        e->e->forward(as_stream(stream), prec, in, out, workspace);
    });
}

int heffte_gb300_executor_backward(heffte_gb300_executor e, void *stream, int prec, const void *in, void *out,
                                   void *workspace){
    return guard([&]{
        if (!e) throw Error(ST_INVALID, "null executor");
        check_prec(prec);
        if (!in || !out) throw Error(ST_INVALID, "null pointer");
        e->e->backward(as_stream(stream), prec, in, out, workspace);
    });
}

// ---------------------------------------------------------------------------
struct heffte_gb300_reshape_s { std::unique_ptr<Reshape> r; };

int heffte_gb300_reshape_create(int nranks, int me, const int *inboxes, const int *outboxes,
                                heffte_gb300_reshape *out){
    return guard([&]{
        if (!out || !inboxes || !outboxes) throw Error(ST_INVALID, "null pointer");
        *out = nullptr;
        if (nranks < 1) throw Error(ST_INVALID, "a reshape needs at least one rank");
        std::vector<Box3> ib, ob;
        for (int r = 0; r < nranks; r++){
            int const *a = inboxes + 9 * r, *b = outboxes + 9 * r;
            ib.emplace_back(std::array<long long, 3>{a[0], a[1], a[2]}, std::array<long long, 3>{a[3], a[4], a[5]},
                            order_of(a + 6));
            ob.emplace_back(std::array<long long, 3>{b[0], b[1], b[2]}, std::array<long long, 3>{b[3], b[4], b[5]},
                            order_of(b + 6));
        }
        auto R = make_reshape(nranks, me, ib, ob);
        auto *h = new heffte_gb300_reshape_s;
        h->r = std::move(R);
        *out = h;
    });
}

int heffte_gb300_reshape_destroy(heffte_gb300_reshape r){ return guard([&]{ delete r; }); }
long long heffte_gb300_reshape_send_size(heffte_gb300_reshape r){ return r ? r->r->send_total : -1; }
long long heffte_gb300_reshape_recv_size(heffte_gb300_reshape r){ return r ? r->r->recv_total : -1; }

int heffte_gb300_reshape_counts(heffte_gb300_reshape r, long long *send_counts, long long *send_displs,
                                long long *recv_counts, long long *recv_displs){
    return guard([&]{
        if (!r) throw Error(ST_INVALID, "null reshape");
        Reshape const &R = *r->r;
        for (int i = 0; i < R.nranks; i++){
            if (send_counts) send_counts[i] = R.send_counts[i];
            if (send_displs) send_displs[i] = R.send_displs[i];
            if (recv_counts) recv_counts[i] = R.recv_counts[i];
            if (recv_displs) recv_displs[i] = R.recv_displs[i];
        }
    });
}

int heffte_gb300_reshape_pack(heffte_gb300_reshape r, void *stream, int dtype, const void *input, void *send_buffer){
    return guard([&]{
        if (!r) throw Error(ST_INVALID, "null reshape");
        check_dtype(dtype);
        if (r->r->send_total == 0) return;
        if (!input || !send_buffer) throw Error(ST_INVALID, "null pointer");
        r->r->pack(as_stream(stream), dtype, input, send_buffer);
        check_cuda(cudaPeekAtLastError(), "reshape pack");
    });
}

int heffte_gb300_reshape_unpack(heffte_gb300_reshape r, void *stream, int dtype, const void *recv_buffer, void *output){
    return guard([&]{
        if (!r) throw Error(ST_INVALID, "null reshape");
        check_dtype(dtype);
        if (r->r->recv_total == 0) return;
        if (!recv_buffer || !output) throw Error(ST_INVALID, "null pointer");
        r->r->unpack(as_stream(stream), dtype, recv_buffer, output);
        check_cuda(cudaPeekAtLastError(), "reshape unpack");
    });
}

// ---------------------------------------------------------------------------
int heffte_gb300_set_default_options(heffte_gb300_plan_options *o){
    return guard([&]{
        if (!o) throw Error(ST_INVALID, "null options");
        o->use_reorder = 0;
        o->algorithm = 0;
        o->use_pencils = 1;
        o->use_gpu_aware = 1;
    });
}

int heffte_gb300_plan_create(int kind, const int inbox_low[3], const int inbox_high[3], const int *inbox_order,
                             const int outbox_low[3], const int outbox_high[3], const int *outbox_order,
                             int r2c_direction, const heffte_gb300_plan_options *options, void *stream,
                             heffte_gb300_plan *plan){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan pointer");
        *plan = nullptr;
        if (!inbox_low || !inbox_high || !outbox_low || !outbox_high) throw Error(ST_INVALID, "null box pointer");
        if (kind < 0 || kind > 4) throw Error(ST_INVALID, "unknown transform kind");
        Box3 ib({inbox_low[0], inbox_low[1], inbox_low[2]}, {inbox_high[0], inbox_high[1], inbox_high[2]},
                order_of(inbox_order));
        Box3 ob({outbox_low[0], outbox_low[1], outbox_low[2]}, {outbox_high[0], outbox_high[1], outbox_high[2]},
                order_of(outbox_order));
        Options o;
        if (options){
            o.use_reorder = options->use_reorder != 0;
            o.algorithm = options->algorithm;
            o.use_pencils = options->use_pencils != 0;
            o.use_gpu_aware = options->use_gpu_aware != 0;
        }
        auto p = make_plan(kind, ib, ob, r2c_direction, o, as_stream(stream));
        auto *h = new heffte_gb300_plan_s;
        h->p = std::move(p);
        *plan = h;
    });
}

int heffte_gb300_plan_destroy(heffte_gb300_plan plan){ return guard([&]{ delete plan; }); }

int heffte_gb300_plan_set_stream(heffte_gb300_plan plan, void *stream){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        plan->p->stream = as_stream(stream);
    });
}

long long heffte_gb300_size_inbox(heffte_gb300_plan plan){ return plan ? plan->p->size_inbox() : -1; }
long long heffte_gb300_size_outbox(heffte_gb300_plan plan){ return plan ? plan->p->size_outbox() : -1; }
long long heffte_gb300_size_workspace(heffte_gb300_plan plan){ return plan ? plan->p->size_workspace() : -1; }
double heffte_gb300_scale_factor(heffte_gb300_plan plan, int scale){ return plan ? plan->p->get_scale(scale) : 0.0; }

static int exec(heffte_gb300_plan plan, bool fwd, int batch, int prec, const void *in, void *out, void *work, int scale){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        plan->p->execute(fwd, prec, batch, in, out, work, scale);
        check_cuda(cudaPeekAtLastError(), fwd ? "forward transform" : "backward transform");
    });
}

int heffte_gb300_forward(heffte_gb300_plan plan, int prec, const void *input, void *output, void *workspace, int scale){
    return exec(plan, true, 1, prec, input, output, workspace, scale);
}
int heffte_gb300_backward(heffte_gb300_plan plan, int prec, const void *input, void *output, void *workspace, int scale){
    return exec(plan, false, 1, prec, input, output, workspace, scale);
}
int heffte_gb300_forward_batch(heffte_gb300_plan plan, int batch, int prec, const void *input, void *output,
                               void *workspace, int scale){
    return exec(plan, true, batch, prec, input, output, workspace, scale);
}
int heffte_gb300_backward_batch(heffte_gb300_plan plan, int batch, int prec, const void *input, void *output,
                                void *workspace, int scale){
    return exec(plan, false, batch, prec, input, output, workspace, scale);
}

long long heffte_gb300_convolve_workspace(heffte_gb300_plan plan){ return plan ? plan->p->convolve_workspace() : -1; }

int heffte_gb300_convolve_route(heffte_gb300_plan plan, int prec, int two_inputs, int *fused_dim){
    return guard([&]{
        if (!plan || !fused_dim) throw Error(ST_INVALID, "null plan or result pointer");
        if (prec != 0 && prec != 1) throw Error(ST_INVALID, "precision must be 0 (single) or 1 (double)");
        // 256-byte aligned stand-ins: the check only looks at the alignment
        void *aligned = reinterpret_cast<void*>((uintptr_t)1 << 20);
        *fused_dim = plan->p->convolve_fused_dim(prec, aligned, two_inputs ? aligned : nullptr);
    });
}

int heffte_gb300_convolve(heffte_gb300_plan plan, int prec, const void *x, const void *y, void *output,
                          void *workspace, int scale){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        plan->p->convolve(prec, x, y, output, workspace, scale);
        check_cuda(cudaPeekAtLastError(), "convolution");
    });
}

// ---------------------------------------------------------------------------
// batches of uneven boxes, autotuner
// ---------------------------------------------------------------------------
struct heffte_gb300_boxbatch_s { std::unique_ptr<Batch> b; };

int heffte_gb300_boxbatch_create(int kind, int prec, int nboxes, const int *sizes, void *stream,
                                 heffte_gb300_boxbatch *out){
    return guard([&]{
        if (!out || !sizes) throw Error(ST_INVALID, "null pointer");
        *out = nullptr;
        if (nboxes < 1) throw Error(ST_INVALID, "a batch needs at least one box");
        std::vector<std::array<int, 3>> sz(nboxes);
        for (int i = 0; i < nboxes; i++) sz[i] = {sizes[3 * i], sizes[3 * i + 1], sizes[3 * i + 2]};
        auto b = make_batch(kind, prec, sz, as_stream(stream));
        auto *h = new heffte_gb300_boxbatch_s;
        h->b = std::move(b);
        *out = h;
    });
}

int heffte_gb300_boxbatch_destroy(heffte_gb300_boxbatch b){ return guard([&]{ delete b; }); }

long long heffte_gb300_boxbatch_input_offset(heffte_gb300_boxbatch b, int box){
    return (b && box >= 0 && box < (int)b->b->in_offsets.size()) ? b->b->in_offsets[box] : -1;
}
long long heffte_gb300_boxbatch_output_offset(heffte_gb300_boxbatch b, int box){
    return (b && box >= 0 && box < (int)b->b->out_offsets.size()) ? b->b->out_offsets[box] : -1;
}
long long heffte_gb300_boxbatch_input_size(heffte_gb300_boxbatch b){ return b ? b->b->in_total : -1; }
long long heffte_gb300_boxbatch_output_size(heffte_gb300_boxbatch b){ return b ? b->b->out_total : -1; }
long long heffte_gb300_boxbatch_workspace_size(heffte_gb300_boxbatch b){ return b ? b->b->workspace_elems() : -1; }

int heffte_gb300_boxbatch_forward(heffte_gb300_boxbatch b, const void *input, void *output, int scale){
    return guard([&]{
        if (!b) throw Error(ST_INVALID, "null batch");
        b->b->run(true, input, output, nullptr, scale);
        check_cuda(cudaPeekAtLastError(), "batched forward transform");
    });
}

int heffte_gb300_boxbatch_backward(heffte_gb300_boxbatch b, const void *input, void *output, void *workspace, int scale){
    return guard([&]{
        if (!b) throw Error(ST_INVALID, "null batch");
        b->b->run(false, input, output, workspace, scale);
        check_cuda(cudaPeekAtLastError(), "batched backward transform");
    });
}

int heffte_gb300_boxbatch_configure(heffte_gb300_boxbatch b, int prefetch, int tile_kb, int group_mb, int values){
    return guard([&]{
        if (!b) throw Error(ST_INVALID, "null batch");
        Batch const &B = *b->b;
        BatchConfig c;
        c.prefetch = prefetch;
        c.tile_kb = tile_kb;
        c.group_mb = group_mb;
        c.values = values;
        b->b = make_batch(B.kind, B.prec, B.sizes, B.stream, c);
    });
}

int heffte_gb300_boxbatch_config(heffte_gb300_boxbatch b, int *prefetch, int *tile_kb, int *group_mb, int *values){
    return guard([&]{
        if (!b || !prefetch || !tile_kb || !group_mb || !values) throw Error(ST_INVALID, "null pointer");
        *prefetch = b->b->config.prefetch;
        *tile_kb = b->b->config.tile_kb;
        *group_mb = b->b->config.group_mb;
        *values = b->b->values;
    });
}

int heffte_gb300_boxbatch_autotune(heffte_gb300_boxbatch b, const void *input, void *output, void *back,
                                   void *workspace, int reps, int *prefetch, int *tile_kb, int *group_mb,
                                   int *values, double *ms){
    return guard([&]{
        if (!b) throw Error(ST_INVALID, "null batch");
        BatchConfig c = autotune_batch(b->b, input, output, back, workspace, reps, ms);
        if (prefetch) *prefetch = c.prefetch;
        if (tile_kb) *tile_kb = c.tile_kb;
        if (group_mb) *group_mb = c.group_mb;
        if (values) *values = b->b->values;
    });
}

int heffte_gb300_set_dependency_wait_budget(long long clocks){
    return guard([&]{ set_dependency_wait_budget(clocks); });
}

long long heffte_gb300_dependency_wait_budget(void){ return dependency_wait_budget(); }

int heffte_gb300_boxbatch_hold_dependencies(heffte_gb300_boxbatch b, int hold){
    return guard([&]{
        if (!b) throw Error(ST_INVALID, "null batch");
        b->b->hold_dependencies(hold != 0);
    });
}

int heffte_gb300_tune(int prec, int nlengths, const int *lengths, const char *cache_path, void *stream, int *measured){
    return guard([&]{
        if (!lengths && nlengths > 0) throw Error(ST_INVALID, "null pointer");
        check_prec(prec);
        std::vector<int> l(lengths, lengths + nlengths);
        int m = tune_lengths(l, prec, as_stream(stream), cache_path ? std::string(cache_path) : std::string());
        if (measured) *measured = m;
    });
}

int heffte_gb300_tune_load(const char *cache_path, int *entries){
    return guard([&]{
        if (!cache_path) throw Error(ST_INVALID, "null path");
        int n = tune_load(cache_path);
        if (entries) *entries = n;
    });
}

int heffte_gb300_tune_clear(void){ return guard([&]{ tune_clear(); }); }

// ---------------------------------------------------------------------------
// plan knobs and the learned selector
// ---------------------------------------------------------------------------
int heffte_gb300_plan_set_knobs(heffte_gb300_plan plan, int variant, int tile_div, int radix_policy){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        if (variant < 0 || variant > 1 || (tile_div != 1 && tile_div != 2) || radix_policy < 0 || radix_policy > 1)
            throw Error(ST_INVALID, "invalid knobs");
        Plan3D &p = *plan->p;
        Knobs k = p.knobs;
        k.variant = variant; k.tile_div = tile_div; k.radix_policy = radix_policy;
        plan->p = make_plan(p.kind, p.inbox, p.outbox, p.r2c_dir, p.opts, p.stream, k);
    });
}

int heffte_gb300_plan_set_tensor_cores(heffte_gb300_plan plan, int enable){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        if (enable != 0 && enable != 1) throw Error(ST_INVALID, "enable must be 0 or 1");
        Plan3D &p = *plan->p;
        Knobs k = p.knobs;
        k.tensor_cores = enable;
        plan->p = make_plan(p.kind, p.inbox, p.outbox, p.r2c_dir, p.opts, p.stream, k);
    });
}

int heffte_gb300_plan_set_convolution_fusion(heffte_gb300_plan plan, int enable){
    return guard([&]{
        if (!plan) throw Error(ST_INVALID, "null plan");
        if (enable != 0 && enable != 1) throw Error(ST_INVALID, "enable must be 0 or 1");
        plan->p->knobs.conv_fused = enable;
    });
}

int heffte_gb300_plan_features(int kind, int prec, const int size[3], float *features){
    return guard([&]{
        if (!size || !features) throw Error(ST_INVALID, "null pointer");
        plan_features(kind, prec, size, features);
    });
}

int heffte_gb300_candidate_options(int candidate, heffte_gb300_plan_options *options, int *variant, int *tile_div,
                                   int *radix_policy){
    return guard([&]{
        if (candidate < 0 || candidate >= kCandidates) throw Error(ST_INVALID, "candidate out of range");
        Options o; Knobs k;
        candidate_knobs(candidate, o, k);
        if (options){ options->use_reorder = o.use_reorder; options->algorithm = 0; options->use_pencils = 1; options->use_gpu_aware = 1; }
        if (variant) *variant = k.variant;
        if (tile_div) *tile_div = k.tile_div;
        if (radix_policy) *radix_policy = k.radix_policy;
    });
}

struct heffte_gb300_mlp_s { std::unique_ptr<Mlp> m; };

int heffte_gb300_mlp_create(int nin, int nhidden, int nout, unsigned long long seed, heffte_gb300_mlp *out){
    return guard([&]{
        if (!out) throw Error(ST_INVALID, "null pointer");
        *out = nullptr;
        auto *h = new heffte_gb300_mlp_s;
        try { h->m = std::make_unique<Mlp>(nin, nhidden, nout, seed); } catch (...) { delete h; throw; }
        *out = h;
    });
}
int heffte_gb300_mlp_destroy(heffte_gb300_mlp m){ return guard([&]{ delete m; }); }
long long heffte_gb300_mlp_num_params(heffte_gb300_mlp m){ return m ? m->m->nparams : -1; }

int heffte_gb300_mlp_get_params(heffte_gb300_mlp m, float *host){
    return guard([&]{
        if (!m || !host) throw Error(ST_INVALID, "null pointer");
        check_cuda(cudaMemcpy(host, m->m->params, m->m->nparams * sizeof(float), cudaMemcpyDeviceToHost), "copy params");
    });
}
int heffte_gb300_mlp_set_params(heffte_gb300_mlp m, const float *host){
    return guard([&]{
        if (!m || !host) throw Error(ST_INVALID, "null pointer");
        check_cuda(cudaMemcpy(m->m->params, host, m->m->nparams * sizeof(float), cudaMemcpyHostToDevice), "copy params");
    });
}

int heffte_gb300_mlp_loss_grad(heffte_gb300_mlp m, const float *X, const float *T, int n, float *loss, float *host_grads){
    return guard([&]{
        if (!m || !X || !T || n < 1) throw Error(ST_INVALID, "invalid arguments");
        m->m->loss_and_grad(nullptr, X, T, n);
        check_cuda(cudaDeviceSynchronize(), "mlp gradient");
        if (loss) check_cuda(cudaMemcpy(loss, m->m->loss_d, sizeof(float), cudaMemcpyDeviceToHost), "copy loss");
        if (host_grads) check_cuda(cudaMemcpy(host_grads, m->m->grads, m->m->nparams * sizeof(float), cudaMemcpyDeviceToHost), "copy grads");
    });
}

int heffte_gb300_mlp_train(heffte_gb300_mlp m, const float *X, const float *T, int n, int steps, float lr, void *stream,
                           float *final_loss){
    return guard([&]{
        if (!m || !X || !T || n < 1 || steps < 0) throw Error(ST_INVALID, "invalid arguments");
        float l = m->m->train(as_stream(stream), X, T, n, steps, lr);
        if (final_loss) *final_loss = l;
    });
}

int heffte_gb300_mlp_predict(heffte_gb300_mlp m, const float *X, float *Y, int n, void *stream){
    return guard([&]{
        if (!m || !X || !Y || n < 1) throw Error(ST_INVALID, "invalid arguments");
        m->m->forward(as_stream(stream), X, n);
        check_cuda(cudaMemcpyAsync(Y, m->m->y, (size_t)n * m->m->nout * sizeof(float), cudaMemcpyDeviceToDevice,
                                   as_stream(stream)), "copy predictions");
    });
}

int heffte_gb300_select(heffte_gb300_mlp m, int kind, int prec, const int size[3], int *candidate){
    return guard([&]{
        if (!m || !size || !candidate) throw Error(ST_INVALID, "null pointer");
        if (m->m->nin != kFeatures || m->m->nout != kCandidates) throw Error(ST_INVALID, "the network does not match the selector's features / candidates");
        float f[kFeatures];
        plan_features(kind, prec, size, f);
        check_cuda(cudaMemcpy(m->m->xrow, f, sizeof(f), cudaMemcpyHostToDevice), "copy features");
        m->m->forward(nullptr, m->m->xrow, 1);
        float y[kCandidates];
        check_cuda(cudaMemcpy(y, m->m->y, sizeof(y), cudaMemcpyDeviceToHost), "copy prediction");
        int best = 0;
        for (int c = 1; c < kCandidates; c++) if (y[c] < y[best]) best = c;
        *candidate = best;
    });
}

int heffte_gb300_tuned_choice(int prec, int length, int *radices, int *nradices, int *tpb, double *us){
    return guard([&]{
        if (!radices || !nradices || !tpb) throw Error(ST_INVALID, "null pointer");
        TuneChoice c = tuned_choice(length, prec);
        *nradices = (int)c.radices.size();
        for (size_t i = 0; i < c.radices.size() && i < 16; i++) radices[i] = c.radices[i];
        *tpb = c.tpb;
        if (us) *us = c.us;
    });
}

} // extern "C"
