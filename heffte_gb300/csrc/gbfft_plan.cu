// Single-rank fft3d plan for the GB300 backend: stage sequencing of
// compute_transform (src/heffte_compute_transform.cpp:15-258) and the setup
// of fft3d / fft3d_r2c (include/heffte_fft3d.h:599-651,
// include/heffte_fft3d_r2c.h:325-340), rebuilt around fused device passes:
//   * every 1-D pass reads its source buffer and writes its destination
//     directly (no copy_n of the input, no separate scale pass: the scale
//     factor is folded into the last pass);
//   * use_reorder = false runs strided passes in the input layout, the last
//     pass writing the output box order directly;
//   * use_reorder = true inserts transposes (transpose_unpack kernels) so that
//     every pass runs along the fastest dimension, as reshape3d_transpose does
//     (include/heffte_reshape3d.h:443-487).
#include "gbfft_plan.h"
#include <cmath>

namespace gbfft {

bool valid_order(std::array<int, 3> const &o){
    return (o[0] != o[1] && o[0] != o[2] && o[1] != o[2] &&
            o[0] >= 0 && o[0] < 3 && o[1] >= 0 && o[1] < 3 && o[2] >= 0 && o[2] < 3);
}

Layout pass_layout(Box3 const &box, int dim, std::array<int, 3> const &ref_order){
    int a = -1, b = -1;
    for (int i = 0; i < 3; i++){
        int d = ref_order[i];
        if (d == dim) continue;
        if (a < 0) a = d; else b = d;
    }
    auto s = box.strides();
    Layout L;
    L.count = box.size[a];
    L.dist = s[a];
    L.bstride = s[b];
    L.estride = s[dim];
    return L;
}

static long long batch_count(Box3 const &box, int dim){ return box.count() / box.size[dim]; }

// offsets of buffers inside a workspace are rounded to 32 elements (256
// bytes for complex<float>) so that they keep the workspace's alignment
static long long round32(long long n){ return (n + 31) / 32 * 32; }

// gather / scatter mode of a composite length for a kernel kind
static int line_mode(int kernel_kind, bool dct1){
    switch (kernel_kind){
        case K_R2C: return LM_R2C;
        case K_C2R: return LM_C2R;
        case K_R2R_F: return dct1 ? LM_DCT1 : LM_R2R_F;
        case K_R2R_B: return dct1 ? LM_DCT1 : LM_R2R_B;
        default: return LM_C2C;
    }
}

// ---------------------------------------------------------------------------
// executors
// ---------------------------------------------------------------------------
std::unique_ptr<Executor> make_executor(int kind, Box3 const &box, std::vector<int> const &dims){
    if (box.empty()) return nullptr;
    if (!valid_order(box.order)) throw Error(ST_INVALID, "invalid box order");
    if (dims.empty() || dims.size() > 3) throw Error(ST_INVALID, "executor needs 1 to 3 dimensions");
    if (kind == EX_R2C && dims.size() != 1) throw Error(ST_INVALID, "r2c executor works along one dimension");
    auto e = std::make_unique<Executor>();
    e->kind = kind;
    e->box = box;
    e->dims = dims;
    for (int d : dims){
        if (d < 0 || d > 2) throw Error(ST_INVALID, "invalid dimension");
        int n = (int)box.size[d];
        if (kind == EX_COS1){
            // DCT-I of n values runs on an FFT of length 2(n - 1)
            if (n < 2 || !supported_length(2 * (n - 1), 1))
                throw Error(ST_UNSUPPORTED, "DCT-I length " + std::to_string(n) + " is not supported (needs n >= 2 and "
                            "2(n-1) <= " + std::to_string(max_length(1)) + ")");
            e->ffts.push_back(get_fft1d(2 * (n - 1)));
        } else {
            if (!supported_length(n, 1))
                throw Error(ST_UNSUPPORTED, "transform length " + std::to_string(box.size[d]) + " is outside [1, " +
                            std::to_string(max_length(1)) + "]");
            e->ffts.push_back(get_fft1d(n));
        }
        int mode = (kind == EX_C2C) ? LM_C2C : (kind == EX_R2C ? LM_R2C : (kind == EX_COS1 ? LM_DCT1 : LM_R2R_F));
        e->scratch_elems = std::max(e->scratch_elems, composite_scratch_elems(*e->ffts.back(), mode, batch_count(box, d)));
    }
    return e;
}

Executor::~Executor(){
    if (cached) cudaFree(cached);
}

LaunchCfg Executor::config(int prec, void *work) const{
    LaunchCfg cfg;
    size_t need = (size_t)scratch_elems * ((prec == 0) ? sizeof(float2) : sizeof(double2));
    if (need == 0) return cfg;
    if (!work){
        std::lock_guard<std::mutex> lk(cache_mu);
        if (cached_bytes < need){
            if (cached) check_cuda(cudaFree(cached), "cudaFree(executor workspace)");
            cached = nullptr;
            cached_bytes = 0;
            check_cuda(cudaMalloc(&cached, need), "cudaMalloc(executor workspace)");
            cached_bytes = need;
        }
        work = cached;
    }
    cfg.scratch = work;
    cfg.scratch_bytes = need;
    return cfg;
}

void Executor::forward(cudaStream_t s, int prec, void const *in, void *out, void *work, double scale) const{
    LaunchCfg cfg = config(prec, work);
    if (kind == EX_R2C){
        Box3 cb = box.r2c(dims[0]);
        launch_r2c(s, *ffts[0], prec, pass_layout(box, dims[0], box.order), pass_layout(cb, dims[0], box.order),
                   in, out, batch_count(box, dims[0]), scale, cfg);
        return;
    }
    void const *src = in;
    for (size_t i = 0; i < dims.size(); i++){
        double sc = (i + 1 == dims.size()) ? scale : 1.0;
        Layout L = pass_layout(box, dims[i], box.order);
        long long G = batch_count(box, dims[i]);
        if (kind == EX_C2C) launch_c2c(s, *ffts[i], prec, true, L, L, src, out, G, sc, cfg);
        else if (kind == EX_COS1) launch_dct1(s, *ffts[i], prec, true, (int)box.size[dims[i]], L, L, src, out, G, sc, cfg);
        else launch_r2r(s, *ffts[i], prec, true, kind == EX_SIN, L, L, src, out, G, sc, cfg);
        src = out;
    }
}

void Executor::backward(cudaStream_t s, int prec, void const *in, void *out, void *work, double scale) const{
    LaunchCfg cfg = config(prec, work);
    if (kind == EX_R2C){
        Box3 cb = box.r2c(dims[0]);
        launch_c2r(s, *ffts[0], prec, pass_layout(cb, dims[0], box.order), pass_layout(box, dims[0], box.order),
                   in, out, batch_count(box, dims[0]), scale, cfg);
        return;
    }
    void const *src = in;
    for (size_t i = 0; i < dims.size(); i++){
        double sc = (i + 1 == dims.size()) ? scale : 1.0;
        Layout L = pass_layout(box, dims[i], box.order);
        long long G = batch_count(box, dims[i]);
        if (kind == EX_C2C) launch_c2c(s, *ffts[i], prec, false, L, L, src, out, G, sc, cfg);
        else if (kind == EX_COS1) launch_dct1(s, *ffts[i], prec, false, (int)box.size[dims[i]], L, L, src, out, G, sc, cfg);
        else launch_r2r(s, *ffts[i], prec, false, kind == EX_SIN, L, L, src, out, G, sc, cfg);
        src = out;
    }
}

std::shared_ptr<Fft1D> fft_for(int N, int radix_policy){
    if (radix_policy == 1){
        std::vector<int> r = default_radices(N);
        std::sort(r.begin(), r.end());
        if (!r.empty()) return get_fft1d(N, r);
    }
    return get_fft1d(N);
}

// ---------------------------------------------------------------------------
// plan construction
// ---------------------------------------------------------------------------
namespace {

enum { B_IN = 0, B_OUT = 1, B_WA = 2, B_WB = 3 };

struct PassSpec {
    int kind;      // K_C2C_F ... (kernel kind)
    int dim;
};

std::array<int, 3> order_with_first(std::array<int, 3> const &cur, int d){
    std::array<int, 3> o{d, 0, 0};
    int k = 1;
    for (int i = 0; i < 3; i++) if (cur[i] != d) o[k++] = cur[i];
    return o;
}

// Builds the op list for one direction.
//   passes : the 1-D passes in execution order
//   src_box: input box (with its order), dst_box: output box (with its order)
//   inter  : box geometry of the intermediate (complex for r2c/c2r) data
//   out_holds_inter: the output buffer has the element type of the intermediate data
std::vector<Op> build_ops(std::vector<PassSpec> const &passes, Box3 const &src_box, Box3 const &dst_box,
                          Box3 const &inter_geom, bool reorder, bool out_holds_inter, bool in_aliases_out,
                          int &work_buffers, int radix_policy, bool dct1 = false, bool pad_work = false){
    // drop length-1 complex passes (identity), keep at least one op to move
    // the data; a length-1 r2r transform is not the identity (REDFT10 of one
    // value is twice the value) and r2c/c2r change the element type
    std::vector<PassSpec> ps;
    for (auto const &p : passes){
        bool c2c = (p.kind == K_C2C_F || p.kind == K_C2C_B);
        if (!c2c || inter_geom.size[p.dim] > 1) ps.push_back(p);
    }
    std::vector<Op> ops;
    // logical walk: current box (geometry + order) of the data
    Box3 cur = src_box;
    for (size_t i = 0; i < ps.size(); i++){
        PassSpec const &p = ps[i];
        if (reorder && cur.order[0] != p.dim){
            Op r;
            r.type = Op::RESHAPE;
            r.sbox = cur;
            r.dbox = cur.with_order(order_with_first(cur.order, p.dim));
            ops.push_back(r);
            cur = r.dbox;
        }
        Op f;
        f.type = Op::FFT;
        f.kind = p.kind;
        f.dim = p.dim;
        f.sbox = cur;
        Box3 next = cur;
        if (p.kind == K_R2C){
            next = cur.r2c(p.dim);
        } else if (p.kind == K_C2R){
            next = dst_box.with_order(cur.order);
        }
        f.dbox = next;
        f.ref_order = cur.order;
        int n = (int)((p.kind == K_R2C) ? cur.size[p.dim] : (p.kind == K_C2R ? dst_box.size[p.dim] : cur.size[p.dim]));
        f.fft = fft_for(dct1 ? 2 * (n - 1) : n, radix_policy);
        ops.push_back(f);
        cur = next;
    }
    if (ops.empty()){
        Op c;
        c.type = Op::COPY;
        c.sbox = src_box;
        c.dbox = dst_box;
        ops.push_back(c);
        cur = dst_box;
    }
    // mark the scale carrier: the last FFT (or the copy)
    for (int i = (int)ops.size() - 1; i >= 0; i--){
        if (ops[i].type != Op::RESHAPE){ ops[i].last = true; break; }
    }
    // final layout: the last op writes the output order directly (an FFT
    // pass can write any order); a reorder plan ends with a transpose when
    // its last pass leaves another order.
    bool last_is_fft = ops.back().type != Op::RESHAPE;
    if (reorder && cur.order != dst_box.order){
        Op r;
        r.type = Op::RESHAPE;
        r.sbox = cur;
        r.dbox = cur.with_order(dst_box.order);
        ops.push_back(r);
        last_is_fft = false;
    } else if (last_is_fft){
        ops.back().dbox = ops.back().dbox.with_order(dst_box.order);
    }
    (void)last_is_fft;
    // buffer assignment
    bool has_reshape = false;
    for (auto const &o : ops) has_reshape = has_reshape || (o.type == Op::RESHAPE);
    Op const &first = ops.front();
    bool first_changes_layout = (first.type != Op::FFT) || first.kind == K_R2C || first.kind == K_C2R ||
                                first.sbox.order != first.dbox.order;
    bool orders_kept = true;
    for (auto const &o : ops) orders_kept = orders_kept && (o.sbox.order == o.dbox.order);
    bool x_is_out = !has_reshape && out_holds_inter && orders_kept && !(in_aliases_out && first_changes_layout) &&
                    !pad_work;
    int cur_buf = B_IN;
    int used = 0;
    for (size_t i = 0; i < ops.size(); i++){
        Op &o = ops[i];
        o.src = cur_buf;
        bool final_op = (i + 1 == ops.size());
        if (final_op || (x_is_out && o.type == Op::FFT)){
            o.dst = B_OUT;
        } else if (o.type == Op::FFT && cur_buf != B_IN && o.sbox.order == o.dbox.order){
            o.dst = cur_buf;              // in place
        } else {
            o.dst = (cur_buf == B_WA) ? B_WB : B_WA;
            used = std::max(used, (o.dst == B_WA) ? 1 : 2);
        }
        cur_buf = o.dst;
    }
    work_buffers = used;
    // workspace-resident data with padded rows (padded_pitch): an odd extent
    // of complex<float> rows (e.g. the 257 of a 512-point r2c box) gives row
    // pitches that are not multiples of 16 bytes, which the tensor-memory-
    // access loads of the column passes require
    if (pad_work){
        auto padded = [](Box3 b){ b.pitch0 = padded_pitch(b.size[b.order[0]]); return b; };
        for (auto &o : ops){
            if (o.type != Op::FFT) continue;
            if (o.src == B_WA || o.src == B_WB) o.sbox = padded(o.sbox);
            if (o.dst == B_WA || o.dst == B_WB) o.dbox = padded(o.dbox);
        }
    }
    return ops;
}

} // namespace

std::unique_ptr<Plan3D> make_plan(int kind, Box3 const &inbox, Box3 const &outbox, int r2c_dir, Options const &o,
                                  cudaStream_t stream, Knobs const &knobs){
    if (!valid_order(inbox.order) || !valid_order(outbox.order)) throw Error(ST_INVALID, "invalid box order");
    if (inbox.empty()) throw Error(ST_INVALID, "empty input box");
    auto p = std::make_unique<Plan3D>();
    p->kind = kind;
    p->inbox = inbox;
    p->r2c_dir = r2c_dir;
    p->opts = o;
    p->stream = stream;
    p->knobs = knobs;
    // single rank: the boxes are the whole world (heffte_fft3d.h:270-297 on MPI_COMM_SELF)
    if (kind == PK_R2C){
        if (r2c_dir < 0 || r2c_dir > 2) throw Error(ST_INVALID, "r2c_direction must be 0, 1 or 2");
        Box3 expect = inbox.r2c(r2c_dir);
        if (outbox.lo != expect.lo || outbox.hi != expect.hi)
            throw Error(ST_INVALID, "on one rank the r2c output box must be inbox.r2c(r2c_direction)");
    } else {
        if (outbox.lo != inbox.lo || outbox.hi != inbox.hi)
            throw Error(ST_INVALID, "on one rank the input and output boxes must cover the same indexes");
    }
    p->outbox = outbox;
    for (int d = 0; d < 3; d++){
        int n = (int)inbox.size[d];
        if (kind == PK_COS1){
            if (n < 2 || !supported_length(2 * (n - 1), 1))
                throw Error(ST_UNSUPPORTED, "DCT-I length " + std::to_string(n) + " is not supported (needs n >= 2 and "
                            "2(n-1) <= " + std::to_string(max_length(1)) + ")");
            continue;
        }
        if (!supported_length(n, 1))
            throw Error(ST_UNSUPPORTED, "transform length " + std::to_string(n) + " is outside [1, " +
                        std::to_string(max_length(1)) + "]");
    }
    std::array<int, 3> io = inbox.order, oo = outbox.order;
    bool reorder = o.use_reorder;
    int wf = 0, wb = 0, wfa = 0;
    if (kind == PK_C2C || kind == PK_COS || kind == PK_SIN || kind == PK_COS1){
        bool r2r = (kind != PK_C2C);
        bool dct1 = (kind == PK_COS1);
        std::vector<PassSpec> fwd, bwd;
        for (int i = 0; i < 3; i++) fwd.push_back({r2r ? K_R2R_F : K_C2C_F, io[i]});
        for (int i = 0; i < 3; i++) bwd.push_back({r2r ? K_R2R_B : K_C2C_B, oo[i]});
        p->fwd = build_ops(fwd, inbox, outbox, inbox, reorder, true, false, wf, knobs.radix_policy, dct1);
        p->fwd_alias = p->fwd;
        p->bwd = build_ops(bwd, outbox, inbox, inbox, reorder, true, false, wb, knobs.radix_policy, dct1);
        p->work_buf_elems = inbox.count();
        p->work_elems = std::max(wf, wb) * inbox.count();
        double n = (double)inbox.count();
        // include/heffte_fft3d.h:635-650: 1/(64 N) for the cos/sin tags, 1/(64 prod(n_i - 1)) for DCT-I
        double n1 = (double)(inbox.size[0] - 1) * (double)(inbox.size[1] - 1) * (double)(inbox.size[2] - 1);
        p->scale_factor = dct1 ? 1.0 / (64.0 * n1) : (r2r ? 1.0 / (64.0 * n) : 1.0 / n);
    } else {
        Box3 cgeom = inbox.r2c(r2c_dir);
        // the complex intermediate goes through a padded workspace when its
        // fastest extent is odd (plans without reshapes)
        bool pad_f = !reorder && (cgeom.size[io[0]] % 2 == 1);
        bool pad_b = !reorder && (cgeom.size[oo[0]] % 2 == 1);
        std::vector<PassSpec> fwd{{K_R2C, r2c_dir}}, bwd;
        for (int i = 0; i < 3; i++) if (io[i] != r2c_dir) fwd.push_back({K_C2C_F, io[i]});
        // backward c2c passes: with a padded workspace the slowest dimension
        // goes first, so that the caller's unpadded half spectrum (rows of an
        // odd number of values, not 16-byte aligned) is read by the pass
        // whose batch planes are contiguous, which merges them into one and
        // loads its column tiles by tensor map; the order of the separable
        // passes changes rounding only
        if (pad_b){ for (int i = 2; i >= 0; i--) if (oo[i] != r2c_dir) bwd.push_back({K_C2C_B, oo[i]}); }
        else { for (int i = 0; i < 3; i++) if (oo[i] != r2c_dir) bwd.push_back({K_C2C_B, oo[i]}); }
        bwd.push_back({K_C2R, r2c_dir});
        p->fwd = build_ops(fwd, inbox, outbox, cgeom, reorder, true, false, wf, knobs.radix_policy, false, pad_f);
        p->fwd_alias = build_ops(fwd, inbox, outbox, cgeom, reorder, true, true, wfa, knobs.radix_policy, false, pad_f);
        p->bwd = build_ops(bwd, outbox, inbox, cgeom, reorder, false, false, wb, knobs.radix_policy, false, pad_b);
        long long per = cgeom.count();
        for (auto const *ops : {&p->fwd, &p->fwd_alias, &p->bwd})
            for (auto const &o : *ops){
                if (o.src == B_WA || o.src == B_WB) per = std::max(per, o.sbox.alloc_count());
                if (o.dst == B_WA || o.dst == B_WB) per = std::max(per, o.dbox.alloc_count());
            }
        p->work_buf_elems = per;
        p->work_elems = std::max(std::max(wf, wfa), wb) * per;
        p->scale_factor = 1.0 / (double)inbox.count();
    }
    // composite lengths (four-step, Bluestein) run in a scratch region after
    // the work buffers, sized for the largest batch of lines of any pass
    long long sc = 0;
    for (auto const *ops : {&p->fwd, &p->fwd_alias, &p->bwd})
        for (auto const &op : *ops)
            if (op.type == Op::FFT)
                sc = std::max(sc, composite_scratch_elems(*op.fft, line_mode(op.kind, kind == PK_COS1),
                                                          op.sbox.count() / op.sbox.size[op.dim]));
    if (sc > 0){
        // workspace elements are complex for c2c / r2c plans, real for r2r plans
        long long per_complex = (kind == PK_C2C || kind == PK_R2C) ? 1 : 2;
        p->scratch_elems = sc;
        p->scratch_offset = round32(p->work_elems);
        p->work_elems = p->scratch_offset + per_complex * sc;
    }
    return p;
}

Plan3D::~Plan3D(){
    if (cached_work) cudaFree(cached_work);
    if (conv_cache) cudaFree(conv_cache);
}

double Plan3D::get_scale(int scaling) const{
    if (scaling == 0) return 1.0;
    return (scaling == 2) ? std::sqrt(scale_factor) : scale_factor;
}

static int elem_dtype(int kind, int prec, bool complex_side){
    if (kind == PK_COS || kind == PK_SIN || kind == PK_COS1) return prec == 0 ? DT_FLOAT : DT_DOUBLE;
    if (complex_side) return prec == 0 ? DT_CFLOAT : DT_CDOUBLE;
    return prec == 0 ? DT_FLOAT : DT_DOUBLE;
}

void Plan3D::execute(bool forward, int prec, int batch, void const *in, void *out, void *work, int scaling){
    if (prec != 0 && prec != 1) throw Error(ST_INVALID, "precision must be 0 (single) or 1 (double)");
    if (scaling < 0 || scaling > 2) throw Error(ST_INVALID, "invalid scaling");
    if (batch < 0) throw Error(ST_INVALID, "negative batch size");
    if (batch == 0) return;
    if (!in || !out) throw Error(ST_INVALID, "null input or output pointer");
    // element types on each side
    bool r2c = (kind == PK_R2C);
    int in_dt = elem_dtype(kind, prec, r2c ? !forward : true);
    int out_dt = elem_dtype(kind, prec, r2c ? forward : true);
    int work_dt = elem_dtype(kind, prec, true);
    size_t in_es = elem_size(in_dt), out_es = elem_size(out_dt), work_es = elem_size(work_dt);
    long long in_cnt = forward ? size_inbox() : size_outbox();
    long long out_cnt = forward ? size_outbox() : size_inbox();
    bool alias = (in == out);
    std::vector<Op> const &ops = forward ? (alias ? fwd_alias : fwd) : bwd;
    // the workspace: 2 halves of work_elems/2 ... one box each
    long long per_buf = work_buf_elems;
    size_t need = (size_t)work_elems * work_es;
    char *wbase = reinterpret_cast<char*>(work);
    if (need > 0 && !wbase){
        if (cached_bytes < need){
            if (cached_work) check_cuda(cudaFree(cached_work), "cudaFree(workspace)");
            cached_work = nullptr;
            cached_bytes = 0;
            check_cuda(cudaMalloc(&cached_work, need), "cudaMalloc(workspace)");
            cached_bytes = need;
        }
        wbase = reinterpret_cast<char*>(cached_work);
    }
    double sc = get_scale(scaling);
    LaunchCfg cfg;
    cfg.variant = (knobs.variant == 1) ? 1 : 0;
    cfg.tpb_div = std::max(1, knobs.tile_div);
    cfg.tc = knobs.tensor_cores;
    if (scratch_elems > 0){
        cfg.scratch = wbase + (size_t)scratch_offset * work_es;
        cfg.scratch_bytes = (size_t)scratch_elems * ((prec == 0) ? sizeof(float2) : sizeof(double2));
    }
    for (int j = 0; j < batch; j++){
        void *bufs[4];
        bufs[0] = const_cast<char*>(reinterpret_cast<char const*>(in)) + (size_t)j * in_cnt * in_es;
        bufs[1] = reinterpret_cast<char*>(out) + (size_t)j * out_cnt * out_es;
        bufs[2] = wbase;
        bufs[3] = wbase ? wbase + (size_t)per_buf * work_es : nullptr;
        for (auto const &op : ops){
            void const *src = bufs[op.src];
            void *dst = bufs[op.dst];
            double s = op.last ? sc : 1.0;
            if (op.type == Op::FFT){
                Layout Li = pass_layout(op.sbox, op.dim, op.ref_order);
                Layout Lo = pass_layout(op.dbox, op.dim, op.ref_order);
                long long G = op.sbox.count() / op.sbox.size[op.dim];
                switch (op.kind){
                    case K_C2C_F: launch_c2c(stream, *op.fft, prec, true, Li, Lo, src, dst, G, s, cfg); break;
                    case K_C2C_B: launch_c2c(stream, *op.fft, prec, false, Li, Lo, src, dst, G, s, cfg); break;
                    case K_R2C: launch_r2c(stream, *op.fft, prec, Li, Lo, src, dst, G, s, cfg); break;
                    case K_C2R: launch_c2r(stream, *op.fft, prec, Li, Lo, src, dst, G, s, cfg); break;
                    case K_R2R_F:
                    case K_R2R_B: {
                        bool f = (op.kind == K_R2R_F);
                        if (kind == PK_COS1)
                            launch_dct1(stream, *op.fft, prec, f, (int)op.sbox.size[op.dim], Li, Lo, src, dst, G, s, cfg);
                        else
                            launch_r2r(stream, *op.fft, prec, f, kind == PK_SIN, Li, Lo, src, dst, G, s, cfg);
                        break;
                    }
                }
            } else if (op.type == Op::RESHAPE){
                Box3 const &A = op.sbox, &B = op.dbox;
                int m[3];
                for (int a = 0; a < 3; a++) m[a] = B.find_order(A.order[a]);
                int dt = (op.src == 0) ? in_dt : ((op.dst == 1) ? out_dt : work_dt);
                launch_transpose_unpack(stream, dt, B.osize(0), B.osize(1), B.osize(2), B.osize(0),
                                        B.osize(0) * B.osize(1), A.osize(0), A.osize(0) * A.osize(1),
                                        m[0], m[1], src, dst);
            } else {
                size_t bytes = (size_t)op.dbox.count() * out_es;
                if (src != dst) check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream), "copy");
                if (s != 1.0){
                    long long reals = (long long)(bytes / ((prec == 0) ? 4 : 8));
                    launch_scale(stream, prec, reals, dst, s);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// convolution (benchmarks/convolution.cpp: forward, pointwise product, backward)
// ---------------------------------------------------------------------------
// Fused route (no reshapes, the same order on both sides; r2c plans with the
// r2c along the fastest dimension): the forward passes along two dimensions
// (for r2c: the r2c pass, then a c2c pass on the half spectrum), then ONE
// pass along the third that transforms each column forward, multiplies it by
// y's column (or squares it), scales and transforms it back (gbfft_conv.cuh),
// then the backward passes along the two other dimensions.  Five passes over
// the (half-spectrum) box for a self-convolution where the unfused sequence
// makes six transform passes and a product pass.

// The box the spectra live in: the c2c box itself, or the r2c half spectrum
// with padded rows (padded_pitch), whose column tiles load by tensor map.
Box3 Plan3D::conv_box() const{
    if (kind != PK_R2C) return inbox;
    Box3 b = inbox.r2c(r2c_dir);
    b.pitch0 = padded_pitch(b.size[b.order[0]]);
    return b;
}


long long Plan3D::convolve_workspace() const{
    return round32(work_elems) + 2 * round32(std::max(conv_box().alloc_count(), size_outbox()));
}

int Plan3D::convolve_fused_dim(int prec, void *xb, void const *yb) const{
    if (kind != PK_C2C && kind != PK_R2C) return -1;
    if (opts.use_reorder || inbox.order != outbox.order) return -1;
    if (kind == PK_R2C && r2c_dir != inbox.order[0]) return -1;
    if (!knobs.conv_fused || knobs.tensor_cores || knobs.variant == 1 || knobs.radix_policy != 0) return -1;
    Box3 const B = conv_box();
    for (int d = 0; d < 3; d++) if (B.size[d] < 2) return -1;
    for (int fi : {2, 1}){
        int f = B.order[fi];
        auto ff = get_fft1d((int)B.size[f]);
        if (launch_conv_pass(stream, *ff, prec, pass_layout(B, f, B.order), xb, yb, B.count() / B.size[f], 1.0, true))
            return f;
    }
    return -1;
}

bool Plan3D::convolve_fused(int prec, void const *x, void const *y, void *out, void *w1, void *w2, double scale){
    bool const r2c = (kind == PK_R2C);
    // spectra: c2c in the output (x) and the first workspace box (y);
    // r2c in the two workspace boxes
    void *xb = r2c ? w1 : out;
    void *yb = y ? (r2c ? w2 : w1) : nullptr;
    int f = convolve_fused_dim(prec, xb, yb);
    if (f < 0) return false;
    Box3 const B = conv_box();
    std::array<int, 3> const io = B.order;
    LaunchCfg cfg;
    int rest[2], k = 0;
    for (int i = 0; i < 3; i++) if (io[i] != f) rest[k++] = io[i];
    int const d0 = rest[0], d1 = rest[1];
    auto ff = get_fft1d((int)B.size[f]);
    auto f1 = get_fft1d((int)B.size[d1]);
    auto f0 = get_fft1d((int)inbox.size[d0]);       // the real length for r2c
    Layout const Lf = pass_layout(B, f, io), L1 = pass_layout(B, d1, io);
    Layout const L0c = pass_layout(B, d0, io), L0r = pass_layout(inbox, d0, io);
    long long const Gf = B.count() / B.size[f], G1 = B.count() / B.size[d1], G0 = inbox.count() / inbox.size[d0];
    auto first = [&](void const *src, void *dst){
        if (r2c) launch_r2c(stream, *f0, prec, L0r, L0c, src, dst, G0, 1.0, cfg);
        else launch_c2c(stream, *f0, prec, true, L0c, L0c, src, dst, G0, 1.0, cfg);
    };
    // y first: y may alias out
    if (y){
        first(y, yb);
        launch_c2c(stream, *f1, prec, true, L1, L1, yb, yb, G1, 1.0, cfg);
    }
    first(x, xb);
    launch_c2c(stream, *f1, prec, true, L1, L1, xb, xb, G1, 1.0, cfg);
    if (!launch_conv_pass(stream, *ff, prec, Lf, xb, yb, Gf, scale, false))
        throw Error(ST_CUDA, "fused convolution pass refused after its check passed");
    launch_c2c(stream, *f1, prec, false, L1, L1, xb, xb, G1, 1.0, cfg);
    if (r2c) launch_c2r(stream, *f0, prec, L0c, L0r, xb, out, G0, 1.0, cfg);
    else launch_c2c(stream, *f0, prec, false, L0c, L0c, xb, out, G0, 1.0, cfg);
    return true;
}

void Plan3D::convolve(int prec, void const *x, void const *y, void *out, void *work, int scaling){
    if (prec != 0 && prec != 1) throw Error(ST_INVALID, "precision must be 0 (single) or 1 (double)");
    if (scaling < 0 || scaling > 2) throw Error(ST_INVALID, "invalid scaling");
    if (!x || !out) throw Error(ST_INVALID, "null input or output pointer");
    if (kind != PK_C2C && kind != PK_R2C) throw Error(ST_UNSUPPORTED, "convolution needs a c2c or r2c plan");
    bool self = (y == nullptr || y == x);
    size_t ces = (prec == 0) ? 8 : 16;
    size_t need = (size_t)convolve_workspace() * ces;
    char *w = static_cast<char*>(work);
    if (!w){
        if (conv_cache_bytes < need){
            if (conv_cache) check_cuda(cudaFree(conv_cache), "cudaFree(convolution workspace)");
            conv_cache = nullptr;
            conv_cache_bytes = 0;
            check_cuda(cudaMalloc(&conv_cache, need), "cudaMalloc(convolution workspace)");
            conv_cache_bytes = need;
        }
        w = static_cast<char*>(conv_cache);
    }
    long long const box = round32(std::max(conv_box().alloc_count(), size_outbox()));
    char *w1 = w + (size_t)round32(work_elems) * ces; // spectrum of x
    char *w2 = w1 + (size_t)box * ces;                // spectrum of y
    if (convolve_fused(prec, x, self ? nullptr : y, out, w1, w2, get_scale(scaling))) return;
    // unfused: both forward transforms, the product kernel, the backward
    // transform carrying the scale
    if (!self) execute(true, prec, 1, y, w2, w, 0);
    execute(true, prec, 1, x, w1, w, 0);
    launch_pointwise(stream, prec, size_outbox(), w1, self ? nullptr : w2, 1.0);
    execute(false, prec, 1, w1, out, w, scaling);
}

} // namespace gbfft
