// Batches of many small 3-D r2c / c2r transforms of uneven sizes in ONE
// persistent kernel launch, replayed as a CUDA graph.
//
// The work of a batch is a list of "units": one 1-D pass of one box (r2c along
// x, then c2c along y and z; the reverse order backward).  Units are cut into
// tiles and enumerated pass-major; persistent CTAs take tiles from a global
// atomic counter.  A tile of pass p of box b first waits until every tile of
// pass p-1 of box b has completed (a per-unit completion counter).  Because
// tiles are handed out in order, the tiles waited for have already been taken
// by running CTAs, so the wait always ends; it is bounded anyway, and a wait
// that gives up records DEV_TIMEOUT_DEPENDENCY in the device status word.
// Data written by other CTAs is read with L1-bypassing loads (tile_* device
// functions use __ldcg).  Radix plans and tile sizes per transform length come
// from the autotuner when it has measured them (gbfft_tune.cu).
#include "gbfft_batch.h"
#include "gbfft_batch_kernel.cuh"
#include <algorithm>
#include <atomic>
#include <numeric>

namespace gbfft {

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static constexpr int kBatchThreads = 256;

static std::atomic<long long> g_dep_budget{kWaitBudgetClocks};
long long dependency_wait_budget(){ return g_dep_budget.load(); }
void set_dependency_wait_budget(long long clocks){
    if (clocks < 0) throw Error(ST_INVALID, "the wait budget must be >= 0 clocks");
    g_dep_budget.store(clocks);
}

// Test hook: every pass dependency waits for one tile more than its pass has
// (hold = true), so each such wait runs out of its budget; hold = false
// restores the tables.
void Batch::hold_dependencies(bool hold){
    for (int dir = 0; dir < 2; dir++){
        std::vector<BatchUnit> &u = dir == 0 ? h_fwd_units : h_bwd_units;
        for (auto &U : u) U.dep_extra = (hold && U.dep >= 0) ? 1 : 0;
        check_cuda(cudaMemcpy(dir == 0 ? d_fwd_units : d_bwd_units, u.data(), u.size() * sizeof(BatchUnit),
                              cudaMemcpyHostToDevice), "copy units");
    }
}

Batch::~Batch(){
    if (fwd_exec) cudaGraphExecDestroy(fwd_exec);
    if (bwd_exec) cudaGraphExecDestroy(bwd_exec);
    if (fwd_graph) cudaGraphDestroy(fwd_graph);
    if (bwd_graph) cudaGraphDestroy(bwd_graph);
    for (void *p : device_allocs) cudaFree(p);
}

static void const *batch_kernel(int prec, bool fwd, int values, bool r2c, bool s5, bool twt){
    if (values == 8) return batch_kernel_e8(prec, fwd, r2c, s5);
    if (twt) return batch_kernel_e16_r2c5_tw(fwd);
    if (r2c) return s5 ? batch_kernel_e16_r2c5(prec, fwd) : batch_kernel_e16_r2c(prec, fwd);
    return batch_kernel_e16_any(prec, fwd);
}

static int tile_tpb(Plan1D const &P, bool cols, size_t csize, size_t smem_cap, int tune_tpb){
    int const T = P.T, N = P.N;
    int tpb = (tune_tpb > 0) ? tune_tpb : std::max(1, kBatchThreads / T);
    tpb = std::min(tpb, std::max(1, kBatchThreads / T));
    size_t unit = cols ? (size_t)N * csize : (size_t)(N + (N >> 4) + 1) * csize;
    while (tpb > 1 && tpb * unit > smem_cap) tpb--;
    return tpb;
}

// Radix plan of N with radices up to 8 (the 8-values-per-thread kernel):
// radix-8 stages, the remaining power of two as 4 or 4 x 4 (never a radix 2
// beside an 8), then the odd primes; empty when N has a prime factor above 7.
static std::vector<int> radices_upto8(int N){
    std::vector<int> odd;
    int n = N;
    for (int p : {7, 5, 3})
        while (n % p == 0){ odd.push_back(p); n /= p; }
    int a = 0;
    while (n % 2 == 0){ n /= 2; a++; }
    if (n != 1) return {};
    std::vector<int> r;
    int q = a / 3, rem = a % 3;
    if (rem == 1 && q >= 1){ q -= 1; r = {4, 4}; }
    else if (rem == 1) r = {2};
    else if (rem == 2) r = {4};
    for (int i = 0; i < q; i++) r.insert(r.begin(), 8);
    r.insert(r.end(), odd.begin(), odd.end());
    return r;
}

// Threads per transform when each thread holds `values` values: a stage of
// radix R gives each thread values / R butterflies.
static int threads_per_transform(Plan1D const &P, int values){
    int T = 1;
    for (int s = 0; s < P.nstages; s++){
        int per = values / P.st[s].R;
        T = std::max(T, (P.st[s].NR + per - 1) / per);
    }
    return T;
}

std::unique_ptr<Batch> make_batch(int kind, int prec, std::vector<std::array<int, 3>> const &sizes, cudaStream_t stream,
                                  BatchConfig const &config){
    if (kind != PK_R2C && kind != PK_C2C) throw Error(ST_UNSUPPORTED, "batches support c2c and r2c boxes");
    if (prec != 0 && prec != 1) throw Error(ST_INVALID, "precision must be 0 or 1");
    if (sizes.empty()) throw Error(ST_INVALID, "empty batch");
    if (config.prefetch != 0 && config.prefetch != 1) throw Error(ST_INVALID, "prefetch must be 0 or 1");
    if (config.tile_kb < 8 || config.tile_kb > 96) throw Error(ST_INVALID, "tile size must be 8 to 96 KB");
    if (config.group_mb < 0 || config.group_mb > 4096) throw Error(ST_INVALID, "group size must be 0 to 4096 MB");
    if (config.values != 0 && config.values != 8 && config.values != 16)
        throw Error(ST_INVALID, "values per thread must be 0 (automatic), 8 or 16");
    if (config.tuned_plans != 0 && config.tuned_plans != 1) throw Error(ST_INVALID, "tuned_plans must be 0 or 1");
    auto b = std::make_unique<Batch>();
    b->kind = kind; b->prec = prec; b->sizes = sizes; b->stream = stream;
    b->config = config;
    size_t csize = (prec == 0) ? sizeof(float2) : sizeof(double2);
    size_t rsize = csize / 2;
    bool r2c = (kind == PK_R2C);
    long long in_off = 0, out_off = 0;
    for (auto const &s : sizes){
        for (int d = 0; d < 3; d++){
            if (s[d] < 1 || !direct_length(s[d]))
                throw Error(ST_UNSUPPORTED, "box side " + std::to_string(s[d]) + " is not supported in a batch "
                            "(sides up to " + std::to_string(kMaxDirectLength) + " with prime factors 2, 3, 5, 7, 11, 13)");
        }
        long long n = (long long)s[0] * s[1] * s[2];
        long long nc = r2c ? (long long)(s[0] / 2 + 1) * s[1] * s[2] : n;
        b->in_offsets.push_back(in_off);
        b->out_offsets.push_back(out_off);
        in_off += n;
        out_off += nc;
    }
    b->in_total = in_off;
    b->out_total = out_off;
    // distinct lengths -> plan table (tuned radix plans where available)
    std::vector<int> lens;
    for (auto const &s : sizes) for (int d = 0; d < 3; d++) lens.push_back(s[d]);
    std::sort(lens.begin(), lens.end());
    lens.erase(std::unique(lens.begin(), lens.end()), lens.end());
    // 16 values per thread unless 8 are asked for (8: radix plans up to 8,
    // fewer registers but twice the threads per transform; measured slower
    // on 256 uneven r2c boxes, 1.58 against 1.42 ms per forward + backward)
    bool const fits8 = std::all_of(lens.begin(), lens.end(), [](int N){ return N == 1 || !radices_upto8(N).empty(); });
    if (config.values == 8 && !fits8)
        throw Error(ST_UNSUPPORTED, "8 values per thread need box sides with prime factors up to 7");
    int const values = (config.values == 0) ? 16 : config.values;
    b->values = values;
    std::map<int, int> plan_of;
    std::vector<Plan1D> plans;
    std::vector<void const*> tws;
    std::vector<int> tpb_hint;
    for (int N : lens){
        TuneChoice tc = config.tuned_plans ? tuned_choice(N, prec) : TuneChoice{};
        std::vector<int> rad = tc.radices;
        int hint = tc.tpb;
        if (values == 8){
            // a tuned plan only if its radices fit; its tile was timed at 16 values
            bool ok = !rad.empty() && std::all_of(rad.begin(), rad.end(), [](int r){ return r <= 8; });
            if (!ok) rad = (N == 1) ? std::vector<int>{} : radices_upto8(N);
            hint = 0;
        }
        auto f = get_fft1d(N, rad);
        Plan1D P = f->plan;
        P.T = threads_per_transform(P, values);
        plan_of[N] = (int)plans.size();
        plans.push_back(P);
        tws.push_back(f->twiddles(prec, stream));
        b->ffts.push_back(f);
        tpb_hint.push_back(hint);
    }
    // every plan 5-smooth (radices 2, 3, 4, 5, 8, 16): the kernels without
    // the radix-7/11/13 stages
    bool s5 = true;
    for (auto const &P : plans)
        for (int st = 0; st < P.nstages; st++){
            int const R = P.st[st].R;
            s5 = s5 && (R == 2 || R == 3 || R == 4 || R == 5 || R == 8 || R == 16);
        }
    b->s5 = s5;
    size_t smem_cap = (size_t)config.tile_kb * 1024;
    // units: forward = (r2c|c2c x), c2c y, c2c z; backward = c2c z, c2c y, (c2r|c2c x)
    auto build = [&](bool fwd, std::vector<BatchUnit> &units, long long &total){
        std::vector<std::vector<BatchUnit>> per_pass(3);
        for (size_t i = 0; i < sizes.size(); i++){
            auto const &s = sizes[i];
            Box3 rbox({0, 0, 0}, {s[0] - 1, s[1] - 1, s[2] - 1}, {0, 1, 2});
            Box3 cbox = r2c ? rbox.r2c(0) : rbox;
            double sc = 1.0 / (double)rbox.count();
            int order_dims[3] = {0, 1, 2};
            for (int k = 0; k < 3; k++){
                int d = fwd ? order_dims[k] : order_dims[2 - k];
                BatchUnit U{};
                bool first = (k == 0), lastp = (k == 2);
                bool is_r2x = r2c && d == 0;
                U.kind = is_r2x ? (fwd ? K_R2C : K_C2R) : (fwd ? K_C2C_F : K_C2C_B);
                Box3 const &sb = (is_r2x && fwd) ? rbox : cbox;
                Box3 const &db = (is_r2x && !fwd) ? rbox : cbox;
                U.Li = pass_layout(sb, d, {0, 1, 2});
                U.Lo = pass_layout(db, d, {0, 1, 2});
                U.cols = (d != 0);
                U.G = sb.count() / sb.size[d];      // transforms of the box this pass reads
                U.plan = plan_of[(int)rbox.size[d]];
                Fft1D const &f = *b->ffts[U.plan];
                bool paired = is_r2x;
                U.tpb = tile_tpb(plans[U.plan], U.cols, csize, smem_cap, tpb_hint[U.plan]);
                long long units_n = paired ? (U.G + 1) / 2 : U.G;
                U.tiles = (units_n + U.tpb - 1) / U.tpb;
                // buffers: forward input -> output (in place after the first pass);
                // backward input -> workspace -> output (the input is preserved)
                if (fwd){
                    U.src = first ? 0 : 1;
                    U.dst = 1;
                    U.in_off = first ? b->in_offsets[i] : b->out_offsets[i];
                    U.out_off = b->out_offsets[i];
                } else {
                    U.src = first ? 0 : 2;
                    U.dst = lastp ? 1 : 2;
                    U.in_off = b->out_offsets[i];
                    U.out_off = lastp ? b->in_offsets[i] : b->out_offsets[i];
                }
                U.last = lastp ? 1 : 0;
                U.scale = sc;
                // tiles whose input is one span (lines back to back) or rows of
                // adjacent columns can be copied ahead into shared memory
                long long len = (U.kind == K_C2R) ? f.N / 2 + 1 : f.N;
                if (!U.cols)
                    U.pf = U.Li.estride == 1 && U.Li.dist == len && (U.G <= U.Li.count || U.Li.bstride == U.Li.count * len);
                else
                    U.pf = (U.kind == K_C2C_F || U.kind == K_C2C_B) && U.Li.dist == 1;
                per_pass[k].push_back(U);
            }
        }
        units.clear();
        total = 0;
        int nb = (int)sizes.size();
        std::vector<int> pos(3 * nb);      // pos[k * nb + box] = unit index of pass k of box
        auto emit = [&](int k, int i){
            BatchUnit U = per_pass[k][i];
            U.dep = (k == 0) ? -1 : pos[(k - 1) * nb + i];
            U.tile0 = total;
            total += U.tiles;
            pos[k * nb + i] = (int)units.size();
            units.push_back(U);
        };
        // larger boxes first (balances the tail)
        std::vector<int> idx(nb);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int c){ return per_pass[0][a].tiles > per_pass[0][c].tiles; });
        if (config.group_mb <= 0){
            // pass-major: pass 0 of every box, then pass 1, then pass 2
            for (int k = 0; k < 3; k++)
                for (int i : idx) emit(k, i);
        } else {
            // groups of boxes of about group_mb MB of spectrum each, in a
            // three-step software pipeline: step s queues pass 2 of group s-2,
            // pass 1 of group s-1 and pass 0 of group s, so a box's data is
            // read again by its next pass about two groups' worth of work
            // later, while it is still in L2 (every unit still comes after
            // the unit it depends on)
            std::vector<std::vector<int>> groups(1);
            long long const cap = (long long)config.group_mb << 20;
            long long acc = 0;
            for (int i : idx){
                auto const &sz = sizes[i];
                long long bytes = (long long)(r2c ? sz[0] / 2 + 1 : sz[0]) * sz[1] * sz[2] * (long long)csize;
                if (!groups.back().empty() && acc + bytes > cap){ groups.emplace_back(); acc = 0; }
                groups.back().push_back(i);
                acc += bytes;
            }
            int const ng = (int)groups.size();
            for (int st = 0; st < ng + 2; st++)
                for (int k = 2; k >= 0; k--){
                    int g = st - k;
                    if (g < 0 || g >= ng) continue;
                    for (int i : groups[g]) emit(k, i);
                }
        }
    };
    std::vector<BatchUnit> fu, bu;
    build(true, fu, b->fwd_tiles);
    build(false, bu, b->bwd_tiles);
    // every element a unit touches must lie inside its buffer (checked on the host)
    auto last_elem = [](Layout const &L, long long G, long long N){
        long long blocks = (G + L.count - 1) / L.count;
        return (blocks - 1) * L.bstride + (std::min(G, L.count) - 1) * L.dist + (N - 1) * L.estride;
    };
    for (auto const *v : {&fu, &bu}){
        bool fwd = (v == &fu);
        // a unit waits only for units queued before it (no CTA can wait on a
        // tile that no CTA has claimed yet)
        for (size_t j = 0; j < v->size(); j++){
            if ((*v)[j].dep >= (int)j) throw Error(ST_INVALID, "internal error: batch unit queued before its dependency");
            // the kernels run r2c / c2r units as line tiles only (they are the
            // x passes), and those of r2c batches their c2c units as column tiles
            if (((*v)[j].kind == K_R2C || (*v)[j].kind == K_C2R) && (*v)[j].cols)
                throw Error(ST_INVALID, "internal error: r2c batch unit along a strided dimension");
            if (kind == PK_R2C && ((*v)[j].kind == K_C2C_F || (*v)[j].kind == K_C2C_B) && !(*v)[j].cols)
                throw Error(ST_INVALID, "internal error: c2c unit of an r2c batch along x");
            if (kind == PK_C2C && ((*v)[j].kind == K_R2C || (*v)[j].kind == K_C2R))
                throw Error(ST_INVALID, "internal error: r2c unit in a c2c batch");
        }
        for (auto const &U : *v){
            long long N = b->ffts[U.plan]->N;
            // forward: input (in_total) -> output (out_total); backward: input
            // and workspace hold half spectra (out_total), the output the boxes (in_total)
            long long in_cap = (fwd && U.src == 0) ? b->in_total : b->out_total;
            long long out_cap = (!fwd && U.dst == 1) ? b->in_total : b->out_total;
            long long in_len = (U.kind == K_C2R) ? N / 2 + 1 : N;
            long long out_len = (U.kind == K_R2C) ? N / 2 + 1 : N;
            if (U.in_off + last_elem(U.Li, U.G, in_len) >= in_cap || U.out_off + last_elem(U.Lo, U.G, out_len) >= out_cap)
                throw Error(ST_INVALID, "internal error: batch unit exceeds its buffer");
        }
    }
    b->nunits = (int)fu.size();
    b->h_fwd_units = fu;
    b->h_bwd_units = bu;
    // device tables
    auto dalloc = [&](size_t bytes) -> void* {
        void *p = nullptr;
        check_cuda(cudaMalloc(&p, std::max<size_t>(bytes, 16)), "cudaMalloc(batch tables)");
        b->device_allocs.push_back(p);
        return p;
    };
    b->d_fwd_units = dalloc(fu.size() * sizeof(BatchUnit));
    b->d_bwd_units = dalloc(bu.size() * sizeof(BatchUnit));
    b->d_plans = dalloc(plans.size() * sizeof(Plan1D));
    b->d_tws = dalloc(tws.size() * sizeof(void*));
    b->d_counters = dalloc(sizeof(unsigned long long) + fu.size() * sizeof(int));
    check_cuda(cudaMemcpy(b->d_fwd_units, fu.data(), fu.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice), "copy units");
    check_cuda(cudaMemcpy(b->d_bwd_units, bu.data(), bu.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice), "copy units");
    check_cuda(cudaMemcpy(b->d_plans, plans.data(), plans.size() * sizeof(Plan1D), cudaMemcpyHostToDevice), "copy plans");
    check_cuda(cudaMemcpy(b->d_tws, tws.data(), tws.size() * sizeof(void*), cudaMemcpyHostToDevice), "copy twiddle table");
    // launch geometry: persistent CTAs, as many as fit
    size_t smem = 0;
    for (auto const *v : {&fu, &bu})
        for (auto const &U : *v){
            Fft1D const &f = *b->ffts[U.plan];
            size_t unit = U.cols ? (size_t)f.N * csize : (size_t)(f.N + (f.N >> 4) + 1) * csize;
            smem = std::max(smem, unit * U.tpb);
        }
    // the prefetch buffer: the largest tile input of the units that can prefetch
    size_t pf_bytes = 0;
    for (auto const *v : {&fu, &bu})
        for (auto const &U : *v){
            if (!U.pf) continue;
            Fft1D const &f = *b->ffts[U.plan];
            size_t es = (U.kind == K_R2C) ? rsize : csize;
            size_t per = (U.kind == K_R2C || U.kind == K_C2R) ? 2 : 1;
            size_t len = (U.kind == K_C2R) ? f.N / 2 + 1 : f.N;
            pf_bytes = std::max(pf_bytes, U.cols ? (size_t)f.N * U.tpb * es : (size_t)U.tpb * per * len * es);
        }
    smem = (smem + 15) / 16 * 16;
    b->pf_offset = (config.prefetch && pf_bytes > 0) ? (int)smem : -1;
    if (b->pf_offset > 0) smem += (pf_bytes + 15) / 16 * 16;
    // the twiddle tables of all plans in shared memory (the float r2c kernel
    // of 5-smooth plans with 16 values per thread), when they are few and small
    size_t tw_total = 0;
    for (Plan1D const &P : plans)
        for (int s = 1; s < P.nstages; s++) tw_total += (size_t)P.st[s].Ns * (P.st[s].R - 1);
    bool const twt = prec == 0 && values == 16 && kind == PK_R2C && s5 && (int)plans.size() <= kBatchTwPlans &&
                     tw_total * csize <= 24 * 1024;
    b->nplans = (int)plans.size();
    b->tw_off = twt ? (int)smem : -1;
    if (twt) smem += (tw_total * csize + 15) / 16 * 16;
    b->smem = smem;
    for (bool fwd : {true, false}){
        void const *kern = batch_kernel(prec, fwd, values, kind == PK_R2C, s5, b->tw_off > 0);
        int nb_sm = 1;
        check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_sm, kern, kBatchThreads, smem), "occupancy");
        (fwd ? b->grid : b->grid_bwd) = std::max(1, nb_sm) * num_sms();
    }
    return b;
}

// Builds (once) the graph of one direction: reset the counters, run the kernel.
static void build_graph(Batch &b, bool fwd){
    cudaGraph_t &g = fwd ? b.fwd_graph : b.bwd_graph;
    cudaGraphExec_t &e = fwd ? b.fwd_exec : b.bwd_exec;
    check_cuda(cudaGraphCreate(&g, 0), "cudaGraphCreate");
    cudaMemsetParams ms{};
    ms.dst = b.d_counters;
    ms.value = 0;
    ms.elementSize = 1;
    ms.width = sizeof(unsigned long long) + (size_t)b.nunits * sizeof(int);
    ms.height = 1;
    cudaGraphNode_t mnode, knode;
    check_cuda(cudaGraphAddMemsetNode(&mnode, g, nullptr, 0, &ms), "cudaGraphAddMemsetNode");
    b.args_units = fwd ? b.d_fwd_units : b.d_bwd_units;
    b.args_nunits = b.nunits;
    b.args_plans = b.d_plans;
    b.args_tws = b.d_tws;
    b.args_bufs = BatchBufs{nullptr, nullptr, nullptr};
    b.args_counter = reinterpret_cast<unsigned long long*>(b.d_counters);
    b.args_done = reinterpret_cast<int*>(reinterpret_cast<char*>(b.d_counters) + sizeof(unsigned long long));
    b.args_total = fwd ? b.fwd_tiles : b.bwd_tiles;
    b.args_status = device_status();
    b.args_scaling = 0;
    b.args_budget = dependency_wait_budget();
    void *args[] = {&b.args_units, &b.args_nunits, &b.args_plans, &b.args_tws, &b.args_bufs, &b.args_counter,
                    &b.args_done, &b.args_total, &b.args_status, &b.args_scaling, &b.args_budget, &b.pf_offset,
                    &b.nplans, &b.tw_off};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(batch_kernel(b.prec, fwd, b.values, b.kind == PK_R2C, b.s5, b.tw_off > 0));
    kp.gridDim = dim3((unsigned)(fwd ? b.grid : b.grid_bwd));
    kp.blockDim = dim3(kBatchThreads);
    kp.sharedMemBytes = (unsigned)b.smem;
    kp.kernelParams = args;
    check_cuda(cudaGraphAddKernelNode(&knode, g, &mnode, 1, &kp), "cudaGraphAddKernelNode");
    check_cuda(cudaGraphInstantiate(&e, g, 0), "cudaGraphInstantiate");
    (fwd ? b.fwd_knode : b.bwd_knode) = knode;
}

// Times forward + backward of every launch shape (the tuned radix plans or
// the default ones, 16 or 8 values per thread, queue order pass-major or in
// groups of 16 MB, prefetch on / off, tile bounds of 48, 32 and 24 KB: 2 to 5
// CTAs per SM) on the caller's buffers
// and leaves `b` built with the fastest; the untuned default is a candidate,
// so tuning never makes the batch slower than it was (within the timing noise).
BatchConfig autotune_batch(std::unique_ptr<Batch> &b, void const *in, void *out, void *back, void *work, int reps,
                           double *best_ms){
    if (!in || !out || !back || !work) throw Error(ST_INVALID, "null pointer");
    reps = std::max(reps, 1);
    Batch const &B0 = *b;
    int const kind = B0.kind, prec = B0.prec;
    std::vector<std::array<int, 3>> const sizes = B0.sizes;
    cudaStream_t const s = B0.stream;
    BatchConfig best = B0.config;
    double best_t = 1e300;
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
    check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
    std::vector<BatchConfig> shapes;
    for (int tp : {1, 0})
        for (int vals : {16, 8})
            for (int gm : {0, 16})
                for (int pf : {0, 1})
                    for (int kb : {48, 32, 24}){
                        BatchConfig c;
                        c.prefetch = pf;
                        c.tile_kb = kb;
                        c.group_mb = gm;
                        c.values = vals;
                        c.tuned_plans = tp;
                        shapes.push_back(c);
                    }
    {
        for (BatchConfig const &c : shapes){
            std::unique_ptr<Batch> cand;
            try {
                cand = make_batch(kind, prec, sizes, s, c);
            } catch (Error const &e){
                if (e.code == ST_UNSUPPORTED && c.values == 8) continue;     // sides with factors above 7
                throw;
            }
            for (int i = 0; i < 2; i++){
                cand->run(true, in, out, nullptr, 0);
                cand->run(false, out, back, work, 0);
            }
            check_cuda(cudaEventRecord(e0, s), "cudaEventRecord");
            for (int i = 0; i < reps; i++){
                cand->run(true, in, out, nullptr, 0);
                cand->run(false, out, back, work, 0);
            }
            check_cuda(cudaEventRecord(e1, s), "cudaEventRecord");
            check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0.f;
            check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            double t = ms / reps;
            if (t < best_t){ best_t = t; best = c; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b = make_batch(kind, prec, sizes, s, best);
    if (best_ms) *best_ms = best_t;
    return best;
}

void Batch::run(bool fwd, void const *in, void *out, void *work, int scaling){
    if (!in || !out) throw Error(ST_INVALID, "null pointer");
    if (scaling < 0 || scaling > 2) throw Error(ST_INVALID, "invalid scaling");
    if (!fwd && !work) throw Error(ST_INVALID, "the backward batch needs a workspace of size_workspace() elements");
    cudaGraphExec_t &e = fwd ? fwd_exec : bwd_exec;
    if (!e) build_graph(*this, fwd);
    // point the kernel node at this call's buffers
    args_units = fwd ? d_fwd_units : d_bwd_units;
    args_nunits = nunits;
    args_plans = d_plans;
    args_tws = d_tws;
    args_bufs = BatchBufs{in, out, work};
    args_counter = reinterpret_cast<unsigned long long*>(d_counters);
    args_done = reinterpret_cast<int*>(reinterpret_cast<char*>(d_counters) + sizeof(unsigned long long));
    args_total = fwd ? fwd_tiles : bwd_tiles;
    args_status = device_status();
    args_scaling = scaling;
    args_budget = dependency_wait_budget();
    void *args[] = {&args_units, &args_nunits, &args_plans, &args_tws, &args_bufs, &args_counter, &args_done,
                    &args_total, &args_status, &args_scaling, &args_budget, &pf_offset, &nplans, &tw_off};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(batch_kernel(prec, fwd, values, kind == PK_R2C, s5, tw_off > 0));
    kp.gridDim = dim3((unsigned)(fwd ? grid : grid_bwd));
    kp.blockDim = dim3(kBatchThreads);
    kp.sharedMemBytes = (unsigned)smem;
    kp.kernelParams = args;
    check_cuda(cudaGraphExecKernelNodeSetParams(e, fwd ? fwd_knode : bwd_knode, &kp), "cudaGraphExecKernelNodeSetParams");
    check_cuda(cudaGraphLaunch(e, stream), "cudaGraphLaunch");
}

} // namespace gbfft
