// Batched multi-box transforms and the per-length autotuner.
#pragma once
#include "gbfft_plan.h"
#include <map>
#include <string>

namespace gbfft {

// ---------------------------------------------------------------------------
// autotuner (gbfft_tune.cu)
// ---------------------------------------------------------------------------
struct TuneChoice {
    std::vector<int> radices;   // empty: default plan
    int tpb = 0;                // transforms per tile of the generic kernels, 0: default
    double us = 0;              // measured time of the choice (lines + columns probe)
};

// Choice for a length, from the tuning table (empty when never measured).
TuneChoice tuned_choice(int N, int prec);
// Candidate radix plans of a length (the default plan first).
std::vector<std::vector<int>> radix_candidates(int N);
// Measures every candidate of every length on the current device and keeps
// the fastest; results are appended to `cache_path` (if not empty) after each
// length, so an interrupted run resumes where it stopped.  Returns the number
// of lengths measured (lengths already in the table are skipped).
int tune_lengths(std::vector<int> const &lengths, int prec, cudaStream_t s, std::string const &cache_path);
// Loads a cache written by tune_lengths for this device; returns entries read.
int tune_load(std::string const &cache_path);
void tune_clear();
std::string device_key();

// ---------------------------------------------------------------------------
// batch of boxes (gbfft_batch.cu)
// ---------------------------------------------------------------------------
struct BatchBufs { void const *in; void *out; void *work; };
// Launch shape of a batch: prefetch = 1 copies each CTA's next tile into
// shared memory while it transforms the current one (when the next tile's
// pass dependency is already met); tile_kb bounds the shared memory of one
// tile's exchange buffer (smaller tiles: more CTAs per SM); group_mb > 0
// queues the boxes in groups of about that many MB of spectrum, each group's
// passes two groups apart (its data stays in L2 between them), 0 queues
// pass 0 of every box, then pass 1, then pass 2; values: complex values each
// thread holds (8: radix plans up to 8, fewer registers, box sides with prime
// factors up to 7; 16 or 0: any plan).
struct BatchConfig {
    int prefetch = 0;
    int tile_kb = 48;
    int group_mb = 0;
    int values = 0;
    int tuned_plans = 1;    // radix plans from the tuning table (1) or the defaults (0)
};
struct BatchUnit;   // one 1-D pass of one box (gbfft_batch.cu)

struct Batch {
    int kind = PK_R2C;
    int prec = 0;
    std::vector<std::array<int, 3>> sizes;
    cudaStream_t stream = nullptr;
    std::vector<long long> in_offsets, out_offsets;
    long long in_total = 0, out_total = 0;
    std::vector<std::shared_ptr<Fft1D>> ffts;
    std::vector<void*> device_allocs;
    void *d_fwd_units = nullptr, *d_bwd_units = nullptr, *d_plans = nullptr, *d_tws = nullptr, *d_counters = nullptr;
    int nunits = 0;
    long long fwd_tiles = 0, bwd_tiles = 0;
    size_t smem = 0;
    BatchConfig config;
    int pf_offset = -1;    // byte offset of the prefetch buffer in dynamic shared memory (-1: none)
    int values = 16;       // complex values per thread of the kernel in use (8 or 16)
    bool s5 = false;       // every radix plan 5-smooth (the kernels without radix 7, 11, 13)
    int tw_off = -1;       // byte offset of the twiddle tables in dynamic shared memory (-1: read from global memory)
    int nplans = 0;        // radix plans of the batch (entries of the plan and twiddle tables)
    int grid = 0;          // persistent CTAs of the forward kernel
    int grid_bwd = 0;      // and of the backward kernel
    cudaGraph_t fwd_graph = nullptr, bwd_graph = nullptr;
    cudaGraphExec_t fwd_exec = nullptr, bwd_exec = nullptr;
    cudaGraphNode_t fwd_knode = nullptr, bwd_knode = nullptr;
    // kernel-node arguments (the graph node points at these)
    void *args_units = nullptr;
    int args_nunits = 0;
    void *args_plans = nullptr, *args_tws = nullptr;
    BatchBufs args_bufs{};
    unsigned long long *args_counter = nullptr;
    int *args_done = nullptr;
    long long args_total = 0;
    int *args_status = nullptr;
    int args_scaling = 0;
    long long args_budget = 0;
    // host copies of the unit tables (their layout is private to gbfft_batch.cu)
    std::vector<BatchUnit> h_fwd_units, h_bwd_units;
    ~Batch();
    void hold_dependencies(bool hold);
    long long workspace_elems() const { return out_total; }
    void run(bool fwd, void const *in, void *out, void *work, int scaling);
};

// Times the launch shapes of a batch on the caller's buffers (input ->
// output forward, output -> back backward with work) and rebuilds `b` with
// the fastest; returns it (and its ms per forward + backward).
BatchConfig autotune_batch(std::unique_ptr<Batch> &b, void const *in, void *out, void *back, void *work, int reps,
                           double *best_ms);

// Clock budget of the batch kernel's waits for another CTA's pass of the same
// box (default kWaitBudgetClocks); read at every launch.
long long dependency_wait_budget();
void set_dependency_wait_budget(long long clocks);

std::unique_ptr<Batch> make_batch(int kind, int prec, std::vector<std::array<int, 3>> const &sizes, cudaStream_t stream,
                                  BatchConfig const &config = BatchConfig{});

} // namespace gbfft
