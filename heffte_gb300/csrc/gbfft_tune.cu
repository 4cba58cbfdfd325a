// Autotuner of the per-length radix plan and tile size of the generic
// (runtime-radix) kernels, used by the batched multi-box path.
//
// For a length N every candidate radix plan (ordered factorisations into the
// supported radices, at most four stages) is timed with CUDA events inside the
// batched kernel itself (a batch of N^3 boxes, r2c forward + backward, the
// tile of 256 threads / T transforms that kernel uses); the fastest is kept.
// Results live
// in a process-wide table and, when a cache path is given, are appended to a
// tab-separated file after every length, keyed by the device (name, SM count,
// driver and library versions): a later run loads the file and skips what was
// measured, so an interrupted tuning resumes where it stopped.
#include "gbfft_batch.h"
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <sstream>

namespace gbfft {

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, TuneChoice> g_table;   // (prec, N) -> choice
}

std::string device_key(){
    int dev = 0, drv = 0;
    cudaDeviceProp p{};
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaGetDeviceProperties(&p, dev), "cudaGetDeviceProperties");
    cudaDriverGetVersion(&drv);
    std::ostringstream os;
    os << p.name << "|sm" << p.major << p.minor << "x" << p.multiProcessorCount << "|drv" << drv << "|lib10000";
    std::string s = os.str();
    for (char &c : s) if (c == '\t' || c == '\n') c = ' ';
    return s;
}

TuneChoice tuned_choice(int N, int prec){
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find({prec, N});
    return (it == g_table.end()) ? TuneChoice{} : it->second;
}

void tune_clear(){
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.clear();
}

static void gen(int n, int max_r, std::vector<int> &cur, std::vector<std::vector<int>> &out){
    if (n == 1){ if (!cur.empty()) out.push_back(cur); return; }
    if (cur.size() >= 4) return;
    static const int radices[] = {16, 13, 11, 8, 7, 5, 4, 3, 2};
    for (int r : radices){
        if (r > max_r || n % r) continue;
        cur.push_back(r);
        gen(n / r, r, cur, out);
        cur.pop_back();
    }
}

std::vector<std::vector<int>> radix_candidates(int N){
    std::vector<std::vector<int>> sets, out;
    std::vector<int> cur;
    gen(N, 16, cur, sets);
    std::vector<int> def = default_radices(N);
    if (!def.empty()) out.push_back(def);
    // fewer stages first; each multiset in descending and ascending order
    std::stable_sort(sets.begin(), sets.end(), [](auto const &a, auto const &b){ return a.size() < b.size(); });
    for (auto const &s : sets){
        std::vector<int> asc(s.rbegin(), s.rend());
        std::vector<int> const *both[2] = {&s, &asc};
        for (auto const *v : both){
            bool dup = false;
            for (auto const &o : out) dup = dup || (o == *v);
            if (!dup) out.push_back(*v);
        }
        if (out.size() >= 10) break;
    }
    return out;
}

int tune_load(std::string const &path){
    std::ifstream f(path);
    if (!f) return 0;
    std::string key = device_key(), line;
    int n = 0;
    std::lock_guard<std::mutex> lk(g_mu);
    while (std::getline(f, line)){
        std::istringstream is(line);
        std::string k, rad;
        int prec, N, tpb;
        double us;
        if (!std::getline(is, k, '\t')) continue;
        if (k != key) continue;
        if (!(is >> prec >> N >> rad >> tpb >> us)) continue;
        TuneChoice c;
        std::istringstream rs(rad);
        std::string tok;
        while (std::getline(rs, tok, ',')) if (!tok.empty()) c.radices.push_back(std::stoi(tok));
        c.tpb = tpb;
        c.us = us;
        g_table[{prec, N}] = c;
        n++;
    }
    return n;
}

// Times one candidate inside the batched kernel it is tuned for: a batch of
// boxes whose three sides are all N (the batch reads the candidate from the
// table), r2c forward + backward, at `values` values per thread.
static double time_in_batch(cudaStream_t s, int N, int prec, void *in, void *out, void *work, int nbox, int values){
    std::vector<std::array<int, 3>> sizes(nbox, std::array<int, 3>{N, N, N});
    BatchConfig c;
    c.values = values;
    auto b = make_batch(PK_R2C, prec, sizes, s, c);
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    auto once = [&]{ b->run(true, in, out, nullptr, 0); b->run(false, out, in, work, 0); };
    once();
    once();
    const int reps = 5;
    check_cuda(cudaEventRecord(e0, s), "event record");
    for (int r = 0; r < reps; r++) once();
    check_cuda(cudaEventRecord(e1, s), "event record");
    check_cuda(cudaEventSynchronize(e1), "event sync");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 1e3 * ms / reps;
}

int tune_lengths(std::vector<int> const &lengths, int prec, cudaStream_t s, std::string const &cache_path){
    if (!cache_path.empty()) tune_load(cache_path);
    std::string key = device_key();
    int measured = 0;
    size_t csize = (prec == 0) ? sizeof(float2) : sizeof(double2);
    for (int N : lengths){
        {
            std::lock_guard<std::mutex> lk(g_mu);
            if (g_table.count({prec, N})) continue;
        }
        if (!direct_length(N) || N < 2) continue;
        // boxes of N^3, enough of them for about 2^24 values per batch
        long long per = (long long)N * N * N;
        int nbox = (int)std::max<long long>(1, std::min<long long>(64, (1LL << 24) / per));
        size_t elems = (size_t)per * nbox;
        void *in = nullptr, *out = nullptr, *work = nullptr;
        check_cuda(cudaMalloc(&in, elems * csize), "cudaMalloc(tuning buffer)");
        check_cuda(cudaMalloc(&out, elems * csize), "cudaMalloc(tuning buffer)");
        check_cuda(cudaMalloc(&work, elems * csize), "cudaMalloc(tuning buffer)");
        check_cuda(cudaMemsetAsync(in, 0, elems * csize, s), "memset");
        TuneChoice best;
        best.us = 1e30;
        for (auto const &rad : radix_candidates(N)){
            std::shared_ptr<Fft1D> f;
            try { f = get_fft1d(N, rad); } catch (Error const &){ continue; }
            if (f->plan.T > 256) continue;
            int deft = std::max(1, 256 / f->plan.T);
            {
                std::lock_guard<std::mutex> lk(g_mu);
                g_table[{prec, N}] = TuneChoice{rad, deft, 0};
            }
            double us = time_in_batch(s, N, prec, in, out, work, nbox, 16);
            if (us < best.us){ best.us = us; best.radices = rad; best.tpb = deft; }
        }
        cudaFree(in);
        cudaFree(out);
        cudaFree(work);
        {
            std::lock_guard<std::mutex> lk(g_mu);
            g_table[{prec, N}] = best;
        }
        measured++;
        if (!cache_path.empty()){
            std::ofstream f(cache_path, std::ios::app);
            f << key << '\t' << prec << ' ' << N << ' ';
            for (size_t i = 0; i < best.radices.size(); i++) f << (i ? "," : "") << best.radices[i];
            f << ' ' << best.tpb << ' ' << best.us << '\n';
        }
    }
    return measured;
}

} // namespace gbfft
