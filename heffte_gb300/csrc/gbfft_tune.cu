// Autotuner of the per-length radix plan and tile size of the generic
// (runtime-radix) kernels, used by the batched multi-box path.
//
// For a length N every candidate radix plan (ordered factorisations into the
// supported radices, at most four stages) and two tile sizes are timed with
// CUDA events on two probes that stand for the two pass shapes of a box
// (contiguous lines and strided columns); the fastest is kept.  Results live
// in a process-wide table and, when a cache path is given, are appended to a
// tab-separated file after every length, keyed by the device (name, SM count,
// driver and library versions): a later run loads the file and skips what was
// measured, so an interrupted tuning resumes where it stopped.
#include "gbfft_batch.h"
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

static double time_candidate(cudaStream_t s, Fft1D &f, int prec, int tpb, void *buf, void *buf2, long long G){
    Layout lines{G, f.N, (long long)G * f.N, 1};
    Layout cols{G, 1, (long long)G, G};
    LaunchCfg cfg;
    cfg.variant = 1;
    cfg.tpb = tpb;
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    auto once = [&]{
        launch_c2c(s, f, prec, true, lines, lines, buf, buf2, G, 1.0, cfg);
        launch_c2c(s, f, prec, true, cols, cols, buf2, buf, G, 1.0, cfg);
    };
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
        if (!supported_length(N, prec) || N < 2) continue;
        long long G = std::max<long long>(256, (1LL << 21) / N);
        void *buf = nullptr, *buf2 = nullptr;
        check_cuda(cudaMalloc(&buf, (size_t)G * N * csize), "cudaMalloc(tuning buffer)");
        check_cuda(cudaMalloc(&buf2, (size_t)G * N * csize), "cudaMalloc(tuning buffer)");
        check_cuda(cudaMemsetAsync(buf, 0, (size_t)G * N * csize, s), "memset");
        TuneChoice best;
        best.us = 1e30;
        for (auto const &rad : radix_candidates(N)){
            std::shared_ptr<Fft1D> f;
            try { f = get_fft1d(N, rad); } catch (Error const &){ continue; }
            if (f->plan.T > 512) continue;
            int deft = std::max(1, 256 / f->plan.T);
            for (int tpb : {deft, std::max(1, deft / 2)}){
                double us = time_candidate(s, *f, prec, tpb, buf, buf2, G);
                if (us < best.us){ best.us = us; best.radices = rad; best.tpb = tpb; }
            }
        }
        cudaFree(buf);
        cudaFree(buf2);
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
