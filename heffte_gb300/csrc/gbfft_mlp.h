// Learned plan selector: MLP with hand-written CUDA training / inference.
#pragma once
#include "gbfft_plan.h"

namespace gbfft {

constexpr int kFeatures = 18;    // plan_features()
constexpr int kCandidates = 16;  // use_reorder x kernel family x tile size x radix order

struct Mlp {
    int nin, nh, nout;
    long long nparams = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr, *loss_d = nullptr;
    float *h1 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr, *dh1 = nullptr, *dh2 = nullptr;
    float *xrow = nullptr;   // one feature row (nin floats) for single-transform selection
    int cap = 0;
    long long step = 0;
    Mlp(int in, int hidden, int out, unsigned long long seed);
    ~Mlp();
    // parameter layout: W1 [in x H], b1 [H], W2 [H x H], b2 [H], W3 [H x out], b3 [out] (row-major)
    long long off_w1() const { return 0; }
    long long off_b1() const { return (long long)nin * nh; }
    long long off_w2() const { return off_b1() + nh; }
    long long off_b2() const { return off_w2() + (long long)nh * nh; }
    long long off_w3() const { return off_b2() + nh; }
    long long off_b3() const { return off_w3() + (long long)nh * nout; }
    void ensure(int B);
    void forward(cudaStream_t s, float const *X, int B);                          // result in y
    void loss_and_grad(cudaStream_t s, float const *X, float const *T, int B);   // loss_d, grads
    float train(cudaStream_t s, float const *X, float const *T, int B, int steps, float lr);
};

// Features of a transform (kFeatures floats).
void plan_features(int kind, int prec, int const size[3], float *f);
// Options / knobs of candidate c in [0, kCandidates).
void candidate_knobs(int c, Options &o, Knobs &kn);

} // namespace gbfft
