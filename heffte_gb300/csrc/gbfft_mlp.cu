// Learned plan selection: a 3-layer MLP (in -> H -> H -> out, ReLU) trained
// on the GPU by hand-written forward, backward and Adam kernels, FP32.
//
// The network maps the features of a transform (sizes, kind, precision,
// factor structure; plan_features below) to the predicted log2 slow-down of
// each candidate plan relative to the best one; the selector picks the
// candidate with the smallest prediction.  The candidates are the 16
// combinations of use_reorder x kernel family x tile size x radix order.
#include "gbfft_plan.h"
#include "gbfft_mlp.h"
#include <cmath>
#include <random>

namespace gbfft {

// ---------------------------------------------------------------------------
// kernels (sizes are tiny: one thread per output element, loops over K / B)
// ---------------------------------------------------------------------------
// Y[B x N] = act(X[B x K] W[K x N] + b[N])
__global__ void k_dense_fwd(float const *__restrict__ X, float const *__restrict__ W, float const *__restrict__ b,
                            float *__restrict__ Y, int B, int K, int N, int relu){
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * N) return;
    int r = i / N, c = i % N;
    float acc = b[c];
    for (int k = 0; k < K; k++) acc = fmaf(X[r * K + k], W[k * N + c], acc);
    Y[i] = (relu && acc < 0.f) ? 0.f : acc;
}

// dY = 2 (Y - T) / (B N); loss accumulates sum (Y - T)^2 / (B N)
__global__ void k_mse(float const *__restrict__ Y, float const *__restrict__ T, float *__restrict__ dY,
                      float *__restrict__ loss, int n){
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.f;
    if (i < n){
        d = Y[i] - T[i];
        dY[i] = 2.f * d / (float)n;
    }
    // warp reduction of the squared error, one atomic per warp
    float sq = d * d / (float)n;
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, sq);
}

// dW[K x N] = X^T dY, db[N] = sum_rows dY
__global__ void k_dense_bwd_w(float const *__restrict__ X, float const *__restrict__ dY, float *__restrict__ dW,
                              float *__restrict__ db, int B, int K, int N){
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < K * N){
        int k = i / N, c = i % N;
        float acc = 0.f;
        for (int r = 0; r < B; r++) acc = fmaf(X[r * K + k], dY[r * N + c], acc);
        dW[i] = acc;
    } else if (i < K * N + N){
        int c = i - K * N;
        float acc = 0.f;
        for (int r = 0; r < B; r++) acc += dY[r * N + c];
        db[c] = acc;
    }
}

// dX[B x K] = (dY W^T) * relu'(X)   (X: the ReLU output feeding this layer)
__global__ void k_dense_bwd_x(float const *__restrict__ dY, float const *__restrict__ W, float const *__restrict__ X,
                              float *__restrict__ dX, int B, int K, int N){
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * K) return;
    int r = i / K, k = i % K;
    float acc = 0.f;
    for (int c = 0; c < N; c++) acc = fmaf(dY[r * N + c], W[k * N + c], acc);
    dX[i] = (X[i] > 0.f) ? acc : 0.f;
}

__global__ void k_adam(float *__restrict__ p, float const *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2){
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

static unsigned blocks_for(long long n){ return (unsigned)((n + 255) / 256); }

// ---------------------------------------------------------------------------
Mlp::Mlp(int in, int hidden, int out, unsigned long long seed) : nin(in), nh(hidden), nout(out){
    if (in < 1 || hidden < 1 || out < 1) throw Error(ST_INVALID, "MLP sizes must be positive");
    nparams = (long long)nin * nh + nh + (long long)nh * nh + nh + (long long)nh * nout + nout;
    check_cuda(cudaMalloc(&params, nparams * sizeof(float)), "cudaMalloc(mlp)");
    check_cuda(cudaMalloc(&grads, nparams * sizeof(float)), "cudaMalloc(mlp)");
    check_cuda(cudaMalloc(&m, nparams * sizeof(float)), "cudaMalloc(mlp)");
    check_cuda(cudaMalloc(&v, nparams * sizeof(float)), "cudaMalloc(mlp)");
    check_cuda(cudaMemset(m, 0, nparams * sizeof(float)), "memset");
    check_cuda(cudaMemset(v, 0, nparams * sizeof(float)), "memset");
    check_cuda(cudaMalloc(&loss_d, sizeof(float)), "cudaMalloc(mlp)");
    check_cuda(cudaMalloc(&xrow, (size_t)nin * sizeof(float)), "cudaMalloc(mlp)");
    // He initialisation (host RNG, reproducible from the seed), zero biases
    std::vector<float> h(nparams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](long long off, int fan_in, long long count){
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)fan_in));
        for (long long i = 0; i < count; i++) h[off + i] = nd(rng);
    };
    fill(off_w1(), nin, (long long)nin * nh);
    fill(off_w2(), nh, (long long)nh * nh);
    fill(off_w3(), nh, (long long)nh * nout);
    check_cuda(cudaMemcpy(params, h.data(), nparams * sizeof(float), cudaMemcpyHostToDevice), "copy mlp params");
}

Mlp::~Mlp(){
    for (float *p : {params, grads, m, v, loss_d, xrow, h1, h2, y, dy, dh1, dh2}) if (p) cudaFree(p);
}

void Mlp::ensure(int B){
    if (B <= cap) return;
    for (float **p : {&h1, &h2, &y, &dy, &dh1, &dh2}) if (*p){ cudaFree(*p); *p = nullptr; }
    check_cuda(cudaMalloc(&h1, (size_t)B * nh * sizeof(float)), "cudaMalloc(mlp activations)");
    check_cuda(cudaMalloc(&h2, (size_t)B * nh * sizeof(float)), "cudaMalloc(mlp activations)");
    check_cuda(cudaMalloc(&dh1, (size_t)B * nh * sizeof(float)), "cudaMalloc(mlp activations)");
    check_cuda(cudaMalloc(&dh2, (size_t)B * nh * sizeof(float)), "cudaMalloc(mlp activations)");
    check_cuda(cudaMalloc(&y, (size_t)B * nout * sizeof(float)), "cudaMalloc(mlp activations)");
    check_cuda(cudaMalloc(&dy, (size_t)B * nout * sizeof(float)), "cudaMalloc(mlp activations)");
    cap = B;
}

void Mlp::forward(cudaStream_t s, float const *X, int B){
    ensure(B);
    float *P = params;
    k_dense_fwd<<<blocks_for((long long)B * nh), 256, 0, s>>>(X, P + off_w1(), P + off_b1(), h1, B, nin, nh, 1);
    k_dense_fwd<<<blocks_for((long long)B * nh), 256, 0, s>>>(h1, P + off_w2(), P + off_b2(), h2, B, nh, nh, 1);
    k_dense_fwd<<<blocks_for((long long)B * nout), 256, 0, s>>>(h2, P + off_w3(), P + off_b3(), y, B, nh, nout, 0);
    check_cuda(cudaPeekAtLastError(), "mlp forward");
}

void Mlp::loss_and_grad(cudaStream_t s, float const *X, float const *T, int B){
    forward(s, X, B);
    float *G = grads, *P = params;
    check_cuda(cudaMemsetAsync(loss_d, 0, sizeof(float), s), "memset");
    k_mse<<<blocks_for((long long)B * nout), 256, 0, s>>>(y, T, dy, loss_d, B * nout);
    k_dense_bwd_w<<<blocks_for((long long)nh * nout + nout), 256, 0, s>>>(h2, dy, G + off_w3(), G + off_b3(), B, nh, nout);
    k_dense_bwd_x<<<blocks_for((long long)B * nh), 256, 0, s>>>(dy, P + off_w3(), h2, dh2, B, nh, nout);
    k_dense_bwd_w<<<blocks_for((long long)nh * nh + nh), 256, 0, s>>>(h1, dh2, G + off_w2(), G + off_b2(), B, nh, nh);
    k_dense_bwd_x<<<blocks_for((long long)B * nh), 256, 0, s>>>(dh2, P + off_w2(), h1, dh1, B, nh, nh);
    k_dense_bwd_w<<<blocks_for((long long)nin * nh + nh), 256, 0, s>>>(X, dh1, G + off_w1(), G + off_b1(), B, nin, nh);
    check_cuda(cudaPeekAtLastError(), "mlp backward");
}

float Mlp::train(cudaStream_t s, float const *X, float const *T, int B, int steps, float lr){
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = 0; i < steps; i++){
        loss_and_grad(s, X, T, B);
        step++;
        float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
        k_adam<<<blocks_for(nparams), 256, 0, s>>>(params, grads, m, v, (int)nparams, lr, b1, b2, eps, c1, c2);
    }
    check_cuda(cudaPeekAtLastError(), "mlp training");
    float l = 0;
    check_cuda(cudaMemcpyAsync(&l, loss_d, sizeof(float), cudaMemcpyDeviceToHost, s), "copy loss");
    check_cuda(cudaStreamSynchronize(s), "mlp training sync");
    return l;
}

// ---------------------------------------------------------------------------
// features and candidates
// ---------------------------------------------------------------------------
static int n_factor(int n, int p){ int c = 0; while (n % p == 0){ n /= p; c++; } return c; }

void plan_features(int kind, int prec, int const size[3], float *f){
    int k = 0;
    double total = 1;
    for (int d = 0; d < 3; d++){
        int n = size[d];
        total *= n;
        f[k++] = (float)(std::log2((double)n) / 10.0);
    }
    f[k++] = (float)(std::log2(total) / 30.0);
    f[k++] = (kind == PK_C2C) ? 1.f : 0.f;
    f[k++] = (kind == PK_R2C) ? 1.f : 0.f;
    f[k++] = (kind == PK_COS || kind == PK_SIN || kind == PK_COS1) ? 1.f : 0.f;
    f[k++] = (float)prec;
    for (int d = 0; d < 3; d++){
        int n = size[d];
        bool pow2 = n > 0 && (n & (n - 1)) == 0;
        f[k++] = pow2 ? 1.f : 0.f;
        f[k++] = (float)(n_factor(n, 3) + n_factor(n, 5)) / 4.f;
        f[k++] = (float)(n_factor(n, 7) + n_factor(n, 11) + n_factor(n, 13)) / 2.f;
    }
    f[k++] = (float)(std::log2((double)std::max(size[0], 1)) - std::log2((double)std::max(std::max(size[1], size[2]), 1))) / 10.f;
    // k == kFeatures
}

void candidate_knobs(int c, Options &o, Knobs &kn){
    o.use_reorder = (c & 1) != 0;
    kn.variant = (c >> 1) & 1;
    kn.tile_div = ((c >> 2) & 1) ? 2 : 1;
    kn.radix_policy = (c >> 3) & 1;
}

} // namespace gbfft
