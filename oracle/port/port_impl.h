/*
 * Body of the C restatement of heFFTe's stock backend, instantiated twice by
 * heffte_port.c (REAL = float with suffix _f, REAL = double with suffix _d).
 * Test infrastructure / CPU baseline only; see heffte_port.c.
 */
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUF)
#define CPX FN(cpx)
#define NODE FN(node)

typedef struct { REAL re, im; } CPX;

static inline CPX FN(cmul)(CPX a, CPX b){ CPX r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline CPX FN(cadd)(CPX a, CPX b){ CPX r = {a.re + b.re, a.im + b.im}; return r; }
static inline CPX FN(csub)(CPX a, CPX b){ CPX r = {a.re - b.re, a.im - b.im}; return r; }
static inline CPX FN(mul_i)(CPX a){ CPX r = {-a.im, a.re}; return r; }
static inline CPX FN(mul_neg_i)(CPX a){ CPX r = {a.im, -a.re}; return r; }
/* omega<F>::get (stock_fft/heffte_stock_algos.h:31-37): the angle is formed in
 * the working precision, exactly as the reference does. */
static inline CPX FN(omega)(size_t power, size_t n, int sign){
    REAL a = (REAL)(2. * M_PI) * ((REAL)power) / ((REAL)n);
    CPX r = {(REAL)cos(a), (REAL)(sign * sin(a))};
    return r;
}

/* One node of the call tree (stock_fft/heffte_stock_algos.h:69-80). */
typedef struct NODE {
    size_t sz;
    int type;
    size_t left, right;      /* offsets to the children */
    CPX *work;               /* composite workspace, sz entries */
} NODE;

static size_t FN(init_tree)(NODE *root, size_t n){
    size_t k;
    int type = port_classify(n, &k);
    root->sz = n; root->type = type; root->left = root->right = 0;
    root->work = (type == PORT_COMPOSITE) ? (CPX*)calloc(n, sizeof(CPX)) : NULL;
    if (type != PORT_COMPOSITE) return 1;
    size_t q = n / k;
    size_t l = FN(init_tree)(root + 1, k);
    size_t r = FN(init_tree)(root + 1 + l, q);
    root->left = 1; root->right = 1 + l;
    return 1 + l + r;
}

static void FN(free_tree)(NODE *root, size_t count){
    for (size_t i = 0; i < count; i++) free(root[i].work);
    free(root);
}

static void FN(run)(CPX *x, CPX *y, size_t s_in, size_t s_out, NODE *node, int sign);

/* DFT_helper (heffte_stock_algos.h:83-122): direct O(n^2) DFT with twiddle recurrences. */
static void FN(dft)(size_t n, CPX *x, CPX *y, size_t s_in, size_t s_out, int sign){
    if (n == 1){ y[0] = x[0]; return; }
    CPX w0 = FN(omega)(1, n, sign), wk = w0, wkn = w0;
    CPX t = x[0];
    for (size_t i = 1; i < n; i++) t = FN(cadd)(t, x[i * s_in]);
    y[0] = t;
    for (size_t k = 1; k < n; k++){
        t = x[0];
        for (size_t i = 1; i < n; i++){
            t = FN(cadd)(FN(cmul)(wkn, x[i * s_in]), t);
            wkn = FN(cmul)(wkn, wk);
        }
        y[k * s_out] = t;
        wk = FN(cmul)(wk, w0);
        wkn = wk;
    }
}

/* pow2_FFT_helper (heffte_stock_algos.h:131-165): recursive radix-2 DIT. */
static void FN(pow2)(size_t n, CPX *x, CPX *y, size_t s_in, size_t s_out, int sign){
    if (n == 2){
        CPX a = x[0], b = x[s_in];
        y[0] = FN(cadd)(a, b); y[s_out] = FN(csub)(a, b);
        return;
    }
    size_t m = n / 2;
    FN(pow2)(m, x, y, s_in * 2, s_out, sign);
    FN(pow2)(m, x + s_in, y + s_out * m, s_in * 2, s_out, sign);
    CPX w1 = FN(omega)(1, n, sign), wj = w1;
    CPX yj = y[0];
    y[0] = FN(cadd)(y[0], y[m * s_out]);
    y[m * s_out] = FN(csub)(yj, y[m * s_out]);
    for (size_t j = 1; j < m; j++){
        size_t a = j * s_out, b = (j + m) * s_out;
        yj = y[a];
        CPX t = FN(cmul)(wj, y[b]);
        y[a] = FN(cadd)(yj, t);
        y[b] = FN(csub)(yj, t);
        wj = FN(cmul)(wj, w1);
    }
}

/* pow4_FFT_helper (heffte_stock_algos.h:175-260): recursive radix-4 DIT. */
static void FN(pow4)(size_t n, CPX *x, CPX *y, size_t s_in, size_t s_out, int sign){
    if (n == 4){
        CPX x0 = x[0], x1 = x[s_in], x2 = x[2 * s_in], x3 = x[3 * s_in];
        CPX a = FN(cadd)(x0, x2), b = FN(csub)(x0, x2), c = FN(cadd)(x1, x3), d = FN(csub)(x1, x3);
        CPX dr = (sign < 0) ? FN(mul_neg_i)(d) : FN(mul_i)(d);
        y[0] = FN(cadd)(a, c);
        y[s_out] = FN(cadd)(b, dr);
        y[2 * s_out] = FN(csub)(a, c);
        y[3 * s_out] = FN(csub)(b, dr);
        return;
    }
    size_t m = n / 4;
    for (int q = 0; q < 4; q++) FN(pow4)(m, x + q * s_in, y + q * s_out * m, s_in * 4, s_out, sign);
    CPX w1 = FN(omega)(1, n, sign), w2 = FN(cmul)(w1, w1), w3 = FN(cmul)(w2, w1);
    CPX wk1 = {1, 0}, wk2 = {1, 0}, wk3 = {1, 0};
    for (size_t k = 0; k < m; k++){
        size_t k0 = k * s_out, k1 = (k + m) * s_out, k2 = (k + 2 * m) * s_out, k3 = (k + 3 * m) * s_out;
        CPX y0 = y[k0], y1 = FN(cmul)(wk1, y[k1]), y2 = FN(cmul)(wk2, y[k2]), y3 = FN(cmul)(wk3, y[k3]);
        CPX a = FN(cadd)(y0, y2), b = FN(csub)(y0, y2), c = FN(cadd)(y1, y3), d = FN(csub)(y1, y3);
        CPX dr = (sign < 0) ? FN(mul_neg_i)(d) : FN(mul_i)(d);
        y[k0] = FN(cadd)(a, c); y[k1] = FN(cadd)(b, dr); y[k2] = FN(csub)(a, c); y[k3] = FN(csub)(b, dr);
        if (k == 0){ wk1 = w1; wk2 = w2; wk3 = w3; }
        else { wk1 = FN(cmul)(wk1, w1); wk2 = FN(cmul)(wk2, w2); wk3 = FN(cmul)(wk3, w3); }
    }
}

/* pow3_FFT_helper (heffte_stock_algos.h:368-433): recursive radix-3 DIT. */
static void FN(pow3)(size_t n, CPX *x, CPX *y, size_t s_in, size_t s_out, CPX p120, CPX m120, int sign){
    if (n == 3){
        CPX x0 = x[0], x1 = x[s_in], x2 = x[2 * s_in];
        y[0] = FN(cadd)(FN(cadd)(x0, x1), x2);
        y[s_out] = FN(cadd)(FN(cadd)(x0, FN(cmul)(p120, x1)), FN(cmul)(m120, x2));
        y[2 * s_out] = FN(cadd)(FN(cadd)(x0, FN(cmul)(m120, x1)), FN(cmul)(p120, x2));
        return;
    }
    size_t m = n / 3;
    for (int q = 0; q < 3; q++) FN(pow3)(m, x + q * s_in, y + q * m * s_out, s_in * 3, s_out, p120, m120, sign);
    CPX w1 = FN(omega)(1, n, sign), w2 = FN(cmul)(w1, w1);
    CPX wk1 = {1, 0}, wk2 = {1, 0};
    for (size_t k = 0; k < m; k++){
        size_t k1 = k * s_out, k2 = (m + k) * s_out, k3 = (2 * m + k) * s_out;
        CPX t0 = y[k1], t1 = FN(cmul)(wk1, y[k2]), t2 = FN(cmul)(wk2, y[k3]);
        y[k1] = FN(cadd)(FN(cadd)(t0, t1), t2);
        y[k2] = FN(cadd)(FN(cadd)(t0, FN(cmul)(p120, t1)), FN(cmul)(m120, t2));
        y[k3] = FN(cadd)(FN(cadd)(t0, FN(cmul)(m120, t1)), FN(cmul)(p120, t2));
        if (k == 0){ wk1 = w1; wk2 = w2; }
        else { wk1 = FN(cmul)(wk1, w1); wk2 = FN(cmul)(wk2, w2); }
    }
}

/* composite_FFT (heffte_stock_algos.h:270-305): N = N1 * N2 four-step with
 * the N2-point transforms first, a twiddle, then the N1-point transforms. */
static void FN(composite)(CPX *x, CPX *y, size_t s_in, size_t s_out, NODE *node, int sign){
    NODE *left = node + node->left, *right = node + node->right;
    size_t n = node->sz, n1 = left->sz, n2 = right->sz;
    CPX *z = node->work;
    CPX w1 = FN(omega)(1, n, sign);
    CPX wj1 = {1, 0};
    for (size_t j1 = 0; j1 < n1; j1++){
        CPX wk2 = wj1;
        FN(run)(&x[j1 * s_in], &z[n2 * j1], n1 * s_in, 1, right, sign);
        if (j1 > 0){
            for (size_t k2 = 1; k2 < n2; k2++){
                z[j1 * n2 + k2] = FN(cmul)(z[j1 * n2 + k2], wk2);
                wk2 = FN(cmul)(wk2, wj1);
            }
        }
        wj1 = FN(cmul)(wj1, w1);
    }
    for (size_t k2 = 0; k2 < n2; k2++) FN(run)(&z[k2], &y[k2 * s_out], n2, n2 * s_out, left, sign);
}

static void FN(run)(CPX *x, CPX *y, size_t s_in, size_t s_out, NODE *node, int sign){
    switch (node->type){
        case PORT_POW2: FN(pow2)(node->sz, x, y, s_in, s_out, sign); break;
        case PORT_POW4: FN(pow4)(node->sz, x, y, s_in, s_out, sign); break;
        case PORT_POW3: {
            CPX p = {(REAL)-0.5, (REAL)(-sqrt(3.) / 2.)}, m = {(REAL)-0.5, (REAL)(sqrt(3.) / 2.)};
            if (sign < 0) FN(pow3)(node->sz, x, y, s_in, s_out, p, m, sign);
            else FN(pow3)(node->sz, x, y, s_in, s_out, m, p, sign);
            break;
        }
        case PORT_COMPOSITE: FN(composite)(x, y, s_in, s_out, node, sign); break;
        default: FN(dft)(node->sz, x, y, s_in, s_out, sign); break;
    }
}

/* Per-thread plan: the tree plus contiguous in/out line buffers, the analogue
 * of plan_stock_fft (heffte_backend_stock.h:339-407, non-SIMD branch). */
typedef struct {
    size_t n, count;
    NODE *tree;
    CPX *inp, *out;
} FN(plan);

static void FN(plan_init)(FN(plan) *p, size_t n){
    p->n = n;
    p->count = port_num_nodes(n);
    p->tree = (NODE*)calloc(p->count, sizeof(NODE));
    FN(init_tree)(p->tree, n);
    p->inp = (CPX*)malloc(n * sizeof(CPX));
    p->out = (CPX*)malloc(n * sizeof(CPX));
}
static void FN(plan_free)(FN(plan) *p){
    FN(free_tree)(p->tree, p->count); free(p->inp); free(p->out);
}

/* Batched in-place c2c along one dimension, the stock_fft_executor
 * (heffte_backend_stock.h:448-548): `howmany` transforms of length n with
 * element stride `stride` and batch distance `dist`, repeated over `blocks`
 * blocks `block_stride` apart.  Lines are shared among OpenMP threads. */
static void FN(c2c_batch)(size_t n, long long howmany, long long stride, long long dist,
                          long long blocks, long long block_stride, int sign, CPX *data, int threads){
    long long total = howmany * blocks;
    #pragma omp parallel num_threads(threads)
    {
        FN(plan) p; FN(plan_init)(&p, n);
        #pragma omp for schedule(static)
        for (long long t = 0; t < total; t++){
            CPX *base = data + (t / howmany) * block_stride + (t % howmany) * dist;
            for (size_t i = 0; i < n; i++) p.inp[i] = base[i * stride];
            FN(run)(p.inp, p.out, 1, 1, p.tree, sign);
            for (size_t i = 0; i < n; i++) base[i * stride] = p.out[i];
        }
        FN(plan_free)(&p);
    }
}

/* Batched r2c (forward) / c2r (backward) along one dimension
 * (plan_stock_fft<F>::execute, heffte_backend_stock.h:339-380). */
static void FN(r2c_batch)(size_t n, long long howmany, long long stride, long long rdist, long long cdist,
                          long long blocks, long long rblock, long long cblock, const REAL *in, CPX *out, int threads){
    long long total = howmany * blocks;
    #pragma omp parallel num_threads(threads)
    {
        FN(plan) p; FN(plan_init)(&p, n);
        #pragma omp for schedule(static)
        for (long long t = 0; t < total; t++){
            const REAL *rb = in + (t / howmany) * rblock + (t % howmany) * rdist;
            CPX *cb = out + (t / howmany) * cblock + (t % howmany) * cdist;
            for (size_t i = 0; i < n; i++){ p.inp[i].re = rb[i * stride]; p.inp[i].im = 0; }
            FN(run)(p.inp, p.out, 1, 1, p.tree, -1);
            for (size_t i = 0; i < (n + 2) / 2; i++) cb[i * stride] = p.out[i];
        }
        FN(plan_free)(&p);
    }
}
static void FN(c2r_batch)(size_t n, long long howmany, long long stride, long long rdist, long long cdist,
                          long long blocks, long long rblock, long long cblock, const CPX *in, REAL *out, int threads){
    long long total = howmany * blocks;
    #pragma omp parallel num_threads(threads)
    {
        FN(plan) p; FN(plan_init)(&p, n);
        #pragma omp for schedule(static)
        for (long long t = 0; t < total; t++){
            const CPX *cb = in + (t / howmany) * cblock + (t % howmany) * cdist;
            REAL *rb = out + (t / howmany) * rblock + (t % howmany) * rdist;
            p.inp[0] = cb[0];
            for (size_t i = 1; i < (n + 2) / 2; i++){
                p.inp[i] = cb[i * stride];
                p.inp[n - i].re = p.inp[i].re; p.inp[n - i].im = -p.inp[i].im;
            }
            FN(run)(p.inp, p.out, 1, 1, p.tree, 1);
            for (size_t i = 0; i < n; i++) rb[i * stride] = p.out[i].re;
        }
        FN(plan_free)(&p);
    }
}

/* Executor geometry of one dimension of a box in order (0,1,2), from
 * fft1d_get_howmany / fft1d_get_stride (heffte_geometry.h:159-174) and the
 * executor constructors (heffte_backend_stock.h:448-465). */
static void FN(dim_geometry)(const long long nsz[3], int dim, long long *howmany, long long *stride,
                             long long *dist, long long *blocks, long long *block_stride){
    if (dim == 0){ *howmany = nsz[1] * nsz[2]; *stride = 1; *dist = nsz[0]; *blocks = 1; *block_stride = 0; }
    else if (dim == 1){ *howmany = nsz[0]; *stride = nsz[0]; *dist = 1; *blocks = nsz[2]; *block_stride = nsz[0] * nsz[1]; }
    else { *howmany = nsz[0] * nsz[1]; *stride = nsz[0] * nsz[1]; *dist = 1; *blocks = 1; *block_stride = 0; }
}

static void FN(scale)(long long n, REAL *d, double f, int threads){
    #pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) d[i] *= (REAL)f;
}

#undef CPX
#undef NODE
#undef FN
#undef CAT
#undef CAT_
