/*
 * heffte_port: a plain-C restatement of heFFTe's stock (CPU) backend for the
 * fft3d hot path.  TEST INFRASTRUCTURE AND CPU BASELINE ONLY: the tests use it
 * as a checker and bench.py times it as the CPU baseline; the product path
 * never links, loads or calls it.
 *
 * What it restates (reference file:line):
 *   call tree + radix choice     include/stock_fft/heffte_stock_tree.h:42-242
 *   pow2/pow4/pow3/composite/DFT include/stock_fft/heffte_stock_algos.h:34-433
 *   batched executors            include/heffte_backend_stock.h:339-548
 *   r2r pre/post processors      include/heffte_r2r_executor.h:43-180
 *   r2r scale factors            include/heffte_fft3d.h:635-650
 *   pack / transpose-unpack      include/heffte_pack3d.h:89-197
 *   3-D stage sequence           src/heffte_compute_transform.cpp:15-258
 * The 3-D drivers run the strided-executor plan of a single rank with the
 * box in order (0,1,2) (no reorder), which is the plan the reference builds
 * for backends whose default is use_reorder = false.  Rader's algorithm (only
 * used by the reference for primes above 100000) is not restated: such
 * lengths fall back to the direct DFT leaf.
 *
 * Lines are distributed over OpenMP threads; the reference stock backend is
 * single-threaded, so `threads = 1` is the reference's own configuration.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

enum { PORT_POW2, PORT_POW3, PORT_POW4, PORT_COMPOSITE, PORT_DISCRETE };

static int port_power_of(size_t n, size_t p){
    if (n == 1) return 0;
    while (n % p == 0) n /= p;
    return n == 1;
}

/* factor() with the reference's priority list (heffte_stock_tree.h:20-60):
 * 4, 2, 3, 5, 7, 11, 13, 16, then primes; the first divisor found wins. */
static size_t port_factor(size_t f){
    static const size_t first[] = {4, 2, 3, 5, 7, 11, 13, 16, 17, 19, 23, 29, 31, 37, 41, 43, 47};
    for (size_t i = 0; i < sizeof(first) / sizeof(first[0]); i++) if (f % first[i] == 0) return first[i];
    for (size_t k = 53; k * k <= f; k += 2) if (f % k == 0) return k;
    return f;
}

/* fptrFactorHelper (heffte_stock_tree.h:160-205). */
static int port_classify(size_t n, size_t *k){
    *k = n;
    if (port_power_of(n, 4)) return PORT_POW4;
    if (port_power_of(n, 2)) return PORT_POW2;
    if (port_power_of(n, 3)) return PORT_POW3;
    size_t base = 0;
    if (n % 4 == 0) base = 4; else if (n % 2 == 0) base = 2; else if (n % 3 == 0) base = 3;
    if (base){
        size_t ell = n;
        while (ell % base == 0) ell /= base;
        *k = n / ell;
        return PORT_COMPOSITE;
    }
    size_t f = port_factor(n);
    if (f == n) return PORT_DISCRETE;
    *k = f;
    return PORT_COMPOSITE;
}

static size_t port_num_nodes(size_t n){
    size_t k;
    int t = port_classify(n, &k);
    if (t != PORT_COMPOSITE) return 1;
    return 1 + port_num_nodes(k) + port_num_nodes(n / k);
}

#define REAL float
#define SUF _f
#include "port_impl.h"
#undef REAL
#undef SUF
#define REAL double
#define SUF _d
#include "port_impl.h"
#undef REAL
#undef SUF

/* ----------------------------------------------------------------------- */
/* 3-D drivers                                                              */
/* ----------------------------------------------------------------------- */

static double port_scale_factor(int scaling, double count){
    if (scaling == 0) return 1.0;
    return (scaling == 1) ? 1.0 / count : sqrt(1.0 / count);
}

#define C2C_PASSES(SUFX, CT)                                                        \
    for (int d = 0; d < 3; d++){                                                    \
        long long hm, st, di, bl, bs;                                               \
        dim_geometry##SUFX(nsz, d, &hm, &st, &di, &bl, &bs);                        \
        c2c_batch##SUFX((size_t)nsz[d], hm, st, di, bl, bs, sign, (CT*)out, threads); \
    }

/* fft3d<stock>::forward/backward on a single rank, in order (0,1,2):
 * copy input to output, three strided executor stages in place, optional
 * scaling (heffte_fft3d.h:375-384, :662-678). prec 0 = complex<float>. */
int port_fft3d_c2c(int prec, const long long nsz[3], int direction, int scaling,
                   const void *in, void *out, int threads){
    long long count = nsz[0] * nsz[1] * nsz[2];
    int sign = (direction == 0) ? -1 : 1;
    size_t esz = (prec == 0) ? 8 : 16;
    if (in != out) memcpy(out, in, (size_t)count * esz);
    double f = port_scale_factor(scaling, (double)count);
    if (prec == 0){
        C2C_PASSES(_f, cpx_f)
        if (scaling) scale_f(2 * count, (float*)out, f, threads);
    }else{
        C2C_PASSES(_d, cpx_d)
        if (scaling) scale_d(2 * count, (double*)out, f, threads);
    }
    return 0;
}

/* Geometry of an r2c stage along `dim` (heffte_backend_stock.h:560-575). */
static void port_r2c_geometry(const long long n[3], int dim, long long *howmany, long long *stride,
                              long long *rdist, long long *cdist, long long *blocks,
                              long long *rblock, long long *cblock){
    *blocks = 1; *rblock = 0; *cblock = 0;
    if (dim == 0){ *howmany = n[1] * n[2]; *stride = 1; *rdist = n[0]; *cdist = n[0] / 2 + 1; }
    else if (dim == 1){
        *howmany = n[0]; *stride = n[0]; *rdist = 1; *cdist = 1; *blocks = n[2];
        *rblock = n[0] * n[1]; *cblock = n[0] * (n[1] / 2 + 1);
    }else { *howmany = n[0] * n[1]; *stride = n[0] * n[1]; *rdist = 1; *cdist = 1; }
}

/* fft3d_r2c<stock> on a single rank, order (0,1,2).  direction 0: real in ->
 * complex out of size n with n[r2c_dir] -> n[r2c_dir]/2+1; direction 1: the
 * inverse (the complex input is not modified, as in the reference, which
 * copies it to a buffer first, src/heffte_compute_transform.cpp:212-220). */
int port_fft3d_r2c(int prec, const long long n[3], int r2c_dir, int direction, int scaling,
                   const void *in, void *out, int threads){
    long long cn[3] = {n[0], n[1], n[2]};
    cn[r2c_dir] = n[r2c_dir] / 2 + 1;
    long long rcount = n[0] * n[1] * n[2], ccount = cn[0] * cn[1] * cn[2];
    long long hm, st, rd, cd, bl, rb, cb;
    port_r2c_geometry(n, r2c_dir, &hm, &st, &rd, &cd, &bl, &rb, &cb);
    double f = port_scale_factor(scaling, (double)rcount);
    size_t esz = (prec == 0) ? 8 : 16;
    if (direction == 0){
        if (prec == 0) r2c_batch_f((size_t)n[r2c_dir], hm, st, rd, cd, bl, rb, cb, (const float*)in, (cpx_f*)out, threads);
        else r2c_batch_d((size_t)n[r2c_dir], hm, st, rd, cd, bl, rb, cb, (const double*)in, (cpx_d*)out, threads);
        for (int d = 0; d < 3; d++){
            if (d == r2c_dir) continue;
            long long h2, s2, d2, b2, bs2;
            if (prec == 0){ dim_geometry_f(cn, d, &h2, &s2, &d2, &b2, &bs2); c2c_batch_f((size_t)cn[d], h2, s2, d2, b2, bs2, -1, (cpx_f*)out, threads); }
            else { dim_geometry_d(cn, d, &h2, &s2, &d2, &b2, &bs2); c2c_batch_d((size_t)cn[d], h2, s2, d2, b2, bs2, -1, (cpx_d*)out, threads); }
        }
        if (scaling){
            if (prec == 0) scale_f(2 * ccount, (float*)out, f, threads); else scale_d(2 * ccount, (double*)out, f, threads);
        }
    }else{
        void *tmp = malloc((size_t)ccount * esz);
        memcpy(tmp, in, (size_t)ccount * esz);
        for (int d = 2; d >= 0; d--){
            if (d == r2c_dir) continue;
            long long h2, s2, d2, b2, bs2;
            if (prec == 0){ dim_geometry_f(cn, d, &h2, &s2, &d2, &b2, &bs2); c2c_batch_f((size_t)cn[d], h2, s2, d2, b2, bs2, 1, (cpx_f*)tmp, threads); }
            else { dim_geometry_d(cn, d, &h2, &s2, &d2, &b2, &bs2); c2c_batch_d((size_t)cn[d], h2, s2, d2, b2, bs2, 1, (cpx_d*)tmp, threads); }
        }
        if (prec == 0) c2r_batch_f((size_t)n[r2c_dir], hm, st, rd, cd, bl, rb, cb, (const cpx_f*)tmp, (float*)out, threads);
        else c2r_batch_d((size_t)n[r2c_dir], hm, st, rd, cd, bl, rb, cb, (const cpx_d*)tmp, (double*)out, threads);
        free(tmp);
        if (scaling){
            if (prec == 0) scale_f(rcount, (float*)out, f, threads); else scale_d(rcount, (double*)out, f, threads);
        }
    }
    return 0;
}

/* One line of the real-to-real executor (heffte_r2r_executor.h:221-245):
 * pre-process into the extended signal, r2c/c2r of the extended length,
 * post-process.  kind 0 cos, 1 sin, 2 cos1. */
#define R2R_LINE(SUFX, RT, CT)                                                          \
static void r2r_line##SUFX(int kind, int direction, long long N, RT *x, RT *sig, CT *csig, \
                          plan##SUFX *p){                                              \
    long long M = (kind == 2) ? 4 * (N - 1) : 4 * N;                                   \
    long long i;                                                                        \
    if (direction == 0){                                                                \
        if (kind == 0){                                                                 \
            for (i = 0; i < N; i++){ sig[2*i] = 0; sig[2*i+1] = x[i]; }                 \
            sig[2*N] = 0;                                                               \
            for (i = 0; i < 2*N; i++) sig[4*N - i] = sig[i];                            \
        }else if (kind == 1){                                                           \
            for (i = 0; i < N; i++){ sig[2*i] = 0; sig[2*i+1] = x[i]; }                 \
            sig[2*N] = 0;                                                               \
            for (i = 0; i < N; i++){ sig[4*N - 2*i] = 0; sig[4*N - 2*i - 1] = -x[i]; }  \
        }else{                                                                          \
            for (i = 0; i < N - 1; i++){ sig[2*i] = x[i]; sig[2*i+1] = 0; }             \
            for (i = 1; i < N; i++){ sig[4*(N-1) - 2*i] = x[i]; sig[4*(N-1) - 2*i + 1] = 0; } \
        }                                                                               \
        for (i = 0; i < M; i++){ p->inp[i].re = sig[i]; p->inp[i].im = 0; }            \
        run##SUFX(p->inp, p->out, 1, 1, p->tree, -1);                                   \
        if (kind == 1) for (i = 0; i < N; i++) x[i] = -p->out[i+1].im;                  \
        else for (i = 0; i < N; i++) x[i] = p->out[i].re;                               \
    }else{                                                                              \
        long long H = M / 2 + 1;                                                        \
        for (i = 0; i < H; i++){ csig[i].re = 0; csig[i].im = 0; }                      \
        if (kind == 0){                                                                 \
            for (i = 0; i < N; i++){ csig[i].re = x[i]; }                               \
            csig[N].re = 0;                                                             \
            for (i = 0; i < N; i++){ csig[N + 1 + i].re = -x[N - 1 - i]; }              \
        }else if (kind == 1){                                                           \
            for (i = 0; i < N; i++){ csig[i+1].re = 0; csig[i+1].im = -x[i]; }          \
            csig[2*N].re = 0; csig[2*N].im = 0;                                         \
            for (i = 0; i < N - 1; i++){ csig[N + i + 1].re = 0; csig[N + i + 1].im = -x[N - i - 2]; } \
        }else{                                                                          \
            for (i = 0; i < N; i++){ csig[i].re = x[i]; }                               \
            for (i = N; i < 2*N - 1; i++){ csig[i].re = x[2*N - 2 - i]; }               \
        }                                                                               \
        p->inp[0] = csig[0];                                                            \
        for (i = 1; i < (M + 2) / 2; i++){                                              \
            p->inp[i] = csig[i]; p->inp[M - i].re = csig[i].re; p->inp[M - i].im = -csig[i].im; \
        }                                                                               \
        run##SUFX(p->inp, p->out, 1, 1, p->tree, 1);                                    \
        if (kind == 2) for (i = 0; i < N; i++) x[i] = p->out[2*i].re;                   \
        else for (i = 0; i < N; i++) x[i] = p->out[2*i+1].re;                           \
    }                                                                                   \
}
R2R_LINE(_f, float, cpx_f)
R2R_LINE(_d, double, cpx_d)

#define R2R_PASS(SUFX, RT, CT)                                                          \
    {                                                                                   \
        long long N = n[d];                                                             \
        long long M = (kind == 2) ? 4 * (N - 1) : 4 * N;                                \
        long long st = (d == 0) ? 1 : ((d == 1) ? n[0] : n[0] * n[1]);                  \
        long long lines = (n[0] * n[1] * n[2]) / N;                                     \
        _Pragma("omp parallel num_threads(threads)")                                    \
        {                                                                               \
            plan##SUFX p; plan_init##SUFX(&p, (size_t)M);                               \
            RT *line = (RT*)malloc((size_t)N * sizeof(RT));                             \
            RT *sig = (RT*)malloc((size_t)(M + 2) * sizeof(RT));                        \
            CT *csig = (CT*)malloc((size_t)(M / 2 + 2) * sizeof(CT));                   \
            _Pragma("omp for schedule(static)")                                         \
            for (long long t = 0; t < lines; t++){                                      \
                long long base;                                                         \
                if (d == 0) base = t * N;                                               \
                else if (d == 1) base = (t / n[0]) * n[0] * n[1] + (t % n[0]);          \
                else base = t;                                                          \
                RT *o = (RT*)out;                                                       \
                for (long long i = 0; i < N; i++) line[i] = o[base + i * st];           \
                r2r_line##SUFX(kind, direction, N, line, sig, csig, &p);                \
                for (long long i = 0; i < N; i++) o[base + i * st] = line[i];           \
            }                                                                           \
            free(line); free(sig); free(csig); plan_free##SUFX(&p);                     \
        }                                                                               \
    }

/* rtransform<stock_cos|stock_sin|stock_cos1> on a single rank, order (0,1,2).
 * Scale factors follow heffte_fft3d.h:635-650 for the stock tags. */
int port_rtransform(int kind, int prec, const long long n[3], int direction, int scaling,
                    const void *in, void *out, int threads){
    long long count = n[0] * n[1] * n[2];
    size_t esz = (prec == 0) ? 4 : 8;
    if (in != out) memcpy(out, in, (size_t)count * esz);
    for (int d = 0; d < 3; d++){
        if (prec == 0) R2R_PASS(_f, float, cpx_f)
        else R2R_PASS(_d, double, cpx_d)
    }
    if (scaling){
        double sf = (kind == 2) ? 1.0 / (64.0 * (double)(n[0] - 1) * (double)(n[1] - 1) * (double)(n[2] - 1))
                                : 1.0 / ((double)count * 64.0);
        if (scaling == 2) sf = sqrt(sf);
        if (prec == 0) scale_f(count, (float*)out, sf, threads); else scale_d(count, (double*)out, sf, threads);
    }
    return 0;
}

/* Pack (op 0), unpack (op 1) and transpose-unpack (op 2) with the plan
 * fields of pack_plan_3d (heffte_pack3d.h:31-45); elements are esize bytes. */
int port_pack(int op, int esize, const long long size[3], long long ls, long long ps,
              long long bls, long long bps, const int map[3], const void *src, void *dst){
    const char *s = (const char*)src;
    char *d = (char*)dst;
    size_t e = (size_t)esize;
    for (long long k = 0; k < size[2]; k++)
        for (long long j = 0; j < size[1]; j++)
            for (long long i = 0; i < size[0]; i++){
                long long so, dof;
                if (op == 0){ so = k * ps + j * ls + i; dof = (k * size[1] + j) * size[0] + i; }
                else if (op == 1){ so = (k * size[1] + j) * size[0] + i; dof = k * ps + j * ls + i; }
                else {
                    dof = k * ps + j * ls + i;
                    if (map[0] == 0 && map[1] == 1) so = k * bps + j * bls + i;
                    else if (map[0] == 0 && map[1] == 2) so = j * bps + k * bls + i;
                    else if (map[0] == 1 && map[1] == 0) so = k * bps + i * bls + j;
                    else if (map[0] == 1 && map[1] == 2) so = i * bps + k * bls + j;
                    else if (map[0] == 2 && map[1] == 0) so = j * bps + i * bls + k;
                    else so = i * bps + j * bls + k;
                }
                memcpy(d + (size_t)dof * e, s + (size_t)so * e, e);
            }
    return 0;
}

/* data_scaling::apply (heffte_pack3d.h:205-233) on n reals. */
int port_scale(int prec, long long n, void *data, double factor, int threads){
    if (prec == 0) scale_f(n, (float*)data, factor, threads); else scale_d(n, (double*)data, factor, threads);
    return 0;
}
