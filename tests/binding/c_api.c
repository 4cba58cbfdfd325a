/*
 * The reference's C API (include/heffte_c.h, src/heffte_c.cpp) with the GB300
 * backend id: a C program that creates plans with Heffte_BACKEND_GB300 and
 * runs heffte_forward_* / heffte_backward_* on device buffers.  Built by
 * tests/test_reference_binding.py against a copy of heffte_c.cpp and
 * heffte_c_defines.h carrying the maintainer's edit (the new id).
 *
 * usage: c_api <prec 0|1> <r2c 0|1> <n0> <n1> <n2> <prefix>
 * Reads <prefix>_in.bin (forward input) and <prefix>_fin.bin (backward input),
 * writes <prefix>_fwd.bin (forward, scale none) and <prefix>_bwd.bin
 * (backward, scale full), and prints the plan's backend id and sizes.
 */
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include "heffte_c.h"

static void *read_file(const char *prefix, const char *suffix, size_t bytes){
    char path[4096];
    snprintf(path, sizeof(path), "%s%s", prefix, suffix);
    FILE *f = fopen(path, "rb");
    void *buf = malloc(bytes ? bytes : 1);
    if (!f || fread(buf, 1, bytes, f) != bytes){ fprintf(stderr, "cannot read %s\n", path); exit(1); }
    fclose(f);
    return buf;
}

static void write_file(const char *prefix, const char *suffix, const void *dev, size_t bytes){
    char path[4096];
    void *h = malloc(bytes ? bytes : 1);
    snprintf(path, sizeof(path), "%s%s", prefix, suffix);
    if (cudaMemcpy(h, dev, bytes, cudaMemcpyDeviceToHost) != cudaSuccess){ fprintf(stderr, "D2H failed\n"); exit(1); }
    FILE *f = fopen(path, "wb");
    fwrite(h, 1, bytes, f);
    fclose(f);
    free(h);
}

static void *to_device(const void *h, size_t bytes){
    void *d = NULL;
    if (cudaMalloc(&d, bytes ? bytes : 1) != cudaSuccess || cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess){
        fprintf(stderr, "device copy failed\n");
        exit(1);
    }
    return d;
}

int main(int argc, char **argv){
    if (argc != 7){ fprintf(stderr, "usage: c_api prec r2c n0 n1 n2 prefix\n"); return 2; }
    int prec = atoi(argv[1]), r2c = atoi(argv[2]);
    int n[3] = {atoi(argv[3]), atoi(argv[4]), atoi(argv[5])};
    const char *prefix = argv[6];
    int lo[3] = {0, 0, 0}, hi[3] = {n[0] - 1, n[1] - 1, n[2] - 1}, ohi[3] = {n[0] - 1, n[1] - 1, n[2] - 1};
    heffte_plan plan;
    heffte_plan_options options;
    if (heffte_set_default_options(Heffte_BACKEND_GB300, &options) != Heffte_SUCCESS){ fprintf(stderr, "options\n"); return 1; }
    int rc;
    if (r2c){
        ohi[0] = n[0] / 2;   /* r2c along dimension 0: outbox = inbox.r2c(0) */
        rc = heffte_plan_create_r2c(Heffte_BACKEND_GB300, lo, hi, NULL, lo, ohi, NULL, 0, MPI_COMM_SELF, &options, &plan);
    } else {
        rc = heffte_plan_create(Heffte_BACKEND_GB300, lo, hi, NULL, lo, ohi, NULL, MPI_COMM_SELF, NULL, &plan);
    }
    if (rc != Heffte_SUCCESS){ fprintf(stderr, "plan create failed: %d\n", rc); return 1; }
    size_t rs = prec ? sizeof(double) : sizeof(float), cs = 2 * rs;
    size_t nin = (size_t)heffte_size_inbox(plan), nout = (size_t)heffte_size_outbox(plan);
    size_t in_es = r2c ? rs : cs;
    void *hin = read_file(prefix, "_in.bin", nin * in_es);
    void *hfin = read_file(prefix, "_fin.bin", nout * cs);
    void *din = to_device(hin, nin * in_es), *dfin = to_device(hfin, nout * cs);
    void *dout = NULL, *dback = NULL, *dwork = NULL;
    size_t nw = (size_t)heffte_size_workspace(plan);
    if (cudaMalloc(&dout, nout * cs) != cudaSuccess || cudaMalloc(&dback, nin * in_es) != cudaSuccess ||
        cudaMalloc(&dwork, (nw ? nw : 1) * cs) != cudaSuccess){ fprintf(stderr, "cudaMalloc failed\n"); return 1; }
    if (r2c && prec == 0){
        heffte_forward_s2c(plan, (const float*)din, dout, Heffte_SCALE_NONE);
        heffte_backward_c2s_buffered(plan, dfin, (float*)dback, dwork, Heffte_SCALE_FULL);
    } else if (r2c){
        heffte_forward_d2z_buffered(plan, (const double*)din, dout, dwork, Heffte_SCALE_NONE);
        heffte_backward_z2d(plan, dfin, (double*)dback, Heffte_SCALE_FULL);
    } else if (prec == 0){
        heffte_forward_c2c(plan, din, dout, Heffte_SCALE_NONE);
        heffte_backward_c2c_buffered(plan, dfin, dback, dwork, Heffte_SCALE_FULL);
    } else {
        heffte_forward_z2z_buffered(plan, din, dout, dwork, Heffte_SCALE_NONE);
        heffte_backward_z2z(plan, dfin, dback, Heffte_SCALE_FULL);
    }
    if (cudaDeviceSynchronize() != cudaSuccess){ fprintf(stderr, "device error\n"); return 1; }
    write_file(prefix, "_fwd.bin", dout, nout * cs);
    write_file(prefix, "_bwd.bin", dback, nin * in_es);
    printf("%d %d %zu %zu\n", heffte_get_backend(plan), heffte_is_r2c(plan), nin, nout);
    heffte_plan_destroy(plan);
    cudaFree(din); cudaFree(dfin); cudaFree(dout); cudaFree(dback); cudaFree(dwork);
    free(hin); free(hfin);
    return 0;
}
