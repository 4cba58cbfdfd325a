// Data-movement kernels of the location layer (sm_103a):
//   direct pack / unpack, transpose-unpack (6 axis maps), scaling and the
//   real <-> complex conversion.  All copies move whole elements as opaque
//   4/8/16-byte words, so they are bit-exact.
#include "gbfft_internal.h"

namespace gbfft {

struct alignas(16) W16 { uint32_t a, b, c, d; };
struct alignas(8) W8 { uint32_t a, b; };

// dst[k*dps + j*dls + i] = src[k*sps + j*sls + i], i < nf, j < nm, k < ns.
// Rows are handed out to warps; each warp copies its row with consecutive
// lanes on consecutive elements (coalesced on both sides).
template<typename W>
__global__ void __launch_bounds__(256)
k_rowcopy(long long nf, long long nm, long long ns, long long sls, long long sps, long long dls, long long dps,
          W const *__restrict__ src, W *__restrict__ dst){
    long long rows = nm * ns;
    int lane = threadIdx.x & 31;
    long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = warp; r < rows; r += nwarps){
        long long j = r % nm, k = r / nm;
        W const *s = src + k * sps + j * sls;
        W *d = dst + k * dps + j * dls;
        for (long long i = lane; i < nf; i += 32) d[i] = s[i];
    }
}

// Transpose-unpack for the maps whose source-contiguous index is not the
// destination's fastest index.  UNIT = 1: source stride of j is 1 (maps
// (1,0,2), (1,2,0)); UNIT = 2: source stride of k is 1 (maps (2,0,1), (2,1,0)).
// A 32x32 tile (i x u) goes through shared memory: read coalesced along u,
// written coalesced along i.
template<typename W, int UNIT>
__global__ void __launch_bounds__(256)
k_transpose(long long nf, long long nm, long long ns, long long ls, long long ps,
            long long si, long long sw, W const *__restrict__ src, W *__restrict__ dst,
            long long tiles_i, long long tiles_u){
    __shared__ W tile[32][33];
    long long nu = (UNIT == 1) ? nm : ns;
    long long nw = (UNIT == 1) ? ns : nm;
    long long dstride_u = (UNIT == 1) ? ls : ps;
    long long dstride_w = (UNIT == 1) ? ps : ls;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    long long ntile = tiles_i * tiles_u;
    for (long long w = blockIdx.y; w < nw; w += gridDim.y){
        for (long long tl = blockIdx.x; tl < ntile; tl += gridDim.x){
            long long i0 = (tl % tiles_i) * 32, u0 = (tl / tiles_i) * 32;
            #pragma unroll
            for (int r = 0; r < 4; r++){
                long long i = i0 + ty + 8 * r, u = u0 + tx;
                if (i < nf && u < nu) tile[ty + 8 * r][tx] = src[i * si + u + w * sw];
            }
            __syncthreads();
            #pragma unroll
            for (int r = 0; r < 4; r++){
                long long i = i0 + tx, u = u0 + ty + 8 * r;
                if (i < nf && u < nu) dst[i + u * dstride_u + w * dstride_w] = tile[tx][ty + 8 * r];
            }
            __syncthreads();
        }
    }
}

template<typename T>
__global__ void __launch_bounds__(256) k_scale(long long n, T *data, T s){
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long step = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += step) data[i] *= s;
}
// vectorised body for 16-byte aligned buffers
template<typename T, typename V>
__global__ void __launch_bounds__(256) k_scale_vec(long long nv, V *data, T s){
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long step = (long long)gridDim.x * blockDim.x;
    for (; i < nv; i += step){
        V v = data[i];
        T *e = reinterpret_cast<T*>(&v);
        #pragma unroll
        for (int q = 0; q < (int)(sizeof(V) / sizeof(T)); q++) e[q] *= s;
        data[i] = v;
    }
}

template<typename T>
__global__ void __launch_bounds__(256) k_convert(long long n, T const *src, T *dst, int to_complex){
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long step = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += step){
        if (to_complex){ dst[2 * i] = src[i]; dst[2 * i + 1] = (T)0; }
        else dst[i] = src[2 * i];
    }
}

static int grid_for(long long work, int per_block){
    long long b = (work + per_block - 1) / per_block;
    long long cap = (long long)num_sms() * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

template<typename W>
static void rowcopy(cudaStream_t s, long long nf, long long nm, long long ns, long long sls, long long sps,
                    long long dls, long long dps, void const *src, void *dst){
    long long rows = nm * ns;
    int blocks = grid_for(rows * 32, 256);
    k_rowcopy<W><<<blocks, 256, 0, s>>>(nf, nm, ns, sls, sps, dls, dps,
                                        reinterpret_cast<W const*>(src), reinterpret_cast<W*>(dst));
}

template<typename W>
static void transpose(cudaStream_t s, long long nf, long long nm, long long ns, long long ls, long long ps,
                      long long bls, long long bps, int m0, int m1, void const *src, void *dst){
    // source strides of the destination indices (i, j, k) for each map
    long long si = 1, sj = 1, sk = 1;
    if (m0 == 0 && m1 == 1){ si = 1; sj = bls; sk = bps; }
    else if (m0 == 0 && m1 == 2){ si = 1; sj = bps; sk = bls; }
    else if (m0 == 1 && m1 == 0){ si = bls; sj = 1; sk = bps; }
    else if (m0 == 1 && m1 == 2){ si = bps; sj = 1; sk = bls; }
    else if (m0 == 2 && m1 == 0){ si = bls; sj = bps; sk = 1; }
    else { si = bps; sj = bls; sk = 1; }
    if (m0 == 0){
        rowcopy<W>(s, nf, nm, ns, sj, sk, ls, ps, src, dst);
        return;
    }
    long long tiles_i = (nf + 31) / 32;
    if (m0 == 1){
        long long tiles_u = (nm + 31) / 32;
        long long gx = tiles_i * tiles_u;
        dim3 grid((unsigned)std::min<long long>(gx, 1 << 20), (unsigned)std::min<long long>(ns, 65535));
        k_transpose<W, 1><<<grid, 256, 0, s>>>(nf, nm, ns, ls, ps, si, sk, reinterpret_cast<W const*>(src),
                                               reinterpret_cast<W*>(dst), tiles_i, tiles_u);
    } else {
        long long tiles_u = (ns + 31) / 32;
        long long gx = tiles_i * tiles_u;
        dim3 grid((unsigned)std::min<long long>(gx, 1 << 20), (unsigned)std::min<long long>(nm, 65535));
        k_transpose<W, 2><<<grid, 256, 0, s>>>(nf, nm, ns, ls, ps, si, sj, reinterpret_cast<W const*>(src),
                                               reinterpret_cast<W*>(dst), tiles_i, tiles_u);
    }
}

int elem_size(int dtype){
    switch (dtype){
        case DT_FLOAT: return 4;
        case DT_DOUBLE: return 8;
        case DT_CFLOAT: return 8;
        case DT_CDOUBLE: return 16;
        default: return 0;
    }
}

long long strided_extent(long long n0, long long n1, long long n2, long long ls, long long ps, char const *what){
    auto bad = [&](std::string const &why){ return Error(ST_INVALID, std::string(what) + " layout: " + why); };
    if (ls < 0 || ps < 0) throw bad("negative stride");
    // a line must not run into the next one, a plane not into the next plane
    if (n1 > 1 && ls < n0) throw bad("line stride " + std::to_string(ls) + " below the line length " + std::to_string(n0));
    long long plane = 0, span = 0, t = 0;
    if (__builtin_mul_overflow(n1 - 1, ls, &t) || __builtin_add_overflow(t, n0, &plane))
        throw bad("size overflow");
    if (n2 > 1 && ps < plane) throw bad("plane stride " + std::to_string(ps) + " below the plane extent " + std::to_string(plane));
    if (__builtin_mul_overflow(n2 - 1, ps, &t) || __builtin_add_overflow(t, plane, &span))
        throw bad("size overflow");
    return span;
}

void launch_direct_pack(cudaStream_t s, int dtype, long long nf, long long nm, long long ns, long long ls, long long ps,
                        void const *src, void *dst, bool pack){
    int es = elem_size(dtype);
    long long sls = pack ? ls : nf, sps = pack ? ps : nf * nm;
    long long dls = pack ? nf : ls, dps = pack ? nf * nm : ps;
    if (es == 4) rowcopy<uint32_t>(s, nf, nm, ns, sls, sps, dls, dps, src, dst);
    else if (es == 8) rowcopy<W8>(s, nf, nm, ns, sls, sps, dls, dps, src, dst);
    else rowcopy<W16>(s, nf, nm, ns, sls, sps, dls, dps, src, dst);
}

void launch_transpose_unpack(cudaStream_t s, int dtype, long long nf, long long nm, long long ns, long long ls,
                             long long ps, long long bls, long long bps, int m0, int m1, void const *src, void *dst){
    int es = elem_size(dtype);
    if (es == 4) transpose<uint32_t>(s, nf, nm, ns, ls, ps, bls, bps, m0, m1, src, dst);
    else if (es == 8) transpose<W8>(s, nf, nm, ns, ls, ps, bls, bps, m0, m1, src, dst);
    else transpose<W16>(s, nf, nm, ns, ls, ps, bls, bps, m0, m1, src, dst);
}

void launch_scale(cudaStream_t s, int prec, long long n, void *data, double factor){
    if (n <= 0) return;
    bool aligned = (reinterpret_cast<uintptr_t>(data) % 16) == 0;
    if (prec == 0){
        if (aligned){
            long long nv = n / 4;
            if (nv) k_scale_vec<float, float4><<<grid_for(nv, 256), 256, 0, s>>>(nv, reinterpret_cast<float4*>(data), (float)factor);
            long long rem = n - nv * 4;
            if (rem) k_scale<float><<<1, 256, 0, s>>>(rem, reinterpret_cast<float*>(data) + nv * 4, (float)factor);
        } else {
            k_scale<float><<<grid_for(n, 256), 256, 0, s>>>(n, reinterpret_cast<float*>(data), (float)factor);
        }
    } else {
        if (aligned){
            long long nv = n / 2;
            if (nv) k_scale_vec<double, double2><<<grid_for(nv, 256), 256, 0, s>>>(nv, reinterpret_cast<double2*>(data), factor);
            if (n & 1) k_scale<double><<<1, 32, 0, s>>>(1, reinterpret_cast<double*>(data) + n - 1, factor);
        } else {
            k_scale<double><<<grid_for(n, 256), 256, 0, s>>>(n, reinterpret_cast<double*>(data), factor);
        }
    }
}

void launch_convert(cudaStream_t s, int prec, long long n, void const *src, void *dst, bool to_complex){
    if (n <= 0) return;
    if (prec == 0) k_convert<float><<<grid_for(n, 256), 256, 0, s>>>(n, reinterpret_cast<float const*>(src), reinterpret_cast<float*>(dst), to_complex);
    else k_convert<double><<<grid_for(n, 256), 256, 0, s>>>(n, reinterpret_cast<double const*>(src), reinterpret_cast<double*>(dst), to_complex);
}

} // namespace gbfft
