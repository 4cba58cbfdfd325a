// In-place transpose-unpack that allocates nothing.
//
// Some callers cannot call cudaMalloc: programs whose device memory is owned
// by an arena or pool that forbids allocations outside it, real-time loops
// that must not allocate after start-up (an allocation can synchronise the
// device and take an unbounded time), and callers already at the memory limit
// for whom an extra buffer the size of the box is not available.  They still
// need the reshape step that reads and writes the same buffer, which
// otherwise needs a second buffer as large as the box.
//
// This entry point keeps its scratch space in one file-scope device array of
// a fixed size (kNoAllocScratchBytes below).  Every GPU that loads the library
// reserves that array until the process exits.  The device address of the
// array is looked up once per device, on the first call made while that
// device is current (and again on the first call after cudaDeviceReset made a
// new context); make that first call before any stream capture begins.
// All calls share the array and it keeps the last call's contents; calls
// whose work overlaps on the GPU (for example on two streams) race on it.
// The copy into the array and the transpose are enqueued on the caller's
// stream; nothing here calls cudaMalloc, cudaFree or an allocating library.
#include "gbfft_plan.h"
#include "../../include/heffte_gb300.h"
#include <cuda.h>

namespace gbfft {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (no
// link dependency on libcuda); null when the driver does not offer them.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

template<typename F>
F driver_fn(char const *name){
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess){
        cudaGetLastError();
        return nullptr;
    }
    return reinterpret_cast<F>(p);
}

// Unique id of the current context (0 when it cannot be read).  A context
// made after cudaDeviceReset gets a new id, so the cached address below is
// looked up again rather than reused.
unsigned long long current_context_id(){
    static CtxGetCurrentFn get_ctx = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
    static CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_ctx || !get_id || get_ctx(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array for the current device.  The host-side
// symbol is only a handle, so the address is looked up with
// cudaGetSymbolAddress once per device (and context), with that device current.
void *noalloc_scratch(){
    struct Entry { void *ptr; unsigned long long ctx; };
    static Entry cache[64] = {};
    static std::mutex mu;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) throw Error(ST_UNSUPPORTED, "device index out of range for the no-allocation scratch table");
    unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(mu);
    Entry &e = cache[dev];
    if (!e.ptr || e.ctx != ctx){
        void *p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-allocation scratch)");
        e.ptr = p;
        // the lookup makes the context if there was none yet: key on its id now
        e.ctx = current_context_id();
    }
    return e.ptr;
}

} // namespace
} // namespace gbfft

using namespace gbfft;

extern "C" int heffte_gb300_transpose_unpack_inplace_noalloc(void *stream, int dtype, long long nfast, long long nmid,
                                                             long long nslow, long long line_stride,
                                                             long long plane_stride, long long buff_line_stride,
                                                             long long buff_plane_stride, int map0, int map1, int map2,
                                                             void *data){
    try {
        if (dtype < 0 || dtype > 3) throw Error(ST_INVALID, "unknown element type code " + std::to_string(dtype));
        if (nfast < 0 || nmid < 0 || nslow < 0) throw Error(ST_INVALID, "negative size");
        int m[3] = {map0, map1, map2};
        if (!valid_order({map0, map1, map2})) throw Error(ST_INVALID, "map must be a permutation of 0, 1, 2");
        if (nfast == 0 || nmid == 0 || nslow == 0){
            set_last_error("");
            return HEFFTE_GB300_SUCCESS;
        }
        if (!data) throw Error(ST_INVALID, "null pointer");
        // the source occupies the buffer in its own layout: its a-th dimension
        // (fast, mid, slow) is the destination dimension map[a]; both layouts
        // are checked (non-negative, non-overlapping strides, no overflow)
        // before the span of the source is compared with the scratch size
        long long size[3] = {nfast, nmid, nslow};
        strided_extent(nfast, nmid, nslow, line_stride, plane_stride, "destination");
        long long extent = strided_extent(size[m[0]], size[m[1]], size[m[2]], buff_line_stride, buff_plane_stride,
                                          "source");
        long long es = elem_size(dtype);
        if (extent > (long long)(kNoAllocScratchBytes / (size_t)es))
            throw Error(ST_INVALID, "the source of " + std::to_string(extent) + " elements of " + std::to_string(es) +
                        " bytes exceeds the " + std::to_string(kNoAllocScratchBytes >> 20) +
                        " MiB scratch of the no-allocation transpose");
        size_t bytes = (size_t)extent * (size_t)es;
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        void *scratch = noalloc_scratch();
        check_cuda(cudaMemcpyAsync(scratch, data, bytes, cudaMemcpyDeviceToDevice, s), "copy into no-allocation scratch");
        launch_transpose_unpack(s, dtype, nfast, nmid, nslow, line_stride, plane_stride, buff_line_stride,
                                buff_plane_stride, map0, map1, scratch, data);
        check_cuda(cudaPeekAtLastError(), "transpose_unpack kernel launch");
        set_last_error("");
        return HEFFTE_GB300_SUCCESS;
    } catch (Error const &e){
        set_last_error(e.what());
        return e.code;
    } catch (std::exception const &e){
        set_last_error(e.what());
        return HEFFTE_GB300_INVALID;
    }
}
