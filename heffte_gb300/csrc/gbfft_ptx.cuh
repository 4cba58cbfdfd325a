// Inline-PTX helpers for the asynchronous (TMA bulk copy + mbarrier) data
// path on sm_103a.  Every wait is bounded: it gives up after a clock budget
// and reports through a device status word instead of spinning forever.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfft {

// status codes written by kernels into the device status word
enum { DEV_OK = 0, DEV_TIMEOUT_BULK_COPY = 1, DEV_TIMEOUT_DEPENDENCY = 2, DEV_TIMEOUT_MMA = 3 };

// Default clock budget of every bounded wait (about two seconds at 2 GHz).
// The waits for bulk copies and for tensor-core MMAs keep it: a CTA that gave
// up on them early would return while a copy or an MMA may still write its
// shared or tensor memory.  The batch kernel's wait for another CTA's pass of
// the same box has nothing of its own in flight, so its budget is a launch
// argument that can be shortened (heffte_gb300_set_dependency_wait_budget).
constexpr long long kWaitBudgetClocks = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(void const *p){
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count){
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

// make mbarrier initialisation visible to the async proxy (bulk copies)
__device__ __forceinline__ void fence_mbar_init(){
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy shared-memory accesses before
// subsequent async-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async_smem(){
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes){
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity){
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Waits for phase `parity` of the barrier; gives up after ~`budget` clocks,
// records DEV_TIMEOUT_BULK_COPY in *status and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *status,
                                                  long long budget = kWaitBudgetClocks){
    if (mbar_try_wait(bar, parity)) return true;
    long long t0 = clock64();
    while (true){
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > budget){
            if (status) atomicExch(status, DEV_TIMEOUT_BULK_COPY);
            return false;
        }
    }
}

// Tiled 3-D tensor copy global -> shared (TMA) completing on an mbarrier.
// tmap is the address of a CUtensorMap kernel parameter (__grid_constant__).
// The innermost coordinate times the element size must be a multiple of 16.
__device__ __forceinline__ void tma_load_3d(void *dst_smem, void const *tmap, int c0, int c1, int c2, uint64_t *bar){
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(smem_u32(dst_smem)), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2),
                    "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void prefetch_tmap(void const *tmap){
    asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

// 1-D bulk copy global -> shared completing on an mbarrier (transaction bytes).
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst_smem, void const *src_gmem, uint32_t bytes, uint64_t *bar){
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// 1-D bulk copy shared -> global, tracked by bulk groups of the issuing
// thread.  dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_s2g(void *dst_gmem, void const *src_smem, uint32_t bytes){
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                 :: "l"(dst_gmem), "r"(smem_u32(src_smem)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit(){ asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// until at most NG of this thread's bulk groups still read their shared source
template<int NG> __device__ __forceinline__ void bulk_wait_read(){
    asm volatile("cp.async.bulk.wait_group.read %0;" :: "n"(NG) : "memory");
}
// until at most NG of this thread's bulk groups are incomplete
template<int NG> __device__ __forceinline__ void bulk_wait(){
    asm volatile("cp.async.bulk.wait_group %0;" :: "n"(NG) : "memory");
}

} // namespace gbfft
