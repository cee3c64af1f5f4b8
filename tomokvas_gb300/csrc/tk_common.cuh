// tk_common.cuh -- shared device helpers for the GB300 (sm_103a) FDK kernels.
//
// Inline-PTX wrappers for mbarrier and TMA (cp.async.bulk.tensor), bounded
// waits that report instead of hanging, and the host-side error plumbing.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "../../include/tk_fdk.h"

namespace tk {

// ---------------------------------------------------------------------------
// error plumbing (host)

void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define TK_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) return ::tk::cuda_fail(_e, #call);              \
    } while (0)

#define TK_CHECK(cond, code, ...)                                              \
    do {                                                                       \
        if (!(cond)) {                                                         \
            ::tk::set_error(__VA_ARGS__);                                      \
            return (code);                                                     \
        }                                                                      \
    } while (0)

// Device-side error bits written to the error word every kernel receives.
enum : unsigned {
    ERR_BOX_OVERFLOW = 1u << 0,  // a footprint did not fit the staged box
    ERR_WAIT_TIMEOUT = 1u << 1,  // an mbarrier wait gave up
    ERR_BAD_ARGS = 1u << 2,      // kernel saw arguments it cannot handle
};

// ---------------------------------------------------------------------------
// device helpers

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: no TMA stage or MMA batch takes this long

// Wait for phase `parity` of `bar`, giving up after `limit_ns` nanoseconds
// (and after a fixed number of polls).  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && global_timer_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// 3-D tiled TMA load global -> shared, completion signalled on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// 3-D tiled TMA reduce-add shared -> global (FP32), tracked by bulk groups.
// The x coordinate must be a multiple of 16 bytes and no coordinate may be
// negative; parts beyond the tensor's extent are not written.
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap *map, int c0, int c1, int c2, const void *src)
{
    asm volatile(
        "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
        " [%0, {%1, %2, %3}], [%4];" ::"l"(reinterpret_cast<uint64_t>(map)),
        "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(src))
        : "memory");
}
__device__ __forceinline__ void bulk_commit_group() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until at most N committed bulk groups are still reading shared memory.
template <int N> __device__ __forceinline__ void bulk_wait_group_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// Wait until all committed bulk groups have completed.
__device__ __forceinline__ void bulk_wait_group_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Make this thread's shared-memory writes visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// floor(v) and frac(v) with full-rate FP32 adds: for |v| < 2^22,
// fl = v + 1.5*2^23 rounded toward -inf is an integer whose bit pattern is
// kMagicBits + floor(v).
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

}  // namespace tk
