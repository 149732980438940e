// Helpers shared by the fused pruning kernels (CUDA-core and tensor-core).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace p4g {

constexpr double LN2 = 0.693147180559945309417232121458;

// Programmatic dependent launch: wait until the stream's previous kernel has
// completed and its writes are visible (a no-op for an ordinary launch),
// then let the next kernel launch while this one runs.  Every kernel that
// host code launches through launchPdl calls this before it reads anything
// the previous kernel may write; the next kernel can launch only once every
// block of this one has passed the wait, so whatever ran before this kernel
// is complete when the next one starts.
__device__ __forceinline__ void pdlEnter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}


// Per-thread asynchronous copies global -> shared (16 or 4 bytes, both
// addresses aligned to the size); completion is per thread: the issuing
// thread waits for its own copies before reading them.
__device__ __forceinline__ void cpAsync16(void *dstSmem, const void *srcGlobal)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dstSmem)),
                 "l"((unsigned long long)__cvta_generic_to_global(srcGlobal))
                 : "memory");
}
__device__ __forceinline__ void cpAsync4(void *dstSmem, const void *srcGlobal)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dstSmem)),
                 "l"((unsigned long long)__cvta_generic_to_global(srcGlobal))
                 : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// x = m * 2^e with m in [0.5, 1) (x > 0, subnormals included)
__device__ __forceinline__ float frexp32(float x, int *e)
{
    unsigned b = __float_as_uint(x);
    int pre = 0;
    if (((b >> 23) & 0xffu) == 0u) {
        x = x * 0x1p64f;
        b = __float_as_uint(x);
        pre = 64;
    }
    *e = (int)((b >> 23) & 0xffu) - 126 - pre;
    return __uint_as_float((b & 0x807fffffu) | (126u << 23));
}

}  // namespace p4g
