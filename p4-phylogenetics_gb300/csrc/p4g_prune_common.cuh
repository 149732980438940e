// Helpers shared by the fused pruning kernels (CUDA-core and tensor-core).
#pragma once
#include <cuda_runtime.h>

namespace p4g {

constexpr double LN2 = 0.693147180559945309417232121458;

// Programmatic dependent launch: wait until the stream's previous kernel has
// completed and its writes are visible (a no-op for an ordinary launch),
// then let the next kernel launch while this one runs.  Every kernel that
// host code launches through launchPdl begins with this.
__device__ __forceinline__ void pdlEnter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

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
