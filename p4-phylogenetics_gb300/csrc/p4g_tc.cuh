// Blackwell (sm_103a) tensor-core building blocks used by the protein
// pruning kernel: tensor-memory allocation, tcgen05 loads/stores, the
// kind::tf32 MMA with A in tensor memory and B in shared memory, commit to an
// mbarrier and bounded waits.  Inline PTX only.
//
// Layout conventions used throughout (cta_group::1, M = 128):
//  * tensor memory address = (lane << 16) | column; lane = row of A / D,
//    one 32-bit element per column;
//  * a warp reaches lanes [32 * (warp % 4), 32 * (warp % 4) + 32) with the
//    32x32b tcgen05.ld / tcgen05.st shapes, thread t of the warp = lane
//    32 * (warp % 4) + t;
//  * B (N x K, K-major) in shared memory without swizzle, as 8-row x 16-byte
//    core matrices: core matrix (n / 8, k / 4) at
//    (n / 8) * SBO + (k / 4) * LBO, row n % 8 at +16 * (n % 8), element
//    k % 4 at +4 * (k % 4).
#pragma once
#include <stdint.h>

namespace p4g {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Instruction descriptor of tcgen05.mma kind::tf32: D F32, A and B TF32,
// both K-major, no negation, dense, M x N.
__host__ __device__ constexpr uint32_t idescTf32(int M, int N)
{
    return (1u << 4)                       // D format: F32
           | (2u << 7)                     // A format: TF32
           | (2u << 10)                    // B format: TF32
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// Shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;               // descriptor version for tcgen05
    return d;                              // base offset 0, layout type 0 (no swizzle)
}

// ---- tensor memory allocation (one full warp executes these)
__device__ __forceinline__ void tmemAlloc(uint32_t *dstSmem, uint32_t nCols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dstSmem)),
                 "r"(nCols)
                 : "memory");
}
__device__ __forceinline__ void tmemRelinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t nCols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(nCols) : "memory");
}

// ---- fences
__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void waitSt() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void waitLd() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// The same wait naming the 24 registers three ld8 loads filled, so that no use
// of them can be scheduled before it.
__device__ __forceinline__ void waitLd24(float (&v)[3][8])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0][0]), "+f"(v[0][1]), "+f"(v[0][2]), "+f"(v[0][3]), "+f"(v[0][4]), "+f"(v[0][5]),
                   "+f"(v[0][6]), "+f"(v[0][7]), "+f"(v[1][0]), "+f"(v[1][1]), "+f"(v[1][2]), "+f"(v[1][3]),
                   "+f"(v[1][4]), "+f"(v[1][5]), "+f"(v[1][6]), "+f"(v[1][7]), "+f"(v[2][0]), "+f"(v[2][1]),
                   "+f"(v[2][2]), "+f"(v[2][3]), "+f"(v[2][4]), "+f"(v[2][5]), "+f"(v[2][6]), "+f"(v[2][7])
                 :
                 : "memory");
}

// ---- 32x32b loads / stores of 8 consecutive columns
__device__ __forceinline__ void st8(uint32_t taddr, const float (&v)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// ---- MMA: D[tmem] (+)= A[tmem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mmaTf32TS(uint32_t dTaddr, uint32_t aTaddr, uint64_t bDesc, uint32_t idesc,
                                          bool accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(dTaddr),
        "r"(aTaddr), "l"(bDesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// The mbarrier arrives once every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smemAddr(mbar))
                 : "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbarInit(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(mbar)), "r"(count) : "memory");
}
// One potentially blocking test of phase `parity`: the thread may sleep up to
// suspendNs nanoseconds waiting for the phase before the test returns false.
__device__ __forceinline__ bool mbarTryWait(uint64_t *mbar, uint32_t parity, uint32_t suspendNs)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(mbar)), "r"(parity), "r"(suspendNs)
        : "memory");
    return ok != 0;
}
// Bounded wait for phase `parity` of an mbarrier: false if it did not
// complete within maxIter tests of at most 1 us each (the caller records an
// error and stops).
__device__ __forceinline__ bool mbarWait(uint64_t *mbar, uint32_t parity, int maxIter = (1 << 21))
{
    for (int i = 0; i < maxIter; i++)
        if (mbarTryWait(mbar, parity, 1000u)) return true;
    return false;
}

// One arrival on an mbarrier (completes the phase of a count-1 barrier).
__device__ __forceinline__ void mbarArrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(mbar)) : "memory");
}

// ---- untiled bulk copy (TMA) global -> shared, completing on an mbarrier.
// Both addresses 16-byte aligned, bytes a multiple of 16.  The issuing
// thread first arms the barrier with the bytes it expects (this is the
// barrier's one arrival for the phase).
__device__ __forceinline__ void mbarExpectTx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(mbar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulkLoad(void *dstSmem, const void *srcGlobal, uint32_t bytes, uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smemAddr(dstSmem)),
        "l"((unsigned long long)__cvta_generic_to_global(srcGlobal)), "r"(bytes), "r"(smemAddr(mbar))
        : "memory");
}

// FP32 -> TF32 by round-to-nearest (ties away), as the split-precision
// product needs: hi = tf32(x), lo = tf32(x - hi).
__device__ __forceinline__ float toTf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

}  // namespace tc
}  // namespace p4g
