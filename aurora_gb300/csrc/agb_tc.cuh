// Blackwell (sm_103a) tensor-core building blocks in inline PTX: tensor memory (TMEM) allocation,
// tcgen05.mma with BF16 operands and FP32 accumulators in TMEM, mbarrier completion tracking,
// TMEM loads for the epilogue and 1D bulk (TMA) copies into shared memory.
//
// Operand layout in shared memory: K-major, no swizzle.  A tile of R rows x 16 K-elements (BF16)
// is stored as (R / 8) x 2 core matrices of 8 rows x 16 bytes (128 contiguous bytes each, rows of
// 16 bytes); core (g, h) (row group g, K half h) sits at byte (g * 2 + h) * 128.  In the matrix
// descriptor the leading byte offset (between K-adjacent core matrices) is 128 and the stride byte
// offset (between row-adjacent core matrices) is 256.  One MMA instruction consumes K = 16.
//
// Every wait is bounded: a wait that runs out reports failure to the caller, which records an
// error flag, and the kernel still releases its TMEM and returns.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace agb
{
namespace tc
{

constexpr uint32_t kCoreBytes   = 128;  // one 8 x 16-byte core matrix
constexpr uint32_t kSliceLbo    = 128;  // K-adjacent core matrices
constexpr uint32_t kSliceSbo    = 256;  // row-adjacent core matrices
constexpr uint32_t kWaitSpins   = 1u << 22;

__device__ __forceinline__ uint32_t smemAddr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) (k in [0, 16)) inside one K16 slice.
__device__ __forceinline__ uint32_t sliceOffset(uint32_t row, uint32_t k)
{
    return (((row >> 3) * 2 + (k >> 3)) * kCoreBytes) + (row & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading and stride byte
// offsets (all >> 4), descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= uint64_t((addr >> 4) & 0x3FFFu);
    d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// Shared-memory descriptor of a K-major operand in the 32-byte swizzle layout (rows of 32 bytes =
// one K16 block of BF16, 8-row atoms `sbo` bytes apart; the leading byte offset is unused):
// layout type 6 in bits 61-63.
__device__ __forceinline__ uint64_t smemDescSw32(uint32_t addr, uint32_t sbo)
{
    return smemDesc(addr, 16, sbo) | (uint64_t(6) << 61);
}

// Instruction descriptor of tcgen05.mma.kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits
// 24-28.
__host__ __device__ constexpr uint32_t idescBf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fenceMbarInit()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Bounded wait for the given phase parity; false when it did not complete.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity)
{
    uint32_t addr = smemAddr(bar);
    for (uint32_t i = 0; i < kWaitSpins; i++)
    {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(addr), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}

// 1D bulk copy global -> shared (TMA, no tensor map); completion counted on the mbarrier.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
                 : "memory");
}

// Tiled tensor copies global -> shared through a tensor map (TMA); completion counted on the
// mbarrier.  Coordinates are in elements, innermost first; elements outside the tensor read as
// zero.  The innermost coordinate times the element size must be a multiple of 16 bytes, and dst
// 128-byte aligned.
__device__ __forceinline__ void tensorLoad4(void* dst, const void* map, int c0, int c1, int c2, int c3,
    uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                 "%4, %5}], [%6];" ::"r"(smemAddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smemAddr(bar))
                 : "memory");
}
__device__ __forceinline__ void tensorLoad5(void* dst, const void* map, int c0, int c1, int c2, int c3, int c4,
    uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                 "%4, %5, %6}], [%7];" ::"r"(smemAddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smemAddr(bar))
                 : "memory");
}
// Plain arrival (no transaction bytes).
__device__ __forceinline__ void mbarArrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}

__device__ __forceinline__ void fenceProxyAsync()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fenceBeforeSync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fenceAfterSync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// TMEM allocation by one whole warp; the column address is written to *dst (shared memory).
__device__ __forceinline__ void tmemAlloc(uint32_t* dst, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dst)),
        "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// D (TMEM) (+)= A (smem) x B (smem)^T, issued by one thread.
__device__ __forceinline__ void mma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
    uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
        "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}
// The mbarrier receives one arrival once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smemAddr(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread i of the warp gets lane (base lane + i).
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                 "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmemWaitLoad()
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMEM columns to allocate for N FP32 accumulator columns (power of two, at least 32).
__host__ __device__ constexpr uint32_t tmemCols(uint32_t n)
{
    return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}

} // namespace tc
} // namespace agb
