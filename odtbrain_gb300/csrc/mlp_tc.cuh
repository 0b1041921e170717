// Learned-gain MLP inference on the 5th-generation tensor cores: tcgen05.mma
// with operands in shared memory and the FP32 accumulator in tensor memory
// (TMEM), read back with tcgen05.ld for the bias + SiLU epilogue.
//
// A CTA runs two tiles of 128 points at a time, one per warp group of 128
// threads (thread = point = TMEM lane).  Per layer, the group writes its
// BF16 activations (the A operand, 128 x K) into shared memory, one elected
// thread issues the MMAs against the layer's weights (the B operand, kept in
// shared memory for the CTA's lifetime) and commits them to the group's
// mbarrier, and the group reads the 128 x N FP32 result from its TMEM
// columns.  While one group is in its epilogue the tensor pipe works on the
// other group's MMAs.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, row r and 16-byte K chunk c at
//   (r / 8) * SBO + c * 128 + (r % 8) * 16,   SBO = 128 * (K / 8),
// so the descriptor's leading-dimension byte offset (between the two core
// matrices of a K = 16 step) is 128 and its stride-dimension byte offset
// (between 8-row groups) SBO; the k-th K = 16 step starts 256 * k bytes in.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "odt_tma.cuh"

namespace odt {
namespace tc {

// byte offset of (row, 16-byte chunk) in a K-major operand of kchunks chunks
__host__ __device__ constexpr uint32_t kmaj(int row, int chunk, int kchunks)
{
    return (uint32_t)((row >> 3) * (128 * kchunks) + chunk * 128 + (row & 7) * 16);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all >> 4), the fixed 0b001 at bits 46-48,
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) = A * B (+ D when accumulate), issued by one thread.
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// TMEM allocation by one whole warp; the base address is written to
// shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape:
// warp w of a warp group reads lanes 32*(w % 4) ..).  The registers hold
// the values only after tmem_wait: use them through it.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

// Wait for this thread's outstanding tcgen05.ld; the registers pass
// through the wait, so no use of them is scheduled before it.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

}  // namespace tc
}  // namespace odt
