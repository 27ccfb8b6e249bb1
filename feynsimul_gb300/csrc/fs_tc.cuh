// fs_tc.cuh -- fifth-generation tensor-core (tcgen05) helpers shared by the learned
// proposal's batched inference (fs_mlp_tc.cu) and training (fs_mlp_train.cu) kernels: the
// no-swizzle canonical shared-memory layout, matrix and instruction descriptors, the MMA
// issue, its completion barrier (every wait bounded) and the tensor-memory loads.  No
// counterpart in the reference.
//
// Canonical layout of a tile stored "row-major" with K columns (tc_off): 8 x 8 BF16 core
// matrices of 128 contiguous bytes (8 rows of 8 consecutive columns); core matrices adjacent
// along the columns 128 bytes apart, 8-row groups K * 16 bytes apart.  Read as a K-major
// operand (rows = M or N, columns = K) its leading byte offset (next core matrix along K) is
// 128 and its stride byte offset (next 8 rows of M / N) K * 16.  Read as an MN-major operand
// (rows = K, columns = M or N: the transposed matrix, e.g. the activations as the B operand
// of a weight gradient) the same bytes have the leading byte offset K * 16 (next 8 rows,
// i.e. along K) and the stride byte offset 128 (next 8 columns of M / N).
#pragma once
#include <stdint.h>

#ifndef TC_SPIN_LIMIT
#define TC_SPIN_LIMIT (1u << 20)  // try_wait polls before a CTA gives up
#endif

typedef unsigned short fs_bf16;

// element offset of (row r, column k) in a K-major canonical tile with K columns
__device__ __forceinline__ int tc_off(int r, int k, int K)
{
    return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading and stride byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc_lbo_sbo(const fs_bf16 *start, uint32_t lbo, uint32_t sbo)
{
    const uint64_t a = (tc_smem(start) >> 4) & 0x3FFFu;
    return a | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// K-major operand of a tile with K columns: leading byte offset 128 (next core matrix along
// K), stride byte offset K * 16 (next 8-row group)
__device__ __forceinline__ uint64_t tc_desc(const fs_bf16 *start, int K)
{
    return tc_desc_lbo_sbo(start, 128u, (uint32_t)K * 16u);
}

// MN-major operand read from a tile stored with W columns (the columns are M or N, the rows
// K): leading byte offset W * 16 (next 8 rows, along K), stride byte offset 128 (next 8
// columns)
__device__ __forceinline__ uint64_t tc_desc_mn(const fs_bf16 *start, int W)
{
    return tc_desc_lbo_sbo(start, (uint32_t)W * 16u, 128u);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B; mn_a / mn_b mark an
// MN-major ("transposed") operand
__device__ __forceinline__ uint32_t tc_idesc(int M, int N, bool mn_a = false, bool mn_b = false)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((mn_a ? 1u : 0u) << 15) | ((mn_b ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// bounded wait for the barrier phase with this parity; false when the limit is reached
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity)
{
    for (uint32_t i = 0; i < TC_SPIN_LIMIT; i++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(mbar), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores' reads
__device__ __forceinline__ void tc_fence_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 FP32 accumulator columns of this thread's TMEM lane, the load completed before return
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];\n\ttcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// eight BF16 values (k .. k+7 of one row) as one 16-byte shared store
__device__ __forceinline__ void tc_st8(fs_bf16 *dst, const float *h)
{
    uint4 u;
    u.x = fs_pack_bf16(h[0], h[1]);
    u.y = fs_pack_bf16(h[2], h[3]);
    u.z = fs_pack_bf16(h[4], h[5]);
    u.w = fs_pack_bf16(h[6], h[7]);
    *(uint4 *)dst = u;
}

