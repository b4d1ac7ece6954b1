// Fifth-generation tensor cores (tcgen05) for the NeuralCE layer contractions: one elected thread issues
// `tcgen05.mma.cta_group::1.kind::f16` (bf16 operands in shared memory, float32 accumulator in tensor memory),
// completion is signalled on an mbarrier by `tcgen05.commit`, and the epilogue warps read the accumulator with
// `tcgen05.ld.32x32b`.
//
// Operand layout in shared memory (K-major, no swizzle): 8 x 8 bf16 "core matrices" of 128 contiguous bytes
// (8 rows of 16 bytes).  Element (row r, k) of a tile with Kp columns (Kp a multiple of 16) sits at byte
//     ((r / 8) * (Kp / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. the core matrices along K are adjacent (leading byte offset 128) and consecutive groups of 8 rows are
// Kp * 16 bytes apart (stride byte offset).  The A tile is [M = 128 rows][Kp], the B tile [N rows][Kp] (B stored
// N-major over K: B[n][k] = W[k][n]).  One MMA consumes K = 16 (two core matrices along K): step j starts at
// +256 j bytes in both tiles.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace nce {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__host__ __device__ __forceinline__ uint32_t core_off(int r, int k, int Kp) {
    return (uint32_t)((((r >> 3) * (Kp >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading byte offset (K direction), stride byte offset (8-row
// groups), descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: float32 accumulator (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N / 8 at bits 17-22, M / 16 at bits 24-28
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accum) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum) : "memory");
}

// arrive (once) on the mbarrier when every MMA issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// generic-proxy writes to shared memory made visible to the tensor cores (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// wait for the phase of the given parity to complete; gives up after `limit` polls (returns false).  The default of
// 2^20 polls is milliseconds, orders of magnitude above a tile's MMAs.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit = 1u << 20) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n" : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// tensor-memory allocation by one whole warp; the column base is written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 :: "r"(smem_u32(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive float32 columns of this thread's lane (lane quarter of the warp: warp % 4)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__host__ __device__ __forceinline__ uint32_t tmem_cols(int N) {
    uint32_t c = 32;
    while (c < (uint32_t)N) c <<= 1;
    return c;
}

// D[128 x N] (tensor memory) (+)= sum over products of A_p[128 x 16 nk] B_p[N x 16 nk]^T, issued by the calling
// thread: npass = 1 (A0 B0) or 3 (split bf16: A0 B0 + A0 B1 + A1 B0, hi/lo parts).  A and B may have different K
// extents (row-group strides a_sbo, b_sbo): the A tile can hold one K slice of a wider B operand, whose K-steps
// start at B0/B1.  accumulate = false overwrites D with the first product; then commit to mbar.
__device__ __forceinline__ void issue_tile_k(uint32_t tmem_d, const uint8_t *A0, const uint8_t *A1, uint32_t a_sbo,
                                             const uint8_t *B0, const uint8_t *B1, uint32_t b_sbo, int N, int nk,
                                             int npass, bool accumulate, uint64_t *mbar) {
    fence_after();
    const uint32_t idesc = idesc_bf16(128, N);
    const uint32_t a0 = smem_u32(A0), b0 = smem_u32(B0);
    const uint32_t a1 = npass > 1 ? smem_u32(A1) : a0, b1 = npass > 1 ? smem_u32(B1) : b0;
    uint32_t acc = accumulate ? 1u : 0u;
    for (int j = 0; j < nk; ++j) {
        const uint32_t o = (uint32_t)j * 256u;
        mma_bf16(tmem_d, sdesc(a0 + o, 128, a_sbo), sdesc(b0 + o, 128, b_sbo), idesc, acc);
        acc = 1;
        if (npass > 1) {
            mma_bf16(tmem_d, sdesc(a0 + o, 128, a_sbo), sdesc(b1 + o, 128, b_sbo), idesc, 1);
            mma_bf16(tmem_d, sdesc(a1 + o, 128, a_sbo), sdesc(b0 + o, 128, b_sbo), idesc, 1);
        }
    }
    commit(mbar);
}

// the whole K extent Kp of A and B in one call
__device__ __forceinline__ void issue_tile(uint32_t tmem_d, const uint8_t *A0, const uint8_t *A1, const uint8_t *B0,
                                           const uint8_t *B1, int N, int Kp, int npass, uint64_t *mbar) {
    issue_tile_k(tmem_d, A0, A1, (uint32_t)Kp * 16u, B0, B1, (uint32_t)Kp * 16u, N, Kp / 16, npass, false, mbar);
}

}  // namespace umma
}  // namespace nce
