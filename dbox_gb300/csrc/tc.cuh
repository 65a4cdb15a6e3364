// Fifth-generation tensor core (tcgen05) helpers for sm_103a: tensor-memory allocation,
// shared-memory matrix descriptors, single-thread MMA issue with mbarrier completion, and
// tensor-memory loads.  Operands live in shared memory in the 128-byte-swizzled layout:
// a tile of R rows x 64 bf16 (one 128-byte row per row, 16-byte chunks XOR-ed with the row
// index modulo 8) is one "atom"; wider tiles are atoms side by side (`atom_bytes` apart).
// Read K-major (rows = M or N, columns = K) such a tile is the MN-major layout of its
// transpose (leading byte offset = atom_bytes, stride byte offset = 1024), so every tile
// is stored once and used either way through its descriptor.
#pragma once
#include <stdint.h>

namespace dg {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, col) in a swizzled tile of `rows` rows (atoms of 64 columns)
__device__ __forceinline__ uint32_t sw128_offset(int row, int col, int rows) {
    const int atom = col >> 6, c = col & 63;
    return (uint32_t)(atom * rows * 128 + row * 128 + (((c >> 3) ^ (row & 7)) << 4) + ((c & 7) << 1));
}

// shared-memory matrix descriptor (start address, leading / stride byte offsets, 128-byte swizzle)
__device__ __forceinline__ uint64_t desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;                        // descriptor version of this architecture
    d |= (uint64_t)2 << 61;                        // 128-byte swizzle
    return d;
}
// operand descriptor for k-step ks (16 elements of K) of a K-major tile (`atom_bytes` per atom)
__device__ __forceinline__ uint64_t desc_k(uint32_t base, int ks, uint32_t atom_bytes) {
    return desc(base + (uint32_t)(ks >> 2) * atom_bytes + (uint32_t)(ks & 3) * 32u, 16u, 1024u);
}
// operand descriptor for k-step ks of an MN-major read of a tile stored K-major by rows = K
// (the transpose): two 8-row groups per k-step, MN atoms `atom_bytes` apart
__device__ __forceinline__ uint64_t desc_mn(uint32_t base, int ks, uint32_t atom_bytes) {
    return desc(base + (uint32_t)ks * 2048u, atom_bytes, 1024u);
}

// instruction descriptor of kind::f16 with bf16 operands and an f32 accumulator
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B, issued by one thread
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate) : "memory");
}
// arrive on `bar` once every MMA issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// wait for phase `parity` of `bar`; false when `limit` polls ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
    const uint32_t b = smem_addr(bar);
    for (int i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(b), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// tensor memory: one warp allocates / frees `ncols` columns (a power of two, 32..512)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(dst_smem)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive f32 columns of this thread's tensor-memory lane (the warp's 32 lanes), loaded
// and waited for: the wait names the registers, so nothing that reads them is scheduled
// before the load has completed
__device__ __forceinline__ void ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace tc
}  // namespace dg
