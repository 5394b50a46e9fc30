// Inline-PTX helpers for the 5th-generation tensor cores (sm_103a): shared
// memory matrix descriptors, tcgen05.mma / commit / ld, mbarriers with bounded
// waits, and the swizzled operand layouts of the fast tensor-core kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sdbe {
namespace tc5 {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Layout field (bits 61-63) of a shared-memory descriptor.
constexpr uint32_t kNoSwizzle = 0, kSwizzle128 = 2, kSwizzle64 = 4, kSwizzle32 = 6;

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (16-byte units), descriptor version 1 (bit 46), layout.
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) |
           (static_cast<uint64_t>(layout) << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, FP16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u));
}

// The same, issued by one elected lane of a converged warp (the lowest active
// lane, the same one every time).
__device__ __forceinline__ void mma_f16_elect(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n .reg .pred p, e;\n setp.ne.b32 p, %4, 0;\n elect.sync _|e, 0xffffffff;\n"
        " @e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u));
}

// The barrier completes when every tcgen05 operation this thread issued so far has.
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

// commit() by the elected lane of a converged warp (the lane that issued the MMAs).
__device__ __forceinline__ void commit_elect(uint64_t *mbar) {
    asm volatile(
        "{\n .reg .pred e;\n elect.sync _|e, 0xffffffff;\n"
        " @e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}\n" ::"r"(smem_u32(mbar))
        : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_n(uint64_t *mbar, uint32_t n) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(n) : "memory");
}

// 2 TMEM columns of this thread's lane, no wait.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}

// 8 TMEM columns of this thread's lane, no wait.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// One try_wait on the phase with parity `parity`: the thread may sleep in it
// until the phase completes, for at most `hint_ns`.
__device__ __forceinline__ uint32_t mbar_try(uint64_t *mbar, uint32_t parity, uint32_t hint_ns) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity & 1u), "r"(hint_ns)
        : "memory");
    return done;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One try_wait without a time hint: returns at once when the phase has
// completed (the common case in a pipelined consumer, about 20 cycles).
__device__ __forceinline__ uint32_t mbar_poll(uint64_t *mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity & 1u)
        : "memory");
    return done;
}

// Bounded wait for the phase with parity `parity`: a quick poll first, then
// sleeps in try_wait rather than spinning (so waiting warps take no issue
// slots from working ones) and gives up after `limit_ns` of global time;
// false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint64_t limit_ns = 1000000000ull) {
    if (mbar_poll(mbar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try(mbar, parity, 100000u)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor cores (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 TMEM columns of this thread's lane (taddr = base | lane quarter << 16 | column), no wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// Waits for this thread's TMEM loads, then ties the N registers of each of
// a and b to an empty asm after the wait so that no use moves above it.
template <int N>
__device__ __forceinline__ void tmem_wait(uint32_t *a, uint32_t *b) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; i += 4) {
        asm volatile("" : "+r"(a[i]), "+r"(a[i + 1]), "+r"(a[i + 2]), "+r"(a[i + 3]));
        asm volatile("" : "+r"(b[i]), "+r"(b[i + 1]), "+r"(b[i + 2]), "+r"(b[i + 3]));
    }
}

// The same for one array of N registers.
template <int N>
__device__ __forceinline__ void tmem_wait1(uint32_t *a) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; i += 4) asm volatile("" : "+r"(a[i]), "+r"(a[i + 1]), "+r"(a[i + 2]), "+r"(a[i + 3]));
}

// Byte offset of the complex element (row, kc) of a K-major FP16 operand whose
// rows hold (re, im) pairs, in the 128-byte swizzle (rows of 32 complex
// values: 16-byte chunk c of row r stored at chunk c ^ (r % 8); 8-row atoms of
// 1024 bytes) and in the 64-byte swizzle (rows of 16 complex values: chunk c
// at c ^ ((r % 8) / 2); 8-row atoms of 512 bytes).  Atoms must be aligned to
// their size.
__device__ __forceinline__ uint32_t sw128_off(int row, int kc) {
    return static_cast<uint32_t>((row >> 3) * 1024 + (row & 7) * 128 + ((((kc >> 2) ^ (row & 7)) & 7) << 4) +
                                 (kc & 3) * 4);
}
__device__ __forceinline__ uint32_t sw64_off(int row, int kc) {
    return static_cast<uint32_t>((row >> 3) * 512 + (row & 7) * 64 + ((((kc >> 2) ^ ((row & 7) >> 1)) & 3) << 4) +
                                 (kc & 3) * 4);
}

// (a, b) -> the FP16 pair rn(a), rn(b) as a 32-bit word.
__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %2, %1;" : "=r"(r) : "f"(a), "f"(b));
    return r;
}

}  // namespace tc5
}  // namespace sdbe
