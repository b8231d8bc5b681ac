// tc.cuh -- inline-PTX helpers for the 5th-generation tensor cores
// (tcgen05.mma kind::tf32 from shared-memory descriptors, tensor-memory
// allocation and loads, mbarrier commit and bounded waits) and cp.async,
// shared by the mixed-precision kernels.
//
// Shared-memory operands are canonical K-major tiles without swizzle: core
// matrices of 8 rows x 16 bytes (4 TF32) stored as 128 contiguous bytes;
// core matrix (row group g, K group q) of a tile with K extent kc at
// (g * kc/4 + q) * 128 bytes, so that the descriptor's leading (K) byte
// offset is 128 and its stride (row-group) byte offset kc * 32.
#pragma once
#include <cstdint>

namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t desc_kmajor_noswizzle(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;     // descriptor version for tcgen05
    // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
    return d;
}

// K-major operand with 64-byte swizzling: rows of 64 bytes (16 TF32 of K),
// eight-row groups of 512 bytes sbo apart, the 16-byte chunk c of row r
// stored at chunk c ^ ((r >> 1) & 3) (the tile based on a 512-byte
// boundary); the leading byte offset is unused for this layout (1)
__device__ __forceinline__ uint64_t desc_kmajor_sw64(uint32_t saddr, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;     // descriptor version for tcgen05
    d |= (uint64_t)4 << 61;     // swizzling mode: 64 bytes
    return d;
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, K-major, M x N
__host__ __device__ __forceinline__ uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Warp-collective issue: every lane of a converged warp passes the same
// (warp-uniform) operands and one lane, picked once by elect.sync, issues --
// the same lane for the MMAs and their commit, so the commit tracks them.
// the elected lane of a converged warp (1 there, 0 elsewhere); the forms
// below take it, so that one election serves all of a round's MMAs
__device__ __forceinline__ uint32_t elect_lane()
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred e;\n\t.reg .b32 x;\n\t"
        "elect.sync x|e, 0xffffffff;\n\t"
        "selp.u32 %0, 1, 0, e;\n\t}\n"
        : "=r"(r));
    return r;
}

__device__ __forceinline__ void mma_tf32_lead(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc,
                                              uint32_t lead)
{
    asm volatile(
        "{\n\t.reg .pred p, e;\n\t"
        "setp.ne.b32 e, %5, 0;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc), "r"(lead));
}

__device__ __forceinline__ void commit_lead(uint64_t* mbar, uint32_t lead)
{
    asm volatile(
        "{\n\t.reg .pred e;\n\t"
        "setp.ne.b32 e, %1, 0;\n\t"
        "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}\n" ::"r"(
            smem_u32(mbar)),
        "r"(lead)
        : "memory");
}


__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred P;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, P;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the mbarrier, at most limit_ns; true if it
// completed (the clock is read only when the first try fails)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(mbar, parity)) return true;
    const uint64_t t0 = now_ns();
    for (;;) {
        if (mbar_try_wait(mbar, parity)) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// FP32 -> TF32, round to nearest, ties away from zero, on the bits: finite
// inputs (a carry into the exponent gives the next binade, as it should)
__device__ __forceinline__ float tf32_rna(float x)
{
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// asynchronous global -> shared copies (16 bytes through L2 only, 8 bytes)
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
                 "l"((unsigned long long)__cvta_generic_to_global(src))
                 : "memory");
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)),
                 "l"((unsigned long long)__cvta_generic_to_global(src))
                 : "memory");
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)),
                 "l"((unsigned long long)__cvta_generic_to_global(src))
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

}  // namespace tc
