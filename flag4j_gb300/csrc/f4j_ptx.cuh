// f4j_ptx.cuh -- inline-PTX helpers for sm_103a: mbarriers with bounded
// waits, TMA tiled loads, and the tcgen05 (TMEM / UMMA) instructions.
#pragma once
#include <cuda.h>
#include <cstdint>

// Every spin-wait gives up after this many polls (each try_wait may suspend
// for a short hint), records a code in the status word and lets the caller
// unwind.  A healthy pipeline never comes close.
#ifndef F4J_WAIT_LIMIT
#define F4J_WAIT_LIMIT (1u << 26)
#endif

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t f4j_globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: returns false (after recording `code`) if the phase has not
// completed within F4J_WAIT_NS nanoseconds of wall time (or F4J_WAIT_LIMIT
// polls, whichever comes first).  Healthy waits last micro- to milliseconds.
#ifndef F4J_WAIT_NS
#define F4J_WAIT_NS 2000000000ull
#endif
__device__ __forceinline__ bool mbar_wait_ns(uint64_t* bar, uint32_t parity, int* status, int code,
                                             uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = f4j_globaltimer_ns();
    for (uint32_t it = 0; it < F4J_WAIT_LIMIT; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && f4j_globaltimer_ns() - t0 > limit_ns) break;
    }
    if (status) atomicExch(status, code);
    return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status, int code) {
    return mbar_wait_ns(bar, parity, status, code, F4J_WAIT_NS);
}

// Asynchronous 4- / 8-byte copies global -> shared (no register staging; the
// source and destination are aligned to the copy size), and the wait for all
// of this thread's copies.  Other lanes see the data after a __syncwarp.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// 2-D / 3-D TMA tiled loads into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------------- tcgen05
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f8f6f4, one CTA.
__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Two MMAs accumulating into d_tmem over consecutive K = 32 steps of 64-byte
// swizzled rows: descriptor low words a_lo, b_lo (the second step 32 bytes on),
// shared high word hi.
__device__ __forceinline__ void umma_f8_k64(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo, uint32_t hi,
                                            uint32_t idesc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t.reg .b32 a1, b1;\n\t"
        "setp.ne.b32 p, %5, 0;\n\t"
        "mov.b64 da, {%1, %3};\n\tmov.b64 db, {%2, %3};\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], da, db, %4, p;\n\t"
        "add.u32 a1, %1, 2;\n\tadd.u32 b1, %2, 2;\n\t"
        "mov.b64 da, {a1, %3};\n\tmov.b64 db, {b1, %3};\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], da, db, %4, p;\n\t}" ::"r"(d_tmem),
        "r"(a_lo), "r"(b_lo), "r"(hi), "r"(idesc), "r"(1u)
        : "memory");
}

// Arrive on `bar` once all prior tcgen05.mma of this thread have completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 columns of 32-bit TMEM words into 32 registers per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// 32 lanes x 16 columns of 32-bit TMEM words into 16 registers per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 32 columns of 32-bit TMEM words set to zero.
__device__ __forceinline__ void tmem_zero32(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr),
        "r"(z)
        : "memory");
}

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor for a K-major operand tile written by TMA
// with 128-byte swizzle: rows of 128 bytes, 8-row swizzle atoms 1024 bytes
// apart (stride byte offset), leading byte offset unused for this layout.
__device__ __forceinline__ uint64_t umma_desc_sw128(const void* smem_tile) {
    uint64_t addr = smem_u32(smem_tile);
    uint64_t d = 0;
    d |= (addr & 0x3FFFFull) >> 4;          // bits 0-13: start address >> 4
    d |= (uint64_t)(16 >> 4) << 16;         // bits 16-29: leading byte offset >> 4 (ignored)
    d |= (uint64_t)(1024 >> 4) << 32;       // bits 32-45: stride byte offset >> 4
    d |= (uint64_t)1 << 46;                 // bits 46-47: descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                 // bits 61-63: swizzle mode 2 = 128-byte
    return d;
}

// Same for 64-byte rows written with 64-byte swizzle: 8-row atoms of 512 bytes.
__device__ __forceinline__ uint64_t umma_desc_sw64(const void* smem_tile) {
    uint64_t addr = smem_u32(smem_tile);
    uint64_t d = 0;
    d |= (addr & 0x3FFFFull) >> 4;          // bits 0-13: start address >> 4
    d |= (uint64_t)(16 >> 4) << 16;         // bits 16-29: leading byte offset >> 4 (ignored)
    d |= (uint64_t)(512 >> 4) << 32;        // bits 32-45: stride byte offset >> 4
    d |= (uint64_t)1 << 46;                 // bits 46-47: descriptor version (sm_100 family)
    d |= (uint64_t)4 << 61;                 // bits 61-63: swizzle mode 4 = 64-byte
    return d;
}

// Instruction descriptor, kind::f8f6f4: E4M3 x E4M3 -> F32, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_e4m3_f32(int M, int N) {
    return (1u << 4)                       // bits 4-5: D format F32
           | (0u << 7)                     // bits 7-9: A format E4M3
           | (0u << 10)                    // bits 10-12: B format E4M3
           | ((uint32_t)(N >> 3) << 17)    // bits 17-22: N >> 3
           | ((uint32_t)(M >> 4) << 24);   // bits 24-28: M >> 4
}
