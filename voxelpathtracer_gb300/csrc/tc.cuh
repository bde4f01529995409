// Blackwell tensor-core primitives for sm_103a, as inline PTX: tcgen05.mma
// (kind::f16 with BF16 operands, FP32 accumulators in tensor memory), TMEM
// allocation and loads, shared-memory matrix descriptors and mbarriers.
//
// Operand tiles are staged in shared memory in the canonical K-major layout
// without swizzle: the tile is cut into "core matrices" of 8 rows x 16 bytes
// (8 BF16 values of K), each 128 contiguous bytes with row r at +16r. Core
// matrices adjacent along K are LBO bytes apart and those adjacent along M
// (or N) are SBO bytes apart. Every helper here uses LBO = 128 (K-adjacent
// core matrices contiguous) and SBO = K_tile * 16, so element (r, k) of a tile
// with K_tile columns sits at
//     (r / 8) * K_tile * 16 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// One MMA consumes K = 16, i.e. two core matrices along K; the k-th MMA of a
// tile starts 256 * k bytes after the tile.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace vpt {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__host__ __device__ __forceinline__ uint32_t tile_offset(int r, int k, int ktile) {
    return (uint32_t)((r >> 3) * ktile * 16 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4),
// descriptor version 1 (bits 46-47), no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Descriptor of a swizzled K-major tile: rows of `row_bytes` (32 or 64; the
// TMA box's inner extent) written with the matching TMA swizzle, 8-row
// atoms SBO = 8 * row_bytes apart; layout type 6 = 32-byte swizzle, 4 =
// 64-byte swizzle (bits 61-63). A K step inside the row advances the start
// address by its byte offset.
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t saddr, uint32_t row_bytes) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                                   // LBO (unused for these layouts)
    d |= (uint64_t)(((8u * row_bytes) >> 4) & 0x3FFFu) << 32;  // SBO
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)(row_bytes == 64u ? 4u : 6u) << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 D (bits 4-5 = 1), BF16 A and B
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on the mbarrier once every MMA this thread issued so far is complete.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One warp allocates `ncols` (power of two, >= 32) TMEM columns; the base
// address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w of a
// warpgroup reads lanes 32w..32w+31; taddr carries the lane in bits 16-31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase of `parity` with an iteration limit. On timeout it
// records `where` in *err (first failure wins) and returns false; the caller
// then stops issuing work, waits once more (bounded) and frees its TMEM.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int where) {
    for (int i = 0; i < 2000000; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 16) __nanosleep(64);
    }
    if (err) atomicCAS(err, 0, where);
    return false;
}

// As mbar_wait, for warp-specialised kernels: gives up at once when another
// role has already set *abort, and sets it on its own timeout, so one stuck
// wait ends every role's waits instead of each running out its limit.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, int* err, int where,
                                                   volatile int* abort) {
    for (int i = 0; i < 2000000; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
        if (i > 16) __nanosleep(64);
    }
    *abort = 1;
    if (err) atomicCAS(err, 0, where);
    return false;
}

// Arrival that also announces `bytes` of asynchronous (TMA) writes the
// current phase must wait for.
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// TMA tiled loads (cp.async.bulk.tensor) into shared memory, completing on
// the mbarrier's transaction count; coordinates innermost first. Elements
// outside the tensor read as zero.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const void* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const void* map, int c0, int c1, int c2, int c3, int c4,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

}  // namespace tc
}  // namespace vpt
