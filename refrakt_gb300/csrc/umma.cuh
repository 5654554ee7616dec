// Inline-PTX primitives of the 5th-generation tensor cores (sm_100 family, built for sm_103a):
// tensor-memory allocation, tcgen05.mma with shared-memory matrix descriptors, commit to an
// mbarrier, tensor-memory loads, and the fences between them.
//
// Operand layout ("K-major, no swizzle"): an operand tile of R rows x 64 K-elements (bf16) is
// stored as 8 x 8 core matrices of 8 rows x 16 bytes (128 contiguous bytes each).  Core matrix
// (row group g, K chunk c) sits at byte offset g * 1024 + c * 128, row r of it at + 16 * r.  In
// the matrix descriptor the K-direction stride between core matrices is the leading-dimension
// byte offset (128) and the row-group stride is the stride byte offset (1024); one MMA of K = 16
// covers two K chunks, so the k-th MMA of a 64-wide K block starts 256 * k bytes in.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rfk {
namespace umma {

constexpr uint32_t kTileK = 64;            // bf16 elements of K per stage
constexpr uint32_t kCoreBytes = 128;       // one core matrix: 8 rows x 16 bytes
constexpr uint32_t kGroupBytes = 1024;     // 8 core matrices along K (one 8-row group)

// byte offset of the 16-byte chunk (row, K chunk) inside a K-major no-swizzle tile
__host__ __device__ constexpr uint32_t tile_offset(uint32_t row, uint32_t kchunk) {
    return (row >> 3) * kGroupBytes + kchunk * kCoreBytes + (row & 7u) * 16u;
}

// Shared-memory matrix descriptor (64 bit): start address >> 4 in bits 0-13, leading-dimension
// byte offset >> 4 in bits 16-29, stride byte offset >> 4 in bits 32-45, descriptor version 1 in
// bits 46-47, base offset 0, layout (swizzle) 0 = none in bits 61-63.
__host__ __device__ constexpr uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// The same descriptor for a K-major tile in the 128-byte swizzled layout that a TMA load with
// CU_TENSOR_MAP_SWIZZLE_128B writes: rows of 64 bf16 (128 bytes), 16-byte chunk j of row r
// stored at chunk j ^ (r % 8), 8-row groups 1024 bytes apart (SBO); the leading offset is unused;
// layout type 2 (128-byte swizzle) in bits 61-63.  The tile must start 1024-byte aligned; the
// k-th 16-element step of a 64-wide block starts 32 * k bytes in (the swizzle is applied to the
// computed addresses).
__host__ __device__ constexpr uint64_t smem_desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

// Instruction descriptor of kind::f16 (32 bit): D format F32 (bits 4-5 = 1), A and B BF16 (bits
// 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- mbarrier ------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// one bounded probe of the phase with the given parity; true when it has completed
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// waits for the phase with at most `limit` probes; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ---- async-proxy fences ----------------------------------------------------------------------
// makes this thread's generic-proxy writes to shared memory visible to the tensor cores
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- tensor memory ---------------------------------------------------------------------------
// one full warp: allocates `ncols` columns (power of two >= 32) and writes the base to *dst
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- MMA -------------------------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrives once on `bar` when every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 bit, 16 consecutive columns: lane i of the warp receives row (lane base + i)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// one plain arrival (release semantics at CTA scope)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ---- TMA (cp.async.bulk.tensor) ---------------------------------------------------------------
// sets the phase's expected transaction bytes and arrives once
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// one 2-D box of the tensor map at (x, y) into shared memory; completes `bytes` on `bar`
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* tmap, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// ---- cp.async (16-byte global -> shared, zero-filled when src_bytes = 0) ----------------------
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace umma
}  // namespace rfk
