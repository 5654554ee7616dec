// BF16 GEMM with FP32 accumulation on the 5th-generation tensor cores (tcgen05.mma, accumulator
// in tensor memory), the contraction behind the learned density estimator's 3x3 convolutions.
//
//   C[M x N] (+)= A[M x K] * B[N x K]^T      A, B bf16, K contiguous (K-major), K % 8 == 0
//
// One CTA of 128 threads computes a 128 x BN tile over a range of K (split-K along grid.z).
// Operand tiles of 64 K-elements are staged in shared memory by cp.async in the K-major
// no-swizzle core-matrix layout (umma.cuh) through a 3-stage ring; thread 0 issues four
// M128 x N x K16 MMAs per stage and commits them to the stage's mbarrier, which releases the
// stage for refilling.  The epilogue reads the accumulator with tcgen05.ld (warp w owns rows
// 32w..32w+31) and applies one of: FP32 store, bias + ReLU + BF16 store, FP32 atomic add.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gemm.h"
#include "umma.cuh"

namespace rfk {

namespace {

constexpr int kStages = 3;
constexpr int kThreads = 128;
constexpr uint32_t kBM = 128;
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ int g_gemm_error;  // 0, or 1 + the stage whose mbarrier wait ran out

template <int BN>
__host__ __device__ constexpr size_t gemm_smem() {
    return 1024 + (size_t)kStages * (kBM * 128 + BN * 128) + 64;
}

template <int BN>
__device__ __forceinline__ void load_stage(const GemmArgs& g, uint32_t sA, uint32_t sB, uint32_t m0, uint32_t n0,
                                           uint32_t kbase, uint32_t k1, int tid) {
    // virtual warp v covers rows 8*(v/2) .. +7 and K chunks 4*(v%2) .. +3: 64 contiguous bytes of
    // 8 rows in global memory, four whole core matrices (512 contiguous bytes) in shared memory
#pragma unroll
    for (int i = 0; i < (int)(kBM * 8 / kThreads); i++) {
        const uint32_t idx = tid + kThreads * i, l = idx & 31u, v = idx >> 5;
        const uint32_t r = 8u * (v >> 1) + (l & 7u), kc = 4u * (v & 1u) + (l >> 3);
        const uint32_t row = m0 + r, k = kbase + kc * 8u;
        const bool ok = row < g.M && k < k1;
        const __nv_bfloat16* src = ok ? g.A + (size_t)row * g.lda + k : g.A;
        umma::cp_async16(sA + umma::tile_offset(r, kc), src, ok ? 16u : 0u);
    }
#pragma unroll
    for (int i = 0; i < (int)(BN * 8 / kThreads); i++) {
        const uint32_t idx = tid + kThreads * i, l = idx & 31u, v = idx >> 5;
        const uint32_t r = 8u * (v >> 1) + (l & 7u), kc = 4u * (v & 1u) + (l >> 3);
        const uint32_t row = n0 + r, k = kbase + kc * 8u;
        const bool ok = row < g.N && k < k1;
        const __nv_bfloat16* src = ok ? g.B + (size_t)row * g.ldb + k : g.B;
        umma::cp_async16(sB + umma::tile_offset(r, kc), src, ok ? 16u : 0u);
    }
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) umma_gemm_kernel(const GemmArgs g) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (umma::smem_u32(smem_raw) & 1023u)) & 1023u);
    constexpr uint32_t kA = kBM * 128, kB = BN * 128;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kStages * (kA + kB));
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bar + kStages);
    int* s_fail = reinterpret_cast<int*>(s_tmem + 1);
    const uint32_t base = umma::smem_u32(smem);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
    const uint32_t k0 = blockIdx.z * g.k_per_split;
    const uint32_t k1 = min(g.K, k0 + g.k_per_split);
    const uint32_t nk = k1 > k0 ? (k1 - k0 + umma::kTileK - 1) / umma::kTileK : 0u;
    const uint32_t n_rem = g.N - n0;
    const uint32_t n_tile = ((n_rem < (uint32_t)BN ? n_rem : (uint32_t)BN) + 15u) & ~15u;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;  // tensor-memory columns (power of two)

    if (warp == 0) umma::tmem_alloc(s_tmem, kCols);
    if (tid == 0) {
        for (int s = 0; s < kStages; s++) umma::mbar_init(&bar[s], 1);
        *s_fail = 0;
        umma::fence_mbar_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *s_tmem;
    const uint32_t idesc = umma::idesc_bf16_f32(kBM, n_tile);

    for (int s = 0; s < kStages - 1; s++) {
        if ((uint32_t)s < nk) load_stage<BN>(g, base + s * (kA + kB), base + s * (kA + kB) + kA, m0, n0,
                                             k0 + s * umma::kTileK, k1, tid);
        umma::cp_async_commit();
    }
    for (uint32_t kb = 0; kb < nk; kb++) {
        const uint32_t st = kb % kStages;
        umma::cp_async_wait<kStages - 2>();
        umma::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            const uint32_t a = base + st * (kA + kB), b = a + kA;
#pragma unroll
            for (uint32_t kk = 0; kk < umma::kTileK / 16; kk++)
                umma::mma_bf16(tmem, umma::smem_desc(a + 256u * kk, umma::kCoreBytes, umma::kGroupBytes),
                               umma::smem_desc(b + 256u * kk, umma::kCoreBytes, umma::kGroupBytes), idesc,
                               (kb | kk) != 0u);
            umma::mma_commit(&bar[st]);
        }
        const uint32_t nxt = kb + kStages - 1;
        if (nxt < nk) {
            if (kb >= 1) {  // the stage to refill was last read by the MMAs of block kb - 1
                const uint32_t ps = (kb - 1) % kStages;
                if (!umma::mbar_wait(&bar[ps], ((kb - 1) / kStages) & 1u, kWaitLimit)) {
                    *s_fail = 1;
                    atomicExch(&g_gemm_error, 1 + (int)ps);
                }
            }
            const uint32_t ns = nxt % kStages;
            load_stage<BN>(g, base + ns * (kA + kB), base + ns * (kA + kB) + kA, m0, n0, k0 + nxt * umma::kTileK,
                           k1, tid);
        }
        umma::cp_async_commit();
    }
    if (nk > 0) {
        const uint32_t ls = (nk - 1) % kStages;
        if (!umma::mbar_wait(&bar[ls], ((nk - 1) / kStages) & 1u, kWaitLimit)) {
            *s_fail = 1;
            atomicExch(&g_gemm_error, 1 + (int)ls);
        }
    }
    umma::cp_async_wait<0>();
    __syncthreads();
    umma::fence_after_sync();

    if (*s_fail == 0 && (nk > 0 || g.mode != kGemmAtomicF32)) {
        const uint32_t m = m0 + 32u * warp + lane;
        for (uint32_t c0 = 0; c0 < n_tile; c0 += 16) {
            float v[16];
            if (nk > 0) {
                umma::tmem_ld16(tmem + ((32u * warp) << 16) + c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = 0.0f;
            }
            if (m >= g.M) continue;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const uint32_t n = n0 + c0 + j;
                if (n >= g.N) break;
                const size_t o = (size_t)m * g.ldc + n;
                if (g.mode == kGemmStoreF32) {
                    static_cast<float*>(g.C)[o] = v[j];
                } else if (g.mode == kGemmAtomicF32) {
                    atomicAdd(static_cast<float*>(g.C) + o, v[j]);
                } else {
                    float y = v[j] + (g.bias ? g.bias[n] : 0.0f);
                    if (g.relu) y = fmaxf(y, 0.0f);
                    static_cast<__nv_bfloat16*>(g.C)[o] = __float2bfloat16_rn(y);
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, kCols);
}

template <int BN>
cudaError_t launch_bn(const GemmArgs& g, uint32_t splits, cudaStream_t st) {
    const size_t smem = gemm_smem<BN>();
    cudaError_t e = cudaFuncSetAttribute(umma_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((g.N + BN - 1) / BN, (g.M + kBM - 1) / kBM, splits);
    umma_gemm_kernel<BN><<<grid, kThreads, smem, st>>>(g);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm(GemmArgs g, uint32_t splits, cudaStream_t st) {
    if (g.K % 8 || g.lda % 8 || g.ldb % 8 || g.M == 0 || g.N == 0) return cudaErrorInvalidValue;
    if (((uintptr_t)g.A | (uintptr_t)g.B) & 15) return cudaErrorInvalidValue;
    if (splits == 0) splits = 1;
    const uint32_t kblocks = (g.K + umma::kTileK - 1) / umma::kTileK;
    if (splits > kblocks && kblocks > 0) splits = kblocks;
    const uint32_t per = (kblocks + splits - 1) / splits;
    g.k_per_split = per * umma::kTileK;
    if (splits > 1 && g.mode != kGemmAtomicF32) return cudaErrorInvalidValue;
    if (g.N <= 64) return launch_bn<64>(g, splits, st);
    if (g.N <= 128) return launch_bn<128>(g, splits, st);
    return launch_bn<256>(g, splits, st);
}

cudaError_t gemm_error(int* out) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_gemm_error, sizeof(int));
    const int zero = 0;
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_gemm_error, &zero, sizeof(int));
    return e;
}

}  // namespace rfk
