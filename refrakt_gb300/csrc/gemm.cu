// BF16 GEMM with FP32 accumulation on the 5th-generation tensor cores (tcgen05.mma, accumulator
// in tensor memory), the contraction behind the learned density estimator's 3x3 convolutions.
//
//   C[M x N] (+)= A[M x K] * B[N x K]^T      A, B bf16, K contiguous (K-major), K % 8 == 0
//
// Two pipelines share the MMA issue and the epilogue:
//  * plain matrices (launch_gemm): the persistent, warp-specialised TMA kernel
//    (umma_gemm_tma_kernel, "TMA pipeline" below) — 128-byte swizzled boxes, an mbarrier ring,
//    two tensor-memory accumulators; the cp.async kernel below only stands in when the driver
//    offers no tensor-map encoder;
//  * implicit 3x3 convolution (launch_gemm_conv): the cp.async kernel in conv mode, whose 128
//    threads gather each 128 x 64 block of im2col rows from the NHWC inputs.
// The cp.async kernel: one CTA of 128 threads computes a 128 x BN tile over a range of K
// (split-K along grid.z); operand tiles of 64 K-elements are staged in the K-major no-swizzle
// core-matrix layout (umma.cuh) through a 3-stage ring; thread 0 issues four M128 x N x K16 MMAs
// per stage and commits them to the stage's mbarrier, which releases the stage for refilling.
// Epilogue (both): each warp reads its 32 accumulator rows with tcgen05.ld, stages 32 columns at a
// time in shared memory and writes whole row segments with one of: FP32 store, bias + ReLU + BF16
// store, FP32 atomic add.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
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

// The pixels of a thread's A rows in an implicit convolution: thread tid loads rows
// 16 i + 8 (tid / 64) + tid % 8 (i = 0..7) of the tile at one K chunk per stage (load_stage's
// mapping), so their coordinates are computed once per tile.
struct ConvRows {
    uint32_t p[kBM / 16];    // pixel index, or ~0u past M
    uint32_t yx[kBM / 16];   // y << 16 | x
    uint32_t img[kBM / 16];  // image index (read for an upsampled input only)
};

__device__ __forceinline__ ConvRows conv_rows(const GemmArgs& g, uint32_t m0, int tid) {
    ConvRows cr;
#pragma unroll
    for (int i = 0; i < (int)(kBM / 16); i++) {
        const uint32_t p = m0 + 16u * i + 8u * ((uint32_t)tid >> 6) + ((uint32_t)tid & 7u);
        const uint32_t q = p / g.w, x = p - q * g.w, y = q % g.h;
        cr.p[i] = p < g.M ? p : ~0u;
        cr.yx[i] = (y << 16) | x;
        cr.img[i] = q / g.h;
    }
    return cr;
}

template <int BN, bool CONV>
__device__ __forceinline__ void load_stage(const GemmArgs& g, const ConvRows& cr, uint32_t sA, uint32_t sB, uint32_t m0,
                                           uint32_t n0, uint32_t kbase, uint32_t k1, int tid) {
    // virtual warp v covers rows 8*(v/2) .. +7 and K chunks 4*(v%2) .. +3: 64 contiguous bytes of
    // 8 rows in global memory, four whole core matrices (512 contiguous bytes) in shared memory
    if constexpr (CONV) {
        // this thread's K chunk: one tap and 8 channels of one input
        const uint32_t kc = 4u * (((uint32_t)tid >> 5) & 1u) + (((uint32_t)tid & 31u) >> 3);
        const uint32_t k = kbase + kc * 8u, ct = g.ca + g.cb;
        const uint32_t tap = k / ct, c = k - tap * ct;
        const int dy = (int)(tap / 3u) - 1, dx = (int)(tap % 3u) - 1;
        const bool kok = k < k1;
#pragma unroll
        for (int i = 0; i < (int)(kBM / 16); i++) {
            const uint32_t r = 16u * i + 8u * ((uint32_t)tid >> 6) + ((uint32_t)tid & 7u);
            const int y = (int)(cr.yx[i] >> 16) + dy, x = (int)(cr.yx[i] & 0xFFFFu) + dx;
            const bool ok = kok && cr.p[i] != ~0u && y >= 0 && x >= 0 && y < (int)g.h && x < (int)g.w;
            const __nv_bfloat16* src = g.xb ? g.xb : g.xa;
            if (ok) {
                const uint32_t p = cr.p[i] + (uint32_t)(dy * (int)g.w + dx);  // same image: the row and column are in range
                if (c < g.ca) {
                    if (g.up) {
                        const uint32_t hw = (g.h / 2u) * (g.w / 2u);
                        src = g.xa +
                              ((size_t)cr.img[i] * hw + (size_t)((uint32_t)y >> 1) * (g.w / 2u) + ((uint32_t)x >> 1)) * g.ca + c;
                    } else {
                        src = g.xa + (size_t)p * g.ca + c;
                    }
                } else {
                    src = g.xb + (size_t)p * g.cb + (c - g.ca);
                }
            }
            umma::cp_async16(sA + umma::tile_offset(r, kc), src, ok ? 16u : 0u);
        }
    } else {
#pragma unroll
        for (int i = 0; i < (int)(kBM * 8 / kThreads); i++) {
            const uint32_t idx = tid + kThreads * i, l = idx & 31u, v = idx >> 5;
            const uint32_t r = 8u * (v >> 1) + (l & 7u), kc = 4u * (v & 1u) + (l >> 3);
            const uint32_t row = m0 + r, k = kbase + kc * 8u;
            const bool ok = row < g.M && k < k1;
            const __nv_bfloat16* src = ok ? g.A + (size_t)row * g.lda + k : g.A;
            umma::cp_async16(sA + umma::tile_offset(r, kc), src, ok ? 16u : 0u);
        }
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

constexpr uint32_t kStageLd = 36;  // floats per row of the epilogue's staging block (32 + 4 against bank conflicts)

// writes columns n .. n + min(4, left) - 1 of one output row at element offset o
__device__ __forceinline__ void store4(const GemmArgs& g, size_t o, uint32_t left, float4 v, bool vec) {
    const float e[4] = {v.x, v.y, v.z, v.w};
    if (g.mode == kGemmStoreF32) {
        float* c = static_cast<float*>(g.C) + o;
        if (vec && left >= 4) {
            *reinterpret_cast<float4*>(c) = v;
        } else {
            for (uint32_t j = 0; j < 4 && j < left; j++) c[j] = e[j];
        }
    } else if (g.mode == kGemmAtomicF32) {
        float* c = static_cast<float*>(g.C) + o;
        for (uint32_t j = 0; j < 4 && j < left; j++) atomicAdd(c + j, e[j]);
    } else {
        __nv_bfloat16* c = static_cast<__nv_bfloat16*>(g.C) + o;
        if (vec && left >= 4) {
            const __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
            uint2 u;
            u.x = *reinterpret_cast<const uint32_t*>(&lo);
            u.y = *reinterpret_cast<const uint32_t*>(&hi);
            *reinterpret_cast<uint2*>(c) = u;
        } else {
            for (uint32_t j = 0; j < 4 && j < left; j++) c[j] = __float2bfloat16_rn(e[j]);
        }
    }
}

// The epilogue of one warp's 32 accumulator rows (TMEM lane quarter q: rows 32q .. 32q + 31 of
// the 128 x n_tile tile).  32 columns at a time go through the warp's own 32 rows of a staging
// block in shared memory (`stage`, [128][kStageLd] floats), then the warp writes whole row
// segments, 4 columns per lane: no barrier beyond the warp, so a warp that gives up on a wait
// cannot strand the others.
__device__ __forceinline__ void warp_epilogue(const GemmArgs& g, float* stage, uint32_t tmem, uint32_t q, uint32_t lane,
                                              uint32_t m0, uint32_t n0, uint32_t n_tile, bool have_acc) {
    const bool vec = ((reinterpret_cast<uintptr_t>(g.C) & 15u) == 0) && (g.ldc % 4u == 0);
    float* rows = stage + 32u * q * kStageLd;
    for (uint32_t c0 = 0; c0 < n_tile; c0 += 32) {
#pragma unroll
        for (uint32_t hh = 0; hh < 2; hh++) {
            const uint32_t cc = c0 + 16u * hh;
            if (cc >= n_tile) break;  // n_tile is a multiple of 16
            float v[16];
            if (have_acc) {
                umma::tmem_ld16(tmem + ((32u * q) << 16) + cc, v);
            } else {
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = 0.0f;
            }
            if (g.mode == kGemmStoreBF16) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const uint32_t n = n0 + cc + j;
                    float y = v[j] + ((g.bias && n < g.N) ? g.bias[n] : 0.0f);
                    v[j] = g.relu ? fmaxf(y, 0.0f) : y;
                }
            }
            float4* dst = reinterpret_cast<float4*>(rows + lane * kStageLd + 16u * hh);
#pragma unroll
            for (int j = 0; j < 4; j++) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
        __syncwarp();
        const uint32_t pieces = (n_tile - c0 < 32u ? n_tile - c0 : 32u) / 4u;  // 4-column pieces per row
        for (uint32_t idx = lane; idx < 32u * pieces; idx += 32u) {
            const uint32_t r = idx / pieces, pc = idx - r * pieces;
            const uint32_t m = m0 + 32u * q + r, n = n0 + c0 + 4u * pc;
            if (m >= g.M || n >= g.N) continue;
            const float4 v = *reinterpret_cast<const float4*>(rows + r * kStageLd + 4u * pc);
            store4(g, (size_t)m * g.ldc + n, g.N - n, v, vec);
        }
        __syncwarp();
    }
}

template <int BN, bool CONV>
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
    ConvRows cr;
    if constexpr (CONV) cr = conv_rows(g, m0, tid);

    for (int s = 0; s < kStages - 1; s++) {
        if ((uint32_t)s < nk) load_stage<BN, CONV>(g, cr, base + s * (kA + kB), base + s * (kA + kB) + kA, m0, n0,
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
            load_stage<BN, CONV>(g, cr, base + ns * (kA + kB), base + ns * (kA + kB) + kA, m0, n0,
                                 k0 + nxt * umma::kTileK, k1, tid);
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

    if (*s_fail == 0 && (nk > 0 || g.mode != kGemmAtomicF32))
        warp_epilogue(g, reinterpret_cast<float*>(smem), tmem, (uint32_t)warp, (uint32_t)lane, m0, n0, n_tile, nk > 0);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, kCols);
}

// ---- TMA pipeline ------------------------------------------------------------------------------
// Persistent and warp-specialised.  Each CTA walks its share of the output tiles (grouped: 8
// row tiles side by side, so co-resident CTAs share A rows and B columns in L2).  Warp 0 (one lane)
// loads 64-wide K blocks of A and B with cp.async.bulk.tensor into a ring of stages that runs on
// across tiles, completing each stage's `full` mbarrier by transaction bytes; warp 1 (one lane)
// issues the four MMAs of a full stage and commits them to the stage's `empty` mbarrier (which
// frees it for the next load).  Two tensor-memory accumulators alternate between tiles: the MMA
// lane commits a finished tile to `acc_full[b]`, warps 2-5 drain it (each its TMEM lane quarter,
// through its own rows of a staging block) and release it on `acc_empty[b]`, so a tile's epilogue
// overlaps the next tile's loads and MMAs.  One TMA box per operand and stage: 64 K-elements
// (128 bytes) x R rows in the 128-byte swizzled K-major layout (umma::smem_desc_sw128); rows and K
// past the matrix are zero-filled by the TMA unit.
constexpr int kTmaThreads = 192;
constexpr uint32_t kGroupM = 8;  // row tiles per raster group

template <int BN>
__host__ __device__ constexpr int tma_stages() { return BN >= 256 ? 4 : (BN >= 128 ? 6 : 8); }  // one CTA per SM
template <int BN>
__host__ __device__ constexpr size_t tma_smem() {
    return 1024 + (size_t)tma_stages<BN>() * (kBM * 128 + BN * 128) + (size_t)kBM * kStageLd * 4 + 256;
}

__device__ __forceinline__ void gemm_fail(int* s_fail, int code) {
    *reinterpret_cast<volatile int*>(s_fail) = 1;
    atomicExch(&g_gemm_error, code);
}
__device__ __forceinline__ bool gemm_failed(const int* s_fail) { return *reinterpret_cast<const volatile int*>(s_fail) != 0; }

// tile t of the grid (split-major; within a split, groups of kGroupM row tiles with the row tile
// fastest) -> its origin and K range
struct TileCoord {
    uint32_t m0, n0, k0, nk;
};
__device__ __forceinline__ TileCoord tile_coord(const GemmArgs& g, uint32_t t, uint32_t tiles_m, uint32_t tiles_n,
                                                uint32_t bn) {
    const uint32_t per_split = tiles_m * tiles_n, split = t / per_split, r = t - split * per_split;
    const uint32_t group = r / (kGroupM * tiles_n), first = group * kGroupM;
    const uint32_t gm = min(kGroupM, tiles_m - first), within = r - group * kGroupM * tiles_n;
    TileCoord c;
    c.m0 = (first + within % gm) * kBM;
    c.n0 = (within / gm) * bn;
    c.k0 = split * g.k_per_split;  // a multiple of 64: blocks never straddle splits
    const uint32_t k1 = min(g.K, c.k0 + g.k_per_split);
    c.nk = k1 > c.k0 ? (k1 - c.k0 + umma::kTileK - 1) / umma::kTileK : 0u;
    return c;
}

template <int BN>
__global__ void __launch_bounds__(kTmaThreads, 1)
    umma_gemm_tma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                         const GemmArgs g, uint32_t splits) {
    constexpr int S = tma_stages<BN>();
    constexpr uint32_t kA = kBM * 128, kB = BN * 128;  // bytes of one stage's A and B blocks
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;      // one accumulator; two are allocated
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (umma::smem_u32(smem_raw) & 1023u)) & 1023u);
    float* stage_out = reinterpret_cast<float*>(smem + S * (kA + kB));
    uint64_t* full = reinterpret_cast<uint64_t*>(stage_out + kBM * kStageLd);
    uint64_t* empty = full + S;
    uint64_t* acc_full = empty + S;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(acc_empty + 2);
    int* s_fail = reinterpret_cast<int*>(s_tmem + 1);
    const uint32_t base = umma::smem_u32(smem);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t tiles_m = (g.M + kBM - 1) / kBM, tiles_n = (g.N + BN - 1) / BN;
    const uint32_t tiles = tiles_m * tiles_n * splits;

    if (warp == 1) umma::tmem_alloc(s_tmem, 2 * kCols);
    if (tid == 0) {
        for (int s = 0; s < S; s++) {
            umma::mbar_init(&full[s], 1);
            umma::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            umma::mbar_init(&acc_full[b], 1);
            umma::mbar_init(&acc_empty[b], 4);  // one arrival per epilogue warp
        }
        *s_fail = 0;
        umma::fence_mbar_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *s_tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;  // K blocks issued by this CTA
            for (uint32_t t = blockIdx.x; t < tiles && !gemm_failed(s_fail); t += gridDim.x) {
                const TileCoord c = tile_coord(g, t, tiles_m, tiles_n, BN);
                for (uint32_t kb = 0; kb < c.nk; kb++, it++) {
                    const uint32_t st = it % S, use = it / S;
                    if (use > 0 && !umma::mbar_wait(&empty[st], (use - 1) & 1u, kWaitLimit)) {
                        gemm_fail(s_fail, 1 + (int)st);
                        break;
                    }
                    if (gemm_failed(s_fail)) break;
                    umma::mbar_arrive_expect_tx(&full[st], kA + kB);
                    const uint32_t a = base + st * (kA + kB), b = a + kA;
                    const int kx = (int)(c.k0 + kb * umma::kTileK);
                    umma::tma_load_2d(a, &tmA, kx, (int)c.m0, &full[st]);
                    umma::tma_load_2d(b, &tmB, kx, (int)c.n0, &full[st]);
                }
            }
            if (gemm_failed(s_fail)) {  // let this thread's copies in flight land
                for (uint32_t k = it > (uint32_t)S ? it - S : 0u; k < it; k++)
                    umma::mbar_wait(&full[k % S], (k / S) & 1u, kWaitLimit);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t it = 0, i = 0;  // K blocks consumed, tiles done by this CTA
            for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, i++) {
                const TileCoord c = tile_coord(g, t, tiles_m, tiles_n, BN);
                const uint32_t buf = i & 1u, u = i >> 1;
                const uint32_t n_rem = g.N - c.n0;
                const uint32_t n_tile = ((n_rem < (uint32_t)BN ? n_rem : (uint32_t)BN) + 15u) & ~15u;
                const uint32_t idesc = umma::idesc_bf16_f32(kBM, n_tile);
                bool ok = !gemm_failed(s_fail);
                if (ok && u > 0 && !umma::mbar_wait(&acc_empty[buf], (u - 1) & 1u, kWaitLimit)) {
                    gemm_fail(s_fail, 1 + 2 * S + (int)buf);
                    ok = false;
                }
                umma::fence_after_sync();
                for (uint32_t kb = 0; ok && kb < c.nk; kb++, it++) {
                    const uint32_t st = it % S;
                    if (!umma::mbar_wait(&full[st], (it / S) & 1u, kWaitLimit)) {
                        gemm_fail(s_fail, 1 + S + (int)st);
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const uint32_t a = base + st * (kA + kB), b = a + kA;
#pragma unroll
                    for (uint32_t kk = 0; kk < umma::kTileK / 16; kk++)
                        umma::mma_bf16(tmem + buf * kCols, umma::smem_desc_sw128(a + 32u * kk),
                                       umma::smem_desc_sw128(b + 32u * kk), idesc, (kb | kk) != 0u);
                    umma::mma_commit(&empty[st]);
                }
                umma::mma_commit(&acc_full[buf]);  // arrives once every MMA issued above has completed
                if (!ok) break;
            }
        }
    } else {
        const uint32_t q = (uint32_t)warp & 3u;  // TMEM lane quarter of this warp
        float* rows = stage_out;
        uint32_t i = 0;
        for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, i++) {
            const TileCoord c = tile_coord(g, t, tiles_m, tiles_n, BN);
            const uint32_t buf = i & 1u, u = i >> 1;
            if (!umma::mbar_wait(&acc_full[buf], u & 1u, kWaitLimit)) {
                gemm_fail(s_fail, 3 + 2 * S + (int)buf);
                break;
            }
            umma::fence_after_sync();
            if (gemm_failed(s_fail)) break;
            const uint32_t n_rem = g.N - c.n0;
            const uint32_t n_tile = ((n_rem < (uint32_t)BN ? n_rem : (uint32_t)BN) + 15u) & ~15u;
            if (c.nk > 0 || g.mode != kGemmAtomicF32)
                warp_epilogue(g, rows, tmem + buf * kCols, q, (uint32_t)lane, c.m0, c.n0, n_tile, c.nk > 0);
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&acc_empty[buf]);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 1) umma::tmem_free(tmem, 2 * kCols);
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda); null when absent
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// a [rows x inner] bf16 matrix with row stride ld (elements), read in 128-byte swizzled boxes of
// 64 x box_rows
bool encode_operand(CUtensorMap* m, const __nv_bfloat16* p, uint32_t inner, uint32_t rows, uint32_t ld,
                    uint32_t box_rows) {
    const cuuint64_t dims[2] = {inner, rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2u};
    const cuuint32_t box[2] = {umma::kTileK, box_rows};
    const cuuint32_t estr[2] = {1u, 1u};
    return tensor_map_encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(p), dims, strides,
                                box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// false (nothing launched) when a tensor map cannot be encoded for these operands
template <int BN>
bool launch_tma_bn(const GemmArgs& g, uint32_t splits, cudaStream_t st, cudaError_t* err) {
    CUtensorMap ta, tb;
    if (!encode_operand(&ta, g.A, g.K, g.M, g.lda, kBM) || !encode_operand(&tb, g.B, g.K, g.N, g.ldb, BN)) return false;
    const size_t smem = tma_smem<BN>();
    *err = cudaFuncSetAttribute(umma_gemm_tma_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (*err != cudaSuccess) return true;
    // persistent: as many CTAs as fit at once, each walking tiles t = blockIdx.x + i * gridDim.x
    // (resident CTAs per SM depend on the kernel alone: asked once)
    static const int per_sm = [smem] {
        int n = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, umma_gemm_tma_kernel<BN>, kTmaThreads, smem) ==
                       cudaSuccess
                   ? n
                   : 1;
    }();
    int dev = 0, sms = 0;
    if ((*err = cudaGetDevice(&dev)) != cudaSuccess) return true;
    if ((*err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return true;
    // fewer than two rounds of tiles: one CTA per tile, so a second-round tile goes to whichever SM
    // frees first rather than to a fixed CTA
    const uint64_t tiles = (uint64_t)((g.M + kBM - 1) / kBM) * ((g.N + BN - 1) / BN) * splits;
    const uint64_t resident = (uint64_t)std::max(1, sms * std::max(1, per_sm));
    const uint32_t grid = (uint32_t)(tiles < 2 * resident ? tiles : resident);
    umma_gemm_tma_kernel<BN><<<grid, kTmaThreads, smem, st>>>(ta, tb, g, splits);
    *err = cudaGetLastError();
    return true;
}

template <int BN, bool CONV = false>
cudaError_t launch_bn(const GemmArgs& g, uint32_t splits, cudaStream_t st) {
    const size_t smem = gemm_smem<BN>();
    cudaError_t e =
        cudaFuncSetAttribute(umma_gemm_kernel<BN, CONV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((g.N + BN - 1) / BN, (g.M + kBM - 1) / kBM, splits);
    umma_gemm_kernel<BN, CONV><<<grid, kThreads, smem, st>>>(g);
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
    if (tensor_map_encoder() && g.K > 0 && g.M < (1u << 31) && g.K < (1u << 31)) {  // TMA pipeline
        cudaError_t e = cudaSuccess;
        const bool launched = g.N <= 64    ? launch_tma_bn<64>(g, splits, st, &e)
                              : g.N <= 128 ? launch_tma_bn<128>(g, splits, st, &e)
                                           : launch_tma_bn<256>(g, splits, st, &e);
        if (launched) return e;
    }
    if (g.N <= 64) return launch_bn<64>(g, splits, st);
    if (g.N <= 128) return launch_bn<128>(g, splits, st);
    return launch_bn<256>(g, splits, st);
}

cudaError_t launch_gemm_conv(GemmArgs g, cudaStream_t st) {
    if (g.ca % 8 || g.cb % 8 || g.ca + g.cb == 0 || g.n == 0 || g.h == 0 || g.w == 0 || g.h > 65535 || g.w > 65535)
        return cudaErrorInvalidValue;
    if (!g.xa || (g.cb && !g.xb) || (uint64_t)g.n * g.h * g.w != g.M || g.K != 9u * (g.ca + g.cb) || g.ldb % 8 ||
        g.N == 0 || ((uintptr_t)g.xa | (uintptr_t)g.xb | (uintptr_t)g.B) & 15)
        return cudaErrorInvalidValue;
    g.A = nullptr;
    g.lda = 0;
    g.k_per_split = (g.K + umma::kTileK - 1) / umma::kTileK * umma::kTileK;
    if (g.N <= 64) return launch_bn<64, true>(g, 1, st);
    if (g.N <= 128) return launch_bn<128, true>(g, 1, st);
    return launch_bn<256, true>(g, 1, st);
}

cudaError_t gemm_error(int* out) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_gemm_error, sizeof(int));
    const int zero = 0;
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_gemm_error, &zero, sizeof(int));
    return e;
}

}  // namespace rfk
