// BF16 tensor-core GEMM (gemm.cu), shared with the learned density estimator.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rfk {

enum : int { kGemmStoreF32 = 0, kGemmStoreBF16 = 1, kGemmAtomicF32 = 2 };

struct GemmArgs {
    const __nv_bfloat16* A;  // M x K, row stride lda (elements), 16-byte aligned
    const __nv_bfloat16* B;  // N x K, row stride ldb
    uint32_t M, N, K, lda, ldb;
    void* C;                 // M x N, row stride ldc: float (StoreF32, AtomicF32) or bf16 (StoreBF16)
    uint32_t ldc;
    int mode;
    const float* bias;       // StoreBF16: per column n, may be null
    int relu;                // StoreBF16: max(0, .)
    uint32_t k_per_split;    // set by launch_gemm
    // implicit 3x3 convolution (launch_gemm_conv): A is not read from memory as a matrix but
    // gathered from NHWC inputs as their im2col matrix, row p = pixel (n x h x w), column
    // k = tap * (ca + cb) + c, tap = (dy + 1) * 3 + (dx + 1); channels [0, ca) come from xa (at half
    // resolution, nearest-neighbour upsampled, when up), [ca, ca + cb) from xb
    const __nv_bfloat16* xa;
    const __nv_bfloat16* xb;
    uint32_t ca, cb, n, h, w;
    int up;
};

// splits > 1 partitions K over grid.z and requires kGemmAtomicF32 (C accumulates)
cudaError_t launch_gemm(GemmArgs g, uint32_t splits, cudaStream_t st);
// C = im2col(xa, xb) * B^T without materialising the im2col matrix; M = n h w, K = 9 (ca + cb),
// ca and cb multiples of 8, one split
cudaError_t launch_gemm_conv(GemmArgs g, cudaStream_t st);
// reads and clears the kernels' error word (0 = no bounded wait ran out)
cudaError_t gemm_error(int* out);

}  // namespace rfk
