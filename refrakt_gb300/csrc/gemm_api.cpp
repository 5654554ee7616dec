// C-ABI entries of the tensor-core GEMM and implicit 3x3 convolution (no reference counterpart):
// let a caller, and the tests, run the contractions of the learned density estimator on their own.
#include <cuda_runtime.h>

#include <string>

#include "gemm.h"
#include "internal.h"
#include "refrakt.h"

using namespace rfk;

namespace {

// waits for the launch, then reads the kernels' bounded-wait error word
int finish(const char* fn, cudaError_t e, cudaStream_t st) {
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int werr = 0;
    if (e == cudaSuccess) e = gemm_error(&werr);
    if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string(fn) + ": " + cudaGetErrorString(e));
    if (werr) return fail(RF_ERR_CUDA, std::string(fn) + ": an mbarrier wait ran out (stage " + std::to_string(werr - 1) + ")");
    return RF_OK;
}

}  // namespace

extern "C" int rf_gemm_bf16(const void* A, const void* B, void* C, uint32_t M, uint32_t N, uint32_t K, uint32_t lda,
                            uint32_t ldb, uint32_t ldc, int mode, const float* bias, int relu, uint32_t splits,
                            void* stream) {
    if (!A || !B || !C || M == 0 || N == 0) return fail(RF_ERR_INVALID_ARG, "rf_gemm_bf16: null operand or empty shape");
    if (K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N)
        return fail(RF_ERR_INVALID_ARG, "rf_gemm_bf16: K and the operand strides must be multiples of 8, strides >= K");
    if ((((uintptr_t)A) | ((uintptr_t)B)) & 15) return fail(RF_ERR_INVALID_ARG, "rf_gemm_bf16: operands must be 16-byte aligned");
    if (mode < RF_GEMM_STORE_F32 || mode > RF_GEMM_ATOMIC_F32) return fail(RF_ERR_INVALID_ARG, "rf_gemm_bf16: bad mode");
    if (splits > 1 && mode != RF_GEMM_ATOMIC_F32) return fail(RF_ERR_INVALID_ARG, "rf_gemm_bf16: split K needs RF_GEMM_ATOMIC_F32");
    GemmArgs g{};
    g.A = static_cast<const __nv_bfloat16*>(A);
    g.B = static_cast<const __nv_bfloat16*>(B);
    g.M = M;
    g.N = N;
    g.K = K;
    g.lda = lda;
    g.ldb = ldb;
    g.C = C;
    g.ldc = ldc;
    g.mode = mode;
    g.bias = bias;
    g.relu = relu;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return finish("rf_gemm_bf16", launch_gemm(g, splits, st), st);
}

extern "C" int rf_conv3x3_bf16(const void* xa, uint32_t ca, int up, const void* xb, uint32_t cb, uint32_t n,
                               uint32_t h, uint32_t w, const void* B, uint32_t N, uint32_t ldb, void* C, uint32_t ldc,
                               int mode, const float* bias, int relu, void* stream) {
    if (!xa || !B || !C || (cb && !xb) || n == 0 || h == 0 || w == 0 || N == 0)
        return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: null operand or empty shape");
    if (ca % 8 || cb % 8 || ca + cb == 0 || ldb % 8 || ldb < 9 * (ca + cb) || ldc < N)
        return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: channels and ldb must be multiples of 8, ldb >= 9 (ca + cb)");
    if (h > 65535 || w > 65535 || (uint64_t)n * h * w > 0xFFFFFFFFull)
        return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: image too large");
    if (up && (h % 2 || w % 2)) return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: an upsampled input needs even h, w");
    if ((((uintptr_t)xa) | ((uintptr_t)xb) | ((uintptr_t)B)) & 15)
        return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: operands must be 16-byte aligned");
    if (mode < RF_GEMM_STORE_F32 || mode > RF_GEMM_ATOMIC_F32) return fail(RF_ERR_INVALID_ARG, "rf_conv3x3_bf16: bad mode");
    GemmArgs g{};
    g.xa = static_cast<const __nv_bfloat16*>(xa);
    g.xb = static_cast<const __nv_bfloat16*>(xb);
    g.ca = ca;
    g.cb = cb;
    g.n = n;
    g.h = h;
    g.w = w;
    g.up = up;
    g.B = static_cast<const __nv_bfloat16*>(B);
    g.M = n * h * w;
    g.N = N;
    g.K = 9 * (ca + cb);
    g.ldb = ldb;
    g.C = C;
    g.ldc = ldc;
    g.mode = mode;
    g.bias = bias;
    g.relu = relu;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return finish("rf_conv3x3_bf16", launch_gemm_conv(g, st), st);
}
