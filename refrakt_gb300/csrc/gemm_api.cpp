// C-ABI entry of the tensor-core GEMM (no reference counterpart): lets a caller, and the tests,
// run the contraction of the learned density estimator on its own.
#include <cuda_runtime.h>

#include <string>

#include "gemm.h"
#include "internal.h"
#include "refrakt.h"

using namespace rfk;

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
    cudaError_t e = launch_gemm(g, splits, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int werr = 0;
    if (e == cudaSuccess) e = gemm_error(&werr);
    if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("rf_gemm_bf16: ") + cudaGetErrorString(e));
    if (werr) return fail(RF_ERR_CUDA, "rf_gemm_bf16: an mbarrier wait ran out (stage " + std::to_string(werr - 1) + ")");
    return RF_OK;
}
