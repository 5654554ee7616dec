// Launchers of the learned density estimator's elementwise and data-movement kernels
// (denoise_ops.cu).  NHWC activations, channel counts multiples of 8.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rfk {

cudaError_t launch_im2col_t(const __nv_bfloat16* xa, uint32_t ca, int up, const __nv_bfloat16* xb, uint32_t cb,
                            uint32_t taps, uint32_t n, uint32_t h, uint32_t w, __nv_bfloat16* colt, uint32_t ldp,
                            cudaStream_t st);
cudaError_t launch_avgpool(const __nv_bfloat16* x, uint32_t c, uint32_t n, uint32_t h, uint32_t w, __nv_bfloat16* y,
                           cudaStream_t st);
cudaError_t launch_relu_back(const float* dy, const __nv_bfloat16* y, uint32_t c, uint64_t P, int relu,
                             __nv_bfloat16* dz, __nv_bfloat16* dzt, uint32_t ldp, float* dbias, cudaStream_t st);
cudaError_t launch_split_concat_grad(const float* dx, uint32_t ca, uint32_t cb, uint32_t n, uint32_t h, uint32_t w,
                                     float* dlow, float* dskip, cudaStream_t st);
cudaError_t launch_avgpool_back(const float* dy, uint32_t c, uint32_t n, uint32_t h, uint32_t w, float* dx,
                                cudaStream_t st);
cudaError_t launch_l1_head(const float* z, const float* bias, const __nv_bfloat16* feats, const float* target,
                           uint64_t P, __nv_bfloat16* dpred, __nv_bfloat16* dpred_t, uint32_t ldp, float* dbias,
                           double* loss, cudaStream_t st);
cudaError_t launch_head(const float* z, const float* bias, const __nv_bfloat16* feats, uint64_t P, float* out,
                        cudaStream_t st);
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, uint32_t n, float lr, float b1, float b2,
                        float eps, uint32_t t, uint32_t cout, uint32_t K, uint32_t taps, __nv_bfloat16* w16,
                        __nv_bfloat16* wf16, uint32_t ldf, cudaStream_t st);
cudaError_t launch_features(const float4* bins, uint64_t n, float k2, const double* stats, const float4* base,
                            float level, __nv_bfloat16* out, cudaStream_t st);

}  // namespace rfk
