// Elementwise and data-movement kernels of the learned density estimator (a small U-Net whose
// 3x3 convolutions run as tensor-core GEMMs, gemm.cu).  Activations are NHWC with the channel
// count a multiple of 8, so every pixel's channels are whole 16-byte vectors of bf16.
//
// A convolution's GEMM operand is its im2col matrix: row p = pixel, column k = tap * C + c with
// tap = (dy + 1) * 3 + (dx + 1) — tap-major, so each tap's channels are one contiguous run.  The
// forward and input-gradient GEMMs gather it on the fly (gemm.cu, launch_gemm_conv); the weight
// gradient reads its transpose, materialised here.  A
// decoder convolution reads two inputs, channel-concatenated: the coarser level upsampled by
// nearest neighbour (first Ca channels) and the encoder's skip tensor (next Cb channels).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "denoise_ops.h"

namespace rfk {

namespace {

// transposed im2col for the weight gradient: colT[k][p], k = tap * C + c (C = ca + cb); with
// taps = 1 only the centre tap (a plain transpose, for a 1x1 convolution)
__global__ void im2col_t_kernel(const __nv_bfloat16* __restrict__ xa, uint32_t ca, int up,
                                const __nv_bfloat16* __restrict__ xb, uint32_t cb, uint32_t taps, uint32_t n,
                                uint32_t h, uint32_t w, __nv_bfloat16* __restrict__ colt, uint32_t ldp) {
    const uint32_t ct = ca + cb;
    const uint64_t P = (uint64_t)n * h * w;
    const uint64_t total = P * taps * ct;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = i % P;  // consecutive threads: consecutive pixels (coalesced stores)
        const uint64_t k = i / P;
        const uint32_t tap = taps == 1 ? 4u : (uint32_t)(k / ct), c = (uint32_t)(k % ct);
        const uint32_t x = (uint32_t)(p % w), y = (uint32_t)((p / w) % h), b = (uint32_t)(p / ((uint64_t)w * h));
        const int sy = (int)y + (int)(tap / 3) - 1, sx = (int)x + (int)(tap % 3) - 1;
        __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
        if (sy >= 0 && sx >= 0 && sy < (int)h && sx < (int)w) {
            if (c < ca) {
                const uint32_t ha = up ? h / 2 : h, wa = up ? w / 2 : w;
                const uint32_t ay = up ? (uint32_t)sy / 2 : (uint32_t)sy, ax = up ? (uint32_t)sx / 2 : (uint32_t)sx;
                v = xa[(((uint64_t)b * ha + ay) * wa + ax) * ca + c];
            } else {
                v = xb[(((uint64_t)b * h + sy) * w + sx) * cb + (c - ca)];
            }
        }
        colt[k * ldp + p] = v;
    }
}

// 2x2 average pool, NHWC bf16 (FP32 arithmetic)
__global__ void avgpool_kernel(const __nv_bfloat16* __restrict__ x, uint32_t c, uint32_t n, uint32_t h, uint32_t w,
                               __nv_bfloat16* __restrict__ y) {
    const uint32_t ho = h / 2, wo = w / 2;
    const uint64_t total = (uint64_t)n * ho * wo * c;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ch = (uint32_t)(i % c);
        const uint64_t p = i / c;
        const uint32_t xo = (uint32_t)(p % wo), yo = (uint32_t)((p / wo) % ho), b = (uint32_t)(p / ((uint64_t)wo * ho));
        const uint64_t r0 = (((uint64_t)b * h + 2 * yo) * w + 2 * xo) * c + ch, r1 = r0 + (uint64_t)w * c;
        const float s = __bfloat162float(x[r0]) + __bfloat162float(x[r0 + c]) + __bfloat162float(x[r1]) +
                        __bfloat162float(x[r1 + c]);
        y[i] = __float2bfloat16_rn(0.25f * s);
    }
}

// ReLU backward: dz = dy * (y > 0) as bf16, in the pixel-major layout [P x c] and transposed
// [c x P] (the weight-gradient operand), plus the bias gradient sum_p dz[p, ch] (FP32 atomics)
__global__ void relu_back_kernel(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ y, uint32_t c,
                                 uint64_t P, int relu, __nv_bfloat16* __restrict__ dz, __nv_bfloat16* __restrict__ dzt,
                                 uint32_t ldp, float* __restrict__ dbias) {
    // block: 32 pixels x c channels (c <= 128), transposed through shared memory
    __shared__ float tile[32][129];
    const uint64_t p0 = (uint64_t)blockIdx.x * 32;
    for (uint32_t t = threadIdx.x; t < 32 * c; t += blockDim.x) {
        const uint32_t pl = t / c, ch = t % c;
        const uint64_t p = p0 + pl;
        float g = 0.0f;
        if (p < P) {
            g = dy[p * c + ch];
            if (relu && !(__bfloat162float(y[p * c + ch]) > 0.0f)) g = 0.0f;
            dz[p * c + ch] = __float2bfloat16_rn(g);
        }
        tile[pl][ch] = g;
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < 32 * c; t += blockDim.x) {
        const uint32_t ch = t / 32, pl = t % 32;
        const uint64_t p = p0 + pl;
        if (p < P) dzt[(uint64_t)ch * ldp + p] = __float2bfloat16_rn(tile[pl][ch]);
    }
    for (uint32_t ch = threadIdx.x; ch < c; ch += blockDim.x) {
        float s = 0.0f;
        for (int pl = 0; pl < 32; pl++) s += tile[pl][ch];
        atomicAdd(dbias + ch, s);
    }
}

// gradient of a channel-concatenated input [P x (ca + cb)] (FP32) split back: the skip part is
// added to dskip (FP32, [P x cb]); the upsampled part is summed over each 2x2 block into dlow
// (FP32, [P/4 x ca]) — the adjoint of nearest-neighbour upsampling
__global__ void split_concat_grad_kernel(const float* __restrict__ dx, uint32_t ca, uint32_t cb, uint32_t n,
                                         uint32_t h, uint32_t w, float* __restrict__ dlow, float* __restrict__ dskip) {
    const uint32_t ct = ca + cb;
    const uint32_t ho = h / 2, wo = w / 2;
    // low-resolution part
    const uint64_t tl = (uint64_t)n * ho * wo * ca;
    const uint64_t ts = (uint64_t)n * h * w * cb;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tl + ts; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < tl) {
            const uint32_t ch = (uint32_t)(i % ca);
            const uint64_t p = i / ca;
            const uint32_t xo = (uint32_t)(p % wo), yo = (uint32_t)((p / wo) % ho), b = (uint32_t)(p / ((uint64_t)wo * ho));
            const uint64_t r0 = ((uint64_t)b * h + 2 * yo) * w + 2 * xo, r1 = r0 + w;
            dlow[i] = dx[r0 * ct + ch] + dx[(r0 + 1) * ct + ch] + dx[r1 * ct + ch] + dx[(r1 + 1) * ct + ch];
        } else {
            const uint64_t j = i - tl;
            const uint32_t ch = (uint32_t)(j % cb);
            const uint64_t p = j / cb;
            dskip[j] += dx[p * ct + ca + ch];
        }
    }
}

// adjoint of the 2x2 average pool, accumulated: dx[hi-res] += 0.25 * dy[lo-res]
__global__ void avgpool_back_kernel(const float* __restrict__ dy, uint32_t c, uint32_t n, uint32_t h, uint32_t w,
                                    float* __restrict__ dx) {
    const uint64_t total = (uint64_t)n * h * w * c;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ch = (uint32_t)(i % c);
        const uint64_t p = i / c;
        const uint32_t x = (uint32_t)(p % w), y = (uint32_t)((p / w) % h), b = (uint32_t)(p / ((uint64_t)w * h));
        dx[i] += 0.25f * dy[(((uint64_t)b * (h / 2) + y / 2) * (w / 2) + x / 2) * c + ch];
    }
}

// the plain path's image carried in feature channels 4..6: the network predicts a residual on it
__device__ __forceinline__ float base_of(const __nv_bfloat16* __restrict__ feats, uint64_t p, int ch) {
    return __bfloat162float(feats[p * 8 + 4 + ch]);
}

// output head: pred = base + z + bias (z = [P x 3] FP32 from the 1x1 convolution), L1 loss
// against target [P x 3]; writes d pred = sign(pred - target) / (3P) as bf16 [P x 8] (zero
// padded) and its transpose [8 x P], the bias gradient and the loss sum
__global__ void l1_head_kernel(const float* __restrict__ z, const float* __restrict__ bias,
                               const __nv_bfloat16* __restrict__ feats, const float* __restrict__ target, uint64_t P,
                               __nv_bfloat16* __restrict__ dpred, __nv_bfloat16* __restrict__ dpred_t, uint32_t ldp,
                               float* __restrict__ dbias, double* __restrict__ loss) {
    const float inv = 1.0f / (3.0f * (float)P);
    float db[3] = {0, 0, 0};
    double ls = 0.0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P; p += (uint64_t)gridDim.x * blockDim.x) {
        __align__(16) __nv_bfloat16 g8[8];
        for (int q = 0; q < 8; q++) g8[q] = __float2bfloat16_rn(0.0f);
        for (int ch = 0; ch < 3; ch++) {
            const float d = base_of(feats, p, ch) + z[p * 3 + ch] + bias[ch] - target[p * 3 + ch];
            ls += fabs((double)d);
            const float g = d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f);
            db[ch] += g;
            g8[ch] = __float2bfloat16_rn(g);
            dpred_t[(uint64_t)ch * ldp + p] = g8[ch];
        }
        *reinterpret_cast<uint4*>(dpred + p * 8) = *reinterpret_cast<const uint4*>(g8);
    }
    for (int ch = 0; ch < 3; ch++) {
        float v = db[ch];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(dbias + ch, v);
    }
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, ls);
}

// inference head: out = clamp(base + z + bias, 0, 1)
__global__ void head_kernel(const float* __restrict__ z, const float* __restrict__ bias,
                            const __nv_bfloat16* __restrict__ feats, uint64_t P, float* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < P * 3; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = fminf(fmaxf(base_of(feats, i / 3, (int)(i % 3)) + z[i] + bias[i % 3], 0.0f), 1.0f);
}

// Adam on FP32 master weights; refreshes the bf16 copy used as the forward GEMM operand
// (w16, [cout x K]) and the flipped transpose used by the input-gradient GEMM
// (wf16[ci][tap' * cout + co] = w[co][(8 - tap') * C + ci], C = K / 9), or for a 1x1 layer
// (taps = 1) the plain transpose wf16[ci][co] = w[co][ci] with its row stride ldf.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, uint32_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2, uint32_t cout, uint32_t K, uint32_t taps, __nv_bfloat16* __restrict__ w16,
                            __nv_bfloat16* __restrict__ wf16, uint32_t ldf) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float wi = w[i];
        if (lr > 0.0f) {
            const float gi = g[i];
            const float mi = b1 * m[i] + (1.0f - b1) * gi;
            const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
            w[i] = wi;
        }
        if (w16 == nullptr) continue;  // a bias vector
        const __nv_bfloat16 b = __float2bfloat16_rn(wi);
        w16[i] = b;
        const uint32_t co = i / K, k = i % K;
        const uint32_t C = K / taps, tap = k / C, ci = k % C;
        wf16[(uint64_t)ci * ldf + (uint64_t)(taps - 1 - tap) * cout + co] = b;
    }
}

// input features of a histogram (RGBA sums float4 per bin, W x H): 8 bf16 channels
//   [0] l = log10(1 + a * k2), [1..3] colour * l / a — the tonemap's log-density scaling
//   (tonemap.glsl:18-26) without the gamma step; [4..6] the plain path's tonemapped RGB of the
//   same histogram (base, may be null: zeros), on which the network predicts a residual;
//   [7] `level`, the caller's code of the run's sample count (the noise level)
__global__ void features_kernel(const float4* __restrict__ bins, uint64_t n, float k2, const double* __restrict__ stats,
                                const float4* __restrict__ base, float level, __nv_bfloat16* __restrict__ out) {
    const float k = k2 > 0.0f ? k2 : (float)((double)n / fmax(stats[0], 1e-30));
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 c = bins[i];
        __align__(16) __nv_bfloat16 f[8];
        float l = 0.0f, s = 0.0f;
        if (c.w > 0.0f) {
            l = log10f(1.0f + c.w * k);
            s = l / c.w;
        }
        f[0] = __float2bfloat16_rn(l);
        f[1] = __float2bfloat16_rn(c.x * s);
        f[2] = __float2bfloat16_rn(c.y * s);
        f[3] = __float2bfloat16_rn(c.z * s);
        const float4 bb = base ? base[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        f[4] = __float2bfloat16_rn(bb.x);
        f[5] = __float2bfloat16_rn(bb.y);
        f[6] = __float2bfloat16_rn(bb.z);
        f[7] = __float2bfloat16_rn(level);
        *reinterpret_cast<uint4*>(out + i * 8) = *reinterpret_cast<const uint4*>(f);
    }
}

unsigned grid_for(uint64_t n, unsigned threads) {
    const uint64_t g = (n + threads - 1) / threads;
    return (unsigned)(g < 152ull * 32 ? (g ? g : 1) : 152ull * 32);
}

}  // namespace

cudaError_t launch_im2col_t(const __nv_bfloat16* xa, uint32_t ca, int up, const __nv_bfloat16* xb, uint32_t cb,
                            uint32_t taps, uint32_t n, uint32_t h, uint32_t w, __nv_bfloat16* colt, uint32_t ldp,
                            cudaStream_t st) {
    const uint64_t total = (uint64_t)n * h * w * taps * (ca + cb);
    im2col_t_kernel<<<grid_for(total, 256), 256, 0, st>>>(xa, ca, up, xb, cb, taps, n, h, w, colt, ldp);
    return cudaGetLastError();
}

cudaError_t launch_avgpool(const __nv_bfloat16* x, uint32_t c, uint32_t n, uint32_t h, uint32_t w, __nv_bfloat16* y,
                           cudaStream_t st) {
    avgpool_kernel<<<grid_for((uint64_t)n * (h / 2) * (w / 2) * c, 256), 256, 0, st>>>(x, c, n, h, w, y);
    return cudaGetLastError();
}

cudaError_t launch_relu_back(const float* dy, const __nv_bfloat16* y, uint32_t c, uint64_t P, int relu,
                             __nv_bfloat16* dz, __nv_bfloat16* dzt, uint32_t ldp, float* dbias, cudaStream_t st) {
    if (c > 128) return cudaErrorInvalidValue;
    relu_back_kernel<<<(unsigned)((P + 31) / 32), 256, 0, st>>>(dy, y, c, P, relu, dz, dzt, ldp, dbias);
    return cudaGetLastError();
}

cudaError_t launch_split_concat_grad(const float* dx, uint32_t ca, uint32_t cb, uint32_t n, uint32_t h, uint32_t w,
                                     float* dlow, float* dskip, cudaStream_t st) {
    const uint64_t total = (uint64_t)n * (h / 2) * (w / 2) * ca + (uint64_t)n * h * w * cb;
    split_concat_grad_kernel<<<grid_for(total, 256), 256, 0, st>>>(dx, ca, cb, n, h, w, dlow, dskip);
    return cudaGetLastError();
}

cudaError_t launch_avgpool_back(const float* dy, uint32_t c, uint32_t n, uint32_t h, uint32_t w, float* dx,
                                cudaStream_t st) {
    avgpool_back_kernel<<<grid_for((uint64_t)n * h * w * c, 256), 256, 0, st>>>(dy, c, n, h, w, dx);
    return cudaGetLastError();
}

cudaError_t launch_l1_head(const float* z, const float* bias, const __nv_bfloat16* feats, const float* target,
                           uint64_t P, __nv_bfloat16* dpred, __nv_bfloat16* dpred_t, uint32_t ldp, float* dbias,
                           double* loss, cudaStream_t st) {
    l1_head_kernel<<<grid_for(P, 256), 256, 0, st>>>(z, bias, feats, target, P, dpred, dpred_t, ldp, dbias, loss);
    return cudaGetLastError();
}

cudaError_t launch_head(const float* z, const float* bias, const __nv_bfloat16* feats, uint64_t P, float* out,
                        cudaStream_t st) {
    head_kernel<<<grid_for(P * 3, 256), 256, 0, st>>>(z, bias, feats, P, out);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* w, const float* g, float* m, float* v, uint32_t n, float lr, float b1, float b2,
                        float eps, uint32_t t, uint32_t cout, uint32_t K, uint32_t taps, __nv_bfloat16* w16,
                        __nv_bfloat16* wf16, uint32_t ldf, cudaStream_t st) {
    const float c1 = 1.0f - powf(b1, (float)(t ? t : 1)), c2 = 1.0f - powf(b2, (float)(t ? t : 1));
    adam_kernel<<<grid_for(n, 256), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2, cout, K, taps, w16, wf16, ldf);
    return cudaGetLastError();
}

cudaError_t launch_features(const float4* bins, uint64_t n, float k2, const double* stats, const float4* base,
                            float level, __nv_bfloat16* out, cudaStream_t st) {
    features_kernel<<<grid_for(n, 256), 256, 0, st>>>(bins, n, k2, stats, base, level, out);
    return cudaGetLastError();
}

}  // namespace rfk
