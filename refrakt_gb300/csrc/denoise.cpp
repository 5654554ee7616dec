// Learned density estimation (no reference counterpart): a U-Net that maps a short-run histogram
// to the converged, tonemapped image.  Four levels of 32-48-64-96 channels, two 3x3 convolutions
// + ReLU per level, 2x2 average pooling down, nearest-neighbour upsampling and channel-concatenated
// skip connections up, a 1x1 output convolution to RGB.  Weights are FP32 masters with BF16 copies;
// every 3x3 convolution is an implicit-im2col tcgen05 BF16 GEMM with FP32 accumulation (gemm.cu:
// the GEMM gathers its operand rows from the NHWC activations), and the backward pass and the Adam
// update are the same GEMMs and hand-written kernels (denoise_ops.cu).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "denoise_ops.h"
#include "gemm.h"
#include "internal.h"
#include "kernels.h"
#include "refrakt.h"

using namespace rfk;

namespace {

struct Conv {
    uint32_t ca, cb, cout, taps;  // inputs: ca channels (upsampled when up) + cb skip channels
    int up, relu, level;
    int src_a, src_b;             // activation indices (-1 = network input / none)
    uint32_t K() const { return taps * (ca + cb); }
    uint32_t ldf() const { return (taps * cout + 7) & ~7u; }  // row stride of the flipped transpose
    // FP32 master weights [cout x K] and bias, gradients, Adam moments
    float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr;
    float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
    __nv_bfloat16 *w16 = nullptr, *wf16 = nullptr;
};

struct Act {  // one activation tensor (the output of conv i or of a pool)
    uint32_t c;
    int level;
    __nv_bfloat16* x = nullptr;  // bf16 [P_level x c]
    float* dy = nullptr;         // FP32 gradient, same shape
};

constexpr uint32_t kIn = 8;  // input feature channels (4 used)
const uint32_t kCh[4] = {32, 48, 64, 96};

}  // namespace

struct rf_denoiser {
    rf_denoiser_desc d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<Conv> convs;
    std::vector<Act> acts;          // acts[i] = output of convs[i]; pools appended after
    int out_conv = -1;
    uint64_t P0 = 0;                // pixels at level 0 (max)
    uint32_t H = 0, W = 0, N = 0;   // current shape
    // scratch
    __nv_bfloat16* colt = nullptr;  // [K x P]
    __nv_bfloat16* dz = nullptr;    // [P x cout]
    __nv_bfloat16* dzt = nullptr;   // [cout x P]
    float* dx = nullptr;            // [P x Ctot]
    float* z = nullptr;             // [P0 x 3] output head
    __nv_bfloat16 *dpred = nullptr, *dpred_t = nullptr;
    double* loss = nullptr;
    uint32_t step = 0;
    std::vector<void*> allocs;
};

namespace {

int cuda_fail(cudaError_t e, const char* what) { return fail(RF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

template <class T>
cudaError_t dalloc(rf_denoiser* d, T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T) + 16);
    if (e == cudaSuccess) {
        d->allocs.push_back(*p);
        e = cudaMemset(*p, 0, n * sizeof(T) + 16);
    }
    return e;
}

uint64_t level_pixels(uint32_t n, uint32_t h, uint32_t w, int level) {
    return (uint64_t)n * (h >> level) * (w >> level);
}

void build_graph(rf_denoiser* D) {
    auto conv = [&](uint32_t ca, uint32_t cb, uint32_t cout, int level, int src_a, int src_b, int up, uint32_t taps,
                    int relu) {
        Conv c{};
        c.ca = ca;
        c.cb = cb;
        c.cout = cout;
        c.level = level;
        c.src_a = src_a;
        c.src_b = src_b;
        c.up = up;
        c.taps = taps;
        c.relu = relu;
        D->convs.push_back(c);
        Act a{};
        a.c = cout;
        a.level = level;
        D->acts.push_back(a);
        return (int)D->convs.size() - 1;
    };
    // encoder
    int prev = -1;
    uint32_t cin = kIn;
    std::vector<int> skip(4, -1);
    for (int l = 0; l < 4; l++) {
        int a = conv(cin, 0, kCh[l], l, prev, -1, 0, 9, 1);
        int b = conv(kCh[l], 0, kCh[l], l, a, -1, 0, 9, 1);
        skip[l] = b;
        prev = b;
        cin = kCh[l];
    }
    // decoder
    int low = skip[3];
    for (int l = 2; l >= 0; l--) {
        int a = conv(kCh[l + 1], kCh[l], kCh[l], l, low, skip[l], 1, 9, 1);
        int b = conv(kCh[l], 0, kCh[l], l, a, -1, 0, 9, 1);
        low = b;
    }
    D->out_conv = conv(kCh[0], 0, 3, 0, low, -1, 0, 1, 0);
    // pooled activations: the input of encoder conv 'a' at levels 1..3
    for (int l = 1; l < 4; l++) {
        Act p{};
        p.c = kCh[l - 1];
        p.level = l;
        D->acts.push_back(p);
        const int pi = (int)D->acts.size() - 1;
        // encoder conv 'a' of level l is convs[2 l]; its input is the pool of level l - 1's output
        D->convs[2 * l].src_a = pi;
    }
}

// ---- forward ---------------------------------------------------------------------------------
int forward(rf_denoiser* D, const __nv_bfloat16* input, bool need_out) {
    const uint32_t n = D->N, h = D->H, w = D->W;
    cudaStream_t st = D->stream;
    for (size_t i = 0; i < D->convs.size(); i++) {
        Conv& c = D->convs[i];
        const int l = c.level;
        const uint32_t hl = h >> l, wl = w >> l;
        const uint64_t P = level_pixels(n, h, w, l);
        // pooled input of an encoder conv
        if (c.src_a >= (int)D->convs.size()) {
            Act& pa = D->acts[c.src_a];
            const Act& from = D->acts[2 * (l - 1) + 1];  // encoder conv 'b' of the level above
            cudaError_t e = launch_avgpool(from.x, pa.c, n, h >> (l - 1), w >> (l - 1), pa.x, st);
            if (e != cudaSuccess) return cuda_fail(e, "avgpool");
        }
        const __nv_bfloat16* xa = c.src_a < 0 ? input : D->acts[c.src_a].x;
        const __nv_bfloat16* xb = c.src_b < 0 ? nullptr : D->acts[c.src_b].x;
        GemmArgs g{};
        if (c.taps == 9) {  // implicit convolution: the GEMM gathers its im2col rows from xa, xb
            g.xa = xa;
            g.xb = xb;
            g.ca = c.ca;
            g.cb = c.cb;
            g.n = n;
            g.h = hl;
            g.w = wl;
            g.up = c.up;
        } else {
            g.A = xa;
            g.lda = c.ca;
        }
        g.B = c.w16;
        g.M = (uint32_t)P;
        g.N = c.cout;
        g.K = c.K();
        g.ldb = c.K();
        if ((int)i == D->out_conv) {
            if (!need_out) continue;
            g.C = D->z;
            g.ldc = 3;
            g.mode = kGemmStoreF32;
        } else {
            g.C = D->acts[i].x;
            g.ldc = c.cout;
            g.mode = kGemmStoreBF16;
            g.bias = c.b;
            g.relu = c.relu;
        }
        cudaError_t e = c.taps == 9 ? launch_gemm_conv(g, st) : launch_gemm(g, 1, st);
        if (e != cudaSuccess) return cuda_fail(e, "conv gemm");
    }
    return RF_OK;
}

uint32_t splits_for(uint64_t P) {
    const uint64_t kb = (P + 63) / 64;
    uint64_t s = kb / 256;  // >= 256 K blocks per CTA
    if (s < 1) s = 1;
    if (s > 64) s = 64;
    return (uint32_t)s;
}

// ---- backward + Adam -------------------------------------------------------------------------
int backward(rf_denoiser* D, const __nv_bfloat16* input, const float* target, float lr) {
    const uint32_t n = D->N, h = D->H, w = D->W;
    cudaStream_t st = D->stream;
    cudaError_t e = cudaSuccess;
    // zero gradients
    for (auto& a : D->acts)
        if (e == cudaSuccess) e = cudaMemsetAsync(a.dy, 0, level_pixels(n, h, w, a.level) * a.c * sizeof(float), st);
    for (auto& c : D->convs) {
        if (e == cudaSuccess) e = cudaMemsetAsync(c.gw, 0, (size_t)c.cout * c.K() * sizeof(float), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(c.gb, 0, c.cout * sizeof(float), st);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(D->loss, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_fail(e, "gradient clear");
    const uint64_t P0 = level_pixels(n, h, w, 0);

    for (int i = (int)D->convs.size() - 1; i >= 0; i--) {
        Conv& c = D->convs[i];
        const int l = c.level;
        const uint32_t hl = h >> l, wl = w >> l;
        const uint64_t P = level_pixels(n, h, w, l);
        const uint32_t ldp = (uint32_t)((P + 7) & ~7ull);  // row stride of the transposed operands
        const __nv_bfloat16* xa = c.src_a < 0 ? input : D->acts[c.src_a].x;
        const __nv_bfloat16* xb = c.src_b < 0 ? nullptr : D->acts[c.src_b].x;
        const __nv_bfloat16* dzp;
        const __nv_bfloat16* dztp;
        uint32_t ldz;
        if (i == D->out_conv) {
            e = launch_l1_head(D->z, c.b, input, target, P0, D->dpred, D->dpred_t, ldp, c.gb, D->loss, st);
            if (e != cudaSuccess) return cuda_fail(e, "l1 head");
            dzp = D->dpred;
            dztp = D->dpred_t;
            ldz = 8;
        } else {
            e = launch_relu_back(D->acts[i].dy, D->acts[i].x, c.cout, P, c.relu, D->dz, D->dzt, ldp, c.gb, st);
            if (e != cudaSuccess) return cuda_fail(e, "relu backward");
            dzp = D->dz;
            dztp = D->dzt;
            ldz = c.cout;
        }
        // weight gradient: gw[cout x K] += dz^T[cout x P] * col[P x K]
        GemmArgs gw{};
        gw.A = dztp;
        gw.lda = ldp;
        e = launch_im2col_t(xa, c.ca, c.up, xb, c.cb, c.taps, n, hl, wl, D->colt, ldp, st);
        if (e != cudaSuccess) return cuda_fail(e, "im2col_t");
        gw.B = D->colt;
        gw.ldb = ldp;
        gw.M = c.cout;
        gw.N = c.K();
        gw.K = (uint32_t)P;
        gw.C = c.gw;
        gw.ldc = c.K();
        gw.mode = kGemmAtomicF32;
        e = launch_gemm(gw, splits_for(P), st);
        if (e != cudaSuccess) return cuda_fail(e, "weight-gradient gemm");
        if (c.src_a < 0) continue;  // first layer: no input gradient
        // input gradient: dX[P x Ctot] = conv(dz, flipped transposed weights)
        GemmArgs gx{};
        if (c.taps == 9) {  // implicit convolution of dz
            gx.xa = dzp;
            gx.ca = c.cout;
            gx.n = n;
            gx.h = hl;
            gx.w = wl;
            gx.K = 9 * c.cout;
        } else {
            gx.A = dzp;
            gx.lda = ldz;
            gx.K = ldz;  // dpred is zero beyond its 3 channels; wf16 rows are zero there too
        }
        gx.B = c.wf16;
        gx.ldb = c.ldf();
        gx.M = (uint32_t)P;
        gx.N = c.ca + c.cb;
        const bool concat = c.cb > 0;
        const bool pooled = !concat && c.src_a >= (int)D->convs.size();
        if (!concat && !pooled) {  // straight into the source activation's gradient
            gx.C = D->acts[c.src_a].dy;
            gx.ldc = c.ca;
            gx.mode = kGemmAtomicF32;
        } else {
            gx.C = D->dx;
            gx.ldc = c.ca + c.cb;
            gx.mode = kGemmStoreF32;
        }
        e = c.taps == 9 ? launch_gemm_conv(gx, st) : launch_gemm(gx, 1, st);
        if (e != cudaSuccess) return cuda_fail(e, "input-gradient gemm");
        if (concat) {
            e = launch_split_concat_grad(D->dx, c.ca, c.cb, n, hl, wl, D->acts[c.src_a].dy, D->acts[c.src_b].dy, st);
            if (e != cudaSuccess) return cuda_fail(e, "concat gradient");
        } else if (pooled) {
            const int from = 2 * (l - 1) + 1;  // encoder conv 'b' of the level above
            e = launch_avgpool_back(D->dx, c.ca, n, h >> (l - 1), w >> (l - 1), D->acts[from].dy, st);
            if (e != cudaSuccess) return cuda_fail(e, "pool gradient");
        }
    }
    // Adam
    D->step++;
    for (auto& c : D->convs) {
        e = launch_adam(c.w, c.gw, c.mw, c.vw, c.cout * c.K(), lr, 0.9f, 0.999f, 1e-8f, D->step, c.cout, c.K(), c.taps,
                        c.w16, c.wf16, c.ldf(), st);
        if (e == cudaSuccess)
            e = launch_adam(c.b, c.gb, c.mb, c.vb, c.cout, lr, 0.9f, 0.999f, 1e-8f, D->step, c.cout, 1, 1, nullptr,
                            nullptr, 0, st);
        if (e != cudaSuccess) return cuda_fail(e, "adam");
    }
    return RF_OK;
}

int refresh_bf16(rf_denoiser* D) {
    for (auto& c : D->convs) {
        cudaError_t e = launch_adam(c.w, c.gw, c.mw, c.vw, c.cout * c.K(), 0.0f, 0.9f, 0.999f, 1e-8f, 1, c.cout, c.K(),
                                    c.taps, c.w16, c.wf16, c.ldf(), D->stream);
        if (e != cudaSuccess) return cuda_fail(e, "weight refresh");
    }
    return RF_OK;
}

int check_shape(rf_denoiser* D, uint32_t n, uint32_t h, uint32_t w) {
    if (n == 0 || h == 0 || w == 0 || h % 8 || w % 8)
        return fail(RF_ERR_INVALID_ARG, "denoiser: batch >= 1 and height, width multiples of 8 required");
    if ((uint64_t)n * h * w > D->P0) return fail(RF_ERR_CAPACITY, "denoiser: batch x height x width over the created capacity");
    D->N = n;
    D->H = h;
    D->W = w;
    return RF_OK;
}

}  // namespace

extern "C" {

int rf_denoiser_create(const rf_denoiser_desc* desc, rf_denoiser** out) {
    if (!desc || !out || desc->max_pixels == 0) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_create: bad arguments");
    *out = nullptr;
    auto* D = new rf_denoiser();
    D->d = *desc;
    D->device = desc->device;
    D->P0 = desc->max_pixels;
    auto bail = [&](int rc) { rf_denoiser_destroy(D); return rc; };
    if (cudaSetDevice(D->device) != cudaSuccess) return bail(fail(RF_ERR_NO_DEVICE, "rf_denoiser_create: no such device"));
    cudaError_t e = cudaStreamCreateWithFlags(&D->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "stream"));
    build_graph(D);
    // parameters, He-normal initialisation from a seeded generator
    std::mt19937_64 gen(desc->seed);
    for (auto& c : D->convs) {
        const size_t nw = (size_t)c.cout * c.K();
        std::vector<float> hw(nw);
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)c.K()));
        for (size_t k = 0; k < nw; k++) hw[k] = nd(gen);
        if (c.taps == 9 && c.src_a < 0)  // network input: zero the padding channel's weights
            for (uint32_t co = 0; co < c.cout; co++)
                for (uint32_t t = 0; t < 9; t++) hw[(size_t)co * c.K() + t * kIn + kIn - 1] = 0.0f;
        if (c.taps == 1)  // the output layer starts at zero: the first prediction is the plain image
            std::fill(hw.begin(), hw.end(), 0.0f);
        if (e == cudaSuccess) e = dalloc(D, &c.w, nw);
        if (e == cudaSuccess) e = dalloc(D, &c.gw, nw);
        if (e == cudaSuccess) e = dalloc(D, &c.mw, nw);
        if (e == cudaSuccess) e = dalloc(D, &c.vw, nw);
        if (e == cudaSuccess) e = dalloc(D, &c.b, c.cout);
        if (e == cudaSuccess) e = dalloc(D, &c.gb, c.cout);
        if (e == cudaSuccess) e = dalloc(D, &c.mb, c.cout);
        if (e == cudaSuccess) e = dalloc(D, &c.vb, c.cout);
        if (e == cudaSuccess) e = dalloc(D, &c.w16, nw);
        if (e == cudaSuccess) e = dalloc(D, &c.wf16, (size_t)(c.ca + c.cb) * c.ldf());
        if (e == cudaSuccess) e = cudaMemcpy(c.w, hw.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "rf_denoiser_create: parameters"));
    }
    // activations and scratch at the maximum size
    size_t colt = 0, dx = 0, dz = 0;
    for (auto& a : D->acts) {
        const uint64_t P = D->P0 >> (2 * a.level);
        if (e == cudaSuccess) e = dalloc(D, &a.x, P * a.c);
        if (e == cudaSuccess) e = dalloc(D, &a.dy, P * a.c);
    }
    for (auto& c : D->convs) {
        const uint64_t P = ((D->P0 >> (2 * c.level)) + 7) & ~7ull;
        colt = std::max<size_t>(colt, P * c.K());
        dx = std::max<size_t>(dx, P * (c.ca + c.cb));
        dz = std::max<size_t>(dz, P * std::max<uint32_t>(c.cout, 8));
    }
    if (e == cudaSuccess) e = dalloc(D, &D->colt, colt);
    if (e == cudaSuccess) e = dalloc(D, &D->dz, dz);
    if (e == cudaSuccess) e = dalloc(D, &D->dzt, dz);
    if (e == cudaSuccess) e = dalloc(D, &D->dx, dx);
    if (e == cudaSuccess) e = dalloc(D, &D->z, D->P0 * 3);
    if (e == cudaSuccess) e = dalloc(D, &D->dpred, D->P0 * 8);
    if (e == cudaSuccess) e = dalloc(D, &D->dpred_t, ((D->P0 + 7) & ~7ull) * 8);
    if (e == cudaSuccess) e = dalloc(D, &D->loss, 1);
    if (e != cudaSuccess) return bail(cuda_fail(e, "rf_denoiser_create: activations"));
    if (int rc = refresh_bf16(D)) return bail(rc);
    e = cudaStreamSynchronize(D->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "rf_denoiser_create"));
    *out = D;
    return RF_OK;
}

int rf_denoiser_destroy(rf_denoiser* D) {
    if (!D) return RF_OK;
    cudaSetDevice(D->device);
    if (D->stream) cudaStreamSynchronize(D->stream);
    for (void* p : D->allocs) cudaFree(p);
    if (D->stream) cudaStreamDestroy(D->stream);
    delete D;
    return RF_OK;
}

int rf_denoiser_set_stream(rf_denoiser* D, void* stream) {
    if (!D) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_set_stream: null");
    D->stream = static_cast<cudaStream_t>(stream);  // the caller's stream from here on
    return RF_OK;
}

int rf_denoiser_sync(rf_denoiser* D) {
    if (!D) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_sync: null");
    cudaSetDevice(D->device);
    cudaError_t e = cudaStreamSynchronize(D->stream);
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_sync");
    return RF_OK;
}

int rf_denoiser_num_layers(const rf_denoiser* D) { return D ? (int)D->convs.size() : -1; }

int rf_denoiser_layer(const rf_denoiser* D, int i, rf_denoiser_layer_info* out) {
    if (!D || !out || i < 0 || i >= (int)D->convs.size()) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_layer: bad index");
    const Conv& c = D->convs[i];
    out->in_a = c.ca;
    out->in_b = c.cb;
    out->out = c.cout;
    out->taps = c.taps;
    out->upsample = c.up;
    out->relu = c.relu;
    out->level = c.level;
    auto src = [&](int s) {
        if (s < 0) return -1;
        if (s < (int)D->convs.size()) return s;
        return -100 - (D->acts[s].level);  // pooled output of the level above's last conv
    };
    out->src_a = src(c.src_a);
    out->src_b = src(c.src_b);
    return RF_OK;
}

size_t rf_denoiser_num_params(const rf_denoiser* D) {
    if (!D) return 0;
    size_t n = 0;
    for (auto& c : D->convs) n += (size_t)c.cout * c.K() + c.cout;
    return n;
}

int rf_denoiser_get_params(rf_denoiser* D, float* host, size_t cap) {
    if (!D || !host || cap < rf_denoiser_num_params(D)) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_get_params: bad arguments");
    cudaSetDevice(D->device);
    cudaError_t e = cudaStreamSynchronize(D->stream);
    size_t o = 0;
    for (auto& c : D->convs) {
        const size_t nw = (size_t)c.cout * c.K();
        if (e == cudaSuccess) e = cudaMemcpy(host + o, c.w, nw * sizeof(float), cudaMemcpyDeviceToHost);
        o += nw;
        if (e == cudaSuccess) e = cudaMemcpy(host + o, c.b, c.cout * sizeof(float), cudaMemcpyDeviceToHost);
        o += c.cout;
    }
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_get_params");
    return RF_OK;
}

int rf_denoiser_set_params(rf_denoiser* D, const float* host, size_t count) {
    if (!D || !host || count != rf_denoiser_num_params(D)) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_set_params: bad arguments");
    cudaSetDevice(D->device);
    cudaError_t e = cudaStreamSynchronize(D->stream);
    size_t o = 0;
    for (auto& c : D->convs) {
        const size_t nw = (size_t)c.cout * c.K();
        if (e == cudaSuccess) e = cudaMemcpy(c.w, host + o, nw * sizeof(float), cudaMemcpyHostToDevice);
        o += nw;
        if (e == cudaSuccess) e = cudaMemcpy(c.b, host + o, c.cout * sizeof(float), cudaMemcpyHostToDevice);
        o += c.cout;
    }
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_set_params");
    return refresh_bf16(D);
}

int rf_denoiser_features(const float* bins_rgba, uint32_t width, uint32_t height, float k2, const float* base_rgba,
                         float level, void* out_bf16, void* stream) {
    if (!bins_rgba || !out_bf16 || !width || !height) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_features: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* stats = nullptr;
    cudaError_t e = cudaSuccess;
    if (!(k2 > 0.0f)) {
        e = cudaMallocAsync(&stats, 3 * sizeof(double), st);
        if (e == cudaSuccess) e = launch_stats(reinterpret_cast<const float4*>(bins_rgba), width, height, stats, st);
    }
    if (e == cudaSuccess)
        e = launch_features(reinterpret_cast<const float4*>(bins_rgba), (uint64_t)width * height, k2, stats,
                            reinterpret_cast<const float4*>(base_rgba), level, static_cast<__nv_bfloat16*>(out_bf16), st);
    if (stats) cudaFreeAsync(stats, st);
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_features");
    return RF_OK;
}

int rf_denoiser_infer(rf_denoiser* D, const void* feats, uint32_t n, uint32_t h, uint32_t w, float* out_rgb) {
    if (!D || !feats || !out_rgb) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_infer: null argument");
    if (int rc = check_shape(D, n, h, w)) return rc;
    cudaSetDevice(D->device);
    if (int rc = forward(D, static_cast<const __nv_bfloat16*>(feats), true)) return rc;
    const Conv& oc = D->convs[D->out_conv];
    cudaError_t e = launch_head(D->z, oc.b, static_cast<const __nv_bfloat16*>(feats), (uint64_t)n * h * w, out_rgb,
                                D->stream);
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_infer");
    return RF_OK;
}

int rf_denoiser_train_step(rf_denoiser* D, const void* feats, const float* target_rgb, uint32_t n, uint32_t h,
                           uint32_t w, float lr, double* loss) {
    if (!D || !feats || !target_rgb) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_train_step: null argument");
    if (int rc = check_shape(D, n, h, w)) return rc;
    cudaSetDevice(D->device);
    const auto* in = static_cast<const __nv_bfloat16*>(feats);
    if (int rc = forward(D, in, true)) return rc;
    if (int rc = backward(D, in, target_rgb, lr)) return rc;
    if (loss) {
        double l = 0;
        cudaError_t e = cudaMemcpyAsync(&l, D->loss, sizeof(double), cudaMemcpyDeviceToHost, D->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(D->stream);
        if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_train_step");
        *loss = l / (3.0 * (double)n * h * w);
    }
    return RF_OK;
}

int rf_denoiser_gradients(rf_denoiser* D, float* host, size_t cap) {
    if (!D || !host || cap < rf_denoiser_num_params(D)) return fail(RF_ERR_INVALID_ARG, "rf_denoiser_gradients: bad arguments");
    cudaSetDevice(D->device);
    cudaError_t e = cudaStreamSynchronize(D->stream);
    size_t o = 0;
    for (auto& c : D->convs) {
        const size_t nw = (size_t)c.cout * c.K();
        if (e == cudaSuccess) e = cudaMemcpy(host + o, c.gw, nw * sizeof(float), cudaMemcpyDeviceToHost);
        o += nw;
        if (e == cudaSuccess) e = cudaMemcpy(host + o, c.gb, c.cout * sizeof(float), cudaMemcpyDeviceToHost);
        o += c.cout;
    }
    if (e != cudaSuccess) return cuda_fail(e, "rf_denoiser_gradients");
    return RF_OK;
}

}  // extern "C"
