// Image passes after the chaos game: adaptive density estimation, FP64 histogram statistics
// and the log-density tonemap with a supersample box filter.
//
// The reference does density estimation as a GL point-sprite raster pass with additive
// blending (src/main.cpp:490-515, shaders/density_vert.glsl:26-63, density_frag.glsl:9-18):
// every non-empty bin becomes a sprite of radius r = max(min, min(R, int(R / a^curve))) whose
// fragments add color * (1 - d^2) * (2/pi) / r^2.  Here each CTA owns an output tile and gathers
// it from the tile and its halo staged in shared memory, walking either the whole box of the
// tile's largest radius or only its large discs, whichever is less work for that tile (radii
// above 12 gather from global memory).  The disc is the symmetric restatement
// 4 (dx^2 + dy^2) <= (2r + 1)^2 with
// d^2 = (dx^2 + dy^2) / (r + 0.5)^2 (the GL sprite's sub-pixel centring depends on point
// rasterisation rules).  Radii come from thresholds on a, computed on the host in FP64, and
// the kernel weights from a per-radius table, so every radius and weight is exactly defined.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "kernels.h"

namespace rfk {

constexpr int kDeMaxSmemR = 12;  // radius handled through shared-memory tiles

struct DeTables {
    float thr[101];      // thr[k-1]: bin radius >= k  <=>  a <= thr (curve > 0) or a >= thr (curve < 0)
    int R, min_r, mode;  // mode 0: curve > 0, 1: curve < 0, 2: curve == 0 (radius R)
    int wbase[102];      // offset of radius r's (r+1)^2 weights
};

__device__ __forceinline__ int de_radius(float a, const DeTables& T) {
    int r;
    if (T.mode == 2) r = T.R;
    else {
        // thresholds are monotone: binary search for the largest k with the condition true
        int lo = 0, hi = T.R;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            const bool ok = (T.mode == 0) ? (a <= T.thr[mid - 1]) : (a >= T.thr[mid - 1]);
            if (ok) lo = mid; else hi = mid - 1;
        }
        r = lo;
    }
    return r > T.min_r ? r : T.min_r;  // max(min, min(R, int(R / a^curve))), density_vert.glsl:35-44
}

// pass 1: radius per bin (255 = empty)
__global__ void de_radius_kernel(const float4* __restrict__ in, size_t n, const DeTables T, uint8_t* __restrict__ rad) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float a = in[i].w;
        rad[i] = (a == 0.0f || a != a) ? (uint8_t)255 : (uint8_t)de_radius(a, T);
    }
}

// pass 2: a CTA owns a 32 x 8 output tile.  It stages the colours and radii of the tile and
// its R halo in shared memory and forms each output bin as a gather in one of two ways, chosen
// per tile by their work:
//   box  — sum the bins within the tile's largest radius rmax whose disc covers the output:
//          up to (2 rmax + 1)^2 taps per output, rows whose largest disc cannot reach the output
//          skipped and each row's span cut to its largest radius;
//   list — the discs of radius 0 and 1 from the 3 x 3 neighbourhood, plus a compact list of the
//          tile's larger discs (those reaching the tile), which every thread walks in the same
//          order (shared-memory broadcasts): 9 + list-length taps per output.
// Dense regions (radius 0 and 1 at converged sample counts, a few sparse bins) take the list;
// sparse fringes full of large discs take the box.  The sum is deterministic either way.
constexpr int kDsX = 32, kDsY = 8, kDsThreads = 256;

template <int R>
__host__ __device__ constexpr size_t de_tile_smem() {
    return (size_t)(kDsX + 2 * R) * (kDsY + 2 * R) * (16 + 4 + 1) + 16 + 64 + 4 * (kDsY + 2 * R);
}

template <int R>
__global__ void __launch_bounds__(kDsThreads) de_tile_kernel(
    const float4* __restrict__ in, const uint8_t* __restrict__ rad, uint32_t w, uint32_t h,
    const float* __restrict__ weights, const DeTables T, float4* __restrict__ out) {
    constexpr int SW = kDsX + 2 * R, SH = kDsY + 2 * R, NS = SW * SH, NO = kDsX * kDsY;
    extern __shared__ __align__(16) unsigned char smem[];
    float4* s_c = reinterpret_cast<float4*>(smem);                  // NS colours
    int* s_list = reinterpret_cast<int*>(s_c + NS);                 // indices of discs of radius >= 2
    uint8_t* s_r = reinterpret_cast<uint8_t*>(s_list + NS);         // NS radii (255: empty)
    int* s_stat = reinterpret_cast<int*>(s_r + ((NS + 15) & ~15));  // [0] rmax, [1..8] per-warp counts
    int* s_rowmax = s_stat + 16;                                     // SH: largest radius per staged row
    const int tx0 = blockIdx.x * kDsX, ty0 = blockIdx.y * kDsY;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_stat[0] = 0;
    for (int i = threadIdx.x; i < SH; i += kDsThreads) s_rowmax[i] = -1;
    __syncthreads();
    int rmax = 0, nl = 0;
    // stage the tile + halo; list the large discs that reach the tile in source order (a
    // ballot-and-prefix compaction, so the list and the sums are the same on every run)
    for (int i0 = 0; i0 < NS; i0 += kDsThreads) {
        const int i = i0 + (int)threadIdx.x;
        bool big = false;
        if (i < NS) {
            const int gx = tx0 - R + i % SW, gy = ty0 - R + i / SW;
            uint8_t r = 255;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (gx >= 0 && gy >= 0 && gx < (int)w && gy < (int)h) {
                const size_t gi = (size_t)gy * w + gx;
                r = rad[gi];
                if (r != 255) v = in[gi];
            }
            s_r[i] = r;
            s_c[i] = v;
            if (r != 255) atomicMax(&s_rowmax[i / SW], (int)r);
            if (r != 255 && gx - r <= tx0 + kDsX - 1 && gx + r >= tx0 && gy - r <= ty0 + kDsY - 1 && gy + r >= ty0) {
                rmax = max(rmax, (int)r);
                big = r >= 2;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, big);
        if (lane == 0) s_stat[1 + warp] = __popc(m);
        __syncthreads();
        int off = nl, tot = 0;
        for (int q = 0; q < kDsThreads / 32; q++) {
            const int c = s_stat[1 + q];
            if (q < warp) off += c;
            tot += c;
        }
        if (big) s_list[off + __popc(m & ((1u << lane) - 1u))] = i;
        nl += tot;
        __syncthreads();
    }
    atomicMax(&s_stat[0], rmax);
    __syncthreads();
    const int rm = s_stat[0];
    const bool use_list = 9 + nl < (2 * rm + 1) * (2 * rm + 1);
    for (int o = threadIdx.x; o < NO; o += kDsThreads) {
        const int ox = o % kDsX, oy = o / kDsX;
        float4 a4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (use_list) {
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int si = (oy + R + dy) * SW + ox + R + dx;
                    const int r = s_r[si];
                    if (r > 1 || (r == 0 && (dx | dy))) continue;  // r = 255 (empty) fails r > 1
                    const float wt = r == 0 ? 1.0f : weights[T.wbase[1] + (dy ? 1 : 0) * 2 + (dx ? 1 : 0)];
                    const float4 v = s_c[si];
                    a4.x = fmaf(v.x, wt, a4.x);
                    a4.y = fmaf(v.y, wt, a4.y);
                    a4.z = fmaf(v.z, wt, a4.z);
                    a4.w = fmaf(v.w, wt, a4.w);
                }
            for (int k = 0; k < nl; k++) {
                const int si = s_list[k];
                const int r = s_r[si];
                const int ax = abs(ox + R - si % SW), ay = abs(oy + R - si / SW);
                if (4 * (ax * ax + ay * ay) > (2 * r + 1) * (2 * r + 1)) continue;
                const float wt = weights[T.wbase[r] + ay * (r + 1) + ax];
                const float4 v = s_c[si];
                a4.x = fmaf(v.x, wt, a4.x);
                a4.y = fmaf(v.y, wt, a4.y);
                a4.z = fmaf(v.z, wt, a4.z);
                a4.w = fmaf(v.w, wt, a4.w);
            }
        } else {
            for (int dy = -rm; dy <= rm; dy++) {
                const int ay = dy < 0 ? -dy : dy;
                const int rr = min(rm, s_rowmax[oy + R + dy]);  // no disc of this row reaches |dy| rows
                if (rr < ay) continue;
                for (int dx = -rr; dx <= rr; dx++) {
                    const int si = (oy + R + dy) * SW + ox + R + dx;
                    const int r = s_r[si];
                    const int ax = dx < 0 ? -dx : dx;
                    if (r == 255 || ax > r || ay > r) continue;
                    float wt = 1.0f;
                    if (r > 0) {
                        if (4 * (ax * ax + ay * ay) > (2 * r + 1) * (2 * r + 1)) continue;
                        wt = weights[T.wbase[r] + ay * (r + 1) + ax];
                    }
                    const float4 v = s_c[si];
                    a4.x = fmaf(v.x, wt, a4.x);
                    a4.y = fmaf(v.y, wt, a4.y);
                    a4.z = fmaf(v.z, wt, a4.z);
                    a4.w = fmaf(v.w, wt, a4.w);
                }
            }
        }
        const int gx = tx0 + ox, gy = ty0 + oy;
        if (gx < (int)w && gy < (int)h) out[(size_t)gy * w + gx] = a4;
    }
}

template <int R>
static cudaError_t set_de_tile_smem() {
    return cudaFuncSetAttribute(de_tile_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)de_tile_smem<R>());
}

// the DE kernels' shared-memory limits, set once per device before any launch (also before a
// stream capture that contains DE)
cudaError_t density_prepare() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static bool done[64] = {};
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    e = set_de_tile_smem<3>();
    if (e == cudaSuccess) e = set_de_tile_smem<6>();
    if (e == cudaSuccess) e = set_de_tile_smem<9>();
    if (e == cudaSuccess) e = set_de_tile_smem<kDeMaxSmemR>();
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

template <int R>
static cudaError_t launch_de_tile(const float4* in, const uint8_t* rad, uint32_t w, uint32_t h, const float* dw,
                                  const DeTables& T, float4* out, cudaStream_t st) {
    const size_t smem = de_tile_smem<R>();
    cudaError_t e = density_prepare();
    if (e != cudaSuccess) return e;
    const dim3 grid((w + kDsX - 1) / kDsX, (h + kDsY - 1) / kDsY);
    de_tile_kernel<R><<<grid, kDsThreads, smem, st>>>(in, rad, w, h, dw, T, out);
    return cudaGetLastError();
}

// large radii: the gather straight from global memory
__global__ void de_gather_global_kernel(const float4* __restrict__ in, const uint8_t* __restrict__ rad,
                                        uint32_t w, uint32_t h, const float* __restrict__ weights,
                                        const DeTables T, float4* __restrict__ out) {
    const int ox = blockIdx.x * blockDim.x + threadIdx.x, oy = blockIdx.y;
    if (ox >= (int)w) return;
    const int Rm = T.R > T.min_r ? T.R : T.min_r;
    float4 acc = make_float4(0, 0, 0, 0);
    for (int dy = -Rm; dy <= Rm; dy++) {
        const int gy = oy + dy;
        if (gy < 0 || gy >= (int)h) continue;
        for (int dx = -Rm; dx <= Rm; dx++) {
            const int gx = ox + dx;
            if (gx < 0 || gx >= (int)w) continue;
            const size_t gi = (size_t)gy * w + gx;
            const int r = rad[gi];
            if (r == 255) continue;
            const int ax = dx < 0 ? -dx : dx, ay = dy < 0 ? -dy : dy;
            if (ax > r || ay > r) continue;
            float wt;
            if (r == 0) wt = 1.0f;
            else {
                if (4 * (ax * ax + ay * ay) > (2 * r + 1) * (2 * r + 1)) continue;
                wt = weights[T.wbase[r] + ay * (r + 1) + ax];
            }
            const float4 v = in[gi];
            acc.x = fmaf(v.x, wt, acc.x);
            acc.y = fmaf(v.y, wt, acc.y);
            acc.z = fmaf(v.z, wt, acc.z);
            acc.w = fmaf(v.w, wt, acc.w);
        }
    }
    out[(size_t)oy * w + ox] = acc;
}

// FP64 sum and max of the density channel, count of non-empty bins
__global__ void stats_kernel(const float4* __restrict__ in, size_t n, double* out) {
    double s = 0.0, m = 0.0;
    unsigned long long nz = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double a = (double)in[i].w;
        s += a;
        m = a > m ? a : m;
        nz += (a > 0.0) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
        nz += __shfl_down_sync(0xffffffffu, nz, o);
    }
    __shared__ double ss[32], sm[32];
    __shared__ unsigned long long sn[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { ss[wid] = s; sm[wid] = m; sn[wid] = nz; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? ss[lane] : 0.0;
        m = lane < nw ? sm[lane] : 0.0;
        nz = lane < nw ? sn[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_down_sync(0xffffffffu, s, o);
            m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
            nz += __shfl_down_sync(0xffffffffu, nz, o);
        }
        if (lane == 0) {
            atomicAdd(out, s);
            // a >= 0: the IEEE bit pattern orders like the value
            atomicMax(reinterpret_cast<unsigned long long*>(out + 1), (unsigned long long)__double_as_longlong(m));
            atomicAdd(reinterpret_cast<unsigned long long*>(out + 2), nz);
        }
    }
}

// tonemap.glsl:18-38 with an ss x ss box filter: per bin c *= 0.5*brightness*log10(1 + a*k2)/a,
// mean over the block, then z = a^(1/gamma), rgb = clamp(mix(rgb^(1/gamma), (z/a)*rgb, vibrancy)).
// A block with no density (where the shader would divide 0 by 0) is opaque black.
__global__ void tonemap_kernel(const float4* __restrict__ in, uint32_t w, uint32_t h, uint32_t ss, float gamma,
                               float brightness, float vibrancy, float k2, const double* __restrict__ stats,
                               float4* __restrict__ out_f32, uchar4* __restrict__ out8) {
    const uint32_t ow = w / ss, oh = h / ss;
    const uint32_t ox = blockIdx.x * blockDim.x + threadIdx.x, oy = blockIdx.y;
    if (ox >= ow || oy >= oh) return;
    float k = k2;
    if (!(k > 0.0f)) {
        const double sum = stats ? stats[0] : 0.0;
        k = sum > 0.0 ? (float)((double)w * (double)h / sum) : 1.0f;
    }
    float4 acc = make_float4(0, 0, 0, 0);
    for (uint32_t j = 0; j < ss; j++) {
        const float4* row = in + (size_t)(oy * ss + j) * w + (size_t)ox * ss;
        for (uint32_t i = 0; i < ss; i++) {
            const float4 c = row[i];
            if (c.w > 0.0f) {
                const float ls = 0.5f * brightness * log1pf(c.w * k) * 0.434294481903251827651128918916f / c.w;
                acc.x = fmaf(c.x, ls, acc.x);
                acc.y = fmaf(c.y, ls, acc.y);
                acc.z = fmaf(c.z, ls, acc.z);
                acc.w = fmaf(c.w, ls, acc.w);
            }
        }
    }
    const float inv = 1.0f / (float)(ss * ss);
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    const float a = acc.w * inv;
    if (a > 0.0f) {
        const float ig = 1.0f / gamma;
        const float gf = powf(a, ig) / a;
        const float rgb[3] = {acc.x * inv, acc.y * inv, acc.z * inv};
        float res[3];
        for (int q = 0; q < 3; q++) {
            const float v = powf(rgb[q], ig) * (1.0f - vibrancy) + gf * rgb[q] * vibrancy;
            res[q] = fminf(fmaxf(v, 0.0f), 1.0f);
        }
        o = make_float4(res[0], res[1], res[2], 1.0f);
    }
    const size_t oi = (size_t)oy * ow + ox;
    if (out_f32) out_f32[oi] = o;
    if (out8) out8[oi] = make_uchar4((unsigned char)lrintf(o.x * 255.0f), (unsigned char)lrintf(o.y * 255.0f),
                                     (unsigned char)lrintf(o.z * 255.0f), 255);
}

// ---------------------------------------------------------------------------------------------
static void de_tables(int R, int min_r, float curve, DeTables& T, std::vector<float>& wts) {
    T.R = R;
    T.min_r = min_r;
    T.mode = (curve > 0.0f) ? 0 : (curve < 0.0f ? 1 : 2);
    for (int k = 1; k <= R; k++) {
        // int(R / a^curve) >= k  <=>  a^curve <= R / k
        const double t = std::pow((double)R / (double)k, 1.0 / (double)curve);
        float f = (float)t;
        if (T.mode == 0 && (double)f > t) f = std::nextafter(f, -INFINITY);  // a <= f  <=>  a <= t
        if (T.mode == 1 && (double)f < t) f = std::nextafter(f, INFINITY);   // a >= f  <=>  a >= t
        T.thr[k - 1] = f;
    }
    wts.clear();
    const int rmax = R > min_r ? R : min_r;
    for (int r = 0; r <= rmax && r <= 100; r++) {
        T.wbase[r] = (int)wts.size();
        const double nf = 0.63661977236 / (double)(r > 0 ? r * r : 1);
        const double den = (r + 0.5) * (r + 0.5);
        for (int ay = 0; ay <= r; ay++)
            for (int ax = 0; ax <= r; ax++) {
                const int d2 = ax * ax + ay * ay;
                wts.push_back(r == 0 ? 1.0f : (float)((1.0 - (double)d2 / den) * nf));
            }
    }
}

static cudaError_t launch_density_passes(const float4* in, uint32_t w, uint32_t h, const DeTables& T, float4* out,
                                         uint8_t* rad, const float* dw, cudaStream_t st);

cudaError_t launch_density(const float4* in, uint32_t w, uint32_t h, int R, int min_r, float curve, float4* out,
                           cudaStream_t st) {
    DeTables T;
    std::vector<float> wts;
    de_tables(R, min_r, curve, T, wts);
    const size_t n = (size_t)w * h;
    uint8_t* rad = nullptr;
    float* dw = nullptr;
    cudaError_t e = cudaMallocAsync(&rad, n, st);
    if (e != cudaSuccess) return e;
    e = cudaMallocAsync(&dw, wts.size() * sizeof(float), st);
    if (e != cudaSuccess) { cudaFreeAsync(rad, st); return e; }
    cudaMemcpyAsync(dw, wts.data(), wts.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    e = launch_density_passes(in, w, h, T, out, rad, dw, st);
    cudaFreeAsync(rad, st);
    cudaFreeAsync(dw, st);
    return e;
}

size_t density_weight_count(int R, int min_r) {
    const int rmax = R > min_r ? R : min_r;
    size_t n = 0;
    for (int r = 0; r <= rmax && r <= 100; r++) n += (size_t)(r + 1) * (r + 1);
    return n;
}

static cudaError_t launch_density_passes(const float4* in, uint32_t w, uint32_t h, const DeTables& T, float4* out,
                                         uint8_t* rad, const float* dw, cudaStream_t st) {
    const size_t n = (size_t)w * h;
    de_radius_kernel<<<1024, 256, 0, st>>>(in, n, T, rad);
    const int rmax = T.R > T.min_r ? T.R : T.min_r;
    if (rmax <= 3) return launch_de_tile<3>(in, rad, w, h, dw, T, out, st);
    if (rmax <= 6) return launch_de_tile<6>(in, rad, w, h, dw, T, out, st);
    if (rmax <= 9) return launch_de_tile<9>(in, rad, w, h, dw, T, out, st);
    if (rmax <= kDeMaxSmemR) return launch_de_tile<kDeMaxSmemR>(in, rad, w, h, dw, T, out, st);
    else de_gather_global_kernel<<<dim3((w + 127) / 128, h), 128, 0, st>>>(in, rad, w, h, dw, T, out);
    return cudaGetLastError();
}

// The same two passes with scratch the caller provides (a byte per bin for the radii, `dw_cap`
// floats for the kernel weights); nothing is allocated.
cudaError_t launch_density_scratch(const float4* in, uint32_t w, uint32_t h, int R, int min_r, float curve,
                                   float4* out, uint8_t* rad, float* dw, size_t dw_cap, cudaStream_t st) {
    DeTables T;
    std::vector<float> wts;
    de_tables(R, min_r, curve, T, wts);
    if (wts.size() > dw_cap) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(dw, wts.data(), wts.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    return launch_density_passes(in, w, h, T, out, rad, dw, st);
}

void density_weights(int R, int min_r, std::vector<float>& wts) {
    DeTables T;
    de_tables(R, min_r, 1.0f, T, wts);
}

cudaError_t launch_density_resident(const float4* in, uint32_t w, uint32_t h, int R, int min_r, float curve,
                                    float4* out, uint8_t* rad, const float* dw, cudaStream_t st) {
    DeTables T;
    std::vector<float> wts;
    de_tables(R, min_r, curve, T, wts);
    return launch_density_passes(in, w, h, T, out, rad, dw, st);
}

cudaError_t launch_stats(const float4* in, uint32_t w, uint32_t h, double* out3, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out3, 0, 3 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    stats_kernel<<<1024, 256, 0, st>>>(in, (size_t)w * h, out3);
    return cudaGetLastError();
}

// out2 = (sum h, sum h^2) of a hit-count histogram, FP64; out2 must start at zero
__global__ void hit_moments_kernel(const uint32_t* __restrict__ hits, size_t n, double* out2) {
    double s = 0.0, q = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = (double)hits[i];
        s += v;
        q += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out2, s);
        atomicAdd(out2 + 1, q);
    }
}

cudaError_t launch_hit_moments(const uint32_t* hits, uint32_t w, uint32_t h, double* out2, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    hit_moments_kernel<<<256, 256, 0, st>>>(hits, (size_t)w * h, out2);
    return cudaGetLastError();
}

cudaError_t launch_tonemap(const float4* in, uint32_t w, uint32_t h, uint32_t ss, float gamma, float brightness,
                           float vibrancy, float k2, const double* stats, float4* out_f32, uchar4* out8,
                           cudaStream_t st) {
    const uint32_t ow = w / ss, oh = h / ss;
    tonemap_kernel<<<dim3((ow + 127) / 128, oh), 128, 0, st>>>(in, w, h, ss, gamma, brightness, vibrancy, k2, stats,
                                                               out_f32, out8);
    return cudaGetLastError();
}

}  // namespace rfk
