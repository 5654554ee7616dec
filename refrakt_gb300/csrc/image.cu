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
    double wsum[101];    // the weights of a whole disc of radius r, summed in FP64
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

// block-wide FP64 sum, added to *out by one thread per block (blockDim.x a multiple of 32, <= 1024)
__device__ __forceinline__ void block_sum_to(double s, double* out) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = s;
    __syncthreads();
    if (wid == 0) {
        s = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(out, s);
    }
}

// pass 1 of the fused image tail: the radius per bin, and the total density of the estimator's
// output, sum_out a = sum over bins of a * (the kernel weights of its disc inside the grid) — the
// log-density scale's sum (k2 = W * H / sum a) without a pass over the output.  A whole disc's
// weights come from T.wsum; a disc cut by the grid's edge adds, per row inside the grid,
// the difference of two prefix sums of that row's FP32 weights, staged per CTA in shared memory
// for every radius up to kDeMaxSmemR (the fused path's radii).
constexpr int kRowPrefixFloats = 1638;  // sum over r <= 12 of (r + 1) rows of 2r + 2 prefix sums

__global__ void de_radius_sum_kernel(const float4* __restrict__ in, uint32_t w, uint32_t h, const DeTables T,
                                     const float* __restrict__ weights, uint8_t* __restrict__ rad,
                                     double* __restrict__ sum_out) {
    __shared__ float s_pre[kRowPrefixFloats];
    __shared__ int s_pbase[kDeMaxSmemR + 1];
    const int rmax = min(kDeMaxSmemR, T.R > T.min_r ? T.R : T.min_r);
    if (threadIdx.x == 0) {
        int off = 0;
        for (int r = 0; r <= kDeMaxSmemR; r++) {
            s_pbase[r] = off;
            off += (r + 1) * (2 * r + 2);
        }
    }
    __syncthreads();
    // row (r, ay): pre[j] = sum of the disc's weights at dx = -r .. -r + j - 1
    for (int q = threadIdx.x; q < (rmax + 1) * (rmax + 1); q += blockDim.x) {
        const int r = q / (rmax + 1), ay = q % (rmax + 1);
        if (r < 1 || ay > r) continue;
        float* pre = s_pre + s_pbase[r] + ay * (2 * r + 2);
        float acc = 0.0f;
        pre[0] = 0.0f;
        for (int dx = -r; dx <= r; dx++) {
            const int ax = dx < 0 ? -dx : dx;
            if (4 * (ax * ax + ay * ay) <= (2 * r + 1) * (2 * r + 1)) acc += weights[T.wbase[r] + ay * (r + 1) + ax];
            pre[dx + r + 1] = acc;
        }
    }
    __syncthreads();
    // a thread's bins (a few dozen) are summed in FP32, the partial sums in FP64 (this part's
    // FP64 rate is a small fraction of its FP32 rate)
    __shared__ float s_wsum[kDeMaxSmemR + 1];
    for (int r = threadIdx.x; r <= kDeMaxSmemR; r += blockDim.x) s_wsum[r] = (float)T.wsum[r];
    __syncthreads();
    const uint32_t n = w * h;  // < 2^32 (the caller's grids hold fewer bins)
    float s = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float a = in[i].w;
        if (a == 0.0f || a != a) {
            rad[i] = 255;
            continue;
        }
        const int r = de_radius(a, T);
        rad[i] = (uint8_t)r;
        const int y = (int)(i / w), x = (int)(i - (uint32_t)y * w);
        if (x >= r && y >= r && x + r < (int)w && y + r < (int)h) {  // the whole disc (r = 0: weight 1)
            s = fmaf(a, s_wsum[r], s);
            continue;
        }
        const int dx0 = max(-r, -x), dx1 = min(r, (int)w - 1 - x);
        float ws = 0.0f;
        for (int dy = max(-r, -y); dy <= min(r, (int)h - 1 - y); dy++) {
            const float* pre = s_pre + s_pbase[r] + (dy < 0 ? -dy : dy) * (2 * r + 2);
            ws += pre[dx1 + r + 1] - pre[dx0 + r];
        }
        s = fmaf(a, ws, s);
    }
    block_sum_to((double)s, sum_out);
}

// tonemap.glsl:26: the per-bin log-density scale 0.5*brightness*log10(1 + a*k)/a (a > 0)
__device__ __forceinline__ float tonemap_log_scale(float a, float k, float brightness) {
    return 0.5f * brightness * log1pf(a * k) * 0.434294481903251827651128918916f / a;
}

// tonemap.glsl:28-37 on a filtered (r, g, b, a): z = a^(1/gamma), rgb = clamp(mix(rgb^(1/gamma),
// (z/a)*rgb, vibrancy)), alpha 1; no density is opaque black
__device__ __forceinline__ float4 tonemap_finish(float r, float g, float b, float a, float gamma, float vibrancy) {
    if (!(a > 0.0f)) return make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    const float ig = 1.0f / gamma;
    const float gf = powf(a, ig) / a;
    const float rgb[3] = {r, g, b};
    float res[3];
    for (int q = 0; q < 3; q++) {
        const float v = powf(rgb[q], ig) * (1.0f - vibrancy) + gf * rgb[q] * vibrancy;
        res[q] = fminf(fmaxf(v, 0.0f), 1.0f);
    }
    return make_float4(res[0], res[1], res[2], 1.0f);
}

// tonemap.glsl:18-38 for one output pixel from its ss x ss block of bins (rows `stride` apart):
// per bin c *= 0.5*brightness*log10(1 + a*k)/a, mean over the block, then tonemap_finish.
__device__ __forceinline__ float4 tonemap_block(const float4* src, size_t stride, uint32_t ss, float k, float gamma,
                                                float brightness, float vibrancy) {
    float4 acc = make_float4(0, 0, 0, 0);
    for (uint32_t j = 0; j < ss; j++) {
        const float4* row = src + (size_t)j * stride;
        for (uint32_t i = 0; i < ss; i++) {
            const float4 c = row[i];
            if (c.w > 0.0f) {
                const float ls = tonemap_log_scale(c.w, k, brightness);
                acc.x = fmaf(c.x, ls, acc.x);
                acc.y = fmaf(c.y, ls, acc.y);
                acc.z = fmaf(c.z, ls, acc.z);
                acc.w = fmaf(c.w, ls, acc.w);
            }
        }
    }
    const float inv = 1.0f / (float)(ss * ss);
    return tonemap_finish(acc.x * inv, acc.y * inv, acc.z * inv, acc.w * inv, gamma, vibrancy);
}

// the log-density scale: k2 when given, else bins / sum(a) from the FP64 statistics
__device__ __forceinline__ float tonemap_scale(float k2, const double* stats, uint32_t w, uint32_t h) {
    if (k2 > 0.0f) return k2;
    const double sum = stats ? stats[0] : 0.0;
    return sum > 0.0 ? (float)((double)w * (double)h / sum) : 1.0f;
}

__device__ __forceinline__ uchar4 to_rgba8(float4 o) {
    return make_uchar4((unsigned char)lrintf(o.x * 255.0f), (unsigned char)lrintf(o.y * 255.0f),
                       (unsigned char)lrintf(o.z * 255.0f), 255);
}

// the tonemap a DE tile kernel applies to its own output (TM = true)
struct TmArgs {
    uint32_t ss;
    float gamma, brightness, vibrancy, k2;
    const double* stats;  // [0] = sum of the estimator's output density (k2 <= 0)
    float4* out_f32;      // (w / ss) x (h / ss), may be null
    uchar4* out8;         // may be null
};

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

// With TM the tile's output stays in shared memory and the CTA tonemaps its (32/ss) x (8/ss)
// output pixels from it (ss dividing 8): the estimator's output never goes through DRAM.
// Shared memory of a tile CTA: NS staged colours (float4), NS list entries, NS packed source
// records, the weight table of radii up to R, per-warp counts and the rmax slot, per staged row
// its largest radius; with TM the tile's NO outputs.
template <int R>
__host__ __device__ constexpr int de_weight_count() { return (R + 1) * (R + 2) * (2 * R + 3) / 6; }  // sum (r+1)^2

template <int R, bool TM = false>
__host__ __device__ constexpr size_t de_tile_smem() {
    return (((size_t)(kDsX + 2 * R) * (kDsY + 2 * R) * (16 + 4 + 4) + 4 * (size_t)de_weight_count<R>() + 16 * 4 +
             4 * (kDsY + 2 * R) + 15) & ~(size_t)15) +
           (TM ? (size_t)kDsX * kDsY * 16 : 0);
}

// A staged source bin as one word: the disc's squared-distance limit r^2 + r (bits 0-8: a tap at
// squared distance d2 is inside the disc exactly when d2 <= limit, the symmetric restatement of
// 4 d2 <= (2r + 1)^2), the offset of radius r's weights in the table (bits 9-18) and the table's
// row length r + 1 (bits 19-23).  An empty bin is a radius-0 disc of colour zero: it adds zero.
__device__ __forceinline__ uint32_t de_pack(int r) {
    return (uint32_t)(r * r + r) | ((uint32_t)(r * (r + 1) * (2 * r + 1) / 6) << 9) | ((uint32_t)(r + 1) << 19);
}

// one tap: source record p at offset (ax, ay) (squared distance d2) into the accumulator
__device__ __forceinline__ void de_tap(float4& a4, uint32_t p, int ax, int ay, int d2, const float* s_wt,
                                       const float4& v) {
    const bool in = d2 <= (int)(p & 0x1ffu);
    const float wt = in ? s_wt[((p >> 9) & 0x3ffu) + ay * (int)(p >> 19) + ax] : 0.0f;
    a4.x = fmaf(v.x, wt, a4.x);
    a4.y = fmaf(v.y, wt, a4.y);
    a4.z = fmaf(v.z, wt, a4.z);
    a4.w = fmaf(v.w, wt, a4.w);
}

template <int R, bool TM = false>
__global__ void __launch_bounds__(kDsThreads) de_tile_kernel(
    const float4* __restrict__ in, const uint8_t* __restrict__ rad, uint32_t w, uint32_t h,
    const float* __restrict__ weights, const DeTables T, float4* __restrict__ out, const TmArgs tm) {
    constexpr int SW = kDsX + 2 * R, SH = kDsY + 2 * R, NS = SW * SH, NO = kDsX * kDsY, NW = de_weight_count<R>();
    extern __shared__ __align__(16) unsigned char smem[];
    float4* s_c = reinterpret_cast<float4*>(smem);                  // NS colours (zero where empty)
    int* s_list = reinterpret_cast<int*>(s_c + NS);                 // indices of discs of radius >= 2
    uint32_t* s_pk = reinterpret_cast<uint32_t*>(s_list + NS);      // NS packed source records
    float* s_wt = reinterpret_cast<float*>(s_pk + NS);              // weights of radii 0..R
    int* s_stat = reinterpret_cast<int*>(s_wt + NW);                // [0] rmax, [1..8] per-warp counts
    int* s_rowmax = s_stat + 16;                                     // SH: largest radius per staged row
    float4* s_out = reinterpret_cast<float4*>(smem + ((de_tile_smem<R, false>() + 15) & ~(size_t)15));  // TM: NO outputs
    const int tx0 = blockIdx.x * kDsX, ty0 = blockIdx.y * kDsY;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_stat[0] = 0;
    for (int i = threadIdx.x; i < SH; i += kDsThreads) s_rowmax[i] = -1;
    {  // the weight table holds radii up to this launch's largest (<= R); the rest stays zero
        const int rl = T.R > T.min_r ? T.R : T.min_r;
        const int nw = (rl + 1) * (rl + 2) * (2 * rl + 3) / 6;
        for (int i = threadIdx.x; i < NW; i += kDsThreads) s_wt[i] = i < nw ? weights[i] : 0.0f;
    }
    __syncthreads();
    int rmax = 0, nl = 0;
    // stage the tile + halo; list the large discs that reach the tile in source order (a
    // ballot-and-prefix compaction, so the list and the sums are the same on every run)
    for (int i0 = 0; i0 < NS; i0 += kDsThreads) {
        const int i = i0 + (int)threadIdx.x;
        bool big = false;
        if (i < NS) {
            const int gx = tx0 - R + i % SW, gy = ty0 - R + i / SW;
            int r = 255;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (gx >= 0 && gy >= 0 && gx < (int)w && gy < (int)h) {
                const size_t gi = (size_t)gy * w + gx;
                r = rad[gi];
                if (r != 255) v = in[gi];
            }
            s_pk[i] = de_pack(r == 255 ? 0 : r);
            s_c[i] = v;
            if (r != 255) atomicMax(&s_rowmax[i / SW], r);
            if (r != 255 && gx - r <= tx0 + kDsX - 1 && gx + r >= tx0 && gy - r <= ty0 + kDsY - 1 && gy + r >= ty0) {
                rmax = max(rmax, r);
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
            // discs of radius 0 and 1 from the 3 x 3 neighbourhood, then the listed larger discs
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int si = (oy + R + dy) * SW + ox + R + dx;
                    const uint32_t p = s_pk[si];
                    if ((p & 0x1ffu) > 2u) continue;  // radius >= 2: in the list
                    de_tap(a4, p, dx * dx, dy * dy, dx * dx + dy * dy, s_wt, s_c[si]);
                }
            for (int k = 0; k < nl; k++) {
                const int si = s_list[k];
                const int ax = abs(ox + R - si % SW), ay = abs(oy + R - si / SW);
                if (ax > R || ay > R) continue;
                de_tap(a4, s_pk[si], ax, ay, ax * ax + ay * ay, s_wt, s_c[si]);
            }
        } else {
            for (int dy = -rm; dy <= rm; dy++) {
                const int ay = dy < 0 ? -dy : dy;
                const int rr = min(rm, s_rowmax[oy + R + dy]);  // no disc of this row reaches |dy| rows
                if (rr < ay) continue;
                const int row = (oy + R + dy) * SW + ox + R;
                for (int dx = -rr; dx <= rr; dx++) {
                    const int ax = dx < 0 ? -dx : dx;
                    de_tap(a4, s_pk[row + dx], ax, ay, ax * ax + ay * ay, s_wt, s_c[row + dx]);
                }
            }
        }
        const int gx = tx0 + ox, gy = ty0 + oy;
        if (out && gx < (int)w && gy < (int)h) out[(size_t)gy * w + gx] = a4;
        if (TM) s_out[o] = a4;
    }
    if (TM) {
        __syncthreads();
        const uint32_t ss = tm.ss, pw = kDsX / ss, ph = kDsY / ss, ow = w / ss, oh = h / ss;
        const float k = tonemap_scale(tm.k2, tm.stats, w, h);
        for (uint32_t p = threadIdx.x; p < pw * ph; p += kDsThreads) {
            const uint32_t px = p % pw, py = p / pw;
            const uint32_t gx = tx0 / ss + px, gy = ty0 / ss + py;
            if (gx >= ow || gy >= oh) continue;
            const float4 o = tonemap_block(s_out + (size_t)py * ss * kDsX + px * ss, kDsX, ss, k, tm.gamma,
                                           tm.brightness, tm.vibrancy);
            const size_t oi = (size_t)gy * ow + gx;
            if (tm.out_f32) tm.out_f32[oi] = o;
            if (tm.out8) tm.out8[oi] = to_rgba8(o);
        }
    }
}

template <int R>
static cudaError_t set_de_tile_smem() {
    cudaError_t e = cudaFuncSetAttribute(de_tile_kernel<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)de_tile_smem<R, false>());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(de_tile_kernel<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)de_tile_smem<R, true>());
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
                                  const DeTables& T, float4* out, cudaStream_t st, const TmArgs* tm = nullptr) {
    cudaError_t e = density_prepare();
    if (e != cudaSuccess) return e;
    const dim3 grid((w + kDsX - 1) / kDsX, (h + kDsY - 1) / kDsY);
    if (tm)
        de_tile_kernel<R, true><<<grid, kDsThreads, de_tile_smem<R, true>(), st>>>(in, rad, w, h, dw, T, out, *tm);
    else
        de_tile_kernel<R, false><<<grid, kDsThreads, de_tile_smem<R, false>(), st>>>(in, rad, w, h, dw, T, out, TmArgs{});
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

// tonemap.glsl:18-38 with an ss x ss box filter (tonemap_block), one output pixel per thread
__global__ void tonemap_kernel(const float4* __restrict__ in, uint32_t w, uint32_t h, uint32_t ss, float gamma,
                               float brightness, float vibrancy, float k2, const double* __restrict__ stats,
                               float4* __restrict__ out_f32, uchar4* __restrict__ out8) {
    const uint32_t ow = w / ss, oh = h / ss;
    const uint32_t ox = blockIdx.x * blockDim.x + threadIdx.x, oy = blockIdx.y;
    if (ox >= ow || oy >= oh) return;
    const float k = tonemap_scale(k2, stats, w, h);
    const float4 o = tonemap_block(in + (size_t)oy * ss * w + (size_t)ox * ss, w, ss, k, gamma, brightness, vibrancy);
    const size_t oi = (size_t)oy * ow + ox;
    if (out_f32) out_f32[oi] = o;
    if (out8) out8[oi] = to_rgba8(o);
}

// The tonemap with flam3's spatial filter in place of the ss x ss box (no counterpart in the
// reference, which ignores flam3's filter and filter_shape, flame.cpp:166-176): output pixel
// (ox, oy) is the weighted sum, by the separable taps c[i] c[j], of the log-scaled bins of the
// fwidth x fwidth window starting at (ox ss - pad, oy ss - pad), pad = (fwidth - ss) / 2, then
// tonemap_finish.  A CTA stages the log-scaled bins of its tile's windows once in shared memory.
struct FilterArgs {
    int fwidth, pad;
    int tw, th;        // output pixels per CTA tile
    float taps[kMaxFilterTaps];
};

__global__ void __launch_bounds__(256) tonemap_filter_kernel(const float4* __restrict__ in, uint32_t w, uint32_t h,
                                                             uint32_t ss, float gamma, float brightness,
                                                             float vibrancy, float k2, const double* __restrict__ stats,
                                                             const FilterArgs F, float4* __restrict__ out_f32,
                                                             uchar4* __restrict__ out8) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* s_l = reinterpret_cast<float4*>(smem);
    const int rw = F.tw * (int)ss + F.fwidth - (int)ss, rh = F.th * (int)ss + F.fwidth - (int)ss;
    const int ox0 = blockIdx.x * F.tw, oy0 = blockIdx.y * F.th;
    const int gx0 = ox0 * (int)ss - F.pad, gy0 = oy0 * (int)ss - F.pad;
    const float k = tonemap_scale(k2, stats, w, h);
    for (int i = threadIdx.x; i < rw * rh; i += blockDim.x) {
        const int gx = gx0 + i % rw, gy = gy0 + i / rw;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (gx >= 0 && gy >= 0 && gx < (int)w && gy < (int)h) {
            const float4 c = in[(size_t)gy * w + gx];
            if (c.w > 0.0f) {
                const float ls = tonemap_log_scale(c.w, k, brightness);
                v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
            }
        }
        s_l[i] = v;
    }
    __syncthreads();
    const uint32_t ow = w / ss, oh = h / ss;
    for (int p = threadIdx.x; p < F.tw * F.th; p += blockDim.x) {
        const int px = p % F.tw, py = p / F.tw;
        const uint32_t ox = ox0 + px, oy = oy0 + py;
        if (ox >= ow || oy >= oh) continue;
        float4 acc = make_float4(0, 0, 0, 0);
        for (int j = 0; j < F.fwidth; j++) {
            const float4* row = s_l + (size_t)(py * (int)ss + j) * rw + px * (int)ss;
            float4 r = make_float4(0, 0, 0, 0);
            for (int i = 0; i < F.fwidth; i++) {
                const float4 v = row[i];
                const float c = F.taps[i];
                r.x = fmaf(v.x, c, r.x);
                r.y = fmaf(v.y, c, r.y);
                r.z = fmaf(v.z, c, r.z);
                r.w = fmaf(v.w, c, r.w);
            }
            const float c = F.taps[j];
            acc.x = fmaf(r.x, c, acc.x);
            acc.y = fmaf(r.y, c, acc.y);
            acc.z = fmaf(r.z, c, acc.z);
            acc.w = fmaf(r.w, c, acc.w);
        }
        const float4 o = tonemap_finish(acc.x, acc.y, acc.z, acc.w, gamma, vibrancy);
        const size_t oi = (size_t)oy * ow + ox;
        if (out_f32) out_f32[oi] = o;
        if (out8) out8[oi] = to_rgba8(o);
    }
}

// flam3's filter functions and their supports: Gaussian exp(-2x^2) sqrt(2/pi) on [-1.5, 1.5],
// box on [-0.5, 0.5], triangle 1 - |x| and the cubic Hermite 2|x|^3 - 3x^2 + 1 on [-1, 1]
static double filter_support(int shape) { return shape == RF_FILTER_BOX ? 0.5 : (shape == RF_FILTER_GAUSSIAN ? 1.5 : 1.0); }
static double filter_value(int shape, double x) {
    const double t = std::fabs(x);
    switch (shape) {
        case RF_FILTER_GAUSSIAN: return std::exp(-2.0 * x * x) * std::sqrt(2.0 / 3.14159265358979323846);
        case RF_FILTER_BOX: return t <= 0.5 ? 1.0 : 0.0;
        case RF_FILTER_TRIANGLE: return t < 1.0 ? 1.0 - t : 0.0;
        case RF_FILTER_HERMITE: return t < 1.0 ? (2.0 * t - 3.0) * t * t + 1.0 : 0.0;
        default: return 0.0;
    }
}

// The taps: the window spans fw = 2 * support * ss * radius bins, rounded up to an integer width
// of the parity of ss (so it centres on the output pixel's ss x ss block), sampled at each
// cell's centre with the coordinate stretched so the window covers the support, normalised in
// FP64.  Returns fwidth, or -1 beyond kMaxFilterTaps.
int filter_taps(uint32_t ss, float radius, int shape, float* taps) {
    const double support = filter_support(shape);
    const double fw = 2.0 * support * (double)ss * (double)radius;
    int fwidth = (int)fw + 1;
    if ((fwidth ^ (int)ss) & 1) fwidth++;
    if (fwidth > kMaxFilterTaps) return -1;
    const double adjust = fw > 0.0 ? support * (double)fwidth / fw : 1.0;
    double t[kMaxFilterTaps], sum = 0.0;
    for (int i = 0; i < fwidth; i++) {
        t[i] = filter_value(shape, ((2.0 * i + 1.0) / (double)fwidth - 1.0) * adjust);
        sum += t[i];
    }
    for (int i = 0; i < fwidth; i++) taps[i] = (float)(t[i] / sum);
    return fwidth;
}

cudaError_t launch_tonemap_filter(const float4* in, uint32_t w, uint32_t h, uint32_t ss, float radius, int shape,
                                  float gamma, float brightness, float vibrancy, float k2, const double* stats,
                                  float4* out_f32, uchar4* out8, cudaStream_t st) {
    FilterArgs F{};
    F.fwidth = filter_taps(ss, radius, shape, F.taps);
    if (F.fwidth < 0) return cudaErrorInvalidValue;
    F.pad = (F.fwidth - (int)ss) / 2;
    // the largest tile whose staged windows fit in 96 KB of shared memory
    static const int tiles[][2] = {{32, 8}, {16, 8}, {8, 8}, {8, 4}, {4, 4}, {2, 2}, {1, 1}};
    size_t smem = 0;
    for (const auto& t : tiles) {
        F.tw = t[0];
        F.th = t[1];
        smem = (size_t)(F.tw * ss + F.fwidth - ss) * (F.th * ss + F.fwidth - ss) * sizeof(float4);
        if (smem <= 96 * 1024) break;
    }
    if (smem > 96 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(tonemap_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    if (e != cudaSuccess) return e;
    const uint32_t ow = w / ss, oh = h / ss;
    const dim3 grid((ow + F.tw - 1) / F.tw, (oh + F.th - 1) / F.th);
    tonemap_filter_kernel<<<grid, 256, smem, st>>>(in, w, h, ss, gamma, brightness, vibrancy, k2, stats, F, out_f32,
                                                   out8);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
static void de_tables(int R, int min_r, float curve, DeTables& T, std::vector<float>& wts) {
    T = DeTables{};
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
        // the whole disc: the table's weights of every (dx, dy) with 4 (dx^2 + dy^2) <= (2r + 1)^2
        double s = 0.0;
        for (int dy = -r; dy <= r; dy++)
            for (int dx = -r; dx <= r; dx++) {
                const int ax = dx < 0 ? -dx : dx, ay = dy < 0 ? -dy : dy;
                if (r == 0) s += 1.0;
                else if (4 * (ax * ax + ay * ay) <= (2 * r + 1) * (2 * r + 1))
                    s += (double)wts[T.wbase[r] + ay * (r + 1) + ax];
            }
        T.wsum[r] = s;
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

// the tile kernel for the largest radius (rmax <= kDeMaxSmemR)
static cudaError_t launch_tile_for(int rmax, const float4* in, const uint8_t* rad, uint32_t w, uint32_t h,
                                   const float* dw, const DeTables& T, float4* out, cudaStream_t st,
                                   const TmArgs* tm) {
    if (rmax <= 3) return launch_de_tile<3>(in, rad, w, h, dw, T, out, st, tm);
    if (rmax <= 6) return launch_de_tile<6>(in, rad, w, h, dw, T, out, st, tm);
    if (rmax <= 9) return launch_de_tile<9>(in, rad, w, h, dw, T, out, st, tm);
    return launch_de_tile<kDeMaxSmemR>(in, rad, w, h, dw, T, out, st, tm);
}

static cudaError_t launch_density_passes(const float4* in, uint32_t w, uint32_t h, const DeTables& T, float4* out,
                                         uint8_t* rad, const float* dw, cudaStream_t st) {
    const size_t n = (size_t)w * h;
    de_radius_kernel<<<1024, 256, 0, st>>>(in, n, T, rad);
    const int rmax = T.R > T.min_r ? T.R : T.min_r;
    if (rmax <= kDeMaxSmemR) return launch_tile_for(rmax, in, rad, w, h, dw, T, out, st, nullptr);
    de_gather_global_kernel<<<dim3((w + 127) / 128, h), 128, 0, st>>>(in, rad, w, h, dw, T, out);
    return cudaGetLastError();
}

bool density_tonemap_fused(int R, int min_r, uint32_t ss) {
    const int rmax = R > min_r ? R : min_r;
    return rmax <= kDeMaxSmemR && ss >= 1 && kDsX % ss == 0 && kDsY % ss == 0;
}

// The image tail of a frame (main.cpp:490-535: the density-estimation raster pass, then the
// tonemap pass) in two passes: pass 1 finds every bin's radius and, for an automatic k2, the FP64
// density sum of the estimator's output (de_radius_sum_kernel); pass 2 estimates each 32 x 8 tile
// in shared memory and tonemaps it there, so the estimator's FP32 output never reaches DRAM.
// Where that does not apply (density_tonemap_fused false: ss does not divide the tile, or radii
// beyond the shared-memory path) the estimator writes `de_scratch`, then the statistics and
// tonemap passes run on it.  rad: a byte per bin; dw: the weight table (density_weights);
// stats: 3 doubles.
cudaError_t launch_density_tonemap(const float4* in, uint32_t w, uint32_t h, int R, int min_r, float curve,
                                   uint32_t ss, float gamma, float brightness, float vibrancy, float k2,
                                   float4* out_f32, uchar4* out8, uint8_t* rad, const float* dw, double* stats,
                                   float4* de_scratch, cudaStream_t st) {
    DeTables T;
    std::vector<float> wts;
    de_tables(R, min_r, curve, T, wts);
    const bool need_sum = !(k2 > 0.0f);
    cudaError_t e;
    if (!density_tonemap_fused(R, min_r, ss)) {
        if (!de_scratch) return cudaErrorInvalidValue;
        e = launch_density_passes(in, w, h, T, de_scratch, rad, dw, st);
        if (e == cudaSuccess && need_sum) e = launch_stats(de_scratch, w, h, stats, st);
        if (e == cudaSuccess)
            e = launch_tonemap(de_scratch, w, h, ss, gamma, brightness, vibrancy, k2, need_sum ? stats : nullptr,
                               out_f32, out8, st);
        return e;
    }
    if (need_sum) {
        e = cudaMemsetAsync(stats, 0, 3 * sizeof(double), st);
        if (e != cudaSuccess) return e;
        de_radius_sum_kernel<<<1024, 256, 0, st>>>(in, w, h, T, dw, rad, stats);
    } else {
        de_radius_kernel<<<1024, 256, 0, st>>>(in, (size_t)w * h, T, rad);
    }
    const TmArgs tm{ss, gamma, brightness, vibrancy, k2, need_sum ? stats : nullptr, out_f32, out8};
    return launch_tile_for(R > min_r ? R : min_r, in, rad, w, h, dw, T, nullptr, st, &tm);
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
