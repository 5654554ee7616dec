// Launch interface of the device kernels (kernels.cu, image.cu), shared with the host runtime.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <vector>

#include "chaos_args.h"
#include "refrakt.h"

namespace rfk {



size_t chaos_smem(int slots, uint32_t prog_words, uint32_t steps, uint32_t tile_bins = 0, int pipe = 0);
constexpr size_t kMaxCtaSmem = 232448;  // dynamic shared memory a CTA may opt into (227 KB)
bool chaos_shape_supported(int threads, int slots);
cudaError_t launch_chaos(int threads, int slots, const ChaosArgs& a, uint32_t grid, cudaStream_t st);
cudaError_t launch_merge_records(float4* rec, size_t n, float4* bins, uint32_t* hits, cudaStream_t st);
cudaError_t launch_init_rng(uint4* rng, uint64_t n, uint64_t seed, cudaStream_t st);
cudaError_t launch_shuffle_table(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed, cudaStream_t st,
                                 uint32_t phases = 0);
cudaError_t launch_animate(const uint32_t* base, uint32_t words, uint32_t T, float tss, uint32_t* out,
                           uint32_t stride, cudaStream_t st);
cudaError_t launch_probe(const uint32_t* prog, int xform, uint32_t n, const float* in, uint32_t* rng,
                         int first_run, float* out, cudaStream_t st);

// image passes (image.cu)
cudaError_t launch_density(const float4* in, uint32_t w, uint32_t h, int radius, int min_radius, float curve,
                           float4* out, cudaStream_t st);
size_t density_weight_count(int radius, int min_radius);
// Kernel weights of density estimation depend on the radii alone: `density_weights` builds them on
// the host, and `launch_density_resident` runs both passes with those weights already on the
// device (`dw`) and a byte of radius scratch per bin (`rad`) — no allocation and no host copy,
// so the passes can be captured in a CUDA graph and replayed.
void density_weights(int radius, int min_radius, std::vector<float>& out);
cudaError_t density_prepare();  // per-device kernel attributes; call before capturing DE in a graph
cudaError_t launch_density_resident(const float4* in, uint32_t w, uint32_t h, int radius, int min_radius,
                                    float curve, float4* out, uint8_t* radius_scratch, const float* weights,
                                    cudaStream_t st);
// (sum h, sum h^2) of a hit-count histogram in FP64 (the splat autotuner's concentration measure)
cudaError_t launch_hit_moments(const uint32_t* hits, uint32_t w, uint32_t h, double* out2, cudaStream_t st);
cudaError_t launch_stats(const float4* in, uint32_t w, uint32_t h, double* out3, cudaStream_t st);
cudaError_t launch_tonemap(const float4* in, uint32_t w, uint32_t h, uint32_t ss, float gamma, float brightness,
                           float vibrancy, float k2, const double* stats, float4* out_f32, uchar4* out8,
                           cudaStream_t st);
// The tonemap with flam3's spatial filter (rf_filter_shape) in place of the ss x ss box; taps
// (filter_taps, at most kMaxFilterTaps: 2 * support * ss * radius < 63) normalised on the host.
constexpr int kMaxFilterTaps = 64;
int filter_taps(uint32_t ss, float radius, int shape, float* taps);
cudaError_t launch_tonemap_filter(const float4* in, uint32_t w, uint32_t h, uint32_t ss, float radius, int shape,
                                  float gamma, float brightness, float vibrancy, float k2, const double* stats,
                                  float4* out_f32, uchar4* out8, cudaStream_t st);
// Density estimation and tonemap in one sequence (image.cu): with density_tonemap_fused the
// estimator's output stays on chip and `de_scratch` is not touched (may be null); otherwise it is
// the estimator's output.  rad: a byte per bin; dw: density_weights(R, min_r); stats: 3 doubles.
bool density_tonemap_fused(int radius, int min_radius, uint32_t ss);
cudaError_t launch_density_tonemap(const float4* in, uint32_t w, uint32_t h, int radius, int min_radius, float curve,
                                   uint32_t ss, float gamma, float brightness, float vibrancy, float k2,
                                   float4* out_f32, uchar4* out8, uint8_t* rad, const float* dw, double* stats,
                                   float4* de_scratch, cudaStream_t st);

}  // namespace rfk
