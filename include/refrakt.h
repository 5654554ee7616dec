/*
 * refrakt_gb300 — C ABI of the GB300 fractal-flame renderer.
 *
 * Drop-in for the chaos-game path of untrioctium/refrakt, whose interface is two C++
 * classes: `flame_compiler` (src/variation_table.hpp:20-59) and `flame`
 * (src/flame.hpp:41-173).  Each entry point below names the reference member it replaces.
 *
 * Conventions
 *  - Every function returns an `int` status (RF_OK = 0) unless stated otherwise; on failure
 *    rf_last_error() returns a message for the calling thread.
 *  - Handles are opaque.  Device pointers are plain CUDA device addresses; `stream` arguments
 *    are `cudaStream_t` values passed as `void*` (NULL = the legacy default stream).
 *  - Histogram ("bins") layout, row-major, row 0 = top row (the reference writes row
 *    (H - y - 1), shaders/flame.glsl:84):
 *      bins_rgba : float[4 * W * H]  — (sum palette.r, sum palette.g, sum palette.b, sum opacity)
 *                  per bin, the reference's vec4 bins (flame.glsl:84);
 *      bins_hits : uint32[W * H]     — exact count of points drawn into the bin.
 *  - There is no process-wide mutable state: every simulation lives in its own rf_sim.
 */
#ifndef REFRAKT_GB300_H
#define REFRAKT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RF_ABI_VERSION 1

#if defined(__GNUC__)
#define RF_API __attribute__((visibility("default")))
#else
#define RF_API
#endif

enum rf_status {
    RF_OK = 0,
    RF_ERR_INVALID_ARG = 1,   /* null handle, bad size, inconsistent arguments */
    RF_ERR_PARSE = 2,         /* malformed flam3 XML or variation YAML */
    RF_ERR_UNKNOWN_NAME = 3,  /* unknown attribute in a genome (flame.cpp:196) */
    RF_ERR_UNSUPPORTED = 4,   /* variation that does not compile in the reference, or unknown to the kernels */
    RF_ERR_CAPACITY = 5,      /* parameter buffer over 1024 floats, too many xforms, too large a histogram */
    RF_ERR_CUDA = 6,          /* a CUDA runtime call failed */
    RF_ERR_NEEDS_WARMUP = 7,  /* rf_draw_to_bins before rf_warmup for this flame (flame.hpp:86) */
    RF_ERR_IO = 8,            /* file could not be read or written */
    RF_ERR_NO_DEVICE = 9,     /* no CUDA device of the supported architecture */
    RF_ERR_TIMEOUT = 10       /* a bounded device-side wait gave up (a chaos launch's walker exchange);
                                 the results of that launch are invalid */
};

typedef struct rf_compiler rf_compiler;
typedef struct rf_flame rf_flame;
typedef struct rf_sim rf_sim;

/* Message describing the last failure on this thread (never NULL). */
RF_API const char* rf_last_error(void);
RF_API int rf_abi_version(void);

/* ------------------------------------------------------------------------------------------
 * Variation table — replaces flame_compiler (src/variation_table.hpp:20-59).
 * ---------------------------------------------------------------------------------------- */

/* flame_compiler::flame_compiler() (variation_table.cpp:182-215).  `yaml_path` = NULL uses the
   built-in table of the reference's variations.yaml; a path loads that file and checks each
   entry against the kernels' implementations. */
RF_API int  rf_compiler_create(const char* yaml_path, rf_compiler** out);
RF_API void rf_compiler_destroy(rf_compiler* c);
/* is_variation / is_param / is_common (variation_table.hpp:39-41): 1 = yes, 0 = no. */
RF_API int  rf_compiler_is_variation(const rf_compiler* c, const char* name);
RF_API int  rf_compiler_is_param(const rf_compiler* c, const char* name);
RF_API int  rf_compiler_is_common(const rf_compiler* c, const char* name);
/* 1 when the GPU kernels evaluate this variation (0 for the reference's non-compiling ones). */
RF_API int  rf_compiler_is_supported(const rf_compiler* c, const char* name);
/* param_owner (variation_table.hpp:43): writes the owning variation's name. */
RF_API int  rf_compiler_param_owner(const rf_compiler* c, const char* param, char* buf, size_t cap);
/* variations() (variation_table.hpp:47): count and i-th name (map order). */
RF_API int  rf_compiler_num_variations(const rf_compiler* c);
RF_API int  rf_compiler_variation_name(const rf_compiler* c, int i, char* buf, size_t cap);
/* get_parameters_for_variation (variation_table.hpp:44): comma-separated list. */
RF_API int  rf_compiler_variation_params(const rf_compiler* c, const char* name, char* buf, size_t cap);

/* ------------------------------------------------------------------------------------------
 * Genomes — replaces flame::load_flame and the public genome fields (flame.hpp:41-61, 84).
 * ---------------------------------------------------------------------------------------- */

/* flame::load_flame(path, compiler) (flame.cpp:160-226); NULL result there = error status here. */
RF_API int  rf_flame_load(const char* flam3_path, const rf_compiler* c, rf_flame** out);
RF_API int  rf_flame_load_xml(const char* flam3_xml, const rf_compiler* c, rf_flame** out);
RF_API void rf_flame_free(rf_flame* f);
/* Serialise (flam3 XML, reference attribute set).  *needed receives the byte count incl. NUL. */
RF_API int  rf_flame_to_xml(const rf_flame* f, char* buf, size_t cap, size_t* needed);

/* Seeded synthetic genomes for the benchmark workloads (no reference counterpart). */
enum rf_synth_kind {
    RF_SYNTH_SMALL = 0,      /* 3 xforms, linear/sinusoidal/spherical, affine U[-1,1] */
    RF_SYNTH_RANDOM = 1,     /* n xforms, 3 variations each from the supported set, affine U[-1.2,1.2] */
    RF_SYNTH_CONTRACT = 2,   /* 6 xforms, linear parts x0.05, translations U[-0.02,0.02] */
    RF_SYNTH_SPACEFILL = 3   /* 16 xforms, spherical + swirl */
};
typedef struct {
    int32_t  kind;              /* rf_synth_kind */
    uint32_t n_xforms;          /* RF_SYNTH_RANDOM only; 0 = 8 */
    uint64_t seed;
    int32_t  final_xform;       /* RF_SYNTH_RANDOM: 1 adds a final xform */
    int32_t  force_parametric;  /* RF_SYNTH_RANDOM: xforms 0..2 carry julian, ngon, pdj */
    uint32_t width, height;     /* bin grid the camera is framed for */
} rf_synth_desc;
RF_API int  rf_flame_synthesize(const rf_synth_desc* d, const rf_compiler* c, rf_flame** out);

/* A genome from plain C structures (no XML), for FFI callers that build genomes in code: the
   fields of flame.hpp:21-61 with variations and parameters by name.  The result is validated
   like a loaded genome (flame.cpp:160-226): unknown names, missing parameters and variations
   the reference cannot compile are errors. */
typedef struct {
    float weight, color, color_speed, opacity;
    float coefs[6];             /* flam3 coefs order: c00 c01 c10 c11 c20 c21 */
    int32_t has_post;
    float post[6];
    uint32_t n_vars;            /* variations: names and weights */
    const char* const* var_names;
    const float* var_weights;
    uint32_t n_params;          /* parameters of those variations: names and values */
    const char* const* param_names;
    const float* param_values;
} rf_xform_desc;
typedef struct {
    uint32_t size[2];
    float center[2];
    float scale, rotate;
    int32_t estimator_radius, estimator_min;
    float estimator_curve;
    float gamma, vibrancy, brightness;
    const float* palette_rgb;   /* 256 x 3 floats in [0, 1] */
    uint32_t n_xforms;
    const rf_xform_desc* xforms;
    const rf_xform_desc* final_xform;  /* may be NULL */
} rf_genome_desc;
RF_API int  rf_flame_from_struct(const rf_genome_desc* d, const rf_compiler* c, rf_flame** out);

/* Genome at t in [0, 1] between a and b (animation frames; the reference only rotates affines
   over time, main.cpp:383-395).  The shorter genome's missing xforms are padded with zero
   selection weight; affines, post, weights, colours, variation weights (0 where absent) and shared
   parameters are lerped. */
RF_API int  rf_flame_interpolate(const rf_flame* a, const rf_flame* b, float t, rf_flame** out);

typedef struct {
    uint32_t size[2];           /* flame.hpp:47 */
    float    center[2];
    float    scale, rotate;
    int32_t  estimator_radius, estimator_min;
    float    estimator_curve;
    float    gamma, vibrancy, brightness;
    uint32_t num_xforms;
    int32_t  has_final;
    uint32_t total_params;      /* flat parameter buffer size (flame.cpp:68) */
    float    filter;            /* flam3 spatial filter radius in output pixels (0: the ss x ss box) */
    int32_t  filter_shape;      /* rf_filter_shape of flam3's filter_shape attribute */
} rf_flame_info;
RF_API int  rf_flame_get_info(const rf_flame* f, rf_flame_info* out);
/* The mutable view fields the reference UI edits in place (main.cpp:324-381). */
RF_API int  rf_flame_set_view(rf_flame* f, const float center[2], float scale, float rotate);
RF_API int  rf_flame_set_tonemap(rf_flame* f, float gamma, float brightness, float vibrancy);
RF_API int  rf_flame_set_estimator(rf_flame* f, int radius, int min_radius, float curve);
/* Edit one xform attribute by its flam3 name (weight, color, coefs index via "coefs0".."coefs5",
   a variation or parameter name).  xform = -1 addresses the final xform. */
RF_API int  rf_flame_set_xform_value(rf_flame* f, int xform, const char* name, float value);
/* copy_flame_data_to_buffer (flame.cpp:74-103): writes the flat FP32 parameter buffer. */
RF_API int  rf_flame_param_buffer(const rf_flame* f, float* out, size_t cap, size_t* count);
/* buffer_map_ as JSON (flame.cpp:33-71, printed by print_debug_info, flame.hpp:130). */
RF_API int  rf_flame_param_layout(const rf_flame* f, char* buf, size_t cap, size_t* needed);
/* The 2x3 screen affine draw_to_bins builds (flame.cpp:289-296) for a W x H bin grid. */
RF_API int  rf_flame_screen_affine(const rf_flame* f, uint32_t width, uint32_t height, float out6[6]);
/* RNG draws one evaluation of xform i consumes (i = -1: final xform), first_run colour excluded. */
RF_API int  rf_flame_xform_draws(const rf_flame* f, int xform);

/* ------------------------------------------------------------------------------------------
 * Simulation — replaces flame::set_sim_parameters / warmup / draw_to_bins (flame.cpp:105-330).
 * ---------------------------------------------------------------------------------------- */

typedef struct {
    uint64_t walkers;           /* total walker slots N (multiple of cta_slots * temporal_samples) */
    uint32_t temporal_samples;  /* T (flame.cpp:109) */
    uint32_t shuffle_count;     /* permutations in the walker-shuffle table (flame.cpp:110) */
    uint64_t seed;              /* slot i's JSF32 state = warmup_ctx(i + seed * N) */
    uint32_t cta_slots;         /* walker slots per CTA — the walker shuffle's mixing domain:
                                   256, 512, 1024, 2048 or 4096 (0 = 4096) */
    uint32_t cta_threads;       /* threads per CTA: 256, 512 or 1024, dividing cta_slots
                                   (0 = min(cta_slots, 1024)) */
    uint32_t steps_per_launch;  /* passes per persistent launch L, at most 256 (0 = 256; 1 = the
                                   reference's per-pass global gather).  Walkers mix within their
                                   CTA's slots every pass and across CTAs every L passes; L does
                                   not change the histogram's noise (the domains are independent
                                   chaos games), and longer launches spend less on the launch
                                   boundary (the 1080p frame: 47.8 Gpoints/s at 32, 50.8 at 256) */
    int32_t  device;            /* CUDA device ordinal */
    int32_t  specialize;        /* genome-specialised kernels compiled at run time (NVRTC) for each
                                   genome structure rf_warmup meets: 0 = when the run-time compiler
                                   loads (else the interpreted kernel), 1 = required, -1 = never */
} rf_sim_desc;

/* flame::set_sim_parameters(total_particles, temporal_samples, shuffle_count). */
RF_API int  rf_sim_create(const rf_sim_desc* d, rf_sim** out);
RF_API int  rf_sim_destroy(rf_sim* s);
RF_API int  rf_sim_set_stream(rf_sim* s, void* stream);
/* Records the xform index every 256-walker group used per pass (debug / parity). */
RF_API int  rf_sim_enable_xid_trace(rf_sim* s, uint32_t max_passes);
RF_API int  rf_sim_read_xid_trace(rf_sim* s, uint8_t* out, size_t cap, uint32_t* passes);
/* flame::needs_warmup() (flame.hpp:86): 1 when f is not the warmed flame or was edited since. */
RF_API int  rf_needs_warmup(const rf_sim* s, const rf_flame* f);
/* flame::warmup(num_passes, tss_width) (flame.cpp:228-281): one first-run pass (start points,
   jitter, random colours) followed by num_passes passes, nothing drawn. */
RF_API int  rf_warmup(rf_sim* s, rf_flame* f, uint32_t num_passes, float tss_width);

/* Splat strategy for rf_draw_to_bins: one L2 reduction per point (GLOBAL), warp-aggregated
   reductions of the points that share a bin (WARP), or per warp and pass the aggregated form
   when a cheap test finds two lanes sharing a bin (AUTO, the default).  AUTO also serves compact
   attractors with the shared-memory tile splat (RF_SPLAT_TILE below): after the second drawing
   launch of >= 32 passes on a bin grid of at most 2^24 bins, when the caller passes a count plane
   (direct layout, not during stream capture), the call synchronises once, reads the counts back
   and fits the tile that fits beside the walkers and holds the most hits (the hit bins'
   bounding box, else the best square-ish window); if it holds >= 25 % of the hits, the next
   drawing launch of the same length runs through it, timed against the first, and the faster
   splat is kept (decided without a host wait once that launch has finished; rf_sim_splat_tile
   reports it).  Counts never change with the strategy; colour sums only in
   FP32 summation order.  The genome-specialised kernel is compiled with the strategy set at
   rf_warmup; setting another one later makes the next draw call fetch (or, the first time,
   compile) the kernel for it. */
enum rf_splat { RF_SPLAT_AUTO = 0, RF_SPLAT_GLOBAL = 1, RF_SPLAT_WARP = 2, RF_SPLAT_TILE = 3 };
/* flame::draw_to_bins(bins, bins_width, num_iter) (flame.cpp:283-330): num_iter passes over
   every walker, drawing into caller-owned device bins.  bins_hits may be NULL.  When `drawn`
   is non-NULL the call synchronises and stores the number of points binned (the reference's
   return value); when NULL it returns without synchronising. */
/* Bin layout of the drawing passes: the caller's planes directly (DIRECT), or interleaved 32-byte
   records {RGBA, count} in a library buffer merged into the caller's planes at the end of each
   draw call (INTERLEAVED: one DRAM sector per point instead of two; pays for itself when the bins
   exceed L2).  AUTO: INTERLEAVED when a count plane is given and the planes exceed 256 MB. */
enum rf_bin_layout { RF_BINS_AUTO = 0, RF_BINS_DIRECT = 1, RF_BINS_INTERLEAVED = 2 };
RF_API int  rf_set_bin_layout(rf_sim* s, int layout);
RF_API int  rf_draw_to_bins(rf_sim* s, rf_flame* f, float* bins_rgba, uint32_t* bins_hits,
                     uint32_t width, uint32_t height, uint32_t num_iter, uint64_t* drawn);
RF_API int  rf_set_splat(rf_sim* s, int splat);
/* RF_SPLAT_TILE: a per-CTA histogram tile in shared memory for compact attractors.  The bins of
   columns [x0, x0 + w) and rows [y0, y0 + h) (row 0 at the top, as the bins) accumulate in each
   CTA's shared memory over a launch (aggregated within the warp where lanes share a bin) and are
   added to the caller's bins once at the launch's end; points outside go to the L2, aggregated
   the same way.  The tile must lie inside a bin grid of fewer than 2^31 bins and fit beside the
   CTA's walkers (w * h * 20 bytes: about 1,500 bins beside 4096 slots of a small genome, 6,500
   beside 2048); the batched launch does not use it (RF_SPLAT_GLOBAL there). */
RF_API int  rf_set_splat_tile(rf_sim* s, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h);
/* The walker reset that shaders/flame.glsl:68 keeps commented out: after an xform, a walker whose
   x or y is NaN or beyond +-1e10 (math.glsl:22 `badval`) restarts at (2u1 - 1, 2u2 - 1) from two
   randf() draws of its slot, with opacity 0 (that step is not drawn).  0 (default) = the
   reference's behaviour: such a walker stays lost and is never drawn again, so over thousands of
   passes a genome with singular variations (spherical, julian ...) binns fewer and fewer points.
   Takes effect from the next rf_warmup / rf_draw_to_bins launch. */
RF_API int  rf_set_bad_value_reset(rf_sim* s, int on);
/* The walker exchange of the genome-specialised chaos kernel.  A Sim with four slots per thread
   builds its shuffle table so that a pass's first phase takes no walker of the previous pass's
   last phase and its last phase none of the first (the histogram noise is that of uniform
   permutations).  RF_EXCHANGE_BARRIER: one CTA barrier per pass.  RF_EXCHANGE_PIPELINED: two
   CTA-wide mbarriers instead — a warp starts the next pass as soon as every warp has finished
   three phases of this one, so the slowest warps' last phase overlaps the next pass (faster on
   genomes of unequal, costly xforms; slower on cheap ones with contended splats).
   RF_EXCHANGE_AUTO (default): after a warmup of a new genome structure (or a change of splat,
   tile or walker reset) the first two drawing launches of >= 32 passes and equal length run one
   form each, timed with CUDA events, and the faster runs from then on (decided without a host
   wait, once the second launch has finished; not during stream capture, where the pipelined form
   runs).  All forms give
   identical results.  A pipelined wait that runs out (bounded) makes the next synchronising call
   (rf_draw_to_bins with `drawn`, rf_sim_counters, rf_render) return RF_ERR_TIMEOUT. */
enum rf_exchange { RF_EXCHANGE_BARRIER = 0, RF_EXCHANGE_PIPELINED = 1, RF_EXCHANGE_AUTO = 2 };
RF_API int  rf_set_exchange(rf_sim* s, int mode);
/* The form the Sim's next drawing launch runs: 0 barrier, 1 pipelined (-1: null sim). */
RF_API int  rf_sim_exchange(const rf_sim* s);
/* The shared-memory tile the drawing passes use (RF_SPLAT_TILE's, or the one RF_SPLAT_AUTO chose):
   1 and x0, y0, w, h in out, 0 when there is none, -1 on a null argument or a failed call.
   Synchronises the Sim's stream when RF_SPLAT_AUTO's timing of a fitted tile is still pending. */
RF_API int  rf_sim_splat_tile(rf_sim* s, uint32_t out[4]);
/* [0] points binned and [1] points emitted (opacity > 0) by the last rf_draw_to_bins call,
   [2] walker-steps since rf_warmup. */
RF_API int  rf_sim_counters(rf_sim* s, uint64_t out[3]);

/* ------------------------------------------------------------------------------------------
 * Image passes — replace the GL density-estimation raster pass (main.cpp:490-515,
 * shaders/density_{vert,frag}.glsl) and the tonemap compute pass (main.cpp:522-535,
 * shaders/tonemap.glsl).  All pointers are device pointers.
 * ---------------------------------------------------------------------------------------- */

/* Adaptive density estimation: out (float4 per bin) = every bin with a > 0 spread over a disc
   of radius max(min, min(R, int(R / a^curve))), kernel (1 - d^2) * (2/pi) / r^2 with
   d = |offset| / (r + 0.5); r = 0 copies the bin.  R <= 100 (main.cpp:502). */
RF_API int rf_density_estimate(const float* bins_rgba, uint32_t width, uint32_t height, int radius,
                        int min_radius, float curve, float* out_rgba, void* stream);
/* rf_density_estimate without any device allocation (no counterpart in the reference).
   For callers that cannot call cudaMalloc — e.g. a plug-in inside a host application that owns
   the device memory pool, or a frame loop with a fixed memory budget that must not enter the
   allocator.  Its scratch (bin radii, kernel weights) lives in static device arrays of the
   library: at most 8,388,608 bins (one 3840x2160 grid) and 65,535 rows; larger grids return
   RF_ERR_CAPACITY.  The first call on a device looks the arrays up and fills the kernel-weight
   table with one synchronous copy (make it before any stream capture); later calls copy nothing
   from the host.  Calls share the radius scratch, so calls that overlap on the GPU race and must
   be serialised. */
RF_API int rf_density_estimate_static(const float* bins_rgba, uint32_t width, uint32_t height, int radius,
                                      int min_radius, float curve, float* out_rgba, void* stream);
/* The tonemap with flam3's spatial filter in place of the ss x ss box — the flam3 `filter` (radius
   in output pixels) and `filter_shape` attributes the reference ignores (flame.cpp:166-176).  The
   separable window is fwidth = int(2 * support * ss * radius) + 1 bins wide, made the parity of
   ss, sampled at cell centres and normalised; each output pixel weighs the log-scaled bins of its
   window (bins beyond the grid count as empty), then gamma / vibrancy / clamp as rf_tonemap.
   radius <= 0 is rf_tonemap's box; 2 * support * ss * radius must stay below 63. */
enum rf_filter_shape { RF_FILTER_GAUSSIAN = 0, RF_FILTER_BOX = 1, RF_FILTER_TRIANGLE = 2, RF_FILTER_HERMITE = 3 };
RF_API int rf_tonemap_filter(const float* rgba, uint32_t width, uint32_t height, uint32_t ss, float filter_radius,
                             int filter_shape, float gamma, float brightness, float vibrancy, float k2, float* out_f32,
                             uint8_t* out_rgba8, void* stream);
/* The reference's image tail (main.cpp:490-535: the density-estimation raster pass, then the
   tonemap pass) in one call: rf_density_estimate followed by rf_tonemap of its output, the same
   arithmetic, with k2 <= 0 taking bins / sum(a) of the estimator's output (FP64).  For radii up
   to 12 and ss dividing 8 the estimator's output stays in on-chip memory (each 32 x 8 tile is
   tonemapped where it is estimated) and the density sum comes from the radius pass, so the FP32
   output plane is never written; otherwise the passes run one after another.  Scratch comes from
   cudaMallocAsync on `stream`. */
RF_API int rf_density_tonemap(const float* bins_rgba, uint32_t width, uint32_t height, int radius, int min_radius,
                              float curve, uint32_t ss, float gamma, float brightness, float vibrancy, float k2,
                              float* out_f32, uint8_t* out_rgba8, void* stream);
/* FP64 statistics of the density channel: out[0] = sum of a, out[1] = max a, out[2] = bins with a > 0. */
RF_API int rf_hist_stats(const float* rgba, uint32_t width, uint32_t height, double* out3, void* stream);
/* Log-density tonemap (tonemap.glsl:18-38) with a box supersample filter of ss x ss bins:
   per bin c *= 0.5*brightness*log10(1 + a*k2)/a, mean over each ss x ss block, then
   gamma/vibrancy/clamp.  k2 <= 0 selects k2 = bins / sum(a) from rf_hist_stats.  Output is
   (width/ss) x (height/ss); out_f32 (float4) and/or out_rgba8 may be NULL. */
RF_API int rf_tonemap(const float* rgba, uint32_t width, uint32_t height, uint32_t ss, float gamma,
               float brightness, float vibrancy, float k2, float* out_f32, uint8_t* out_rgba8,
               void* stream);

/* ------------------------------------------------------------------------------------------
 * Walker shuffle — replaces create_shuffle_buffer / make_shuffle_buffers (shuffle_buffers.cpp).
 * ---------------------------------------------------------------------------------------- */
/* `count` keyed permutations of [0, n) (n <= 65536) into device memory out[count * n]. */
RF_API int rf_shuffle_generate(uint32_t n, uint32_t count, uint64_t seed, uint16_t* out, void* stream);

/* ------------------------------------------------------------------------------------------
 * Single-step probe (parity tests): one dispatch() of xform i (-1 = final) per point.
 * in_xyc: device float[3n]; rng: device uint32[4n] (advanced in place); out: device float[4n].
 * ---------------------------------------------------------------------------------------- */
RF_API int rf_probe_xform(rf_flame* f, int xform, uint32_t n, const float* in_xyc, uint32_t* rng,
                   int first_run, float* out_xycw, void* stream);

/* ------------------------------------------------------------------------------------------
 * Host convenience: one whole frame from host memory to host memory (end-to-end path).
 * ---------------------------------------------------------------------------------------- */
typedef struct {
    uint32_t width, height;     /* output image size */
    uint32_t supersample;       /* bins = (width*ss) x (height*ss) */
    uint32_t fuse_passes;       /* rf_warmup passes */
    uint64_t points;            /* target points (rounded up to whole passes) */
    float    tss_width;
    float    k2;                /* tonemap k2 (<= 0: automatic) */
    int32_t  density_estimation;/* 1: run the adaptive DE with the genome's estimator fields */
    int32_t  stop_on_binned;    /* 0: `points` walker-steps are computed; 1: passes are drawn until
                                   `points` points are binned — the reference's quality stop
                                   (main.cpp:411-412, accumulated < quality * W * H) — reading
                                   the binned count back between rounds of passes, at most 16x the
                                   passes of one step per point */
} rf_render_desc;
/* Renders `f` into out_rgba8 (host memory, width*height*4 bytes).  stats (may be NULL):
   [0] points computed, [1] points binned, [2] milliseconds on the device. */
RF_API int rf_render(rf_sim* s, rf_flame* f, const rf_render_desc* d, uint8_t* out_rgba8, double* stats);

/* ------------------------------------------------------------------------------------------
 * Batched rendering.  No counterpart in the reference, which renders one genome per call
 * (flame.cpp:146 draw_to_bins); this draws many genomes — animation frames, independent
 * genomes with different xform counts and bin grids — in one persistent launch pulling work
 * units from a queue, then runs each genome's density estimation and tonemap.  A work unit is a
 * self-contained chaos game of `cta_slots` walkers of one genome (own seeds, start points,
 * fuse passes, walker shuffle) run inside one CTA.  The sequence is captured once in a CUDA
 * graph (use_graph) and replayed by rf_batch_run.
 *
 * Unit u of an item is the reference's chaos game of one temporal sample of cta_slots walkers
 * seeded with s = item.seed + u * 0x9E3779B97F4A7C15 (slot i: warmup_ctx(i + s * cta_slots),
 * flame.cpp:138-141), fuse_passes discarded passes then its drawing passes; after the first pass
 * walkers are exchanged through one of 1024 shared permutations of the unit (keyed by
 * 0x5EED + cta_slots) and, at the first drawing pass, through a keyed permutation of the unit.
 * Items with equal seeds share their walkers' random streams (coherent animation frames).
 * ---------------------------------------------------------------------------------------- */
typedef struct rf_batch rf_batch;
typedef struct {
    const rf_flame* flame;      /* compiled genome; read at rf_batch_create only */
    uint32_t width, height;     /* output image size */
    uint32_t supersample;       /* bins = (width*ss) x (height*ss); 0 = 1 */
    uint64_t points;            /* points to draw (rounded up to whole unit passes) */
    uint64_t seed;              /* seeds of the genome's walkers and shuffles */
} rf_batch_item;
typedef struct {
    uint32_t fuse_passes;       /* discarded passes at the start of every unit; 0 = 20 */
    uint32_t cta_slots;         /* walkers per unit (1024, 2048, 4096); 0 = autotune: timed on a
                                   probe batch, then kept for the process per device and set of
                                   genome structures (the one cache shared between batches, behind
                                   a lock).  Give it explicitly for units that do not depend on
                                   timing or on earlier batches. */
    uint32_t unit_passes;       /* drawing passes per unit; 0 = the length whose units finish
                                   first on the device's SMs (deterministic for given items) */
    int32_t  density_estimation;/* 1: adaptive DE with each genome's estimator fields */
    float    k2;                /* tonemap k2 (<= 0: automatic per genome) */
    int32_t  use_graph;         /* 1: capture the whole batch in a CUDA graph */
    int32_t  device;
    int32_t  splat;             /* rf_splat; AUTO chooses per genome from its probe histogram */
    int32_t  image_f32;         /* 1: keep each tonemapped image in FP32 too (rf_batch_image_f32) */
    int32_t  specialize;        /* genome structures with >= 2 units per SM (or the only
                                   structure of the batch) get their own launch of a specialised
                                   kernel compiled at run time: 0 = when the run-time compiler
                                   loads, 1 = required, -1 = never; 2 = every structure (a one-time
                                   compilation of about a second per structure, in parallel, for
                                   batches rendered repeatedly; the launches overlap on forked
                                   streams) */
    int32_t  bad_value_reset;   /* 1: walkers that leave the plane restart, as rf_set_bad_value_reset */
} rf_batch_desc;
RF_API int rf_batch_create(const rf_batch_item* items, uint32_t n, const rf_batch_desc* d, rf_batch** out);
/* Enqueues one whole batch (clear, draw, DE, tonemap) on the batch's own stream. */
RF_API int rf_batch_run(rf_batch* b);
/* Waits for the last run.  stats (may be NULL, 4 doubles): [0] points computed, [1] points
   binned, [2] milliseconds on the device, [3] walker-steps including fuse passes. */
RF_API int rf_batch_sync(rf_batch* b, double* stats);
/* Copies item i's image (width*height*4 bytes) to host memory. */
RF_API int rf_batch_image(rf_batch* b, uint32_t i, uint8_t* out_rgba8);
/* Device pointers of item i's bins (float4 RGBA sums, u32 hits) and the bin grid size. */
RF_API int rf_batch_bins(rf_batch* b, uint32_t i, float** rgba, uint32_t** hits, uint32_t* width, uint32_t* height);
/* Copies item i's bins to host memory (either pointer may be NULL). */
RF_API int rf_batch_read_bins(rf_batch* b, uint32_t i, float* host_rgba, uint32_t* host_hits);
/* Item i's FP32 tonemapped image, RGBA float [height][width][4], to device or host memory
   (the batch must be created with image_f32). */
RF_API int rf_batch_image_f32(rf_batch* b, uint32_t i, float* dst_rgba);
/* Learned-DE input features of item i's bins (rf_denoiser_features) into device memory; the
   base channels carry the item's FP32 image when the batch keeps one (image_f32, supersample 1). */
RF_API int rf_batch_features(rf_batch* b, uint32_t i, float k2, float level, void* dst_bf16);
/* The autotuned shape: walkers per unit, number of units, drawing passes per unit. */
RF_API int rf_batch_info(const rf_batch* b, uint32_t* cta_slots, uint32_t* units, uint32_t* unit_passes);
/* 1 when item i is drawn by a genome-specialised kernel, 0 by the interpreted one, -1 bad index. */
RF_API int rf_batch_specialized(const rf_batch* b, uint32_t i);
/* The splat strategy chosen for item i (RF_SPLAT_GLOBAL or RF_SPLAT_WARP); -1 for a bad index. */
RF_API int rf_batch_splat(const rf_batch* b, uint32_t i);
RF_API int rf_batch_destroy(rf_batch* b);

/* ------------------------------------------------------------------------------------------
 * Tensor-core GEMM of the learned density estimator (no reference counterpart; the reference
 * has no learned path).  C[M x N] (+)= A[M x K] * B[N x K]^T with A, B bf16 device matrices,
 * K contiguous (row strides lda, ldb in elements, multiples of 8, 16-byte aligned bases), FP32
 * accumulation on tcgen05 tensor cores.  Modes: RF_GEMM_STORE_F32 (C float), RF_GEMM_STORE_BF16
 * (C bf16 = relu?(acc + bias[n])), RF_GEMM_ATOMIC_F32 (C float += acc; required for splits > 1,
 * which partitions K over CTAs).  Synchronises the stream.
 * ---------------------------------------------------------------------------------------- */
enum rf_gemm_mode { RF_GEMM_STORE_F32 = 0, RF_GEMM_STORE_BF16 = 1, RF_GEMM_ATOMIC_F32 = 2 };
RF_API int rf_gemm_bf16(const void* A, const void* B, void* C, uint32_t M, uint32_t N, uint32_t K, uint32_t lda,
                        uint32_t ldb, uint32_t ldc, int mode, const float* bias, int relu, uint32_t splits,
                        void* stream);
/* 3x3 convolution (stride 1, zero padding 1) as an implicit GEMM on the same tensor cores: the
 * GEMM gathers its im2col rows from the inputs instead of reading a materialised matrix.
 * Inputs are NHWC bf16: xa [n, h/2, w/2, ca] when up (nearest-neighbour upsampled to h x w) else
 * [n, h, w, ca]; xb [n, h, w, cb] (channel-concatenated after xa; NULL when cb = 0); ca, cb
 * multiples of 8.  B holds the weights as [N x 9 (ca + cb)] bf16 (row stride ldb), column
 * k = tap * (ca + cb) + c with tap = (dy + 1) * 3 + (dx + 1).  C [n h w x N] (row stride ldc),
 * mode and bias / relu as rf_gemm_bf16 (one split).  Synchronises the stream. */
RF_API int rf_conv3x3_bf16(const void* xa, uint32_t ca, int up, const void* xb, uint32_t cb, uint32_t n, uint32_t h,
                           uint32_t w, const void* B, uint32_t N, uint32_t ldb, void* C, uint32_t ldc, int mode,
                           const float* bias, int relu, void* stream);

/* ------------------------------------------------------------------------------------------
 * Learned density estimation (no reference counterpart).  A U-Net maps the features of a
 * short-run histogram to the converged, tonemapped RGB image: 4 levels of 32-48-64-96
 * channels, two 3x3 convolutions + ReLU per level, 2x2 average pooling, nearest-neighbour
 * upsampling with channel-concatenated skips, a 1x1 output convolution.  BF16 weights (FP32
 * masters), FP32 accumulation on the tcgen05 tensor cores; forward, backward and Adam are the
 * library's own kernels.  Tensors are device memory, NHWC: features bf16 [n, h, w, 8], images
 * and targets FP32 [n, h, w, 3]; h and w multiples of 8.  The denoiser runs on its own stream
 * (or the one set by rf_denoiser_set_stream); train_step with loss != NULL synchronises.
 * ---------------------------------------------------------------------------------------- */
typedef struct rf_denoiser rf_denoiser;
typedef struct {
    uint64_t max_pixels;        /* capacity: n * h * w of the largest call */
    uint64_t seed;              /* He-normal initialisation */
    int32_t  device;
} rf_denoiser_desc;
typedef struct {
    uint32_t in_a, in_b, out, taps;  /* input channels (in_b: skip, concatenated), outputs, 9 or 1 */
    int32_t  upsample, relu, level;  /* in_a upsampled 2x; ReLU; resolution level (0 = full) */
    int32_t  src_a, src_b;           /* producing layer, -1 the features / none, -100-l the pool
                                        of level l's input (the level above's last encoder conv) */
} rf_denoiser_layer_info;
RF_API int rf_denoiser_create(const rf_denoiser_desc* d, rf_denoiser** out);
RF_API int rf_denoiser_destroy(rf_denoiser* d);
RF_API int rf_denoiser_set_stream(rf_denoiser* d, void* stream);
/* Waits for the denoiser's stream (infer returns without waiting). */
RF_API int rf_denoiser_sync(rf_denoiser* d);
RF_API int rf_denoiser_num_layers(const rf_denoiser* d);
RF_API int rf_denoiser_layer(const rf_denoiser* d, int i, rf_denoiser_layer_info* out);
/* Parameters in layer order, each layer its weights [out][tap][in_a + in_b] then its bias. */
RF_API size_t rf_denoiser_num_params(const rf_denoiser* d);
RF_API int rf_denoiser_get_params(rf_denoiser* d, float* host, size_t cap);
RF_API int rf_denoiser_set_params(rf_denoiser* d, const float* host, size_t count);
/* Gradients of the last train_step, same layout as the parameters. */
RF_API int rf_denoiser_gradients(rf_denoiser* d, float* host, size_t cap);
/* Features of a histogram (bins float4 RGBA sums, width x height): [log10(1 + a k2),
   rgb * log10(1 + a k2) / a, base.rgb, level] as bf16; k2 <= 0 takes W*H / sum(a) (FP64
   reduction).  base_rgba (may be NULL) is the plain path's FP32 tonemapped image of the same
   histogram (rf_tonemap out_f32): the network predicts a residual on it.  level codes the run's
   sample count for a network trained on several (refrakt_gb300.learned uses log2(spp) / 10). */
RF_API int rf_denoiser_features(const float* bins_rgba, uint32_t width, uint32_t height, float k2,
                                const float* base_rgba, float level, void* out_bf16, void* stream);
/* out_rgb = clamp(base + net(feats), 0, 1). */
RF_API int rf_denoiser_infer(rf_denoiser* d, const void* feats, uint32_t n, uint32_t h, uint32_t w, float* out_rgb);
/* One Adam step (lr; betas 0.9, 0.999; eps 1e-8) on the mean L1 loss against target_rgb. */
RF_API int rf_denoiser_train_step(rf_denoiser* d, const void* feats, const float* target_rgb, uint32_t n, uint32_t h,
                                  uint32_t w, float lr, double* loss);

/* ------------------------------------------------------------------------------------------
 * Genome-specialised chaos kernels (no reference counterpart; the reference generates GLSL per
 * genome, variation_table.cpp:217-264).  The CUDA source the run-time compiler builds for this
 * genome's structure and CTA shape (`needed` receives its size incl. NUL), and a compile-only
 * check that needs no device (cubin size in *cubin_bytes).
 * ---------------------------------------------------------------------------------------- */
RF_API int rf_flame_kernel_source(const rf_flame* f, uint32_t cta_threads, uint32_t cta_slots, char* buf, size_t cap,
                                  size_t* needed);
RF_API int rf_flame_kernel_compile(const rf_flame* f, uint32_t cta_threads, uint32_t cta_slots, size_t* cubin_bytes);
/* 1 when the sim's next launches use a specialised kernel (after rf_warmup), else 0. */
RF_API int rf_sim_specialized(const rf_sim* s);

/* Writes an RGBA8 image as an uncompressed PNG. */
RF_API int rf_write_png(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);

#ifdef __cplusplus
}
#endif
#endif
