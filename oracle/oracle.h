/*
 * CPU oracle for the fractal-flame chaos game — TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in scalar C++, the arithmetic of the reference renderer
 * (untrioctium/refrakt): its GLSL iterate shader, variation library, density
 * estimation and tonemap.  It is the checker for the CUDA path.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it; the
 * product library never links, calls or falls back to it.
 *
 * Every function names the reference file:line it follows.  Arithmetic is
 * templated on the real type: FP64 for the correctness oracle, FP32 (with no
 * floating-point contraction) for the bit-exact and CPU-baseline modes.
 */
#ifndef REFRAKT_ORACLE_H
#define REFRAKT_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_genome orc_genome;

/* JSF32 (shaders/include/random.glsl:29-37, src/util.hpp:80-95). */
void     orc_jsf_warmup(uint32_t seed, uint32_t state[4]);
uint32_t orc_jsf_next(uint32_t state[4]);      /* returns the new `a`, as the GLSL ranval does */
float    orc_randf(uint32_t state[4]);         /* random.glsl:39-41 */

/* Start points (src/hammersley.cpp:29-48): count*4 floats (x, y, 0, 0). */
void orc_sample_points(uint32_t count, float* out4);

/* Keyed permutations used by the kernel's walker-shuffle schedule. */
uint32_t orc_feistel(uint32_t x, uint32_t n, uint64_t key);
uint64_t orc_derive_key(uint64_t seed, uint64_t a, uint64_t b, uint64_t tag);
/* `count` permutations of the kernel's shuffle table over n slots (out: count * n); phases as
   orc_chaos_cfg.table_phases */
void orc_shuffle_table(uint32_t n, uint32_t count, uint64_t seed, uint32_t phases, uint32_t* out);

/* Genome: reference flam3 loader semantics (src/flame.cpp:160-226). */
int  orc_genome_from_xml(const char* xml, orc_genome** out, char* err, int errlen);
void orc_genome_free(orc_genome* g);
int  orc_genome_num_xforms(const orc_genome* g);
int  orc_genome_has_final(const orc_genome* g);
/* flat parameter buffer (src/flame.cpp:33-103); returns total_params or -1 */
int  orc_genome_param_buffer(const orc_genome* g, float* out, int cap);
/* its layout as the reference's buffer_map_ JSON (flame.cpp:33-71: per xform weight, affine[6],
   post[6], variations, param, color, color_speed, opacity, rotation_frequency; final_xform;
   size) — what the reference renders its shader templates with.  Returns the length (the
   text is truncated to cap - 1 bytes and NUL-terminated). */
int  orc_genome_layout_json(const orc_genome* g, char* out, int cap);
/* the flat parameter buffer of temporal sample t of T after animate.tpl.glsl's rotation */
int  orc_animate_params(const orc_genome* g, uint32_t T, float tss_width, uint32_t t, float* out, int cap);
/* camera + tonemap fields: size[2], center[2], scale, rotate, est_radius, est_min, est_curve,
   gamma, vibrancy, brightness  -> 12 doubles */
void orc_genome_info(const orc_genome* g, double* out12);
/* screen affine (src/flame.cpp:289-296) for a bin grid */
void orc_screen_affine(const orc_genome* g, uint32_t width, uint32_t height, float out6[6]);
/* RNG draws one evaluation of xform xi consumes (xi = -1: final xform) */
int  orc_xform_draws(const orc_genome* g, int xi, int first_run);

/* xform selection (shaders/templates/xform_select.tpl.glsl) */
int orc_select_xform(const orc_genome* g, float r);

/* One dispatch() of xform xi (-1 = final) on n points.
   in: n*3 (x, y, c); rng: n*4 states, advanced in place; out: n*4 (x, y, c, opacity). */
int orc_eval_xform(const orc_genome* g, int xi, int fp64, int n, const float* in_xyc,
                   uint32_t* rng, int first_run, double* out);

/* Chaos game restated from shaders/flame.glsl:41-90 and src/flame.cpp:228-330. */
typedef struct {
    uint64_t walkers;          /* total walker slots N */
    uint32_t temporal_samples; /* T; N/T walkers per temporal sample */
    uint64_t seed;             /* slot i is seeded with warmup_ctx(i + seed*N) */
    uint32_t fuse_passes;      /* passes before drawing; pass 0 is the jitter (first_run) pass */
    uint32_t draw_passes;
    uint32_t width, height;    /* bin grid */
    int      fp64;             /* 1: double arithmetic; 0: float, no contraction */
    int      shuffle_mode;     /* 0: fresh uniform permutation per pass (reference scheme)
                                  1: the CUDA kernel's documented schedule */
    uint32_t cta_slots;        /* shuffle_mode 1: slots per CTA */
    uint32_t steps_per_launch; /* shuffle_mode 1: passes per launch (L) */
    uint32_t table_size;       /* shuffle_mode 1: permutations in the local table */
    float    tss_width;        /* temporal sample width (animate.tpl.glsl) */
    int      threads;          /* worker threads (>=1) */
    int      table_seed_set;   /* shuffle_mode 1: 1 = the local table is keyed by table_seed, */
    uint64_t table_seed;       /*   0 = by seed (the batched launch shares one table) */
    int      badval_reset;     /* 1: the walker reset flame.glsl:68 keeps commented out */
    uint32_t table_phases;     /* shuffle_mode 1: 0 = uniform table permutations; S > 1 = the
                                  pipelined table of S phases per pass: the first cta_slots/S
                                  destinations draw their sources from the first
                                  cta_slots*(S-1)/S slots only (the library uses S = 4) */
} orc_chaos_cfg;

/* rgba: W*H*4 doubles (may be NULL), hits: W*H u64 (may be NULL),
   xid_trace: (fuse+draw) * (N/256) bytes (may be NULL),
   counters[0] = drawn (in bounds, w>0), counters[1] = emitted (w>0). */
int orc_chaos(const orc_genome* g, const orc_chaos_cfg* cfg, double* rgba, uint64_t* hits,
              uint8_t* xid_trace, uint64_t* counters);

/* The xid sequence alone, predicted from RNG draw counts (no walker arithmetic; without the
   walker reset, whose draws depend on the walker). */
int orc_xid_sequence(const orc_genome* g, uint64_t walkers, uint32_t temporal_samples,
                     uint64_t seed, uint32_t fuse_passes, uint32_t draw_passes, uint8_t* out);

/* Multi-threaded FP32 transcription used as the timed CPU baseline: walker slices
   with private float histograms merged at the end, optionally with the walker reset of
   flame.glsl:68.  Returns points computed; *binned_out (may be NULL) the points binned. */
uint64_t orc_cpu_baseline(const orc_genome* g, uint64_t walkers, uint32_t passes,
                          uint32_t width, uint32_t height, int threads, uint64_t seed, int badval_reset,
                          float* rgba_out, uint32_t* hits_out, uint64_t* binned_out);

/* The density estimator's radius of a bin with density a (density_vert.glsl:35-44) and the
   kernel weight at offset (dx, dy) of a disc of radius r (density_frag.glsl:9-18, symmetric
   restatement); the weight is -1 outside the disc. */
int    orc_de_radius(double a, int radius, int min_radius, double curve);
double orc_de_weight(int dx, int dy, int r);

/* Adaptive density estimation (shaders/density_vert.glsl:26-63, density_frag.glsl:9-18),
   symmetric restatement: d = |delta|^2/(r+0.5)^2. in/out W*H*4 doubles. */
int orc_density_estimate(const double* in, uint32_t w, uint32_t h, int radius, int min_radius,
                         double curve, double* out);
/* Log-density tonemap (shaders/tonemap.glsl:18-38) with an ss x ss box filter applied after the
   per-bin log scaling.  out (W/ss)*(H/ss)*4 doubles. */
int orc_tonemap(const double* in, uint32_t w, uint32_t h, uint32_t ss, double gamma, double brightness,
                double vibrancy, double k2, double* out);
/* The flam3 spatial filter in place of the box (no counterpart in the reference, which ignores
   flam3's filter / filter_shape, flame.cpp:166-176): shape 0 gaussian, 1 box, 2 triangle,
   3 hermite; a separable kernel of fwidth taps (orc_filter_kernel), each output pixel the
   weighted sum of the log-scaled bins of its fwidth x fwidth window, then gamma / vibrancy /
   clamp as tonemap.glsl.  orc_filter_kernel writes the normalised 1-D taps (cap >= 64) and
   returns fwidth, or -1. */
int orc_filter_kernel(uint32_t ss, double radius, int shape, double* taps, int cap);
int orc_tonemap_filter(const double* in, uint32_t w, uint32_t h, uint32_t ss, double radius, int shape,
                       double gamma, double brightness, double vibrancy, double k2, double* out);
/* Box supersample filter: out[(W/ss)*(H/ss)*4] = mean of ss*ss blocks. */
int orc_downsample(const double* in, uint32_t w, uint32_t h, uint32_t ss, double* out);

#ifdef __cplusplus
}
#endif
#endif
