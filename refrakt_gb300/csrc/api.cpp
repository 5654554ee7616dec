// C ABI of refrakt_gb300 (include/refrakt.h): the host runtime around the device kernels.
//
// Replaces the reference's flame_compiler / flame classes (src/variation_table.hpp:20-59,
// src/flame.hpp:41-173) and its GL dispatch loop (src/flame.cpp:105-330, src/main.cpp:490-535).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "internal.h"
#include "kernels.h"

namespace rfk {

static thread_local std::string g_err;
int fail(int status, const std::string& msg) {
    g_err = msg;
    return status;
}
void clear_error() { g_err.clear(); }

static int cuda_fail(cudaError_t e, const char* what) {
    return fail(RF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define RF_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

static std::atomic<uint64_t> g_uid{1};

}  // namespace rfk

using namespace rfk;

#include "handles.h"
#include "specialize.h"

namespace {

// rf_sim's splat setting as ChaosArgs.splat's code: 0 global, 1 warp-aggregated, 2 adaptive
int splat_code(int splat) {
    return splat == RF_SPLAT_WARP ? 1 : splat == RF_SPLAT_GLOBAL ? 0 : splat == RF_SPLAT_TILE ? 3 : 2;
}

}  // namespace

namespace {

constexpr size_t kInterleaveMinBytes = 256ull << 20;  // bins + counts above ~2x L2: interleave

int set_device(const rf_sim* s) {
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return RF_OK;
}

size_t copy_out(const std::string& s, char* buf, size_t cap) {
    if (buf && cap) {
        size_t n = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), n);
        buf[n] = 0;
    }
    return s.size() + 1;
}

// The pipelined walker exchange (chaos_body.cuh, PIPE) runs in the specialised kernels when the
// Sim's shuffle table was built for it (4 slots per thread) and its two mbarriers fit in shared
// memory beside the tile splat's bins.
bool use_pipe(const rf_sim* s, uint32_t tile_bins) {
    return s->table_phases >= 3 && chaos_smem(s->slots, s->prog_words, s->L, tile_bins, 1) <= kMaxCtaSmem;
}

void reset_exchange_tuning(rf_sim* s);

bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

// The tile (x0, y0, w, h) of at most `cap` bins that holds the most hits — the bounding box of the
// hit bins when it fits, else the window of about sqrt(cap) x sqrt(cap) bins with the largest sum
// (2D prefix sums) — and the share of all hits inside it.
double fit_splat_tile(const std::vector<uint32_t>& h, uint32_t W, uint32_t H, uint32_t cap, uint32_t t[4]) {
    uint64_t total = 0;
    uint32_t x0 = W, x1 = 0, y0 = H, y1 = 0;
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++)
            if (const uint32_t v = h[(size_t)y * W + x]) {
                total += v;
                x0 = std::min(x0, x); x1 = std::max(x1, x);
                y0 = std::min(y0, y); y1 = std::max(y1, y);
            }
    if (!total || !cap) return 0.0;
    if ((uint64_t)(x1 - x0 + 1) * (y1 - y0 + 1) <= cap) {
        t[0] = x0; t[1] = y0; t[2] = x1 - x0 + 1; t[3] = y1 - y0 + 1;
        return 1.0;
    }
    const uint32_t w = std::min<uint32_t>(W, std::max<uint32_t>(1, (uint32_t)std::sqrt((double)cap)));
    const uint32_t hh = std::min<uint32_t>(H, cap / w);
    std::vector<uint64_t> P((size_t)(W + 1) * (H + 1), 0);
    for (uint32_t y = 0; y < H; y++) {
        uint64_t row = 0;
        for (uint32_t x = 0; x < W; x++) {
            row += h[(size_t)y * W + x];
            P[(size_t)(y + 1) * (W + 1) + x + 1] = P[(size_t)y * (W + 1) + x + 1] + row;
        }
    }
    uint64_t best = 0;
    t[0] = t[1] = 0; t[2] = w; t[3] = hh;
    for (uint32_t y = 0; y + hh <= H; y++)
        for (uint32_t x = 0; x + w <= W; x++) {
            const uint64_t v = P[(size_t)(y + hh) * (W + 1) + x + w] - P[(size_t)y * (W + 1) + x + w] -
                               P[(size_t)(y + hh) * (W + 1) + x] + P[(size_t)y * (W + 1) + x];
            if (v > best) { best = v; t[0] = x; t[1] = y; }
        }
    return (double)best / (double)total;
}

// RF_SPLAT_AUTO for compact attractors.  After the second drawing launch of >= 32 passes on a grid
// (timed; the first warms the grid up), the counts are read back once and a tile fitted; if it
// holds >= 25 % of the hits, the next launch of the same length runs with it (timed) and the
// faster splat is kept.  Grids above kAutoTileMaxBins are not read back (their planes go through
// interleaved records by default).
constexpr uint64_t kAutoTileMaxBins = 1ull << 24;
int fit_auto_tile(rf_sim* s, const uint32_t* hits, uint32_t W, uint32_t H) {
    s->auto_tile_state = -1;
    std::vector<uint32_t> h((size_t)W * H);
    RF_CUDA(cudaStreamSynchronize(s->stream));
    RF_CUDA(cudaMemcpy(h.data(), hits, h.size() * 4, cudaMemcpyDeviceToHost));
    const size_t used = (chaos_smem(s->slots, s->prog_words, s->L, 0, 1) + 15) & ~(size_t)15;
    const uint32_t cap = used < kMaxCtaSmem ? (uint32_t)std::min<size_t>((kMaxCtaSmem - used) / 20, 65536) : 0u;
    uint32_t t[4];
    if (fit_splat_tile(h, W, H, cap, t) >= 0.25) {
        s->auto_tile_state = 3;
        memcpy(s->auto_tile, t, sizeof t);
    }
    return RF_OK;
}

// RF_SPLAT_AUTO, both launches timed: keep the tile if its launch was faster, once it has finished
void decide_auto_tile(rf_sim* s) {
    const cudaError_t q = cudaEventQuery(s->tile_ev[3]);
    if (q == cudaErrorNotReady) {
        if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();  // clear only this status
        return;
    }
    float t0 = 0.0f, t1 = 0.0f;
    const bool ok = q == cudaSuccess && cudaEventElapsedTime(&t0, s->tile_ev[0], s->tile_ev[1]) == cudaSuccess &&
                    cudaEventElapsedTime(&t1, s->tile_ev[2], s->tile_ev[3]) == cudaSuccess;
    s->auto_tile_state = ok && t1 < t0 ? 1 : -1;
    reset_exchange_tuning(s);  // time the exchange forms on the kernel that stays
}

// RF_EXCHANGE_AUTO starts over (a new genome structure, splat, tile or reset changes the kernels)
void reset_exchange_tuning(rf_sim* s) {
    s->tune_step = 0;
    s->tune_pipe = 1;
}

// The exchange form of the next launch (1 pipelined); *measure = 0 / 1 when RF_EXCHANGE_AUTO times
// this launch as the barrier / pipelined form, else -1.  Drawing launches of >= 32 passes are
// timed, the second one only at the first one's length.
int exchange_for_launch(rf_sim* s, bool draw, uint32_t steps, bool may_measure, int* measure) {
    *measure = -1;
    if (s->exchange != RF_EXCHANGE_AUTO) return s->exchange == RF_EXCHANGE_PIPELINED ? 1 : 0;
    if (s->tune_step == 2) {  // both forms timed: decide once the second launch has finished
        const cudaError_t q = cudaEventQuery(s->tune_ev[3]);
        if (q == cudaSuccess) {
            float tb = 0.0f, tp = 0.0f;
            if (cudaEventElapsedTime(&tb, s->tune_ev[0], s->tune_ev[1]) == cudaSuccess &&
                cudaEventElapsedTime(&tp, s->tune_ev[2], s->tune_ev[3]) == cudaSuccess)
                s->tune_pipe = tp <= tb ? 1 : 0;
            s->tune_step = 3;
        } else if (q == cudaErrorNotReady) {
            if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();  // clear only this status
        } else {
            s->tune_step = 3;  // the events failed: keep the default
        }
    }
    if (s->tune_step < 2 && draw && steps >= 32 && (s->tune_step == 0 || steps == s->tune_passes) && s->tune_ev[0] &&
        may_measure && !capturing(s->stream)) {
        if (s->tune_step == 0) s->tune_passes = steps;
        *measure = s->tune_step;
        return s->tune_step;
    }
    return s->tune_pipe;
}

// RF_ERR_TIMEOUT when a pipelined exchange wait in an earlier launch ran out (counters[3]); call
// after the stream was synchronised
int check_exchange(rf_sim* s) {
    unsigned long long n = 0;
    RF_CUDA(cudaMemcpy(&n, s->counters + 3, sizeof n, cudaMemcpyDeviceToHost));
    if (n) return fail(RF_ERR_TIMEOUT, std::to_string(n) + " walker-exchange waits of the chaos kernel ran out; "
                                       "the histogram of those launches is invalid");
    return RF_OK;
}

// the chaos kernel reads these counters as unsigned long long
int launch_passes(rf_sim* s, uint32_t passes, bool first_run, bool draw, float4* bins, uint32_t* hits,
                  uint32_t W, uint32_t H, const float ss[6]) {
    uint32_t done = 0;
    while (done < passes) {
        const uint32_t steps = std::min(s->L, passes - done);
        ChaosArgs a{};
        a.progs = s->progs;
        a.prog_stride = s->prog_stride;
        a.prog_words = s->prog_words;
        a.walk_in = s->walk[s->cur];
        a.walk_out = s->walk[s->cur ^ 1];
        a.rng = s->rng;
        a.table = s->table;
        a.table_size = s->table_size;
        a.ppts = s->ppts;
        a.chunks_per_ts = s->ppts / s->slots;
        a.pass0 = s->pass;
        a.steps = steps;
        a.seed = s->d.seed;
        a.first_run = (first_run && done == 0) ? 1 : 0;
        a.draw = draw ? 1 : 0;
        // RF_SPLAT_AUTO's tile: settle a pending decision, then see whether this launch is timed
        const bool tile_grid = draw && s->splat == RF_SPLAT_AUTO && s->rgba_shift == 0 && hits &&
                               (uint64_t)W * H <= kAutoTileMaxBins && s->tile_ev[0] && !capturing(s->stream);
        if (tile_grid && (s->auto_tile_wh[0] != W || s->auto_tile_wh[1] != H)) {
            s->auto_tile_state = 0;  // a new grid
            s->auto_tile_wh[0] = W;
            s->auto_tile_wh[1] = H;
        }
        if (s->auto_tile_state == 4) decide_auto_tile(s);
        int tile_timed = -1;  // 0: the untiled launch, 1: the tiled one
        const bool tile_warmup = tile_grid && steps >= 32 && s->auto_tile_state == 0;  // not timed: the grid's first
        if (tile_grid && steps >= 32 && s->auto_tile_state == 2) tile_timed = 0;
        if (tile_grid && steps == s->auto_tile_passes && s->auto_tile_state == 3) tile_timed = 1;
        const bool auto_tile = draw && s->splat == RF_SPLAT_AUTO && s->rgba_shift == 0 && s->auto_tile_wh[0] == W &&
                               s->auto_tile_wh[1] == H && (s->auto_tile_state == 1 || tile_timed == 1);
        a.splat = auto_tile ? 3 : splat_code(s->splat);
        a.reset = s->reset;
        a.rgba_shift = s->rgba_shift;
        a.count_shift = s->count_shift;
        if (ss) memcpy(a.ss, ss, sizeof(a.ss));
        const uint32_t* tl = auto_tile ? s->auto_tile : s->tile;
        a.tile_x0 = tl[0];
        a.tile_y0 = tl[1];
        a.tile_w = tl[2];
        a.tile_h = tl[3];
        a.W = W;
        a.H = H;
        a.bins = bins;
        a.hits = hits;
        a.palette = s->palette;
        a.counters = s->counters;
        a.trace = s->trace;
        a.trace_passes = s->trace_passes;
        a.n_groups = (uint32_t)(s->N / kGroup);
        const uint32_t grid = (uint32_t)(s->N / s->slots);
        const uint32_t tile_bins = a.splat == 3 && a.draw ? a.tile_w * a.tile_h : 0u;
        int measure = -1;
        // (RF_SPLAT_AUTO's tile is timed first, in the pipelined form; the exchange after it)
        const bool tile_busy = tile_warmup || tile_timed >= 0 || (s->splat == RF_SPLAT_AUTO && s->auto_tile_state >= 2);
        const int want = s->spec ? exchange_for_launch(s, a.draw, steps, !tile_busy, &measure) : 0;
        const int pipe = want && s->spec && use_pipe(s, tile_bins) ? 1 : 0;
        if (s->spec && (s->spec_splat != a.splat || s->spec_reset != a.reset || s->spec_pipe != pipe)) {
            // the splat strategy, the reset or the exchange changed since warmup: the kernel compiled for them
            const void* k = nullptr;
            if (int rc = spec_kernel(s->spec_prog, (int)s->threads, (int)s->slots, s->device, &k, SpecKind::Chaos,
                                     a.splat, a.reset, pipe))
                return rc;
            s->spec = k;
            s->spec_splat = a.splat;
            s->spec_reset = a.reset;
            s->spec_pipe = pipe;
        }
        if (chaos_smem(s->slots, a.prog_words, a.steps, tile_bins) > kMaxCtaSmem)
            return fail(RF_ERR_CAPACITY, "splat tile of " + std::to_string(tile_bins) +
                                         " bins exceeds the shared memory beside " + std::to_string(s->slots) +
                                         " walker slots");
        if (measure >= 0 && cudaEventRecord(s->tune_ev[2 * measure], s->stream) != cudaSuccess) measure = -1;
        if (tile_timed >= 0 && cudaEventRecord(s->tile_ev[2 * tile_timed], s->stream) != cudaSuccess) tile_timed = -1;
        cudaError_t e = s->spec ? launch_spec(s->spec, (int)s->threads, (int)s->slots, a, grid,
                                              chaos_smem(s->slots, a.prog_words, a.steps, tile_bins, pipe), s->stream)
                                : launch_chaos((int)s->threads, (int)s->slots, a, grid, s->stream);
        if (e != cudaSuccess) return cuda_fail(e, "chaos kernel launch");
        if (measure >= 0 && cudaEventRecord(s->tune_ev[2 * measure + 1], s->stream) == cudaSuccess)
            s->tune_step = measure + 1;
        const bool tile_recorded = tile_timed >= 0 && cudaEventRecord(s->tile_ev[2 * tile_timed + 1], s->stream) == cudaSuccess;
        s->cur ^= 1;
        s->pass += steps;
        done += steps;
        if (tile_warmup) s->auto_tile_state = 2;
        if (tile_timed == 0) {
            if (!tile_recorded) {
                s->auto_tile_state = -1;
            } else {
                s->auto_tile_passes = steps;
                if (int rc = fit_auto_tile(s, hits, W, H)) return rc;  // -> 3 (a candidate) or -1
            }
        } else if (tile_timed == 1) {
            s->auto_tile_state = tile_recorded ? 4 : -1;
        }
    }
    return RF_OK;
}

// The drawing passes into the caller's planes, or — for histograms well above L2 with a count
// plane — into interleaved 32-byte records (RGBA and count in one DRAM sector) merged into the
// caller's planes afterwards.
int draw_passes(rf_sim* s, uint32_t passes, float4* bins, uint32_t* hits, uint32_t W, uint32_t H, const float ss[6]) {
    const size_t nb = (size_t)W * H;
    bool il = s->bin_layout == RF_BINS_INTERLEAVED;
    if (s->bin_layout == RF_BINS_AUTO) il = hits != nullptr && nb * 20 > kInterleaveMinBytes;
    if (!il) return launch_passes(s, passes, false, true, bins, hits, W, H, ss);
    if (s->rec_n < nb) {
        cudaFree(s->rec);
        s->rec = nullptr;
        s->rec_n = 0;
        RF_CUDA(cudaMalloc((void**)&s->rec, nb * 32));
        RF_CUDA(cudaMemsetAsync(s->rec, 0, nb * 32, s->stream));
        s->rec_n = nb;
    }
    s->rgba_shift = 1;
    s->count_shift = 3;
    const int rc = launch_passes(s, passes, false, true, s->rec, hits ? reinterpret_cast<uint32_t*>(s->rec) + 4 : nullptr,
                                 W, H, ss);
    s->rgba_shift = 0;
    s->count_shift = 0;
    if (rc) return rc;
    RF_CUDA(launch_merge_records(s->rec, nb, bins, hits, s->stream));
    return RF_OK;
}

}  // namespace

extern "C" {

const char* rf_last_error(void) { return g_err.c_str(); }
int rf_abi_version(void) { return RF_ABI_VERSION; }

// ---------------------------------------------------------------------------------------------
// compiler
// ---------------------------------------------------------------------------------------------
int rf_compiler_create(const char* yaml_path, rf_compiler** out) {
    if (!out) return fail(RF_ERR_INVALID_ARG, "rf_compiler_create: out is NULL");
    *out = nullptr;
    auto* c = new rf_compiler();
    if (yaml_path) {
        if (int rc = load_registry_yaml(yaml_path, c->reg)) { delete c; return rc; }
    } else {
        c->reg = builtin_registry();
    }
    *out = c;
    return RF_OK;
}
void rf_compiler_destroy(rf_compiler* c) { delete c; }
int rf_compiler_is_variation(const rf_compiler* c, const char* n) { return (c && n && c->reg->vars.count(n)) ? 1 : 0; }
int rf_compiler_is_param(const rf_compiler* c, const char* n) { return (c && n && c->reg->param_owner.count(n)) ? 1 : 0; }
int rf_compiler_is_common(const rf_compiler* c, const char* n) { return (c && n && c->reg->common.count(n)) ? 1 : 0; }
int rf_compiler_is_supported(const rf_compiler* c, const char* n) {
    if (!c || !n) return 0;
    auto it = c->reg->vars.find(n);
    return (it != c->reg->vars.end() && it->second.kernel_id >= 0) ? 1 : 0;
}
int rf_compiler_param_owner(const rf_compiler* c, const char* p, char* buf, size_t cap) {
    if (!c || !p) return fail(RF_ERR_INVALID_ARG, "rf_compiler_param_owner: null argument");
    auto it = c->reg->param_owner.find(p);
    if (it == c->reg->param_owner.end()) return fail(RF_ERR_UNKNOWN_NAME, std::string("not a parameter: ") + p);
    copy_out(it->second, buf, cap);
    return RF_OK;
}
int rf_compiler_num_variations(const rf_compiler* c) { return c ? (int)c->reg->vars.size() : 0; }
int rf_compiler_variation_name(const rf_compiler* c, int i, char* buf, size_t cap) {
    if (!c || i < 0 || i >= (int)c->reg->vars.size()) return fail(RF_ERR_INVALID_ARG, "variation index out of range");
    auto it = c->reg->vars.begin();
    std::advance(it, i);
    copy_out(it->first, buf, cap);
    return RF_OK;
}
int rf_compiler_variation_params(const rf_compiler* c, const char* name, char* buf, size_t cap) {
    if (!c || !name) return fail(RF_ERR_INVALID_ARG, "rf_compiler_variation_params: null argument");
    auto it = c->reg->vars.find(name);
    if (it == c->reg->vars.end()) return fail(RF_ERR_UNKNOWN_NAME, std::string("not a variation: ") + name);
    std::string s;
    for (size_t k = 0; k < it->second.params.size(); k++) s += (k ? "," : "") + it->second.params[k];
    copy_out(s, buf, cap);
    return RF_OK;
}

// ---------------------------------------------------------------------------------------------
// flames
// ---------------------------------------------------------------------------------------------
static int new_flame(Genome&& g, const rf_compiler* c, rf_flame** out) {
    auto* f = new rf_flame();
    f->g = std::move(g);
    f->reg = c->reg;
    f->uid = g_uid.fetch_add(1);
    *out = f;
    return RF_OK;
}

int rf_flame_load_xml(const char* xml, const rf_compiler* c, rf_flame** out) {
    if (!xml || !c || !out) return fail(RF_ERR_INVALID_ARG, "rf_flame_load_xml: null argument");
    *out = nullptr;
    Genome g;
    if (int rc = genome_from_xml(xml, *c->reg, g)) return rc;
    return new_flame(std::move(g), c, out);
}

int rf_flame_load(const char* path, const rf_compiler* c, rf_flame** out) {
    if (!path || !c || !out) return fail(RF_ERR_INVALID_ARG, "rf_flame_load: null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(RF_ERR_IO, std::string("cannot read ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return rf_flame_load_xml(ss.str().c_str(), c, out);
}

void rf_flame_free(rf_flame* f) { delete f; }

int rf_flame_to_xml(const rf_flame* f, char* buf, size_t cap, size_t* needed) {
    if (!f) return fail(RF_ERR_INVALID_ARG, "rf_flame_to_xml: null flame");
    size_t n = copy_out(genome_to_xml(f->g), buf, cap);
    if (needed) *needed = n;
    return RF_OK;
}

int rf_flame_synthesize(const rf_synth_desc* d, const rf_compiler* c, rf_flame** out) {
    if (!d || !c || !out) return fail(RF_ERR_INVALID_ARG, "rf_flame_synthesize: null argument");
    *out = nullptr;
    Genome g;
    if (int rc = genome_synthesize(d->kind, d->seed, d->n_xforms, d->final_xform, d->force_parametric, d->width,
                                   d->height, *c->reg, g))
        return rc;
    return new_flame(std::move(g), c, out);
}

int rf_flame_from_struct(const rf_genome_desc* d, const rf_compiler* c, rf_flame** out) {
    if (!d || !c || !out || (d->n_xforms && !d->xforms) || !d->palette_rgb)
        return fail(RF_ERR_INVALID_ARG, "rf_flame_from_struct: null argument");
    *out = nullptr;
    Genome g;
    g.size[0] = d->size[0];
    g.size[1] = d->size[1];
    g.center[0] = d->center[0];
    g.center[1] = d->center[1];
    g.scale = d->scale;
    g.rotate = d->rotate;
    g.est_radius = d->estimator_radius;
    g.est_min = d->estimator_min;
    g.est_curve = d->estimator_curve;
    g.gamma = d->gamma;
    g.vibrancy = d->vibrancy;
    g.brightness = d->brightness;
    for (int i = 0; i < 256; i++) {
        for (int k = 0; k < 3; k++) g.palette[i][k] = d->palette_rgb[3 * i + k];
        g.palette[i][3] = 1.0f;
    }
    const Registry& reg = *c->reg;
    auto xform = [&](const rf_xform_desc& s, Xform& x) -> int {
        x.weight = s.weight;
        x.color = s.color;
        x.color_speed = s.color_speed;
        x.opacity = s.opacity;
        for (int k = 0; k < 6; k++) x.affine[k] = s.coefs[k];
        x.has_post = s.has_post != 0;
        for (int k = 0; k < 6; k++) x.post[k] = x.has_post ? s.post[k] : (k == 0 || k == 3 ? 1.0f : 0.0f);
        if ((s.n_vars && (!s.var_names || !s.var_weights)) || (s.n_params && (!s.param_names || !s.param_values)))
            return fail(RF_ERR_INVALID_ARG, "rf_flame_from_struct: null name or value array");
        for (uint32_t k = 0; k < s.n_vars; k++) {
            if (!s.var_names[k] || !reg.vars.count(s.var_names[k]))
                return fail(RF_ERR_UNKNOWN_NAME, std::string("unknown variation ") + (s.var_names[k] ? s.var_names[k] : "(null)"));
            x.vars[s.var_names[k]] = s.var_weights[k];
        }
        for (uint32_t k = 0; k < s.n_params; k++) {
            if (!s.param_names[k] || !reg.param_owner.count(s.param_names[k]))
                return fail(RF_ERR_UNKNOWN_NAME, std::string("unknown parameter ") + (s.param_names[k] ? s.param_names[k] : "(null)"));
            x.params[s.param_names[k]] = s.param_values[k];
        }
        return RF_OK;
    };
    g.xforms.resize(d->n_xforms);
    for (uint32_t i = 0; i < d->n_xforms; i++)
        if (int rc = xform(d->xforms[i], g.xforms[i])) return rc;
    if (d->final_xform) {
        g.has_final = true;
        if (int rc = xform(*d->final_xform, g.final_xf)) return rc;
    }
    if (int rc = genome_validate(g, reg)) return rc;
    return new_flame(std::move(g), c, out);
}

int rf_flame_interpolate(const rf_flame* a, const rf_flame* b, float t, rf_flame** out) {
    if (!a || !b || !out) return fail(RF_ERR_INVALID_ARG, "rf_flame_interpolate: null argument");
    *out = nullptr;
    if (a->reg != b->reg) return fail(RF_ERR_INVALID_ARG, "rf_flame_interpolate: flames from different variation tables");
    Genome g;
    if (int rc = genome_interpolate(a->g, b->g, t, *a->reg, g)) return rc;
    auto* f = new rf_flame();
    f->g = std::move(g);
    f->reg = a->reg;
    f->uid = g_uid.fetch_add(1);
    *out = f;
    return RF_OK;
}

int rf_flame_get_info(const rf_flame* f, rf_flame_info* o) {
    if (!f || !o) return fail(RF_ERR_INVALID_ARG, "rf_flame_get_info: null argument");
    const Genome& g = f->g;
    o->size[0] = g.size[0]; o->size[1] = g.size[1];
    o->center[0] = g.center[0]; o->center[1] = g.center[1];
    o->scale = g.scale; o->rotate = g.rotate;
    o->estimator_radius = g.est_radius; o->estimator_min = g.est_min; o->estimator_curve = g.est_curve;
    o->gamma = g.gamma; o->vibrancy = g.vibrancy; o->brightness = g.brightness;
    o->num_xforms = (uint32_t)g.xforms.size();
    o->has_final = g.has_final ? 1 : 0;
    std::vector<float> buf;
    o->total_params = (genome_param_buffer(g, buf, nullptr) == 0) ? (uint32_t)buf.size() : 0;
    o->filter = g.filter;
    o->filter_shape = g.filter_shape;
    return RF_OK;
}

int rf_flame_set_view(rf_flame* f, const float center[2], float scale, float rotate) {
    if (!f || !center) return fail(RF_ERR_INVALID_ARG, "rf_flame_set_view: null argument");
    f->g.center[0] = center[0]; f->g.center[1] = center[1];
    f->g.scale = scale; f->g.rotate = rotate;
    return RF_OK;  // the view does not invalidate walkers (draw_to_bins rebuilds the screen affine)
}

int rf_flame_set_tonemap(rf_flame* f, float gamma, float brightness, float vibrancy) {
    if (!f) return fail(RF_ERR_INVALID_ARG, "rf_flame_set_tonemap: null flame");
    f->g.gamma = gamma; f->g.brightness = brightness; f->g.vibrancy = vibrancy;
    return RF_OK;
}

int rf_flame_set_estimator(rf_flame* f, int radius, int min_radius, float curve) {
    if (!f) return fail(RF_ERR_INVALID_ARG, "rf_flame_set_estimator: null flame");
    f->g.est_radius = radius; f->g.est_min = min_radius; f->g.est_curve = curve;
    return RF_OK;
}

int rf_flame_set_xform_value(rf_flame* f, int xi, const char* name, float v) {
    if (!f || !name) return fail(RF_ERR_INVALID_ARG, "rf_flame_set_xform_value: null argument");
    Xform* x = nullptr;
    if (xi < 0) { if (!f->g.has_final) return fail(RF_ERR_INVALID_ARG, "genome has no final xform"); x = &f->g.final_xf; }
    else if (xi < (int)f->g.xforms.size()) x = &f->g.xforms[xi];
    else return fail(RF_ERR_INVALID_ARG, "xform index out of range");
    Xform before = *x;
    std::string n = name;
    if (n == "weight") x->weight = v;
    else if (n == "color") x->color = v;
    else if (n == "color_speed") x->color_speed = v;
    else if (n == "opacity") x->opacity = v;
    else if (n == "animate") x->rotation_frequency = v > 0 ? 1.0f : 0.0f;
    else if (n.size() == 6 && n.compare(0, 5, "coefs") == 0 && n[5] >= '0' && n[5] <= '5') x->affine[n[5] - '0'] = v;
    else if (n.size() == 5 && n.compare(0, 4, "post") == 0 && n[4] >= '0' && n[4] <= '5') {
        if (!x->has_post) { x->has_post = true; float id[6] = {1, 0, 0, 1, 0, 0}; memcpy(x->post, id, sizeof id); }
        x->post[n[4] - '0'] = v;
    } else if (f->reg->param_owner.count(n)) x->params[n] = v;
    else if (f->reg->vars.count(n)) x->vars[n] = v;
    else return fail(RF_ERR_UNKNOWN_NAME, "unknown xform field " + n);
    if (int rc = genome_validate(f->g, *f->reg)) { *x = before; return rc; }
    f->version++;
    return RF_OK;
}

int rf_flame_param_buffer(const rf_flame* f, float* out, size_t cap, size_t* count) {
    if (!f) return fail(RF_ERR_INVALID_ARG, "rf_flame_param_buffer: null flame");
    std::vector<float> buf;
    if (int rc = genome_param_buffer(f->g, buf, nullptr)) return rc;
    if (out) memcpy(out, buf.data(), std::min(cap, buf.size()) * sizeof(float));
    if (count) *count = buf.size();
    return RF_OK;
}

int rf_flame_param_layout(const rf_flame* f, char* out, size_t cap, size_t* needed) {
    if (!f) return fail(RF_ERR_INVALID_ARG, "rf_flame_param_layout: null flame");
    std::vector<float> buf;
    std::string js;
    genome_param_buffer(f->g, buf, &js);
    size_t n = copy_out(js, out, cap);
    if (needed) *needed = n;
    return RF_OK;
}

int rf_flame_screen_affine(const rf_flame* f, uint32_t w, uint32_t h, float out6[6]) {
    if (!f || !out6) return fail(RF_ERR_INVALID_ARG, "rf_flame_screen_affine: null argument");
    if (f->g.size[1] == 0) return fail(RF_ERR_INVALID_ARG, "genome size is zero");
    genome_screen_affine(f->g, w, h, out6);
    return RF_OK;
}

int rf_flame_xform_draws(const rf_flame* f, int xi) {
    if (!f) return -1;
    return genome_xform_draws(f->g, *f->reg, xi);
}

// ---------------------------------------------------------------------------------------------
// simulation
// ---------------------------------------------------------------------------------------------
int rf_sim_create(const rf_sim_desc* d, rf_sim** out) {
    if (!d || !out) return fail(RF_ERR_INVALID_ARG, "rf_sim_create: null argument");
    *out = nullptr;
    const uint32_t slots = d->cta_slots ? d->cta_slots : 4096;
    const uint32_t threads = d->cta_threads ? d->cta_threads : std::min<uint32_t>(slots, 1024);
    const uint32_t T = d->temporal_samples ? d->temporal_samples : 1;
    if (!chaos_shape_supported((int)threads, (int)slots))
        return fail(RF_ERR_INVALID_ARG, "cta_slots / cta_threads: 256x256, 512x512, 1024 or 2048 slots on 512 threads, "
                                        "1024, 2048 or 4096 slots on 1024 threads");
    if (d->walkers == 0 || d->walkers % T) return fail(RF_ERR_INVALID_ARG, "walkers must be a positive multiple of temporal_samples");
    const uint64_t ppts = d->walkers / T;
    if (ppts % slots) return fail(RF_ERR_INVALID_ARG, "walkers per temporal sample must be a multiple of cta_slots");
    if (ppts > 0x7fffffffull) return fail(RF_ERR_CAPACITY, "too many walkers per temporal sample");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RF_ERR_NO_DEVICE, "no CUDA device");
    if (d->device < 0 || d->device >= ndev) return fail(RF_ERR_INVALID_ARG, "device ordinal out of range");
    auto* s = new rf_sim();
    s->d = *d;
    s->device = d->device;
    s->N = d->walkers;
    s->T = T;
    s->ppts = (uint32_t)ppts;
    s->slots = slots;
    s->threads = threads;
    s->L = d->steps_per_launch ? std::min<uint32_t>(d->steps_per_launch, 256) : 256;
    s->table_size = d->shuffle_count ? d->shuffle_count : 1024;
    auto cleanup = [&](int rc) { rf_sim_destroy(s); return rc; };
    if (int rc = set_device(s)) { delete s; return rc; }
    cudaError_t e;
#define ALLOC(ptr, bytes) \
    if ((e = cudaMalloc((void**)&(ptr), (bytes))) != cudaSuccess) return cleanup(cuda_fail(e, "cudaMalloc"));
    ALLOC(s->walk[0], s->N * sizeof(float4));
    ALLOC(s->walk[1], s->N * sizeof(float4));
    ALLOC(s->rng, s->N * sizeof(uint4));
    ALLOC(s->table, (size_t)s->table_size * slots * sizeof(uint16_t));
    ALLOC(s->base_prog, kProgMaxWords * sizeof(uint32_t));
    s->prog_stride = kProgMaxWords;
    ALLOC(s->progs, (size_t)T * s->prog_stride * sizeof(uint32_t));
    ALLOC(s->palette, 256 * sizeof(float4));
    ALLOC(s->counters, 8 * sizeof(unsigned long long));
#undef ALLOC
    if ((e = launch_init_rng(s->rng, s->N, d->seed, s->stream)) != cudaSuccess) return cleanup(cuda_fail(e, "rng init"));
    // the pipelined exchange's permutations, for 4 slots per thread
    s->table_phases = slots / threads >= 3 ? slots / threads : 0;
    if ((e = launch_shuffle_table(s->table, slots, s->table_size, d->seed, s->stream, s->table_phases)) != cudaSuccess)
        return cleanup(cuda_fail(e, "shuffle table"));
    if ((e = cudaMemsetAsync(s->counters, 0, 8 * sizeof(unsigned long long), s->stream)) != cudaSuccess)
        return cleanup(cuda_fail(e, "memset"));
    for (auto& ev : s->tune_ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cleanup(cuda_fail(e, "event"));
    for (auto& ev : s->tile_ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cleanup(cuda_fail(e, "event"));
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cleanup(cuda_fail(e, "sim init"));
    *out = s;
    return RF_OK;
}

int rf_sim_destroy(rf_sim* s) {
    if (!s) return RF_OK;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    void* ptrs[] = {s->rec, s->walk[0], s->walk[1], s->rng, s->table, s->base_prog, s->progs, s->palette, s->counters,
                    s->trace, s->r_bins, s->r_hits, s->r_de, s->r_img, s->r_stats, s->r_rad, s->r_dw};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto ev : s->tune_ev)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : s->tile_ev)
        if (ev) cudaEventDestroy(ev);
    delete s;
    return RF_OK;
}

int rf_sim_set_stream(rf_sim* s, void* stream) {
    if (!s) return fail(RF_ERR_INVALID_ARG, "rf_sim_set_stream: null sim");
    s->stream = (cudaStream_t)stream;
    return RF_OK;
}

int rf_sim_enable_xid_trace(rf_sim* s, uint32_t max_passes) {
    if (!s) return fail(RF_ERR_INVALID_ARG, "rf_sim_enable_xid_trace: null sim");
    if (int rc = set_device(s)) return rc;
    if (s->trace) { cudaFree(s->trace); s->trace = nullptr; s->trace_passes = 0; }
    if (max_passes == 0) return RF_OK;
    const size_t bytes = (size_t)max_passes * (s->N / kGroup);
    RF_CUDA(cudaMalloc((void**)&s->trace, bytes));
    RF_CUDA(cudaMemsetAsync(s->trace, 0xff, bytes, s->stream));
    s->trace_passes = max_passes;
    return RF_OK;
}

int rf_sim_read_xid_trace(rf_sim* s, uint8_t* out, size_t cap, uint32_t* passes) {
    if (!s || !s->trace) return fail(RF_ERR_INVALID_ARG, "xid trace not enabled");
    if (int rc = set_device(s)) return rc;
    const size_t bytes = std::min(cap, (size_t)s->trace_passes * (s->N / kGroup));
    RF_CUDA(cudaStreamSynchronize(s->stream));
    RF_CUDA(cudaMemcpy(out, s->trace, bytes, cudaMemcpyDeviceToHost));
    if (passes) *passes = std::min(s->pass, s->trace_passes);
    return RF_OK;
}

int rf_needs_warmup(const rf_sim* s, const rf_flame* f) {
    if (!s || !f) return 1;
    return (s->warmed_uid != f->uid || s->warmed_version != f->version) ? 1 : 0;
}

int rf_warmup(rf_sim* s, rf_flame* f, uint32_t num_passes, float tss_width) {
    if (!s || !f) return fail(RF_ERR_INVALID_ARG, "rf_warmup: null argument");
    if (int rc = set_device(s)) return rc;
    std::vector<uint32_t> prog;
    if (int rc = genome_program(f->g, *f->reg, prog)) return rc;
    if (int rc = genome_validate(f->g, *f->reg)) return rc;
    s->prog_words = (uint32_t)prog.size();
    s->spec = nullptr;
    if (prog != s->spec_prog) {
        reset_exchange_tuning(s);
        s->auto_tile_state = 0;
    }
    if (s->d.specialize >= 0) {
        const void* k = nullptr;
        const int pipe = s->exchange != RF_EXCHANGE_BARRIER && use_pipe(s, 0) ? 1 : 0;
        const int rc = spec_kernel(prog, (int)s->threads, (int)s->slots, s->device, &k, SpecKind::Chaos,
                                   splat_code(s->splat), s->reset, pipe);
        if (rc == RF_OK) {
            s->spec = k;
            s->spec_splat = splat_code(s->splat);
            s->spec_reset = s->reset;
            s->spec_pipe = pipe;
            s->spec_prog = prog;
        } else if (s->d.specialize > 0) {
            return rc;  // required
        }
    }
    RF_CUDA(cudaMemcpyAsync(s->base_prog, prog.data(), prog.size() * 4, cudaMemcpyHostToDevice, s->stream));
    RF_CUDA(launch_animate(s->base_prog, s->prog_words, s->T, tss_width, s->progs, s->prog_stride, s->stream));
    RF_CUDA(cudaMemcpyAsync(s->palette, f->g.palette, sizeof(f->g.palette), cudaMemcpyHostToDevice, s->stream));
    RF_CUDA(cudaMemsetAsync(s->counters, 0, 8 * sizeof(unsigned long long), s->stream));
    // the pageable uploads above complete before the call returns; keep the host copy alive
    RF_CUDA(cudaStreamSynchronize(s->stream));
    s->pass = 0;
    // flame::warmup: one first-run pass (sample points, jitter, random colours), then num_passes
    if (int rc = launch_passes(s, 1 + num_passes, true, false, nullptr, nullptr, 0, 0, nullptr)) return rc;
    s->warmed_uid = f->uid;
    s->warmed_version = f->version;
    return RF_OK;
}

int rf_sim_specialized(const rf_sim* s) { return s && s->spec ? 1 : 0; }

int rf_flame_kernel_source(const rf_flame* f, uint32_t cta_threads, uint32_t cta_slots, char* buf, size_t cap,
                           size_t* needed) {
    if (!f || !cta_threads || cta_slots % cta_threads) return fail(RF_ERR_INVALID_ARG, "rf_flame_kernel_source: bad arguments");
    std::vector<uint32_t> prog;
    if (int rc = genome_program(f->g, *f->reg, prog)) return rc;
    const std::string src = spec_source(prog, (int)cta_threads, (int)(cta_slots / cta_threads));
    if (needed) *needed = src.size() + 1;
    if (buf && cap) {
        const size_t n = std::min(cap - 1, src.size());
        memcpy(buf, src.data(), n);
        buf[n] = 0;
        if (n < src.size()) return fail(RF_ERR_CAPACITY, "rf_flame_kernel_source: buffer too small");
    }
    return RF_OK;
}

int rf_flame_kernel_compile(const rf_flame* f, uint32_t cta_threads, uint32_t cta_slots, size_t* cubin_bytes) {
    if (!f || !cta_threads || cta_slots % cta_threads) return fail(RF_ERR_INVALID_ARG, "rf_flame_kernel_compile: bad arguments");
    std::vector<uint32_t> prog;
    if (int rc = genome_program(f->g, *f->reg, prog)) return rc;
    std::vector<char> cubin;
    if (int rc = spec_compile(spec_source(prog, (int)cta_threads, (int)(cta_slots / cta_threads)), cubin)) return rc;
    if (cubin_bytes) *cubin_bytes = cubin.size();
    return RF_OK;
}

int rf_set_bin_layout(rf_sim* s, int layout) {
    if (!s || layout < RF_BINS_AUTO || layout > RF_BINS_INTERLEAVED) return fail(RF_ERR_INVALID_ARG, "rf_set_bin_layout: bad arguments");
    s->bin_layout = layout;
    return RF_OK;
}

int rf_set_splat(rf_sim* s, int splat) {
    if (!s) return fail(RF_ERR_INVALID_ARG, "rf_set_splat: null sim");
    if (splat != s->splat) reset_exchange_tuning(s);
    s->auto_tile_state = 0;
    s->splat = splat;
    return RF_OK;
}

int rf_set_splat_tile(rf_sim* s, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h) {
    if (!s) return fail(RF_ERR_INVALID_ARG, "rf_set_splat_tile: null sim");
    if ((uint64_t)w * h > 65536) return fail(RF_ERR_CAPACITY, "rf_set_splat_tile: more than 65,536 bins");
    reset_exchange_tuning(s);
    s->tile[0] = x0;
    s->tile[1] = y0;
    s->tile[2] = w;
    s->tile[3] = h;
    return RF_OK;
}

int rf_set_bad_value_reset(rf_sim* s, int on) {
    if (!s || (on != 0 && on != 1)) return fail(RF_ERR_INVALID_ARG, "rf_set_bad_value_reset: null sim or flag not 0/1");
    if (on != s->reset) reset_exchange_tuning(s);
    s->reset = on;
    return RF_OK;
}

int rf_set_exchange(rf_sim* s, int mode) {
    if (!s || mode < RF_EXCHANGE_BARRIER || mode > RF_EXCHANGE_AUTO)
        return fail(RF_ERR_INVALID_ARG, "rf_set_exchange: null sim or unknown mode");
    s->exchange = mode;
    reset_exchange_tuning(s);
    return RF_OK;
}

int rf_sim_splat_tile(rf_sim* s, uint32_t out[4]) {
    if (!s || !out) return -1;
    if (s->auto_tile_state == 4) {  // the timed tile launch: settle the decision
        if (set_device(s) != RF_OK || cudaStreamSynchronize(s->stream) != cudaSuccess) return -1;
        decide_auto_tile(s);
    }
    const uint32_t* t = s->splat == RF_SPLAT_TILE ? s->tile
                        : (s->splat == RF_SPLAT_AUTO && s->auto_tile_state == 1) ? s->auto_tile : nullptr;
    if (!t) return 0;
    memcpy(out, t, 4 * sizeof(uint32_t));
    return 1;
}

int rf_sim_exchange(const rf_sim* s) {
    if (!s) return -1;
    const uint32_t tile_bins = s->splat == RF_SPLAT_TILE                              ? s->tile[2] * s->tile[3]
                               : s->splat == RF_SPLAT_AUTO && s->auto_tile_state == 1 ? s->auto_tile[2] * s->auto_tile[3]
                                                                                      : 0u;
    if (!s->spec || !use_pipe(s, tile_bins)) return 0;
    if (s->exchange != RF_EXCHANGE_AUTO) return s->exchange == RF_EXCHANGE_PIPELINED ? 1 : 0;
    return s->tune_pipe;
}

int rf_draw_to_bins(rf_sim* s, rf_flame* f, float* bins_rgba, uint32_t* bins_hits, uint32_t W, uint32_t H,
                    uint32_t num_iter, uint64_t* drawn) {
    if (!s || !f || !bins_rgba) return fail(RF_ERR_INVALID_ARG, "rf_draw_to_bins: null argument");
    if (W == 0 || H == 0 || W > 65536 || H > 65536) return fail(RF_ERR_INVALID_ARG, "bin grid must be 1..65536 on each side");
    if ((uint64_t)W * H >= 0xffffffffull) return fail(RF_ERR_CAPACITY, "bin grid must hold fewer than 2^32 - 1 bins");
    if (rf_needs_warmup(s, f)) return fail(RF_ERR_NEEDS_WARMUP, "flame changed or not warmed up: call rf_warmup");
    if (f->g.size[1] == 0) return fail(RF_ERR_INVALID_ARG, "genome size is zero");
    if (((uintptr_t)bins_rgba) & 15) return fail(RF_ERR_INVALID_ARG, "bins_rgba must be 16-byte aligned");
    if (s->splat == RF_SPLAT_TILE && ((uint64_t)s->tile[0] + s->tile[2] > W || (uint64_t)s->tile[1] + s->tile[3] > H))
        return fail(RF_ERR_INVALID_ARG, "rf_draw_to_bins: the splat tile does not lie inside the bin grid");
    if (s->splat == RF_SPLAT_TILE && (uint64_t)W * H >= 0x80000000ull)
        return fail(RF_ERR_CAPACITY, "rf_draw_to_bins: the tile splat takes bin grids of fewer than 2^31 bins");
    if (int rc = set_device(s)) return rc;
    float ss[6];
    genome_screen_affine(f->g, W, H, ss);
    // [0] drawn, [1] emitted count this call
    RF_CUDA(cudaMemsetAsync(s->counters, 0, 2 * sizeof(unsigned long long), s->stream));
    if (int rc = draw_passes(s, num_iter, (float4*)bins_rgba, bins_hits, W, H, ss)) return rc;
    if (drawn) {
        unsigned long long c[1];
        RF_CUDA(cudaStreamSynchronize(s->stream));
        if (int rc = check_exchange(s)) return rc;
        RF_CUDA(cudaMemcpy(c, s->counters, sizeof c, cudaMemcpyDeviceToHost));
        *drawn = c[0];
    }
    return RF_OK;
}

int rf_sim_counters(rf_sim* s, uint64_t out[3]) {
    if (!s || !out) return fail(RF_ERR_INVALID_ARG, "rf_sim_counters: null argument");
    if (int rc = set_device(s)) return rc;
    unsigned long long c[3];
    RF_CUDA(cudaStreamSynchronize(s->stream));
    if (int rc = check_exchange(s)) return rc;
    RF_CUDA(cudaMemcpy(c, s->counters, sizeof c, cudaMemcpyDeviceToHost));
    for (int i = 0; i < 3; i++) out[i] = c[i];
    return RF_OK;
}

// ---------------------------------------------------------------------------------------------
// image passes
// ---------------------------------------------------------------------------------------------
int rf_density_estimate(const float* in, uint32_t w, uint32_t h, int radius, int min_radius, float curve, float* out,
                        void* stream) {
    if (!in || !out || w == 0 || h == 0) return fail(RF_ERR_INVALID_ARG, "rf_density_estimate: bad arguments");
    if (radius < 0 || radius > 100 || min_radius < 0 || min_radius > 100)
        return fail(RF_ERR_INVALID_ARG, "estimator radii must be within 0..100 (main.cpp:502)");
    if (in == out) return fail(RF_ERR_INVALID_ARG, "rf_density_estimate: in and out must differ");
    if (h > 65535) return fail(RF_ERR_CAPACITY, "rf_density_estimate: more than 65535 rows");
    RF_CUDA(launch_density((const float4*)in, w, h, radius, min_radius, curve, (float4*)out, (cudaStream_t)stream));
    return RF_OK;
}

int rf_tonemap_filter(const float* rgba, uint32_t w, uint32_t h, uint32_t ss, float radius, int shape, float gamma,
                      float brightness, float vibrancy, float k2, float* out_f32, uint8_t* out8, void* stream) {
    if (!(radius > 0.0f)) return rf_tonemap(rgba, w, h, ss, gamma, brightness, vibrancy, k2, out_f32, out8, stream);
    if (!rgba || w == 0 || h == 0 || ss == 0 || w % ss || h % ss)
        return fail(RF_ERR_INVALID_ARG, "rf_tonemap_filter: bad arguments (width and height must be multiples of ss)");
    if (shape < RF_FILTER_GAUSSIAN || shape > RF_FILTER_HERMITE) return fail(RF_ERR_INVALID_ARG, "unknown filter shape");
    float taps[kMaxFilterTaps];
    if (filter_taps(ss, radius, shape, taps) < 0)
        return fail(RF_ERR_CAPACITY, "rf_tonemap_filter: the filter window exceeds 64 bins");
    cudaStream_t st = (cudaStream_t)stream;
    double* stats = nullptr;
    if (!(k2 > 0.0f)) {
        RF_CUDA(cudaMallocAsync((void**)&stats, 3 * sizeof(double), st));
        cudaError_t e = launch_stats((const float4*)rgba, w, h, stats, st);
        if (e != cudaSuccess) { cudaFreeAsync(stats, st); return cuda_fail(e, "stats"); }
    }
    cudaError_t e = launch_tonemap_filter((const float4*)rgba, w, h, ss, radius, shape, gamma, brightness, vibrancy,
                                          k2, stats, (float4*)out_f32, (uchar4*)out8, st);
    if (stats) cudaFreeAsync(stats, st);
    if (e != cudaSuccess) return cuda_fail(e, "rf_tonemap_filter");
    return RF_OK;
}

int rf_density_tonemap(const float* in, uint32_t w, uint32_t h, int radius, int min_radius, float curve, uint32_t ss,
                       float gamma, float brightness, float vibrancy, float k2, float* out_f32, uint8_t* out8,
                       void* stream) {
    if (!in || w == 0 || h == 0 || ss == 0 || w % ss || h % ss)
        return fail(RF_ERR_INVALID_ARG, "rf_density_tonemap: bad arguments (width and height must be multiples of ss)");
    if (radius < 0 || radius > 100 || min_radius < 0 || min_radius > 100)
        return fail(RF_ERR_INVALID_ARG, "estimator radii must be within 0..100 (main.cpp:502)");
    if (h > 65535 || h / ss > 65535) return fail(RF_ERR_CAPACITY, "rf_density_tonemap: more than 65535 rows");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)w * h;
    std::vector<float> wts;
    density_weights(radius, min_radius, wts);
    const bool fused = density_tonemap_fused(radius, min_radius, ss);
    uint8_t* rad = nullptr;
    float* dw = nullptr;
    double* stats = nullptr;
    float4* de = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&rad, n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dw, wts.size() * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&stats, 3 * sizeof(double), st);
    if (e == cudaSuccess && !fused) e = cudaMallocAsync((void**)&de, n * sizeof(float4), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw, wts.data(), wts.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = launch_density_tonemap((const float4*)in, w, h, radius, min_radius, curve, ss, gamma, brightness, vibrancy,
                                   k2, (float4*)out_f32, (uchar4*)out8, rad, dw, stats, de, st);
    for (void* p : {(void*)rad, (void*)dw, (void*)stats, (void*)de})
        if (p) cudaFreeAsync(p, st);
    if (e != cudaSuccess) return cuda_fail(e, "rf_density_tonemap");
    return RF_OK;
}

int rf_hist_stats(const float* rgba, uint32_t w, uint32_t h, double* out3, void* stream) {
    if (!rgba || !out3) return fail(RF_ERR_INVALID_ARG, "rf_hist_stats: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    double* d = nullptr;
    RF_CUDA(cudaMallocAsync((void**)&d, 3 * sizeof(double), st));
    cudaError_t e = launch_stats((const float4*)rgba, w, h, d, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out3, d, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "rf_hist_stats");
    uint64_t nz;
    memcpy(&nz, &out3[2], 8);
    out3[2] = (double)nz;
    return RF_OK;
}

int rf_tonemap(const float* rgba, uint32_t w, uint32_t h, uint32_t ss, float gamma, float brightness, float vibrancy,
               float k2, float* out_f32, uint8_t* out8, void* stream) {
    if (!rgba || w == 0 || h == 0 || ss == 0 || w % ss || h % ss)
        return fail(RF_ERR_INVALID_ARG, "rf_tonemap: bad arguments (width and height must be multiples of ss)");
    cudaStream_t st = (cudaStream_t)stream;
    double* stats = nullptr;
    if (!(k2 > 0.0f)) {
        RF_CUDA(cudaMallocAsync((void**)&stats, 3 * sizeof(double), st));
        cudaError_t e = launch_stats((const float4*)rgba, w, h, stats, st);
        if (e != cudaSuccess) { cudaFreeAsync(stats, st); return cuda_fail(e, "stats"); }
    }
    cudaError_t e = launch_tonemap((const float4*)rgba, w, h, ss, gamma, brightness, vibrancy, k2, stats,
                                   (float4*)out_f32, (uchar4*)out8, st);
    if (stats) cudaFreeAsync(stats, st);
    if (e != cudaSuccess) return cuda_fail(e, "tonemap");
    return RF_OK;
}

int rf_shuffle_generate(uint32_t n, uint32_t count, uint64_t seed, uint16_t* out, void* stream) {
    if (!out || n == 0 || n > 65536 || count == 0) return fail(RF_ERR_INVALID_ARG, "rf_shuffle_generate: bad arguments");
    RF_CUDA(launch_shuffle_table(out, n, count, seed, (cudaStream_t)stream));
    return RF_OK;
}

int rf_probe_xform(rf_flame* f, int xform, uint32_t n, const float* in, uint32_t* rng, int first_run, float* out,
                   void* stream) {
    if (!f || !in || !rng || !out) return fail(RF_ERR_INVALID_ARG, "rf_probe_xform: null argument");
    if (xform >= (int)f->g.xforms.size() || (xform < 0 && !f->g.has_final))
        return fail(RF_ERR_INVALID_ARG, "xform index out of range");
    std::vector<uint32_t> prog;
    if (int rc = genome_program(f->g, *f->reg, prog)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* d = nullptr;
    RF_CUDA(cudaMallocAsync((void**)&d, prog.size() * 4, st));
    cudaError_t e = cudaMemcpyAsync(d, prog.data(), prog.size() * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n) e = launch_probe(d, xform, n, in, rng, first_run, out, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "rf_probe_xform");
    return RF_OK;
}

// ---------------------------------------------------------------------------------------------
// end-to-end frame
// ---------------------------------------------------------------------------------------------
int rf_render(rf_sim* s, rf_flame* f, const rf_render_desc* d, uint8_t* out, double* stats) {
    if (!s || !f || !d || !out) return fail(RF_ERR_INVALID_ARG, "rf_render: null argument");
    const uint32_t ss = d->supersample ? d->supersample : 1;
    if (d->width == 0 || d->height == 0) return fail(RF_ERR_INVALID_ARG, "rf_render: empty image");
    if (f->g.size[1] == 0) return fail(RF_ERR_INVALID_ARG, "genome size is zero");
    if ((uint64_t)d->width * ss > 65536 || (uint64_t)d->height * ss > 65536)
        return fail(RF_ERR_INVALID_ARG, "rf_render: bin grid too large");
    const uint32_t W = d->width * ss, H = d->height * ss;
    if ((uint64_t)W * H >= 0xffffffffull)
        return fail(RF_ERR_INVALID_ARG, "rf_render: bin grid too large");
    if (int rc = set_device(s)) return rc;
    const size_t nb = (size_t)W * H, ni = (size_t)d->width * d->height;
    if (s->r_bins_n != nb) {
        cudaFree(s->r_bins); cudaFree(s->r_hits); cudaFree(s->r_de); cudaFree(s->r_rad);
        s->r_bins = nullptr; s->r_hits = nullptr; s->r_de = nullptr; s->r_rad = nullptr; s->r_bins_n = 0;
        RF_CUDA(cudaMalloc((void**)&s->r_bins, nb * sizeof(float4)));
        RF_CUDA(cudaMalloc((void**)&s->r_hits, nb * sizeof(uint32_t)));
        RF_CUDA(cudaMalloc((void**)&s->r_de, nb * sizeof(float4)));
        s->r_bins_n = nb;
    }
    if (s->r_img_n != ni) {
        cudaFree(s->r_img);
        s->r_img = nullptr; s->r_img_n = 0;
        RF_CUDA(cudaMalloc((void**)&s->r_img, ni * sizeof(uchar4)));
        s->r_img_n = ni;
    }
    if (!s->r_stats) RF_CUDA(cudaMalloc((void**)&s->r_stats, 4 * sizeof(double)));
    float ssa[6];
    genome_screen_affine(f->g, W, H, ssa);
    cudaEvent_t e0, e1;
    RF_CUDA(cudaEventCreate(&e0));
    RF_CUDA(cudaEventCreate(&e1));
    auto done = [&](int rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; };
    if (cudaEventRecord(e0, s->stream) != cudaSuccess) return done(fail(RF_ERR_CUDA, "event record"));
    // fuse_passes counts every discarded pass, the first-run pass included
    if (int rc = rf_warmup(s, f, d->fuse_passes ? d->fuse_passes - 1 : 0, d->tss_width)) return done(rc);
    const uint64_t passes1 = (d->points + s->N - 1) / s->N;  // passes of one walker-step per point
    if (passes1 > 0xffffffffull / 16) return done(fail(RF_ERR_CAPACITY, "rf_render: too many passes"));
    cudaError_t e = cudaMemsetAsync(s->r_bins, 0, nb * sizeof(float4), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->r_hits, 0, nb * sizeof(uint32_t), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->counters, 0, 2 * sizeof(unsigned long long), s->stream);
    if (e != cudaSuccess) return done(cuda_fail(e, "rf_render clear"));
    uint64_t passes = passes1;
    if (int rc = draw_passes(s, (uint32_t)passes1, s->r_bins, s->r_hits, W, H, ssa)) return done(rc);
    if (d->stop_on_binned) {
        // main.cpp:411-412: keep drawing while the binned count is below the target.  Each round
        // reads the count back and draws the passes the measured binned-per-pass rate predicts
        // for the rest (at least one), up to 16x the first round.
        for (;;) {
            unsigned long long got = 0;
            e = cudaMemcpyAsync(&got, s->counters, sizeof got, cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) return done(cuda_fail(e, "rf_render binned count"));
            if (got >= d->points || passes >= 16 * passes1) break;
            const double rate = (double)got / (double)passes;  // points binned per pass
            uint64_t more = rate > 0.0 ? (uint64_t)std::ceil((double)(d->points - got) / rate) : passes1;
            more = std::max<uint64_t>(1, std::min<uint64_t>(more, 16 * passes1 - passes));
            if (int rc = draw_passes(s, (uint32_t)more, s->r_bins, s->r_hits, W, H, ssa)) return done(rc);
            passes += more;
        }
    }
    const bool flam3_filter = f->g.filter > 0.0f && ss > 1;
    if (flam3_filter) {
        // the genome's flam3 spatial filter over the supersampled (density-estimated) bins
        float taps[kMaxFilterTaps];
        if (filter_taps(ss, f->g.filter, f->g.filter_shape, taps) < 0)
            return done(fail(RF_ERR_CAPACITY, "rf_render: the genome's filter window exceeds 64 bins"));
        const float4* src = s->r_bins;
        if (d->density_estimation && (f->g.est_radius > 0 || f->g.est_min > 0)) {
            e = launch_density(s->r_bins, W, H, std::min(100, f->g.est_radius), std::min(100, f->g.est_min),
                               f->g.est_curve, s->r_de, s->stream);
            if (e != cudaSuccess) return done(cuda_fail(e, "density estimation"));
            src = s->r_de;
        }
        if (!(d->k2 > 0.0f)) e = launch_stats(src, W, H, s->r_stats, s->stream);
        if (e == cudaSuccess)
            e = launch_tonemap_filter(src, W, H, ss, f->g.filter, f->g.filter_shape, f->g.gamma, f->g.brightness,
                                      f->g.vibrancy, d->k2, d->k2 > 0.0f ? nullptr : s->r_stats, nullptr, s->r_img,
                                      s->stream);
    } else if (d->density_estimation && (f->g.est_radius > 0 || f->g.est_min > 0)) {
        // main.cpp:490-535: density estimation and tonemap, the estimator's output kept on chip
        const int R = std::min(100, f->g.est_radius), mn = std::min(100, f->g.est_min);
        if (!s->r_rad) {
            e = cudaMalloc((void**)&s->r_rad, nb);
            if (e != cudaSuccess) return done(cuda_fail(e, "cudaMalloc"));
            s->r_rad_n = nb;
        }
        if (!s->r_dw) {  // every radius up to 100: the table is a prefix of itself for any R
            std::vector<float> wts;
            density_weights(100, 0, wts);
            e = cudaMalloc((void**)&s->r_dw, wts.size() * sizeof(float));
            if (e == cudaSuccess) e = cudaMemcpy(s->r_dw, wts.data(), wts.size() * sizeof(float), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return done(cuda_fail(e, "density weights"));
        }
        e = launch_density_tonemap(s->r_bins, W, H, R, mn, f->g.est_curve, ss, f->g.gamma, f->g.brightness,
                                   f->g.vibrancy, d->k2, nullptr, s->r_img, s->r_rad, s->r_dw, s->r_stats, s->r_de,
                                   s->stream);
    } else {
        const double* st = nullptr;
        if (!(d->k2 > 0.0f)) {
            e = launch_stats(s->r_bins, W, H, s->r_stats, s->stream);
            if (e != cudaSuccess) return done(cuda_fail(e, "stats"));
            st = s->r_stats;
        }
        e = launch_tonemap(s->r_bins, W, H, ss, f->g.gamma, f->g.brightness, f->g.vibrancy, d->k2, st, nullptr,
                           s->r_img, s->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, s->r_img, ni * sizeof(uchar4), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return done(cuda_fail(e, "rf_render"));
    if (int rc = check_exchange(s)) return done(rc);
    if (stats) {
        unsigned long long c[2];
        float ms = 0;
        cudaMemcpy(c, s->counters, sizeof c, cudaMemcpyDeviceToHost);
        cudaEventElapsedTime(&ms, e0, e1);
        stats[0] = (double)passes * (double)s->N;
        stats[1] = (double)c[0];
        stats[2] = ms;
    }
    return done(RF_OK);
}

// ---------------------------------------------------------------------------------------------
// PNG output (stored deflate blocks; no compression library needed)
// ---------------------------------------------------------------------------------------------
namespace {
uint32_t crc32_update(uint32_t c, const uint8_t* p, size_t n) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t v = i;
            for (int k = 0; k < 8; k++) v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
        init = true;
    }
    c ^= 0xffffffffu;
    for (size_t i = 0; i < n; i++) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xffffffffu;
}
void put_be32(std::string& s, uint32_t v) {
    s += (char)(v >> 24); s += (char)(v >> 16); s += (char)(v >> 8); s += (char)v;
}
void chunk(std::string& out, const char* type, const std::string& data) {
    put_be32(out, (uint32_t)data.size());
    std::string td = std::string(type, 4) + data;
    out += td;
    put_be32(out, crc32_update(0, (const uint8_t*)td.data(), td.size()));
}
}  // namespace

int rf_write_png(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h) {
    if (!path || !rgba8 || w == 0 || h == 0) return fail(RF_ERR_INVALID_ARG, "rf_write_png: bad arguments");
    std::string raw;
    raw.reserve((size_t)(w * 4 + 1) * h);
    for (uint32_t y = 0; y < h; y++) {
        raw += '\0';  // filter type 0
        raw.append((const char*)rgba8 + (size_t)y * w * 4, (size_t)w * 4);
    }
    std::string z = "\x78\x01";
    uint32_t a = 1, b = 0;
    for (unsigned char ch : raw) { a = (a + ch) % 65521; b = (b + a) % 65521; }
    for (size_t p = 0; p < raw.size() || p == 0; p += 65535) {
        size_t n = std::min<size_t>(65535, raw.size() - p);
        bool last = p + n >= raw.size();
        z += (char)(last ? 1 : 0);
        z += (char)(n & 0xff); z += (char)(n >> 8);
        z += (char)(~n & 0xff); z += (char)((~n >> 8) & 0xff);
        z.append(raw, p, n);
        if (last) break;
    }
    put_be32(z, (b << 16) | a);
    std::string png = "\x89PNG\r\n\x1a\n";
    std::string ihdr;
    put_be32(ihdr, w); put_be32(ihdr, h);
    ihdr += (char)8; ihdr += (char)6; ihdr += (char)0; ihdr += (char)0; ihdr += (char)0;
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", "");
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(RF_ERR_IO, std::string("cannot write ") + path);
    f.write(png.data(), (std::streamsize)png.size());
    return f ? RF_OK : fail(RF_ERR_IO, std::string("write failed: ") + path);
}

}  // extern "C"
