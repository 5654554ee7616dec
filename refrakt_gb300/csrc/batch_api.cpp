// Batched rendering (no reference counterpart): many genomes — animation frames and independent
// genomes with different xform counts and bin grids — in one persistent chaos launch driven by a
// work queue, followed by per-genome density estimation and tonemap, the whole sequence
// captured once in a CUDA graph and replayed.
//
// An autotuner picks the work-unit shape: the walkers per unit (1024, 2048 or 4096 — the walker
// shuffle's mixing domain) by timing a short probe batch of the actual genomes on each shape and
// weighting throughput by the shape's statistical efficiency, and the drawing passes per unit
// that finish the batch first on the persistent CTAs (simulated longest-first), counting each
// unit's fuse passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <map>
#include <mutex>
#include <queue>
#include <string>
#include <cstring>
#include <vector>

#include "batch.h"
#include "specialize.h"
#include "denoise_ops.h"
#include "handles.h"
#include "kernels.h"

using namespace rfk;

namespace {

struct Item {
    rf_batch_item desc;
    std::vector<uint32_t> prog;
    uint32_t W = 0, H = 0, ss = 1;
    float4* bins = nullptr;
    uint32_t* hits = nullptr;
    float4* de = nullptr;
    uchar4* img = nullptr;
    float4* img_f32 = nullptr;  // FP32 tonemapped image (rf_batch_desc.image_f32)
    float4* palette = nullptr;
    uint32_t* dprog = nullptr;
    uint32_t splat = 0;       // warp-aggregated splat for this genome
    int group = -1;           // specialised launch group (-1: the interpreted launch)
    std::string structure;    // genome structure (specialisation key)
    uint8_t* rad = nullptr;   // density estimation: a radius byte per bin
    float* dw = nullptr;      // density estimation: kernel weights of every radius
    uint64_t passes = 0;  // drawing passes of SLOTS walkers the item needs
    int est_radius = 0, est_min = 0;
    float est_curve = 0, gamma = 0, brightness = 0, vibrancy = 0;
};

constexpr uint64_t kUnitSeedStride = 0x9e3779b97f4a7c15ull;  // unit u of an item: seed + u * stride
constexpr uint64_t kTableSeed = 0x5eed;                      // shared table: keyed by kTableSeed + slots
constexpr uint32_t kSpecMinUnitsPerSM = 2;  // a structure gets a persistent launch from 2 units per SM
constexpr unsigned kCompileThreads = 16;    // run-time compilations in parallel
constexpr double kCompactShare = 16.0;  // probe points sharing a point's bin above this: compact attractor

// unit shape (walkers per unit) chosen per device and set of genome structures
std::mutex g_shape_mu;
std::map<std::string, uint32_t> g_shape_cache;

// Histogram L1 noise of a mixing domain relative to the reference's global shuffle, measured on
// the CPU oracle (tests/test_oracle_self.py): variance grows with its square.
double mixing_efficiency(uint32_t slots) {
    const double l1 = slots >= 4096 ? 1.00 : slots >= 2048 ? 1.05 : 1.20;
    return 1.0 / (l1 * l1);
}

}  // namespace

struct SpecGroup {  // units of one genome structure, drawn by its specialised persistent kernel
    const void* kernel = nullptr;
    int grid = 0;
    uint32_t first = 0, count = 0;
};

struct rf_batch {
    int device = 0;
    std::vector<SpecGroup> groups;
    uint32_t interp_first = 0, interp_count = 0;
    cudaStream_t stream = nullptr;
    rf_batch_desc d{};
    std::vector<Item> items;
    uint32_t threads = 1024, slots = 4096, unit_passes = 0, fuse = 20;
    uint16_t* table = nullptr;
    uint32_t table_size = 1024;
    BatchInstance* dinst = nullptr;
    BatchUnit* dunits = nullptr;
    uint32_t n_units = 0;
    unsigned int* queue = nullptr;
    unsigned long long* counters = nullptr;
    uint32_t max_prog_words = 0;
    double* stats = nullptr;  // per item 3 doubles
    unsigned char* pool = nullptr;  // every item's buffers (rf_batch_create)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the persistent launches after the first run on their own streams, forked from and joined to
    // `stream`: a launch's CTAs take the SMs the previous launch's finished CTAs leave
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> fork_join;  // [0] fork, [1 + k] join of aux[k]
    uint64_t points = 0;
};

namespace {

void destroy_batch(rf_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    void* ptrs[] = {b->pool, b->table, b->dinst, b->dunits, b->queue, b->counters, b->stats};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    for (auto ev : b->fork_join)
        if (ev) cudaEventDestroy(ev);
    for (auto s : b->aux)
        if (s) cudaStreamDestroy(s);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int cuda_err(cudaError_t e, const char* what) {
    return fail(RF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Passes until the last CTA finishes when unit_passes = per cuts every item's drawing passes
// into equal units (as build_tables does), each also running the fuse passes, and `ctas`
// persistent CTAs take them longest first (each the next unit when it finishes its own).
double unit_makespan(const std::vector<uint64_t>& need, uint64_t per, uint32_t fuse, int ctas) {
    std::vector<uint64_t> len;
    for (uint64_t nd : need) {
        const uint64_t nu = std::max<uint64_t>(1, (nd + per - 1) / per), u = (nd + nu - 1) / nu;
        for (uint64_t i = 0; i < nu; i++) len.push_back(u + fuse);
    }
    std::sort(len.rbegin(), len.rend());
    std::priority_queue<uint64_t, std::vector<uint64_t>, std::greater<uint64_t>> load;
    for (int i = 0; i < std::max(1, ctas); i++) load.push(0);
    uint64_t last = 0;
    for (uint64_t l : len) {
        const uint64_t t = load.top() + l;
        load.pop();
        load.push(t);
        last = std::max(last, t);
    }
    return (double)last;
}

// Builds the instance and unit tables for a shape; `probe_passes` > 0 builds an autotuner probe
// instead (one unit per item, `probe_fuse` then `probe_passes` passes).
int build_tables(rf_batch* b, uint32_t slots, uint32_t unit_passes, uint32_t probe_passes, uint32_t max_items,
                 uint32_t probe_fuse = 0) {
    std::vector<BatchInstance> inst;
    std::vector<BatchUnit> units;
    const size_t n = std::min<size_t>(b->items.size(), max_items);
    for (size_t i = 0; i < n; i++) {
        Item& it = b->items[i];
        BatchInstance I{};
        I.prog = it.dprog;
        I.prog_words = (uint32_t)it.prog.size();
        I.fuse = probe_passes ? probe_fuse : b->fuse;
        I.palette = it.palette;
        I.bins = it.bins;
        I.hits = it.hits;
        I.W = it.W;
        I.H = it.H;
        I.splat = it.splat;
        I.reset = b->d.bad_value_reset ? 1u : 0u;
        genome_screen_affine(b->items[i].desc.flame->g, it.W, it.H, I.ss);
        inst.push_back(I);
        if (probe_passes) {
            units.push_back(BatchUnit{(uint32_t)i, probe_passes, it.desc.seed});
            continue;
        }
        const uint64_t need = (it.desc.points + slots - 1) / slots;  // drawing passes of `slots` walkers
        const uint64_t nu = std::max<uint64_t>(1, (need + unit_passes - 1) / unit_passes);
        const uint64_t per = (need + nu - 1) / nu;
        for (uint64_t u = 0; u < nu; u++)
            units.push_back(BatchUnit{(uint32_t)i, (uint32_t)per, it.desc.seed + u * kUnitSeedStride});
        it.passes = per * nu;
    }
    // by launch group (specialised groups in order, the interpreted launch last), then longest
    // units first, instances interleaved, so each queue's tail is short
    auto rank = [&](const BatchUnit& u) {
        const int g = probe_passes ? -1 : b->items[u.instance].group;
        return g < 0 ? (int)b->groups.size() : g;
    };
    std::stable_sort(units.begin(), units.end(), [&](const BatchUnit& x, const BatchUnit& y) {
        const int rx = rank(x), ry = rank(y);
        return rx != ry ? rx < ry : x.draw > y.draw;
    });
    if (!probe_passes) {
        for (auto& g : b->groups) g.count = 0;
        b->interp_count = 0;
        for (const BatchUnit& u : units) {
            const int g = b->items[u.instance].group;
            if (g < 0) b->interp_count++;
            else b->groups[g].count++;
        }
        uint32_t f = 0;
        for (auto& g : b->groups) { g.first = f; f += g.count; }
        b->interp_first = f;
    }
    cudaFree(b->dinst);
    cudaFree(b->dunits);
    b->dinst = nullptr;
    b->dunits = nullptr;
    cudaError_t e = cudaMalloc((void**)&b->dinst, inst.size() * sizeof(BatchInstance));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->dunits, units.size() * sizeof(BatchUnit));
    if (e == cudaSuccess) e = cudaMemcpy(b->dinst, inst.data(), inst.size() * sizeof(BatchInstance), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->dunits, units.data(), units.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_err(e, "batch tables");
    b->n_units = (uint32_t)units.size();
    return RF_OK;
}

int make_table(rf_batch* b, uint32_t slots) {
    cudaFree(b->table);
    b->table = nullptr;
    cudaError_t e = cudaMalloc((void**)&b->table, (size_t)b->table_size * slots * sizeof(uint16_t));
    if (e == cudaSuccess) e = launch_shuffle_table(b->table, slots, b->table_size, kTableSeed + slots, b->stream);
    if (e != cudaSuccess) return cuda_err(e, "batch shuffle table");
    return RF_OK;
}

BatchArgs args_for(rf_batch* b, uint32_t first = 0, uint32_t count = ~0u, uint32_t queue = 0) {
    BatchArgs a{};
    a.inst = b->dinst;
    a.units = b->dunits + first;
    a.n_units = count == ~0u ? b->n_units : count;
    a.queue = b->queue + queue;
    a.table = b->table;
    a.table_size = b->table_size;
    a.max_prog_words = b->max_prog_words;
    a.counters = b->counters;
    return a;
}

// the whole batch on b->stream: clear, persistent chaos launch, per-item DE and tonemap
int enqueue(rf_batch* b) {
    cudaStream_t st = b->stream;
    cudaError_t e = cudaMemsetAsync(b->queue, 0, (b->groups.size() + 1) * sizeof(unsigned int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->counters, 0, 3 * sizeof(unsigned long long), st);
    for (auto& it : b->items) {
        if (e != cudaSuccess) break;
        const size_t nb = (size_t)it.W * it.H;
        e = cudaMemsetAsync(it.bins, 0, nb * sizeof(float4), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(it.hits, 0, nb * sizeof(uint32_t), st);
    }
    if (e != cudaSuccess) return cuda_err(e, "batch clear");
    // the persistent launches: the first on `st`, each further one on an auxiliary stream forked
    // after the clears, all joined before the image passes
    std::vector<int> launches;  // group index, or groups.size() for the interpreted launch
    for (size_t g = 0; g < b->groups.size(); g++)
        if (b->groups[g].count) launches.push_back((int)g);
    if (b->interp_count) launches.push_back((int)b->groups.size());
    const size_t extra = launches.empty() ? 0 : launches.size() - 1;
    while (e == cudaSuccess && b->aux.size() < extra) {
        cudaStream_t s2 = nullptr;
        e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
        if (e == cudaSuccess) b->aux.push_back(s2);
    }
    while (e == cudaSuccess && b->fork_join.size() < extra + 1) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) b->fork_join.push_back(ev);
    }
    if (e == cudaSuccess && extra) e = cudaEventRecord(b->fork_join[0], st);
    for (size_t k = 0; k < launches.size() && e == cudaSuccess; k++) {
        cudaStream_t ls = k ? b->aux[k - 1] : st;
        if (k) e = cudaStreamWaitEvent(ls, b->fork_join[0], 0);
        const int g = launches[k];
        if (e != cudaSuccess) break;
        if (g < (int)b->groups.size()) {
            const SpecGroup& G = b->groups[g];
            e = launch_batch_spec(G.kernel, (int)b->threads, (int)b->slots, G.grid,
                                  args_for(b, G.first, G.count, (uint32_t)g), ls);
        } else {
            e = launch_batch((int)b->threads, (int)b->slots,
                             args_for(b, b->interp_first, b->interp_count, (uint32_t)b->groups.size()), ls, nullptr);
        }
        if (e == cudaSuccess && k) e = cudaEventRecord(b->fork_join[k], ls);
    }
    for (size_t k = 1; k < launches.size() && e == cudaSuccess; k++) e = cudaStreamWaitEvent(st, b->fork_join[k], 0);
    if (e != cudaSuccess) return cuda_err(e, "batch kernel");
    for (size_t i = 0; i < b->items.size(); i++) {
        Item& it = b->items[i];
        if (it.de) {  // density estimation and tonemap, the estimator's output kept on chip where it fits
            e = launch_density_tonemap(it.bins, it.W, it.H, std::min(100, it.est_radius), std::min(100, it.est_min),
                                       it.est_curve, it.ss, it.gamma, it.brightness, it.vibrancy, b->d.k2, it.img_f32,
                                       it.img, it.rad, it.dw, b->stats + 3 * i, it.de, st);
            if (e != cudaSuccess) return cuda_err(e, "batch density estimation and tonemap");
            continue;
        }
        const double* stt = nullptr;
        if (!(b->d.k2 > 0.0f)) {
            e = launch_stats(it.bins, it.W, it.H, b->stats + 3 * i, st);
            if (e != cudaSuccess) return cuda_err(e, "batch stats");
            stt = b->stats + 3 * i;
        }
        e = launch_tonemap(it.bins, it.W, it.H, it.ss, it.gamma, it.brightness, it.vibrancy, b->d.k2, stt, it.img_f32,
                           it.img, st);
        if (e != cudaSuccess) return cuda_err(e, "batch tonemap");
    }
    return RF_OK;
}

}  // namespace

extern "C" {

int rf_batch_create(const rf_batch_item* items, uint32_t n, const rf_batch_desc* d, rf_batch** out) {
    if (!items || !n || !d || !out) return fail(RF_ERR_INVALID_ARG, "rf_batch_create: bad arguments");
    *out = nullptr;
    for (uint32_t i = 0; i < n; i++) {
        const rf_flame* f = items[i].flame;
        if (!f || !items[i].width || !items[i].height || !items[i].points)
            return fail(RF_ERR_INVALID_ARG, "rf_batch_create: item without genome, size or points");
        if (f->g.size[1] == 0) return fail(RF_ERR_INVALID_ARG, "rf_batch_create: genome size is zero");
        const uint32_t ss = items[i].supersample ? items[i].supersample : 1;
        if ((uint64_t)items[i].width * ss > 65536 || (uint64_t)items[i].height * ss > 65536 ||
            (uint64_t)items[i].width * ss * items[i].height * ss >= 0xffffffffull)
            return fail(RF_ERR_INVALID_ARG, "rf_batch_create: bin grid too large");
    }
    if (d->cta_slots && d->cta_slots != 1024 && d->cta_slots != 2048 && d->cta_slots != 4096)
        return fail(RF_ERR_INVALID_ARG, "rf_batch_desc.cta_slots must be 0, 1024, 2048 or 4096");
    auto* b = new rf_batch();
    b->d = *d;
    b->device = d->device;
    b->fuse = d->fuse_passes ? d->fuse_passes : 20;
    auto bail = [&](int rc) { destroy_batch(b); return rc; };
    if (cudaSetDevice(b->device) != cudaSuccess) return bail(fail(RF_ERR_NO_DEVICE, "rf_batch_create: no such device"));
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_err(e, "stream"));
    // Every item's device buffers are carved from one allocation: its small constants (palette,
    // program, DE kernel weights) packed at the start and uploaded with one copy, then the bin
    // planes, DE buffers and images, each 256-byte aligned.
    struct Offsets {
        size_t pal, prog, dw, bins, hits, de, rad, img, img_f32;
    };
    constexpr size_t kNone = ~(size_t)0;
    std::vector<Offsets> off(n);
    std::vector<uint8_t> consts;
    const auto put = [&](const void* src, size_t bytes) {
        const size_t o = consts.size();
        consts.resize(o + ((bytes + 255) & ~(size_t)255), 0);
        memcpy(consts.data() + o, src, bytes);
        return o;
    };
    b->items.reserve(n);
    for (uint32_t i = 0; i < n; i++) {
        const rf_flame* f = items[i].flame;
        b->items.emplace_back();
        Item& it = b->items.back();
        it.desc = items[i];
        it.ss = items[i].supersample ? items[i].supersample : 1;
        it.W = items[i].width * it.ss;
        it.H = items[i].height * it.ss;
        if (int rc = genome_program(f->g, *f->reg, it.prog)) return bail(rc);
        it.est_radius = f->g.est_radius; it.est_min = f->g.est_min; it.est_curve = f->g.est_curve;
        it.gamma = f->g.gamma; it.brightness = f->g.brightness; it.vibrancy = f->g.vibrancy;
        off[i].pal = put(f->g.palette, 256 * sizeof(float4));
        off[i].prog = put(it.prog.data(), it.prog.size() * 4);
        off[i].dw = kNone;
        if (d->density_estimation && (it.est_radius > 0 || it.est_min > 0)) {
            std::vector<float> wts;
            density_weights(std::min(100, it.est_radius), std::min(100, it.est_min), wts);
            off[i].dw = put(wts.data(), wts.size() * sizeof(float));
        }
        b->max_prog_words = std::max(b->max_prog_words, (uint32_t)it.prog.size());
        b->points += items[i].points;
    }
    size_t pool = consts.size();
    const auto take = [&](size_t bytes) {
        const size_t o = pool;
        pool += (bytes + 255) & ~(size_t)255;
        return o;
    };
    for (uint32_t i = 0; i < n; i++) {
        const Item& it = b->items[i];
        const size_t nb = (size_t)it.W * it.H, np = (size_t)items[i].width * items[i].height;
        off[i].bins = take(nb * sizeof(float4));
        off[i].hits = take(nb * sizeof(uint32_t));
        off[i].de = off[i].dw != kNone ? take(nb * sizeof(float4)) : kNone;
        off[i].rad = off[i].dw != kNone ? take(nb) : kNone;
        off[i].img = take(np * sizeof(uchar4));
        off[i].img_f32 = d->image_f32 ? take(np * sizeof(float4)) : kNone;
    }
    e = cudaMalloc((void**)&b->pool, pool);
    if (e == cudaSuccess) e = cudaMemcpy(b->pool, consts.data(), consts.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bail(cuda_err(e, "rf_batch_create allocation"));
    for (uint32_t i = 0; i < n; i++) {
        Item& it = b->items[i];
        unsigned char* base = b->pool;
        const auto at = [&](size_t o) -> void* { return o == kNone ? nullptr : base + o; };
        it.palette = static_cast<float4*>(at(off[i].pal));
        it.dprog = static_cast<uint32_t*>(at(off[i].prog));
        it.dw = static_cast<float*>(at(off[i].dw));
        it.bins = static_cast<float4*>(at(off[i].bins));
        it.hits = static_cast<uint32_t*>(at(off[i].hits));
        it.de = static_cast<float4*>(at(off[i].de));
        it.rad = static_cast<uint8_t*>(at(off[i].rad));
        it.img = static_cast<uchar4*>(at(off[i].img));
        it.img_f32 = static_cast<float4*>(at(off[i].img_f32));
    }
    e = cudaMalloc((void**)&b->queue, ((size_t)n + 1) * sizeof(unsigned int));  // a counter per group (<= items)
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->counters, 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->stats, 3 * sizeof(double) * n);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) return bail(cuda_err(e, "rf_batch_create"));

    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    // --- autotune the unit shape on a probe batch of the actual genomes; the choice is kept per
    // device and set of genome structures, so the frames of an animation probe once
    for (auto& it : b->items) it.structure = spec_structure(it.prog);
    std::string shape_key;
    {
        std::vector<std::string> st;
        for (auto& it : b->items) st.push_back(it.structure);
        std::sort(st.begin(), st.end());
        st.erase(std::unique(st.begin(), st.end()), st.end());
        shape_key = std::to_string(b->device);
        for (auto& x : st) shape_key += "|" + x;
    }
    std::vector<uint32_t> shapes = {1024, 2048, 4096};
    if (d->cta_slots) {
        shapes = {d->cta_slots};
    } else {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        auto hit = g_shape_cache.find(shape_key);
        if (hit != g_shape_cache.end()) shapes = {hit->second};
    }
    double best = -1.0;
    for (uint32_t slots : shapes) {
        if (shapes.size() == 1) { b->slots = slots; break; }
        if (int rc = make_table(b, slots)) return bail(rc);
        const uint32_t probe_items = std::min<uint32_t>(n, (uint32_t)sms);
        if (int rc = build_tables(b, slots, 0, 64, probe_items)) return bail(rc);
        b->slots = slots;
        cudaMemsetAsync(b->queue, 0, sizeof(unsigned int), b->stream);
        cudaMemsetAsync(b->counters, 0, 3 * sizeof(unsigned long long), b->stream);
        cudaEventRecord(b->ev0, b->stream);
        e = launch_batch(1024, (int)slots, args_for(b), b->stream, nullptr);
        cudaEventRecord(b->ev1, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return bail(cuda_err(e, "autotune probe"));
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        const double rate = (double)probe_items * slots * 64 / std::max(1e-3, (double)ms) * mixing_efficiency(slots);
        if (rate > best) { best = rate; b->slots = slots; }
    }
    b->threads = 1024;
    if (!d->cta_slots) {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        g_shape_cache[shape_key] = b->slots;
    }
    if (int rc = make_table(b, b->slots)) return bail(rc);
    // --- splat strategy per genome: a compact attractor (its 16-pass probe unit's points share
    // their bins with many others) takes the warp-aggregated reductions
    if (d->splat == RF_SPLAT_AUTO) {
        constexpr uint32_t kProbe = 16;
        for (auto& it : b->items) {
            const size_t nb = (size_t)it.W * it.H;
            e = cudaMemsetAsync(it.bins, 0, nb * sizeof(float4), b->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(it.hits, 0, nb * sizeof(uint32_t), b->stream);
            if (e != cudaSuccess) return bail(cuda_err(e, "splat probe"));
        }
        if (int rc = build_tables(b, b->slots, 0, kProbe, n, b->fuse)) return bail(rc);
        cudaMemsetAsync(b->queue, 0, sizeof(unsigned int), b->stream);
        e = launch_batch((int)b->threads, (int)b->slots, args_for(b), b->stream, nullptr);
        for (uint32_t i = 0; i < n && e == cudaSuccess; i++)
            e = launch_hit_moments(b->items[i].hits, b->items[i].W, b->items[i].H, b->stats + 3 * i, b->stream);
        std::vector<double> st(3 * (size_t)n);
        if (e == cudaSuccess) e = cudaMemcpyAsync(st.data(), b->stats, st.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return bail(cuda_err(e, "splat probe"));
        // sum h^2 / sum h = the mean count of the bin a probe point fell into: about 1 + points /
        // bins for a spread attractor, large where a warp's points pile into the same few bins
        for (uint32_t i = 0; i < n; i++)
            b->items[i].splat = st[3 * i + 1] >= kCompactShare * std::max(1.0, st[3 * i]) ? 1u : 0u;
    } else {
        for (auto& it : b->items) it.splat = d->splat == RF_SPLAT_WARP ? 1u : 0u;
    }
    // --- drawing passes per unit: the candidate whose units, taken longest first by the
    // persistent CTAs, finish first (a batch of few points wants one short unit per SM even at a
    // large fuse share; a large batch several units per CTA for balance); within 2 % the longer
    // units win (fewer fuse passes)
    std::vector<uint64_t> need;
    uint64_t total_passes = 0;
    for (auto& it : b->items) {
        need.push_back((it.desc.points + b->slots - 1) / b->slots);
        total_passes += need.back();
    }
    uint64_t per = d->unit_passes;
    if (per == 0) {
        std::vector<uint64_t> cands = {20ull * b->fuse};
        for (uint64_t k : {1, 2, 3, 4, 6, 8, 12, 16}) cands.push_back((total_passes + k * sms - 1) / (k * sms));
        double best_t = 0.0;
        for (uint64_t c : cands) {
            c = std::min<uint64_t>(std::max<uint64_t>(c, 1), 1u << 20);
            const double t = unit_makespan(need, c, b->fuse, sms);
            if (per == 0 || t < best_t * 0.98 || (t <= best_t * 1.02 && c > per)) {
                if (per == 0 || t < best_t) best_t = t;
                per = c;
            }
        }
    }
    per = std::min<uint64_t>(std::max<uint64_t>(per, 1), 1u << 20);
    b->unit_passes = (uint32_t)per;
    // --- genome-specialised kernels for the structures with >= 2 units per SM (animation frames
    // share one), compiled in parallel and cached across batches, each a persistent launch of its
    // own; the other structures share the interpreted persistent launch, or with specialize = 2 get
    // their own kernels too (the launches overlap on forked streams; their compilation costs about
    // a second per structure once, and the cache keeps them).  (Giving every structure
    // its own kernel, the small ones launched concurrently on auxiliary streams, measured slower:
    // 24.9 against 26.9 Gpoints/s on the 184-image batch — a CTA per unit balances worse than one
    // persistent queue.)  Structures whose kernel does not compile stay interpreted.
    if (d->specialize >= 0) {
        std::map<std::string, uint64_t> units_of;
        std::map<std::string, const Item*> rep;
        for (auto& it : b->items) {
            units_of[it.structure] += std::max<uint64_t>(1, ((it.desc.points + b->slots - 1) / b->slots + per - 1) / per);
            rep.emplace(it.structure, &it);
        }
        std::vector<std::pair<uint64_t, std::string>> order;
        for (auto& kv : units_of)  // (a batch of one structure always: no other launch to balance against)
            if (kv.second >= (uint64_t)kSpecMinUnitsPerSM * sms || units_of.size() == 1 || d->specialize == 2)
                order.push_back({kv.second, kv.first});
        std::sort(order.rbegin(), order.rend());
        std::vector<const void*> kern(order.size(), nullptr);
        std::vector<int> rcs(order.size(), RF_OK);
        std::atomic<size_t> next{0};
        auto worker = [&]() {
            for (size_t j; (j = next++) < order.size();)
                rcs[j] = spec_kernel(rep[order[j].second]->prog, (int)b->threads, (int)b->slots, b->device, &kern[j],
                                     SpecKind::Batch);
        };
        const unsigned nt = std::max(1u, std::min<unsigned>(kCompileThreads, (unsigned)order.size()));
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; t++) pool.emplace_back(worker);
        worker();
        for (auto& t : pool) t.join();
        cudaSetDevice(b->device);
        for (size_t j = 0; j < order.size(); j++) {
            int grid = rcs[j] == RF_OK ? batch_spec_grid(kern[j], (int)b->threads, (int)b->slots, b->max_prog_words) : 0;
            if (rcs[j] != RF_OK || grid == 0) {
                if (d->specialize == 1)
                    return bail(rcs[j] != RF_OK ? rcs[j] : fail(RF_ERR_CUDA, "specialised batch kernel: no resident CTA"));
                continue;
            }
            SpecGroup G;
            G.kernel = kern[j];
            G.grid = grid;
            b->groups.push_back(G);
            for (auto& it : b->items)
                if (it.structure == order[j].second) it.group = (int)b->groups.size() - 1;
        }
    }
    if (int rc = build_tables(b, b->slots, b->unit_passes, 0, n)) return bail(rc);
    if (d->use_graph) {
        e = density_prepare();
        if (e != cudaSuccess) return bail(cuda_err(e, "density estimation set-up"));
        e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return bail(cuda_err(e, "graph capture"));
        int rc = enqueue(b);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->stream, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return bail(rc); }
        if (e != cudaSuccess) return bail(cuda_err(e, "graph capture"));
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) return bail(cuda_err(e, "graph instantiate"));
    }
    e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bail(cuda_err(e, "rf_batch_create"));
    *out = b;
    return RF_OK;
}

int rf_batch_run(rf_batch* b) {
    if (!b) return fail(RF_ERR_INVALID_ARG, "rf_batch_run: null batch");
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(RF_ERR_CUDA, "cudaSetDevice");
    cudaError_t e = cudaEventRecord(b->ev0, b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_run");
    if (b->exec) {
        e = cudaGraphLaunch(b->exec, b->stream);
        if (e != cudaSuccess) return cuda_err(e, "graph launch");
    } else if (int rc = enqueue(b)) {
        return rc;
    }
    e = cudaEventRecord(b->ev1, b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_run");
    return RF_OK;
}

int rf_batch_sync(rf_batch* b, double* st) {
    if (!b) return fail(RF_ERR_INVALID_ARG, "rf_batch_sync: null batch");
    cudaSetDevice(b->device);
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_sync");
    if (st) {
        unsigned long long c[3];
        float ms = 0;
        cudaMemcpy(c, b->counters, sizeof c, cudaMemcpyDeviceToHost);
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        uint64_t drawn_pts = 0;
        for (auto& it : b->items) drawn_pts += it.passes * b->slots;
        st[0] = (double)drawn_pts;
        st[1] = (double)c[0];
        st[2] = ms;
        st[3] = (double)c[2];
    }
    return RF_OK;
}

int rf_batch_image(rf_batch* b, uint32_t i, uint8_t* host_rgba8) {
    if (!b || i >= b->items.size() || !host_rgba8) return fail(RF_ERR_INVALID_ARG, "rf_batch_image: bad arguments");
    cudaSetDevice(b->device);
    const Item& it = b->items[i];
    cudaError_t e = cudaMemcpyAsync(host_rgba8, it.img, (size_t)it.desc.width * it.desc.height * 4,
                                    cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_image");
    return RF_OK;
}

int rf_batch_bins(rf_batch* b, uint32_t i, float** rgba, uint32_t** hits, uint32_t* width, uint32_t* height) {
    if (!b || i >= b->items.size()) return fail(RF_ERR_INVALID_ARG, "rf_batch_bins: bad arguments");
    const Item& it = b->items[i];
    if (rgba) *rgba = (float*)it.bins;
    if (hits) *hits = it.hits;
    if (width) *width = it.W;
    if (height) *height = it.H;
    return RF_OK;
}

int rf_batch_read_bins(rf_batch* b, uint32_t i, float* host_rgba, uint32_t* host_hits) {
    if (!b || i >= b->items.size()) return fail(RF_ERR_INVALID_ARG, "rf_batch_read_bins: bad arguments");
    cudaSetDevice(b->device);
    const Item& it = b->items[i];
    const size_t nb = (size_t)it.W * it.H;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess && host_rgba) e = cudaMemcpy(host_rgba, it.bins, nb * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && host_hits) e = cudaMemcpy(host_hits, it.hits, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_read_bins");
    return RF_OK;
}

int rf_batch_specialized(const rf_batch* b, uint32_t i) {
    if (!b || i >= b->items.size()) return -1;
    return b->items[i].group >= 0 ? 1 : 0;
}

int rf_batch_splat(const rf_batch* b, uint32_t i) {
    if (!b || i >= b->items.size()) return -1;
    return b->items[i].splat ? RF_SPLAT_WARP : RF_SPLAT_GLOBAL;
}

int rf_batch_image_f32(rf_batch* b, uint32_t i, float* dst_rgba) {
    if (!b || i >= b->items.size() || !dst_rgba) return fail(RF_ERR_INVALID_ARG, "rf_batch_image_f32: bad arguments");
    const Item& it = b->items[i];
    if (!it.img_f32) return fail(RF_ERR_INVALID_ARG, "rf_batch_image_f32: batch created without image_f32");
    cudaSetDevice(b->device);
    cudaError_t e = cudaMemcpyAsync(dst_rgba, it.img_f32, (size_t)it.desc.width * it.desc.height * sizeof(float4),
                                    cudaMemcpyDefault, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_image_f32");
    return RF_OK;
}

int rf_batch_features(rf_batch* b, uint32_t i, float k2, float level, void* dst_bf16) {
    if (!b || i >= b->items.size() || !dst_bf16) return fail(RF_ERR_INVALID_ARG, "rf_batch_features: bad arguments");
    const Item& it = b->items[i];
    cudaSetDevice(b->device);
    cudaError_t e = cudaSuccess;
    if (!(k2 > 0.0f)) e = launch_stats(it.bins, it.W, it.H, b->stats + 3 * i, b->stream);
    if (e == cudaSuccess)
        e = launch_features(it.bins, (uint64_t)it.W * it.H, k2, b->stats + 3 * i, it.ss == 1 ? it.img_f32 : nullptr,
                            level, static_cast<__nv_bfloat16*>(dst_bf16), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_err(e, "rf_batch_features");
    return RF_OK;
}

int rf_batch_info(const rf_batch* b, uint32_t* cta_slots, uint32_t* units, uint32_t* unit_passes) {
    if (!b) return fail(RF_ERR_INVALID_ARG, "rf_batch_info: null batch");
    if (cta_slots) *cta_slots = b->slots;
    if (units) *units = b->n_units;
    if (unit_passes) *unit_passes = b->unit_passes;
    return RF_OK;
}

int rf_batch_destroy(rf_batch* b) {
    destroy_batch(b);
    return RF_OK;
}

}  // extern "C"
