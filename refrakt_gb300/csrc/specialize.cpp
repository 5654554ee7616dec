// Genome-specialised chaos kernels, compiled at run time.
//
// The reference generates GLSL per genome: each xform's dispatch() is straight-line code of its
// own variations (src/variation_table.cpp:97-165, 217-264).  The interpreted kernel instead walks
// the compiled program's term list through an out-of-line switch over all 68 variations, and its
// largest stall is instruction fetch: the warps of one scheduler run different xforms, and the
// variation code they touch exceeds the instruction caches.  Here the genome's structure — xform
// count, each xform's variation ids, flags, parameter offsets, precalc mask and post flag, and
// the final xform — becomes C++ source: one inlined evaluator per xform, variation ids as
// constants (each variation's switch folds to its own case), the shared kernel body
// (chaos_body.cuh) instantiated on it.  Weights, affines, colours and parameters are still read
// from the program in shared memory, so every genome of one structure (animation frames,
// interactive edits) reuses one compiled kernel.
//
// NVRTC compiles the source for sm_103a (loaded with dlopen, so the library does not depend on
// it at load time); the cubin is loaded with cudaLibraryLoadData and launched through the
// runtime API.  Kernels are cached per (device, source).
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "chaos_args.h"
#include "internal.h"
#include "program.h"
#include "specialize.h"

namespace rfk {

// embedded copies of the device headers (generated at build time, rtc_headers.cpp)
extern const int kRtcHeaderCount;
extern const char* const kRtcHeaderNames[];
extern const char* const kRtcHeaderSources[];

namespace {

// ---- NVRTC through dlopen ----------------------------------------------------------------------
typedef int nvrtcResult_;
typedef struct _nvrtcProgram* nvrtcProgram_;
struct Nvrtc {
    nvrtcResult_ (*create)(nvrtcProgram_*, const char*, const char*, int, const char* const*, const char* const*);
    nvrtcResult_ (*compile)(nvrtcProgram_, int, const char* const*);
    nvrtcResult_ (*log_size)(nvrtcProgram_, size_t*);
    nvrtcResult_ (*log)(nvrtcProgram_, char*);
    nvrtcResult_ (*cubin_size)(nvrtcProgram_, size_t*);
    nvrtcResult_ (*cubin)(nvrtcProgram_, char*);
    nvrtcResult_ (*destroy)(nvrtcProgram_*);
    bool ok = false;
    std::string why;
};

const Nvrtc& nvrtc() {
    static Nvrtc n = [] {
        Nvrtc r{};
        const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"};
        void* h = nullptr;
        for (const char* nm : names)
            if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            r.why = "libnvrtc not found";
            return r;
        }
        r.create = (decltype(r.create))dlsym(h, "nvrtcCreateProgram");
        r.compile = (decltype(r.compile))dlsym(h, "nvrtcCompileProgram");
        r.log_size = (decltype(r.log_size))dlsym(h, "nvrtcGetProgramLogSize");
        r.log = (decltype(r.log))dlsym(h, "nvrtcGetProgramLog");
        r.cubin_size = (decltype(r.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
        r.cubin = (decltype(r.cubin))dlsym(h, "nvrtcGetCUBIN");
        r.destroy = (decltype(r.destroy))dlsym(h, "nvrtcDestroyProgram");
        r.ok = r.create && r.compile && r.log_size && r.log && r.cubin_size && r.cubin && r.destroy;
        if (!r.ok) r.why = "libnvrtc lacks a required entry point";
        return r;
    }();
    return n;
}

// ---- source generation -------------------------------------------------------------------------
void emit_xform(std::ostringstream& o, const std::vector<uint32_t>& prog, uint32_t off, bool is_final) {
    const uint32_t npre = prog[off + X_NPRE], nterm = prog[off + X_NTERM], mask = prog[off + X_MASK];
    const bool post = prog[off + X_HASPOST] != 0;
    o << "  const uint32_t* blk = prog + " << off << "u;\n"
      << "  const float* fb = reinterpret_cast<const float*>(blk);\n"
      << "  float vx = fmaf(fb[" << X_AFF + 0 << "], x, fmaf(fb[" << X_AFF + 2 << "], y, fb[" << X_AFF + 4 << "]));\n"
      << "  float vy = fmaf(fb[" << X_AFF + 1 << "], x, fmaf(fb[" << X_AFF + 3 << "], y, fb[" << X_AFF + 5 << "]));\n"
      << "  Pre pc;\n";
    uint32_t e = off + X_TERMS;
    for (uint32_t k = 0; k < npre; k++, e += 3) {
        const uint32_t id = prog[e] & 0xffu, widx = e + 1 - off, poff = prog[e + 2];
        o << "  { pc.x = vx; pc.y = vy; const float wt = fb[" << widx << "];\n"
          << "    const float2 d = vary_impl(" << id << "u, pc, wt, fb + " << X_AFF << ", fb + " << poff << ", rng);\n"
          << "    vx = __fadd_rn(vx, __fmul_rn(wt, d.x)); vy = __fadd_rn(vy, __fmul_rn(wt, d.y)); }\n";
    }
    o << "  precalc(pc, vx, vy, " << mask << "u);\n  float rx = 0.0f, ry = 0.0f;\n";
    for (uint32_t k = 0; k < nterm; k++, e += 3) {
        const uint32_t id = prog[e] & 0xffu, widx = e + 1 - off, poff = prog[e + 2];
        const bool wmul = !(prog[e] & kTermNoWeightMul);
        o << "  { const float wt = fb[" << widx << "];\n"
          << "    float2 d = vary_impl(" << id << "u, pc, wt, fb + " << X_AFF << ", fb + " << poff << ", rng);\n";
        if (wmul) o << "    d.x = __fmul_rn(wt, d.x); d.y = __fmul_rn(wt, d.y);\n";
        if (k == 0) o << "    rx = d.x; ry = d.y; }\n";
        else o << "    rx = __fadd_rn(rx, d.x); ry = __fadd_rn(ry, d.y); }\n";
    }
    if (post)
        o << "  { const float px = fmaf(fb[" << X_POST + 0 << "], rx, fmaf(fb[" << X_POST + 2 << "], ry, fb["
          << X_POST + 4 << "]));\n"
          << "    const float py = fmaf(fb[" << X_POST + 1 << "], rx, fmaf(fb[" << X_POST + 3 << "], ry, fb["
          << X_POST + 5 << "]));\n    rx = px; ry = py; }\n";
    o << (is_final ? "  const float cin = c;\n" : "  const float cin = first_run ? randf(rng) : c;\n")
      << "  c = __fadd_rn(__fmul_rn(cin, fb[" << X_OMCS << "]), __fmul_rn(fb[" << X_COLOR << "], fb[" << X_CS
      << "]));\n  x = rx; y = ry; op = fb[" << X_OPACITY << "];\n";
}

struct Spec {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
};

std::mutex g_mu;
std::map<std::string, std::unique_ptr<Spec>> g_cache;  // key: device + source

}  // namespace

// struct GenEval: one inlined evaluator per xform of this genome's structure
static std::string gen_eval(const std::vector<uint32_t>& prog) {
    std::ostringstream o;
    o << "namespace rfk {\n"
      << "struct GenEval {\n  static __device__ __forceinline__ void apply(const uint32_t* __restrict__ prog, int xi, "
         "uint32_t, float& x, float& y, float& c, float& op, bool first_run, Jsf& rng) {\n    switch (xi) {\n";
    const uint32_t nx = prog[H_NX];
    for (uint32_t k = 0; k < nx; k++) {
        o << (k + 1 == nx ? "    default: {\n" : "    case " + std::to_string(k) + ": {\n");
        emit_xform(o, prog, prog[H_XOFF + k], false);
        o << "      break; }\n";
    }
    if (prog[H_HASFINAL] && prog[H_FINAL]) {
        o << "    case -1: {\n";
        emit_xform(o, prog, prog[H_FINAL], true);
        o << "      break; }\n";
    }
    o << "    }\n  }\n};\n}  // namespace rfk\n";
    return o.str();
}

std::string spec_source(const std::vector<uint32_t>& prog, int threads, int spt, SpecKind kind, int splat, int reset,
                        int pipe) {
    std::ostringstream o;
    o << "// generated: genome-specialised " << (kind == SpecKind::Batch ? "batch" : "chaos") << " kernel\n"
      << (kind == SpecKind::Batch ? "#include \"batch_body.cuh\"\n" : "#include \"chaos_body.cuh\"\n")
      << gen_eval(prog);
    if (kind == SpecKind::Batch)
        o << "extern \"C\" __global__ void __launch_bounds__(" << threads << ", " << 1024 / threads
          << ") rfk_batch_spec(const rfk::BatchArgs A) {\n  rfk::batch_body<" << threads << ", " << spt
          << ", rfk::GenEval>(A);\n}\n";
    else
        o << "extern \"C\" __global__ void __launch_bounds__(" << threads << ", " << 1024 / threads
          << ") rfk_chaos_spec(const rfk::ChaosArgs A) {\n  rfk::chaos_body<" << threads << ", " << spt
          << ", rfk::GenEval, " << (splat >= 0 ? splat : -1) << ", " << (reset >= 0 ? reset : -1) << ", "
          << (pipe ? 1 : 0) << ">(A);\n}\n";
    return o.str();
}

std::string spec_structure(const std::vector<uint32_t>& prog) { return gen_eval(prog); }

bool spec_available(std::string* why) {
    const Nvrtc& n = nvrtc();
    if (!n.ok && why) *why = n.why;
    return n.ok;
}

int spec_compile(const std::string& src, std::vector<char>& cubin) {
    const Nvrtc& n = nvrtc();
    if (!n.ok) return fail(RF_ERR_UNSUPPORTED, "run-time compilation unavailable: " + n.why);
    nvrtcProgram_ p = nullptr;
    if (n.create(&p, src.c_str(), "rfk_chaos_spec.cu", kRtcHeaderCount, kRtcHeaderSources, kRtcHeaderNames) != 0)
        return fail(RF_ERR_CUDA, "nvrtcCreateProgram failed");
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-DRFK_RTC=1"};
    const int rc = n.compile(p, 3, opts);
    if (rc != 0) {
        size_t ls = 0;
        n.log_size(p, &ls);
        std::string log(ls, '\0');
        if (ls) n.log(p, &log[0]);
        n.destroy(&p);
        return fail(RF_ERR_CUDA, "run-time compilation of the specialised kernel failed: " + log.substr(0, 2000));
    }
    size_t cs = 0;
    n.cubin_size(p, &cs);
    cubin.assign(cs, 0);
    n.cubin(p, cubin.data());
    n.destroy(&p);
    return RF_OK;
}

int spec_kernel(const std::vector<uint32_t>& prog, int threads, int slots, int device, const void** out,
                SpecKind kind, int splat, int reset, int pipe) {
    *out = nullptr;
    if (prog.size() < (size_t)H_XOFF || prog[H_MAGIC] != kProgMagic)
        return fail(RF_ERR_INVALID_ARG, "spec_kernel: not a compiled genome");
    const std::string src = spec_source(prog, threads, slots / threads, kind, splat, reset, pipe);
    const std::string key = std::to_string(device) + "\n" + src;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            *out = reinterpret_cast<const void*>(it->second->kernel);
            return RF_OK;
        }
    }
    // compile and load outside the lock, so several structures compile in parallel
    std::vector<char> cubin;
    if (int rc = spec_compile(src, cubin)) return rc;
    auto spec = std::make_unique<Spec>();
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaLibraryLoadData(&spec->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess)
        e = cudaLibraryGetKernel(&spec->kernel, spec->lib, kind == SpecKind::Batch ? "rfk_batch_spec" : "rfk_chaos_spec");
    if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("loading the specialised kernel: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_mu);
    auto ins = g_cache.emplace(key, std::move(spec));  // a concurrent compile of the same source keeps the first
    *out = reinterpret_cast<const void*>(ins.first->second->kernel);
    return RF_OK;
}

cudaError_t launch_spec(const void* kernel, int threads, int slots, const ChaosArgs& a, uint32_t grid,
                        size_t smem, cudaStream_t st) {
    (void)slots;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {const_cast<ChaosArgs*>(&a)};
    return cudaLaunchKernel(kernel, dim3(grid), dim3(threads), args, smem, st);
}

}  // namespace rfk
