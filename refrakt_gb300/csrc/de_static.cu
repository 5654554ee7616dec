// Density estimation that allocates no device memory.
//
// rf_density_estimate needs two pieces of scratch per call — one byte per bin for the disc radii
// and a table of kernel weights — and takes them from cudaMallocAsync.  Some callers cannot
// allocate: a plug-in that runs inside a host application which owns the device memory pool and
// forbids allocations outside it, or a frame loop with a fixed, pre-budgeted memory footprint that
// must not call the allocator (cudaMalloc may synchronise the device).  For them this file keeps
// the scratch in file-scope static device arrays of a fixed size, present on every GPU that loads
// the library until the process exits: kStaticDeMaxBins bytes of radii (8 MiB, one 3840x2160 bin
// grid) and the weights of every radius up to 100 (1.4 MB).
//
// In host code a __device__ array's name stands for a host-side shadow, not a device address, so
// the device address is looked up with cudaGetSymbolAddress once per device, with that device
// current, on the first call made on it.  That first call also fills the weight table — the
// weights of every radius up to 100, which do not depend on the call's arguments (a radius's
// weights sit at the same offset whatever the largest radius) — with one synchronous copy; it
// should come before any stream capture.  Later calls copy nothing from the host.  Every call on
// a device shares the radius array and leaves its radii in it; each call rewrites every bin's
// radius before reading it, so nothing has to start at zero.  Calls that overlap on the GPU (two
// streams at once) race on the shared radii and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "internal.h"
#include "kernels.h"

namespace rfk {

constexpr size_t kStaticDeMaxBins = (size_t)8 << 20;  // 8,388,608 bins
constexpr size_t kStaticDeMaxWeights = 348551;       // sum of (r + 1)^2 for r = 0..100

static __device__ __align__(256) uint8_t g_de_radius_scratch[kStaticDeMaxBins];
static __device__ __align__(256) float g_de_weight_scratch[kStaticDeMaxWeights];

namespace {

constexpr int kMaxDevices = 64;

struct StaticScratch {
    uint8_t* radius = nullptr;
    float* weights = nullptr;
};

std::mutex g_scratch_mu;
StaticScratch g_scratch[kMaxDevices];

// device addresses of the static scratch on the current device, looked up once per device
int scratch_for_current_device(StaticScratch& out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(RF_ERR_CAPACITY, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    StaticScratch& s = g_scratch[dev];
    if (!s.radius) {
        void* rad = nullptr;
        void* wts = nullptr;
        e = cudaGetSymbolAddress(&rad, g_de_radius_scratch);
        if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&wts, g_de_weight_scratch);
        if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        // the weights of every radius up to 100, once per device
        std::vector<float> table;
        density_weights(100, 0, table);
        if (table.size() != kStaticDeMaxWeights) return fail(RF_ERR_CAPACITY, "static weight table size mismatch");
        e = cudaMemcpy(wts, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("static weight table: ") + cudaGetErrorString(e));
        s.radius = static_cast<uint8_t*>(rad);
        s.weights = static_cast<float*>(wts);
    }
    out = s;
    return RF_OK;
}

}  // namespace
}  // namespace rfk

using namespace rfk;

extern "C" int rf_density_estimate_static(const float* in, uint32_t w, uint32_t h, int radius, int min_radius,
                                          float curve, float* out, void* stream) {
    if (!in || !out || w == 0 || h == 0) return fail(RF_ERR_INVALID_ARG, "rf_density_estimate_static: bad arguments");
    if (radius < 0 || radius > 100 || min_radius < 0 || min_radius > 100)
        return fail(RF_ERR_INVALID_ARG, "estimator radii must be within 0..100 (main.cpp:502)");
    if (in == out) return fail(RF_ERR_INVALID_ARG, "rf_density_estimate_static: in and out must differ");
    if ((size_t)w * (size_t)h > kStaticDeMaxBins)
        return fail(RF_ERR_CAPACITY, "rf_density_estimate_static: " + std::to_string((size_t)w * h) +
                                         " bins exceed the static scratch of " + std::to_string(kStaticDeMaxBins) +
                                         " bins; use rf_density_estimate");
    if (h > 65535) return fail(RF_ERR_CAPACITY, "rf_density_estimate_static: more than 65535 rows");
    StaticScratch s;
    if (int rc = scratch_for_current_device(s)) return rc;
    cudaError_t e = launch_density_resident((const float4*)in, w, h, radius, min_radius, curve, (float4*)out, s.radius,
                                            s.weights, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(RF_ERR_CUDA, std::string("rf_density_estimate_static: ") + cudaGetErrorString(e));
    return RF_OK;
}
