// Genome-specialised chaos kernels compiled at run time (specialize.cpp).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "chaos_args.h"

namespace rfk {

enum class SpecKind { Chaos, Batch };

// CUDA source of the specialised kernel for a compiled genome and CTA shape; splat >= 0 (chaos
// kernels) fixes the splat strategy (ChaosArgs.splat's codes) at compile time and reset >= 0 the
// walker reset (ChaosArgs.reset), -1 leaves them to the launch; pipe = 1 compiles the pipelined
// walker exchange (chaos_body.cuh; spt 4), which needs a shuffle table built with `phases` = spt
std::string spec_source(const std::vector<uint32_t>& prog, int threads, int spt, SpecKind kind = SpecKind::Chaos,
                        int splat = -1, int reset = -1, int pipe = 0);
// the structure part of that source: equal for genomes that can share one specialised kernel
std::string spec_structure(const std::vector<uint32_t>& prog);
// compiles source for sm_103a with the run-time compiler (no device needed)
int spec_compile(const std::string& src, std::vector<char>& cubin);
// true when the run-time compiler can be loaded (else *why says why)
bool spec_available(std::string* why);
// the compiled kernel for this genome's structure (cached); RF_OK or a status with rf_last_error
int spec_kernel(const std::vector<uint32_t>& prog, int threads, int slots, int device, const void** out,
                SpecKind kind = SpecKind::Chaos, int splat = -1, int reset = -1, int pipe = 0);
cudaError_t launch_spec(const void* kernel, int threads, int slots, const ChaosArgs& a, uint32_t grid, size_t smem,
                        cudaStream_t st);

}  // namespace rfk
