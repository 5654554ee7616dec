// Batched rendering, interpreted kernel: the persistent launch of batch_body.cuh on the program
// interpreter.  Genome-specialised batch kernels for large same-structure groups (animation
// frames) are compiled at run time (specialize.cpp).
#include <cuda_runtime.h>

#include "batch.h"
#include "batch_body.cuh"

namespace rfk {

template <int THREADS, int SPT>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batch_kernel(const BatchArgs A) {
    batch_body<THREADS, SPT, InterpEval>(A);
}

template <int THREADS, int SPT>
static cudaError_t launch_batch_t(const BatchArgs& a, cudaStream_t st, int* grid_out) {
    const size_t smem = batch_smem_bytes(THREADS * SPT, a.max_prog_words);
    auto kern = batch_kernel<THREADS, SPT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = sms * per_sm;  // persistent: one resident wave pulls every unit
    if (grid_out) *grid_out = grid;
    kern<<<grid, THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

int batch_spec_grid(const void* kernel, int threads, int slots, uint32_t max_prog_words) {
    const size_t smem = batch_smem_bytes(slots, max_prog_words);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return sms * per_sm;
}

cudaError_t launch_batch_spec(const void* kernel, int threads, int slots, int grid, const BatchArgs& a,
                              cudaStream_t st) {
    void* args[] = {const_cast<BatchArgs*>(&a)};
    return cudaLaunchKernel(kernel, dim3(grid), dim3(threads), args, batch_smem_bytes(slots, a.max_prog_words), st);
}

cudaError_t launch_batch(int threads, int slots, const BatchArgs& a, cudaStream_t st, int* grid_out) {
    switch (threads * 8 + slots / threads) {
    case 512 * 8 + 2: return launch_batch_t<512, 2>(a, st, grid_out);
    case 1024 * 8 + 1: return launch_batch_t<1024, 1>(a, st, grid_out);
    case 1024 * 8 + 2: return launch_batch_t<1024, 2>(a, st, grid_out);
    case 1024 * 8 + 4: return launch_batch_t<1024, 4>(a, st, grid_out);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace rfk
