// Fixed-width integer types for headers that are also compiled at run time (NVRTC has no C
// library headers); under nvcc and host compilers these come from <stdint.h> and <stddef.h>.
#pragma once

#ifdef __CUDACC_RTC__
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned long size_t;
#else
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#endif
