// Forced include of the checker build of the reference's VBD device functions — TEST
// INFRASTRUCTURE ONLY. The reference's headers declare its kernels and stream-taking
// launchers next to the host/device functions; on the host those qualifiers are empty.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <algorithm>
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __builtin_align__(n) alignas(n)
typedef struct CUstream_st* cudaStream_t;
