// Shared definitions for the GB300 BCGS kernels.
//
// Layout conventions (the reference's, include/orth.h): every tall matrix is
// column-major FP64 with a leading dimension `ld` >= rows; element (r, c) lives at
// p[r + c * ld]. Column offsets are always formed in 64-bit arithmetic (the
// reference forms them in `int`, SRC/orth.c:174,183,207, which overflows at
// m * n >= 2^31).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bcgs {

using i64 = long long;

// Number of SMs on GB300; grids are sized in multiples of it.
constexpr int kNumSMsDefault = 152;

// Status word layout (device-resident, int32 each), read back by the host API.
//   [0] first Cholesky breakdown: 1-based block step, 0 if none
//   [1] dpotrf-style info of that breakdown (1-based column)
//   [2] bounded-wait timeout flag (reserved; no kernel here spins on a peer)
//   [3] internal argument error flag
constexpr int kStatusWords = 4;

__host__ __device__ inline i64 ceil_div(i64 a, i64 b) { return (a + b - 1) / b; }

}  // namespace bcgs

#define BCGS_CUDA_TRY(expr)                                          \
    do {                                                             \
        cudaError_t _e = (expr);                                     \
        if (_e != cudaSuccess) return (int)_e;                       \
    } while (0)
