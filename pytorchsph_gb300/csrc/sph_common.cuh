// Shared device helpers of the GB300 SPH hot path (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sph_gb300.h"

namespace sph {

// Records the last CUDA error text for sph_last_error().
void set_error(const char* where, cudaError_t err);
void set_error_text(const char* text);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define SPH_CHECK_LAUNCH(where)                            \
  do {                                                     \
    cudaError_t e_ = cudaGetLastError();                   \
    if (e_ != cudaSuccess) {                               \
      ::sph::set_error(where, e_);                         \
      return SPH_ERR_CUDA;                                 \
    }                                                      \
  } while (0)

#define SPH_REQUIRE(cond, msg)                 \
  do {                                         \
    if (!(cond)) {                             \
      ::sph::set_error_text(msg);              \
      return SPH_ERR_INVALID_ARGUMENT;         \
    }                                          \
  } while (0)

constexpr int kNumSMs = 152;

inline int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)(b < 1 ? 1 : b);
}

// The reference pair predicate, cppSrc/neighSearch.cpp:222-223 as compiled with the
// reference's flags (GCC contracts dx*dx + dy*dy into fmaf(dx, dx, dy*dy)):
//   sqrtf(fmaf(dx, dx, dy*dy)) < h_i,  dx = x_i - x_j (i = query).
// Every operation is spelled as a round-to-nearest intrinsic so nvcc can neither
// contract nor approximate it.  Returns the distance through *dist.
__device__ __forceinline__ bool pair_pred(float xi, float yi, float xj, float yj, float hi, float* dist) {
  float dx = __fsub_rn(xi, xj);
  float dy = __fsub_rn(yi, yj);
  float d = __fsqrt_rn(__fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
  *dist = d;
  return d < hi;
}

// Cell coordinate of sortPositions, src/modules/neighborSearch.py:46:
//   ceil((x - qmin) / hmax) in float32, then int32 conversion.
__device__ __forceinline__ int cell_coord(float x, float qmin, float hmax) {
  return (int)ceilf(__fdiv_rn(__fsub_rn(x, qmin), hmax));
}

// Wendland C2 in 2D, src/kernels.py:20-24: W(q) = 7/(pi h^2) (1-q)^4 (1+4q).
// c_w = 7/(pi h^2) precomputed by the caller.
__device__ __forceinline__ float wendland(float q, float c_w) {
  float a = 1.0f - q;
  float a2 = a * a;
  return a2 * a2 * (1.0f + 4.0f * q) * c_w;
}

__device__ __forceinline__ void flag(int32_t* status, int32_t f) {
  if (status) atomicOr(status, f);
}

}  // namespace sph
