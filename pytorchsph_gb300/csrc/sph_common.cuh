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
// contract nor approximate it.
__device__ __forceinline__ float dist2_ref(float xi, float yi, float xj, float yj) {
  float dx = __fsub_rn(xi, xj);
  float dy = __fsub_rn(yi, yj);
  return __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
}

// Square-root-free form of the same predicate.  For a float v >= 0 and a float h > 0,
// with IEEE round-to-nearest sqrt:  RN(sqrt(v)) < h  <=>  sqrt(v) < m, where m is the
// midpoint between h and its float predecessor (RN(x) <= pred(h) exactly when x < m; a tie
// x = m cannot occur because m^2 has an odd ~50-bit significand while v has 24 bits).
// m^2 is exact in double, so the predicate is  v <= F  with F the largest float below
// m^2.  F is computed once per query particle; the candidate loop then needs no sqrt.
// The double arithmetic is slow on GB300, so kernels take F from a table computed once
// (grid_threshold, SphParams::thr) whenever the support is the common one.
__host__ __device__ __forceinline__ float sq_threshold(float h) {
  if (!(h > 0.f)) return -1.0f;          // sqrt(v) >= 0 >= h: nothing passes (NaN h too)
  if (isinf(h)) return 3.40282347e38f;   // every finite v passes
  float p = nextafterf(h, 0.0f);
  double m = ((double)p + (double)h) * 0.5;
  double m2 = m * m;
#ifdef __CUDA_ARCH__
  float f = __double2float_rn(m2);
#else
  float f = (float)m2;                   // round to nearest, as on the device
#endif
  if ((double)f >= m2) f = nextafterf(f, 0.0f);
  return f;
}

// sq_threshold(h) for a query of support h in grid g: the grid carries the value for its
// largest support (threshold_support, or the cell size hmax when that is 0), computed once
// by sph_grid_build.
__device__ __forceinline__ float grid_threshold(float h, const sph_grid& g) {
  const float hs = g.threshold_support > 0.f ? g.threshold_support : g.hmax;
  return (h == hs && g.hmax_threshold > 0.f) ? g.hmax_threshold : sq_threshold(h);
}

// Reference predicate with the distance: true iff sqrtf(fmaf(dx,dx,dy*dy)) < h_i.
__device__ __forceinline__ bool pair_pred(float xi, float yi, float xj, float yj, float hi, float* dist) {
  float v = dist2_ref(xi, yi, xj, yj);
  float d = __fsqrt_rn(v);
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

// A grid is usable only if its cells fit the cell table.
__device__ __forceinline__ bool grid_ok(const sph_grid& g, int32_t cap) {
  return g.num_cells <= cap && g.cells_x > 0 && g.cells_y > 0;
}

// Up to kMaxArrays per-particle arrays moved together into a new order (4-, 8- or 16-byte
// rows): the permute kernel and the counting sort's in-cell fix copy row src of every
// in[k] to row dst of out[k].
constexpr int kMaxArrays = 8;
struct ArraySet {
  const void* in[kMaxArrays];
  void* out[kMaxArrays];
  int32_t bytes[kMaxArrays];
  int32_t count;
};

// The set from host arrays of `count` entries; false for a count above kMaxArrays, a
// missing or shared in/out pointer, or a row size other than 4, 8 or 16 bytes.
inline bool array_set_from(int32_t count, const int32_t* elem_bytes, const void* const* in, void* const* out,
                           ArraySet* a) {
  if (count < 0 || count > kMaxArrays || (count > 0 && (!elem_bytes || !in || !out))) return false;
  a->count = count;
  for (int k = 0; k < kMaxArrays; ++k) {
    a->in[k] = nullptr;
    a->out[k] = nullptr;
    a->bytes[k] = 4;
  }
  for (int k = 0; k < count; ++k) {
    if (!in[k] || !out[k] || in[k] == out[k] || (elem_bytes[k] != 4 && elem_bytes[k] != 8 && elem_bytes[k] != 16))
      return false;
    a->in[k] = in[k];
    a->out[k] = out[k];
    a->bytes[k] = elem_bytes[k];
  }
  return true;
}

__device__ __forceinline__ void copy_rows(const ArraySet& a, int64_t dst, int64_t src) {
#pragma unroll
  for (int k = 0; k < kMaxArrays; ++k) {
    if (k >= a.count) break;
    switch (a.bytes[k]) {
      case 4:
        static_cast<uint32_t*>(a.out[k])[dst] = static_cast<const uint32_t*>(a.in[k])[src];
        break;
      case 8:
        static_cast<uint2*>(a.out[k])[dst] = static_cast<const uint2*>(a.in[k])[src];
        break;
      default:
        static_cast<uint4*>(a.out[k])[dst] = static_cast<const uint4*>(a.in[k])[src];
        break;
    }
  }
}

__device__ __forceinline__ void flag(int32_t* status, int32_t f) {
  if (status) atomicOr(status, f);
}

}  // namespace sph
