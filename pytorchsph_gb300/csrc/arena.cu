// Pooled serving arena: the bookkeeping kernels of admitting a scene into free particle slots
// and retiring it.  The batch kernels treat a slot with scene index -1 as empty (the sort puts
// it in the sentinel cell after every scene's cells, and no scene searches that cell).
#include "sph_common.cuh"

namespace sph {

__global__ void k_arena_set_ids(int32_t* __restrict__ sid, int32_t* __restrict__ uid, int64_t begin, int64_t count,
                                int32_t scene) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  sid[begin + k] = scene;
  uid[begin + k] = (int32_t)k;
}

__global__ void k_arena_extract(const float2* __restrict__ x, const float2* __restrict__ v,
                                const float* __restrict__ rho, const int32_t* __restrict__ sid,
                                const int32_t* __restrict__ uid, int64_t n, int32_t scene, float2* __restrict__ xo,
                                float2* __restrict__ vo, float* __restrict__ ro) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || sid[i] != scene) return;
  const int32_t u = uid[i];
  xo[u] = x[i];
  vo[u] = v[i];
  ro[u] = rho[i];
}

__global__ void k_arena_retire(int32_t* __restrict__ sid, int64_t n, int32_t scene) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && sid[i] == scene) sid[i] = -1;
}

// Several scenes at once: a particle of scene s with row0[s] >= 0 goes to output row
// row0[s] + uid (uid < rows[s], else skipped), and with `retire` its slot is freed.
__global__ void k_arena_extract_many(const float2* __restrict__ x, const float2* __restrict__ v,
                                     const float* __restrict__ rho, int32_t* __restrict__ sid,
                                     const int32_t* __restrict__ uid, int64_t n, const int64_t* __restrict__ row0,
                                     const int32_t* __restrict__ rows, int32_t nslots, float2* __restrict__ xo,
                                     float2* __restrict__ vo, float* __restrict__ ro, int retire) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s = sid[i];
  if (s < 0 || s >= nslots) return;
  const int64_t r0 = row0[s];
  if (r0 < 0) return;
  if (xo) {
    const int32_t u = uid[i];
    if (u >= 0 && u < rows[s]) {
      xo[r0 + u] = x[i];
      vo[r0 + u] = v[i];
      ro[r0 + u] = rho[i];
    }
  }
  if (retire) sid[i] = -1;
}

}  // namespace sph

using namespace sph;

extern "C" {

sph_status_t sph_arena_set_ids(int32_t* sid, int32_t* uid, int64_t begin, int64_t count, int32_t scene,
                               void* stream) {
  SPH_REQUIRE(sid && uid && begin >= 0 && count >= 0 && count < (1LL << 31) && scene >= 0,
              "arena_set_ids: bad arguments");
  if (count == 0) return SPH_OK;
  k_arena_set_ids<<<grid_for(count, 256), 256, 0, as_stream(stream)>>>(sid, uid, begin, count, scene);
  SPH_CHECK_LAUNCH("arena_set_ids");
  return SPH_OK;
}

sph_status_t sph_arena_extract(const float* x, const float* v, const float* rho, const int32_t* sid,
                               const int32_t* uid, int64_t n, int32_t scene, float* x_out, float* v_out,
                               float* rho_out, void* stream) {
  SPH_REQUIRE(n >= 0 && x && v && rho && sid && uid && x_out && v_out && rho_out && scene >= 0,
              "arena_extract: bad arguments");
  if (n == 0) return SPH_OK;
  k_arena_extract<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(x), reinterpret_cast<const float2*>(v), rho, sid, uid, n, scene,
      reinterpret_cast<float2*>(x_out), reinterpret_cast<float2*>(v_out), rho_out);
  SPH_CHECK_LAUNCH("arena_extract");
  return SPH_OK;
}

sph_status_t sph_arena_extract_many(const float* x, const float* v, const float* rho, int32_t* sid,
                                    const int32_t* uid, int64_t n, const int64_t* row0, const int32_t* rows,
                                    int32_t nslots, float* x_out, float* v_out, float* rho_out, int32_t retire,
                                    void* stream) {
  const bool out = x_out || v_out || rho_out;
  SPH_REQUIRE(n >= 0 && sid && row0 && rows && nslots >= 0 && (!out || (x_out && v_out && rho_out && x && v && rho
                                                                          && uid)),
              "arena_extract_many: bad arguments");
  if (n == 0 || nslots == 0) return SPH_OK;
  k_arena_extract_many<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(x), reinterpret_cast<const float2*>(v), rho, sid, uid, n, row0, rows, nslots,
      reinterpret_cast<float2*>(x_out), reinterpret_cast<float2*>(v_out), rho_out, retire ? 1 : 0);
  SPH_CHECK_LAUNCH("arena_extract_many");
  return SPH_OK;
}

sph_status_t sph_arena_retire(int32_t* sid, int64_t n, int32_t scene, void* stream) {
  SPH_REQUIRE(n >= 0 && sid && scene >= 0, "arena_retire: bad arguments");
  if (n == 0) return SPH_OK;
  k_arena_retire<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(sid, n, scene);
  SPH_CHECK_LAUNCH("arena_retire");
  return SPH_OK;
}

}  // extern "C"
