// Periodic boundaries (src/modules/periodicBC.py) on sm_103a.
//
// 1. Ghost copies as the reference makes them (createGhostParticlesKernel, periodicBC.py:23-103):
//    the particles within band = buffer * support of the domain's edges, in the reference's
//    category order (x+, x-, then y+, y-, then the corners x+y+, x+y-, x-y+, x-y-), each
//    category in increasing particle index, with the position offset of its copy.  One flag
//    pass, one scan per category, one fill pass: the same order every run.
// 2. A periodic neighbor search without copies: the cell grid tiles the periodic box exactly,
//    neighbor cells wrap around, and a neighbor seen through an edge is tested at its image
//    position x_j + offset, formed in float32 as the reference forms its ghost positions.  The
//    result is the reference's pair set of real particles against real particles and ghosts,
//    with each ghost replaced by (its particle, the offset code of its category).
#include "sph_common.cuh"

namespace sph {

constexpr int kGhostCats = 8;

struct PBox {
  float minx, miny;
  float lx, ly;        // (float)(max - min): the offset the reference adds to its ghosts
  float thx_hi, thx_lo, thy_hi, thy_lo;   // band thresholds: x >= thx_hi, x < thx_lo, ...
  int px, py;
};

// Category bits of particle p: 0 x+, 1 x-, 2 y+, 3 y-, 4 x+y+, 5 x+y-, 6 x-y+, 7 x-y-
// (only the categories the periodic directions enable).
__device__ __forceinline__ int ghost_bits(float2 p, const PBox& B) {
  const bool xp = p.x >= B.thx_hi, xn = p.x < B.thx_lo, yp = p.y >= B.thy_hi, yn = p.y < B.thy_lo;
  int m = 0;
  if (B.px) m |= (xp ? 1 : 0) | (xn ? 2 : 0);
  if (B.py) m |= (yp ? 4 : 0) | (yn ? 8 : 0);
  if (B.px && B.py) m |= ((xp && yp) ? 16 : 0) | ((xp && yn) ? 32 : 0) | ((xn && yp) ? 64 : 0) | ((xn && yn) ? 128 : 0);
  return m;
}

__device__ __forceinline__ float2 ghost_offset(int c, const PBox& B) {
  switch (c) {
    case 0: return make_float2(-B.lx, 0.f);
    case 1: return make_float2(B.lx, 0.f);
    case 2: return make_float2(0.f, -B.ly);
    case 3: return make_float2(0.f, B.ly);
    case 4: return make_float2(-B.lx, -B.ly);
    case 5: return make_float2(-B.lx, B.ly);
    case 6: return make_float2(B.lx, -B.ly);
    default: return make_float2(B.lx, B.ly);
  }
}

__global__ void k_ghost_flags(const float2* __restrict__ pos, int64_t n, PBox B, int32_t* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = ghost_bits(pos[i], B);
#pragma unroll
  for (int c = 0; c < kGhostCats; ++c) flags[c * n + i] = (m >> c) & 1;
}

// slot[c * (n + 1) + i] = exclusive scan of category c's flags; slot[c * (n + 1) + n] its count.
__global__ void k_ghost_fill(const float2* __restrict__ pos, int64_t n, PBox B, const int32_t* __restrict__ slot,
                             int64_t capacity, int64_t* __restrict__ indices, float2* __restrict__ offsets,
                             int32_t* __restrict__ counts, int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t base[kGhostCats];
  int64_t b = 0;
#pragma unroll
  for (int c = 0; c < kGhostCats; ++c) {
    base[c] = b;
    b += slot[c * (n + 1) + n];
  }
  if (i == 0) {
#pragma unroll
    for (int c = 0; c < kGhostCats; ++c) counts[c] = slot[c * (n + 1) + n];
    if (b > capacity) atomicOr(status, SPH_FLAG_PAIR_CAPACITY);
  }
  if (i >= n) return;
  const int m = ghost_bits(pos[i], B);
#pragma unroll
  for (int c = 0; c < kGhostCats; ++c) {
    if (!((m >> c) & 1)) continue;
    const int64_t k = base[c] + slot[c * (n + 1) + i];
    if (k < capacity) {
      indices[k] = i;
      offsets[k] = ghost_offset(c, B);
    }
  }
}

// ---------------------------------------------------------------------------- periodic search
struct PGrid {
  float minx, miny, lx, ly;   // box origin and the image offsets (float)(max - min)
  float wx, wy;               // cell width: (max - min) / cells >= support
  int cx, cy;                 // cells per direction (>= 3 along a periodic direction)
  int px, py;
};

__device__ __forceinline__ int pcell(float v, float mn, float w, int cells) {
  int c = (int)floorf((v - mn) / w);
  return c < 0 ? 0 : (c >= cells ? cells - 1 : c);
}

__global__ void k_pcell_keys(const float2* __restrict__ pos, int64_t n, PGrid G, uint32_t* __restrict__ keys,
                             int32_t* __restrict__ cell_count, int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = pos[i];
  if (!(isfinite(p.x) && isfinite(p.y))) {
    atomicOr(status, SPH_FLAG_NONFINITE);
  }
  const uint32_t k = (uint32_t)(pcell(p.x, G.minx, G.wx, G.cx) + G.cx * pcell(p.y, G.miny, G.wy, G.cy));
  keys[i] = k;
  atomicAdd(cell_count + k, 1);
}

// Visit every pair (i, j, code) of query i: the 3 x 3 cells around i's cell, wrapped along
// periodic directions; code = (sx + 1) | (sy + 1) << 2 with s the image shift (-1, 0, +1).
template <typename Fn>
__device__ __forceinline__ void periodic_pairs(int64_t i, const float2* __restrict__ pos,
                                               const float2* __restrict__ spos, const uint32_t* __restrict__ order,
                                               const int32_t* __restrict__ cell_start, const PGrid& G, float thr,
                                               Fn&& fn) {
  const float2 pi = pos[i];
  const int ci = pcell(pi.x, G.minx, G.wx, G.cx), cj = pcell(pi.y, G.miny, G.wy, G.cy);
  for (int dy = -1; dy <= 1; ++dy) {
    int yy = cj + dy, sy = 0;
    if (yy < 0 || yy >= G.cy) {
      if (!G.py) continue;
      sy = yy < 0 ? -1 : 1;
      yy = yy < 0 ? yy + G.cy : yy - G.cy;
    }
    for (int dx = -1; dx <= 1; ++dx) {
      int xx = ci + dx, sx = 0;
      if (xx < 0 || xx >= G.cx) {
        if (!G.px) continue;
        sx = xx < 0 ? -1 : 1;
        xx = xx < 0 ? xx + G.cx : xx - G.cx;
      }
      // the image of a particle seen through the low edge lies at x - L, through the high edge
      // at x + L (the reference's x+ ghosts carry -L, its x- ghosts +L)
      const float ox = sx < 0 ? -G.lx : (sx > 0 ? G.lx : 0.f);
      const float oy = sy < 0 ? -G.ly : (sy > 0 ? G.ly : 0.f);
      const int c = xx + G.cx * yy;
      for (int s = cell_start[c], e = cell_start[c + 1]; s < e; ++s) {
        const float2 pj = spos[s];
        const float gx = sx ? __fadd_rn(pj.x, ox) : pj.x;
        const float gy = sy ? __fadd_rn(pj.y, oy) : pj.y;
        if (dist2_ref(pi.x, pi.y, gx, gy) <= thr) fn((int64_t)order[s], (sx + 1) | ((sy + 1) << 2));
      }
    }
  }
}

__global__ void k_periodic_count(const float2* __restrict__ pos, const float* __restrict__ support, int64_t n,
                                 const float2* __restrict__ spos, const uint32_t* __restrict__ order,
                                 const int32_t* __restrict__ cell_start, PGrid G, int32_t* __restrict__ counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  periodic_pairs(i, pos, spos, order, cell_start, G, sq_threshold(support[i]), [&](int64_t, int) { ++c; });
  counts[i] = c;
}

// Pairs of query i at offsets[i] ..., ordered by j (insertion into the row as they come).
__global__ void k_periodic_fill(const float2* __restrict__ pos, const float* __restrict__ support, int64_t n,
                                const float2* __restrict__ spos, const uint32_t* __restrict__ order,
                                const int32_t* __restrict__ cell_start, PGrid G, const int64_t* __restrict__ offsets,
                                int64_t capacity, int64_t* __restrict__ cols, int8_t* __restrict__ codes,
                                int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = offsets[i], e = offsets[i + 1];
  if (e > capacity) {
    atomicOr(status, SPH_FLAG_PAIR_CAPACITY);
    return;
  }
  int64_t k = b;
  periodic_pairs(i, pos, spos, order, cell_start, G, sq_threshold(support[i]), [&](int64_t j, int code) {
    if (k >= e) return;
    int64_t u = k++;
    while (u > b && cols[u - 1] > j) {
      cols[u] = cols[u - 1];
      codes[u] = codes[u - 1];
      --u;
    }
    cols[u] = j;
    codes[u] = (int8_t)code;
  });
}

__global__ void k_periodic_rows(const int64_t* __restrict__ offsets, int64_t n, int64_t* __restrict__ rows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t k = offsets[i], e = offsets[i + 1]; k < e; ++k) rows[k] = i;
}

__global__ void k_gather_f2(const uint32_t* __restrict__ order, int64_t n, const float2* __restrict__ in,
                            float2* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = in[order[s]];
}

}  // namespace sph

using namespace sph;

static bool make_box(const float* dmin, const float* dmax, float band, int px, int py, PBox* B) {
  if (!dmin || !dmax || !(dmax[0] > dmin[0]) || !(dmax[1] > dmin[1])) return false;
  B->minx = dmin[0];
  B->miny = dmin[1];
  B->lx = (float)((double)dmax[0] - (double)dmin[0]);
  B->ly = (float)((double)dmax[1] - (double)dmin[1]);
  B->thx_hi = (float)((double)dmax[0] - (double)band);
  B->thx_lo = (float)((double)dmin[0] + (double)band);
  B->thy_hi = (float)((double)dmax[1] - (double)band);
  B->thy_lo = (float)((double)dmin[1] + (double)band);
  B->px = px != 0;
  B->py = py != 0;
  return true;
}

extern "C" {

size_t sph_periodic_ghosts_scratch_bytes(int64_t n) {
  const size_t nn = (size_t)(n > 0 ? n : 1);
  return (size_t)kGhostCats * nn * 4 + (size_t)kGhostCats * (nn + 1) * 4 + sph_scan_scratch_bytes(n) + 512;
}

sph_status_t sph_periodic_ghosts(const float* pos, int64_t n, const float* domain_min, const float* domain_max,
                                 float band, int32_t periodic_x, int32_t periodic_y, int64_t capacity,
                                 int64_t* indices, float* offsets, int32_t* counts, int32_t* status, void* scratch,
                                 size_t scratch_bytes, void* stream) {
  PBox B;
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && capacity >= 0 && counts && status && (n == 0 || pos) &&
                  (capacity == 0 || (indices && offsets)) && make_box(domain_min, domain_max, band, periodic_x,
                                                                      periodic_y, &B),
              "periodic_ghosts: bad arguments");
  if (!scratch || scratch_bytes < sph_periodic_ghosts_scratch_bytes(n)) {
    set_error_text("periodic_ghosts: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const size_t nn = (size_t)(n > 0 ? n : 1);
  int32_t* flags = static_cast<int32_t*>(scratch);
  int32_t* slot = flags + kGhostCats * nn;
  void* scan_s = slot + kGhostCats * (nn + 1);
  const size_t scan_b = sph_scan_scratch_bytes(n);
  if (n == 0) {
    cudaMemsetAsync(counts, 0, kGhostCats * sizeof(int32_t), st);
    SPH_CHECK_LAUNCH("periodic_ghosts");
    return SPH_OK;
  }
  k_ghost_flags<<<grid_for(n, 256), 256, 0, st>>>(reinterpret_cast<const float2*>(pos), n, B, flags);
  for (int c = 0; c < kGhostCats; ++c) {
    sph_status_t s = sph_exclusive_scan_i32(flags + c * n, slot + c * (n + 1), n, scan_s, scan_b, stream);
    if (s != SPH_OK) return s;
  }
  k_ghost_fill<<<grid_for(n, 256), 256, 0, st>>>(reinterpret_cast<const float2*>(pos), n, B, slot, capacity, indices,
                                                 reinterpret_cast<float2*>(offsets), counts, status);
  SPH_CHECK_LAUNCH("periodic_ghosts");
  return SPH_OK;
}

size_t sph_nl_periodic_scratch_bytes(int64_t n, const float* domain_min, const float* domain_max, float cell_size) {
  const size_t nn = (size_t)(n > 0 ? n : 1);
  int cells = 1;
  if (domain_min && domain_max && cell_size > 0.f) {
    const double cx = floor(((double)domain_max[0] - domain_min[0]) / cell_size);
    const double cy = floor(((double)domain_max[1] - domain_min[1]) / cell_size);
    if (cx >= 1 && cy >= 1 && cx * cy < (double)(1 << 28)) cells = (int)(cx * cy);
  }
  return nn * 4 * 4 + nn * 8 + ((size_t)cells + 2) * 4 * 2 + sph_counting_sort_scratch_bytes(n, cells) +
         sph_scan_scratch_bytes(n) + 4096;
}

}  // extern "C"

namespace {

// The periodic grid and the particles sorted into it (both passes rebuild it from `pos`).
struct PSorted {
  PGrid G;
  uint32_t* order;
  float2* spos;
  int32_t* cell_start;
  int32_t* counts;
  void* scan_s;
  size_t scan_b;
};

sph_status_t periodic_setup(const float* pos, int64_t n, const float* domain_min, const float* domain_max,
                            float cell_size, int32_t periodic_x, int32_t periodic_y, int32_t* status, void* scratch,
                            size_t scratch_bytes, cudaStream_t st, PSorted* S) {
  SPH_REQUIRE(n > 0 && n < (1LL << 31) && pos && status && domain_min && domain_max && cell_size > 0.f,
              "nl_periodic: bad arguments");
  PGrid& G = S->G;
  G.minx = domain_min[0];
  G.miny = domain_min[1];
  const double Lx = (double)domain_max[0] - domain_min[0], Ly = (double)domain_max[1] - domain_min[1];
  SPH_REQUIRE(Lx > 0 && Ly > 0, "nl_periodic: empty domain");
  G.lx = (float)Lx;
  G.ly = (float)Ly;
  G.cx = (int)floor(Lx / cell_size);
  G.cy = (int)floor(Ly / cell_size);
  G.px = periodic_x != 0;
  G.py = periodic_y != 0;
  SPH_REQUIRE(G.cx >= 1 && G.cy >= 1 && (double)G.cx * G.cy < (double)(1 << 28), "nl_periodic: too many cells");
  G.wx = (float)(Lx / G.cx);
  G.wy = (float)(Ly / G.cy);
  // cell widths rounded to float may fall below the support: keep them at or above it
  while (G.wx < cell_size && G.cx > 1) G.wx = (float)(Lx / --G.cx);
  while (G.wy < cell_size && G.cy > 1) G.wy = (float)(Ly / --G.cy);
  SPH_REQUIRE((!G.px || G.cx >= 3) && (!G.py || G.cy >= 3),
              "nl_periodic: a periodic direction needs a box of at least three supports");
  const int cells = G.cx * G.cy;
  if (!scratch || scratch_bytes < sph_nl_periodic_scratch_bytes(n, domain_min, domain_max, cell_size)) {
    set_error_text("nl_periodic: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  char* p = static_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  const size_t nn = (size_t)n;
  uint32_t* keys = reinterpret_cast<uint32_t*>(take(nn * 4));
  S->order = reinterpret_cast<uint32_t*>(take(nn * 4));
  uint32_t* skeys = reinterpret_cast<uint32_t*>(take(nn * 4));
  S->counts = reinterpret_cast<int32_t*>(take(nn * 4));
  S->spos = reinterpret_cast<float2*>(take(nn * 8));
  int32_t* cell_count = reinterpret_cast<int32_t*>(take(((size_t)cells + 2) * 4));
  S->cell_start = reinterpret_cast<int32_t*>(take(((size_t)cells + 2) * 4));
  const size_t cs_b = sph_counting_sort_scratch_bytes(n, cells);
  void* cs_s = take(cs_b);
  S->scan_b = sph_scan_scratch_bytes(n);
  S->scan_s = take(S->scan_b);
  cudaMemsetAsync(cell_count, 0, ((size_t)cells + 1) * 4, st);
  k_pcell_keys<<<grid_for(n, 256), 256, 0, st>>>(reinterpret_cast<const float2*>(pos), n, G, keys, cell_count,
                                                 status);
  sph_status_t s = sph_counting_sort(keys, n, cells, cell_count, S->cell_start, S->order, skeys, status, cs_s, cs_b,
                                     st);
  if (s != SPH_OK) return s;
  k_gather_f2<<<grid_for(n, 256), 256, 0, st>>>(S->order, n, reinterpret_cast<const float2*>(pos), S->spos);
  SPH_CHECK_LAUNCH("nl_periodic(grid)");
  return SPH_OK;
}

}  // namespace

extern "C" {

sph_status_t sph_nl_periodic_count(const float* pos, const float* support, int64_t n, const float* domain_min,
                                   const float* domain_max, float cell_size, int32_t periodic_x, int32_t periodic_y,
                                   int64_t* offsets, int32_t* status, void* scratch, size_t scratch_bytes,
                                   void* stream) {
  SPH_REQUIRE(support && offsets, "nl_periodic_count: bad arguments");
  cudaStream_t st = as_stream(stream);
  PSorted S;
  sph_status_t s = periodic_setup(pos, n, domain_min, domain_max, cell_size, periodic_x, periodic_y, status, scratch,
                                  scratch_bytes, st, &S);
  if (s != SPH_OK) return s;
  k_periodic_count<<<grid_for(n, 128), 128, 0, st>>>(reinterpret_cast<const float2*>(pos), support, n, S.spos,
                                                     S.order, S.cell_start, S.G, S.counts);
  s = sph_exclusive_scan_i32_to_i64(S.counts, offsets, n, S.scan_s, S.scan_b, stream);
  if (s != SPH_OK) return s;
  SPH_CHECK_LAUNCH("nl_periodic_count");
  return SPH_OK;
}

sph_status_t sph_nl_periodic_fill(const float* pos, const float* support, int64_t n, const float* domain_min,
                                  const float* domain_max, float cell_size, int32_t periodic_x, int32_t periodic_y,
                                  const int64_t* offsets, int64_t capacity, int64_t* rows, int64_t* cols,
                                  int8_t* codes, int32_t* status, void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(support && offsets && capacity >= 0 && (capacity == 0 || (rows && cols && codes)),
              "nl_periodic_fill: bad arguments");
  cudaStream_t st = as_stream(stream);
  PSorted S;
  sph_status_t s = periodic_setup(pos, n, domain_min, domain_max, cell_size, periodic_x, periodic_y, status, scratch,
                                  scratch_bytes, st, &S);
  if (s != SPH_OK) return s;
  k_periodic_fill<<<grid_for(n, 128), 128, 0, st>>>(reinterpret_cast<const float2*>(pos), support, n, S.spos,
                                                    S.order, S.cell_start, S.G, offsets, capacity, cols, codes,
                                                    status);
  k_periodic_rows<<<grid_for(n, 256), 256, 0, st>>>(offsets, n, rows);
  SPH_CHECK_LAUNCH("nl_periodic_fill");
  return SPH_OK;
}

}  // extern "C"
