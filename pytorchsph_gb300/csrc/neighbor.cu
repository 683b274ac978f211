// Hashed-grid neighbor search on sm_103a.
//
// Native pipeline (particles re-ordered by cell key, dense cell table, CSR pairs):
//   sph_grid_build -> sph_cell_keys -> sph_radix_sort_pairs -> sph_gather_packed
//   -> sph_cell_starts -> sph_nl_count (+ fused density) -> scan -> sph_nl_fill
// In the sorted order the three cells (cx-1..cx+1, cy) of one grid row are contiguous,
// so a particle visits 2r+1 contiguous ranges instead of (2r+1)^2 hash lookups.
//
// Drop-in kernels (sph_nl_hashed_*) consume the reference's own hash-table format
// (src/modules/neighborSearch.py:58-88) and reproduce the pair sets of
// cppSrc/neighSearch.cpp:172-410 and cppSrc/neighSearch_cuda.cu:101-209.
#include <cstdio>

#include "sph_common.cuh"

namespace sph {

// ------------------------------------------------------------------ grid
constexpr int kRedThreads = 256;

struct Bounds {
  float hmax, mnx, mny, mxx, mxy;
  int nonfinite;
};

__global__ void __launch_bounds__(kRedThreads) k_bounds_partial(const float2* __restrict__ pos,
                                                                const float* __restrict__ h, int64_t n,
                                                                Bounds* __restrict__ part) {
  float hm = -INFINITY, mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  int bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float2 p = pos[i];
    float hv = h[i];
    if (!isfinite(p.x) || !isfinite(p.y) || !isfinite(hv)) bad = 1;
    hm = fmaxf(hm, hv);
    mnx = fminf(mnx, p.x);
    mny = fminf(mny, p.y);
    mxx = fmaxf(mxx, p.x);
    mxy = fmaxf(mxy, p.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  __shared__ Bounds sb[kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sb[warp] = Bounds{hm, mnx, mny, mxx, mxy, bad};
  __syncthreads();
  if (threadIdx.x == 0) {
    Bounds b = sb[0];
    for (int w = 1; w < kRedThreads / 32; ++w) {
      b.hmax = fmaxf(b.hmax, sb[w].hmax);
      b.mnx = fminf(b.mnx, sb[w].mnx);
      b.mny = fminf(b.mny, sb[w].mny);
      b.mxx = fmaxf(b.mxx, sb[w].mxx);
      b.mxy = fmaxf(b.mxy, sb[w].mxy);
      b.nonfinite |= sb[w].nonfinite;
    }
    part[blockIdx.x] = b;
  }
}

// Grid of sortPositions, src/modules/neighborSearch.py:34-46, all in float32:
// qMin = minCoord - hMax*1.0, qMax = maxCoord + 2*hMax*1.0, cells = ceil((qMax-qMin)/hMax).
__global__ void k_bounds_final(const Bounds* __restrict__ part, int nparts, int has_min, float min_x, float min_y,
                               int has_max, float max_x, float max_y, int32_t cell_capacity, sph_grid* grid,
                               int32_t* status) {
  if (threadIdx.x != 0) return;
  Bounds b = part[0];
  for (int k = 1; k < nparts; ++k) {
    b.hmax = fmaxf(b.hmax, part[k].hmax);
    b.mnx = fminf(b.mnx, part[k].mnx);
    b.mny = fminf(b.mny, part[k].mny);
    b.mxx = fmaxf(b.mxx, part[k].mxx);
    b.mxy = fmaxf(b.mxy, part[k].mxy);
    b.nonfinite |= part[k].nonfinite;
  }
  float hs = __fmul_rn(b.hmax, 1.0f);
  float two_hs = __fmul_rn(__fmul_rn(2.0f, b.hmax), 1.0f);
  float qmin_x = __fsub_rn(has_min ? min_x : b.mnx, hs);
  float qmin_y = __fsub_rn(has_min ? min_y : b.mny, hs);
  float qmax_x = __fadd_rn(has_max ? max_x : b.mxx, two_hs);
  float qmax_y = __fadd_rn(has_max ? max_y : b.mxy, two_hs);
  float ex = __fdiv_rn(__fsub_rn(qmax_x, qmin_x), hs);
  float ey = __fdiv_rn(__fsub_rn(qmax_y, qmin_y), hs);
  sph_grid g;
  g.qmin[0] = qmin_x;
  g.qmin[1] = qmin_y;
  g.hmax = b.hmax;
  g.reserved = 0.f;
  g.reserved2 = 0;
  bool ok = b.nonfinite == 0 && b.hmax > 0.f && isfinite(ex) && isfinite(ey) && ex < 2.0e9f && ey < 2.0e9f;
  int cx = ok ? (int)ceilf(ex) : 0;
  int cy = ok ? (int)ceilf(ey) : 0;
  long long nc = (long long)cx * (long long)cy;
  if (!ok) flag(status, SPH_FLAG_NONFINITE);
  if (nc > (long long)cell_capacity) {
    flag(status, SPH_FLAG_CELL_CAPACITY);
  }
  g.cells_x = cx;
  g.cells_y = cy;
  g.num_cells = nc > (long long)cell_capacity ? cell_capacity + 1 : (int)nc;
  *grid = g;
}

// A grid is usable only if its cells fit the cell table.
__device__ __forceinline__ bool grid_ok(const sph_grid& g, int32_t cap) {
  return g.num_cells <= cap && g.cells_x > 0 && g.cells_y > 0;
}

__global__ void k_cell_keys(const float2* __restrict__ pos, int64_t n, const sph_grid* __restrict__ gp,
                            int32_t cell_capacity, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                            int32_t* status) {
  const sph_grid g = *gp;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 p = pos[i];
  uint32_t key = (uint32_t)cell_capacity;  // sentinel: sorts last, never searched
  if (!isfinite(p.x) || !isfinite(p.y)) {
    flag(status, SPH_FLAG_NONFINITE);
  } else if (grid_ok(g, cell_capacity)) {
    int ix = cell_coord(p.x, g.qmin[0], g.hmax);
    int iy = cell_coord(p.y, g.qmin[1], g.hmax);
    if (ix >= 0 && iy >= 0 && ix < g.cells_x && iy < g.cells_y)
      key = (uint32_t)(ix + g.cells_x * iy);
    else
      flag(status, SPH_FLAG_OUT_OF_GRID);
  }
  keys[i] = key;
  vals[i] = (uint32_t)i;
}

// cell_start[c] = lower_bound(sorted_keys, c).  One thread per cell; a binary search over
// the (L2-resident) key array needs no clearing pass and no long serial gap fills.
__global__ void k_cell_starts(const uint32_t* __restrict__ keys, int64_t n, int32_t cap,
                              int32_t* __restrict__ cell_start) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > cap) return;
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if ((int64_t)keys[mid] < c) lo = mid + 1; else hi = mid;
  }
  cell_start[c] = (int32_t)lo;
}

__global__ void k_gather_packed(const uint32_t* __restrict__ order, int64_t n, const float2* __restrict__ pos,
                                const float* __restrict__ h, const float* __restrict__ a, float4* __restrict__ out) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint32_t o = order[s];
  float2 p = pos[o];
  out[s] = make_float4(p.x, p.y, h ? h[o] : 0.f, a ? a[o] : 0.f);
}

// ------------------------------------------------------------------ CSR search
// Visits every candidate j of sorted particle s in the fixed order
// (row cy-r .. cy+r, then ascending sorted index) and calls f(j, dist) for pairs.
template <typename F>
__device__ __forceinline__ void for_each_neighbor(const float4* __restrict__ packed, const int32_t* __restrict__ cell_start,
                                                  const sph_grid& g, int r, uint32_t key, float4 pi, F&& f) {
  const int cx = (int)(key % (uint32_t)g.cells_x);
  const int cy = (int)(key / (uint32_t)g.cells_x);
  const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
  for (int yy = max(cy - r, 0); yy <= min(cy + r, g.cells_y - 1); ++yy) {
    const int row = yy * g.cells_x;
    const int b = __ldg(cell_start + row + x0);
    const int e = __ldg(cell_start + row + x1 + 1);
    for (int j = b; j < e; ++j) {
      float4 pj = __ldg(packed + j);
      float d;
      if (pair_pred(pi.x, pi.y, pj.x, pj.y, pi.z, &d)) f(j, d, pj);
    }
  }
}

__global__ void __launch_bounds__(256) k_nl_count(const float4* __restrict__ packed, int64_t n,
                                                  const uint32_t* __restrict__ keys,
                                                  const int32_t* __restrict__ cell_start,
                                                  const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                  float inv_support, float c_w, int32_t* __restrict__ counts,
                                                  float* __restrict__ rho) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const sph_grid g = *gp;
  uint32_t key = keys[s];
  int cnt = 0;
  float acc = 0.f;
  if (grid_ok(g, cap) && key < (uint32_t)g.num_cells) {
    float4 pi = packed[s];
    if (rho) {
      for_each_neighbor(packed, cell_start, g, r, key, pi, [&](int, float d, float4 pj) {
        ++cnt;
        acc += wendland(d * inv_support, c_w) * pj.w;
      });
    } else {
      for_each_neighbor(packed, cell_start, g, r, key, pi, [&](int, float, float4) { ++cnt; });
    }
  }
  counts[s] = cnt;
  if (rho) rho[s] = acc;
}

__global__ void __launch_bounds__(256) k_nl_fill(const float4* __restrict__ packed, int64_t n,
                                                 const uint32_t* __restrict__ keys,
                                                 const int32_t* __restrict__ cell_start,
                                                 const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                 const int32_t* __restrict__ offsets, int64_t pair_capacity,
                                                 int32_t* __restrict__ cols, int32_t* status) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const sph_grid g = *gp;
  uint32_t key = keys[s];
  if (!(grid_ok(g, cap) && key < (uint32_t)g.num_cells)) return;
  if ((int64_t)offsets[s + 1] > pair_capacity) {  // the row does not fit: write nothing
    flag(status, SPH_FLAG_PAIR_CAPACITY);
    return;
  }
  float4 pi = packed[s];
  int32_t o = offsets[s];
  for_each_neighbor(packed, cell_start, g, r, key, pi, [&](int j, float, float4) { cols[o++] = j; });
}

// Query points (any order, e.g. wall or ghost particles) against the sorted grid, with
// the query's own support in the predicate (dx = x_query - x_j): the pair set of
// buildNeighborListUnsortedPerParticle, cppSrc/neighSearch.cpp:261-331.
__device__ __forceinline__ bool query_cell(float x, float qmin, float hmax, int* c) {
  float v = ceilf(__fdiv_rn(__fsub_rn(x, qmin), hmax));
  if (!(v > -1.0e9f && v < 1.0e9f)) return false;
  *c = (int)v;
  return true;
}

template <bool kFill>
__global__ void __launch_bounds__(128) k_nl_query(const float2* __restrict__ qpos, const float* __restrict__ qh, int64_t m,
                                                  const float4* __restrict__ packed,
                                                  const int32_t* __restrict__ cell_start,
                                                  const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                  const uint32_t* __restrict__ order, int32_t* __restrict__ counts,
                                                  const int64_t* __restrict__ offsets, int32_t* __restrict__ rows,
                                                  int32_t* __restrict__ cols) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m) return;
  const sph_grid g = *gp;
  int cnt = 0;
  int64_t o = kFill ? offsets[b] : 0;
  float2 xi = qpos[b];
  float hi = qh[b];
  int qx, qy;
  if (grid_ok(g, cap) && query_cell(xi.x, g.qmin[0], g.hmax, &qx) && query_cell(xi.y, g.qmin[1], g.hmax, &qy)) {
    const int x0 = max(qx - r, 0), x1 = min(qx + r, g.cells_x - 1);
    const int y0 = max(qy - r, 0), y1 = min(qy + r, g.cells_y - 1);
    if (x0 <= x1) {
      for (int yy = y0; yy <= y1; ++yy) {
        const int row = yy * g.cells_x;
        const int jb = cell_start[row + x0], je = cell_start[row + x1 + 1];
        for (int j = jb; j < je; ++j) {
          float4 pj = packed[j];
          float d;
          if (pair_pred(xi.x, xi.y, pj.x, pj.y, hi, &d)) {
            if (kFill) {
              rows[o + cnt] = (int32_t)b;
              cols[o + cnt] = order ? (int32_t)order[j] : j;
            }
            ++cnt;
          }
        }
      }
    }
  }
  if (!kFill) counts[b] = cnt;
}

__global__ void k_invert_perm(const uint32_t* __restrict__ order, int64_t n, uint32_t* __restrict__ rank) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) rank[order[s]] = (uint32_t)s;
}

__global__ void k_scatter_f32(const uint32_t* __restrict__ order, const float* __restrict__ in, int64_t n,
                              float* __restrict__ out) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[order[s]] = in[s];
}

__global__ void k_scatter_counts(const uint32_t* __restrict__ order, const int32_t* __restrict__ counts, int64_t n,
                                 int32_t* __restrict__ out) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[order[s]] = counts[s];
}

// One thread per original particle i: its row of the (i, j)-ordered COO list.
__global__ void k_nl_to_coo(const float4* __restrict__ packed, int64_t n, const uint32_t* __restrict__ order,
                            const uint32_t* __restrict__ rank, const int32_t* __restrict__ offsets,
                            const int32_t* __restrict__ cols, const int64_t* __restrict__ orig_offsets,
                            float thr, float support, int64_t* __restrict__ pairs, int64_t P,
                            float* __restrict__ dist, float* __restrict__ radial) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = rank[i];
  const int32_t b = offsets[s], e = offsets[s + 1];
  const int64_t o = orig_offsets[i];
  int64_t* prow = pairs;
  int64_t* pcol = pairs + P;
  for (int k = b; k < e; ++k) {  // insertion sort by original column index
    int64_t jo = (int64_t)order[cols[k]];
    int64_t t = o + (k - b);
    while (t > o && pcol[t - 1] > jo) {
      pcol[t] = pcol[t - 1];
      --t;
    }
    pcol[t] = jo;
  }
  const float4 pi = packed[s];
  for (int k = 0; k < e - b; ++k) {
    prow[o + k] = i;
    if (dist || radial) {
      float4 pj = packed[rank[pcol[o + k]]];
      float dx = pi.x - pj.x, dy = pi.y - pj.y;
      float rr = sqrtf(dx * dx + dy * dy);
      if (dist) {
        if (rr < thr) {
          dist[2 * (o + k)] = 0.f;
          dist[2 * (o + k) + 1] = 0.f;
        } else {
          dist[2 * (o + k)] = dx / rr;
          dist[2 * (o + k) + 1] = dy / rr;
        }
      }
      if (radial) radial[o + k] = rr / support;
    }
  }
}

// ------------------------------------------------------------------ hash map (constructHashMap)
__global__ void k_cell_heads(const uint32_t* __restrict__ keys, int64_t n, int32_t* __restrict__ head) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) head[s] = (s == 0 || keys[s] != keys[s - 1]) ? 1 : 0;
}

__global__ void k_cell_compact(const uint32_t* __restrict__ keys, int64_t n, const int32_t* __restrict__ head,
                               const int32_t* __restrict__ slot, int32_t cells_x, int32_t L,
                               int32_t* __restrict__ c_lin, int32_t* __restrict__ c_begin,
                               uint32_t* __restrict__ c_hash, uint32_t* __restrict__ c_id) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !head[s]) return;
  int32_t c = slot[s];
  int32_t lin = (int32_t)keys[s];
  c_lin[c] = lin;
  c_begin[c] = (int32_t)s;
  long long x = lin % cells_x, y = lin / cells_x;
  c_hash[c] = (uint32_t)((x * 3 + y * 5) % L);
  c_id[c] = (uint32_t)c;
}

__global__ void k_cell_emit(int64_t C, int64_t n, const uint32_t* __restrict__ c_id, const int32_t* __restrict__ c_lin,
                            const int32_t* __restrict__ c_begin, int32_t* __restrict__ cell_indices,
                            int32_t* __restrict__ cum_cell, int32_t* __restrict__ cell_span) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C) return;
  uint32_t c = c_id[k];
  int32_t b = c_begin[c];
  int32_t e = (int64_t)c + 1 < C ? c_begin[c + 1] : (int32_t)n;
  cell_indices[k] = c_lin[c];
  cum_cell[k] = e - b;
  cell_span[k] = b;
}

__global__ void k_table_init(int32_t* __restrict__ table, int32_t L) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < L) {
    table[2 * b] = -1;
    table[2 * b + 1] = 0;
  }
}

__global__ void k_table_fill(const uint32_t* __restrict__ sorted_hash, int64_t C, int32_t* __restrict__ table) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C) return;
  uint32_t hv = sorted_hash[k];
  if (k > 0 && sorted_hash[k - 1] == hv) return;
  int64_t e = k + 1;
  while (e < C && sorted_hash[e] == hv) ++e;
  table[2 * (int64_t)hv] = (int32_t)k;
  table[2 * (int64_t)hv + 1] = (int32_t)(e - k);
}

// ------------------------------------------------------------------ drop-in hashed kernels
// queryHashMap, cppSrc/neighSearch.cpp:93-114 / cppSrc/neighSearch_cuda.cu:76-99.
__device__ __forceinline__ int2 query_hash(int qx, int qy, const int32_t* __restrict__ table,
                                           const int32_t* __restrict__ ci, const int32_t* __restrict__ cc,
                                           const int32_t* __restrict__ cs, int cells_x, int L) {
  if (qx < 0 || qy < 0) return make_int2(-1, -1);
  int qlin = qx + cells_x * qy;
  // the reference computes this in int32; int64 keeps far-away query cells from
  // overflowing into a negative (out-of-table) bucket
  long long qh64 = ((long long)qx * 3 + (long long)qy * 5) % L;
  if (qh64 < 0 || qh64 >= L) return make_int2(-1, -1);
  int qh = (int)qh64;
  int first = table[2 * qh];
  if (first == -1) return make_int2(-1, -1);
  int last = first + table[2 * qh + 1];
  for (int k = first; k < last; ++k)
    if (ci[k] == qlin) return make_int2(cs[k], cs[k] + cc[k]);
  return make_int2(-1, -1);
}

template <bool kFill>
__global__ void k_hashed_query(const float2* __restrict__ qpos, const float* __restrict__ qh, int64_t m,
                               const float2* __restrict__ spos, const int32_t* __restrict__ table,
                               const int32_t* __restrict__ ci, const int32_t* __restrict__ cc,
                               const int32_t* __restrict__ cs, const int32_t* __restrict__ sort,
                               const float* __restrict__ qmin, float hmax, int cells_x, int L, int r,
                               int32_t* __restrict__ counts, const int64_t* __restrict__ offsets,
                               int32_t* __restrict__ rows, int32_t* __restrict__ cols) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m) return;
  float2 xi = qpos[b];
  float hi = qh[b];
  int qx = cell_coord(xi.x, qmin[0], hmax);
  int qy = cell_coord(xi.y, qmin[1], hmax);
  int cnt = 0;
  int64_t o = kFill ? offsets[b] : 0;
  for (int xx = -r; xx <= r; ++xx)
    for (int yy = -r; yy <= r; ++yy) {
      int2 rg = query_hash(qx + xx, qy + yy, table, ci, cc, cs, cells_x, L);
      if (rg.x == -1) continue;
      for (int j = rg.x; j < rg.y; ++j) {
        float2 xj = spos[j];
        float d;
        if (pair_pred(xi.x, xi.y, xj.x, xj.y, hi, &d)) {
          if (kFill) {
            rows[o + cnt] = (int32_t)b;
            cols[o + cnt] = sort[j];
          }
          ++cnt;
        }
      }
    }
  if (!kFill) counts[b] = cnt;
}

template <bool kFill>
__global__ void k_hashed_cells(const float2* __restrict__ spos, const float* __restrict__ sh,
                               const int32_t* __restrict__ table, const int32_t* __restrict__ ci,
                               const int32_t* __restrict__ cc, const int32_t* __restrict__ cs,
                               const int32_t* __restrict__ sort, int64_t C, int cells_x, int L, int r,
                               int32_t* __restrict__ counts, const int64_t* __restrict__ offsets,
                               int32_t* __restrict__ rows, int32_t* __restrict__ cols) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= C) return;
  int cell = ci[b];
  int qx = cell % cells_x, qy = cell / cells_x;
  int2 own = query_hash(qx, qy, table, ci, cc, cs, cells_x, L);
  int cnt = 0;
  int64_t o = kFill ? offsets[b] : 0;
  for (int xx = -r; xx <= r; ++xx)
    for (int yy = -r; yy <= r; ++yy) {
      int2 rg = query_hash(qx + xx, qy + yy, table, ci, cc, cs, cells_x, L);
      if (rg.x == -1) continue;
      for (int i = own.x; i < own.y; ++i) {
        float2 xi = spos[i];
        float hi = sh[i];
        for (int j = rg.x; j < rg.y; ++j) {
          float2 xj = spos[j];
          float d;
          if (pair_pred(xi.x, xi.y, xj.x, xj.y, hi, &d)) {
            if (kFill) {
              rows[o + cnt] = sort[i];
              cols[o + cnt] = sort[j];
            }
            ++cnt;
          }
        }
      }
    }
  if (!kFill) counts[b] = cnt;
}

template <bool kFill>
__global__ void k_hashed_asym(const float2* __restrict__ pa, const float* __restrict__ ha,
                              const int32_t* __restrict__ ta, const int32_t* __restrict__ cia,
                              const int32_t* __restrict__ cca, const int32_t* __restrict__ csa,
                              const int32_t* __restrict__ sa, int64_t Ca, const float2* __restrict__ pb,
                              const int32_t* __restrict__ tb, const int32_t* __restrict__ cib,
                              const int32_t* __restrict__ ccb, const int32_t* __restrict__ csb,
                              const int32_t* __restrict__ sb, int cells_x, int L, int32_t* __restrict__ counts,
                              const int64_t* __restrict__ offsets, int32_t* __restrict__ rows,
                              int32_t* __restrict__ cols) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= Ca) return;
  int cell = cia[b];
  int qx = cell % cells_x, qy = cell / cells_x;
  int2 own = query_hash(qx, qy, ta, cia, cca, csa, cells_x, L);
  int cnt = 0;
  int64_t o = kFill ? offsets[b] : 0;
  for (int xx = -1; xx <= 1; ++xx)
    for (int yy = -1; yy <= 1; ++yy) {
      int2 rg = query_hash(qx + xx, qy + yy, tb, cib, ccb, csb, cells_x, L);
      if (rg.x == -1) continue;
      for (int i = own.x; i < own.y; ++i) {
        float2 xi = pa[i];
        float hi = ha[i];
        for (int j = rg.x; j < rg.y; ++j) {
          float2 xj = pb[j];
          float d;
          if (pair_pred(xi.x, xi.y, xj.x, xj.y, hi, &d)) {
            if (kFill) {
              rows[o + cnt] = sa[i];
              cols[o + cnt] = sb[j];
            }
            ++cnt;
          }
        }
      }
    }
  if (!kFill) counts[b] = cnt;
}

static int key_bits_for(int64_t v) {
  int b = 0;
  while (b < 32 && (((int64_t)1 << b) <= v)) ++b;
  return b;
}

}  // namespace sph

using namespace sph;

extern "C" {

size_t sph_grid_scratch_bytes(int64_t) { return (size_t)(2 * kNumSMs) * sizeof(Bounds) + 64; }

sph_status_t sph_grid_build(const float* pos, const float* support, int64_t n, const float* min_coord,
                            const float* max_coord, int32_t cell_capacity, sph_grid* grid, int32_t* status,
                            void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n > 0 && pos && support && grid && cell_capacity > 0, "grid_build: bad arguments");
  if (!scratch || scratch_bytes < sph_grid_scratch_bytes(n)) {
    set_error_text("grid_build: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  int nparts = (int)std::min<int64_t>(2 * kNumSMs, (n + kRedThreads - 1) / kRedThreads);
  Bounds* part = reinterpret_cast<Bounds*>(scratch);
  k_bounds_partial<<<nparts, kRedThreads, 0, st>>>(reinterpret_cast<const float2*>(pos), support, n, part);
  k_bounds_final<<<1, 32, 0, st>>>(part, nparts, min_coord != nullptr, min_coord ? min_coord[0] : 0.f,
                                   min_coord ? min_coord[1] : 0.f, max_coord != nullptr,
                                   max_coord ? max_coord[0] : 0.f, max_coord ? max_coord[1] : 0.f, cell_capacity,
                                   grid, status);
  SPH_CHECK_LAUNCH("grid_build");
  return SPH_OK;
}

sph_status_t sph_cell_keys(const float* pos, int64_t n, const sph_grid* grid, int32_t cell_capacity,
                               uint32_t* keys, uint32_t* vals, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && pos && grid && keys && vals && cell_capacity > 0, "cell_keys: bad arguments");
  if (n == 0) return SPH_OK;
  k_cell_keys<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(pos), n, grid,
                                                               cell_capacity, keys, vals, status);
  SPH_CHECK_LAUNCH("cell_keys");
  return SPH_OK;
}

int32_t sph_key_bits(int32_t cell_capacity) { return key_bits_for(cell_capacity); }

sph_status_t sph_cell_starts(const uint32_t* sorted_keys, int64_t n, int32_t cell_capacity, int32_t* cell_start,
                             void* stream) {
  SPH_REQUIRE(n >= 0 && cell_capacity > 0 && cell_start && (n == 0 || sorted_keys), "cell_starts: bad arguments");
  k_cell_starts<<<grid_for((int64_t)cell_capacity + 1, 256), 256, 0, as_stream(stream)>>>(sorted_keys, n,
                                                                                           cell_capacity, cell_start);
  SPH_CHECK_LAUNCH("cell_starts");
  return SPH_OK;
}

sph_status_t sph_gather_packed(const uint32_t* order, int64_t n, const float* pos, const float* support,
                               const float* area, float* packed, void* stream) {
  SPH_REQUIRE(n >= 0 && order && pos && packed, "gather_packed: bad arguments");
  if (n == 0) return SPH_OK;
  k_gather_packed<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      order, n, reinterpret_cast<const float2*>(pos), support, area, reinterpret_cast<float4*>(packed));
  SPH_CHECK_LAUNCH("gather_packed");
  return SPH_OK;
}

sph_status_t sph_nl_count(const float* packed, int64_t n, const uint32_t* sorted_keys, const int32_t* cell_start,
                              const sph_grid* grid, int32_t cell_capacity, int32_t search_radius,
                              float kernel_support, int32_t* counts, float* rho, void* stream) {
  SPH_REQUIRE(n >= 0 && packed && sorted_keys && cell_start && grid && counts && search_radius >= 0,
              "nl_count: bad arguments");
  SPH_REQUIRE(!rho || kernel_support > 0.f, "nl_count: kernel_support must be > 0");
  if (n == 0) return SPH_OK;
  float inv = rho ? 1.0f / kernel_support : 0.f;
  float cw = rho ? (float)(7.0 / 3.14159265358979323846) / (kernel_support * kernel_support) : 0.f;
  k_nl_count<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float4*>(packed), n,
                                                               sorted_keys, cell_start, grid, cell_capacity,
                                                               search_radius, inv, cw, counts, rho);
  SPH_CHECK_LAUNCH("nl_count");
  return SPH_OK;
}

sph_status_t sph_nl_fill(const float* packed, int64_t n, const uint32_t* sorted_keys, const int32_t* cell_start,
                             const sph_grid* grid, int32_t cell_capacity, int32_t search_radius,
                             const int32_t* offsets, int64_t pair_capacity, int32_t* cols, int32_t* status,
                             void* stream) {
  SPH_REQUIRE(n >= 0 && packed && sorted_keys && cell_start && grid && offsets && cols, "nl_fill: bad arguments");
  if (n == 0) return SPH_OK;
  k_nl_fill<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float4*>(packed), n,
                                                              sorted_keys, cell_start, grid, cell_capacity,
                                                              search_radius, offsets, pair_capacity, cols, status);
  SPH_CHECK_LAUNCH("nl_fill");
  return SPH_OK;
}

sph_status_t sph_invert_permutation(const uint32_t* order, int64_t n, uint32_t* rank, void* stream) {
  SPH_REQUIRE(n >= 0 && order && rank, "invert_permutation: bad arguments");
  if (n == 0) return SPH_OK;
  k_invert_perm<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, n, rank);
  SPH_CHECK_LAUNCH("invert_permutation");
  return SPH_OK;
}

sph_status_t sph_scatter_counts(const uint32_t* order, const int32_t* counts, int64_t n, int32_t* out, void* stream) {
  SPH_REQUIRE(n >= 0 && order && counts && out, "scatter_counts: bad arguments");
  if (n == 0) return SPH_OK;
  k_scatter_counts<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, counts, n, out);
  SPH_CHECK_LAUNCH("scatter_counts");
  return SPH_OK;
}

sph_status_t sph_scatter_f32(const uint32_t* order, const float* in, int64_t n, float* out, void* stream) {
  SPH_REQUIRE(n >= 0 && order && in && out, "scatter_f32: bad arguments");
  if (n == 0) return SPH_OK;
  k_scatter_f32<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, in, n, out);
  SPH_CHECK_LAUNCH("scatter_f32");
  return SPH_OK;
}

sph_status_t sph_nl_to_coo(const float* packed, int64_t n, const uint32_t* order, const uint32_t* rank,
                           const int32_t* offsets, const int32_t* cols, const int64_t* orig_offsets,
                           float grad_threshold, float kernel_support, int64_t* pairs, int64_t num_pairs,
                           float* dist, float* radial, void* stream) {
  SPH_REQUIRE(n >= 0 && packed && order && rank && offsets && cols && orig_offsets && pairs,
              "nl_to_coo: bad arguments");
  if (n == 0) return SPH_OK;
  k_nl_to_coo<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(reinterpret_cast<const float4*>(packed), n, order,
                                                                rank, offsets, cols, orig_offsets, grad_threshold,
                                                                kernel_support, pairs, num_pairs, dist, radial);
  SPH_CHECK_LAUNCH("nl_to_coo");
  return SPH_OK;
}

// constructHashMap on the GPU -------------------------------------------------------
size_t sph_hash_map_scratch_bytes(int64_t n, int32_t hash_len) {
  size_t nn = (size_t)(n < 1 ? 1 : n) + 1;
  size_t b = 0;
  b += nn * sizeof(int32_t) * 2;  // head, slot(n+1)
  b += nn * sizeof(int32_t) * 2;  // c_lin, c_begin
  b += nn * sizeof(uint32_t) * 2; // c_hash, c_id
  b += sph_scan_scratch_bytes(n) + 64;
  b += sph_radix_sort_scratch_bytes(n, 8) + 64;
  (void)hash_len;
  return b + 1024;
}

sph_status_t sph_hash_map_build(const uint32_t* sorted_keys, int64_t n, int32_t cells_x, int32_t hash_len,
                                int32_t* hash_table, int32_t* cell_indices, int32_t* cum_cell, int32_t* cell_span,
                                int64_t* num_cells_out, void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n > 0 && n < ((int64_t)1 << 31) && sorted_keys && cells_x > 0 && hash_len > 0 && hash_table &&
                  cell_indices && cum_cell && cell_span && num_cells_out,
              "hash_map_build: bad arguments");
  if (!scratch || scratch_bytes < sph_hash_map_scratch_bytes(n, hash_len)) {
    set_error_text("hash_map_build: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  size_t nn = (size_t)n + 1;
  char* p = reinterpret_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  int32_t* head = reinterpret_cast<int32_t*>(take(nn * 4));
  int32_t* slot = reinterpret_cast<int32_t*>(take(nn * 4));
  int32_t* c_lin = reinterpret_cast<int32_t*>(take(nn * 4));
  int32_t* c_begin = reinterpret_cast<int32_t*>(take(nn * 4));
  uint32_t* c_hash = reinterpret_cast<uint32_t*>(take(nn * 4));
  uint32_t* c_id = reinterpret_cast<uint32_t*>(take(nn * 4));
  size_t scan_b = sph_scan_scratch_bytes(n);
  void* scan_s = take(scan_b);
  size_t rs_b = sph_radix_sort_scratch_bytes(n, 8);
  void* rs_s = take(rs_b);

  k_cell_heads<<<grid_for(n, 256), 256, 0, st>>>(sorted_keys, n, head);
  sph_status_t s = sph_exclusive_scan_i32(head, slot, n, scan_s, scan_b, stream);
  if (s != SPH_OK) return s;
  int32_t C32 = 0;
  cudaMemcpyAsync(&C32, slot + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  k_cell_compact<<<grid_for(n, 256), 256, 0, st>>>(sorted_keys, n, head, slot, cells_x, hash_len, c_lin, c_begin,
                                                   c_hash, c_id);
  SPH_CHECK_LAUNCH("hash_map_build(compact)");
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_error("hash_map_build(sync)", e);
    return SPH_ERR_CUDA;
  }
  int64_t C = C32;
  s = sph_radix_sort_pairs(c_hash, c_id, C, key_bits_for(hash_len - 1 > 0 ? hash_len - 1 : 1), 8, rs_s, rs_b,
                           stream);
  if (s != SPH_OK) return s;
  k_cell_emit<<<grid_for(C, 256), 256, 0, st>>>(C, n, c_id, c_lin, c_begin, cell_indices, cum_cell, cell_span);
  k_table_init<<<grid_for(hash_len, 256), 256, 0, st>>>(hash_table, hash_len);
  k_table_fill<<<grid_for(C, 256), 256, 0, st>>>(c_hash, C, hash_table);
  SPH_CHECK_LAUNCH("hash_map_build");
  *num_cells_out = C;
  return SPH_OK;
}

// drop-in hashed-table entry points ------------------------------------------------
sph_status_t sph_nl_hashed_query_count(const float* query_pos, const float* query_support, int64_t m,
                                       const float* sorted_pos, const int32_t* hash_table, const int32_t* cell_indices,
                                       const int32_t* cum_cell, const int32_t* cell_span, const float* qmin,
                                       float hmax, int32_t cells_x, int32_t hash_len, int32_t search_radius,
                                       int32_t* counts, void* stream) {
  SPH_REQUIRE(m >= 0 && hash_len > 0 && cells_x > 0 && hmax > 0.f && search_radius >= 0, "hashed_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_hashed_query<false><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float2*>(sorted_pos),
      hash_table, cell_indices, cum_cell, cell_span, nullptr, qmin, hmax, cells_x, hash_len, search_radius, counts,
      nullptr, nullptr, nullptr);
  SPH_CHECK_LAUNCH("hashed_query_count");
  return SPH_OK;
}

sph_status_t sph_nl_hashed_query_fill(const float* query_pos, const float* query_support, int64_t m,
                                      const float* sorted_pos, const int32_t* hash_table, const int32_t* cell_indices,
                                      const int32_t* cum_cell, const int32_t* cell_span, const int32_t* sort,
                                      const float* qmin, float hmax, int32_t cells_x, int32_t hash_len,
                                      int32_t search_radius, const int64_t* offsets, int32_t* rows, int32_t* cols,
                                      void* stream) {
  SPH_REQUIRE(m >= 0 && hash_len > 0 && cells_x > 0 && hmax > 0.f && search_radius >= 0, "hashed_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_hashed_query<true><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float2*>(sorted_pos),
      hash_table, cell_indices, cum_cell, cell_span, sort, qmin, hmax, cells_x, hash_len, search_radius, nullptr,
      offsets, rows, cols);
  SPH_CHECK_LAUNCH("hashed_query_fill");
  return SPH_OK;
}

sph_status_t sph_nl_hashed_cells_count(const float* sorted_pos, const float* sorted_support, const int32_t* hash_table,
                                       const int32_t* cell_indices, const int32_t* cum_cell, const int32_t* cell_span,
                                       int64_t num_cells, int32_t cells_x, int32_t hash_len, int32_t search_radius,
                                       int32_t* counts, void* stream) {
  SPH_REQUIRE(num_cells >= 0 && hash_len > 0 && cells_x > 0 && search_radius >= 0, "hashed_cells: bad arguments");
  if (num_cells == 0) return SPH_OK;
  k_hashed_cells<false><<<grid_for(num_cells, 64), 64, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(sorted_pos), sorted_support, hash_table, cell_indices, cum_cell, cell_span,
      nullptr, num_cells, cells_x, hash_len, search_radius, counts, nullptr, nullptr, nullptr);
  SPH_CHECK_LAUNCH("hashed_cells_count");
  return SPH_OK;
}

sph_status_t sph_nl_hashed_cells_fill(const float* sorted_pos, const float* sorted_support, const int32_t* hash_table,
                                      const int32_t* cell_indices, const int32_t* cum_cell, const int32_t* cell_span,
                                      const int32_t* sort, int64_t num_cells, int32_t cells_x, int32_t hash_len,
                                      int32_t search_radius, const int64_t* offsets, int32_t* rows, int32_t* cols,
                                      void* stream) {
  SPH_REQUIRE(num_cells >= 0 && hash_len > 0 && cells_x > 0 && search_radius >= 0, "hashed_cells: bad arguments");
  if (num_cells == 0) return SPH_OK;
  k_hashed_cells<true><<<grid_for(num_cells, 64), 64, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(sorted_pos), sorted_support, hash_table, cell_indices, cum_cell, cell_span,
      sort, num_cells, cells_x, hash_len, search_radius, nullptr, offsets, rows, cols);
  SPH_CHECK_LAUNCH("hashed_cells_fill");
  return SPH_OK;
}

sph_status_t sph_nl_hashed_asym_count(const float* pos_a, const float* support_a, const int32_t* table_a,
                                      const int32_t* cell_indices_a, const int32_t* cum_cell_a,
                                      const int32_t* cell_span_a, int64_t num_cells_a, const float* pos_b,
                                      const int32_t* table_b, const int32_t* cell_indices_b, const int32_t* cum_cell_b,
                                      const int32_t* cell_span_b, int32_t cells_x, int32_t hash_len, int32_t* counts,
                                      void* stream) {
  SPH_REQUIRE(num_cells_a >= 0 && hash_len > 0 && cells_x > 0, "hashed_asym: bad arguments");
  if (num_cells_a == 0) return SPH_OK;
  k_hashed_asym<false><<<grid_for(num_cells_a, 64), 64, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(pos_a), support_a, table_a, cell_indices_a, cum_cell_a, cell_span_a, nullptr,
      num_cells_a, reinterpret_cast<const float2*>(pos_b), table_b, cell_indices_b, cum_cell_b, cell_span_b, nullptr,
      cells_x, hash_len, counts, nullptr, nullptr, nullptr);
  SPH_CHECK_LAUNCH("hashed_asym_count");
  return SPH_OK;
}

sph_status_t sph_nl_hashed_asym_fill(const float* pos_a, const float* support_a, const int32_t* table_a,
                                     const int32_t* cell_indices_a, const int32_t* cum_cell_a,
                                     const int32_t* cell_span_a, const int32_t* sort_a, int64_t num_cells_a,
                                     const float* pos_b, const int32_t* table_b, const int32_t* cell_indices_b,
                                     const int32_t* cum_cell_b, const int32_t* cell_span_b, const int32_t* sort_b,
                                     int32_t cells_x, int32_t hash_len, const int64_t* offsets, int32_t* rows,
                                     int32_t* cols, void* stream) {
  SPH_REQUIRE(num_cells_a >= 0 && hash_len > 0 && cells_x > 0, "hashed_asym: bad arguments");
  if (num_cells_a == 0) return SPH_OK;
  k_hashed_asym<true><<<grid_for(num_cells_a, 64), 64, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(pos_a), support_a, table_a, cell_indices_a, cum_cell_a, cell_span_a, sort_a,
      num_cells_a, reinterpret_cast<const float2*>(pos_b), table_b, cell_indices_b, cum_cell_b, cell_span_b, sort_b,
      cells_x, hash_len, nullptr, offsets, rows, cols);
  SPH_CHECK_LAUNCH("hashed_asym_fill");
  return SPH_OK;
}

sph_status_t sph_nl_query_count(const float* query_pos, const float* query_support, int64_t m, const float* packed,
                                const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity,
                                int32_t search_radius, int32_t* counts, void* stream) {
  SPH_REQUIRE(m >= 0 && packed && cell_start && grid && counts && search_radius >= 0, "nl_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_nl_query<false><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float4*>(packed),
      cell_start, grid, cell_capacity, search_radius, nullptr, counts, nullptr, nullptr, nullptr);
  SPH_CHECK_LAUNCH("nl_query_count");
  return SPH_OK;
}

sph_status_t sph_nl_query_fill(const float* query_pos, const float* query_support, int64_t m, const float* packed,
                               const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity,
                               int32_t search_radius, const uint32_t* order, const int64_t* offsets, int32_t* rows,
                               int32_t* cols, void* stream) {
  SPH_REQUIRE(m >= 0 && packed && cell_start && grid && offsets && rows && cols && search_radius >= 0,
              "nl_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_nl_query<true><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float4*>(packed),
      cell_start, grid, cell_capacity, search_radius, order, nullptr, offsets, rows, cols);
  SPH_CHECK_LAUNCH("nl_query_fill");
  return SPH_OK;
}

}  // extern "C"
