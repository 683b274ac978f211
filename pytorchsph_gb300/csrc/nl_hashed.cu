// Drop-in neighbor-list kernels over the reference's own hash-table format
// (hashTable [L,2] = (first slot, #cells), cellIndices / cumCell (= counts) /
// cellSpan (= begins) in hash order; src/modules/neighborSearch.py:58-88).  They reproduce
// the pair sets of cppSrc/neighSearch.cpp:172-410 and cppSrc/neighSearch_cuda.cu:101-209,
// two passes each (count, then fill at scanned int64 offsets).
#include "sph_common.cuh"

namespace sph {

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
  const float thr = sq_threshold(qh[b]);
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
        if (dist2_ref(xi.x, xi.y, xj.x, xj.y) <= thr) {
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
        const float thr = sq_threshold(sh[i]);
        for (int j = rg.x; j < rg.y; ++j) {
          float2 xj = spos[j];
          if (dist2_ref(xi.x, xi.y, xj.x, xj.y) <= thr) {
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
        const float thr = sq_threshold(ha[i]);
        for (int j = rg.x; j < rg.y; ++j) {
          float2 xj = pb[j];
          if (dist2_ref(xi.x, xi.y, xj.x, xj.y) <= thr) {
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

}  // namespace sph

using namespace sph;

extern "C" {

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

}  // extern "C"
