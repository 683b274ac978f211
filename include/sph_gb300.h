/*
 * sph_gb300.h — C ABI of the GB300 (sm_103a) SPH hot path.
 *
 * Plain pointers and sizes only: every pointer below is a CUDA device pointer unless
 * its comment says "host".  Arrays are contiguous.  All entry points are asynchronous
 * on the given stream (a cudaStream_t passed as void*; NULL = legacy default stream)
 * unless their comment says they synchronise.  They return an sph_status_t; on
 * SPH_ERR_CUDA the CUDA error string is available from sph_last_error().
 *
 * Kernels that can meet bad data (particles outside the search grid, non-finite
 * values, a pair buffer that is too small) do not trap: they OR a flag into a device
 * status word (int32) that the caller passes in and reads when convenient.
 *
 * The reference interface each entry point replaces is cited beside it
 * (paths inside wi-re/pytorchSPH).
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t sph_status_t;
#define SPH_OK 0
#define SPH_ERR_INVALID_ARGUMENT 1
#define SPH_ERR_CUDA 2
#define SPH_ERR_SCRATCH_TOO_SMALL 3

/* Flags ORed into the device status word by kernels. */
#define SPH_FLAG_OUT_OF_GRID 1      /* a particle's cell lies outside the grid */
#define SPH_FLAG_NONFINITE 2        /* NaN/Inf met in positions or results */
#define SPH_FLAG_PAIR_CAPACITY 4    /* pair count exceeded the pair buffer */
#define SPH_FLAG_CELL_CAPACITY 8    /* grid has more cells than the cell table holds */
#define SPH_FLAG_ITERATION_CAP 16   /* an iterative solve stopped at its maximum iteration count */
#define SPH_FLAG_CELL_ORDER 32      /* a cell held > 2048 particles: their order inside the cell is
                                       not reproducible (the pair set is unaffected) */

/* Uniform search grid, the device-side form of what sortPositions computes
 * (src/modules/neighborSearch.py:30-55): cell size hmax, origin qmin,
 * cell (ix, iy) = ceil((x - qmin) / hmax), linear id ix + cells_x * iy. */
typedef struct sph_grid {
  float qmin[2];
  float hmax;
  float reserved;
  int32_t cells_x;
  int32_t cells_y;
  int32_t num_cells;
  int32_t reserved2;
} sph_grid;

int32_t sph_abi_version(void);
const char* sph_last_error(void);
const char* sph_status_string(sph_status_t status);

/* ---------------------------------------------------------------- primitives */

/* Scratch bytes sph_exclusive_scan_* needs for n items. */
size_t sph_scan_scratch_bytes(int64_t n);
/* out[k] = in[0] + ... + in[k-1] for k <= n (out has n+1 entries; out[n] = total).
 * Replaces torch::cumsum in cppSrc/neighSearch_cuda.cu:250 and the cumsums of
 * src/modules/neighborSearch.py:65,86. */
sph_status_t sph_exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch,
                                    size_t scratch_bytes, void* stream);
sph_status_t sph_exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, void* scratch,
                                           size_t scratch_bytes, void* stream);

/* Allocation-free variant of sph_exclusive_scan_i32.  It has no counterpart in the
 * reference; it exists for callers that cannot allocate device memory: a host runtime
 * bound through this C ABI that only receives device pointers from another owner of
 * GPU memory, or code recording a CUDA graph, where cudaMalloc is not permitted.  The
 * scan's block sums live in a fixed 64 KiB array in the library's device memory (one per
 * GPU, held until the process exits), so n is limited to
 * sph_exclusive_scan_i32_static_max_items() = 33,550,336; larger n is rejected with
 * SPH_ERR_INVALID_ARGUMENT.  Nothing in the array needs to start at zero.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) and should come
 * before any stream capture.  All calls share the one array: calls whose work overlaps on
 * the GPU (different streams, or different host threads) race and corrupt each other. */
int64_t sph_exclusive_scan_i32_static_max_items(void);
sph_status_t sph_exclusive_scan_i32_static(const int32_t* in, int32_t* out, int64_t n, void* stream);

/* Scratch bytes sph_radix_sort_pairs needs. */
size_t sph_radix_sort_scratch_bytes(int64_t n, int32_t digit_bits);
/* Stable LSD radix sort of (keys, vals) by the low key_bits bits of keys, digit_bits
 * (1..8) per pass, in place (the scratch holds the ping-pong copies).
 * Replaces torch.argsort of src/modules/neighborSearch.py:49 and :74. */
sph_status_t sph_radix_sort_pairs(uint32_t* keys, uint32_t* vals, int64_t n, int32_t key_bits,
                                  int32_t digit_bits, void* scratch, size_t scratch_bytes, void* stream);

/* ---------------------------------------------------------------- grid + sort (a1, a2) */

/* Scratch bytes sph_grid_build needs. */
size_t sph_grid_scratch_bytes(int64_t n);
/* Grid of sortPositions (src/modules/neighborSearch.py:34-46): hmax = max(support),
 * qmin = (min_coord or min(pos)) - hmax, qmax = (max_coord or max(pos)) + 2 hmax,
 * cells = ceil((qmax - qmin) / hmax).  min_coord / max_coord are host float[2] or NULL.
 * Writes *grid (device).  Flags SPH_FLAG_CELL_CAPACITY when cells_x*cells_y > cell_capacity. */
sph_status_t sph_grid_build(const float* pos, const float* support, int64_t n, const float* min_coord,
                            const float* max_coord, int32_t cell_capacity, sph_grid* grid,
                            int32_t* status, void* scratch, size_t scratch_bytes, void* stream);
/* keys[i] = linear cell id of pos[i] (the linearIndices of neighborSearch.py:46-47);
 * vals[i] = i when vals != NULL; cell_count[key] += 1 when cell_count != NULL (a zeroed
 * int32 [cell_capacity+1] histogram for sph_counting_sort).
 * A particle outside the grid (or any particle when the grid does not fit cell_capacity)
 * gets the sentinel key cell_capacity, is never searched, and flags SPH_FLAG_OUT_OF_GRID. */
sph_status_t sph_cell_keys(const float* pos, int64_t n, const sph_grid* grid, int32_t cell_capacity,
                           uint32_t* keys, uint32_t* vals, int32_t* cell_count, int32_t* status, void* stream);
/* Number of key bits the radix sort needs for keys 0..cell_capacity (the sentinel included). */
int32_t sph_key_bits(int32_t cell_capacity);
/* Counting sort of particles by cell key (a one-pass radix sort whose digit is the whole
 * key; replaces the argsort of neighborSearch.py:49): cell_start [cell_capacity+2] =
 * exclusive scan of cell_count, which is the cell begin table (cell c holds
 * [cell_start[c], cell_start[c+1])); order[s] = original index of sorted particle s,
 * ordered by (key, index) exactly as a stable sort; sorted_keys[s] = its key.  Leaves
 * cell_count zeroed.  Cells of more than 2048 particles keep an unreproducible inner
 * order and flag SPH_FLAG_CELL_ORDER. */
size_t sph_counting_sort_scratch_bytes(int64_t n, int32_t cell_capacity);
sph_status_t sph_counting_sort(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                               int32_t* cell_start, uint32_t* order, uint32_t* sorted_keys, int32_t* status,
                               void* scratch, size_t scratch_bytes, void* stream);
/* cell_start[c] = first sorted index whose key >= c, for c = 0..cell_capacity+1 (the cell
 * begin table after sph_radix_sort_pairs). */
sph_status_t sph_cell_starts(const uint32_t* sorted_keys, int64_t n, int32_t cell_capacity,
                             int32_t* cell_start, void* stream);
/* Reorder into sorted SoA (the gathers of neighborSearch.py:51-53): xy[s] = pos[order[s]]
 * (float2), sorted_support[s] = support[order[s]], sorted_area[s] = area[order[s]]; the
 * last two may be NULL. */
sph_status_t sph_gather_sorted(const uint32_t* order, int64_t n, const float* pos, const float* support,
                               const float* area, float* xy, float* sorted_support, float* sorted_area,
                               void* stream);

/* constructHashMap (src/modules/neighborSearch.py:58-88) on the GPU from the sorted keys:
 * writes cell_indices/cum_cell(counts)/cell_span(begins) [C] in hash order and
 * hash_table [hash_len, 2]; *num_cells_out (host) receives C.  Synchronises once
 * (to learn C, like the reference's host-side shapes). */
size_t sph_hash_map_scratch_bytes(int64_t n, int32_t hash_len);
sph_status_t sph_hash_map_build(const uint32_t* sorted_keys, int64_t n, int32_t cells_x, int32_t hash_len,
                                int32_t* hash_table, int32_t* cell_indices, int32_t* cum_cell,
                                int32_t* cell_span, int64_t* num_cells_out, void* scratch,
                                size_t scratch_bytes, void* stream);

/* ---------------------------------------------------------------- native CSR search (a4, a5, a9) */

/* Pass 1 of the two-pass CSR build over particles already in sorted order:
 * counts[s] = #{ j : |x_s - x_j| < support_s } over the (2r+1)^2 cells around s, with
 * the reference's predicate sqrtf(fmaf(dx,dx,dy*dy)) < h_s, dx = x_s - x_j.
 * If rho != NULL also rho[s] = sum_j W(|x_s-x_j| / kernel_support) * area_j (Wendland C2,
 * src/modules/density.py:26-30) — the fused search + density. */
sph_status_t sph_nl_count(const float* xy, const float* sorted_support, const float* sorted_area, int64_t n,
                          const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                          int32_t cell_capacity, int32_t search_radius, float kernel_support,
                          int32_t* counts, float* rho, void* stream);
/* Pass 2: cols[offsets[s] + k] = sorted index of the k-th neighbor of s (cell order).
 * offsets = exclusive scan of counts (n+1 entries).  A row that would end beyond
 * pair_capacity is not written and flags SPH_FLAG_PAIR_CAPACITY. */
sph_status_t sph_nl_fill(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                         const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity,
                         int32_t search_radius, const int32_t* offsets, int64_t pair_capacity,
                         int32_t* cols, int32_t* status, void* stream);
/* out[order[s]] = in[s]: a sorted-order field back to original particle order. */
sph_status_t sph_scatter_f32(const uint32_t* order, const float* in, int64_t n, float* out, void* stream);
/* Materialise the reference's fluidNeighbors / fluidDistances / fluidRadialDistances
 * (src/modules/neighborSearch.py:216-227) in original particle order, pairs ordered by
 * (i, j) like the CUDA finalize (:153-157).  order[s] = original index of sorted s,
 * rank[i] = sorted index of original i, orig_offsets = exclusive scan of counts by
 * original index.  dist/radial may be NULL. */
sph_status_t sph_nl_to_coo(const float* xy, int64_t n, const uint32_t* order, const uint32_t* rank,
                           const int32_t* offsets, const int32_t* cols, const int64_t* orig_offsets,
                           float grad_threshold, float kernel_support, int64_t* pairs /* [2, P] */,
                           int64_t num_pairs, float* dist /* [P,2] */, float* radial /* [P] */,
                           void* stream);
/* Original-order counts for sph_nl_to_coo: out[order[s]] = counts[s]. */
sph_status_t sph_scatter_counts(const uint32_t* order, const int32_t* counts, int64_t n, int32_t* out,
                                void* stream);
/* rank[order[s]] = s */
sph_status_t sph_invert_permutation(const uint32_t* order, int64_t n, uint32_t* rank, void* stream);

/* Query points (any order: wall or ghost particles) against the sorted grid:
 * pairs (query b, particle j) with sqrtf(fmaf(dx,dx,dy*dy)) < support_b, dx = x_b - x_j —
 * the pair set of searchExisting / buildNeighborListUnsortedPerParticle
 * (src/modules/neighborSearch.py:231-252, cppSrc/neighSearch.cpp:261-331).
 * Two passes like sph_nl_count/sph_nl_fill; offsets are int64 [m+1]; cols are original
 * particle indices when order != NULL, sorted indices otherwise. */
sph_status_t sph_nl_query_count(const float* query_pos, const float* query_support, int64_t m,
                                const float* xy, const int32_t* cell_start, const sph_grid* grid,
                                int32_t cell_capacity, int32_t search_radius, int32_t* counts, void* stream);
sph_status_t sph_nl_query_fill(const float* query_pos, const float* query_support, int64_t m,
                               const float* xy, const int32_t* cell_start, const sph_grid* grid,
                               int32_t cell_capacity, int32_t search_radius, const uint32_t* order,
                               const int64_t* offsets, int32_t* rows, int32_t* cols, void* stream);

/* ---------------------------------------------------------------- drop-in hashed-table search */

/* buildNeighborListCUDA (cppSrc/neighSearch.cpp:143-170, kernels cppSrc/neighSearch_cuda.cu:101-209)
 * and buildNeighborListUnsortedPerParticle (cppSrc/neighSearch.cpp:261-331): query points
 * (any order) against the reference-format hash table.  rows = query index, cols = sort[j].
 * Two passes: _count writes counts[m]; the caller scans them to offsets (int64 [m+1]);
 * _fill writes the pairs.  qmin is a device float[2]. */
sph_status_t sph_nl_hashed_query_count(const float* query_pos, const float* query_support, int64_t m,
                                       const float* sorted_pos, const int32_t* hash_table,
                                       const int32_t* cell_indices, const int32_t* cum_cell,
                                       const int32_t* cell_span, const float* qmin, float hmax,
                                       int32_t cells_x, int32_t hash_len, int32_t search_radius,
                                       int32_t* counts, void* stream);
sph_status_t sph_nl_hashed_query_fill(const float* query_pos, const float* query_support, int64_t m,
                                      const float* sorted_pos, const int32_t* hash_table,
                                      const int32_t* cell_indices, const int32_t* cum_cell,
                                      const int32_t* cell_span, const int32_t* sort, const float* qmin,
                                      float hmax, int32_t cells_x, int32_t hash_len, int32_t search_radius,
                                      const int64_t* offsets, int32_t* rows, int32_t* cols, void* stream);
/* buildNeighborList (cppSrc/neighSearch.cpp:172-259): every occupied cell of the table
 * against its (2r+1)^2 neighbor cells; rows = sort[i], cols = sort[j].  One count per
 * cell (counts[num_cells]). */
sph_status_t sph_nl_hashed_cells_count(const float* sorted_pos, const float* sorted_support,
                                       const int32_t* hash_table, const int32_t* cell_indices,
                                       const int32_t* cum_cell, const int32_t* cell_span, int64_t num_cells,
                                       int32_t cells_x, int32_t hash_len, int32_t search_radius,
                                       int32_t* counts, void* stream);
sph_status_t sph_nl_hashed_cells_fill(const float* sorted_pos, const float* sorted_support,
                                      const int32_t* hash_table, const int32_t* cell_indices,
                                      const int32_t* cum_cell, const int32_t* cell_span,
                                      const int32_t* sort, int64_t num_cells, int32_t cells_x,
                                      int32_t hash_len, int32_t search_radius, const int64_t* offsets,
                                      int32_t* rows, int32_t* cols, void* stream);
/* buildNeighborListAsymmetric (cppSrc/neighSearch.cpp:333-410): cells of table A against
 * table B (radius 1); rows = sortA[i], cols = sortB[j]. */
sph_status_t sph_nl_hashed_asym_count(const float* pos_a, const float* support_a, const int32_t* table_a,
                                      const int32_t* cell_indices_a, const int32_t* cum_cell_a,
                                      const int32_t* cell_span_a, int64_t num_cells_a, const float* pos_b,
                                      const int32_t* table_b, const int32_t* cell_indices_b,
                                      const int32_t* cum_cell_b, const int32_t* cell_span_b, int32_t cells_x,
                                      int32_t hash_len, int32_t* counts, void* stream);
sph_status_t sph_nl_hashed_asym_fill(const float* pos_a, const float* support_a, const int32_t* table_a,
                                     const int32_t* cell_indices_a, const int32_t* cum_cell_a,
                                     const int32_t* cell_span_a, const int32_t* sort_a, int64_t num_cells_a,
                                     const float* pos_b, const int32_t* table_b,
                                     const int32_t* cell_indices_b, const int32_t* cum_cell_b,
                                     const int32_t* cell_span_b, const int32_t* sort_b, int32_t cells_x,
                                     int32_t hash_len, const int64_t* offsets, int32_t* rows, int32_t* cols,
                                     void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
