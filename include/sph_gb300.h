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
 * cell (ix, iy) = ceil((x - qmin) / hmax), linear id ix + cells_x * iy.
 * sph_grid_build_ratio makes cells of max(support) / ratio: hmax is then the cell size and
 * threshold_support the largest support. */
typedef struct sph_grid {
  float qmin[2];
  float hmax;
  float hmax_threshold;  /* set by sph_grid_build: the pair test's square-root-free threshold
                            for support threshold_support (0 = not set) */
  int32_t cells_x;
  int32_t cells_y;
  int32_t num_cells;
  float threshold_support;  /* the support hmax_threshold belongs to (0: hmax) */
} sph_grid;

/* Physical and numerical parameters of the summations (one scene). */
typedef struct sph_params {
  float support;            /* kernel support h (config particle.support) */
  float rest_density;       /* rho0 (fluid.restDensity) */
  float c0;                 /* speed of sound (fluid.c0) */
  float gamma;              /* Tait exponent (pressure.gamma) */
  float alpha;              /* artificial viscosity (diffusion.alpha) */
  float delta;              /* density diffusion (diffusion.delta) */
  float kinematic;          /* laminar viscosity (diffusion.kinematic) */
  float gravity[2];         /* constant body force (gravity.magnitude * gravity.direction) */
  int32_t point_source;     /* 1: gravity = -g (x - c) (gravity.pointSource with potentialField) */
  float point_magnitude;
  float point_center[2];
  int32_t density_diffusion;   /* 0 none, 1 MOG, 2 deltaSPH (diffusion.densityScheme) */
  int32_t boundary_diffusion;  /* diffusion.boundaryDiffusion */
  int32_t search_radius;       /* cells searched around a particle (1) */
  int32_t cell_capacity;       /* size of the cell tables */
  /* DFSPH (dfsph.*) */
  int32_t min_density_iters, max_density_iters, min_divergence_iters, max_divergence_iters;
  float density_threshold, divergence_threshold;
  float omega_boundary;        /* wall relaxed-Jacobi weight (dfsph.relaxedJacobiOmega) */
  float omega_fluid;           /* fluid relaxed-Jacobi weight (0.3 in the reference, src/modules/dfsph.py:175) */
} sph_params;

/* Fluid particles in cell-sorted order (device arrays) and their CSR neighbor list. */
typedef struct sph_fluid_view {
  const float* x;           /* float2 [n] positions */
  const float* v;           /* float2 [n] velocities */
  const float* rho;         /* [n] relative density rho~ (absolute = rho~ * rest_density) */
  const float* area;        /* [n] particle area A */
  const uint32_t* keys;     /* [n] cell keys of the sorted particles */
  const int32_t* offsets;   /* [n+1] CSR row offsets */
  const int32_t* cols;      /* [P] CSR columns (sorted indices) */
  const int32_t* cell_start;/* [cells+2] fluid cell table */
  int64_t n;
  int64_t pair_capacity;    /* length of cols; a row ending past it was not filled (the fill
                               flagged SPH_FLAG_PAIR_CAPACITY) and reads as empty; 0 = cols
                               holds every row */
} sph_fluid_view;

/* Wall (ghost-particle boundary) particles sorted by their cell in the fluid grid. */
typedef struct sph_wall_view {
  const float* x;           /* float2 [nb] wall positions */
  const float* ghost;       /* float2 [nb] mirrored ghost positions */
  const float* area;        /* [nb] boundaryVolume = pi r^2 */
  const int32_t* cell_start;/* [cells+2] wall cell table in the fluid grid */
  int64_t n;
  float* rho;               /* [nb] wall relative density (written) */
  float* volume;            /* [nb] A_b / rho_b (written) */
  float* pressure;          /* [nb] wall pressure (written) */
} sph_wall_view;

int32_t sph_abi_version(void);
const char* sph_last_error(void);
const char* sph_status_string(sph_status_t status);

/* ---------------------------------------------------------------- primitives */

/* Scratch bytes sph_exclusive_scan_* needs for n items. */
size_t sph_scan_scratch_bytes(int64_t n);
/* out[k] = in[0] + ... + in[k-1] for k <= n (out has n+1 entries; out[n] = total).
 * Replaces torch::cumsum in cppSrc/neighSearch_cuda.cu:250 and the cumsums of
 * src/modules/neighborSearch.py:65,86.  Above 16,384 items: one zeroing of the scratch and
 * one single-pass launch (decoupled look-back); the scratch must not be shared by scans
 * that overlap on the GPU. */
sph_status_t sph_exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch,
                                    size_t scratch_bytes, void* stream);
sph_status_t sph_exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, void* scratch,
                                           size_t scratch_bytes, void* stream);
/* Look-back waits of the scans that gave up (each wait is bounded) since the library was
 * loaded on the current device: 0 unless a scan's output is wrong.  Synchronous. */
uint64_t sph_scan_timeouts(void);

/* Allocation-free variant of sph_exclusive_scan_i32.  It has no counterpart in the
 * reference.  It exists for callers that cannot allocate device memory: a host runtime
 * bound through this C ABI (a service written in another language) that only receives
 * device pointers from the owner of GPU memory and has no allocator of its own, or a
 * serving process whose whole device-memory budget is reserved up front in a pooled
 * arena, where a further allocation would break the budget.  The scan's tile words live
 * in a fixed 64 KiB array in the library's device memory (one per GPU, held until the
 * process exits), so n is limited to sph_exclusive_scan_i32_static_max_items() =
 * 33,550,336; larger n is rejected with SPH_ERR_INVALID_ARGUMENT and nothing runs.  The
 * call clears the tile words it uses before the scan (a memset, no allocation).  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress) and caches
 * it; that first call should come before any stream capture, and the cached address does
 * not survive cudaDeviceReset, so the entry point must not be used on a device after it
 * was reset in the same process.  All calls share the one array: calls whose work overlaps
 * on the GPU (different streams, or different host threads) race and corrupt each other. */
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

/* The grids of nseg particle sets in one launch: set s is particles [seg_offsets[s],
 * seg_offsets[s+1]) of pos / support; min_coords / max_coords are device float[2*nseg] (set
 * s's domain) or NULL; grids device sph_grid[nseg].  Same arithmetic as sph_grid_build.
 * An empty set flags SPH_FLAG_NONFINITE. */
sph_status_t sph_grid_build_segments(const float* pos, const float* support, const int64_t* seg_offsets,
                                     int32_t nseg, const float* min_coords, const float* max_coords,
                                     int32_t cell_capacity, sph_grid* grids, int32_t* status, void* stream);
/* Scratch bytes sph_grid_build needs. */
size_t sph_grid_scratch_bytes(int64_t n);
/* Grid of sortPositions (src/modules/neighborSearch.py:34-46): hmax = max(support),
 * qmin = (min_coord or min(pos)) - hmax, qmax = (max_coord or max(pos)) + 2 hmax,
 * cells = ceil((qmax - qmin) / hmax).  min_coord / max_coord are host float[2] or NULL.
 * Writes *grid (device).  Flags SPH_FLAG_CELL_CAPACITY when cells_x*cells_y > cell_capacity. */
sph_status_t sph_grid_build(const float* pos, const float* support, int64_t n, const float* min_coord,
                            const float* max_coord, int32_t cell_capacity, sph_grid* grid,
                            int32_t* status, void* scratch, size_t scratch_bytes, void* stream);
/* The grid of sph_grid_build (same qmin and the same padded extent) with cells of
 * hmax / cell_ratio, 1 <= cell_ratio <= 8: searched cell_ratio cells out, it gives the
 * same pair sets with fewer candidates per particle.  The pairs of a row come in the order
 * of the finer cells.  No counterpart in the reference (its grid is the ratio-1 one). */
sph_status_t sph_grid_build_ratio(const float* pos, const float* support, int64_t n, const float* min_coord,
                                  const float* max_coord, int32_t cell_ratio, int32_t cell_capacity,
                                  sph_grid* grid, int32_t* status, void* scratch, size_t scratch_bytes,
                                  void* stream);
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
 * order and flag SPH_FLAG_CELL_ORDER.  The sentinel cell (key cell_capacity) is not ordered:
 * its particles keep the scatter's order. */
size_t sph_counting_sort_scratch_bytes(int64_t n, int32_t cell_capacity);
sph_status_t sph_counting_sort(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                               int32_t* cell_start, uint32_t* order, uint32_t* sorted_keys, int32_t* status,
                               void* scratch, size_t scratch_bytes, void* stream);
/* As sph_counting_sort, ordering each cell by (tie[i], i) instead of i: with a particle id as
 * tie key the sorted order no longer depends on the order the particles arrived in. */
sph_status_t sph_counting_sort_tie(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                                   int32_t* cell_start, const uint32_t* tie, uint32_t* order, uint32_t* sorted_keys,
                                   int32_t* status, void* scratch, size_t scratch_bytes, void* stream);
/* sph_counting_sort_tie that also moves `count` (at most 8) per-particle arrays into the
 * sorted order, out[k][s] = in[k][order[s]], in the same launches: the in-cell fix writes
 * each particle's rows where it places the particle (replaces the separate
 * sph_permute_arrays pass; the gathers of src/modules/neighborSearch.py:51-53 applied to
 * the whole state).  elem_bytes, in and out are host arrays of `count` entries (4-, 8- or 16-byte
 * rows); in[k] and out[k] must not overlap. */
sph_status_t sph_counting_sort_permute(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                                       int32_t* cell_start, const uint32_t* tie, uint32_t* order,
                                       uint32_t* sorted_keys, int32_t count, const int32_t* elem_bytes,
                                       const void* const* in, void* const* out, int32_t* status, void* scratch,
                                       size_t scratch_bytes, void* stream);
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
 * writes cell_indices/cum_cell(counts)/cell_span(begins) [C] in hash order (cells of one
 * hash in increasing cell order, as a stable argsort of the hashes gives) and hash_table
 * [hash_len, 2] = (first slot, cells in the bucket), (-1, 0) for an empty bucket.  The
 * number of occupied cells C goes to *num_cells (device int32); the output arrays need room
 * for n entries (C <= n).  Asynchronous: nothing waits on the host. */
size_t sph_hash_map_scratch_bytes(int64_t n, int32_t hash_len);
sph_status_t sph_hash_map_build(const uint32_t* sorted_keys, int64_t n, int32_t cells_x, int32_t hash_len,
                                int32_t* hash_table, int32_t* cell_indices, int32_t* cum_cell,
                                int32_t* cell_span, int32_t* num_cells, void* scratch,
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
/* The same two passes with one candidate test per pair: sph_nl_count_segments tests the
 * cell rows once, in segments of 32 candidates, and keeps each particle's accepted-candidate
 * bit masks (at most 24 segments; more: its rows are scanned again by the fill) in
 * seg_scratch (sph_nl_segments_scratch_bytes(n) bytes) besides counts and rho;
 * sph_nl_fill_segments expands them into the CSR columns.  Same counts, rho, columns and
 * order as sph_nl_count / sph_nl_fill. */
size_t sph_nl_segments_scratch_bytes(int64_t n);
sph_status_t sph_nl_count_segments(const float* xy, const float* sorted_support, const float* sorted_area, int64_t n,
                                   const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                                   int32_t cell_capacity, int32_t search_radius, float kernel_support,
                                   int32_t* counts, float* rho, void* seg_scratch, size_t seg_bytes, void* stream);
sph_status_t sph_nl_fill_segments(const float* xy, const float* sorted_support, int64_t n,
                                  const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                                  int32_t cell_capacity, int32_t search_radius, const int32_t* offsets,
                                  int64_t pair_capacity, int32_t* cols, int32_t* status, const void* seg_scratch,
                                  size_t seg_bytes, void* stream);
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

/* ---------------------------------------------------------------- deltaSPH summations (a8-a19) */

/* mDBC wall density (computeBoundaryDensitymDBC, src/modules/solidBoundary.py:561-617):
 * per wall particle, Shepard and first-order MLS sums over the fluid within h of its ghost,
 * a 3x3 pseudo-inverse solve, rho_b = max(result, 1); writes walls->rho, ->volume
 * (A_b / rho_b) and ->pressure (Tait, solidBoundary.py:802-804). */
sph_status_t sph_mdbc_wall_density(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                   const sph_params* params, void* stream);
/* The deltaSPH right-hand side (deltaSPHSimulation.timestep steps 6-12, src/deltaSPH.py:146-200):
 * dpdt [n] = continuity (src/modules/momentum.py:13-19) + density diffusion (MOG
 * densityDiffusion.py:56-63, or the renormalized deltaSPH scheme :12-52 when
 * density_diffusion = 2, which needs grad_rho float2 [n]; L float4 [n], optional, receives
 * the renormalization matrix); acc float2 [n] = gravity + pressure (pressure.py:13-19) +
 * artificial viscosity (diffusion.py:12-25) + laminar viscosity (laminar.py:12-27), each
 * with its wall part (solidBoundary.py:746-890).  Wall quantities must come from
 * sph_mdbc_wall_density.  scratch: sph_deltasph_scratch_bytes(n) bytes of device memory
 * (per-particle neighbor records, and the segment lists of sph_batch_deltasph_step). */
size_t sph_deltasph_scratch_bytes(int64_t n);
/* Where sph_batch_deltasph_step keeps its segment lists in a scratch of n particles (byte
 * offsets from the scratch's first 32-byte boundary): the uint32 accepted-candidate masks
 * and the int32 segment starts (segment k of particle i at index k * n + i, k <
 * max_segments) and the int32 segment counts (-1: the particle's segments did not fit).
 * For callers that count the bytes a step moves without a host copy of the search. */
sph_status_t sph_deltasph_segment_lists(int64_t n, size_t* masks_offset, size_t* starts_offset,
                                        size_t* counts_offset, int32_t* max_segments);
sph_status_t sph_deltasph_forces(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, float* dpdt, float* acc, float* L, float* grad_rho,
                                 void* scratch, size_t scratch_bytes, void* stream);
/* semiImplicitEuler (src/simulationBase.py:647-652): v' = v + dt a, x' = x + dt (v + dt a),
 * rho' = rho + dt dpdt / rest_density when continuum_density.  dt is a device float. */
sph_status_t sph_integrate_semi_implicit_euler(int64_t n, const float* x, const float* v, const float* rho,
                                               const float* acc, const float* dpdt, const float* dt,
                                               float rest_density, int32_t continuum_density, float* x_out,
                                               float* v_out, float* rho_out, int32_t* status, void* stream);
/* RK4 stage / combination (src/simulationBase.py:679-705): out = base + c*dt*(ku, ka, kd/rest_density). */
sph_status_t sph_rk_axpy(int64_t n, const float* x0, const float* v0, const float* rho0_field, const float* ku,
                         const float* ka, const float* kd, const float* dt, float c, float rest_density, float* x_out,
                         float* v_out, float* rho_out, int32_t* status, void* stream);
/* s = w*k (init) or s += w*k for the RK4 sums of (velocity, acceleration, dpdt). */
sph_status_t sph_rk_accumulate(int64_t n, const float* ku, const float* ka, const float* kd, float w, int32_t init,
                               float* su, float* sa, float* sd, void* stream);
/* out[s] = in[order[s]] for 4-, 8- or 16-byte elements (re-sorting per-particle state). */
sph_status_t sph_permute(const uint32_t* order, int64_t n, int32_t elem_bytes, const void* in, void* out, void* stream);
/* The same for `count` (at most 8) arrays in one pass: out[k][s] = in[k][order[s]], or a
 * plain copy when order is NULL.  elem_bytes, in and out are host arrays of `count` entries;
 * in[k] and out[k] must not overlap. */
sph_status_t sph_permute_arrays(const uint32_t* order, int64_t n, int32_t count, const int32_t* elem_bytes,
                                const void* const* in, void* const* out, void* stream);

/* ---------------------------------------------------------------- batch of independent scenes */
/* Many scenes stepped together: their particles are concatenated in one array with a
 * per-particle scene index `sid`; scene s owns the slots [cell_offset_s, cell_offset_s +
 * num_cells_s] of the shared cell tables (its cells, then one outside slot for particles
 * that left its grid or became non-finite: no neighbors, body forces only), so (scene,
 * cell) keys sort every scene into its own contiguous range and scenes never interact.  The scene table is an array of opaque
 * records of sph_scene_bytes() bytes each, filled with sph_scene_encode and copied to the
 * device. */
size_t sph_scene_bytes(void);
/* Encode one scene record on the host: parameters, its grid (host copy of the sph_grid
 * from sph_grid_build), its cell-table offset and its time step. */
sph_status_t sph_scene_encode(const sph_params* params, const sph_grid* grid_host, int32_t cell_offset, float dt,
                              void* out_host);
/* (scene, cell) keys + per-cell histogram for sph_counting_sort; cell_capacity = the total
 * slot count, sum over scenes of num_cells_s + 1.  Sets SPH_FLAG_OUT_OF_GRID /
 * SPH_FLAG_NONFINITE for particles put in their scene's outside slot.  A particle with a
 * negative scene index (a free slot of a pooled batch) gets the sentinel key cell_capacity,
 * without a flag, and the batch kernels skip it. */
sph_status_t sph_batch_cell_keys(const float* pos, int64_t n, const int32_t* sid, const void* scenes,
                                 int32_t cell_capacity, uint32_t* keys, int32_t* cell_count, int32_t* status,
                                 void* stream);
/* Two-pass CSR over a sorted batch (each particle searches its own scene's cells). */
sph_status_t sph_batch_nl_count(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                                const int32_t* cell_start, const void* scenes, const int32_t* sid, int32_t* counts,
                                void* stream);
sph_status_t sph_batch_nl_fill(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                               const int32_t* cell_start, const void* scenes, const int32_t* sid, const int32_t* offsets,
                               int64_t pair_capacity, int32_t* cols, int32_t* status, void* stream);
/* One semi-implicit-Euler deltaSPH step of every scene of the batch: mDBC wall densities,
 * the right-hand side (as sph_deltasph_forces, each particle with its scene's parameters)
 * and the update with each scene's own dt, written to x_out / v_out / rho_out.  If
 * SPH_FLAG_PAIR_CAPACITY is set in *status when the update runs (the fill overflowed),
 * the step is not applied: the outputs are the sorted inputs unchanged.  dpdt [n], acc
 * float2 [n] and grad_rho float2 [n] carry the renormalized scenes' first pass to their
 * diffusion pass (needed when any_renormalized; grad_rho then holds <grad rho> V, the part
 * of the deltaSPH diffusion that needs the neighbors); scratch as for sph_deltasph_forces.
 * With fluid->offsets and fluid->cols both NULL no neighbor list is needed: the records
 * launch also tests each particle's cell rows in segments of 32 candidates and stores its
 * non-empty segments (start, 32-bit accepted-candidate mask; at most 8, else the force
 * passes test its rows themselves; sph_deltasph_segment_lists), and both force passes visit
 * those pairs in the CSR fill's order (same sums).  Each scene's pair test then uses its own support (sph_params.support),
 * which must be every particle's support.
 * The force passes (pass1, diffusion) run over `groups` (a host array of ngroups entries
 * that tile [0, n) in order; a group holds whole scenes when its bounds are scene bounds):
 * `tpp` lanes per particle (each lane takes every 2nd or 4th segment; the lanes' sums are
 * added by warp shuffles, so the summation order, not the pair set, depends on it) and,
 * when all its scenes share one, the diffusion `scheme`, which selects a kernel compiled for
 * it.  ngroups = 0: one group, one lane, any schemes.
 * `phases` selects the launches (SPH_PHASE_ALL for a step; single phases, in order, let a
 * caller time each kernel): walls = mDBC wall densities, records = per-particle neighbor
 * records, pass1 = first pair pass (+ update of scenes without deltaSPH diffusion),
 * diffusion = deltaSPH diffusion pass (+ update of the other scenes). */
#define SPH_PHASE_WALLS 1
#define SPH_PHASE_RECORDS 2
#define SPH_PHASE_PASS1 4
#define SPH_PHASE_DIFFUSION 8
#define SPH_PHASE_ALL 15
/* A range of sorted particles that the force passes run over with one kernel variant. */
typedef struct sph_force_group {
  int64_t begin, end;  /* sorted particles [begin, end) */
  int32_t tpp;         /* lanes per particle: 1, or 2 or 4 with pairs from the cell rows */
  int32_t scheme;      /* the density diffusion of every scene in the range (0 none, 1 MOG,
                          2 deltaSPH), or -1 when they differ */
} sph_force_group;
sph_status_t sph_batch_deltasph_step(const sph_fluid_view* fluid, const sph_wall_view* walls, const void* scenes,
                                     const int32_t* sid, const int32_t* wall_sid, float* dpdt, float* acc,
                                     float* grad_rho, int32_t any_renormalized, float* x_out, float* v_out,
                                     float* rho_out, int32_t* status, int32_t phases, int32_t ngroups,
                                     const sph_force_group* groups, void* scratch, size_t scratch_bytes,
                                     void* stream);

/* ---------------------------------------------------------------- Module terms (a9-a17) */

/* One summation term over the reference's own pair list, for callers that drive the
 * reference's Module interface (densityModule.evaluate, momentumModule.computeDpDt,
 * densityDiffusionModule.*, pressureModule.computePressureAcceleration,
 * diffusionModule.evaluate, laminarViscosityModule.computeLaminarViscosity).  Arrays are
 * in original particle order: the simulationState fields.  Pairs are fluidNeighbors
 * ordered by row i (offsets from sph_row_offsets), fluidDistances e_ij and
 * fluidRadialDistances q_ij as neighborSearchModule.search writes them
 * (src/modules/neighborSearch.py:216-227). */
typedef struct sph_pair_terms_in {
  const int32_t* offsets;   /* [n+1] first pair of each row */
  const int64_t* cols;      /* [P] j = fluidNeighbors[1] */
  const float* dist;        /* float2 [P] fluidDistances */
  const float* radial;      /* [P] fluidRadialDistances */
  const float* pos;         /* float2 [n] fluidPosition */
  const float* vel;         /* float2 [n] fluidVelocity */
  const float* rho;         /* [n] fluidDensity (relative) */
  const float* volume;      /* [n] fluidVolume */
  const float* area;        /* [n] fluidArea */
  const float* pressure;    /* [n] fluidPressure */
  const float* L;           /* float4 [n] pseudo-inverted normalization matrix (fluidL) */
  const float* grad_rho;    /* float2 [n] renormalized density gradient */
  const float* actual_area; /* [n] fluidActualArea (DFSPH) */
  const float* pred_accel;  /* float2 [n] fluidPredAccel (DFSPH) */
  const float* pred_vel;    /* float2 [n] fluidPredictedVelocity (DFSPH) */
  double dt;                /* time step (DFSPH terms) */
  int64_t n;
} sph_pair_terms_in;

#define SPH_TERM_DENSITY 0                 /* [n]   density.py:26-30 */
#define SPH_TERM_DIVERGENCE 1              /* [n]   momentum.py:31-38 */
#define SPH_TERM_MOG_DIFFUSION 2           /* [n]   densityDiffusion.py:74-82 */
#define SPH_TERM_NORMALIZATION 3           /* [n,4] densityDiffusion.py:30-44 */
#define SPH_TERM_RENORMALIZED_GRADIENT 4   /* [n,2] densityDiffusion.py:45-61 */
#define SPH_TERM_DELTA_DIFFUSION 5         /* [n]   densityDiffusion.py:63-71 */
#define SPH_TERM_PRESSURE_ACCEL 6          /* [n,2] pressure.py:31-38 */
#define SPH_TERM_VELOCITY_DIFFUSION 7      /* [n,2] diffusion.py:30-44 */
#define SPH_TERM_LAMINAR 8                 /* [n,2] laminar.py:30-46 */
/* DFSPH (src/modules/dfsph.py), spiky gradient S_ij = e_ij kGS(q_ij), rho = fluidDensity: */
#define SPH_TERM_DFSPH_ALPHA 9             /* [n,4] (kSum1 x, y, kSum2, 0), dfsph.py:58-72 */
#define SPH_TERM_DFSPH_SOURCE 10           /* [n]   -dt sum A^act_j (v*_i - v*_j) . S_ij, dfsph.py:85-100 */
#define SPH_TERM_DFSPH_PRESSURE_SUM 11     /* [n]   dt^2 sum A^act_j (a_i - a_j) . S_ij, dfsph.py:43-57 */
#define SPH_TERM_DFSPH_ACCEL 12            /* [n,2] -sum A_j rho0 (p_i/(rho_i rho0)^2 + p_j/(rho_j rho0)^2) S_ij, dfsph.py:25-42 */
/* out (=, or += when accumulate) one term per particle; params gives h, rest_density, c0,
 * alpha, delta, kinematic. */
sph_status_t sph_pair_term(int32_t term, const sph_pair_terms_in* in, const sph_params* params, float* out,
                           int32_t accumulate, void* stream);

#define SPH_OP_TAIT 0       /* out = rho0 c0^2/gamma (a^gamma - 1), a = fluidDensity (pressure.py:103) */
#define SPH_OP_VOLUME 1     /* out = a / b: fluidArea / fluidDensity (density.py:54) */
#define SPH_OP_PINV2X2 2    /* out float4 = pinv2x2(a float4) (util.py:386-433) */
#define SPH_OP_GRAVITY 3    /* out float2 += gravity at positions a (gravity.py:46-57) */
/* Per-particle operations of the same modules over n particles. */
sph_status_t sph_particle_op(int32_t op, int64_t n, const float* a, const float* b, const sph_params* params,
                             float* out, int32_t accumulate, void* stream);
/* offsets[i] = first index of row i in rows (int64, ascending), offsets[n] = num_pairs. */
sph_status_t sph_row_offsets(const int64_t* rows, int64_t num_pairs, int64_t n, int32_t* offsets, void* stream);
/* Distances of query pairs (searchExisting, src/modules/neighborSearch.py:244-251):
 * d = query_pos[row] - pos[col], r = |d|; dist float2 = d / r (0 when r < threshold),
 * radial = r / query_support[row]. */
sph_status_t sph_pair_geometry(const int32_t* rows, const int32_t* cols, int64_t num_pairs, const float* query_pos,
                               const float* pos, const float* query_support, float threshold, float* dist,
                               float* radial, void* stream);

/* ---------------------------------------------------------------- Boundary-module wall terms (a18) */

/* The solid-wall terms of src/modules/solidBoundary.py for callers of its BoundaryModule
 * interface, over the reference's own wall pair lists: pairs (b, f) of wall (or ghost) b
 * and fluid particle f in wall order (boundaryToFluidNeighbors / ghostToFluidNeighbors of
 * searchExisting) with e = (x_b - x_f) / r and q = r / h, and the same pairs grouped by
 * fluid particle (sph_transpose_pairs).  Fluid arrays in original order. */
typedef struct sph_wall_terms_in {
  const int32_t* wall_offsets;   /* [nb+1] first pair of each wall (sph_row_offsets of rows) */
  const int64_t* rows;           /* [P] wall of each pair */
  const int64_t* cols;           /* [P] fluid particle of each pair */
  const float* dist;             /* float2 [P] e = (x_b - x_f) / r */
  const float* radial;           /* [P] q = r / h */
  const int32_t* fluid_offsets;  /* [n+1] first grouped pair of each fluid particle */
  const int32_t* fluid_pairs;    /* [P] pair indices grouped by fluid particle, ascending */
  const float* pos;              /* float2 [n] fluid positions */
  const float* vel;              /* float2 [n] */
  const float* rho;              /* [n] fluidDensity (relative) */
  const float* area;             /* [n] fluidArea */
  const float* volume;           /* [n] fluidVolume */
  const float* pressure;         /* [n] fluidPressure (deltaSPH) / fluidPressure2 (DFSPH) */
  const float* L;                /* float4 [n] pseudo-inverted fluid normalization matrix */
  const float* actual_area;      /* [n] fluidActualArea */
  const float* pred_accel;       /* float2 [n] fluidPredAccel */
  const float* pred_vel;         /* float2 [n] fluidPredictedVelocity */
  const float* wall_pos;         /* float2 [nb] boundaryPositions */
  const float* wall_ghost;       /* float2 [nb] boundaryGhostPositions */
  const float* wall_area;        /* [nb] boundaryVolume (the wall particle's area) */
  const float* wall_rho;         /* [nb] boundaryDensity (relative) */
  const float* wall_volume;      /* [nb] boundaryVolume / boundaryDensity */
  const float* wall_pressure;    /* [nb] boundaryPressure */
  const float* wall_actual_area; /* [nb] boundaryActualArea */
  const float* wall_term;        /* [nb] static wall-wall density term */
  double dt;
  int64_t n, nb;
} sph_wall_terms_in;

/* fluid-side sums, out per fluid particle (=, or += when accumulate) */
#define SPH_WALL_DENSITY 0                 /* [n]   sum W A_b (:522-549) */
#define SPH_WALL_DPDT 1                    /* [n]   continuity wall part (:746-770) */
#define SPH_WALL_NORMALIZATION 2           /* [n,4] L wall part (:676-694) */
#define SPH_WALL_RENORMALIZED_GRADIENT 3   /* [n,2] <grad rho> wall part (:695-717) */
#define SPH_WALL_PRESSURE_ACCEL 4          /* [n,2] (:846-896) */
#define SPH_WALL_VELOCITY_DIFFUSION 5      /* [n,2] (:820-844) */
#define SPH_WALL_DFSPH_ALPHA 6             /* [n,4] (kSum1 x, y, kSum2, 0) PBSPH (:443-479) */
#define SPH_WALL_DFSPH_SOURCE 7            /* [n]   (:481-520) */
#define SPH_WALL_DFSPH_PRESSURE_SUM 8      /* [n]   (:405-441) */
#define SPH_WALL_DFSPH_ACCEL 9             /* [n,2] PBSPH (:310-403) */
/* wall-side sums, out per wall (=) */
#define SPH_BWALL_DENSITY 20               /* [nb]  min(term + sum W A_f, 1) (:522-549) */
#define SPH_BWALL_MDBC 21                  /* [nb]  mDBC density from ghost pairs (:561-617) */
#define SPH_BWALL_DFSPH_ALPHA 22           /* [nb]  boundaryAlpha (:443-479) */
#define SPH_BWALL_DFSPH_SOURCE 23          /* [nb]  boundarySource, density solve (:481-520) */
#define SPH_BWALL_DFSPH_PRESSURE_SUM 24    /* [nb]  boundary kernel sum (:405-441) */
/* wall pressures of the MLS schemes (solidBoundary.py:772-808) over the ghost pair list
 * (ghostToFluidNeighbors; for deltaMLS / MLSPressure queried from the wall positions,
 * :639-640), fluid pressure in `pressure`: */
#define SPH_BWALL_GHOST_MLS_PRESSURE 25    /* [nb]  ghostMLS: precomputeMLS at the ghost (src/util.py:332-384),
                                              p_b = sum_j (pinv(M_b) e1 . b_j) W_j V_j p_j, b_j = (1, x_j - x_g),
                                              M_b = sum_j 2 b_j b_j^T V_j W_j, V_j = A_j / (rho~_j rho0) */
#define SPH_BWALL_DELTA_MLS_PRESSURE 26    /* [nb]  deltaMLS: the same at the wall position */
#define SPH_BWALL_MLS_PRESSURE 27          /* [nb]  MLSPressure: prepareMLSBoundaries + evalMLSBoundaries
                                              (src/util.py:283-330) with V_j = volume, clamped at 0 */
sph_status_t sph_wall_term(int32_t term, const sph_wall_terms_in* in, const sph_params* params, float* out,
                           int32_t accumulate, void* stream);
/* Pairs grouped by column (fluid particle): col_offsets [n+1], pairs [num_pairs] = pair
 * indices, ascending inside each column. */
size_t sph_transpose_pairs_scratch_bytes(int64_t n);
sph_status_t sph_transpose_pairs(const int64_t* cols, int64_t num_pairs, int64_t n, int32_t* col_offsets,
                                 int32_t* pairs, void* scratch, size_t scratch_bytes, void* stream);

/* Pooled serving arena (continuous batching without rebuilding the batch): fixed-capacity
 * particle arrays whose free slots carry scene index -1.  No reference counterpart: the
 * reference steps one scene at a time. */
/* sid[begin + k] = scene, uid[begin + k] = k for k < count (a newly admitted scene). */
sph_status_t sph_arena_set_ids(int32_t* sid, int32_t* uid, int64_t begin, int64_t count, int32_t scene,
                               void* stream);
/* Scene `scene`'s x (float2), v (float2), rho in its own particle order: out[uid[i]] = in[i] for
 * every i < n with sid[i] == scene. */
sph_status_t sph_arena_extract(const float* x, const float* v, const float* rho, const int32_t* sid,
                               const int32_t* uid, int64_t n, int32_t scene, float* x_out, float* v_out,
                               float* rho_out, void* stream);
/* sid[i] = -1 for every i < n with sid[i] == scene (its particles leave the batch at the next sort). */
sph_status_t sph_arena_retire(int32_t* sid, int64_t n, int32_t scene, void* stream);
/* Several scenes of a pooled batch in one pass over its n slots: for every slot table entry s
 * (0 <= s < nslots) with row0[s] >= 0, the particles of scene s go to the output rows
 * row0[s] + particle id (ids >= rows[s] are skipped), and with `retire` their slots are
 * freed (scene index -1).  x_out, v_out, rho_out all NULL: retire only (x, v, rho, uid may
 * then be NULL).  row0 [nslots] int64 and rows [nslots] int32 are device arrays. */
sph_status_t sph_arena_extract_many(const float* x, const float* v, const float* rho, int32_t* sid,
                                    const int32_t* uid, int64_t n, const int64_t* row0, const int32_t* rows,
                                    int32_t nslots, float* x_out, float* v_out, float* rho_out, int32_t retire,
                                    void* stream);

/* ---------------------------------------------------------------- delta+ surface detection and shifting (f3) */

/* The surface detection and particle shifting of src/modules/deltaPlus.py
 * (deltaPlusModule.detectSurface :242-245 = computeNormalizationmatrix :116-130,
 * computeFluidNormal :132-163, detectFluidSurface :165-205; shift :247-251 =
 * computeShiftAmount :81-115, adjustShiftingAmount :207-240) over the reference's own pair
 * lists.  Fluid arrays in original order; pairs as the Module interface holds them:
 *   fluid pairs fluidNeighbors (i, j), i-ordered, e_ij = (x_i - x_j) / r, q = r / h;
 *   wall pairs boundaryToFluidNeighbors (b, f), b-ordered, e = (x_b - x_f) / r, and the same
 *   pairs grouped by fluid particle (sph_transpose_pairs);
 *   wall-wall pairs boundaryToBoundaryNeighbors (b, c), b-ordered, with the reference's
 *   boundaryToBoundaryNeighborDistances e = (x_c - x_b) / r (the opposite sign of
 *   fluidDistances, solidBoundary.py:180-191, 624-634). */
typedef struct sph_surface_in {
  const int32_t* offsets;            /* [n+1] fluid pair rows */
  const int64_t* cols;               /* [P] j */
  const float* dist;                 /* float2 [P] e_ij */
  const float* radial;               /* [P] q_ij */
  const int32_t* wall_offsets;       /* [nb+1] wall pair rows */
  const int64_t* wall_rows;          /* [Pb] b */
  const int64_t* wall_cols;          /* [Pb] f */
  const float* wall_dist;            /* float2 [Pb] (x_b - x_f) / r */
  const float* wall_radial;          /* [Pb] */
  const int32_t* fluid_wall_offsets; /* [n+1] wall pairs grouped by fluid particle */
  const int32_t* fluid_wall_pairs;   /* [Pb] pair indices, ascending per fluid particle */
  const int32_t* ww_offsets;         /* [nb+1] wall-wall pair rows */
  const int64_t* ww_cols;            /* [Pw] c */
  const float* ww_dist;              /* float2 [Pw] (x_c - x_b) / r */
  const float* ww_radial;            /* [Pw] */
  const float* pos;                  /* float2 [n] fluidPosition */
  const float* vel;                  /* float2 [n] fluidVelocity */
  const float* rho;                  /* [n] fluidDensity (relative) */
  const float* area;                 /* [n] fluidArea */
  const float* volume;               /* [n] fluidVolume */
  const float* matrix;               /* float4 [count] a 2x2 matrix per row (SPH_SURF_PINV_EIG) */
  const float* L;                    /* float4 [n] fluidL (pseudo-inverted normalization matrix) */
  const float* lambda;               /* [n] fluidLambda */
  const float* normal;               /* float2 [n] fluidNormal */
  const float* mask;                 /* [n] angle mask (SPH_SURF_CLASSIFY) / fluidSurfaceMask (adjust) */
  const float* shift;                /* float2 [n] shiftAmount (SPH_SURF_SHIFT_ADJUST) */
  const float* wall_pos;             /* float2 [nb] boundaryPositions */
  const float* wall_area;            /* [nb] boundaryVolume (the wall particle's area) */
  const float* wall_rho;             /* [nb] boundaryDensity (relative) */
  const float* wall_volume;          /* [nb] boundaryVolume / boundaryDensity */
  const float* wall_lambda;          /* [nb] the walls' eigVals[:, 1] */
  const float* pressure;             /* [n] fluid pressure (pressureModule.pressure) */
  const float* wall_pressure;        /* [nb] wall pressure */
  float packing;                     /* particle.packing: k0 = W(packing) of the shift */
  float cfl;                         /* shift CFL (1.5 in the reference) */
  int64_t n, nb;                     /* fluid and wall particles (SPH_SURF_PINV_EIG: n rows) */
} sph_surface_in;

#define SPH_SURF_PINV_EIG 0            /* out float4 [n] = pinv2x2(matrix), out2 float2 [n] = its eigVals
                                          (singular values, larger first; src/util.py:386-433) */
#define SPH_SURF_WALL_NORMALIZATION 1  /* out float4 [nb] = the wall's own normalization matrix:
                                          wall->fluid pairs + wall-wall pairs (solidBoundary.py:679-693) */
#define SPH_SURF_NORMAL 2              /* out float2 [n] lambdaGrad, out2 float2 [n] fluidNormal
                                          (deltaPlus.py:132-163; the wall part takes the wall's volume as
                                          fluidArea[b] / fluidDensity[b], as the reference indexes it: every
                                          wall index in the pairs must be below n) */
#define SPH_SURF_ANGLE_MASK 3          /* out [n] 1 where arccos(max dot) > pi/6 and lambda < 0.6, else 0;
                                          out2 float2 [n] (angleMin, angleMax) of the fluid pairs, or NULL
                                          (deltaPlus.py:165-188) */
#define SPH_SURF_CLASSIFY 4            /* out [n] fluidSurfaceMask: 0 surface, 1 near surface (2/3 where
                                          lambda < 0.5), 2 bulk (deltaPlus.py:189-205) */
#define SPH_SURF_SHIFT 5               /* out float2 [n] shiftAmount = -cfl Ma 4 h^2 (fluid + wall sums),
                                          Ma = max |v| / c0; out2 = device scratch of sph_surface_scratch_bytes()
                                          (deltaPlus.py:81-115) */
#define SPH_SURF_SHIFT_ADJUST 6        /* out float2 [n] fluidUpdate (length capped at 0.05 h, projected on
                                          the tangent where mask < 1.5, zero where mask < 0.5); out2 [n] the
                                          updated fluidSurfaceMask (deltaPlus.py:207-240) */
#define SPH_SURF_PRESSURE_ACCEL 7      /* out float2 [n] computePressureAccelDeltaPlus over the fluid pairs
                                          (pressure.py:31-51): -1/rho_i sum_j p_ij V_j gradW_ij with
                                          p_ij = p_i + p_j where p_i >= 0 or mask_i < 1.5, else p_j - p_i */
#define SPH_SURF_WALL_PRESSURE_ACCEL 8 /* out float2 [n] the same over the wall pairs with the wall
                                          pressure and wall volume (solidBoundary.py:876-884) */
size_t sph_surface_scratch_bytes(void);
/* One step of the delta+ module; params gives support, c0.  Asynchronous. */
sph_status_t sph_surface_term(int32_t term, const sph_surface_in* in, const sph_params* params, float* out,
                              float* out2, void* stream);

/* ---------------------------------------------------------------- periodic boundaries (f4) */

/* createGhostParticlesKernel (src/modules/periodicBC.py:23-103) on the GPU: the ghost copies
 * of the particles within `band` (= buffer * support) of the domain edges, in the reference's
 * order: categories x+, x- (periodic_x), y+, y- (periodic_y), then x+y+, x+y-, x-y+, x-y-
 * (both), each in increasing particle index.  indices [capacity] (int64) and offsets float2
 * [capacity] (the position offset of each copy, -+(max - min) in float32) receive the
 * concatenated lists, counts [8] (device) the length of each category (0 for a disabled
 * one); more than `capacity` copies flags SPH_FLAG_PAIR_CAPACITY.  domain_min / domain_max
 * are host float[2]. */
size_t sph_periodic_ghosts_scratch_bytes(int64_t n);
sph_status_t sph_periodic_ghosts(const float* pos, int64_t n, const float* domain_min, const float* domain_max,
                                 float band, int32_t periodic_x, int32_t periodic_y, int64_t capacity,
                                 int64_t* indices, float* offsets, int32_t* counts, int32_t* status, void* scratch,
                                 size_t scratch_bytes, void* stream);
/* Periodic neighbor search without ghost copies: a cell grid of cells >= cell_size tiling the
 * box [domain_min, domain_max) exactly (at least three cells along a periodic direction),
 * neighbor cells wrapped around periodic edges, and a neighbor seen through an edge tested at
 * its image position (x_j +- (max - min), rounded to float32 as the reference's ghost
 * positions are) with the reference predicate sqrtf(fmaf(dx,dx,dy*dy)) < support_i.  The
 * pairs are the reference's pairs of real particles against real particles and ghosts
 * (createGhostParticlesKernel + its search), each ghost replaced by its particle: rows /
 * cols int64 in (i, j) order and codes int8 = (sx + 1) | (sy + 1) << 2 with s the image
 * shift in units of the box length.  Two passes with the same arguments: count writes
 * offsets [n+1] (int64), fill the `capacity` pairs. */
size_t sph_nl_periodic_scratch_bytes(int64_t n, const float* domain_min, const float* domain_max, float cell_size);
sph_status_t sph_nl_periodic_count(const float* pos, const float* support, int64_t n, const float* domain_min,
                                   const float* domain_max, float cell_size, int32_t periodic_x, int32_t periodic_y,
                                   int64_t* offsets, int32_t* status, void* scratch, size_t scratch_bytes,
                                   void* stream);
sph_status_t sph_nl_periodic_fill(const float* pos, const float* support, int64_t n, const float* domain_min,
                                  const float* domain_max, float cell_size, int32_t periodic_x, int32_t periodic_y,
                                  const int64_t* offsets, int64_t capacity, int64_t* rows, int64_t* cols,
                                  int8_t* codes, int32_t* status, void* scratch, size_t scratch_bytes, void* stream);

/* ---------------------------------------------------------------- differentiable rollouts */

/* A free fluid (no walls) stepped by the deltaSPH right-hand side (src/deltaSPH.py:146-200:
 * gravity or point source, continuity, MOG density diffusion when density_diffusion = 1,
 * Tait pressure with gamma 7, artificial and laminar viscosity) and semi-implicit Euler, in
 * float (fp64 = 0) or double (fp64 = 1): x, v, acc are 2-vectors, rho relative density.
 * Pairs: the (i, j)-ordered reference list in original order as row offsets + int64
 * columns (sph_row_offsets of fluidNeighbors), symmetric (one support for all particles). */
sph_status_t sph_drop_rhs(int32_t fp64, int64_t n, const int32_t* offsets, const int64_t* cols, const void* x,
                          const void* v, const void* rho, const void* area, const sph_params* params, void* acc,
                          void* dpdt, void* stream);
/* In place: v += dt acc, x += dt v (new v), rho += dt dpdt / rest_density. */
sph_status_t sph_drop_integrate(int32_t fp64, int64_t n, void* x, void* v, void* rho, const void* acc,
                                const void* dpdt, double dt, double rest_density, void* stream);
/* Discrete adjoint of one step at state (x, v, rho) with the pairs of that state: from the
 * adjoint (lx1, lv1, lr1) of the next state, the adjoint (lx0, lv0, lr0) of this one and
 * dalpha[i] = particle i's share of dLoss/d(params->alpha) for this step.  Vector-Jacobian
 * products by forward-mode dual numbers per pair; each particle gathers over its own row
 * (no atomics). */
sph_status_t sph_drop_adjoint(int32_t fp64, int64_t n, const int32_t* offsets, const int64_t* cols, const void* x,
                              const void* v, const void* rho, const void* area, const sph_params* params, double dt,
                              const void* lx1, const void* lv1, const void* lr1, void* lx0, void* lv0, void* lr0,
                              void* dalpha, void* stream);

/* ---------------------------------------------------------------- DFSPH (a20-a25) */

/* Device work arrays of one DFSPH solve (fluid arrays [n] in sorted order, wall arrays [nb]). */
typedef struct sph_dfsph_buffers {
  float* rho;               /* relative density incl. the wall contribution */
  float* volume;            /* A / fluid-only density (fluidVolume) */
  float* actual_area;       /* A / rho (fluidActualArea) */
  float* vstar;             /* float2 predicted velocity */
  float* alpha;
  float* source;
  float* pressure;          /* fluidPressure2 */
  float* pred_accel;        /* float2 fluidPredAccel */
  float* residual;
  float* wall_rho;          /* wall density (summation, <= 1) */
  float* wall_actual_area;
  float* wall_alpha;
  float* wall_source;
  float* wall_pressure;
  float* wall_residual;
  const float* wall_density_term;  /* static wall-wall kernel sum (sph_dfsph_wall_wall_term) */
  double* partials;         /* [sph_dfsph_partials_count()] */
  float* errors;            /* [max iterations + 1] error of every iteration */
  int32_t* iters;           /* [1] iterations run */
  float* records;           /* [9 n], 16-byte aligned: per-particle pair records of the Jacobi sweeps */
} sph_dfsph_buffers;

size_t sph_dfsph_partials_count(void);
/* Static wall-wall density term sum_b' W(|x_b - x_b'| / h) A_b' (solidBoundary.py:180-200). */
sph_status_t sph_dfsph_wall_wall_term(const sph_wall_view* walls, const sph_grid* grid, const sph_params* params,
                                      float* term, void* stream);
/* Summation density with walls (density.py:26-34 + evalBoundaryDensitySummation,
 * solidBoundary.py:522-549): bufs->rho = rho_fluid + sum_b W A_b, ->volume = A / rho_fluid,
 * ->actual_area = A / rho; wall_rho = min(term + sum_f W A_f, 1), wall_actual_area. */
sph_status_t sph_dfsph_densities(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, const float* rho_fluid, const sph_dfsph_buffers* bufs,
                                 void* stream);
/* One DFSPH pressure solve (DFSPH(), src/modules/dfsph.py:263-311): predicted velocity
 * v* = v + dt acc_in, alpha and source (with PBSPH wall terms when density != 0), then the
 * relaxed-Jacobi loop of densitySolve / divergenceSolve (:195-260) as a single cooperative
 * kernel with an in-kernel reduction of the mean error, bounded by the maximum iteration
 * count; leaves the final predicted acceleration in bufs->pred_accel and the iteration
 * count in bufs->iters.  A non-finite pressure flags SPH_FLAG_NONFINITE (the reference
 * raises 'Pressure solver became unstable!'). */
sph_status_t sph_dfsph_solve(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                             const sph_params* params, const sph_dfsph_buffers* bufs, const float* acc_in,
                             const float* dt, int32_t density, int32_t* status, void* stream);
/* DFSPH steps 11-12 (src/dfsph.py:187-194): acc += artificial viscosity (with walls) +
 * laminar viscosity, with V = A / fluid-only density and rho incl. walls.  Uses
 * bufs->records as scratch for its pair records. */
sph_status_t sph_dfsph_viscosity(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, const sph_dfsph_buffers* bufs, float* acc, void* stream);
/* a += b (float2 [n]); a = (x, y) (float2 [n]). */
sph_status_t sph_add_float2(int64_t n, const float* b, float* a, void* stream);
sph_status_t sph_fill_float2(int64_t n, float x, float y, float* a, void* stream);
/* Adaptive time step (adaptiveTimeSteppingModule.updateTimestep, src/modules/adaptiveDT.py:59-95)
 * entirely on the device: dt <- min(max(target, dt/2), 1.05 dt). */
size_t sph_dt_scratch_bytes(void);
sph_status_t sph_update_dt(int64_t n, const float* v, const float* acc, float support, float kinematic, float cfl,
                           float c0, int32_t acoustic_from_c0, float dt_min, float dt_max, float* dt, void* scratch,
                           size_t scratch_bytes, void* stream);

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
