// Search grid, cell keys and the sort of particles by cell key (sm_103a).
//
// Two sorts are provided; both order particles by (cell key, original index), which is
// what a stable sort of the keys gives:
//   * sph_counting_sort — single-digit radix (counting) sort where the digit is the whole
//     cell key: a global per-cell histogram (atomics, filled by sph_cell_keys), one
//     exclusive scan that is directly the cell begin table, an atomic scatter, and a
//     per-cell fix-up that restores index order inside each cell.  ~6 launches.
//   * sph_radix_sort_pairs (scan_sort.cu) — multi-pass LSD radix sort with 1..8-bit
//     digits; its cell table comes from sph_cell_starts (binary search per cell).
#include <cstdio>

#include "sph_math.cuh"

namespace sph {

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

__device__ sph_grid make_grid(const Bounds& b, int has_min, float min_x, float min_y, int has_max, float max_x,
                              float max_y, int32_t cell_capacity, int32_t* status, int ratio);

// Grid of sortPositions, src/modules/neighborSearch.py:34-46, all in float32:
// qMin = minCoord - hMax*1.0, qMax = maxCoord + 2*hMax*1.0, cells = ceil((qMax-qMin)/hMax).
__global__ void k_bounds_final(const Bounds* __restrict__ part, int nparts, int has_min, float min_x, float min_y,
                               int has_max, float max_x, float max_y, int32_t cell_capacity, sph_grid* grid,
                               int32_t* status, int ratio) {
  __shared__ Bounds sb[32];
  Bounds b{-INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, 0};
  for (int k = threadIdx.x; k < nparts; k += 32) {
    Bounds p = part[k];
    b.hmax = fmaxf(b.hmax, p.hmax);
    b.mnx = fminf(b.mnx, p.mnx);
    b.mny = fminf(b.mny, p.mny);
    b.mxx = fmaxf(b.mxx, p.mxx);
    b.mxy = fmaxf(b.mxy, p.mxy);
    b.nonfinite |= p.nonfinite;
  }
  sb[threadIdx.x] = b;
  __syncwarp();
  if (threadIdx.x != 0) return;
  for (int k = 1; k < 32; ++k) {
    b.hmax = fmaxf(b.hmax, sb[k].hmax);
    b.mnx = fminf(b.mnx, sb[k].mnx);
    b.mny = fminf(b.mny, sb[k].mny);
    b.mxx = fmaxf(b.mxx, sb[k].mxx);
    b.mxy = fmaxf(b.mxy, sb[k].mxy);
    b.nonfinite |= sb[k].nonfinite;
  }
  *grid = make_grid(b, has_min, min_x, min_y, has_max, max_x, max_y, cell_capacity, status, ratio);
}

// The grid of one particle set from its bounds (thread-local).
__device__ sph_grid make_grid(const Bounds& b, int has_min, float min_x, float min_y, int has_max, float max_x,
                              float max_y, int32_t cell_capacity, int32_t* status, int ratio) {
  float hs = __fmul_rn(b.hmax, 1.0f);
  float two_hs = __fmul_rn(__fmul_rn(2.0f, b.hmax), 1.0f);
  float qmin_x = __fsub_rn(has_min ? min_x : b.mnx, hs);
  float qmin_y = __fsub_rn(has_min ? min_y : b.mny, hs);
  float qmax_x = __fadd_rn(has_max ? max_x : b.mxx, two_hs);
  float qmax_y = __fadd_rn(has_max ? max_y : b.mxy, two_hs);
  const float cell = ratio > 1 ? __fdiv_rn(hs, (float)ratio) : hs;
  float ex = __fdiv_rn(__fsub_rn(qmax_x, qmin_x), cell);
  float ey = __fdiv_rn(__fsub_rn(qmax_y, qmin_y), cell);
  sph_grid g;
  g.qmin[0] = qmin_x;
  g.qmin[1] = qmin_y;
  g.hmax = cell;
  g.hmax_threshold = sq_threshold(b.hmax);
  g.threshold_support = b.hmax;
  bool ok = b.nonfinite == 0 && b.hmax > 0.f && isfinite(ex) && isfinite(ey) && ex < 2.0e9f && ey < 2.0e9f;
  int cx = ok ? (int)ceilf(ex) : 0;
  int cy = ok ? (int)ceilf(ey) : 0;
  long long nc = (long long)cx * (long long)cy;
  if (!ok) flag(status, SPH_FLAG_NONFINITE);
  if (nc > (long long)cell_capacity) flag(status, SPH_FLAG_CELL_CAPACITY);
  g.cells_x = cx;
  g.cells_y = cy;
  g.num_cells = nc > (long long)cell_capacity ? cell_capacity + 1 : (int)nc;
  return g;
}

// Grids of many particle sets at once (one block per set): set s is the particles
// [seg[s], seg[s+1]) of the concatenated arrays, with its own optional domain
// min_coords[2s..2s+1] / max_coords[2s..2s+1].  Same arithmetic as sph_grid_build.
__global__ void __launch_bounds__(kRedThreads) k_grid_segments(const float2* __restrict__ pos,
                                                               const float* __restrict__ h,
                                                               const int64_t* __restrict__ seg, int nseg,
                                                               const float* __restrict__ min_coords,
                                                               const float* __restrict__ max_coords,
                                                               int32_t cell_capacity, sph_grid* __restrict__ grids,
                                                               int32_t* status) {
  const int s = blockIdx.x;
  if (s >= nseg) return;
  float hm = -INFINITY, mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  int bad = 0;
  for (int64_t i = seg[s] + threadIdx.x; i < seg[s + 1]; i += blockDim.x) {
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
  if (threadIdx.x != 0) return;
  Bounds b = sb[0];
  for (int w = 1; w < kRedThreads / 32; ++w) {
    b.hmax = fmaxf(b.hmax, sb[w].hmax);
    b.mnx = fminf(b.mnx, sb[w].mnx);
    b.mny = fminf(b.mny, sb[w].mny);
    b.mxx = fmaxf(b.mxx, sb[w].mxx);
    b.mxy = fmaxf(b.mxy, sb[w].mxy);
    b.nonfinite |= sb[w].nonfinite;
  }
  grids[s] = make_grid(b, min_coords != nullptr, min_coords ? min_coords[2 * s] : 0.f,
                       min_coords ? min_coords[2 * s + 1] : 0.f, max_coords != nullptr,
                       max_coords ? max_coords[2 * s] : 0.f, max_coords ? max_coords[2 * s + 1] : 0.f,
                       cell_capacity, status, 1);
}

// counter[key] += 1 for every lane, one atomic per distinct key of the warp: particles come
// nearly sorted from the previous step, so a warp's lanes share a few cells and their
// atomics would otherwise serialize.
__device__ __forceinline__ void warp_count(int32_t* __restrict__ counter, uint32_t key) {
  const unsigned peers = __match_any_sync(__activemask(), key);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(counter + key, __popc(peers));
}

// As warp_count for the lanes with `in`, except that the sentinel key takes one atomic per
// block: the sentinel cell can hold millions of particles (the free slots of a pooled
// batch), and one atomic per warp on its single counter would serialize.  Every thread of
// the block calls it (blocks of a multiple of 32 threads).
__device__ __forceinline__ void block_count(int32_t* __restrict__ counter, uint32_t key, bool in, uint32_t sentinel) {
  __shared__ int s_n;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const bool sent = in && key == sentinel;
  if (in && !sent) warp_count(counter, key);
  const unsigned b = __ballot_sync(0xffffffffu, sent);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s_n, __popc(b));
  __syncthreads();
  if (threadIdx.x == 0 && s_n) atomicAdd(counter + sentinel, s_n);
}

__global__ void k_cell_keys(const float2* __restrict__ pos, int64_t n, const sph_grid* __restrict__ gp,
                            int32_t cell_capacity, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                            int32_t* __restrict__ cell_count, int32_t* status) {
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
  if (vals) vals[i] = (uint32_t)i;
  if (cell_count) warp_count(cell_count, key);
}

// Batch of scenes: key = coff_s + ix + cells_x_s * iy with scene s's own grid.  Scene s owns
// the slots coff_s .. coff_s + num_cells_s: its cells, then one outside slot for particles
// that left its grid (or became non-finite).  Those particles have no neighbors and move
// under body forces only, and every scene stays one contiguous range of the sorted order.
// A scene whose slots do not fit the table gets the sentinel cell_capacity.
__global__ void k_batch_cell_keys(const float2* __restrict__ pos, int64_t n, const int32_t* __restrict__ sid,
                                  const SceneDev* __restrict__ scenes, int32_t cell_capacity,
                                  uint32_t* __restrict__ keys, int32_t* __restrict__ cell_count, int32_t* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < n;   // no early exit: the whole block takes part in block_count
  uint32_t key = (uint32_t)cell_capacity;
  if (in) {
    // a particle of no scene (scene index < 0: a free or retired slot of a pooled batch) goes
    // to the sentinel cell after every scene's cells, without a flag
    const int32_t s = sid[i];
    const SceneDev& S = scenes[s < 0 ? 0 : s];
    const sph_grid& g = S.g;
    const float2 p = pos[i];
    const bool fits = s >= 0 && S.coff >= 0 && S.coff + g.num_cells < cell_capacity;
    if (fits) key = (uint32_t)(S.coff + g.num_cells);
    if (s < 0) {
    } else if (!isfinite(p.x) || !isfinite(p.y)) {
      flag(status, SPH_FLAG_NONFINITE);
    } else {
      int ix = cell_coord(p.x, g.qmin[0], g.hmax);
      int iy = cell_coord(p.y, g.qmin[1], g.hmax);
      if (ix >= 0 && iy >= 0 && ix < g.cells_x && iy < g.cells_y && fits)
        key = (uint32_t)(S.coff + ix + g.cells_x * iy);
      else
        flag(status, SPH_FLAG_OUT_OF_GRID);
    }
    keys[i] = key;
  }
  block_count(cell_count, key, in, (uint32_t)cell_capacity);
}

// Counting-sort scatter: slot = cell_start[key] + (remaining count of the cell) - 1, one
// atomic per distinct key of the warp (the lanes of a key take consecutive slots); the
// sentinel key takes one atomic per block (block_count).  Decrementing the histogram leaves
// it all zero for the next sort.
__global__ void k_count_scatter(const uint32_t* __restrict__ keys, int64_t n, const int32_t* __restrict__ cell_start,
                                int32_t* __restrict__ cell_count, uint32_t* __restrict__ tmp, uint32_t sentinel) {
  __shared__ int s_n, s_left;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < n;   // no early exit: the whole block takes part in the sentinel slots
  const uint32_t k = in ? keys[i] : 0u;
  const bool sent = in && k == sentinel;
  const int lane = (int)(threadIdx.x & 31);
  if (in && !sent) {
    const unsigned peers = __match_any_sync(__activemask(), k);
    const int leader = __ffs(peers) - 1;
    int left = 0;
    if (lane == leader) left = atomicSub(cell_count + k, __popc(peers));
    left = __shfl_sync(peers, left, leader);
    const int slot = cell_start[k] + left - 1 - __popc(peers & ((1u << lane) - 1u));
    tmp[slot] = (uint32_t)i;
  }
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const unsigned b = __ballot_sync(0xffffffffu, sent);
  int base = 0;
  if (lane == 0 && b) base = atomicAdd(&s_n, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  __syncthreads();
  if (threadIdx.x == 0 && s_n) s_left = atomicSub(cell_count + sentinel, s_n);
  __syncthreads();
  if (sent) tmp[cell_start[sentinel] + s_left - 1 - base - __popc(b & ((1u << lane) - 1u))] = (uint32_t)i;
}

constexpr int kRankSortMax = 1024;   // large cells up to this size are ranked in shared memory
constexpr int kSmallCell = 48;    // cells up to this size are ordered by ranking, one thread per particle
constexpr int kBlockSortMax = 2048;  // larger cells: one block, bitonic sort in shared memory

// Sort key inside a cell: the particle's index, or (tie[index], index) when a tie key is
// given (e.g. a particle id, which makes the order independent of the previous order).
__device__ __forceinline__ uint64_t cell_rank(uint32_t x, const uint32_t* __restrict__ tie) {
  return tie ? (((uint64_t)__ldg(tie + x)) << 32) | x : (uint64_t)x;
}

// Per-slot fix-up of ascending (tie, index) order inside every cell, and the sorted keys.
// After the scatter, cell c's particles fill [cell_start[c], cell_start[c+1]) in atomic
// order; the thread of slot t counts the cell's particles that rank below its own and
// writes its particle to that place (k comparisons per particle, L1-resident).  Cells larger
// than kSmallCell are queued for k_cell_fix_large by the thread of their first slot.
// The sentinel cell (the key cell_capacity: particles outside every grid, or of no scene in
// a pooled batch) keeps the scatter order: nothing reads its order.
__global__ void __launch_bounds__(256) k_cell_fix(const uint32_t* __restrict__ keys, int64_t n,
                                                  const int32_t* __restrict__ cell_start,
                                                  const uint32_t* __restrict__ tmp, const uint32_t* __restrict__ tie,
                                                  uint32_t* __restrict__ order, uint32_t* __restrict__ sorted_keys,
                                                  int32_t* __restrict__ big_list, int32_t* __restrict__ big_count,
                                                  const ArraySet rows, uint32_t sentinel) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t x = tmp[t];
  const uint32_t c = __ldg(keys + x);
  sorted_keys[t] = c;
  if (c == sentinel) {
    order[t] = x;
    copy_rows(rows, t, x);
    return;
  }
  const int b = __ldg(cell_start + c), e = __ldg(cell_start + c + 1);
  if (e - b > kSmallCell) {
    if (t == b) big_list[atomicAdd(big_count, 1)] = (int32_t)c;
    return;
  }
  const uint64_t mine = cell_rank(x, tie);
  int rank = 0;
  for (int u = b; u < e; ++u) rank += cell_rank(__ldg(tmp + u), tie) < mine;
  order[b + rank] = x;
  copy_rows(rows, b + rank, x);
}

// One block per large cell, its (tie, index) ranks in shared memory: up to kRankSortMax
// entries each thread counts the smaller ranks of its entries (one barrier); above that a
// bitonic sort, up to kBlockSortMax entries.  Bigger cells keep the atomic scatter order
// (their pair set is unchanged; only the order inside that cell is not reproducible) and
// flag SPH_FLAG_CELL_ORDER.
__global__ void __launch_bounds__(512) k_cell_fix_large(const int32_t* __restrict__ cell_start,
                                                        const uint32_t* __restrict__ tmp,
                                                        const uint32_t* __restrict__ tie,
                                                        uint32_t* __restrict__ order,
                                                        const int32_t* __restrict__ big_list,
                                                        const int32_t* __restrict__ big_count, int32_t* status,
                                                        const ArraySet rows) {
  __shared__ uint64_t s[kBlockSortMax];
  const int nbig = *big_count;
  for (int q = blockIdx.x; q < nbig; q += gridDim.x) {
    const int c = big_list[q];
    const int b = cell_start[c], e = cell_start[c + 1];
    const int k = e - b;
    if (k > kBlockSortMax) {
      for (int t = threadIdx.x; t < k; t += blockDim.x) {
        order[b + t] = tmp[b + t];
        copy_rows(rows, b + t, tmp[b + t]);
      }
      if (threadIdx.x == 0) flag(status, SPH_FLAG_CELL_ORDER);
      continue;
    }
    if (k <= kRankSortMax) {
      for (int t = threadIdx.x; t < k; t += blockDim.x) s[t] = cell_rank(tmp[b + t], tie);
      __syncthreads();
      for (int t = threadIdx.x; t < k; t += blockDim.x) {
        const uint64_t mine = s[t];
        int rank = 0;
#pragma unroll 4
        for (int u = 0; u < k; ++u) rank += s[u] < mine;   // every lane reads the same word
        order[b + rank] = (uint32_t)(mine & 0xffffffffu);
        copy_rows(rows, b + rank, (uint32_t)(mine & 0xffffffffu));
      }
      __syncthreads();
      continue;
    }
    int p2 = 1;
    while (p2 < k) p2 <<= 1;
    for (int t = threadIdx.x; t < p2; t += blockDim.x) s[t] = t < k ? cell_rank(tmp[b + t], tie) : ~0ull;
    __syncthreads();
    for (int size = 2; size <= p2; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < p2; t += blockDim.x) {
          int u = t ^ stride;
          if (u > t) {
            bool up = (t & size) == 0;
            uint64_t a = s[t], bb = s[u];
            if ((a > bb) == up) {
              s[t] = bb;
              s[u] = a;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int t = threadIdx.x; t < k; t += blockDim.x) {
      order[b + t] = (uint32_t)(s[t] & 0xffffffffu);
      copy_rows(rows, b + t, (uint32_t)(s[t] & 0xffffffffu));
    }
    __syncthreads();
  }
}

// cell_start[c] = lower_bound(sorted_keys, c) for c = 0..cap+1 (used after the LSD radix sort).
__global__ void k_cell_starts(const uint32_t* __restrict__ keys, int64_t n, int32_t cap,
                              int32_t* __restrict__ cell_start) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > (int64_t)cap + 1) return;
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if ((int64_t)keys[mid] < c) lo = mid + 1; else hi = mid;
  }
  cell_start[c] = (int32_t)lo;
}

__global__ void k_gather_sorted(const uint32_t* __restrict__ order, int64_t n, const float2* __restrict__ pos,
                                const float* __restrict__ h, const float* __restrict__ a, float2* __restrict__ xy,
                                float* __restrict__ sh, float* __restrict__ sa) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint32_t o = order[s];
  xy[s] = pos[o];
  if (sh) sh[s] = h[o];
  if (sa) sa[s] = a[o];
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

__global__ void k_invert_perm(const uint32_t* __restrict__ order, int64_t n, uint32_t* __restrict__ rank) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) rank[order[s]] = (uint32_t)s;
}

// ------------------------------------------------------------------ constructHashMap
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

// The occupied-cell count C = num_cells[0] is read on the device (the total of the head scan),
// so the map is built without a host round trip; launched over n >= C threads.
__global__ void k_cell_emit(const int32_t* __restrict__ num_cells, int64_t n, const uint32_t* __restrict__ c_id,
                            const int32_t* __restrict__ c_lin, const int32_t* __restrict__ c_begin,
                            int32_t* __restrict__ cell_indices, int32_t* __restrict__ cum_cell,
                            int32_t* __restrict__ cell_span) {
  const int64_t C = *num_cells;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C) return;
  uint32_t c = c_id[k];
  int32_t b = c_begin[c];
  int32_t e = (int64_t)c + 1 < C ? c_begin[c + 1] : (int32_t)n;
  cell_indices[k] = c_lin[c];
  cum_cell[k] = e - b;
  cell_span[k] = b;
}

// Every slot of the hash-sort input starts as the sentinel hash L (above every real hash), so
// the n-item sort puts the C occupied cells first, in (hash, cell) order, and the rest after.
__global__ void k_hash_sentinel(uint32_t* __restrict__ c_hash, uint32_t* __restrict__ c_id, int64_t n, int32_t L) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    c_hash[k] = (uint32_t)L;
    c_id[k] = (uint32_t)k;
  }
}

__global__ void k_table_init(int32_t* __restrict__ table, int32_t L) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < L) {
    table[2 * b] = -1;
    table[2 * b + 1] = 0;
  }
}

__global__ void k_table_fill(const uint32_t* __restrict__ sorted_hash, const int32_t* __restrict__ num_cells,
                             int32_t* __restrict__ table) {
  const int64_t C = *num_cells;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C) return;
  uint32_t hv = sorted_hash[k];
  if (k > 0 && sorted_hash[k - 1] == hv) return;
  int64_t e = k + 1;
  while (e < C && sorted_hash[e] == hv) ++e;
  table[2 * (int64_t)hv] = (int32_t)k;
  table[2 * (int64_t)hv + 1] = (int32_t)(e - k);
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
  return sph_grid_build_ratio(pos, support, n, min_coord, max_coord, 1, cell_capacity, grid, status, scratch,
                              scratch_bytes, stream);
}

sph_status_t sph_grid_build_ratio(const float* pos, const float* support, int64_t n, const float* min_coord,
                                  const float* max_coord, int32_t cell_ratio, int32_t cell_capacity, sph_grid* grid,
                                  int32_t* status, void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n > 0 && pos && support && grid && cell_capacity > 0 && cell_capacity < 0x7ffffffe &&
                  cell_ratio >= 1 && cell_ratio <= 8,
              "grid_build: bad arguments");
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
                                   grid, status, (int)cell_ratio);
  SPH_CHECK_LAUNCH("grid_build");
  return SPH_OK;
}

sph_status_t sph_grid_build_segments(const float* pos, const float* support, const int64_t* seg_offsets,
                                     int32_t nseg, const float* min_coords, const float* max_coords,
                                     int32_t cell_capacity, sph_grid* grids, int32_t* status, void* stream) {
  SPH_REQUIRE(nseg >= 0 && (nseg == 0 || (pos && support && seg_offsets && grids && status)) && cell_capacity > 0 &&
                  cell_capacity < 0x7ffffffe,
              "grid_build_segments: bad arguments");
  if (nseg == 0) return SPH_OK;
  k_grid_segments<<<nseg, kRedThreads, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(pos), support,
                                                               seg_offsets, nseg, min_coords, max_coords,
                                                               cell_capacity, grids, status);
  SPH_CHECK_LAUNCH("grid_build_segments");
  return SPH_OK;
}

sph_status_t sph_cell_keys(const float* pos, int64_t n, const sph_grid* grid, int32_t cell_capacity, uint32_t* keys,
                           uint32_t* vals, int32_t* cell_count, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && pos && grid && keys && cell_capacity > 0, "cell_keys: bad arguments");
  if (n == 0) return SPH_OK;
  k_cell_keys<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(pos), n, grid,
                                                               cell_capacity, keys, vals, cell_count, status);
  SPH_CHECK_LAUNCH("cell_keys");
  return SPH_OK;
}

int32_t sph_key_bits(int32_t cell_capacity) { return key_bits_for(cell_capacity); }

sph_status_t sph_batch_cell_keys(const float* pos, int64_t n, const int32_t* sid, const void* scenes,
                                 int32_t cell_capacity, uint32_t* keys, int32_t* cell_count, int32_t* status,
                                 void* stream) {
  SPH_REQUIRE(n >= 0 && pos && sid && scenes && keys && cell_count && cell_capacity > 0,
              "batch_cell_keys: bad arguments");
  if (n == 0) return SPH_OK;
  k_batch_cell_keys<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(pos), n, sid,
                                                                     static_cast<const SceneDev*>(scenes),
                                                                     cell_capacity, keys, cell_count, status);
  SPH_CHECK_LAUNCH("batch_cell_keys");
  return SPH_OK;
}

size_t sph_counting_sort_scratch_bytes(int64_t n, int32_t cell_capacity) {
  size_t b = (size_t)(n < 1 ? 1 : n) * sizeof(uint32_t) + 256;          // scatter target
  b += ((size_t)cell_capacity + 1) * sizeof(int32_t) + 256;              // large-cell list
  b += 256;                                                               // large-cell count
  b += sph_scan_scratch_bytes((int64_t)cell_capacity + 1) + 256;
  return b;
}

sph_status_t sph_counting_sort(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                               int32_t* cell_start, uint32_t* order, uint32_t* sorted_keys, int32_t* status,
                               void* scratch, size_t scratch_bytes, void* stream) {
  return sph_counting_sort_tie(keys, n, cell_capacity, cell_count, cell_start, nullptr, order, sorted_keys, status,
                               scratch, scratch_bytes, stream);
}

static sph_status_t counting_sort_impl(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                                       int32_t* cell_start, const uint32_t* tie, uint32_t* order,
                                       uint32_t* sorted_keys, const ArraySet& rows, int32_t* status, void* scratch,
                                       size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n >= 0 && n < ((int64_t)1 << 31) && keys && cell_count && cell_start && order && sorted_keys &&
                  cell_capacity > 0,
              "counting_sort: bad arguments");
  if (!scratch || scratch_bytes < sph_counting_sort_scratch_bytes(n, cell_capacity)) {
    set_error_text("counting_sort: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  char* p = reinterpret_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  uint32_t* tmp = reinterpret_cast<uint32_t*>(take((size_t)(n < 1 ? 1 : n) * sizeof(uint32_t)));
  int32_t* big_list = reinterpret_cast<int32_t*>(take(((size_t)cell_capacity + 1) * sizeof(int32_t)));
  int32_t* big_count = reinterpret_cast<int32_t*>(take(sizeof(int32_t)));
  size_t scan_b = sph_scan_scratch_bytes((int64_t)cell_capacity + 1);
  void* scan_s = take(scan_b);
  const int64_t slots = (int64_t)cell_capacity + 1;  // cells 0..cap-1 and the sentinel cap
  sph_status_t s = sph_exclusive_scan_i32(cell_count, cell_start, slots, scan_s, scan_b, stream);
  if (s != SPH_OK) return s;
  if (n == 0) return SPH_OK;
  cudaMemsetAsync(big_count, 0, sizeof(int32_t), st);
  k_count_scatter<<<grid_for(n, 256), 256, 0, st>>>(keys, n, cell_start, cell_count, tmp, (uint32_t)cell_capacity);
  k_cell_fix<<<grid_for(n, 256), 256, 0, st>>>(keys, n, cell_start, tmp, tie, order, sorted_keys, big_list,
                                               big_count, rows, (uint32_t)cell_capacity);
  k_cell_fix_large<<<4 * kNumSMs, 512, 0, st>>>(cell_start, tmp, tie, order, big_list, big_count, status, rows);
  SPH_CHECK_LAUNCH("counting_sort");
  return SPH_OK;
}

sph_status_t sph_counting_sort_tie(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                                   int32_t* cell_start, const uint32_t* tie, uint32_t* order, uint32_t* sorted_keys,
                                   int32_t* status, void* scratch, size_t scratch_bytes, void* stream) {
  ArraySet none;
  array_set_from(0, nullptr, nullptr, nullptr, &none);
  return counting_sort_impl(keys, n, cell_capacity, cell_count, cell_start, tie, order, sorted_keys, none, status,
                            scratch, scratch_bytes, stream);
}

sph_status_t sph_counting_sort_permute(const uint32_t* keys, int64_t n, int32_t cell_capacity, int32_t* cell_count,
                                       int32_t* cell_start, const uint32_t* tie, uint32_t* order,
                                       uint32_t* sorted_keys, int32_t count, const int32_t* elem_bytes,
                                       const void* const* in, void* const* out, int32_t* status, void* scratch,
                                       size_t scratch_bytes, void* stream) {
  ArraySet rows;
  SPH_REQUIRE(array_set_from(count, elem_bytes, in, out, &rows),
              "counting_sort_permute: at most 8 arrays, each with distinct in/out and 4, 8 or 16-byte rows");
  return counting_sort_impl(keys, n, cell_capacity, cell_count, cell_start, tie, order, sorted_keys, rows, status,
                            scratch, scratch_bytes, stream);
}

sph_status_t sph_cell_starts(const uint32_t* sorted_keys, int64_t n, int32_t cell_capacity, int32_t* cell_start,
                             void* stream) {
  SPH_REQUIRE(n >= 0 && cell_capacity > 0 && cell_start && (n == 0 || sorted_keys), "cell_starts: bad arguments");
  k_cell_starts<<<grid_for((int64_t)cell_capacity + 2, 256), 256, 0, as_stream(stream)>>>(sorted_keys, n,
                                                                                           cell_capacity, cell_start);
  SPH_CHECK_LAUNCH("cell_starts");
  return SPH_OK;
}

sph_status_t sph_gather_sorted(const uint32_t* order, int64_t n, const float* pos, const float* support,
                               const float* area, float* xy, float* sorted_support, float* sorted_area,
                               void* stream) {
  SPH_REQUIRE(n >= 0 && order && pos && xy, "gather_sorted: bad arguments");
  SPH_REQUIRE(!sorted_support || support, "gather_sorted: sorted_support needs support");
  SPH_REQUIRE(!sorted_area || area, "gather_sorted: sorted_area needs area");
  if (n == 0) return SPH_OK;
  k_gather_sorted<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, n, reinterpret_cast<const float2*>(pos),
                                                                    support, area, reinterpret_cast<float2*>(xy),
                                                                    sorted_support, sorted_area);
  SPH_CHECK_LAUNCH("gather_sorted");
  return SPH_OK;
}

sph_status_t sph_scatter_f32(const uint32_t* order, const float* in, int64_t n, float* out, void* stream) {
  SPH_REQUIRE(n >= 0 && order && in && out, "scatter_f32: bad arguments");
  if (n == 0) return SPH_OK;
  k_scatter_f32<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, in, n, out);
  SPH_CHECK_LAUNCH("scatter_f32");
  return SPH_OK;
}

sph_status_t sph_scatter_counts(const uint32_t* order, const int32_t* counts, int64_t n, int32_t* out, void* stream) {
  SPH_REQUIRE(n >= 0 && order && counts && out, "scatter_counts: bad arguments");
  if (n == 0) return SPH_OK;
  k_scatter_counts<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, counts, n, out);
  SPH_CHECK_LAUNCH("scatter_counts");
  return SPH_OK;
}

sph_status_t sph_invert_permutation(const uint32_t* order, int64_t n, uint32_t* rank, void* stream) {
  SPH_REQUIRE(n >= 0 && order && rank, "invert_permutation: bad arguments");
  if (n == 0) return SPH_OK;
  k_invert_perm<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, n, rank);
  SPH_CHECK_LAUNCH("invert_permutation");
  return SPH_OK;
}

size_t sph_hash_map_scratch_bytes(int64_t n, int32_t hash_len) {
  size_t nn = (size_t)(n < 1 ? 1 : n) + 1;
  size_t b = 6 * (nn * sizeof(int32_t) + 256);
  b += sph_scan_scratch_bytes(n) + 256;
  b += sph_radix_sort_scratch_bytes(n, 8) + 256;
  (void)hash_len;
  return b + 1024;
}

sph_status_t sph_hash_map_build(const uint32_t* sorted_keys, int64_t n, int32_t cells_x, int32_t hash_len,
                                int32_t* hash_table, int32_t* cell_indices, int32_t* cum_cell, int32_t* cell_span,
                                int32_t* num_cells, void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n > 0 && n < ((int64_t)1 << 31) && sorted_keys && cells_x > 0 && hash_len > 0 &&
                  hash_len < 0x7fffffff && hash_table && cell_indices && cum_cell && cell_span && num_cells,
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
  k_hash_sentinel<<<grid_for(n, 256), 256, 0, st>>>(c_hash, c_id, n, hash_len);
  k_cell_compact<<<grid_for(n, 256), 256, 0, st>>>(sorted_keys, n, head, slot, cells_x, hash_len, c_lin, c_begin,
                                                   c_hash, c_id);
  SPH_CHECK_LAUNCH("hash_map_build(compact)");
  const int32_t* C = slot + n;  // occupied cells (the scan total), on the device
  cudaError_t e = cudaMemcpyAsync(num_cells, C, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) {
    set_error("hash_map_build(count)", e);
    return SPH_ERR_CUDA;
  }
  // stable sort of all n slots by hash, the sentinel L included in the key width
  s = sph_radix_sort_pairs(c_hash, c_id, n, key_bits_for(hash_len), 8, rs_s, rs_b, stream);
  if (s != SPH_OK) return s;
  k_cell_emit<<<grid_for(n, 256), 256, 0, st>>>(C, n, c_id, c_lin, c_begin, cell_indices, cum_cell, cell_span);
  k_table_init<<<grid_for(hash_len, 256), 256, 0, st>>>(hash_table, hash_len);
  k_table_fill<<<grid_for(n, 256), 256, 0, st>>>(c_hash, C, hash_table);
  SPH_CHECK_LAUNCH("hash_map_build");
  return SPH_OK;
}

}  // extern "C"
