// Two-pass CSR neighbor list over particles in cell-sorted order (sm_103a).
//
// Layout: xy (float2, sorted), sorted support h, sorted area A, sorted cell keys, and the
// cell begin table cell_start[c] (cell c = [cell_start[c], cell_start[c+1])).  With the
// linear cell id ix + cells_x*iy, the cells (cx-r .. cx+r, yy) of one grid row are
// contiguous in the sorted order, so a particle scans 2r+1 contiguous index ranges.
//
// The pair test is the reference's sqrtf(fmaf(dx,dx,dy*dy)) < h_i in its square-root-free
// exact form v <= F_i (sq_threshold); the distance is taken only for accepted pairs that
// need it (density).
#include "sph_math.cuh"

namespace sph {

// Segments kept per particle by the one-scene search (the batch step's force passes keep
// kMaxSegments): a particle with more goes on the dense list.  24 covers three cell rows of
// up to 8 x 32 candidates each, ~9x the density of a jittered lattice at support 3 dx.
constexpr int kSearchSegments = 24;

// segment_mask with the density terms of the accepted candidates added to acc in index
// order, in the same unrolled pass: the terms of a candidate pair are formed together on
// the paired float32 instructions and only the accepted ones are added (the caller scales
// the sum by c_w).  Distance r = v * rsqrt(max(v, 1e-30)): 0 for the particle itself,
// within a few ulp of sqrt(v) otherwise.  W(q) / c_w = (1-q)^4 (1+4q), src/kernels.py:20-24.
__device__ __forceinline__ uint32_t segment_mask_density(const float2* __restrict__ x, const float* __restrict__ sa,
                                                         int c, int e, float xi, float yi, float thr,
                                                         float inv_support, float& acc) {
  const int len = min(e - c, 32);
  uint32_t m = 0;
  const float2 qx = make_float2(xi, xi), qy = make_float2(yi, yi), is2 = make_float2(inv_support, inv_support);
#pragma unroll
  for (int t = 0; t < 32; t += 2) {
    if (t < len) {
      const bool two = t + 1 < len;
      const float2 a = __ldg(x + c + t), b = two ? __ldg(x + c + t + 1) : a;
      const float2 dx = __fadd2_rn(qx, make_float2(-a.x, -b.x));
      const float2 dy = __fadd2_rn(qy, make_float2(-a.y, -b.y));
      const float2 v = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
      const bool in0 = v.x <= thr, in1 = two && v.y <= thr;
      if (in0) m |= 1u << t;
      if (in1) m |= 2u << t;
      if (in0 || in1) {
        const float2 rs = __fmul2_rn(make_float2(rsqrt_normal(fmaxf(v.x, 1e-30f)), rsqrt_normal(fmaxf(v.y, 1e-30f))), is2);
        const float2 q = __fmul2_rn(v, rs);
        const float2 am = __fadd2_rn(make_float2(1.f, 1.f), make_float2(-q.x, -q.y));
        const float2 a2 = __fmul2_rn(am, am);
        const float2 w = __fmul2_rn(__fmul2_rn(a2, a2), __ffma2_rn(make_float2(4.f, 4.f), q, make_float2(1.f, 1.f)));
        if (in0) acc = fmaf(w.x, __ldg(sa + c + t), acc);
        if (in1) acc = fmaf(w.y, __ldg(sa + c + t + 1), acc);
      }
    }
  }
  return m;
}

template <typename F>
__device__ __forceinline__ void scan_candidates(const float2* __restrict__ xy, const int32_t* __restrict__ cell_start,
                                                const sph_grid& g, int r, int cx, int cy, float xi, float yi,
                                                float thr, F&& f) {
  const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
  if (x0 > x1) return;
  const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
  for (int yy = y0; yy <= y1; ++yy) {
    const int row = yy * g.cells_x;
    const int b = __ldg(cell_start + row + x0);
    const int e = __ldg(cell_start + row + x1 + 1);
    for (int j = b; j < e; ++j) {
      const float2 pj = __ldg(xy + j);
      const float v = dist2_ref(xi, yi, pj.x, pj.y);
      if (v <= thr) f(j, v);
    }
  }
}

__global__ void __launch_bounds__(256) k_nl_count(const float2* __restrict__ xy, const float* __restrict__ sh,
                                                  const float* __restrict__ sa, int64_t n,
                                                  const uint32_t* __restrict__ keys,
                                                  const int32_t* __restrict__ cell_start,
                                                  const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                  float inv_support, float c_w, int32_t* __restrict__ counts,
                                                  float* __restrict__ rho) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const sph_grid g = *gp;
  const uint32_t key = keys[s];
  int cnt = 0;
  float acc = 0.f;
  if (grid_ok(g, cap) && key < (uint32_t)g.num_cells) {
    const float2 pi = xy[s];
    const float thr = grid_threshold(sh[s], g);
    const int cx = (int)(key % (uint32_t)g.cells_x), cy = (int)(key / (uint32_t)g.cells_x);
    if (rho) {   // the candidates in segments of 32, as k_nl_segments, so both give the same sums
      const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
      const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
      for (int yy = y0; yy <= y1 && x0 <= x1; ++yy) {
        const int row = yy * g.cells_x;
        const int b = __ldg(cell_start + row + x0), e = __ldg(cell_start + row + x1 + 1);
        for (int c = b; c < e; c += 32) {
          cnt += __popc(segment_mask_density(xy, sa, c, e, pi.x, pi.y, thr, inv_support, acc));
        }
      }
      acc *= c_w;
    } else {
      scan_candidates(xy, cell_start, g, r, cx, cy, pi.x, pi.y, thr, [&](int, float) { ++cnt; });
    }
  }
  counts[s] = cnt;
  if (rho) rho[s] = acc;
}

constexpr int kFillStage = 8192;  // CSR columns one 256-thread block builds in shared memory (32 KiB)

// Writes the row [offsets[s], offsets[s+1]) of particle s with the columns `scan` emits.
// The rows of one block are one contiguous span of cols, written through a shared-memory
// stage in windows of kFillStage columns: for each window the rows that reach into it emit
// their columns that fall inside it (a row across a window edge is emitted once per window
// it touches), and the block stores the window with coalesced stores.  A block whose span
// ends past the column buffer writes its rows in place instead, and a row that does not
// fit is skipped with SPH_FLAG_PAIR_CAPACITY set.  Every thread of the block must call
// this (inactive ones with active = false): it holds block barriers.
template <typename Scan>
__device__ __forceinline__ void staged_fill(int64_t s, int64_t n, bool active, const int32_t* __restrict__ offsets,
                                            int64_t pair_capacity, int32_t* __restrict__ cols, int32_t* status,
                                            Scan&& scan) {
  __shared__ int32_t stage[kFillStage];
  const int64_t b0 = (int64_t)blockIdx.x * blockDim.x;
  const int64_t b1 = min(b0 + (int64_t)blockDim.x, n);
  const int64_t span0 = offsets[b0], span1 = offsets[b1];
  const bool staged = span0 >= 0 && span1 >= span0 && span1 <= pair_capacity;  // the same in the whole block
  if (!staged) {
    if (!active) return;
    if ((int64_t)offsets[s + 1] <= pair_capacity) {
      int32_t o = offsets[s];
      const int32_t e = offsets[s + 1];
      if (o >= 0) scan([&](int j) {   // writes stay inside the row even if offsets disagree with the scan
        if (o < e) cols[o++] = j;
      });
    } else {
      flag(status, SPH_FLAG_PAIR_CAPACITY);
    }
    return;
  }
  if (span1 - span0 <= kFillStage) {   // one window
    if (active) {
      int32_t o = offsets[s] - (int32_t)span0;
      const int32_t e = offsets[s + 1] - (int32_t)span0;
      if (o >= 0) scan([&](int j) {
        if (o < e) stage[o++] = j;
      });
    }
    __syncthreads();
    for (int k = threadIdx.x; k < (int)(span1 - span0); k += blockDim.x) cols[span0 + k] = stage[k];
    return;
  }
  const int64_t r0 = active ? offsets[s] : 0, r1 = active ? offsets[s + 1] : 0;
  for (int64_t w0 = span0; w0 < span1; w0 += kFillStage) {
    const int64_t w1 = min(w0 + (int64_t)kFillStage, span1);
    if (active && r0 < w1 && r1 > w0) {
      int64_t o = r0;
      scan([&](int j) {
        if (o >= w0 && o < w1 && o < r1) stage[o - w0] = j;
        ++o;
      });
    }
    __syncthreads();
    for (int64_t k = threadIdx.x; k < w1 - w0; k += blockDim.x) cols[w0 + k] = stage[k];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_nl_fill(const float2* __restrict__ xy, const float* __restrict__ sh, int64_t n,
                                                 const uint32_t* __restrict__ keys,
                                                 const int32_t* __restrict__ cell_start,
                                                 const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                 const int32_t* __restrict__ offsets, int64_t pair_capacity,
                                                 int32_t* __restrict__ cols, int32_t* status) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const sph_grid g = *gp;
  const uint32_t key = s < n ? keys[s] : 0xffffffffu;
  const bool active = s < n && grid_ok(g, cap) && key < (uint32_t)g.num_cells;
  float2 pi = make_float2(0.f, 0.f);
  float thr = 0.f;
  if (active) {
    pi = xy[s];
    thr = grid_threshold(sh[s], g);
  }
  const int cx = active ? (int)(key % (uint32_t)g.cells_x) : 0, cy = active ? (int)(key / (uint32_t)g.cells_x) : 0;
  staged_fill(s, n, active, offsets, pair_capacity, cols, status, [&](auto&& emit) {
    scan_candidates(xy, cell_start, g, r, cx, cy, pi.x, pi.y, thr, [&](int j, float) { emit(j); });
  });
}

// One candidate pass for count, density and the CSR fill: particle s's cell rows are
// tested in segments of 32 candidates (segment_mask); the non-empty segments are stored for
// k_nl_fill_segments, the count is their bit count, and the density visits the set bits in
// order, the order of k_nl_count, so both give the same sums.  A particle with more than
// kSearchSegments segments gets nseg[s] = -1 and goes on the dense list, whose rows
// k_nl_fill_dense writes one warp per particle.
__global__ void __launch_bounds__(256) k_nl_segments(const float2* __restrict__ xy, const float* __restrict__ sh,
                                                     const float* __restrict__ sa, int64_t n,
                                                     const uint32_t* __restrict__ keys,
                                                     const int32_t* __restrict__ cell_start,
                                                     const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                     float inv_support, float c_w, int32_t* __restrict__ counts,
                                                     float* __restrict__ rho, int32_t* __restrict__ nseg,
                                                     int32_t* __restrict__ seg_start, uint32_t* __restrict__ seg_mask,
                                                     int32_t* __restrict__ dense_list, int32_t* __restrict__ dense_count) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const sph_grid g = *gp;
  const uint32_t key = keys[s];
  int cnt = 0, k = 0;
  float acc = 0.f;
  if (grid_ok(g, cap) && key < (uint32_t)g.num_cells) {
    const float2 pi = xy[s];
    const float thr = grid_threshold(sh[s], g);
    const int cx = (int)(key % (uint32_t)g.cells_x), cy = (int)(key / (uint32_t)g.cells_x);
    const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
    const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
    for (int yy = y0; yy <= y1 && x0 <= x1; ++yy) {
      const int row = yy * g.cells_x;
      const int b = __ldg(cell_start + row + x0), e = __ldg(cell_start + row + x1 + 1);
      for (int c = b; c < e; c += 32) {
        uint32_t w = rho ? segment_mask_density(xy, sa, c, e, pi.x, pi.y, thr, inv_support, acc)
                         : segment_mask(xy, c, e, pi.x, pi.y, thr);
        if (w == 0) continue;
        if (k < kSearchSegments) {
          seg_start[(int64_t)k * n + s] = c;
          seg_mask[(int64_t)k * n + s] = w;
        }
        ++k;
        cnt += __popc(w);
      }
    }
  }
  counts[s] = cnt;
  if (rho) rho[s] = acc * c_w;
  nseg[s] = k <= kSearchSegments ? k : -1;
  if (k > kSearchSegments) dense_list[atomicAdd(dense_count, 1)] = (int32_t)s;
}

// The CSR columns from the stored segments (no pair tests).  Rows of the dense list are left
// to k_nl_fill_dense, which runs after this kernel (a staged block may copy placeholder
// entries over them first).
__global__ void __launch_bounds__(256) k_nl_fill_segments(const float2* __restrict__ xy,
                                                          const float* __restrict__ sh, int64_t n,
                                                          const uint32_t* __restrict__ keys,
                                                          const int32_t* __restrict__ cell_start,
                                                          const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                          const int32_t* __restrict__ offsets, int64_t pair_capacity,
                                                          int32_t* __restrict__ cols, int32_t* status,
                                                          const int32_t* __restrict__ nseg,
                                                          const int32_t* __restrict__ seg_start,
                                                          const uint32_t* __restrict__ seg_mask) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const sph_grid g = *gp;
  const uint32_t key = s < n ? keys[s] : 0xffffffffu;
  const bool active = s < n && grid_ok(g, cap) && key < (uint32_t)g.num_cells;
  const int ns = active ? nseg[s] : 0;
  const int64_t b0 = (int64_t)blockIdx.x * blockDim.x, b1 = min(b0 + (int64_t)blockDim.x, n);
  const int64_t span0 = offsets[b0], span1 = offsets[b1];
  if (span0 >= 0 && span1 - span0 > kFillStage && span1 <= pair_capacity) {   // the same in the whole block
    // Rows too long for one stage: each warp writes its 32 rows one after another, the lanes
    // taking one candidate bit each; lane k holds segment k of the row, and the exclusive
    // scan of the segments' bit counts places them, so a segment goes out as one contiguous
    // store of its accepted candidates.  The next row's segments are loaded while a row is
    // written.
    const int lane = threadIdx.x & 31;
    const uint32_t below = (1u << lane) - 1u;
    const int64_t r0 = active ? offsets[s] : 0, r1 = active ? offsets[s + 1] : 0;
    auto load_row = [&](int t, int& nst, int& c, uint32_t& m) {
      nst = __shfl_sync(0xffffffffu, ns, t);
      const int64_t st = __shfl_sync(0xffffffffu, s, t);
      c = 0;
      m = 0;
      if (nst > 0 && nst <= kSearchSegments && lane < nst) {
        c = seg_start[(int64_t)lane * n + st];
        m = seg_mask[(int64_t)lane * n + st];
      }
    };
    int nst_next, c_next;
    uint32_t m_next;
    load_row(0, nst_next, c_next, m_next);
    for (int t = 0; t < 32; ++t) {
      const int nst = nst_next, c = c_next;
      uint32_t m = m_next;
      if (t + 1 < 32) load_row(t + 1, nst_next, c_next, m_next);
      if (nst <= 0 || nst > kSearchSegments) continue;   // nothing, or a dense row
      const int64_t o = __shfl_sync(0xffffffffu, r0, t), e = __shfl_sync(0xffffffffu, r1, t);
      m = clip_segment(m, c, (int)n);
      const int cnt = __popc(m);
      int incl = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
      }
      const int excl = incl - cnt;
      for (int k = 0; k < nst; ++k) {
        const int ck = __shfl_sync(0xffffffffu, c, k);
        const uint32_t mk = __shfl_sync(0xffffffffu, m, k);
        const int bk = __shfl_sync(0xffffffffu, excl, k);
        if ((mk >> lane) & 1u) {
          const int64_t pos = o + bk + __popc(mk & below);
          if (pos < e) cols[pos] = ck + lane;
        }
      }
    }
    return;
  }
  staged_fill(s, n, active, offsets, pair_capacity, cols, status, [&](auto&& emit) {
    if (ns < 0 || ns > kSearchSegments) return;   // a dense row
    for (int k = 0; k < ns; ++k) {
      const int c = seg_start[(int64_t)k * n + s];
      uint32_t w = clip_segment(seg_mask[(int64_t)k * n + s], c, (int)n);
      while (w) {
        const int j = c - 1 + __ffs(w);
        w &= w - 1;
        emit(j);
      }
    }
  });
}

// The rows of the dense list, one warp per particle: each sweep tests 32 candidates of a
// cell row at once, and the accepted ones are written in order through a ballot, so the row
// goes out in coalesced stores.  A row that does not fit the column buffer is skipped with
// SPH_FLAG_PAIR_CAPACITY set.
__global__ void __launch_bounds__(128) k_nl_fill_dense(const float2* __restrict__ xy, const float* __restrict__ sh,
                                                       const uint32_t* __restrict__ keys,
                                                       const int32_t* __restrict__ cell_start,
                                                       const sph_grid* __restrict__ gp, int32_t cap, int r,
                                                       const int32_t* __restrict__ offsets, int64_t pair_capacity,
                                                       int32_t* __restrict__ cols, int32_t* status,
                                                       const int32_t* __restrict__ dense_list,
                                                       const int32_t* __restrict__ dense_count) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  const int nd = *dense_count;
  const sph_grid g = *gp;
  for (int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < nd; q += warps) {
    const int s = dense_list[q];
    int o = offsets[s];
    const int end = offsets[s + 1];
    if ((int64_t)end > pair_capacity || o < 0) {
      if (lane == 0) flag(status, SPH_FLAG_PAIR_CAPACITY);
      continue;
    }
    const uint32_t key = keys[s];
    const float2 pi = xy[s];
    const float thr = grid_threshold(sh[s], g);
    const int cx = (int)(key % (uint32_t)g.cells_x), cy = (int)(key / (uint32_t)g.cells_x);
    const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
    const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
    for (int yy = y0; yy <= y1 && x0 <= x1; ++yy) {
      const int row = yy * g.cells_x;
      const int b = __ldg(cell_start + row + x0), e = __ldg(cell_start + row + x1 + 1);
      for (int c = b; c < e; c += 32) {
        const int j = c + lane;
        bool hit = false;
        if (j < e) {
          const float2 pj = __ldg(xy + j);
          hit = dist2_ref(pi.x, pi.y, pj.x, pj.y) <= thr;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, hit);
        const int pos = o + __popc(m & ((1u << lane) - 1u));
        if (hit && pos < end) cols[pos] = j;
        o += __popc(m);
      }
    }
  }
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
                                                  const float2* __restrict__ xy,
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
  const float2 xi = qpos[b];
  const float thr = grid_threshold(qh[b], g);
  int qx, qy;
  if (grid_ok(g, cap) && query_cell(xi.x, g.qmin[0], g.hmax, &qx) && query_cell(xi.y, g.qmin[1], g.hmax, &qy)) {
    scan_candidates(xy, cell_start, g, r, qx, qy, xi.x, xi.y, thr, [&](int j, float) {
      if (kFill) {
        rows[o + cnt] = (int32_t)b;
        cols[o + cnt] = order ? (int32_t)order[j] : j;
      }
      ++cnt;
    });
  }
  if (!kFill) counts[b] = cnt;
}

// One thread per original particle i: its row of the (i, j)-ordered COO list, plus the
// reference's fluidDistances / fluidRadialDistances (src/modules/neighborSearch.py:218-223).
__global__ void k_nl_to_coo(const float2* __restrict__ xy, int64_t n, const uint32_t* __restrict__ order,
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
  const float2 pi = xy[s];
  for (int k = 0; k < e - b; ++k) {
    prow[o + k] = i;
    if (dist || radial) {
      float2 pj = xy[rank[pcol[o + k]]];
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

// ---------------------------------------------------------------------------- batch of scenes
// Keys are global: scene s's cells occupy [coff_s, coff_s + num_cells_s) of the cell table.
__global__ void __launch_bounds__(256) k_batch_nl_count(const float2* __restrict__ xy, const float* __restrict__ sh,
                                                        int64_t n, const uint32_t* __restrict__ keys,
                                                        const int32_t* __restrict__ cell_start,
                                                        const SceneDev* __restrict__ scenes,
                                                        const int32_t* __restrict__ sid, int32_t* __restrict__ counts) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const SceneDev& S = scenes[sid[s]];
  const uint32_t key = keys[s] - (uint32_t)S.coff;
  int cnt = 0;
  if (keys[s] >= (uint32_t)S.coff && key < (uint32_t)S.g.num_cells) {
    const float2 pi = xy[s];
    const float thr = grid_threshold(sh[s], S.g);
    const int cx = (int)(key % (uint32_t)S.g.cells_x), cy = (int)(key / (uint32_t)S.g.cells_x);
    scan_candidates(xy, cell_start + S.coff, S.g, S.P.search_radius, cx, cy, pi.x, pi.y, thr,
                    [&](int, float) { ++cnt; });
  }
  counts[s] = cnt;
}

__global__ void __launch_bounds__(256) k_batch_nl_fill(const float2* __restrict__ xy, const float* __restrict__ sh,
                                                       int64_t n, const uint32_t* __restrict__ keys,
                                                       const int32_t* __restrict__ cell_start,
                                                       const SceneDev* __restrict__ scenes,
                                                       const int32_t* __restrict__ sid,
                                                       const int32_t* __restrict__ offsets, int64_t pair_capacity,
                                                       int32_t* __restrict__ cols, int32_t* status) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const SceneDev* S = s < n ? scenes + sid[s] : scenes;
  const uint32_t key = s < n ? keys[s] - (uint32_t)S->coff : 0xffffffffu;
  const bool active = s < n && keys[s] >= (uint32_t)S->coff && key < (uint32_t)S->g.num_cells;
  float2 pi = make_float2(0.f, 0.f);
  float thr = 0.f;
  int cx = 0, cy = 0;
  if (active) {
    pi = xy[s];
    thr = grid_threshold(sh[s], S->g);
    cx = (int)(key % (uint32_t)S->g.cells_x);
    cy = (int)(key / (uint32_t)S->g.cells_x);
  }
  staged_fill(s, n, active, offsets, pair_capacity, cols, status, [&](auto&& emit) {
    scan_candidates(xy, cell_start + S->coff, S->g, S->P.search_radius, cx, cy, pi.x, pi.y, thr,
                    [&](int j, float) { emit(j); });
  });
}

}  // namespace sph

using namespace sph;

extern "C" {

sph_status_t sph_batch_nl_count(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                                const int32_t* cell_start, const void* scenes, const int32_t* sid, int32_t* counts,
                                void* stream) {
  SPH_REQUIRE(n >= 0 && xy && sorted_support && sorted_keys && cell_start && scenes && sid && counts,
              "batch_nl_count: bad arguments");
  if (n == 0) return SPH_OK;
  k_batch_nl_count<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(xy), sorted_support, n, sorted_keys, cell_start,
      static_cast<const SceneDev*>(scenes), sid, counts);
  SPH_CHECK_LAUNCH("batch_nl_count");
  return SPH_OK;
}

sph_status_t sph_batch_nl_fill(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                               const int32_t* cell_start, const void* scenes, const int32_t* sid, const int32_t* offsets,
                               int64_t pair_capacity, int32_t* cols, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && xy && sorted_support && sorted_keys && cell_start && scenes && sid && offsets && cols,
              "batch_nl_fill: bad arguments");
  if (n == 0) return SPH_OK;
  k_batch_nl_fill<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(xy), sorted_support, n, sorted_keys, cell_start,
      static_cast<const SceneDev*>(scenes), sid, offsets, pair_capacity, cols, status);
  SPH_CHECK_LAUNCH("batch_nl_fill");
  return SPH_OK;
}

sph_status_t sph_nl_count(const float* xy, const float* sorted_support, const float* sorted_area, int64_t n,
                          const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                          int32_t cell_capacity, int32_t search_radius, float kernel_support, int32_t* counts,
                          float* rho, void* stream) {
  SPH_REQUIRE(n >= 0 && xy && sorted_support && sorted_keys && cell_start && grid && counts && search_radius >= 0,
              "nl_count: bad arguments");
  SPH_REQUIRE(!rho || (kernel_support > 0.f && sorted_area), "nl_count: density needs kernel_support > 0 and areas");
  if (n == 0) return SPH_OK;
  float inv = rho ? 1.0f / kernel_support : 0.f;
  float cw = rho ? (float)(7.0 / 3.14159265358979323846) / (kernel_support * kernel_support) : 0.f;
  k_nl_count<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(xy), sorted_support,
                                                               sorted_area, n, sorted_keys, cell_start, grid,
                                                               cell_capacity, search_radius, inv, cw, counts, rho);
  SPH_CHECK_LAUNCH("nl_count");
  return SPH_OK;
}

size_t sph_nl_segments_scratch_bytes(int64_t n) {
  return (size_t)(n > 0 ? n : 0) * (kSearchSegments * (sizeof(int32_t) + sizeof(uint32_t)) + 2 * sizeof(int32_t)) +
         256 + 16;
}

// seg_mask [kSearchSegments n], seg_start [kSearchSegments n], nseg [n], the dense list [n] and its
// count inside the scratch.
static bool segments_from_scratch(void* scratch, size_t bytes, int64_t n, int32_t** nseg, int32_t** start,
                                  uint32_t** mask, int32_t** dense_list, int32_t** dense_count) {
  if (!scratch || bytes < sph_nl_segments_scratch_bytes(n)) return false;
  const uintptr_t p = (reinterpret_cast<uintptr_t>(scratch) + 15) & ~(uintptr_t)15;
  *mask = reinterpret_cast<uint32_t*>(p);
  *start = reinterpret_cast<int32_t*>(*mask + (size_t)kSearchSegments * n);
  *nseg = *start + (size_t)kSearchSegments * n;
  *dense_list = *nseg + n;
  *dense_count = *dense_list + n;
  return true;
}

sph_status_t sph_nl_count_segments(const float* xy, const float* sorted_support, const float* sorted_area, int64_t n,
                                   const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                                   int32_t cell_capacity, int32_t search_radius, float kernel_support,
                                   int32_t* counts, float* rho, void* seg_scratch, size_t seg_bytes, void* stream) {
  SPH_REQUIRE(n >= 0 && n < ((int64_t)1 << 31) && xy && sorted_support && sorted_keys && cell_start && grid &&
                  counts && search_radius >= 0,
              "nl_count_segments: bad arguments");
  SPH_REQUIRE(!rho || (kernel_support > 0.f && sorted_area),
              "nl_count_segments: density needs kernel_support > 0 and areas");
  int32_t *nseg, *start, *dense_list, *dense_count;
  uint32_t* mask;
  SPH_REQUIRE(segments_from_scratch(seg_scratch, seg_bytes, n, &nseg, &start, &mask, &dense_list, &dense_count),
              "nl_count_segments: scratch smaller than sph_nl_segments_scratch_bytes(n)");
  if (n == 0) return SPH_OK;
  cudaMemsetAsync(dense_count, 0, sizeof(int32_t), as_stream(stream));
  float inv = rho ? 1.0f / kernel_support : 0.f;
  float cw = rho ? (float)(7.0 / 3.14159265358979323846) / (kernel_support * kernel_support) : 0.f;
  k_nl_segments<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(xy), sorted_support, sorted_area, n, sorted_keys, cell_start, grid,
      cell_capacity, search_radius, inv, cw, counts, rho, nseg, start, mask, dense_list, dense_count);
  SPH_CHECK_LAUNCH("nl_count_segments");
  return SPH_OK;
}

sph_status_t sph_nl_fill_segments(const float* xy, const float* sorted_support, int64_t n,
                                  const uint32_t* sorted_keys, const int32_t* cell_start, const sph_grid* grid,
                                  int32_t cell_capacity, int32_t search_radius, const int32_t* offsets,
                                  int64_t pair_capacity, int32_t* cols, int32_t* status, const void* seg_scratch,
                                  size_t seg_bytes, void* stream) {
  SPH_REQUIRE(n >= 0 && n < ((int64_t)1 << 31) && xy && sorted_support && sorted_keys && cell_start && grid &&
                  offsets && cols,
              "nl_fill_segments: bad arguments");
  int32_t *nseg, *start, *dense_list, *dense_count;
  uint32_t* mask;
  SPH_REQUIRE(segments_from_scratch(const_cast<void*>(seg_scratch), seg_bytes, n, &nseg, &start, &mask,
                                    &dense_list, &dense_count),
              "nl_fill_segments: scratch smaller than sph_nl_segments_scratch_bytes(n)");
  if (n == 0) return SPH_OK;
  cudaStream_t st = as_stream(stream);
  k_nl_fill_segments<<<grid_for(n, 256), 256, 0, st>>>(reinterpret_cast<const float2*>(xy), sorted_support, n,
                                                       sorted_keys, cell_start, grid, cell_capacity, search_radius,
                                                       offsets, pair_capacity, cols, status, nseg, start, mask);
  k_nl_fill_dense<<<kNumSMs * 8, 128, 0, st>>>(reinterpret_cast<const float2*>(xy), sorted_support, sorted_keys,
                                               cell_start, grid, cell_capacity, search_radius, offsets, pair_capacity,
                                               cols, status, dense_list, dense_count);
  SPH_CHECK_LAUNCH("nl_fill_segments");
  return SPH_OK;
}

sph_status_t sph_nl_fill(const float* xy, const float* sorted_support, int64_t n, const uint32_t* sorted_keys,
                         const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity, int32_t search_radius,
                         const int32_t* offsets, int64_t pair_capacity, int32_t* cols, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && xy && sorted_support && sorted_keys && cell_start && grid && offsets && cols,
              "nl_fill: bad arguments");
  if (n == 0) return SPH_OK;
  k_nl_fill<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(xy), sorted_support, n,
                                                              sorted_keys, cell_start, grid, cell_capacity,
                                                              search_radius, offsets, pair_capacity, cols, status);
  SPH_CHECK_LAUNCH("nl_fill");
  return SPH_OK;
}

sph_status_t sph_nl_to_coo(const float* xy, int64_t n, const uint32_t* order, const uint32_t* rank,
                           const int32_t* offsets, const int32_t* cols, const int64_t* orig_offsets,
                           float grad_threshold, float kernel_support, int64_t* pairs, int64_t num_pairs, float* dist,
                           float* radial, void* stream) {
  SPH_REQUIRE(n >= 0 && xy && order && rank && offsets && cols && orig_offsets && pairs, "nl_to_coo: bad arguments");
  if (n == 0) return SPH_OK;
  k_nl_to_coo<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(reinterpret_cast<const float2*>(xy), n, order, rank,
                                                                offsets, cols, orig_offsets, grad_threshold,
                                                                kernel_support, pairs, num_pairs, dist, radial);
  SPH_CHECK_LAUNCH("nl_to_coo");
  return SPH_OK;
}

sph_status_t sph_nl_query_count(const float* query_pos, const float* query_support, int64_t m, const float* xy,
                                const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity,
                                int32_t search_radius, int32_t* counts, void* stream) {
  SPH_REQUIRE(m >= 0 && query_pos && query_support && xy && cell_start && grid && counts && search_radius >= 0,
              "nl_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_nl_query<false><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float2*>(xy), cell_start,
      grid, cell_capacity, search_radius, nullptr, counts, nullptr, nullptr, nullptr);
  SPH_CHECK_LAUNCH("nl_query_count");
  return SPH_OK;
}

sph_status_t sph_nl_query_fill(const float* query_pos, const float* query_support, int64_t m, const float* xy,
                               const int32_t* cell_start, const sph_grid* grid, int32_t cell_capacity,
                               int32_t search_radius, const uint32_t* order, const int64_t* offsets, int32_t* rows,
                               int32_t* cols, void* stream) {
  SPH_REQUIRE(m >= 0 && query_pos && query_support && xy && cell_start && grid && offsets && rows && cols &&
                  search_radius >= 0,
              "nl_query: bad arguments");
  if (m == 0) return SPH_OK;
  k_nl_query<true><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(query_pos), query_support, m, reinterpret_cast<const float2*>(xy), cell_start,
      grid, cell_capacity, search_radius, order, nullptr, offsets, rows, cols);
  SPH_CHECK_LAUNCH("nl_query_fill");
  return SPH_OK;
}

}  // extern "C"
