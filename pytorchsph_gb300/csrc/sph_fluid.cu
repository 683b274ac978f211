// deltaSPH right-hand side on sm_103a: one thread (or 2 / 4 lanes) per fluid particle in
// cell-sorted order, gathering over its pairs (a CSR row, or its segment list of accepted
// candidates from the cell rows) and over the wall particles of the neighboring cells.
// Every sum is a gather into registers — no atomics, deterministic order: fluid neighbors in
// cell order, then walls, added to the fluid sum the way the reference adds its wall
// module's result (`x += simulation.boundaryModule...`).
//
// Each kernel body takes its scene's grid, parameters and cell-table offset explicitly, so
// the same code serves one scene (sph_* entry points) and a batch of independent scenes
// concatenated in one particle array (sph_batch_* entry points, scene table + per-particle
// scene index).
//
// Reference formulas (relative density rho~, absolute rho = rho~ rho0, V = A / rho~):
//   continuity     src/modules/momentum.py:13-19 (+ wall solidBoundary.py:746-770)
//   MOG diffusion  src/modules/densityDiffusion.py:56-63
//   deltaSPH diff. src/modules/densityDiffusion.py:12-52 (+ wall L / grad parts,
//                  solidBoundary.py:676-717), pinv2x2 src/util.py:386-433
//   Tait EOS       src/modules/pressure.py:82-83 (wall: solidBoundary.py:802-804)
//   pressure acc.  src/modules/pressure.py:13-19 (+ wall solidBoundary.py:846-890)
//   art. viscosity src/modules/diffusion.py:12-25 (+ wall solidBoundary.py:820-844)
//   laminar visc.  src/modules/laminar.py:12-27 (index choices kept: r = x_j - x_i, mu_j = rho_i nu)
//   gravity        src/modules/gravity.py:46-57
//   mDBC density   src/modules/solidBoundary.py:561-617
#include <cstring>

#include "sph_math.cuh"

namespace sph {

// ---------------------------------------------------------------------------- mDBC
// Shepard and first-order MLS sums over the fluid particles within h of wall b's ghost
// (accumulated in double), the 3x3 pseudo-inverse solve, then wall density, volume and
// Tait pressure.
__device__ __forceinline__ void mdbc_body(int b, const FluidView& F, const WallView& W, const sph_grid& g,
                                          const SphParams& P, int coff) {
  const float2 xg = W.xg[b];
  const float thr = P.thr;
  // float sums (GB300's FP64 rate is low); the 3x3 solve below runs in double
  float nom = 0, den = 0, gx = 0, gy = 0, vgx = 0, vgy = 0, px = 0, py = 0;
  float m00 = 0, m01 = 0, m10 = 0, m11 = 0;
  int cnt = 0;
  const int32_t* cs = F.cell_start + coff;
  if (grid_ok(g, P.cell_capacity)) {
    float fcx = ceilf(__fdiv_rn(__fsub_rn(xg.x, g.qmin[0]), g.hmax));
    float fcy = ceilf(__fdiv_rn(__fsub_rn(xg.y, g.qmin[1]), g.hmax));
    if (fcx > -1e9f && fcx < 1e9f && fcy > -1e9f && fcy < 1e9f) {
      const int cx = (int)fcx, cy = (int)fcy, r = P.search_radius;
      const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
      const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
      if (x0 <= x1) {
        for (int yy = y0; yy <= y1; ++yy) {
          const int row = yy * g.cells_x;
          const int j0 = cs[row + x0], j1 = cs[row + x1 + 1];
          for (int j = j0; j < j1; ++j) {
            const float2 xj = F.x[j];
            if (!(dist2_ref(xg.x, xg.y, xj.x, xj.y) <= thr)) continue;
            // e = (x_g - x_j) / r from one rsqrt (zero below r = 1e-7, as the reference's e_ij)
            const float dx = xg.x - xj.x, dy = xg.y - xj.y;
            const float r2 = dx * dx + dy * dy;
            const float ir = r2 >= 1e-14f ? rsqrt_normal(r2) : 0.f;
            const float q = r2 * ir * P.inv_h;
            const float k = kW(q, P.c_w);
            const float gwr = kGW(q, P.c_g) * ir;
            const float ggx = gwr * dx, ggy = gwr * dy;
            const float Aj = F.area[j];
            const float mass = Aj * P.rho0;
            const float Vj = Aj * rcp_normal(F.rho[j]);
            const float xx = xj.x - xg.x, xy = xj.y - xg.y;
            nom += mass * k;
            den += Vj * k;
            gx += mass * ggx;
            gy += mass * ggy;
            vgx += Vj * ggx;
            vgy += Vj * ggy;
            px += Vj * k * xx;
            py += Vj * k * xy;
            m00 += Vj * xx * ggx;
            m01 += Vj * xx * ggy;
            m10 += Vj * xy * ggx;
            m11 += Vj * xy * ggy;
            ++cnt;
          }
        }
      }
    }
  }
  double rho_b = 1.0;
  if (cnt > 0) rho_b = ((double)nom / (double)den) / P.rho0;
  if (cnt > 10) {
    const double A[3][3] = {{den, px, py}, {vgx, m00, m01}, {vgy, m10, m11}};
    const double bb[3] = {nom, gx, gy};
    double res[3];
    pinv3_solve(A, bb, res);
    const float2 xb = W.x[b];
    rho_b = (res[0] + ((double)xb.x - xg.x) * res[1] + ((double)xb.y - xg.y) * res[2]) / P.rho0;
  }
  float rb = (float)fmax(rho_b, 1.0);
  W.rho[b] = rb;
  W.vol[b] = W.area[b] / rb;
  W.p[b] = tait(rb, P);
}

// ---------------------------------------------------------------------------- neighbor records
// What neighbor j brings to every pair term, computed once per particle instead of once
// per pair: xv = (x, y, vx, vy) and q = (rho_j, V_j = A_j / rho~_j, p_j V_j with p_j =
// Tait(rho~_j), m_j = rho_j V_j).  Two 16-byte loads per pair replace four scalar loads, a
// division and the Tait power.
// Both float4 of a particle sit in one 32-byte record, so a pair's two loads share one
// 32-byte sector and one address.
struct __align__(32) Rec {
  float4 xv, q;
};

__device__ __forceinline__ void prep_body(int i, const FluidView& F, const SphParams& P, Rec* __restrict__ rec) {
  const float2 x = F.x[i], v = F.v[i];
  const float rt = F.rho[i];
  const float V = F.area[i] / rt, rho = rt * P.rho0;
  rec[i].xv = make_float4(x.x, x.y, v.x, v.y);
  rec[i].q = make_float4(rho, V, tait(rt, P) * V, rho * V);
}

// Pair geometry in the form the sums need: d = x_i - x_j, r2 = |d|^2 and the Wendland
// gradient as gradW_ij = gd * d, gd = kGW(q) / r = -20 c_g (1 - q)^3 / h (zero when
// r < 1e-7, where the reference's e_ij is zero).  Every dot product with gradW then folds
// into gd: (x_j - x_i) . gradW = -gd r2, u . gradW = gd (u . d).
struct PairG {
  float dx, dy, r2, gd;
};

// kScaled = false: gd without its constant factor gk (a sum that is linear in gd takes gk
// once at the end).
template <bool kScaled = true>
__device__ __forceinline__ PairG pair_g(float xi, float yi, float xj, float yj, const SphParams& P) {
  PairG g;
  g.dx = xi - xj;
  g.dy = yi - yj;
  g.r2 = g.dx * g.dx + g.dy * g.dy;
  const bool apart = g.r2 >= 1e-14f;
  const float r = g.r2 * rsqrt_normal(g.r2);   // NaN at r2 = 0, dropped by the select
  const float a = apart ? 1.0f - r * P.inv_h : 0.f;
  g.gd = kScaled ? P.gk * (a * a * a) : a * a * a;
  return g;
}

// ---------------------------------------------------------------------------- cell-row pairs
// The pairs of particle i straight from the cell table, without a CSR list: its candidates
// are the contiguous sorted ranges of its 2r+1 cell rows (cells cx-r..cx+r of each row).
// A range is tested in segments of 32 candidates into a bit mask, and the accepted
// candidates are visited in increasing index: the CSR fill's order, so every sum is the
// same.  Visiting set bits keeps a warp's lanes together the way a CSR row does (a lane
// runs the pair body only for its own neighbors).
//
// The records pass stores each particle's non-empty segments in order, at most
// kMaxSegments: start seg_start[k * n + i] and mask seg_mask[k * n + i] for k < nseg[i]
// (nseg[i] = -1 when there are more; the force passes then test its cell rows
// themselves).  A force pass holds one segment and the next one, loaded ahead, so moving
// on to the next segment costs a lane a register move.
// Every row of the window, tested here (any r); with kTpp lanes per particle, lane `sub`
// takes rows y0 + sub, y0 + sub + kTpp, ...
// kPaired: the candidate tests two at a time (segment_mask) or one at a time; the sums are
// the same either way (which one a pass uses is a measured code-generation choice).
template <int kTpp = 1, bool kPaired = false, typename Fn>
__device__ __forceinline__ void cell_pairs(const FluidView& F, const sph_grid& g, int r, int coff, int cx, int cy,
                                           float xi, float yi, float thr, Fn&& fn, int sub = 0) {
  const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
  if (x0 > x1) return;
  const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
  const int32_t* cs = F.cell_start + coff;
  for (int yy = y0 + sub; yy <= y1; yy += kTpp) {
    const int row = yy * g.cells_x;
    const int b = __ldg(cs + row + x0), e = __ldg(cs + row + x1 + 1);
    for (int c = b; c < e; c += 32) {
      uint32_t w = kPaired ? segment_mask(F.x, c, e, xi, yi, thr) : segment_mask_scalar(F.x, c, e, xi, yi, thr);
      while (w) {
        const int j = c - 1 + __ffs(w);
        w &= w - 1;
        fn(j);
      }
    }
  }
}

// The segment list of particle i.
__device__ __forceinline__ void segments_body(int i, const FluidView& F, const sph_grid& g, int coff, int r,
                                              float thr, int32_t* __restrict__ nseg, int32_t* __restrict__ seg_start,
                                              uint32_t* __restrict__ seg_mask) {
  int cx, cy;
  cell_of(F.keys[i] - (uint32_t)coff, g, &cx, &cy);
  const float2 xi = F.x[i];
  const size_t n = (size_t)F.n;
  int k = 0;
  const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
  const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
  const int32_t* cs = F.cell_start + coff;
  if (x0 <= x1) {
    for (int yy = y0; yy <= y1; ++yy) {
      const int row = yy * g.cells_x;
      const int b = __ldg(cs + row + x0), e = __ldg(cs + row + x1 + 1);
      for (int c = b; c < e; c += 32) {
        const uint32_t w = c + 32 <= F.n ? segment_mask_full(F.x, c, e, xi.x, xi.y, thr)
                                         : segment_mask(F.x, c, e, xi.x, xi.y, thr);
        if (w == 0) continue;
        if (k < kMaxSegments) {
          seg_start[k * n + i] = c;
          seg_mask[k * n + i] = w;
        }
        ++k;
      }
    }
  }
  nseg[i] = k <= kMaxSegments ? k : -1;
}

// The pairs of particle i from its segment list (its cell rows when the list overflowed).
// With kTpp lanes per particle, lane `sub` takes segments sub, sub + kTpp, ... (rows, on the
// overflow path); each lane holds its current segment and its next one, loaded ahead.
template <int kTpp = 1, bool kPaired = false, typename Fn>
__device__ __forceinline__ void stored_pairs(int i, const FluidView& F, const sph_grid& g, int coff, int r,
                                             const int32_t* __restrict__ nseg, const int32_t* __restrict__ seg_start,
                                             const uint32_t* __restrict__ seg_mask, float xi, float yi, float thr,
                                             Fn&& fn, int sub = 0) {
  const int ns = nseg[i];
  if (ns < 0 || ns > kMaxSegments) {
    int cx, cy;
    cell_of(F.keys[i] - (uint32_t)coff, g, &cx, &cy);
    cell_pairs<kTpp, kPaired>(F, g, r, coff, cx, cy, xi, yi, thr, fn, sub);
    return;
  }
  if (ns <= sub) return;
  const size_t n = (size_t)F.n;
  int k = sub;
  int b = seg_start[k * n + i];
  uint32_t w = clip_segment(seg_mask[k * n + i], b, F.n);
  int bn = 0;
  uint32_t wn = 0;
  if (k + kTpp < ns) {
    bn = seg_start[(k + kTpp) * n + i];
    wn = seg_mask[(k + kTpp) * n + i];
  }
  for (;;) {
    while (w == 0) {
      k += kTpp;
      if (k >= ns) return;
      b = bn;
      w = clip_segment(wn, bn, F.n);
      if (k + kTpp < ns) {
        bn = seg_start[(k + kTpp) * n + i];
        wn = seg_mask[(k + kTpp) * n + i];
      }
    }
    const int j = b - 1 + __ffs(w);
    w &= w - 1;
    fn(j);
  }
}

// Sum of v over the kTpp consecutive lanes of one particle (every lane gets the sum; the
// whole warp must take part).
template <int kTpp>
__device__ __forceinline__ float lane_sum(float v) {
#pragma unroll
  for (int o = 1; o < kTpp; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------- pass 1
// dpdt (continuity + MOG), acceleration (gravity, pressure, artificial and laminar
// viscosity) and, for the deltaSPH scheme, the renormalization matrix L_i and the density
// gradient <grad rho>_i = -L_i^+ sum_j 2 (rho_j - rho_i) V_j gradW_ij (+ walls), all in one
// sweep over the row: L_i^+ is applied to the summed vector once instead of to every term.
// For the deltaSPH scheme the diffusion D_i = sum_j psi_ij . gradW_ij V_j, psi_ij =
// 2 (rho_j - rho_i) x_ji / (|x_ji|^2 + eps) - (<grad rho>_i + <grad rho>_j), is split: pass 1
// sums the parts it can, ddiff = 2 sum_j (rho_j - rho_i) (x_ji . gradW) V_j / (|x_ji|^2 + eps)
// - <grad rho>_i . sum_j V_j gradW_ij, and the diffusion pass subtracts
// sum_j (<grad rho>_j V_j) . gradW_ij, the only part that needs the neighbors' gradients.
struct Pass1 {
  float dpdt, ax, ay;
  float4 L;        // renormalization matrix, fluid + walls
  float2 grad_rho;
  float ddiff;     // deltaSPH: the pass-1 part of D_i
};

// Pairs from the segment lists S (kCells) instead of the CSR row.
struct Segments {
  const int32_t* nseg;
  const int32_t* start;
  const uint32_t* mask;
};

// kTpp lanes per particle (kCells only): lane `sub` sums its share of the pairs, the lanes
// add their sums, and lane 0 finishes (walls, gravity, L^+); the other lanes return a zero
// record.  `live` false: a lane past the last particle, which only takes part in the sums.
// kScheme: the density diffusion (0 none, 1 MOG, 2 deltaSPH) fixed at compile time, or -1:
// read from P.diffusion.
template <bool kCells, int kTpp = 1, int kScheme = -1>
__device__ __forceinline__ Pass1 pass1_body(int i, const FluidView& F, const Rec* __restrict__ rec,
                                            const WallView& W, const sph_grid& g,
                                            const SphParams& P, int coff, const Segments& S, int sub = 0,
                                            bool live = true) {
  const float4 si = rec[i].xv;
  const float rhoi = rec[i].q.x, pi = tait(F.rho[i], P);
  const int scheme = kScheme >= 0 ? kScheme : P.diffusion;
  const bool renorm = scheme == 2;
  const float mu8 = 4.0f * (2.0f * rhoi * P.kinematic);   // 4 (mu_i + mu_j), both rho_i nu
  float dp_f = 0.f, mog = 0.f, bx = 0.f, by = 0.f;   // b = sum_j V_j gradW_ij (deltaSPH)
  float pax = 0.f, pay = 0.f, vax = 0.f, vay = 0.f, lax = 0.f, lay = 0.f;
  float l00 = 0.f, l01 = 0.f, l11 = 0.f, gfx = 0.f, gfy = 0.f;
  auto fluid_pair = [&](int j) {
    const float4 sj = __ldg(&rec[j].xv), qj = __ldg(&rec[j].q);
    const float rhoj = qj.x, Vj = qj.y, pVj = qj.z, mj = qj.w;
    const PairG e = pair_g(si.x, si.y, sj.x, sj.y, P);   // gradW = e.gd * d
    const float ux = sj.z - si.z, uy = sj.w - si.w;       // u_j - u_i
    const float ud = ux * e.dx + uy * e.dy;               // (u_j - u_i) . d
    const float ir2 = rcp_normal(e.r2 + P.eps);
    const float rg = -e.gd * e.r2;                        // (x_j - x_i) . gradW
    const float mg = mj * e.gd;
    dp_f -= mg * ud;
    // MOG diffusion (for deltaSPH the first part of its diffusion, formed below from the
    // renormalization product): (rho_j - rho_i) V_j (x_j - x_i) . gradW / (r^2 + eps), x 2 after the sum
    if (scheme == 1) mog += (rhoj - rhoi) * ir2 * rg * Vj;
    const float pf = fmaf(pi, Vj, pVj) * e.gd;            // (p_i + p_j) V_j gd
    pax += pf * e.dx;
    pay += pf * e.dy;
    const float irs = rcp_normal(rhoi + rhoj);
    const float wg = mg * (irs * ir2);
    const float vf = fminf(-ud, 0.f) * wg;                // pi_ij, (u_j - u_i) . (x_j - x_i) = -ud
    vax += vf * e.dx;
    vay += vf * e.dy;
    const float term = e.r2 * irs * wg;                   // laminar: mu8 term (u_j - u_i), mu8 after the sum
    lax += term * ux;
    lay += term * uy;
    if (renorm) {
      // V_j (x_j - x_i) (x) gradW = -t d (x) d: symmetric, one off-diagonal sum
      const float t = Vj * e.gd;
      const float tx = t * e.dx, ty = t * e.dy;
      l00 -= tx * e.dx;
      l01 -= tx * e.dy;
      l11 -= ty * e.dy;
      bx += tx;
      by += ty;
      const float s = (rhoj - rhoi) * t;                  // x 2 after the sum
      gfx += s * e.dx;
      gfy += s * e.dy;
      mog -= s * (e.r2 * ir2);                            // (rho_j - rho_i) V_j (-gd r^2) / (r^2 + eps)
    }
  };
  if constexpr (kCells) {
    if (live) stored_pairs<kTpp>(i, F, g, coff, P.search_radius, S.nseg, S.start, S.mask, si.x, si.y, P.thr,
                                 fluid_pair, sub);
  } else {
    static_assert(kTpp == 1, "CSR rows run one lane per particle");
    const int k0 = F.offsets[i], k1 = row_end(F, i, k0);
    for (int k = k0; k < k1; ++k) fluid_pair(__ldg(F.cols + k));
  }
  if constexpr (kTpp > 1) {
    dp_f = lane_sum<kTpp>(dp_f);
    mog = lane_sum<kTpp>(mog);
    pax = lane_sum<kTpp>(pax);
    pay = lane_sum<kTpp>(pay);
    vax = lane_sum<kTpp>(vax);
    vay = lane_sum<kTpp>(vay);
    lax = lane_sum<kTpp>(lax);
    lay = lane_sum<kTpp>(lay);
    l00 = lane_sum<kTpp>(l00);
    l01 = lane_sum<kTpp>(l01);
    l11 = lane_sum<kTpp>(l11);
    gfx = lane_sum<kTpp>(gfx);
    gfy = lane_sum<kTpp>(gfy);
    bx = lane_sum<kTpp>(bx);
    by = lane_sum<kTpp>(by);
    if (sub != 0 || !live) return Pass1{};
  }
  float dp_w = 0.f, pwx = 0.f, pwy = 0.f, vwx = 0.f, vwy = 0.f;
  float w00 = 0.f, w01 = 0.f, w10 = 0.f, w11 = 0.f, gwx = 0.f, gwy = 0.f;
  if (W.n > 0) {
    int cx, cy;
    cell_of(F.keys[i] - (uint32_t)coff, g, &cx, &cy);
    const float thr = P.thr;
    for_each_wall(
        W, g, P.search_radius, cx, cy, si.x, si.y, thr,
        [&](int b, float2 xb) {
          const PairG e = pair_g(si.x, si.y, xb.x, xb.y, P);   // fluid side: d = x_f - x_b
          const float Vb = W.vol[b], rhob = W.rho[b] * P.rho0, pb = W.p[b];
          const float ud = -(si.z * e.dx + si.w * e.dy);       // (u_b - u_f) . d, walls at rest
          dp_w -= e.gd * ud * Vb * rhob;
          const float pf = (pi + pb) * Vb * e.gd;
          pwx += pf * e.dx;
          pwy += pf * e.dy;
          if (P.boundary_diffusion) {
            const float vf = fminf(-ud, 0.f) * rcp_normal(e.r2 + P.eps) * Vb * rhob *
                             rcp_normal(rhoi + rhob) * e.gd;
            vwx += vf * e.dx;
            vwy += vf * e.dy;
          }
          if (renorm) {
            const float t = Vb * e.gd;
            const float tx = t * e.dx, ty = t * e.dy;
            w00 -= tx * e.dx;
            w01 -= tx * e.dy;
            w10 -= ty * e.dx;
            w11 -= ty * e.dy;
            const float s = (rhob - rhoi) * 2.0f * t;
            gwx += s * e.dx;
            gwy += s * e.dy;
          }
        },
        coff);
  }
  Pass1 o;
  o.dpdt = dp_f + dp_w;
  if (scheme == 1) o.dpdt += P.diff_k * (2.0f * mog);
  float ax, ay;
  if (P.point_source) {
    float dx = si.x - P.point_cx, dy = si.y - P.point_cy;
    float dist = sqrtf(dx * dx + dy * dy);
    if (dist > 1e-7f) {
      dx /= dist;
      dy /= dist;
    }
    ax = -P.point_mag * dx * dist;
    ay = -P.point_mag * dy * dist;
  } else {
    ax = P.gx;
    ay = P.gy;
  }
  const float ir = -1.0f / rhoi;
  ax += ir * pax + ir * pwx;
  ay += ir * pay + ir * pwy;
  ax += P.visc_k * vax + P.visc_k * vwx;
  ay += P.visc_k * vay + P.visc_k * vwy;
  o.ax = ax - mu8 * lax;
  o.ay = ay - mu8 * lay;
  o.L = make_float4(l00 + w00, l01 + w01, l01 + w10, l11 + w11);
  gfx *= 2.0f;
  gfy *= 2.0f;
  o.grad_rho = make_float2(0.f, 0.f);
  o.ddiff = 0.f;
  if (renorm) {
    const float4 Li = pinv2x2_fast(o.L.x, o.L.y, o.L.z, o.L.w);
    const float fx = Li.x * gfx + Li.y * gfy, fy = Li.z * gfx + Li.w * gfy;
    const float wx = Li.x * gwx + Li.y * gwy, wy = Li.z * gwx + Li.w * gwy;
    o.grad_rho = make_float2(-fx - wx, -fy - wy);
    o.ddiff = 2.0f * mog - (o.grad_rho.x * bx + o.grad_rho.y * by);
  }
  return o;
}

// D_i = sum_j [2 (rho_j - rho_i)/(|x_ji|^2 + eps) x_ji - (<grad rho>_i + <grad rho>_j)] . gradW_ij V_j
// (the deltaSPH density diffusion before its h delta c0 factor).
// sum_j (<grad rho>_j V_j) . gradW_ij, the part of the deltaSPH diffusion that needs the
// neighbors' gradients.  kHoldsGV: gbuf holds <grad rho> V (the batch's pass 1 stores it
// so); otherwise it holds <grad rho> and V_j comes from the neighbor record (the same
// product, so both give the same bits).  kCells: pairs from the segment lists instead of the
// CSR row.
template <bool kCells, int kTpp = 1, bool kHoldsGV = true>
__device__ __forceinline__ float diffusion_sum(int i, const FluidView& F, const Rec* __restrict__ rec,
                                               const SphParams& P, const float2* __restrict__ gbuf,
                                               const sph_grid& g, int coff, const Segments& S, int sub = 0,
                                               bool live = true) {
  const float2 xi = F.x[i];
  float acc = 0.f;
  auto pair = [&](int j) {
    const float2 xj = __ldg(F.x + j);
    float2 gv = __ldg(gbuf + j);
    if constexpr (!kHoldsGV) {
      const float Vj = __ldg(&rec[j].q.y);
      gv = make_float2(gv.x * Vj, gv.y * Vj);
    }
    const PairG e = pair_g<false>(xi.x, xi.y, xj.x, xj.y, P);   // gk after the sum
    acc += (gv.x * e.dx + gv.y * e.dy) * e.gd;
  };
  if constexpr (kCells) {
    if (live) stored_pairs<kTpp, true>(i, F, g, coff, P.search_radius, S.nseg, S.start, S.mask, xi.x, xi.y, P.thr,
                                       pair, sub);
  } else {
    static_assert(kTpp == 1, "CSR rows run one lane per particle");
    const int k0 = F.offsets[i], k1 = row_end(F, i, k0);
    for (int k = k0; k < k1; ++k) pair(__ldg(F.cols + k));
  }
  return lane_sum<kTpp>(acc) * P.gk;
}

// semiImplicitEuler, src/simulationBase.py:647-652 with integrateValues :564-569, for one
// particle with its own values.
__device__ __forceinline__ void sie_apply(int i, float2 xi, float2 vi, float rti, float2 ai, float dpi, float dt,
                                          float rho0, int continuum, float2* __restrict__ xo,
                                          float2* __restrict__ vo, float* __restrict__ ro, int32_t* status) {
  const float2 vn = make_float2(vi.x + dt * ai.x, vi.y + dt * ai.y);
  const float2 xn = make_float2(xi.x + dt * (vi.x + dt * ai.x), xi.y + dt * (vi.y + dt * ai.y));
  xo[i] = xn;
  vo[i] = vn;
  const float rn = continuum ? rti + dt * dpi / rho0 : rti;
  ro[i] = rn;
  if (!isfinite(xn.x) || !isfinite(xn.y) || !isfinite(vn.x) || !isfinite(vn.y) || !isfinite(rn))
    flag(status, SPH_FLAG_NONFINITE);
}

// ---------------------------------------------------------------------------- one scene
__global__ void __launch_bounds__(128) k_mdbc(FluidView F, WallView W, const sph_grid* __restrict__ gp, SphParams P) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W.n) return;
  mdbc_body(b, F, W, *gp, P, 0);
}

__global__ void __launch_bounds__(256) k_prep(FluidView F, SphParams P, Rec* __restrict__ rec) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  prep_body(i, F, P, rec);
}

__global__ void __launch_bounds__(128) k_dsph_pass1(FluidView F, const Rec* __restrict__ rec, WallView W,
                                                    const sph_grid* __restrict__ gp, SphParams P,
                                                    float* __restrict__ dpdt, float2* __restrict__ acc,
                                                    float4* __restrict__ Lout, float2* __restrict__ grad_rho) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const Pass1 o = pass1_body<false>(i, F, rec, W, *gp, P, 0, Segments{});
  dpdt[i] = P.diffusion == 2 ? o.dpdt + P.diff_k * o.ddiff : o.dpdt;
  acc[i] = make_float2(o.ax, o.ay);
  if (Lout) Lout[i] = o.L;
  if (grad_rho) grad_rho[i] = o.grad_rho;
}

__global__ void __launch_bounds__(128) k_dsph_diffusion(FluidView F, const Rec* __restrict__ rec, SphParams P,
                                                        const float2* __restrict__ grad_rho, float* __restrict__ dpdt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  dpdt[i] -= P.diff_k * diffusion_sum<false, 1, false>(i, F, rec, P, grad_rho, sph_grid{}, 0, Segments{});
}

__global__ void k_sie(int n, const float2* __restrict__ x, const float2* __restrict__ v,
                      const float* __restrict__ rho, const float2* __restrict__ a, const float* __restrict__ dpdt,
                      const float* __restrict__ dt_ptr, float rho0, int continuum, float2* __restrict__ xo,
                      float2* __restrict__ vo, float* __restrict__ ro, int32_t* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  sie_apply(i, x[i], v[i], rho[i], a[i], continuum ? dpdt[i] : 0.f, *dt_ptr, rho0, continuum, xo, vo, ro, status);
}

// ---------------------------------------------------------------------------- batch of scenes
// scenes[sid[i]] gives particle i's grid, parameters, cell-table offset and time step.
__global__ void __launch_bounds__(128, 8) k_batch_mdbc(FluidView F, WallView W, const SceneDev* __restrict__ scenes,
                                                    const int32_t* __restrict__ wsid) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W.n || wsid[b] < 0) return;   // wall of no scene (free slot of a pooled batch)
  const SceneDev& S = scenes[wsid[b]];
  mdbc_body(b, F, W, S.g, S.P, S.coff);
}

// Neighbor records and, with pairs from the cell rows (nseg != NULL), the segment lists.
__global__ void __launch_bounds__(256) k_batch_prep(FluidView F, const SceneDev* __restrict__ scenes,
                                                    const int32_t* __restrict__ sid, Rec* __restrict__ rec,
                                                    int32_t* __restrict__ nseg,
                                                    int32_t* __restrict__ seg_start, uint32_t* __restrict__ seg_mask) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n || sid[i] < 0) return;   // particle of no scene: never anyone's neighbor
  const SceneDev& S = scenes[sid[i]];
  prep_body(i, F, S.P, rec);
  if (nseg) segments_body(i, F, S.g, S.coff, S.P.search_radius, S.P.thr, nseg, seg_start, seg_mask);
}

// The update of one particle of a batch with its scene's dt.  If the neighbor list
// overflowed (the fill set SPH_FLAG_PAIR_CAPACITY) the step is not applied: the sorted
// inputs are copied unchanged.
__device__ __forceinline__ void batch_update(int i, const FluidView& F, float ax, float ay, float dpdt,
                                             const SceneDev& S, float2* __restrict__ xo, float2* __restrict__ vo,
                                             float* __restrict__ ro, int32_t* status) {
  if (*status & SPH_FLAG_PAIR_CAPACITY) {
    xo[i] = F.x[i];
    vo[i] = F.v[i];
    ro[i] = F.rho[i];
    return;
  }
  sie_apply(i, F.x[i], F.v[i], F.rho[i], make_float2(ax, ay), dpdt, S.dt, S.P.rho0, 1, xo, vo, ro, status);
}

// Pass 1 of the particles [p_lo, p_hi).  Particles of scenes without the deltaSPH density
// diffusion are complete after it and are updated here; the others hand dpdt, acc and
// <grad rho> to k_batch_diffusion, which finishes and updates them.  kCells: pairs from the
// segment lists; kTpp lanes per particle (kCells only).  With kTpp > 1 no lane leaves
// before the lane sums: lanes past p_hi take part with nothing to add.
template <bool kCells, int kTpp, int kScheme>
__global__ void __launch_bounds__(128, 9) k_batch_pass1(FluidView F, const Rec* __restrict__ rec, WallView W,
                                                     const SceneDev* __restrict__ scenes,
                                                     const int32_t* __restrict__ sid, float* __restrict__ dpdt,
                                                     float2* __restrict__ acc, float2* __restrict__ grad_rho,
                                                     const Segments seg, float2* __restrict__ xo,
                                                     float2* __restrict__ vo, float* __restrict__ ro,
                                                     int32_t* status, int p_lo, int p_hi) {
  int i, sub = 0;
  bool live = true;
  if constexpr (kTpp == 1) {
    i = p_lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= p_hi || sid[i] < 0) return;
  } else {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ii = p_lo + g / kTpp;
    sub = (int)(g % kTpp);
    live = ii < p_hi;
    i = live ? (int)ii : p_lo;
    live = live && sid[i] >= 0;   // a particle of no scene takes part in the lane sums only
  }
  const SceneDev& S = scenes[sid[i] < 0 ? 0 : sid[i]];
  const SphParams P = S.P;   // the fields the loop reads, in registers
  const Pass1 o = pass1_body<kCells, kTpp, kScheme>(i, F, rec, W, S.g, P, S.coff, seg, sub, kTpp == 1 || live);
  if (kTpp > 1 && (!live || sub != 0)) return;
  if ((kScheme >= 0 ? kScheme : P.diffusion) == 2) {
    dpdt[i] = o.dpdt + P.diff_k * o.ddiff;
    acc[i] = make_float2(o.ax, o.ay);
    const float Vi = rec[i].q.y;
    grad_rho[i] = make_float2(o.grad_rho.x * Vi, o.grad_rho.y * Vi);   // <grad rho> V for the diffusion pass
    return;
  }
  batch_update(i, F, o.ax, o.ay, o.dpdt, S, xo, vo, ro, status);
}

template <bool kCells, int kTpp>
__global__ void __launch_bounds__(128) k_batch_diffusion(FluidView F, const Rec* __restrict__ rec,
                                                         const SceneDev* __restrict__ scenes,
                                                         const int32_t* __restrict__ sid,
                                                         const float2* __restrict__ grad_rho, const Segments seg,
                                                         const float* __restrict__ dpdt,
                                                         const float2* __restrict__ acc, float2* __restrict__ xo,
                                                         float2* __restrict__ vo, float* __restrict__ ro,
                                                         int32_t* status, int p_lo, int p_hi) {
  int i, sub = 0;
  bool live = true;
  if constexpr (kTpp == 1) {
    i = p_lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= p_hi || sid[i] < 0) return;
  } else {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ii = p_lo + g / kTpp;
    sub = (int)(g % kTpp);
    live = ii < p_hi;
    i = live ? (int)ii : p_lo;
    live = live && sid[i] >= 0;
  }
  const SceneDev& S = scenes[sid[i] < 0 ? 0 : sid[i]];
  const bool act = live && S.P.diffusion == 2;   // the same on all lanes of a particle
  if (kTpp == 1 && !act) return;
  const SphParams P = S.P;   // the fields the loop reads, in registers
  const float sum = diffusion_sum<kCells, kTpp>(i, F, rec, P, grad_rho, S.g, S.coff, seg, sub, kTpp == 1 || act);
  if (kTpp > 1 && (!act || sub != 0)) return;
  const float d = dpdt[i] - P.diff_k * sum;
  const float2 a = acc[i];
  batch_update(i, F, a.x, a.y, d, S, xo, vo, ro, status);
}

// ---------------------------------------------------------------------------- RK4 helpers
// RK4 stage / combination, src/simulationBase.py:679-705: out = base + c * (k_u, k_a, k_d / rho0).
__global__ void k_rk_axpy(int n, const float2* __restrict__ x0, const float2* __restrict__ v0,
                          const float* __restrict__ r0, const float2* __restrict__ ku, const float2* __restrict__ ka,
                          const float* __restrict__ kd, const float* __restrict__ dt_ptr, float c, float rho0,
                          float2* __restrict__ xo, float2* __restrict__ vo, float* __restrict__ ro, int32_t* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float h = c * *dt_ptr;
  const float2 u = ku[i], a = ka[i], x = x0[i], v = v0[i];
  const float2 xn = make_float2(x.x + h * u.x, x.y + h * u.y);
  const float2 vn = make_float2(v.x + h * a.x, v.y + h * a.y);
  const float rn = r0[i] + h * kd[i] / rho0;
  xo[i] = xn;
  vo[i] = vn;
  ro[i] = rn;
  if (!isfinite(xn.x) || !isfinite(xn.y) || !isfinite(vn.x) || !isfinite(vn.y) || !isfinite(rn))
    flag(status, SPH_FLAG_NONFINITE);
}

// s (+)= w * k for the RK4 sums; init = 1 overwrites.
__global__ void k_rk_accum(int n, const float2* __restrict__ ku, const float2* __restrict__ ka,
                           const float* __restrict__ kd, float w, int init, float2* __restrict__ su,
                           float2* __restrict__ sa, float* __restrict__ sd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 u = ku[i], a = ka[i];
  float d = kd[i];
  if (init) {
    su[i] = make_float2(w * u.x, w * u.y);
    sa[i] = make_float2(w * a.x, w * a.y);
    sd[i] = w * d;
  } else {
    float2 s = su[i], t = sa[i];
    su[i] = make_float2(s.x + w * u.x, s.y + w * u.y);
    sa[i] = make_float2(t.x + w * a.x, t.y + w * a.y);
    sd[i] += w * d;
  }
}

// Permute per-particle arrays into a new order: out[s] = in[order[s]] (4-, 8- and 16-byte elements).
template <typename T>
__global__ void k_permute(const uint32_t* __restrict__ order, int n, const T* __restrict__ in, T* __restrict__ out) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = in[order[s]];
}

// Up to kMaxArrays per-particle arrays gathered in one pass: out_k[s] = in_k[order[s]], or
// a plain copy when order is null.  One launch reads order once instead of once per array.
__global__ void __launch_bounds__(256) k_permute_arrays(const uint32_t* __restrict__ order, int n, ArraySet a) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  copy_rows(a, s, order ? (int)order[s] : s);
}

}  // namespace sph

using namespace sph;

extern "C" {

sph_status_t sph_mdbc_wall_density(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                   const sph_params* params, void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && params->support > 0.f, "mdbc: bad arguments");
  if (walls->n == 0) return SPH_OK;
  k_mdbc<<<grid_for(walls->n, 128), 128, 0, as_stream(stream)>>>(to_fluid(fluid), to_walls(walls), grid,
                                                                 to_params(params));
  SPH_CHECK_LAUNCH("mdbc_wall_density");
  return SPH_OK;
}

// Neighbor records (two float4 per particle), then, for pairs from the cell rows, the
// segment lists: kMaxSegments masks and starts and a count per particle.
constexpr size_t kRecordBytes = 2 * sizeof(float4),
                 kMaskBytes = kMaxSegments * (sizeof(uint32_t) + sizeof(int32_t)) + sizeof(int32_t);
size_t sph_deltasph_scratch_bytes(int64_t n) { return (size_t)(n > 0 ? n : 0) * (kRecordBytes + kMaskBytes) + 256; }
static_assert(sizeof(Rec) == kRecordBytes, "a neighbor record is two float4");

sph_status_t sph_deltasph_segment_lists(int64_t n, size_t* masks_offset, size_t* starts_offset,
                                        size_t* counts_offset, int32_t* max_segments) {
  SPH_REQUIRE(n >= 0 && masks_offset && starts_offset && counts_offset && max_segments,
              "deltasph_segment_lists: bad arguments");
  *masks_offset = (size_t)n * kRecordBytes;
  *starts_offset = *masks_offset + (size_t)n * kMaxSegments * sizeof(uint32_t);
  *counts_offset = *starts_offset + (size_t)n * kMaxSegments * sizeof(int32_t);
  *max_segments = kMaxSegments;
  return SPH_OK;
}

}  // extern "C"

// The neighbor records in caller scratch, 32-byte aligned.
static bool records_from_scratch(void* scratch, size_t bytes, int64_t n, Rec** rec, Segments* seg = nullptr) {
  if (!scratch) return false;
  const uintptr_t base = reinterpret_cast<uintptr_t>(scratch);
  const uintptr_t p = (base + 31) & ~(uintptr_t)31;
  if ((p - base) + (size_t)n * (kRecordBytes + (seg ? kMaskBytes : 0)) > bytes) return false;
  *rec = reinterpret_cast<Rec*>(p);
  if (seg) {
    uint32_t* m = reinterpret_cast<uint32_t*>(*rec + n);
    int32_t* st = reinterpret_cast<int32_t*>(m + kMaxSegments * n);
    seg->mask = m;
    seg->start = st;
    seg->nseg = st + kMaxSegments * n;
  }
  return true;
}

extern "C" {

sph_status_t sph_deltasph_forces(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, float* dpdt, float* acc, float* L, float* grad_rho,
                                 void* scratch, size_t scratch_bytes, void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && dpdt && acc && params->support > 0.f, "deltasph_forces: bad arguments");
  SPH_REQUIRE(params->density_diffusion != 2 || grad_rho, "deltasph_forces: deltaSPH diffusion needs grad_rho");
  if (fluid->n == 0) return SPH_OK;
  Rec* rec;
  SPH_REQUIRE(records_from_scratch(scratch, scratch_bytes, fluid->n, &rec),
              "deltasph_forces: scratch smaller than sph_deltasph_scratch_bytes(n)");
  cudaStream_t st = as_stream(stream);
  const FluidView F = to_fluid(fluid);
  const WallView W = to_walls(walls);
  const SphParams P = to_params(params);
  const int nb = grid_for(fluid->n, 128);
  k_prep<<<grid_for(fluid->n, 256), 256, 0, st>>>(F, P, rec);
  k_dsph_pass1<<<nb, 128, 0, st>>>(F, rec, W, grid, P, dpdt, reinterpret_cast<float2*>(acc),
                                   reinterpret_cast<float4*>(L), reinterpret_cast<float2*>(grad_rho));
  if (P.diffusion == 2)
    k_dsph_diffusion<<<nb, 128, 0, st>>>(F, rec, P, reinterpret_cast<const float2*>(grad_rho), dpdt);
  SPH_CHECK_LAUNCH("deltasph_forces");
  return SPH_OK;
}

sph_status_t sph_integrate_semi_implicit_euler(int64_t n, const float* x, const float* v, const float* rho,
                                               const float* acc, const float* dpdt, const float* dt,
                                               float rest_density, int32_t continuum_density, float* x_out,
                                               float* v_out, float* rho_out, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && x && v && rho && acc && dt && x_out && v_out && rho_out,
              "integrate_semi_implicit_euler: bad arguments");
  SPH_REQUIRE(!continuum_density || dpdt, "integrate_semi_implicit_euler: continuum density needs dpdt");
  if (n == 0) return SPH_OK;
  k_sie<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      (int)n, reinterpret_cast<const float2*>(x), reinterpret_cast<const float2*>(v), rho,
      reinterpret_cast<const float2*>(acc), dpdt, dt, rest_density, continuum_density, reinterpret_cast<float2*>(x_out),
      reinterpret_cast<float2*>(v_out), rho_out, status);
  SPH_CHECK_LAUNCH("integrate_semi_implicit_euler");
  return SPH_OK;
}

sph_status_t sph_batch_deltasph_step(const sph_fluid_view* fluid, const sph_wall_view* walls, const void* scenes,
                                     const int32_t* sid, const int32_t* wall_sid, float* dpdt, float* acc,
                                     float* grad_rho, int32_t any_renormalized, float* x_out, float* v_out,
                                     float* rho_out, int32_t* status, int32_t phases, int32_t ngroups,
                                     const sph_force_group* groups, void* scratch, size_t scratch_bytes,
                                     void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(scenes && sid && x_out && v_out && rho_out && status, "batch_deltasph_step: bad arguments");
  SPH_REQUIRE(walls->n == 0 || wall_sid, "batch_deltasph_step: walls need wall_sid");
  SPH_REQUIRE(!any_renormalized || (dpdt && acc && grad_rho),
              "batch_deltasph_step: deltaSPH diffusion needs dpdt, acc, grad_rho");
  // no CSR list (offsets and cols NULL): the pairs come from the cell rows
  const bool cells = !fluid->offsets && !fluid->cols;
  SPH_REQUIRE(cells || (fluid->offsets && fluid->cols), "batch_deltasph_step: give both offsets and cols, or neither");
  SPH_REQUIRE(fluid->cell_start && fluid->keys, "batch_deltasph_step: bad arguments");
  const int n = (int)fluid->n;
  // force groups: by default one group, one lane per particle, any schemes
  const sph_force_group all{0, n, 1, -1};
  SPH_REQUIRE(ngroups >= 0 && (ngroups == 0 || groups), "batch_deltasph_step: bad groups");
  const int ng = ngroups ? ngroups : 1;
  const sph_force_group* G = ngroups ? groups : &all;
  SPH_REQUIRE(G[0].begin == 0 && G[ng - 1].end == n, "batch_deltasph_step: the groups must tile [0, n)");
  for (int k = 0; k < ng; ++k) {
    SPH_REQUIRE(G[k].begin <= G[k].end && (k == 0 || G[k].begin == G[k - 1].end),
                "batch_deltasph_step: the groups must tile [0, n) in order");
    SPH_REQUIRE(G[k].tpp == 1 || (cells && (G[k].tpp == 2 || G[k].tpp == 4)),
                "batch_deltasph_step: lanes per particle must be 1 (2 or 4 with pairs from the cell rows)");
    SPH_REQUIRE(G[k].scheme >= -1 && G[k].scheme <= 2, "batch_deltasph_step: bad diffusion scheme");
  }
  if (n == 0) return SPH_OK;
  Rec* rec;
  Segments seg{};
  SPH_REQUIRE(records_from_scratch(scratch, scratch_bytes, n, &rec, cells ? &seg : nullptr),
              "batch_deltasph_step: scratch smaller than sph_deltasph_scratch_bytes(n)");
  cudaStream_t st = as_stream(stream);
  const FluidView F = to_fluid(fluid);
  const WallView W = to_walls(walls);
  const SceneDev* S = static_cast<const SceneDev*>(scenes);
  if (W.n > 0 && (phases & SPH_PHASE_WALLS)) k_batch_mdbc<<<grid_for(W.n, 128), 128, 0, st>>>(F, W, S, wall_sid);
  if (phases & SPH_PHASE_RECORDS)
    k_batch_prep<<<grid_for(n, 256), 256, 0, st>>>(F, S, sid, rec, const_cast<int32_t*>(seg.nseg),
                                                   const_cast<int32_t*>(seg.start), const_cast<uint32_t*>(seg.mask));
  float2* xo = reinterpret_cast<float2*>(x_out);
  float2* vo = reinterpret_cast<float2*>(v_out);
  float2* gr = reinterpret_cast<float2*>(grad_rho);
  float2* ac = reinterpret_cast<float2*>(acc);
  // kernel variants: CSR rows run one lane and read the scheme per scene; cell rows have 1, 2
  // or 4 lanes and a scheme of MOG, deltaSPH or read per scene
  auto pass1 = [&](int lo, int hi, int t, int scheme) {
    const int nb = grid_for((int64_t)(hi - lo) * t, 128);
#define SPH_PASS1(C, T, K)                                                                                  \
  k_batch_pass1<C, T, K><<<nb, 128, 0, st>>>(F, rec, W, S, sid, dpdt, ac, gr, C ? seg : Segments{}, xo, vo, \
                                             rho_out, status, lo, hi)
    if (!cells) {
      SPH_PASS1(false, 1, -1);
      return;
    }
    const int k = scheme == 1 || scheme == 2 ? scheme : -1;
    if (t == 1) {
      if (k == 2) SPH_PASS1(true, 1, 2);
      else if (k == 1) SPH_PASS1(true, 1, 1);
      else SPH_PASS1(true, 1, -1);
    } else if (t == 2) {
      if (k == 2) SPH_PASS1(true, 2, 2);
      else if (k == 1) SPH_PASS1(true, 2, 1);
      else SPH_PASS1(true, 2, -1);
    } else {
      if (k == 2) SPH_PASS1(true, 4, 2);
      else if (k == 1) SPH_PASS1(true, 4, 1);
      else SPH_PASS1(true, 4, -1);
    }
#undef SPH_PASS1
  };
  for (int k = 0; k < ng && (phases & SPH_PHASE_PASS1); ++k)
    if (G[k].end > G[k].begin) pass1((int)G[k].begin, (int)G[k].end, G[k].tpp, G[k].scheme);
  for (int k = 0; k < ng && any_renormalized && (phases & SPH_PHASE_DIFFUSION); ++k) {
    const int lo = (int)G[k].begin, hi = (int)G[k].end, t = G[k].tpp;
    if (hi <= lo || G[k].scheme == 0 || G[k].scheme == 1) continue;   // no deltaSPH scene in the group
    const int nb = grid_for((int64_t)(hi - lo) * t, 128);
    if (!cells)
      k_batch_diffusion<false, 1><<<nb, 128, 0, st>>>(F, rec, S, sid, gr, Segments{}, dpdt, ac, xo, vo, rho_out,
                                                      status, lo, hi);
    else if (t == 1)
      k_batch_diffusion<true, 1><<<nb, 128, 0, st>>>(F, rec, S, sid, gr, seg, dpdt, ac, xo, vo, rho_out, status, lo,
                                                     hi);
    else if (t == 2)
      k_batch_diffusion<true, 2><<<nb, 128, 0, st>>>(F, rec, S, sid, gr, seg, dpdt, ac, xo, vo, rho_out, status, lo,
                                                     hi);
    else
      k_batch_diffusion<true, 4><<<nb, 128, 0, st>>>(F, rec, S, sid, gr, seg, dpdt, ac, xo, vo, rho_out, status, lo,
                                                     hi);
  }
  SPH_CHECK_LAUNCH("batch_deltasph_step");
  return SPH_OK;
}

size_t sph_scene_bytes(void) { return sizeof(SceneDev); }

sph_status_t sph_scene_encode(const sph_params* params, const sph_grid* grid_host, int32_t cell_offset, float dt,
                              void* out_host) {
  SPH_REQUIRE(params && grid_host && out_host && params->support > 0.f, "scene_encode: bad arguments");
  SceneDev s;
  s.P = to_params(params);
  s.g = *grid_host;
  s.coff = cell_offset;
  s.dt = dt;
  memcpy(out_host, &s, sizeof(s));
  return SPH_OK;
}

sph_status_t sph_rk_axpy(int64_t n, const float* x0, const float* v0, const float* rho0_field, const float* ku,
                         const float* ka, const float* kd, const float* dt, float c, float rest_density, float* x_out,
                         float* v_out, float* rho_out, int32_t* status, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && x0 && v0 && rho0_field && ku && ka && kd && dt && x_out && v_out && rho_out,
              "rk_axpy: bad arguments");
  if (n == 0) return SPH_OK;
  k_rk_axpy<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      (int)n, reinterpret_cast<const float2*>(x0), reinterpret_cast<const float2*>(v0), rho0_field,
      reinterpret_cast<const float2*>(ku), reinterpret_cast<const float2*>(ka), kd, dt, c, rest_density,
      reinterpret_cast<float2*>(x_out), reinterpret_cast<float2*>(v_out), rho_out, status);
  SPH_CHECK_LAUNCH("rk_axpy");
  return SPH_OK;
}

sph_status_t sph_rk_accumulate(int64_t n, const float* ku, const float* ka, const float* kd, float w, int32_t init,
                               float* su, float* sa, float* sd, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && ku && ka && kd && su && sa && sd, "rk_accumulate: bad arguments");
  if (n == 0) return SPH_OK;
  k_rk_accum<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      (int)n, reinterpret_cast<const float2*>(ku), reinterpret_cast<const float2*>(ka), kd, w, init,
      reinterpret_cast<float2*>(su), reinterpret_cast<float2*>(sa), sd);
  SPH_CHECK_LAUNCH("rk_accumulate");
  return SPH_OK;
}

sph_status_t sph_permute_arrays(const uint32_t* order, int64_t n, int32_t count, const int32_t* elem_bytes,
                                const void* const* in, void* const* out, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && count >= 0 && count <= kMaxArrays && (count == 0 || (elem_bytes && in && out)),
              "permute_arrays: bad arguments");
  if (n == 0 || count == 0) return SPH_OK;
  ArraySet a;
  SPH_REQUIRE(array_set_from(count, elem_bytes, in, out, &a),
              "permute_arrays: each array needs distinct in/out and 4, 8 or 16-byte elements");
  k_permute_arrays<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(order, (int)n, a);
  SPH_CHECK_LAUNCH("permute_arrays");
  return SPH_OK;
}

sph_status_t sph_permute(const uint32_t* order, int64_t n, int32_t elem_bytes, const void* in, void* out, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && order && in && out, "permute: bad arguments");
  if (n == 0) return SPH_OK;
  cudaStream_t st = as_stream(stream);
  const int nb = grid_for(n, 256);
  switch (elem_bytes) {
    case 4:
      k_permute<uint32_t><<<nb, 256, 0, st>>>(order, (int)n, static_cast<const uint32_t*>(in), static_cast<uint32_t*>(out));
      break;
    case 8:
      k_permute<uint2><<<nb, 256, 0, st>>>(order, (int)n, static_cast<const uint2*>(in), static_cast<uint2*>(out));
      break;
    case 16:
      k_permute<uint4><<<nb, 256, 0, st>>>(order, (int)n, static_cast<const uint4*>(in), static_cast<uint4*>(out));
      break;
    default:
      set_error_text("permute: elem_bytes must be 4, 8 or 16");
      return SPH_ERR_INVALID_ARGUMENT;
  }
  SPH_CHECK_LAUNCH("permute");
  return SPH_OK;
}

}  // extern "C"
