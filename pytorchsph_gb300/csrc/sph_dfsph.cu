// DFSPH on sm_103a (src/modules/dfsph.py with the solid-wall PBSPH terms of
// src/modules/solidBoundary.py:294-520).
//
// The pressure solve (densitySolve / divergenceSolve, dfsph.py:195-260) runs as ONE
// cooperative kernel: every iteration is  accel from p (all particles)  -> grid barrier ->
// pressure-sum, residual, relaxed-Jacobi update and the block partials of the error ->
// grid barrier -> every block sums the partials in the same order (identical double result
// everywhere, so every block takes the same loop decision).  The loop is bounded by
// max_iters, so every thread meets every barrier the same number of times.
#include <cooperative_groups.h>

#include <mutex>

#include "sph_math.cuh"

namespace cg = cooperative_groups;

namespace sph {

struct DfsphBufs {
  // fluid, sorted order
  float* rho;         // relative density incl. the wall contribution
  float* vol;         // A / rho_fluid_only (fluidVolume)
  float* aact;        // A / rho (fluidActualArea)
  float2* vstar;      // predicted velocity
  float* alpha;
  float* source;
  float* p;           // pressure (fluidPressure2)
  float2* pa;         // predicted pressure acceleration
  float* res;
  // walls
  float* wrho;        // wall relative density (summation, clamped <= 1)
  float* waact;       // A_b / rho_b
  float* walpha;
  float* wsource;
  float* wp;
  float* wres;
  const float* wterm; // static wall-wall density term
  // solver output
  double* partials;   // [gridDim.x] block partial errors
  float* errors;      // [max_iters + 1] error history
  int32_t* iters;     // iteration count
  // pair records of the Jacobi sweeps, one 16-byte gather per neighbor and phase:
  float4* rec_p;      // (x, y, m = A rho0, p / (rho rho0)^2), its pressure part updated every sweep
  float4* rec_a;      // (x, y, predicted pressure acceleration)
  float* fdt;         // dt^2 A_act
};

// ---------------------------------------------------------------- densities
// fluid: rho = rho_fluid (from the count pass) + sum_b W A_b  (solidBoundary.py:522-549)
__global__ void __launch_bounds__(128) k_dfsph_fluid_density(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                             SphParams P, const float* __restrict__ rho_fluid,
                                                             DfsphBufs B) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const float rf = rho_fluid[i];
  float rw = 0.f;
  if (W.n > 0) {
    const sph_grid g = *gp;
    int cx, cy;
    cell_of(F.keys[i], g, &cx, &cy);
    const float2 xi = F.x[i];
    const float thr = P.thr;
    for_each_wall(W, g, P.search_radius, cx, cy, xi.x, xi.y, thr, [&](int b, float2 xb) {
      const Geo e = geo(xb.x, xb.y, xi.x, xi.y, P.inv_h);
      rw += kW(e.q, P.c_w) * W.area[b];
    });
  }
  const float A = F.area[i];
  const float r = rf + rw;
  B.rho[i] = r;
  B.vol[i] = A / rf;
  B.aact[i] = A / r;
}

// walls: rho_b = min(term_b + sum_f W A_f, 1), A_b^act = A_b / rho_b
__global__ void __launch_bounds__(128) k_dfsph_wall_density(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                            SphParams P, DfsphBufs B) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W.n) return;
  const sph_grid g = *gp;
  const float2 xb = W.x[b];
  const float thr = P.thr;
  float s = 0.f;
  int qx, qy;
  float fcx = ceilf(__fdiv_rn(__fsub_rn(xb.x, g.qmin[0]), g.hmax));
  float fcy = ceilf(__fdiv_rn(__fsub_rn(xb.y, g.qmin[1]), g.hmax));
  if (grid_ok(g, P.cell_capacity) && fcx > -1e9f && fcx < 1e9f && fcy > -1e9f && fcy < 1e9f) {
    qx = (int)fcx;
    qy = (int)fcy;
    const int r = P.search_radius;
    const int x0 = max(qx - r, 0), x1 = min(qx + r, g.cells_x - 1);
    const int y0 = max(qy - r, 0), y1 = min(qy + r, g.cells_y - 1);
    if (x0 <= x1)
      for (int yy = y0; yy <= y1; ++yy) {
        const int row = yy * g.cells_x;
        for (int j = F.cell_start[row + x0]; j < F.cell_start[row + x1 + 1]; ++j) {
          const float2 xj = F.x[j];
          if (!(dist2_ref(xb.x, xb.y, xj.x, xj.y) <= thr)) continue;
          const Geo e = geo(xb.x, xb.y, xj.x, xj.y, P.inv_h);
          s += kW(e.q, P.c_w) * F.area[j];
        }
      }
  }
  const float rb = fminf(B.wterm[b] + s, 1.0f);
  B.wrho[b] = rb;
  B.waact[b] = W.area[b] / rb;
}

// static wall-wall density term: sum over wall neighbors of W * A_b' (solidBoundary.py:180-200)
__global__ void __launch_bounds__(128) k_wall_wall_term(WallView W, const sph_grid* __restrict__ gp, SphParams P,
                                                        float* __restrict__ term) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W.n) return;
  const sph_grid g = *gp;
  const float2 xb = W.x[b];
  float fcx = ceilf(__fdiv_rn(__fsub_rn(xb.x, g.qmin[0]), g.hmax));
  float fcy = ceilf(__fdiv_rn(__fsub_rn(xb.y, g.qmin[1]), g.hmax));
  float s = 0.f;
  if (grid_ok(g, P.cell_capacity) && fcx > -1e9f && fcx < 1e9f && fcy > -1e9f && fcy < 1e9f) {
    const float thr = P.thr;
    for_each_wall(W, g, P.search_radius, (int)fcx, (int)fcy, xb.x, xb.y, thr, [&](int c, float2 xc) {
      const Geo e = geo(xb.x, xb.y, xc.x, xc.y, P.inv_h);
      s += kW(e.q, P.c_w) * W.area[c];
    });
  }
  term[b] = s;
}

// ---------------------------------------------------------------- solver set-up
// The spiky gradient of pair (i, j) as gs * d with d = x_i - x_j: spikyGrad = e kGS(q), e =
// d / r, so gs = kGS(q) / r, from one reciprocal square root (0 when r < 1e-7, where the
// reference's e is zero).
__device__ __forceinline__ float spiky_gd(float r2, const SphParams& P) {
  if (!(r2 >= 1e-14f)) return 0.f;
  const float rs = rsqrt_normal(r2);
  return kGS(r2 * rs * P.inv_h, P.c_s) * rs;
}

// The Wendland gradient the same way: gradW = e kGW(q) = gw * d.
__device__ __forceinline__ float wendland_gd(float r2, const SphParams& P) {
  if (!(r2 >= 1e-14f)) return 0.f;
  const float rs = rsqrt_normal(r2);
  return kGW(r2 * rs * P.inv_h, P.c_g) * rs;
}

// v* = v + dt a, and the pair records of the preparation pass: rec_a = (x, y, v*),
// rec_p = (A_act, A_act^2 / (A rho0)) (both rewritten by the solve before it reads them).
__global__ void k_dfsph_vstar(FluidView F, SphParams P, DfsphBufs B, const float2* __restrict__ acc,
                              const float* __restrict__ dt_ptr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const float dt = *dt_ptr;
  const float2 a = acc[i], u = F.v[i], x = F.x[i];
  const float2 vs = make_float2(u.x + dt * a.x, u.y + dt * a.y);
  B.vstar[i] = vs;
  B.rec_a[i] = make_float4(x.x, x.y, vs.x, vs.y);
  const float aa = B.aact[i];
  B.rec_p[i] = make_float4(aa, aa * aa / (F.area[i] * P.rho0), 0.f, 0.f);
}

// The pair records of the viscosity pass: rec_a = (x, y, v), rec_p = (V, rho rho0).
__global__ void k_dfsph_visc_records(FluidView F, SphParams P, DfsphBufs B) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const float2 x = F.x[i], u = F.v[i];
  B.rec_a[i] = make_float4(x.x, x.y, u.x, u.y);
  B.rec_p[i] = make_float4(B.vol[i], B.rho[i] * P.rho0, 0.f, 0.f);
}

// alpha (dfsph.py:58-83 + solidBoundary.py:443-479) and source (dfsph.py:85-100, 154-161 +
// solidBoundary.py:481-520) per fluid particle.  Wall terms only in the density solve.
__global__ void __launch_bounds__(128) k_dfsph_prepare(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                       SphParams P, DfsphBufs B, const float* __restrict__ dt_ptr,
                                                       int density) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const float dt = *dt_ptr;
  const float4 me = B.rec_a[i];
  const float2 xi = make_float2(me.x, me.y);
  const float2 vi = make_float2(me.z, me.w);
  float k1x = 0.f, k1y = 0.f, k2 = 0.f, src = 0.f;
  const int k0 = F.offsets[i], kn = row_end(F, i, k0);
  for (int k = k0; k < kn; ++k) {
    const int j = __ldg(F.cols + k);
    const float4 rj = __ldg(B.rec_a + j);
    const float2 qj = __ldg(reinterpret_cast<const float2*>(B.rec_p + j));   // (A_act, A_act^2 / m)
    const float dx = xi.x - rj.x, dy = xi.y - rj.y;
    const float gd = spiky_gd(dx * dx + dy * dy, P);
    const float gx = gd * dx, gy = gd * dy;
    const float aj = qj.x;
    k1x += aj * gx;
    k1y += aj * gy;
    k2 += qj.y * (gx * gx + gy * gy);
    src += -dt * aj * ((vi.x - rj.z) * gx + (vi.y - rj.w) * gy);
  }
  float w1x = 0.f, w1y = 0.f, w2 = 0.f, wsrc = 0.f;
  if (density && W.n > 0) {
    const sph_grid g = *gp;
    int cx, cy;
    cell_of(F.keys[i], g, &cx, &cy);
    const float thr = P.thr;
    for_each_wall(W, g, P.search_radius, cx, cy, xi.x, xi.y, thr, [&](int b, float2 xb) {
      const Geo e = geo(xb.x, xb.y, xi.x, xi.y, P.inv_h);   // e = (x_b - x_f)/r
      const float gs = kGS(e.q, P.c_s);
      const float gx = gs * e.ex, gy = gs * e.ey;
      const float ab = B.waact[b], Ab = W.area[b];
      w1x += ab * gx;
      w1y += ab * gy;
      w2 += (ab * ab / (Ab * P.rho0)) * (gx * gx + gy * gy);
      wsrc += ab * ((0.f - vi.x) * gx + (0.f - vi.y) * gy);
    });
  }
  k1x += w1x;
  k1y += w1y;
  k2 += w2;
  const float aa = B.aact[i], Ai = F.area[i];
  const float fac = -dt * dt * aa;
  float alpha = fac / (Ai * P.rho0) * (k1x * k1x + k1y * k1y) + fac * k2;
  alpha = fminf(fmaxf(alpha, -1.0f), -1e-7f);
  B.alpha[i] = alpha;
  float s = src + (-dt) * wsrc;
  B.source[i] = density ? 1.0f - B.rho[i] + s : s;
  B.p[i] = 0.f;
}

// wall alpha and source (PBSPH branch, solidBoundary.py:463-466, 499-503)
__global__ void __launch_bounds__(128) k_dfsph_wall_prepare(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                            SphParams P, DfsphBufs B, const float* __restrict__ dt_ptr) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W.n) return;
  const float dt = *dt_ptr;
  const sph_grid g = *gp;
  const float2 xb = W.x[b];
  const float thr = P.thr;
  float t = 0.f, s = 0.f;
  float fcx = ceilf(__fdiv_rn(__fsub_rn(xb.x, g.qmin[0]), g.hmax));
  float fcy = ceilf(__fdiv_rn(__fsub_rn(xb.y, g.qmin[1]), g.hmax));
  if (grid_ok(g, P.cell_capacity) && fcx > -1e9f && fcx < 1e9f && fcy > -1e9f && fcy < 1e9f) {
    const int qx = (int)fcx, qy = (int)fcy, r = P.search_radius;
    const int x0 = max(qx - r, 0), x1 = min(qx + r, g.cells_x - 1);
    const int y0 = max(qy - r, 0), y1 = min(qy + r, g.cells_y - 1);
    if (x0 <= x1)
      for (int yy = y0; yy <= y1; ++yy) {
        const int row = yy * g.cells_x;
        for (int j = F.cell_start[row + x0]; j < F.cell_start[row + x1 + 1]; ++j) {
          const float2 xj = F.x[j];
          if (!(dist2_ref(xb.x, xb.y, xj.x, xj.y) <= thr)) continue;
          const Geo e = geo(xb.x, xb.y, xj.x, xj.y, P.inv_h);   // e = (x_b - x_f)/r
          const float gs = kGS(e.q, P.c_s);
          const float gx = gs * e.ex, gy = gs * e.ey;
          const float af = B.aact[j];
          t += (af * af / (F.area[j] * P.rho0)) * (gx * gx + gy * gy);
          const float2 vj = B.vstar[j];
          s += af * ((0.f - vj.x) * gx + (0.f - vj.y) * gy);
        }
      }
  }
  const float ab = B.waact[b];
  B.walpha[b] = fminf(-dt * dt * ab * t, -0.0001f * P.h * P.h);
  B.wsource[b] = 1.0f - B.wrho[b] + (-dt) * s;
  B.wp[b] = 0.f;
}

// ---------------------------------------------------------------- solver phases

// predicted pressure acceleration of fluid particle i (dfsph.py:25-42 + solidBoundary.py:310-403),
// the fluid pairs from the records rec_p = (x, y, m, p / rho^2)
__device__ __forceinline__ float2 pressure_accel(const FluidView& F, const WallView& W, const sph_grid& g,
                                                 const SphParams& P, const DfsphBufs& B, int i, bool walls) {
  const float4 me = B.rec_p[i];
  const float2 xi = make_float2(me.x, me.y);
  const float ppi = me.w;
  float ax = 0.f, ay = 0.f;
  const int k0 = F.offsets[i], kn = row_end(F, i, k0);
  for (int k = k0; k < kn; ++k) {
    const float4 rj = __ldg(B.rec_p + __ldg(F.cols + k));
    const float dx = xi.x - rj.x, dy = xi.y - rj.y;
    const float f = -rj.z * (ppi + rj.w) * spiky_gd(dx * dx + dy * dy, P);
    ax += f * dx;
    ay += f * dy;
  }
  if (walls) {
    float wx = 0.f, wy = 0.f;
    int cx, cy;
    cell_of(F.keys[i], g, &cx, &cy);
    const float thr = P.thr;
    for_each_wall(W, g, P.search_radius, cx, cy, xi.x, xi.y, thr, [&](int b, float2 xb) {
      // spiky(e_bf) = gd (x_b - x_f), used negated
      const float dx = xb.x - xi.x, dy = xb.y - xi.y;
      const float gd = spiky_gd(dx * dx + dy * dy, P);
      const float rb = B.wrho[b] * P.rho0;
      const float pb = B.wp[b] / (rb * rb);
      const float f = (W.area[b] * P.rho0) * (ppi + pb) * gd;
      wx += f * dx;
      wy += f * dy;
    });
    ax += wx;
    ay += wy;
  }
  return make_float2(ax, ay);
}

__global__ void __launch_bounds__(256, 4) k_dfsph_solve(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                     SphParams P, DfsphBufs B, const float* __restrict__ dt_ptr,
                                                     int density, int min_iters, int max_iters, float thr_err,
                                                     float omega_f, float omega_b, int32_t* status) {
  cg::grid_group grid = cg::this_grid();
  const sph_grid g = *gp;
  const float dt = *dt_ptr;
  const bool walls = density && W.n > 0;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  const double count = (double)F.n + (walls ? (double)W.n : 0.0);
  __shared__ double s_part[8];
  // the pair records: positions, masses and dt^2 A_act are fixed during the solve
  for (int i = tid; i < F.n; i += nthreads) {
    const float2 xi = F.x[i];
    const float ri = B.rho[i] * P.rho0;
    B.rec_p[i] = make_float4(xi.x, xi.y, F.area[i] * P.rho0, B.p[i] / (ri * ri));
    B.fdt[i] = dt * dt * B.aact[i];
  }
  grid.sync();
  double err = 0.0;
  int it = 0;
  while ((it < min_iters || err > (double)thr_err) && it <= max_iters) {
    // phase A: predicted acceleration from the current pressures
    for (int i = tid; i < F.n; i += nthreads) {
      const float2 a = pressure_accel(F, W, g, P, B, i, walls);
      B.pa[i] = a;
      const float4 me = B.rec_p[i];
      B.rec_a[i] = make_float4(me.x, me.y, a.x, a.y);
    }
    grid.sync();
    // phase B: pressure sums, residuals, relaxed Jacobi updates, error partials
    double local = 0.0;
    for (int i = tid; i < F.n; i += nthreads) {
      const float4 me = B.rec_a[i];
      const float2 xi = make_float2(me.x, me.y), pai = make_float2(me.z, me.w);
      float ks = 0.f;
      const int k0 = F.offsets[i], kn = row_end(F, i, k0);
      for (int k = k0; k < kn; ++k) {
        const int j = __ldg(F.cols + k);
        const float4 rj = __ldg(B.rec_a + j);
        const float dx = xi.x - rj.x, dy = xi.y - rj.y;
        ks += __ldg(B.fdt + j) * ((pai.x - rj.z) * dx + (pai.y - rj.w) * dy) * spiky_gd(dx * dx + dy * dy, P);
      }
      if (walls) {
        float wks = 0.f;
        int cx, cy;
        cell_of(F.keys[i], g, &cx, &cy);
        const float thr = P.thr;
        for_each_wall(W, g, P.search_radius, cx, cy, xi.x, xi.y, thr, [&](int b, float2 xb) {
          const float dx = xb.x - xi.x, dy = xb.y - xi.y;
          const float gd = spiky_gd(dx * dx + dy * dy, P);
          wks -= dt * dt * B.waact[b] * gd * (pai.x * dx + pai.y * dy);
        });
        ks += wks;
      }
      const float r = ks - B.source[i];
      B.res[i] = r;
      float pn = B.p[i] - omega_f * r / B.alpha[i];
      if (density) pn = fmaxf(pn, 0.f);
      if (!isfinite(pn)) flag(status, SPH_FLAG_NONFINITE);
      B.p[i] = pn;
      const float ri = B.rho[i] * P.rho0;
      B.rec_p[i].w = pn / (ri * ri);
      local += (double)fmaxf(r, -thr_err);
    }
    if (walls) {
      for (int b = tid; b < W.n; b += nthreads) {
        const float2 xb = W.x[b];
        float bks = 0.f;
        float fcx = ceilf(__fdiv_rn(__fsub_rn(xb.x, g.qmin[0]), g.hmax));
        float fcy = ceilf(__fdiv_rn(__fsub_rn(xb.y, g.qmin[1]), g.hmax));
        if (grid_ok(g, P.cell_capacity) && fcx > -1e9f && fcx < 1e9f && fcy > -1e9f && fcy < 1e9f) {
          const int qx = (int)fcx, qy = (int)fcy, rr = P.search_radius;
          const int x0 = max(qx - rr, 0), x1 = min(qx + rr, g.cells_x - 1);
          const int y0 = max(qy - rr, 0), y1 = min(qy + rr, g.cells_y - 1);
          const float thr = P.thr;
          if (x0 <= x1)
            for (int yy = y0; yy <= y1; ++yy) {
              const int row = yy * g.cells_x;
              for (int j = F.cell_start[row + x0]; j < F.cell_start[row + x1 + 1]; ++j) {
                const float2 xj = F.x[j];
                if (!(dist2_ref(xb.x, xb.y, xj.x, xj.y) <= thr)) continue;
                const float dx = xb.x - xj.x, dy = xb.y - xj.y;
                const float gd = spiky_gd(dx * dx + dy * dy, P);
                const float2 paj = B.pa[j];
                bks -= dt * dt * B.aact[j] * gd * (paj.x * dx + paj.y * dy);
              }
            }
        }
        const float rb = bks - B.wsource[b];
        B.wres[b] = rb;
        B.wp[b] = fmaxf(B.wp[b] - omega_b * rb / B.walpha[b], 0.f);
        local += (double)fmaxf(rb, -thr_err);
      }
    }
    // block partial of the error
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
      B.partials[blockIdx.x] = t;
    }
    grid.sync();
    // phase C: every block forms the same mean error in the same order (a strided sum per
    // thread, then a fixed tree over the block: identical arithmetic in every block)
    double tot = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) tot += B.partials[k];
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    __syncthreads();  // s_part is reused
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = tot;
    __syncthreads();
    tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_part[w];
    err = tot / count;
    if (tid == 0) B.errors[it] = (float)err;
    ++it;
    __syncthreads();
  }
  // final acceleration with the converged pressures (dfsph.py:303-309)
  for (int i = tid; i < F.n; i += nthreads) B.pa[i] = pressure_accel(F, W, g, P, B, i, walls);
  if (tid == 0) *B.iters = it;
}

// ---------------------------------------------------------------- viscosity (DFSPH steps 11-12)
// artificial viscosity with walls and laminar viscosity; V = A / rho_fluid_only (the volume
// set before the wall density is added, src/dfsph.py:151-163), rho = rho~ rho0 incl. walls.
__global__ void __launch_bounds__(128) k_dfsph_viscosity(FluidView F, WallView W, const sph_grid* __restrict__ gp,
                                                         SphParams P, DfsphBufs B, float2* __restrict__ acc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.n) return;
  const float4 me = B.rec_a[i];
  const float2 xi = make_float2(me.x, me.y), vi = make_float2(me.z, me.w);
  const float rhoi = B.rho[i] * P.rho0;
  float vax = 0.f, vay = 0.f, lax = 0.f, lay = 0.f;
  const int k0 = F.offsets[i], kn = row_end(F, i, k0);
  for (int k = k0; k < kn; ++k) {
    const int j = __ldg(F.cols + k);
    const float4 rj = __ldg(B.rec_a + j);
    const float2 qj = __ldg(reinterpret_cast<const float2*>(B.rec_p + j));   // (V, rho rho0)
    const float2 vj = make_float2(rj.z, rj.w);
    const float Vj = qj.x, rhoj = qj.y;
    const float dx = xi.x - rj.x, dy = xi.y - rj.y;
    const float d2 = dx * dx + dy * dy;
    const float gd = wendland_gd(d2, P);
    const float gx = gd * dx, gy = gd * dy;
    const float ux = vj.x - vi.x, uy = vj.y - vi.y;
    const float rx = -dx, ry = -dy;
    const float r2 = rx * rx + ry * ry + P.eps;
    const float pij = fminf(ux * rx + uy * ry, 0.f) / r2;
    const float vf = pij * Vj * rhoj / (rhoi + rhoj);
    vax += vf * gx;
    vay += vf * gy;
    const float mj = rhoj * Vj;
    const float rs = rhoi + rhoj;
    const float term = 4.0f * mj * (2.0f * rhoi * P.kinematic) * (rx * gx + ry * gy) / (rs * rs * r2);
    lax -= term * (vi.x - vj.x);
    lay -= term * (vi.y - vj.y);
  }
  float vwx = 0.f, vwy = 0.f;
  if (W.n > 0 && P.boundary_diffusion) {
    const sph_grid g = *gp;
    int cx, cy;
    cell_of(F.keys[i], g, &cx, &cy);
    const float thr = P.thr;
    for_each_wall(W, g, P.search_radius, cx, cy, xi.x, xi.y, thr, [&](int b, float2 xb) {
      const Geo e = geo(xi.x, xi.y, xb.x, xb.y, P.inv_h);
      const float gw = kGW(e.q, P.c_g);
      const float gx = gw * e.ex, gy = gw * e.ey;
      const float rb = B.wrho[b];
      const float Vb = W.area[b] / rb, rhob = rb * P.rho0;
      const float rx = -e.dx, ry = -e.dy;
      const float r2 = rx * rx + ry * ry + P.eps;
      const float pij = fminf(-vi.x * rx - vi.y * ry, 0.f) / r2;
      const float vf = pij * Vb * rhob / (rhoi + rhob);
      vwx += vf * gx;
      vwy += vf * gy;
    });
  }
  float2 a = acc[i];
  a.x += P.visc_k * vax + P.visc_k * vwx + lax;
  a.y += P.visc_k * vay + P.visc_k * vwy + lay;
  acc[i] = a;
}

// a += pa (fluidAcceleration += fluidPredAccel, src/dfsph.py:179, 185)
__global__ void k_add2(int n, const float2* __restrict__ b, float2* __restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 x = a[i], y = b[i];
  a[i] = make_float2(x.x + y.x, x.y + y.y);
}

__global__ void k_fill2(int n, float gx, float gy, float2* __restrict__ a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = make_float2(gx, gy);
}

// ---------------------------------------------------------------- adaptive dt (adaptiveDT.py:59-95)
__global__ void __launch_bounds__(256) k_dt_partials(int n, const float2* __restrict__ v, const float2* __restrict__ a,
                                                     float h, float* __restrict__ part) {
  float vmax = 0.f, amin = INFINITY;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 u = v[i], b = a[i];
    vmax = fmaxf(vmax, sqrtf(u.x * u.x + u.y * u.y));
    amin = fminf(amin, sqrtf(h / sqrtf(b.x * b.x + b.y * b.y)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    amin = fminf(amin, __shfl_xor_sync(0xffffffffu, amin, o));
  }
  __shared__ float sv[8], sa[8];
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = vmax;
    sa[threadIdx.x >> 5] = amin;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      vmax = fmaxf(vmax, sv[w]);
      amin = fminf(amin, sa[w]);
    }
    part[2 * blockIdx.x] = vmax;
    part[2 * blockIdx.x + 1] = amin;
  }
}

__global__ void k_dt_final(int nparts, const float* __restrict__ part, float h, float kinematic, float cfl, float c0,
                           int acoustic_from_c0, float dt_min, float dt_max, float* __restrict__ dt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float vmax = 0.f, amin = INFINITY;
  for (int k = 0; k < nparts; ++k) {
    vmax = fmaxf(vmax, part[2 * k]);
    amin = fminf(amin, part[2 * k + 1]);
  }
  const double visc = 0.125 * (double)h * h / kinematic;
  const double accdt = 0.25 * (double)amin;
  const double vdt = acoustic_from_c0 ? (double)cfl * h / c0 : 0.4 * (double)h / vmax;
  double m = dt_max;
  if (dt_min != 0.f) {
    m = fmin(m, visc);
    m = fmin(m, accdt);
    if (!isnan(vdt)) m = fmin(m, vdt);
  }
  const double target = m > dt_min ? m : dt_min;
  const double cur = *dt;
  *dt = (float)fmin(fmax(target, cur * 0.5), cur * 1.05);
}

}  // namespace sph

using namespace sph;

// n: the fluid count, which places the pair records inside b->records.
static DfsphBufs to_bufs(const sph_dfsph_buffers* b, int64_t n = 0) {
  DfsphBufs B;
  B.rho = b->rho;
  B.vol = b->volume;
  B.aact = b->actual_area;
  B.vstar = reinterpret_cast<float2*>(b->vstar);
  B.alpha = b->alpha;
  B.source = b->source;
  B.p = b->pressure;
  B.pa = reinterpret_cast<float2*>(b->pred_accel);
  B.res = b->residual;
  B.wrho = b->wall_rho;
  B.waact = b->wall_actual_area;
  B.walpha = b->wall_alpha;
  B.wsource = b->wall_source;
  B.wp = b->wall_pressure;
  B.wres = b->wall_residual;
  B.wterm = b->wall_density_term;
  B.partials = b->partials;
  B.errors = b->errors;
  B.iters = b->iters;
  B.rec_p = b->records ? reinterpret_cast<float4*>(b->records) : nullptr;
  B.rec_a = B.rec_p ? B.rec_p + n : nullptr;
  B.fdt = B.rec_p ? b->records + 8 * n : nullptr;
  return B;
}

// Cooperative grid size of k_dfsph_solve per GPU (resident blocks x SMs), computed on the
// first solve on that GPU; GPUs of one process may differ in SM count.
constexpr int kCoopMaxDevices = 64;
static int g_coop_blocks[kCoopMaxDevices] = {0};
static std::mutex g_coop_mu;

extern "C" {

size_t sph_dfsph_partials_count(void) { return (size_t)kNumSMs * 8; }

sph_status_t sph_dfsph_wall_wall_term(const sph_wall_view* walls, const sph_grid* grid, const sph_params* params,
                                      float* term, void* stream) {
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && term, "dfsph_wall_wall_term: bad arguments");
  if (walls->n == 0) return SPH_OK;
  k_wall_wall_term<<<grid_for(walls->n, 128), 128, 0, as_stream(stream)>>>(to_walls(walls), grid, to_params(params),
                                                                           term);
  SPH_CHECK_LAUNCH("dfsph_wall_wall_term");
  return SPH_OK;
}

sph_status_t sph_dfsph_densities(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, const float* rho_fluid, const sph_dfsph_buffers* bufs,
                                 void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && rho_fluid && bufs, "dfsph_densities: bad arguments");
  cudaStream_t st = as_stream(stream);
  const FluidView F = to_fluid(fluid);
  const WallView W = to_walls(walls);
  const SphParams P = to_params(params);
  const DfsphBufs B = to_bufs(bufs);
  if (fluid->n > 0) k_dfsph_fluid_density<<<grid_for(fluid->n, 128), 128, 0, st>>>(F, W, grid, P, rho_fluid, B);
  if (walls->n > 0) k_dfsph_wall_density<<<grid_for(walls->n, 128), 128, 0, st>>>(F, W, grid, P, B);
  SPH_CHECK_LAUNCH("dfsph_densities");
  return SPH_OK;
}

sph_status_t sph_dfsph_solve(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                             const sph_params* params, const sph_dfsph_buffers* bufs, const float* acc_in,
                             const float* dt, int32_t density, int32_t* status, void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && bufs && acc_in && dt, "dfsph_solve: bad arguments");
  const int n = (int)fluid->n;
  if (n == 0) return SPH_OK;
  cudaStream_t st = as_stream(stream);
  SPH_REQUIRE(bufs->records && (reinterpret_cast<uintptr_t>(bufs->records) & 15) == 0,
              "dfsph_solve: records must be a 16-byte aligned array of 9 n floats");
  FluidView F = to_fluid(fluid);
  WallView W = to_walls(walls);
  SphParams P = to_params(params);
  DfsphBufs B = to_bufs(bufs, n);
  k_dfsph_vstar<<<grid_for(n, 256), 256, 0, st>>>(F, P, B, reinterpret_cast<const float2*>(acc_in), dt);
  k_dfsph_prepare<<<grid_for(n, 128), 128, 0, st>>>(F, W, grid, P, B, dt, density);
  if (density && W.n > 0) k_dfsph_wall_prepare<<<grid_for(W.n, 128), 128, 0, st>>>(F, W, grid, P, B, dt);
  SPH_CHECK_LAUNCH("dfsph_solve(prepare)");
  int dev = 0;
  cudaError_t de = cudaGetDevice(&dev);
  if (de != cudaSuccess || dev < 0 || dev >= kCoopMaxDevices) {
    set_error("dfsph_solve(device)", de);
    return SPH_ERR_CUDA;
  }
  int coop_blocks = 0;
  {
    std::lock_guard<std::mutex> lock(g_coop_mu);
    if (g_coop_blocks[dev] == 0) {
      int per_sm = 0, sms = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dfsph_solve, 256, 0);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess || per_sm < 1 || sms < 1) {
        set_error("dfsph_solve(occupancy)", e);
        return SPH_ERR_CUDA;
      }
      g_coop_blocks[dev] = std::min(per_sm, 8) * sms;
    }
    coop_blocks = g_coop_blocks[dev];
  }
  int blocks = std::min(coop_blocks, (int)sph_dfsph_partials_count());
  blocks = std::min(blocks, std::max(1, (n + 255) / 256));
  int density_i = density;
  int min_it = density ? params->min_density_iters : params->min_divergence_iters;
  int max_it = density ? params->max_density_iters : params->max_divergence_iters;
  float thr = density ? params->density_threshold : params->divergence_threshold;
  float omega_f = params->omega_fluid;
  float omega_b = params->omega_boundary;
  void* args[] = {&F, &W, (void*)&grid, &P, &B, (void*)&dt, &density_i, &min_it, &max_it, &thr, &omega_f, &omega_b,
                  (void*)&status};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_dfsph_solve, blocks, 256, args, 0, st);
  if (e != cudaSuccess) {
    set_error("dfsph_solve(cooperative launch)", e);
    return SPH_ERR_CUDA;
  }
  return SPH_OK;
}

sph_status_t sph_dfsph_viscosity(const sph_fluid_view* fluid, const sph_wall_view* walls, const sph_grid* grid,
                                 const sph_params* params, const sph_dfsph_buffers* bufs, float* acc, void* stream) {
  SPH_VIEW_CHECK(fluid);
  SPH_VIEW_CHECK(walls);
  SPH_REQUIRE(grid && params && bufs && acc, "dfsph_viscosity: bad arguments");
  if (fluid->n == 0) return SPH_OK;
  SPH_REQUIRE(bufs->records && (reinterpret_cast<uintptr_t>(bufs->records) & 15) == 0,
              "dfsph_viscosity: records must be a 16-byte aligned array of 9 n floats");
  const FluidView F = to_fluid(fluid);
  const SphParams P = to_params(params);
  const DfsphBufs B = to_bufs(bufs, fluid->n);
  cudaStream_t st = as_stream(stream);
  k_dfsph_visc_records<<<grid_for(fluid->n, 256), 256, 0, st>>>(F, P, B);
  k_dfsph_viscosity<<<grid_for(fluid->n, 128), 128, 0, st>>>(F, to_walls(walls), grid, P, B,
                                                             reinterpret_cast<float2*>(acc));
  SPH_CHECK_LAUNCH("dfsph_viscosity");
  return SPH_OK;
}

sph_status_t sph_add_float2(int64_t n, const float* b, float* a, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && a && b, "add_float2: bad arguments");
  if (n == 0) return SPH_OK;
  k_add2<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((int)n, reinterpret_cast<const float2*>(b),
                                                           reinterpret_cast<float2*>(a));
  SPH_CHECK_LAUNCH("add_float2");
  return SPH_OK;
}

sph_status_t sph_fill_float2(int64_t n, float x, float y, float* a, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && a, "fill_float2: bad arguments");
  if (n == 0) return SPH_OK;
  k_fill2<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((int)n, x, y, reinterpret_cast<float2*>(a));
  SPH_CHECK_LAUNCH("fill_float2");
  return SPH_OK;
}

size_t sph_dt_scratch_bytes(void) { return (size_t)2 * kNumSMs * 2 * sizeof(float); }

sph_status_t sph_update_dt(int64_t n, const float* v, const float* acc, float support, float kinematic, float cfl,
                           float c0, int32_t acoustic_from_c0, float dt_min, float dt_max, float* dt, void* scratch,
                           size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n > 0 && n < (1LL << 31) && v && acc && dt && kinematic > 0.f, "update_dt: bad arguments");
  if (!scratch || scratch_bytes < sph_dt_scratch_bytes()) {
    set_error_text("update_dt: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  int parts = (int)std::min<int64_t>(2 * kNumSMs, (n + 255) / 256);
  float* part = static_cast<float*>(scratch);
  k_dt_partials<<<parts, 256, 0, st>>>((int)n, reinterpret_cast<const float2*>(v), reinterpret_cast<const float2*>(acc),
                                       support, part);
  k_dt_final<<<1, 32, 0, st>>>(parts, part, support, kinematic, cfl, c0, acoustic_from_c0, dt_min, dt_max, dt);
  SPH_CHECK_LAUNCH("update_dt");
  return SPH_OK;
}

}  // extern "C"
