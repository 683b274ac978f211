// Solid-wall terms of src/modules/solidBoundary.py over the reference's own wall pair lists,
// for callers of the BoundaryModule interface (mDBC walls for deltaSPH, PBSPH walls for
// DFSPH).  Pairs (b, f) are ordered by wall (boundaryToFluidNeighbors / ghostToFluidNeighbors
// from searchExisting) with e = (x_b - x_f) / r and q = r / h; fluid-side sums walk the same
// pairs grouped by fluid particle (sph_transpose_pairs), so every sum is a gather in a fixed
// order: no atomics in the sums.
//
// Reference lines: wall density (summation) :522-549, mDBC :561-617, continuity :746-770,
// L :676-694, <grad rho> :695-717, pressure acceleration :846-896, velocity diffusion
// :820-844, DFSPH alpha :443-479, source :481-520, pressure sum :405-441, acceleration
// :310-403.
#include "sph_math.cuh"

namespace sph {

struct WallTermIn {
  const int32_t* woff;
  const int64_t* rows;
  const int64_t* cols;
  const float2* dist;
  const float* radial;
  const int32_t* foff;
  const int32_t* fpairs;
  const float2* pos;
  const float2* vel;
  const float* rho;
  const float* area;
  const float* volume;
  const float* pressure;
  const float4* L;
  const float* aact;
  const float2* pred_accel;
  const float2* pred_vel;
  const float2* wpos;
  const float2* wghost;
  const float* warea;
  const float* wrho;
  const float* wvol;
  const float* wp;
  const float* waact;
  const float* wterm;
  float dt;
  int n, nb;
};

// Fluid-side wall sums: particle f over its wall pairs.
template <int kTerm>
__global__ void __launch_bounds__(128) k_wall_fluid_term(WallTermIn in, SphParams P, float* __restrict__ out,
                                                         int accumulate) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= in.n) return;
  const int t0 = in.foff[f], t1 = in.foff[f + 1];
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  const float2 xf = in.pos ? in.pos[f] : make_float2(0.f, 0.f);
  const float2 uf = in.vel ? in.vel[f] : make_float2(0.f, 0.f);
  const float rhof = in.rho ? in.rho[f] * P.rho0 : 0.f;
  const float pf = in.pressure ? in.pressure[f] : 0.f;
  const float4 Lf = in.L ? in.L[f] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 vs = in.pred_vel ? in.pred_vel[f] : make_float2(0.f, 0.f);
  const float2 af = in.pred_accel ? in.pred_accel[f] : make_float2(0.f, 0.f);
  for (int t = t0; t < t1; ++t) {
    const int k = in.fpairs[t];
    const int b = (int)in.rows[k];
    if ((unsigned)b >= (unsigned)in.nb) continue;   // a malformed pair list reads nothing out of range
    const float2 e = in.dist[k];          // (x_b - x_f) / r
    const float q = in.radial[k];
    if (kTerm == SPH_WALL_DENSITY) {
      s0 += kW(q, P.c_w) * in.warea[b];
      continue;
    }
    if (kTerm >= SPH_WALL_DFSPH_ALPHA) {
      const float gs = kGS(q, P.c_s);
      const float sx = e.x * gs, sy = e.y * gs;   // spiky gradient with e_bf
      const float ab = in.waact[b];
      if (kTerm == SPH_WALL_DFSPH_ALPHA) {
        s0 += ab * sx;
        s1 += ab * sy;
        s2 += ab * ab / (in.warea[b] * P.rho0) * (sx * sx + sy * sy);
      } else if (kTerm == SPH_WALL_DFSPH_SOURCE) {
        s0 += ab * ((0.f - vs.x) * sx + (0.f - vs.y) * sy);
      } else if (kTerm == SPH_WALL_DFSPH_PRESSURE_SUM) {
        const float fac = in.dt * in.dt * ab;
        s0 += fac * af.x * (-sx) + fac * af.y * (-sy);
      } else if (kTerm == SPH_WALL_DFSPH_ACCEL) {
        const float rb = in.wrho[b] * P.rho0;
        const float c = -(in.warea[b] * P.rho0) * (pf / (rhof * rhof) + in.wp[b] / (rb * rb));
        s0 += c * (-sx);
        s1 += c * (-sy);
      }
      continue;
    }
    // deltaSPH terms: gradW on the fluid side, gb = e_fb kGW(q) = -e kGW(q)
    const float gw = kGW(q, P.c_g);
    const float gx = -e.x * gw, gy = -e.y * gw;
    const float Vb = in.wvol[b], rhob = in.wrho[b] * P.rho0;
    const float2 xb = in.wpos[b];
    const float rx = xb.x - xf.x, ry = xb.y - xf.y;   // x_b - x_f
    if (kTerm == SPH_WALL_DPDT) {
      s0 += ((0.f - uf.x) * gx + (0.f - uf.y) * gy) * Vb * rhob;
    } else if (kTerm == SPH_WALL_NORMALIZATION) {
      s0 += Vb * rx * gx;
      s1 += Vb * rx * gy;
      s2 += Vb * ry * gx;
      s3 += Vb * ry * gy;
    } else if (kTerm == SPH_WALL_RENORMALIZED_GRADIENT) {
      const float ax = Lf.x * gx + Lf.y * gy, ay = Lf.z * gx + Lf.w * gy;
      const float c = (rhob - rhof) * Vb * 2.0f;
      s0 += c * ax;
      s1 += c * ay;
    } else if (kTerm == SPH_WALL_PRESSURE_ACCEL) {
      const float c = (pf + in.wp[b]) * Vb;
      s0 += c * gx;
      s1 += c * gy;
    } else if (kTerm == SPH_WALL_VELOCITY_DIFFUSION) {
      const float r2 = rx * rx + ry * ry + P.eps;
      const float pij = fminf((0.f - uf.x) * rx + (0.f - uf.y) * ry, 0.f) / r2;
      const float c = pij * Vb * rhob / (rhof + rhob);
      s0 += c * gx;
      s1 += c * gy;
    }
  }
  int width = 1;
  float r0 = s0, r1 = s1;
  switch (kTerm) {
    case SPH_WALL_DPDT: r0 = -s0; break;
    case SPH_WALL_NORMALIZATION: width = 4; break;
    case SPH_WALL_RENORMALIZED_GRADIENT: r0 = -s0; r1 = -s1; width = 2; break;
    case SPH_WALL_PRESSURE_ACCEL: r0 = -s0 / rhof; r1 = -s1 / rhof; width = 2; break;
    case SPH_WALL_VELOCITY_DIFFUSION: r0 = P.visc_k * s0; r1 = P.visc_k * s1; width = 2; break;
    case SPH_WALL_DFSPH_ALPHA: width = 4; break;
    case SPH_WALL_DFSPH_SOURCE: r0 = -in.dt * s0; break;
    case SPH_WALL_DFSPH_ACCEL: width = 2; break;
    default: break;
  }
  if (width == 4) {
    float4* o = reinterpret_cast<float4*>(out) + f;
    float4 v = kTerm == SPH_WALL_DFSPH_ALPHA ? make_float4(s0, s1, s2, 0.f) : make_float4(s0, s1, s2, s3);
    if (accumulate) {
      const float4 a = *o;
      v = make_float4(a.x + v.x, a.y + v.y, a.z + v.z, a.w + v.w);
    }
    *o = v;
  } else if (width == 2) {
    float2* o = reinterpret_cast<float2*>(out) + f;
    if (accumulate) {
      const float2 a = *o;
      r0 += a.x;
      r1 += a.y;
    }
    *o = make_float2(r0, r1);
  } else {
    out[f] = accumulate ? out[f] + r0 : r0;
  }
}

// Wall-side sums: wall b over its fluid pairs.
template <int kTerm>
__global__ void __launch_bounds__(128) k_wall_side_term(WallTermIn in, SphParams P, float* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= in.nb) return;
  const int k0 = in.woff[b], k1 = in.woff[b + 1];
  if (kTerm == SPH_BWALL_MDBC) {
    // ghost g of wall b against the fluid (e = (x_g - x_f)/r), solidBoundary.py:561-617
    const float2 xg = in.wghost[b];
    float nom = 0, den = 0, gx = 0, gy = 0, vgx = 0, vgy = 0, px = 0, py = 0;
    float m00 = 0, m01 = 0, m10 = 0, m11 = 0;
    const int cnt = k1 - k0;
    for (int k = k0; k < k1; ++k) {
      const int f = (int)in.cols[k];
      if ((unsigned)f >= (unsigned)in.n) continue;
      const float2 e = in.dist[k];
      const float q = in.radial[k];
      const float w = kW(q, P.c_w);
      const float gw = kGW(q, P.c_g);
      const float ggx = e.x * gw, ggy = e.y * gw;
      const float mass = in.area[f] * P.rho0;
      const float Vf = in.volume[f];
      const float2 xf = in.pos[f];
      const float xx = xf.x - xg.x, xy = xf.y - xg.y;
      nom += mass * w;
      den += Vf * w;
      gx += mass * ggx;
      gy += mass * ggy;
      vgx += Vf * ggx;
      vgy += Vf * ggy;
      px += Vf * w * xx;
      py += Vf * w * xy;
      m00 += Vf * xx * ggx;
      m01 += Vf * xx * ggy;
      m10 += Vf * xy * ggx;
      m11 += Vf * xy * ggy;
    }
    double rho_b = 1.0;
    if (cnt > 0) rho_b = ((double)nom / (double)den) / P.rho0;
    if (cnt > 10) {
      const double A[3][3] = {{den, px, py}, {vgx, m00, m01}, {vgy, m10, m11}};
      const double bb[3] = {nom, gx, gy};
      double res[3];
      pinv3_solve(A, bb, res);
      const float2 xb = in.wpos[b];
      rho_b = (res[0] + ((double)xb.x - xg.x) * res[1] + ((double)xb.y - xg.y) * res[2]) / P.rho0;
    }
    out[b] = (float)fmax(rho_b, 1.0);
    return;
  }
  float s = 0.f;
  for (int k = k0; k < k1; ++k) {
    const int f = (int)in.cols[k];
    if ((unsigned)f >= (unsigned)in.n) continue;
    const float q = in.radial[k];
    if (kTerm == SPH_BWALL_DENSITY) {
      s += kW(q, P.c_w) * in.area[f];
      continue;
    }
    const float2 e = in.dist[k];
    const float gs = kGS(q, P.c_s);
    const float sx = e.x * gs, sy = e.y * gs;
    if (kTerm == SPH_BWALL_DFSPH_ALPHA) {
      const float a = in.aact[f];
      s += a * a / (in.area[f] * P.rho0) * (sx * sx + sy * sy);
    } else if (kTerm == SPH_BWALL_DFSPH_SOURCE) {
      const float2 vs = in.pred_vel[f];
      s += in.aact[f] * ((0.f - vs.x) * sx + (0.f - vs.y) * sy);
    } else if (kTerm == SPH_BWALL_DFSPH_PRESSURE_SUM) {
      const float2 a = in.pred_accel[f];
      const float fac = in.dt * in.dt * in.aact[f];
      s += fac * a.x * (-sx) + fac * a.y * (-sy);
    }
  }
  if (kTerm == SPH_BWALL_DENSITY) {
    out[b] = fminf(in.wterm[b] + s, 1.0f);
  } else if (kTerm == SPH_BWALL_DFSPH_ALPHA) {
    const float h = P.h;
    out[b] = fminf(-in.dt * in.dt * in.waact[b] * s, -0.01f * 0.01f * h * h);
  } else if (kTerm == SPH_BWALL_DFSPH_SOURCE) {
    out[b] = 1.0f - in.wrho[b] + (-in.dt) * s;
  } else {
    out[b] = s;
  }
}

// Pseudo-inverse of the symmetric 2x2 matrix [[a, b], [b, d]] with torch.linalg.pinv's
// default cut-off for float32 input (singular values at or below 2 FLT_EPSILON sigma_max are
// dropped), in double: (o00, o01, o11).
__device__ inline void pinv_sym2(double a, double b, double d, double o[3]) {
  o[0] = o[1] = o[2] = 0.0;
  const double h = 0.5 * (a + d);
  const double r = sqrt(0.25 * (a - d) * (a - d) + b * b);
  const double l[2] = {h + r, h - r};
  const double smax = fmax(fabs(l[0]), fabs(l[1]));
  const double tol = 2.0 * 1.1920928955078125e-07 * smax;
  // eigenvector of l[0]: the larger of (l0 - d, b) and (b, l0 - a); the other one is orthogonal
  double vx = l[0] - d, vy = b;
  const double ux = b, uy = l[0] - a;
  if (ux * ux + uy * uy > vx * vx + vy * vy) {
    vx = ux;
    vy = uy;
  }
  double nv = sqrt(vx * vx + vy * vy);
  if (!(nv > 0.0)) {   // b == 0 and a == d: any basis
    vx = 1.0;
    vy = 0.0;
    nv = 1.0;
  }
  vx /= nv;
  vy /= nv;
  const double ev[2][2] = {{vx, vy}, {-vy, vx}};
  for (int k = 0; k < 2; ++k) {
    if (!(fabs(l[k]) > tol)) continue;
    const double il = 1.0 / l[k];
    o[0] += il * ev[k][0] * ev[k][0];
    o[1] += il * ev[k][0] * ev[k][1];
    o[2] += il * ev[k][1] * ev[k][1];
  }
}

// Wall pressures of the MLS schemes, wall b over its ghost pair list (solidBoundary.py:772-808).
// The moment sums run in float in pair order, as the reference's float32 scatters do; the
// small systems are solved in double with torch.linalg.pinv's cut-off (pinv3_solve,
// pinv_sym2).  Walls whose fluid neighbors lie almost on a line give ill-conditioned systems:
// there the reference's own float32 and float64 runs disagree by more than the pressure.
template <int kTerm>
__global__ void __launch_bounds__(128) k_wall_mls_pressure(WallTermIn in, SphParams P, float* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= in.nb) return;
  const int k0 = in.woff[b], k1 = in.woff[b + 1];
  if (kTerm == SPH_BWALL_MLS_PRESSURE) {
    // prepareMLSBoundaries: Shepard centre d of the neighbors (weights W_j V_j), then the
    // centred moment matrix; evalMLSBoundaries: p_b = alpha + (x_b - d) . pinv(M) sum_j xbar_j k_j p_j
    const float2 xb = in.wpos[b];
    float nx = 0.f, ny = 0.f, den = 0.f;
    for (int k = k0; k < k1; ++k) {
      const int f = (int)in.cols[k];
      if ((unsigned)f >= (unsigned)in.n) continue;
      const float kk = kW(in.radial[k], P.c_w) * in.volume[f];
      const float2 xf = in.pos[f];
      nx += kk * xf.x;
      ny += kk * xf.y;
      den += kk;
    }
    const float2 d = den > 1e-9f ? make_float2(nx / den, ny / den) : xb;
    float m00 = 0.f, m01 = 0.f, m11 = 0.f, vx = 0.f, vy = 0.f, ap = 0.f, as = 0.f;
    for (int k = k0; k < k1; ++k) {
      const int f = (int)in.cols[k];
      if ((unsigned)f >= (unsigned)in.n) continue;
      const float kk = kW(in.radial[k], P.c_w) * in.volume[f];
      const float2 xf = in.pos[f];
      const float bx = xf.x - d.x, by = xf.y - d.y;
      const float pf = in.pressure[f];
      m00 += bx * bx * kk;
      m01 += bx * by * kk;
      m11 += by * by * kk;
      vx += bx * kk * pf;
      vy += by * kk * pf;
      ap += pf * kk;
      as += kk;
    }
    double Mi[3];
    pinv_sym2(m00, m01, m11, Mi);
    const double alpha = as > 1e-6f ? (double)(ap / as) : (double)ap;
    const double cx = Mi[0] * vx + Mi[1] * vy, cy = Mi[1] * vx + Mi[2] * vy;
    const double pb = alpha + ((double)xb.x - d.x) * cx + ((double)xb.y - d.y) * cy;
    out[b] = pb < 0.0 ? 0.f : (float)pb;
    return;
  }
  // precomputeMLS at the ghost (ghostMLS) or the wall position (deltaMLS)
  const float2 xq = kTerm == SPH_BWALL_GHOST_MLS_PRESSURE ? in.wghost[b] : in.wpos[b];
  float m00 = 0.f, m01 = 0.f, m02 = 0.f, m11 = 0.f, m12 = 0.f, m22 = 0.f;
  for (int k = k0; k < k1; ++k) {
    const int f = (int)in.cols[k];
    if ((unsigned)f >= (unsigned)in.n) continue;
    const float t = in.area[f] / (in.rho[f] * P.rho0) * kW(in.radial[k], P.c_w);
    const float2 xf = in.pos[f];
    const float dx = xf.x - xq.x, dy = xf.y - xq.y;
    m00 += 2.0f * t;
    m01 += 2.0f * dx * t;
    m02 += 2.0f * dy * t;
    m11 += 2.0f * (dx * dx) * t;
    m12 += 2.0f * (dx * dy) * t;
    m22 += 2.0f * (dy * dy) * t;
  }
  const double A[3][3] = {{m00, m01, m02}, {m01, m11, m12}, {m02, m12, m22}};
  const double e1[3] = {1.0, 0.0, 0.0};
  double c[3];
  pinv3_solve(A, e1, c);
  float s = 0.f;
  for (int k = k0; k < k1; ++k) {
    const int f = (int)in.cols[k];
    if ((unsigned)f >= (unsigned)in.n) continue;
    const float w = kW(in.radial[k], P.c_w);
    const float V = in.area[f] / (in.rho[f] * P.rho0);
    const float2 xf = in.pos[f];
    const float dx = xf.x - xq.x, dy = xf.y - xq.y;
    const float pg = (float)(c[0] + c[1] * dx + c[2] * dy) * w * V;
    s += pg * in.pressure[f];
  }
  out[b] = s;
}

// Stable grouping of pairs by column: counts, offsets, scatter, then every row restored to
// ascending pair order (rows are short: the walls within h of one particle).
__global__ void k_pair_col_count(const int64_t* __restrict__ cols, int64_t P, int64_t n,
                                 int32_t* __restrict__ counts) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < P && cols[k] >= 0 && cols[k] < n) atomicAdd(counts + cols[k], 1);
}

__global__ void k_pair_col_scatter(const int64_t* __restrict__ cols, int64_t P, int64_t n,
                                   const int32_t* __restrict__ offsets, int32_t* __restrict__ cursor,
                                   int32_t* __restrict__ pairs) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P) return;
  const int64_t c = cols[k];
  if (c < 0 || c >= n) return;   // columns out of range are left out of the grouping
  pairs[offsets[c] + atomicAdd(cursor + c, 1)] = (int32_t)k;
}

__global__ void k_pair_col_order(int n, const int32_t* __restrict__ offsets, int32_t* __restrict__ pairs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int b = offsets[c], e = offsets[c + 1];
  for (int t = b + 1; t < e; ++t) {
    const int32_t x = pairs[t];
    int u = t;
    while (u > b && pairs[u - 1] > x) {
      pairs[u] = pairs[u - 1];
      --u;
    }
    pairs[u] = x;
  }
}

}  // namespace sph

using namespace sph;

static WallTermIn to_wall_terms(const sph_wall_terms_in* in) {
  WallTermIn t;
  t.woff = in->wall_offsets;
  t.rows = in->rows;
  t.cols = in->cols;
  t.dist = reinterpret_cast<const float2*>(in->dist);
  t.radial = in->radial;
  t.foff = in->fluid_offsets;
  t.fpairs = in->fluid_pairs;
  t.pos = reinterpret_cast<const float2*>(in->pos);
  t.vel = reinterpret_cast<const float2*>(in->vel);
  t.rho = in->rho;
  t.area = in->area;
  t.volume = in->volume;
  t.pressure = in->pressure;
  t.L = reinterpret_cast<const float4*>(in->L);
  t.aact = in->actual_area;
  t.pred_accel = reinterpret_cast<const float2*>(in->pred_accel);
  t.pred_vel = reinterpret_cast<const float2*>(in->pred_vel);
  t.wpos = reinterpret_cast<const float2*>(in->wall_pos);
  t.wghost = reinterpret_cast<const float2*>(in->wall_ghost);
  t.warea = in->wall_area;
  t.wrho = in->wall_rho;
  t.wvol = in->wall_volume;
  t.wp = in->wall_pressure;
  t.waact = in->wall_actual_area;
  t.wterm = in->wall_term;
  t.dt = (float)in->dt;
  t.n = (int)in->n;
  t.nb = (int)in->nb;
  return t;
}

extern "C" {

size_t sph_transpose_pairs_scratch_bytes(int64_t n) {
  return 2 * (size_t)(n > 0 ? n : 1) * sizeof(int32_t) + sph_scan_scratch_bytes(n) + 256;
}

sph_status_t sph_transpose_pairs(const int64_t* cols, int64_t num_pairs, int64_t n, int32_t* col_offsets,
                                 int32_t* pairs, void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(num_pairs >= 0 && num_pairs < (1LL << 31) && n >= 0 && n < (1LL << 31) && col_offsets &&
                  (num_pairs == 0 || (cols && pairs)),
              "transpose_pairs: bad arguments");
  if (!scratch || scratch_bytes < sph_transpose_pairs_scratch_bytes(n)) {
    set_error_text("transpose_pairs: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  int32_t* counts = static_cast<int32_t*>(scratch);
  int32_t* cursor = counts + (n > 0 ? n : 1);
  char* scan_scratch = reinterpret_cast<char*>(cursor + (n > 0 ? n : 1));
  const size_t scan_bytes = scratch_bytes - 2 * (size_t)(n > 0 ? n : 1) * sizeof(int32_t);
  if (n == 0) {
    cudaMemsetAsync(col_offsets, 0, sizeof(int32_t), st);
    SPH_CHECK_LAUNCH("transpose_pairs");
    return SPH_OK;
  }
  cudaMemsetAsync(counts, 0, 2 * (size_t)n * sizeof(int32_t), st);
  if (num_pairs > 0)
    k_pair_col_count<<<grid_for(num_pairs, 256), 256, 0, st>>>(cols, num_pairs, n, counts);
  sph_status_t s = sph_exclusive_scan_i32(counts, col_offsets, n, scan_scratch, scan_bytes, stream);
  if (s != SPH_OK) return s;
  if (num_pairs > 0) {
    k_pair_col_scatter<<<grid_for(num_pairs, 256), 256, 0, st>>>(cols, num_pairs, n, col_offsets, cursor, pairs);
    k_pair_col_order<<<grid_for(n, 128), 128, 0, st>>>((int)n, col_offsets, pairs);
  }
  SPH_CHECK_LAUNCH("transpose_pairs");
  return SPH_OK;
}

sph_status_t sph_wall_term(int32_t term, const sph_wall_terms_in* in, const sph_params* params, float* out,
                           int32_t accumulate, void* stream) {
  SPH_REQUIRE(in && params && out && params->support > 0.f && in->n >= 0 && in->n < (1LL << 31) && in->nb >= 0 &&
                  in->nb < (1LL << 31),
              "wall_term: bad arguments");
  SPH_REQUIRE(in->rows && in->cols && in->radial && (term == SPH_WALL_DENSITY || term == SPH_BWALL_DENSITY ||
                                                     in->dist),
              "wall_term: needs the pair list");
  const bool wall_side = term >= SPH_BWALL_DENSITY;
  SPH_REQUIRE(wall_side ? in->wall_offsets != nullptr : (in->fluid_offsets && in->fluid_pairs),
              "wall_term: needs the pair offsets of the summing side");
  // the arrays each term reads
  bool ok = true;
  switch (term) {
    case SPH_WALL_DENSITY: ok = in->wall_area; break;
    case SPH_WALL_DPDT: ok = in->vel && in->wall_volume && in->wall_rho; break;
    case SPH_WALL_NORMALIZATION: ok = in->pos && in->wall_pos && in->wall_volume; break;
    case SPH_WALL_RENORMALIZED_GRADIENT: ok = in->L && in->rho && in->wall_rho && in->wall_volume; break;
    case SPH_WALL_PRESSURE_ACCEL: ok = in->rho && in->pressure && in->wall_pressure && in->wall_volume; break;
    case SPH_WALL_VELOCITY_DIFFUSION:
      ok = in->pos && in->vel && in->rho && in->wall_pos && in->wall_volume && in->wall_rho;
      break;
    case SPH_WALL_DFSPH_ALPHA: ok = in->wall_actual_area && in->wall_area; break;
    case SPH_WALL_DFSPH_SOURCE: ok = in->pred_vel && in->wall_actual_area; break;
    case SPH_WALL_DFSPH_PRESSURE_SUM: ok = in->pred_accel && in->wall_actual_area; break;
    case SPH_WALL_DFSPH_ACCEL: ok = in->rho && in->pressure && in->wall_area && in->wall_rho && in->wall_pressure; break;
    case SPH_BWALL_DENSITY: ok = in->area && in->wall_term; break;
    case SPH_BWALL_MDBC: ok = in->area && in->volume && in->pos && in->wall_ghost && in->wall_pos; break;
    case SPH_BWALL_DFSPH_ALPHA: ok = in->actual_area && in->area && in->wall_actual_area; break;
    case SPH_BWALL_DFSPH_SOURCE: ok = in->actual_area && in->pred_vel && in->wall_rho; break;
    case SPH_BWALL_DFSPH_PRESSURE_SUM: ok = in->actual_area && in->pred_accel; break;
    case SPH_BWALL_GHOST_MLS_PRESSURE: ok = in->pos && in->area && in->rho && in->pressure && in->wall_ghost; break;
    case SPH_BWALL_DELTA_MLS_PRESSURE: ok = in->pos && in->area && in->rho && in->pressure && in->wall_pos; break;
    case SPH_BWALL_MLS_PRESSURE: ok = in->pos && in->volume && in->pressure && in->wall_pos; break;
    default: break;
  }
  SPH_REQUIRE(ok, "wall_term: an array this term reads is missing");
  const WallTermIn t = to_wall_terms(in);
  const SphParams P = to_params(params);
  cudaStream_t st = as_stream(stream);
  const int nbf = grid_for(in->n, 128), nbw = grid_for(in->nb, 128);
  switch (term) {
#define SPH_WF(T) \
  case T:         \
    if (in->n) k_wall_fluid_term<T><<<nbf, 128, 0, st>>>(t, P, out, accumulate); \
    break;
#define SPH_WB(T) \
  case T:         \
    if (in->nb) k_wall_side_term<T><<<nbw, 128, 0, st>>>(t, P, out); \
    break;
    SPH_WF(SPH_WALL_DENSITY)
    SPH_WF(SPH_WALL_DPDT)
    SPH_WF(SPH_WALL_NORMALIZATION)
    SPH_WF(SPH_WALL_RENORMALIZED_GRADIENT)
    SPH_WF(SPH_WALL_PRESSURE_ACCEL)
    SPH_WF(SPH_WALL_VELOCITY_DIFFUSION)
    SPH_WF(SPH_WALL_DFSPH_ALPHA)
    SPH_WF(SPH_WALL_DFSPH_SOURCE)
    SPH_WF(SPH_WALL_DFSPH_PRESSURE_SUM)
    SPH_WF(SPH_WALL_DFSPH_ACCEL)
    SPH_WB(SPH_BWALL_DENSITY)
    SPH_WB(SPH_BWALL_MDBC)
    SPH_WB(SPH_BWALL_DFSPH_ALPHA)
    SPH_WB(SPH_BWALL_DFSPH_SOURCE)
    SPH_WB(SPH_BWALL_DFSPH_PRESSURE_SUM)
#define SPH_WM(T) \
  case T:         \
    if (in->nb) k_wall_mls_pressure<T><<<nbw, 128, 0, st>>>(t, P, out); \
    break;
    SPH_WM(SPH_BWALL_GHOST_MLS_PRESSURE)
    SPH_WM(SPH_BWALL_DELTA_MLS_PRESSURE)
    SPH_WM(SPH_BWALL_MLS_PRESSURE)
#undef SPH_WM
#undef SPH_WF
#undef SPH_WB
    default:
      set_error_text("wall_term: unknown term");
      return SPH_ERR_INVALID_ARGUMENT;
  }
  SPH_CHECK_LAUNCH("wall_term");
  return SPH_OK;
}

}  // extern "C"
