// One SPH summation term at a time over the reference's own pair list, for the Module
// interface (densityModule.evaluate, momentumModule.computeDpDt, ...): the caller holds the
// simulationState arrays in original particle order and the (i, j)-ordered pairs
// fluidNeighbors with fluidDistances (unit vectors e_ij, zero below the gradient threshold)
// and fluidRadialDistances (q_ij = r_ij / h).  One thread gathers one row i; there are no
// atomics and each row is summed in pair order.
//
// Reference formulas (V = volume, rho = rho~ rest_density, gradW_ij = e_ij kGW(q_ij)):
//   density        src/modules/density.py:26-30          sum W(q) A_j
//   divergence     src/modules/momentum.py:31-38         -sum ((u_j - u_i) . gradW) V_j rho_j
//   MOG diffusion  src/modules/densityDiffusion.py:74-82  h delta c0 sum 2 (rho_j - rho_i)/(|x_ji|^2+eps) (x_ji . gradW) V_j
//   L              densityDiffusion.py:30-44              sum V_j (x_j - x_i) (x) gradW
//   <grad rho>     densityDiffusion.py:45-61              -sum 2 (rho_j - rho_i) V_j (L_i gradW)
//   deltaSPH diff. densityDiffusion.py:63-71              h delta c0 sum [2 (rho_j - rho_i)/(|x_ji|^2+eps) x_ji - (g_i + g_j)] . gradW V_j
//   pressure acc.  src/modules/pressure.py:31-38          -1/rho_i sum (p_i + p_j) V_j gradW
//   art. viscosity src/modules/diffusion.py:30-44         h alpha c0 sum pi_ij V_j rho_j/(rho_i + rho_j) gradW
//   laminar        src/modules/laminar.py:30-46           -sum 4 m_j (mu_i + mu_j)(r . gradW)/((rho_i + rho_j)^2 (|r|^2+eps)) (u_i - u_j),
//                                                         r = x_j - x_i, mu_i = mu_j = rho_i nu (the reference's indices)
#include "sph_math.cuh"

namespace sph {

struct TermIn {
  const int32_t* offsets;
  const int64_t* cols;
  const float2* dist;
  const float* radial;
  const float2* pos;
  const float2* vel;
  const float* rho;
  const float* volume;
  const float* area;
  const float* pressure;
  const float4* L;
  const float2* grad_rho;
  const float* aact;
  const float2* pred_accel;
  const float2* pred_vel;
  float dt;
  int n;
};

// DFSPH terms of src/modules/dfsph.py over the pair list (spiky gradient S_ij = e_ij kGS(q)).
template <int kTerm>
__global__ void __launch_bounds__(128) k_dfsph_term(TermIn in, SphParams P, float* __restrict__ out, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const int k0 = in.offsets[i], k1 = in.offsets[i + 1];
  const float dt = in.dt;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  const float2 vi = kTerm == SPH_TERM_DFSPH_SOURCE ? in.pred_vel[i] : make_float2(0.f, 0.f);
  const float2 ai = kTerm == SPH_TERM_DFSPH_PRESSURE_SUM ? in.pred_accel[i] : make_float2(0.f, 0.f);
  float ppi = 0.f;
  if (kTerm == SPH_TERM_DFSPH_ACCEL) {
    const float ri = in.rho[i] * P.rho0;
    ppi = in.pressure[i] / (ri * ri);
  }
  for (int k = k0; k < k1; ++k) {
    const int j = (int)__ldg(in.cols + k);
    const float2 e = __ldg(in.dist + k);
    const float gs = kGS(__ldg(in.radial + k), P.c_s);
    const float sx = e.x * gs, sy = e.y * gs;
    if (kTerm == SPH_TERM_DFSPH_ALPHA) {
      const float aj = __ldg(in.aact + j);
      s0 += aj * sx;
      s1 += aj * sy;
      s2 += aj * aj / (__ldg(in.area + j) * P.rho0) * (sx * sx + sy * sy);
    } else if (kTerm == SPH_TERM_DFSPH_SOURCE) {
      const float2 vj = __ldg(in.pred_vel + j);
      s0 += -dt * __ldg(in.aact + j) * ((vi.x - vj.x) * sx + (vi.y - vj.y) * sy);
    } else if (kTerm == SPH_TERM_DFSPH_PRESSURE_SUM) {
      const float2 aj = __ldg(in.pred_accel + j);
      const float f = dt * dt * __ldg(in.aact + j);
      s0 += f * (ai.x - aj.x) * sx + f * (ai.y - aj.y) * sy;
    } else if (kTerm == SPH_TERM_DFSPH_ACCEL) {
      const float rj = __ldg(in.rho + j) * P.rho0;
      const float ppj = __ldg(in.pressure + j) / (rj * rj);
      const float f = -(__ldg(in.area + j) * P.rho0) * (ppi + ppj);
      s0 += f * sx;
      s1 += f * sy;
    }
  }
  if (kTerm == SPH_TERM_DFSPH_ALPHA) {
    float4* o = reinterpret_cast<float4*>(out) + i;
    float4 v = make_float4(s0, s1, s2, 0.f);
    if (accumulate) {
      const float4 a = *o;
      v = make_float4(a.x + v.x, a.y + v.y, a.z + v.z, a.w);
    }
    *o = v;
  } else if (kTerm == SPH_TERM_DFSPH_ACCEL) {
    float2* o = reinterpret_cast<float2*>(out) + i;
    if (accumulate) {
      const float2 a = *o;
      s0 += a.x;
      s1 += a.y;
    }
    *o = make_float2(s0, s1);
  } else {
    out[i] = accumulate ? out[i] + s0 : s0;
  }
}

template <int kTerm>
__global__ void __launch_bounds__(128) k_pair_term(TermIn in, SphParams P, float* __restrict__ out, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const int k0 = in.offsets[i], k1 = in.offsets[i + 1];
  const float2 xi = kTerm == SPH_TERM_DENSITY ? make_float2(0.f, 0.f) : in.pos[i];
  const float rhoi = (kTerm == SPH_TERM_DENSITY || kTerm == SPH_TERM_NORMALIZATION) ? 0.f : in.rho[i] * P.rho0;
  const float2 ui = (kTerm == SPH_TERM_DIVERGENCE || kTerm == SPH_TERM_VELOCITY_DIFFUSION || kTerm == SPH_TERM_LAMINAR)
                        ? in.vel[i]
                        : make_float2(0.f, 0.f);
  const float pi = kTerm == SPH_TERM_PRESSURE_ACCEL ? in.pressure[i] : 0.f;
  const float4 Li = kTerm == SPH_TERM_RENORMALIZED_GRADIENT ? in.L[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 gi = kTerm == SPH_TERM_DELTA_DIFFUSION ? in.grad_rho[i] : make_float2(0.f, 0.f);
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  for (int k = k0; k < k1; ++k) {
    const int j = (int)__ldg(in.cols + k);
    const float q = __ldg(in.radial + k);
    if (kTerm == SPH_TERM_DENSITY) {
      s0 += kW(q, P.c_w) * __ldg(in.area + j);
      continue;
    }
    const float2 e = __ldg(in.dist + k);
    const float gw = kGW(q, P.c_g);
    const float gx = e.x * gw, gy = e.y * gw;
    const float2 xj = __ldg(in.pos + j);
    const float rx = xj.x - xi.x, ry = xj.y - xi.y;   // x_j - x_i
    const float Vj = __ldg(in.volume + j);
    if (kTerm == SPH_TERM_NORMALIZATION) {
      s0 += rx * gx * Vj;
      s1 += rx * gy * Vj;
      s2 += ry * gx * Vj;
      s3 += ry * gy * Vj;
      continue;
    }
    const float rhoj = __ldg(in.rho + j) * P.rho0;
    if (kTerm == SPH_TERM_DIVERGENCE) {
      const float2 uj = __ldg(in.vel + j);
      s0 += ((uj.x - ui.x) * gx + (uj.y - ui.y) * gy) * Vj * rhoj;
    } else if (kTerm == SPH_TERM_MOG_DIFFUSION) {
      const float r2 = rx * rx + ry * ry + P.eps;
      const float f = 2.0f * (rhoj - rhoi) / r2;
      s0 += (f * rx * gx + f * ry * gy) * Vj;
    } else if (kTerm == SPH_TERM_RENORMALIZED_GRADIENT) {
      const float ax = Li.x * gx + Li.y * gy, ay = Li.z * gx + Li.w * gy;
      const float f = (rhoj - rhoi) * Vj * 2.0f;
      s0 += f * ax;
      s1 += f * ay;
    } else if (kTerm == SPH_TERM_DELTA_DIFFUSION) {
      const float2 gj = __ldg(in.grad_rho + j);
      const float r2 = rx * rx + ry * ry + P.eps;
      const float f = 2.0f * (rhoj - rhoi) / r2;
      const float px = f * rx - (gi.x + gj.x), py = f * ry - (gi.y + gj.y);
      s0 += (px * gx + py * gy) * Vj;
    } else if (kTerm == SPH_TERM_PRESSURE_ACCEL) {
      const float f = (pi + __ldg(in.pressure + j)) * Vj;
      s0 += f * gx;
      s1 += f * gy;
    } else if (kTerm == SPH_TERM_VELOCITY_DIFFUSION) {
      const float2 uj = __ldg(in.vel + j);
      const float r2 = rx * rx + ry * ry + P.eps;
      float pij = (uj.x - ui.x) * rx + (uj.y - ui.y) * ry;
      pij = fminf(pij, 0.f) / r2;
      const float f = pij * Vj * rhoj / (rhoi + rhoj);
      s0 += f * gx;
      s1 += f * gy;
    } else if (kTerm == SPH_TERM_LAMINAR) {
      const float2 uj = __ldg(in.vel + j);
      const float r2 = rx * rx + ry * ry + P.eps;
      const float mu = rhoi * P.kinematic;
      const float mj = rhoj * Vj;
      const float rs = rhoi + rhoj;
      const float t = 4.0f * mj * (mu + mu) * (rx * gx + ry * gy) / (rs * rs * r2);
      s0 += t * (ui.x - uj.x);
      s1 += t * (ui.y - uj.y);
    }
  }
  float r0 = s0, r1 = s1;
  int width = 1;
  switch (kTerm) {
    case SPH_TERM_DIVERGENCE: r0 = -s0; break;
    case SPH_TERM_MOG_DIFFUSION:
    case SPH_TERM_DELTA_DIFFUSION: r0 = P.diff_k * s0; break;
    case SPH_TERM_NORMALIZATION: width = 4; break;
    case SPH_TERM_RENORMALIZED_GRADIENT: r0 = -s0; r1 = -s1; width = 2; break;
    case SPH_TERM_PRESSURE_ACCEL: {
      const float ir = -1.0f / rhoi;
      r0 = ir * s0;
      r1 = ir * s1;
      width = 2;
      break;
    }
    case SPH_TERM_VELOCITY_DIFFUSION: r0 = P.visc_k * s0; r1 = P.visc_k * s1; width = 2; break;
    case SPH_TERM_LAMINAR: r0 = -s0; r1 = -s1; width = 2; break;
    default: break;
  }
  if (width == 4) {
    float4* o = reinterpret_cast<float4*>(out) + i;
    float4 v = make_float4(s0, s1, s2, s3);
    if (accumulate) {
      const float4 a = *o;
      v = make_float4(a.x + v.x, a.y + v.y, a.z + v.z, a.w + v.w);
    }
    *o = v;
  } else if (width == 2) {
    float2* o = reinterpret_cast<float2*>(out) + i;
    if (accumulate) {
      const float2 a = *o;
      r0 += a.x;
      r1 += a.y;
    }
    *o = make_float2(r0, r1);
  } else {
    out[i] = accumulate ? out[i] + r0 : r0;
  }
}

// Per-particle operations of the same modules.
__global__ void k_particle_op(int op, int n, const float* __restrict__ a, const float* __restrict__ b,
                              SphParams P, float* __restrict__ out, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  switch (op) {
    case SPH_OP_TAIT: {  // pressure.py:103: rho0 c0^2 / gamma (rho~^gamma - 1)
      const float p = tait(a[i], P);
      out[i] = accumulate ? out[i] + p : p;
      break;
    }
    case SPH_OP_VOLUME: {  // density.py:54: V = A / rho~
      const float v = a[i] / b[i];
      out[i] = accumulate ? out[i] + v : v;
      break;
    }
    case SPH_OP_PINV2X2: {  // util.py:386-433 on the normalization matrix
      const float4 m = reinterpret_cast<const float4*>(a)[i];
      reinterpret_cast<float4*>(out)[i] = pinv2x2(m.x, m.y, m.z, m.w);
      break;
    }
    case SPH_OP_GRAVITY: {  // gravity.py:46-57; a = positions, out = accelerations (always added)
      const float2 x = reinterpret_cast<const float2*>(a)[i];
      float ax, ay;
      if (P.point_source) {
        float dx = x.x - P.point_cx, dy = x.y - P.point_cy;
        const float dist = sqrtf(dx * dx + dy * dy);
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
      float2* o = reinterpret_cast<float2*>(out) + i;
      const float2 c = *o;
      *o = make_float2(c.x + ax, c.y + ay);
      break;
    }
    default:
      break;
  }
}

// Row offsets of an (i, j)-ordered pair list: offsets[i] = first pair of row i
// (lower bound of i in rows), offsets[n] = P.
__global__ void k_row_offsets(const int64_t* __restrict__ rows, int64_t P, int n, int32_t* __restrict__ offsets) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  int64_t lo = 0, hi = P;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (rows[mid] < i)
      lo = mid + 1;
    else
      hi = mid;
  }
  offsets[i] = (int32_t)lo;
}

// Distances of query pairs, src/modules/neighborSearch.py:244-251: d = x_q[row] - x[col],
// r = |d|; e = d / r (0 when r < threshold); q = r / h_q[row].
__global__ void k_pair_geometry(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, int64_t P,
                                const float2* __restrict__ xq, const float2* __restrict__ xp,
                                const float* __restrict__ hq, float threshold, float2* __restrict__ dist,
                                float* __restrict__ radial) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P) return;
  const int r = rows[k], c = cols[k];
  const float2 a = xq[r], b = xp[c];
  const float dx = a.x - b.x, dy = a.y - b.y;
  const float d = sqrtf(dx * dx + dy * dy);
  dist[k] = d < threshold ? make_float2(0.f, 0.f) : make_float2(dx / d, dy / d);
  radial[k] = d / hq[r];
}

}  // namespace sph

using namespace sph;

extern "C" {

sph_status_t sph_pair_term(int32_t term, const sph_pair_terms_in* in, const sph_params* params, float* out,
                           int32_t accumulate, void* stream) {
  SPH_REQUIRE(in && params && out && params->support > 0.f && in->n >= 0 && in->n < (1LL << 31),
              "pair_term: bad arguments");
  SPH_REQUIRE(in->n == 0 || (in->offsets && in->cols && in->radial), "pair_term: needs offsets, cols, radial");
  const bool dfsph = term >= SPH_TERM_DFSPH_ALPHA && term <= SPH_TERM_DFSPH_ACCEL;
  const bool needs_geo = term != SPH_TERM_DENSITY && !dfsph;
  SPH_REQUIRE(!needs_geo || (in->dist && in->pos && in->volume), "pair_term: needs distances, positions, volumes");
  SPH_REQUIRE(!dfsph || in->dist, "pair_term: needs distances");
  SPH_REQUIRE(!dfsph || term == SPH_TERM_DFSPH_ACCEL || in->actual_area, "pair_term: needs actual areas");
  SPH_REQUIRE((term != SPH_TERM_DFSPH_ALPHA && term != SPH_TERM_DFSPH_ACCEL) || in->area, "pair_term: needs areas");
  SPH_REQUIRE(term != SPH_TERM_DFSPH_SOURCE || in->pred_vel, "pair_term: needs predicted velocities");
  SPH_REQUIRE(term != SPH_TERM_DFSPH_PRESSURE_SUM || in->pred_accel, "pair_term: needs predicted accelerations");
  SPH_REQUIRE(term != SPH_TERM_DFSPH_ACCEL || (in->rho && in->pressure), "pair_term: needs densities, pressures");
  SPH_REQUIRE(term == SPH_TERM_DENSITY || term == SPH_TERM_NORMALIZATION || dfsph || in->rho,
              "pair_term: needs densities");
  SPH_REQUIRE(term != SPH_TERM_DENSITY || in->area, "pair_term: density needs areas");
  SPH_REQUIRE((term != SPH_TERM_DIVERGENCE && term != SPH_TERM_VELOCITY_DIFFUSION && term != SPH_TERM_LAMINAR) ||
                  in->vel,
              "pair_term: needs velocities");
  SPH_REQUIRE(term != SPH_TERM_PRESSURE_ACCEL || in->pressure, "pair_term: needs pressures");
  SPH_REQUIRE(term != SPH_TERM_RENORMALIZED_GRADIENT || in->L, "pair_term: needs the pseudo-inverted L");
  SPH_REQUIRE(term != SPH_TERM_DELTA_DIFFUSION || in->grad_rho, "pair_term: needs <grad rho>");
  if (in->n == 0) return SPH_OK;
  TermIn t;
  t.offsets = in->offsets;
  t.cols = in->cols;
  t.dist = reinterpret_cast<const float2*>(in->dist);
  t.radial = in->radial;
  t.pos = reinterpret_cast<const float2*>(in->pos);
  t.vel = reinterpret_cast<const float2*>(in->vel);
  t.rho = in->rho;
  t.volume = in->volume;
  t.area = in->area;
  t.pressure = in->pressure;
  t.L = reinterpret_cast<const float4*>(in->L);
  t.grad_rho = reinterpret_cast<const float2*>(in->grad_rho);
  t.aact = in->actual_area;
  t.pred_accel = reinterpret_cast<const float2*>(in->pred_accel);
  t.pred_vel = reinterpret_cast<const float2*>(in->pred_vel);
  t.dt = (float)in->dt;
  t.n = (int)in->n;
  const SphParams P = to_params(params);
  const int nb = grid_for(in->n, 128);
  cudaStream_t st = as_stream(stream);
  switch (term) {
#define SPH_TERM_CASE(T)                                              \
  case T:                                                             \
    k_pair_term<T><<<nb, 128, 0, st>>>(t, P, out, accumulate);        \
    break;
    SPH_TERM_CASE(SPH_TERM_DENSITY)
    SPH_TERM_CASE(SPH_TERM_DIVERGENCE)
    SPH_TERM_CASE(SPH_TERM_MOG_DIFFUSION)
    SPH_TERM_CASE(SPH_TERM_NORMALIZATION)
    SPH_TERM_CASE(SPH_TERM_RENORMALIZED_GRADIENT)
    SPH_TERM_CASE(SPH_TERM_DELTA_DIFFUSION)
    SPH_TERM_CASE(SPH_TERM_PRESSURE_ACCEL)
    SPH_TERM_CASE(SPH_TERM_VELOCITY_DIFFUSION)
    SPH_TERM_CASE(SPH_TERM_LAMINAR)
#undef SPH_TERM_CASE
#define SPH_DFSPH_CASE(T)                                             \
  case T:                                                             \
    k_dfsph_term<T><<<nb, 128, 0, st>>>(t, P, out, accumulate);       \
    break;
    SPH_DFSPH_CASE(SPH_TERM_DFSPH_ALPHA)
    SPH_DFSPH_CASE(SPH_TERM_DFSPH_SOURCE)
    SPH_DFSPH_CASE(SPH_TERM_DFSPH_PRESSURE_SUM)
    SPH_DFSPH_CASE(SPH_TERM_DFSPH_ACCEL)
#undef SPH_DFSPH_CASE
    default:
      set_error_text("pair_term: unknown term");
      return SPH_ERR_INVALID_ARGUMENT;
  }
  SPH_CHECK_LAUNCH("pair_term");
  return SPH_OK;
}

sph_status_t sph_particle_op(int32_t op, int64_t n, const float* a, const float* b, const sph_params* params,
                             float* out, int32_t accumulate, void* stream) {
  SPH_REQUIRE(params && out && n >= 0 && n < (1LL << 31) && (n == 0 || a) && op >= SPH_OP_TAIT &&
                  op <= SPH_OP_GRAVITY && (op != SPH_OP_VOLUME || b),
              "particle_op: bad arguments");
  if (n == 0) return SPH_OK;
  k_particle_op<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(op, (int)n, a, b, to_params(params), out,
                                                                  accumulate);
  SPH_CHECK_LAUNCH("particle_op");
  return SPH_OK;
}

sph_status_t sph_pair_geometry(const int32_t* rows, const int32_t* cols, int64_t num_pairs, const float* query_pos,
                               const float* pos, const float* query_support, float threshold, float* dist,
                               float* radial, void* stream) {
  SPH_REQUIRE(num_pairs >= 0 && (num_pairs == 0 || (rows && cols && query_pos && pos && query_support && dist && radial)),
              "pair_geometry: bad arguments");
  if (num_pairs == 0) return SPH_OK;
  k_pair_geometry<<<grid_for(num_pairs, 256), 256, 0, as_stream(stream)>>>(
      rows, cols, num_pairs, reinterpret_cast<const float2*>(query_pos), reinterpret_cast<const float2*>(pos),
      query_support, threshold, reinterpret_cast<float2*>(dist), radial);
  SPH_CHECK_LAUNCH("pair_geometry");
  return SPH_OK;
}

sph_status_t sph_row_offsets(const int64_t* rows, int64_t num_pairs, int64_t n, int32_t* offsets, void* stream) {
  SPH_REQUIRE(offsets && n >= 0 && n < (1LL << 31) && num_pairs >= 0 && num_pairs < (1LL << 31) &&
                  (num_pairs == 0 || rows),
              "row_offsets: bad arguments");
  k_row_offsets<<<grid_for(n + 1, 256), 256, 0, as_stream(stream)>>>(rows, num_pairs, (int)n, offsets);
  SPH_CHECK_LAUNCH("row_offsets");
  return SPH_OK;
}

}  // extern "C"
