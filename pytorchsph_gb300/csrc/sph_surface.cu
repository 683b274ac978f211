// delta+ surface detection and particle shifting (src/modules/deltaPlus.py) over the
// reference's own pair lists, for callers of its Module interface.  The reference computes
// every step with scatter sum / max / min reductions over P-length temporaries; here each
// reduction is a gather over one particle's row (fluid pairs in pair order, then wall pairs
// grouped by fluid particle in pair order), one thread per particle, no atomics in the sums.
//
// Reference lines:
//   computeNormalizationmatrix deltaPlus.py:116-130 (fluid L = densityDiffusion.py:30-44 plus
//     the wall part, solidBoundary.py:676-693; the wall's own L from its fluid and wall pairs)
//   pinv2x2 and its eigVals   src/util.py:386-433
//   computeFluidNormal        deltaPlus.py:132-163
//   detectFluidSurface        deltaPlus.py:165-205
//   computeShiftAmount        deltaPlus.py:81-115
//   adjustShiftingAmount      deltaPlus.py:207-240
#include <algorithm>

#include "sph_math.cuh"

namespace sph {

struct SurfIn {
  const int32_t* off;
  const int64_t* cols;
  const float2* dist;
  const float* radial;
  const int32_t* woff;
  const int64_t* wrows;
  const int64_t* wcols;
  const float2* wdist;
  const float* wradial;
  const int32_t* fwoff;
  const int32_t* fwpairs;
  const int32_t* wwoff;
  const int64_t* wwcols;
  const float2* wwdist;
  const float* wwradial;
  const float2* pos;
  const float2* vel;
  const float* rho;
  const float* area;
  const float* volume;
  const float4* matrix;
  const float4* L;
  const float* lambda;
  const float2* normal;
  const float* mask;
  const float2* shift;
  const float2* wpos;
  const float* warea;
  const float* wrho;
  const float* wvol;
  const float* wlambda;
  const float* pressure;
  const float* wpressure;
  float packing, cfl;
  int n, nb;
};

// Singular values of [[a, b], [c, d]] as pinv2x2 returns them in eigVals: (o1, o2), the pair
// swapped where |o2| > |o1| (src/util.py:408-431).  Same float32 formulas as pinv2x2.
__device__ __forceinline__ float2 sing2x2(float a, float b, float c, float d) {
  const float S1 = a * a + b * b + c * c + d * d;
  const float t = a * a + b * b - c * c - d * d;
  const float u = a * c + b * d;
  const float S2 = sqrtf(t * t + 4 * u * u);
  float o1 = sqrtf((S1 + S2) * 0.5f);
  float o2 = sqrtf((S1 - S2) * 0.5f);
  if (fabsf(o2) > fabsf(o1)) {
    const float s = o1;
    o1 = o2;
    o2 = s;
  }
  return make_float2(o1, o2);
}

// torch.max / scatter 'max' keep a NaN they meet; so do these.
__device__ __forceinline__ float max_nan(float a, float b) {
  if (a != a) return a;
  if (b != b) return b;
  return b > a ? b : a;
}
__device__ __forceinline__ float min_nan(float a, float b) {
  if (a != a) return a;
  if (b != b) return b;
  return b < a ? b : a;
}

__global__ void k_surf_pinv_eig(SurfIn in, float4* __restrict__ pinv, float2* __restrict__ eig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const float4 m = in.matrix[i];
  pinv[i] = pinv2x2(m.x, m.y, m.z, m.w);
  eig[i] = sing2x2(m.x, m.y, m.z, m.w);
}

// The wall's own normalization matrix (solidBoundary.py:679-693):
//   sum over its fluid pairs of V_f (x_f - x_b) (x) gradW(e_bf)        (computeNormalizationMatrix
//   with i = wall, j = fluid, distances = boundaryToFluidNeighborDistances), then
//   plus the sum over its wall pairs of V_c (x_c - x_b) (x) gradW(e'), e' the reference's
//   boundaryToBoundaryNeighborDistances (x_c - x_b) / r: with the fluid's sign convention the
//   wall-wall part enters with the opposite sign of the fluid parts, as in the reference.
// Each part summed in pair order, then added, as the reference adds the two scatters.
__global__ void __launch_bounds__(128) k_surf_wall_L(SurfIn in, SphParams P, float4* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= in.nb) return;
  const float2 xb = in.wpos[b];
  float f00 = 0.f, f01 = 0.f, f10 = 0.f, f11 = 0.f;
  for (int k = in.woff[b], k1 = in.woff[b + 1]; k < k1; ++k) {
    const int f = (int)in.wcols[k];
    if ((unsigned)f >= (unsigned)in.n) continue;
    const float2 e = in.wdist[k];
    const float gw = kGW(in.wradial[k], P.c_g);
    const float gx = e.x * gw, gy = e.y * gw;
    const float2 xf = in.pos[f];
    const float rx = xf.x - xb.x, ry = xf.y - xb.y;
    const float V = in.volume[f];
    f00 += rx * gx * V;
    f01 += rx * gy * V;
    f10 += ry * gx * V;
    f11 += ry * gy * V;
  }
  float w00 = 0.f, w01 = 0.f, w10 = 0.f, w11 = 0.f;
  if (in.wwoff) {
    for (int k = in.wwoff[b], k1 = in.wwoff[b + 1]; k < k1; ++k) {
      const int c = (int)in.wwcols[k];
      if ((unsigned)c >= (unsigned)in.nb) continue;
      const float2 e = in.wwdist[k];
      const float gw = kGW(in.wwradial[k], P.c_g);
      const float gx = e.x * gw, gy = e.y * gw;
      const float2 xc = in.wpos[c];
      const float rx = xc.x - xb.x, ry = xc.y - xb.y;
      const float V = in.wvol[c];
      w00 += rx * gx * V;
      w01 += rx * gy * V;
      w10 += ry * gx * V;
      w11 += ry * gy * V;
    }
  }
  out[b] = make_float4(f00 + w00, f01 + w01, f10 + w10, f11 + w11);
}

// lambdaGrad_i = -sum_j (A_j / rho_j)(lambda_j - lambda_i) L_i gradW_ij
//                - sum_b (A[b] / rho[b])(lambda_b - lambda_i) L_i gradW(e_fb)
// (the wall volume indexes the fluid arrays with the wall index, as deltaPlus.py:150 does);
// fluidNormal = lambdaGrad / (|lambdaGrad| + 0.1 h^2).
__global__ void __launch_bounds__(128) k_surf_normal(SurfIn in, SphParams P, float2* __restrict__ grad,
                                                     float2* __restrict__ normal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const float4 Li = in.L[i];
  const float li = in.lambda[i];
  float sx = 0.f, sy = 0.f;
  for (int k = in.off[i], k1 = in.off[i + 1]; k < k1; ++k) {
    const int j = (int)in.cols[k];
    const float2 e = in.dist[k];
    const float gw = kGW(in.radial[k], P.c_g);
    const float gx = e.x * gw, gy = e.y * gw;
    const float c = (in.area[j] / in.rho[j]) * (in.lambda[j] - li);
    const float cx = Li.x * gx + Li.y * gy, cy = Li.z * gx + Li.w * gy;
    sx += -c * cx;
    sy += -c * cy;
  }
  float wx = 0.f, wy = 0.f;
  if (in.fwoff) {
    for (int t = in.fwoff[i], t1 = in.fwoff[i + 1]; t < t1; ++t) {
      const int k = in.fwpairs[t];
      const int b = (int)in.wrows[k];
      if ((unsigned)b >= (unsigned)in.nb || b >= in.n) continue;
      const float2 e = in.wdist[k];
      const float gw = kGW(in.wradial[k], P.c_g);
      const float gx = -e.x * gw, gy = -e.y * gw;   // kernelGradient(q, -e_bf)
      const float c = (in.area[b] / in.rho[b]) * (in.wlambda[b] - li);
      const float cx = Li.x * gx + Li.y * gy, cy = Li.z * gx + Li.w * gy;
      wx += -c * cx;
      wy += -c * cy;
    }
  }
  const float2 g = make_float2(sx + wx, sy + wy);
  grad[i] = g;
  const float d = sqrtf(g.x * g.x + g.y * g.y) + P.eps;
  normal[i] = make_float2(g.x / d, g.y / d);
}

// Largest cosine between the normal and the directions to the neighbors: fluid pairs j != i
// with -e_ij, wall pairs with e_bf; each part is 0 without pairs (the scatter's fill), and the
// larger of the two parts counts.  mask = arccos(that) > pi/6 and lambda < 0.6.
__global__ void __launch_bounds__(128) k_surf_angle(SurfIn in, float* __restrict__ mask,
                                                    float2* __restrict__ angles) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const float2 ni = in.normal[i];
  bool any = false;
  float mx = 0.f, mn = 0.f;
  for (int k = in.off[i], k1 = in.off[i + 1]; k < k1; ++k) {
    if ((int)in.cols[k] == i) continue;
    const float2 e = in.dist[k];
    const float d = (-e.x) * ni.x + (-e.y) * ni.y;
    if (!any) {
      mx = d;
      mn = d;
      any = true;
    } else {
      mx = max_nan(mx, d);
      mn = min_nan(mn, d);
    }
  }
  bool anyw = false;
  float mw = 0.f;
  if (in.fwoff) {
    for (int t = in.fwoff[i], t1 = in.fwoff[i + 1]; t < t1; ++t) {
      const int k = in.fwpairs[t];
      const float2 e = in.wdist[k];
      const float d = e.x * ni.x + e.y * ni.y;
      mw = anyw ? max_nan(mw, d) : d;
      anyw = true;
    }
  }
  const float s = max_nan(mx, mw);
  const float th = acosf(s);
  mask[i] = (th > 0.52359879f && in.lambda[i] < 0.6f) ? 1.0f : 0.0f;   // float32(pi / 6)
  if (angles) angles[i] = make_float2(acosf(mn), acosf(mx));
}

// mask2 = max over neighbors j != i of mask_j (0 without such pairs); finalMask = 1 where
// mask, 2/3 where only mask2, else 0; then surface 1 where lambda >= 0.5 and finalMask > 0,
// 0 where finalMask > 0.7, bulk 2 where finalMask < 0.1 (deltaPlus.py:189-205, applied in
// the reference's order).
__global__ void __launch_bounds__(128) k_surf_classify(SurfIn in, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  bool any = false;
  float m2 = 0.f;
  for (int k = in.off[i], k1 = in.off[i + 1]; k < k1; ++k) {
    const int j = (int)in.cols[k];
    if (j == i) continue;
    const float v = in.mask[j];
    m2 = any ? max_nan(m2, v) : v;
    any = true;
  }
  float fm = 0.f;
  if (m2 > 0.f) fm = 2.0f / 3.0f;
  if (in.mask[i] > 0.f) fm = 1.0f;
  float s = fm;
  if (in.lambda[i] >= 0.5f && fm > 0.f) s = 1.0f;
  if (fm > 0.7f) s = 0.0f;
  if (fm < 0.1f) s = 2.0f;
  out[i] = s;
}

// max |v_i| into *vmax (float bits of a non-negative value order like unsigned integers;
// *vmax is zeroed before).  A NaN speed is carried as the largest pattern.
__global__ void k_surf_max_speed(SurfIn in, unsigned int* __restrict__ vmax) {
  __shared__ unsigned int s_max[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int m = 0u;
  for (int k = i; k < in.n; k += gridDim.x * blockDim.x) {
    const float2 v = in.vel[k];
    const float sp = sqrtf(v.x * v.x + v.y * v.y);
    const unsigned int u = sp == sp ? __float_as_uint(sp) : 0xffffffffu;
    m = u > m ? u : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned int x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = s_max[w] > m ? s_max[w] : m;
    atomicMax(vmax, m);
  }
}

// shiftAmount_i = -cfl Ma 4 h^2 sum_j (1 + R (W_ij / W(packing))^4) A_j / (rho_i + rho_j) gradW_ij
//                 - cfl Ma 4 h^2 sum_b (1 + R (W_bf / W(packing))^4) A_b / (rho_f + rho_b) gradW(e_fb)
// with R = 0.2 and Ma = max |v| / c0 (deltaPlus.py:81-115).
__global__ void __launch_bounds__(128) k_surf_shift(SurfIn in, SphParams P, const unsigned int* __restrict__ vmax,
                                                    float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const unsigned int u = *vmax;
  const float speed = u == 0xffffffffu ? __int_as_float(0x7fffffff) : __uint_as_float(u);
  const float Ma = speed / P.c0;
  const float k0 = kW(in.packing, P.c_w);
  const float coef = (-in.cfl * Ma) * (4.0f * (P.h * P.h));
  const float rhoi = in.rho[i];
  float sx = 0.f, sy = 0.f;
  for (int k = in.off[i], k1 = in.off[i + 1]; k < k1; ++k) {
    const int j = (int)in.cols[k];
    const float q = in.radial[k];
    const float r = kW(q, P.c_w) / k0;
    const float r2 = r * r;
    const float kt = 1.0f + 0.2f * (r2 * r2);
    const float mass = in.area[j] / (rhoi + in.rho[j]);
    const float2 e = in.dist[k];
    const float gw = kGW(q, P.c_g);
    const float c = kt * mass;
    sx += c * (e.x * gw);
    sy += c * (e.y * gw);
  }
  float wx = 0.f, wy = 0.f;
  if (in.fwoff) {
    for (int t = in.fwoff[i], t1 = in.fwoff[i + 1]; t < t1; ++t) {
      const int k = in.fwpairs[t];
      const int b = (int)in.wrows[k];
      if ((unsigned)b >= (unsigned)in.nb) continue;
      const float q = in.wradial[k];
      const float r = kW(q, P.c_w) / k0;
      const float r2 = r * r;
      const float kt = 1.0f + 0.2f * (r2 * r2);
      const float mass = in.warea[b] / (rhoi + in.wrho[b]);
      const float2 e = in.wdist[k];
      const float gw = kGW(q, P.c_g);
      const float c = kt * mass;
      wx += c * (-e.x * gw);
      wy += c * (-e.y * gw);
    }
  }
  out[i] = make_float2(coef * sx + coef * wx, coef * sy + coef * wy);
}

// fluidUpdate: shift capped at 0.05 h, projected by (I - n n^T) where mask < 1.5, zero where
// mask < 0.5; the mask becomes 1 / 0 / 2 for those regions and the bulk.
__global__ void k_surf_shift_adjust(SurfIn in, SphParams P, float2* __restrict__ out, float* __restrict__ mask_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  float2 s = in.shift[i];
  const float len = sqrtf(s.x * s.x + s.y * s.y);
  const float cap = P.h * 0.05f;
  if (len > cap) s = make_float2(s.x / len * P.h * 0.05f, s.y / len * P.h * 0.05f);
  const float m = in.mask[i];
  const float2 nv = in.normal[i];
  if (m < 1.5f) {
    const float a00 = 1.0f - nv.x * nv.x, a01 = 0.0f - nv.x * nv.y;
    const float a10 = 0.0f - nv.y * nv.x, a11 = 1.0f - nv.y * nv.y;
    s = make_float2(a00 * s.x + a01 * s.y, a10 * s.x + a11 * s.y);
  }
  if (m < 0.5f) s = make_float2(0.f, 0.f);
  out[i] = s;
  float nm = m;
  if (m < 1.5f) nm = 1.0f;
  if (m < 0.5f) nm = 0.0f;
  if (m > 1.5f) nm = 2.0f;
  mask_out[i] = nm;
}

// computePressureAccelDeltaPlus (pressure.py:31-51): the pressure term switches to p_j - p_i
// where p_i < 0 inside the bulk (mask_i >= 1.5), to avoid tensile instability there.  kWall:
// over the wall pairs of particle i (e_fb = -e_bf, the wall's pressure and volume), as
// solidBoundary.py:876-884 calls it with (bf, bb).
template <bool kWall>
__global__ void __launch_bounds__(128) k_surf_pressure_accel(SurfIn in, SphParams P, float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in.n) return;
  const float pi = in.pressure[i];
  const bool plus = pi >= 0.f || in.mask[i] < 1.5f;
  float sx = 0.f, sy = 0.f;
  if (!kWall) {
    for (int k = in.off[i], k1 = in.off[i + 1]; k < k1; ++k) {
      const int j = (int)in.cols[k];
      const float2 e = in.dist[k];
      const float gw = kGW(in.radial[k], P.c_g);
      const float pj = in.pressure[j];
      const float c = (plus ? pi + pj : pj - pi) * in.volume[j];
      sx += c * (e.x * gw);
      sy += c * (e.y * gw);
    }
  } else if (in.fwoff) {
    for (int t = in.fwoff[i], t1 = in.fwoff[i + 1]; t < t1; ++t) {
      const int k = in.fwpairs[t];
      const int b = (int)in.wrows[k];
      if ((unsigned)b >= (unsigned)in.nb) continue;
      const float2 e = in.wdist[k];
      const float gw = kGW(in.wradial[k], P.c_g);
      const float pb = in.wpressure[b];
      const float c = (plus ? pi + pb : pb - pi) * in.wvol[b];
      sx += c * (-e.x * gw);
      sy += c * (-e.y * gw);
    }
  }
  const float ir = -1.0f / (in.rho[i] * P.rho0);
  out[i] = make_float2(ir * sx, ir * sy);
}

}  // namespace sph

using namespace sph;

static SurfIn to_surf(const sph_surface_in* in) {
  SurfIn t;
  t.off = in->offsets;
  t.cols = in->cols;
  t.dist = reinterpret_cast<const float2*>(in->dist);
  t.radial = in->radial;
  t.woff = in->wall_offsets;
  t.wrows = in->wall_rows;
  t.wcols = in->wall_cols;
  t.wdist = reinterpret_cast<const float2*>(in->wall_dist);
  t.wradial = in->wall_radial;
  t.fwoff = in->fluid_wall_offsets;
  t.fwpairs = in->fluid_wall_pairs;
  t.wwoff = in->ww_offsets;
  t.wwcols = in->ww_cols;
  t.wwdist = reinterpret_cast<const float2*>(in->ww_dist);
  t.wwradial = in->ww_radial;
  t.pos = reinterpret_cast<const float2*>(in->pos);
  t.vel = reinterpret_cast<const float2*>(in->vel);
  t.rho = in->rho;
  t.area = in->area;
  t.volume = in->volume;
  t.matrix = reinterpret_cast<const float4*>(in->matrix);
  t.L = reinterpret_cast<const float4*>(in->L);
  t.lambda = in->lambda;
  t.normal = reinterpret_cast<const float2*>(in->normal);
  t.mask = in->mask;
  t.shift = reinterpret_cast<const float2*>(in->shift);
  t.wpos = reinterpret_cast<const float2*>(in->wall_pos);
  t.warea = in->wall_area;
  t.wrho = in->wall_rho;
  t.wvol = in->wall_volume;
  t.wlambda = in->wall_lambda;
  t.pressure = in->pressure;
  t.wpressure = in->wall_pressure;
  t.packing = in->packing;
  t.cfl = in->cfl;
  t.n = (int)in->n;
  t.nb = (int)in->nb;
  return t;
}

extern "C" {

size_t sph_surface_scratch_bytes(void) { return 256; }

sph_status_t sph_surface_term(int32_t term, const sph_surface_in* in, const sph_params* params, float* out,
                              float* out2, void* stream) {
  SPH_REQUIRE(in && params && out && params->support > 0.f && in->n >= 0 && in->n < (1LL << 31) && in->nb >= 0 &&
                  in->nb < (1LL << 31),
              "surface_term: bad arguments");
  const bool fluid_pairs = term == SPH_SURF_NORMAL || term == SPH_SURF_ANGLE_MASK || term == SPH_SURF_CLASSIFY ||
                           term == SPH_SURF_SHIFT;
  SPH_REQUIRE(!fluid_pairs || in->n == 0 || (in->offsets && in->cols), "surface_term: needs the fluid pairs");
  // wall pairs are optional for the fluid-side terms (no walls); all of them or none
  const bool walls = in->fluid_wall_offsets != nullptr;
  SPH_REQUIRE(!walls || (in->fluid_wall_pairs && in->wall_rows && in->wall_dist && in->wall_radial),
              "surface_term: incomplete wall pair list");
  bool ok = true;
  switch (term) {
    case SPH_SURF_PINV_EIG: ok = in->matrix && out2; break;
    case SPH_SURF_WALL_NORMALIZATION:
      ok = in->wall_offsets && in->wall_cols && in->wall_dist && in->wall_radial && in->pos && in->volume &&
           in->wall_pos && (!in->ww_offsets || (in->ww_cols && in->ww_dist && in->ww_radial && in->wall_volume));
      break;
    case SPH_SURF_NORMAL:
      ok = out2 && in->dist && in->radial && in->area && in->rho && in->L && in->lambda && (!walls || in->wall_lambda);
      break;
    case SPH_SURF_ANGLE_MASK: ok = in->dist && in->normal && in->lambda; break;
    case SPH_SURF_CLASSIFY: ok = in->mask && in->lambda; break;
    case SPH_SURF_SHIFT:
      ok = out2 && in->dist && in->radial && in->vel && in->area && in->rho && (!walls || (in->wall_area && in->wall_rho)) &&
           params->c0 > 0.f;
      break;
    case SPH_SURF_SHIFT_ADJUST: ok = out2 && in->shift && in->mask && in->normal; break;
    case SPH_SURF_PRESSURE_ACCEL:
      ok = in->offsets && in->cols && in->dist && in->radial && in->pressure && in->mask && in->volume && in->rho;
      break;
    case SPH_SURF_WALL_PRESSURE_ACCEL:
      ok = in->pressure && in->mask && in->rho && (!walls || (in->wall_pressure && in->wall_volume));
      break;
    default:
      set_error_text("surface_term: unknown term");
      return SPH_ERR_INVALID_ARGUMENT;
  }
  SPH_REQUIRE(ok, "surface_term: an array this term reads or writes is missing");
  const SurfIn t = to_surf(in);
  const SphParams P = to_params(params);
  cudaStream_t st = as_stream(stream);
  const int nbf = grid_for(in->n, 128);
  switch (term) {
    case SPH_SURF_PINV_EIG:
      if (in->n)
        k_surf_pinv_eig<<<grid_for(in->n, 256), 256, 0, st>>>(t, reinterpret_cast<float4*>(out),
                                                              reinterpret_cast<float2*>(out2));
      break;
    case SPH_SURF_WALL_NORMALIZATION:
      if (in->nb) k_surf_wall_L<<<grid_for(in->nb, 128), 128, 0, st>>>(t, P, reinterpret_cast<float4*>(out));
      break;
    case SPH_SURF_NORMAL:
      if (in->n)
        k_surf_normal<<<nbf, 128, 0, st>>>(t, P, reinterpret_cast<float2*>(out), reinterpret_cast<float2*>(out2));
      break;
    case SPH_SURF_ANGLE_MASK:
      if (in->n) k_surf_angle<<<nbf, 128, 0, st>>>(t, out, reinterpret_cast<float2*>(out2));
      break;
    case SPH_SURF_CLASSIFY:
      if (in->n) k_surf_classify<<<nbf, 128, 0, st>>>(t, out);
      break;
    case SPH_SURF_SHIFT: {
      if (!in->n) break;
      unsigned int* vmax = reinterpret_cast<unsigned int*>(out2);
      cudaError_t e = cudaMemsetAsync(vmax, 0, sizeof(unsigned int), st);
      if (e != cudaSuccess) {
        set_error("surface_term(shift)", e);
        return SPH_ERR_CUDA;
      }
      const int blocks = (int)std::min<int64_t>(2 * kNumSMs, (in->n + 255) / 256);
      k_surf_max_speed<<<blocks, 256, 0, st>>>(t, vmax);
      k_surf_shift<<<nbf, 128, 0, st>>>(t, P, vmax, reinterpret_cast<float2*>(out));
      break;
    }
    case SPH_SURF_SHIFT_ADJUST:
      if (in->n)
        k_surf_shift_adjust<<<grid_for(in->n, 256), 256, 0, st>>>(t, P, reinterpret_cast<float2*>(out), out2);
      break;
    case SPH_SURF_PRESSURE_ACCEL:
      if (in->n) k_surf_pressure_accel<false><<<nbf, 128, 0, st>>>(t, P, reinterpret_cast<float2*>(out));
      break;
    case SPH_SURF_WALL_PRESSURE_ACCEL:
      if (in->n) k_surf_pressure_accel<true><<<nbf, 128, 0, st>>>(t, P, reinterpret_cast<float2*>(out));
      break;
  }
  SPH_CHECK_LAUNCH("surface_term");
  return SPH_OK;
}

}  // extern "C"
