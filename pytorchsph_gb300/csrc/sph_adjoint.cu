// Differentiable deltaSPH rollout of a free fluid (no walls): the right-hand side of
// src/deltaSPH.py:146-200 with MOG density diffusion and gravity or the point source, the
// semi-implicit Euler update (src/simulationBase.py:647-652), and the discrete adjoint of
// one step — vector-Jacobian products by forward-mode dual numbers on each pair.
//
// Pairs are the reference's (i, j)-ordered list in original particle order (row offsets +
// columns, as neighborSearchModule.search returns it); the list is symmetric because every
// particle has the same support.  Particle i's adjoint gathers over its own row both
//   (d f_ij / d in_i)^T lambda_out_i   (its own right-hand side)   and
//   (d f_ji / d in_i)^T lambda_out_j   (its neighbors' right-hand sides),
// so there are no atomics and the result does not depend on thread timing.  The same pair
// function (template on the scalar type) gives the forward right-hand side, so forward and
// adjoint differentiate one formula.  Scalars are float or double.
#include "sph_common.cuh"

namespace sph {

template <typename T, int K>
struct Dual {
  T v;
  T d[K];
};

template <typename T>
__device__ __forceinline__ T val(T a) {
  return a;
}
template <typename T, int K>
__device__ __forceinline__ T val(const Dual<T, K>& a) {
  return a.v;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator+(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(const Dual<T, K>& a) {
  Dual<T, K> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator*(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator/(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  const T ib = T(1) / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator+(const Dual<T, K>& a, T b) {
  Dual<T, K> r = a;
  r.v += b;
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator+(T b, const Dual<T, K>& a) {
  return a + b;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(const Dual<T, K>& a, T b) {
  Dual<T, K> r = a;
  r.v -= b;
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(T b, const Dual<T, K>& a) {
  return -(a - b);
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator*(const Dual<T, K>& a, T b) {
  Dual<T, K> r;
  r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator*(T b, const Dual<T, K>& a) {
  return a * b;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator/(const Dual<T, K>& a, T b) {
  return a * (T(1) / b);
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator/(T b, const Dual<T, K>& a) {
  Dual<T, K> one;
  one.v = b;
#pragma unroll
  for (int k = 0; k < K; ++k) one.d[k] = T(0);
  return one / a;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> sqrt_(const Dual<T, K>& a) {
  Dual<T, K> r;
  r.v = sqrt(a.v);
  const T f = T(0.5) / r.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * f;
  return r;
}
template <typename T>
__device__ __forceinline__ T sqrt_(T a) {
  return sqrt(a);
}
template <typename T>
__device__ __forceinline__ T make_const(T c, T) {
  return c;
}
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> make_const(T c, const Dual<T, K>&) {
  Dual<T, K> r;
  r.v = c;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = T(0);
  return r;
}

template <typename T>
struct DropParams {
  T inv_h, cg20;      // 1/h, 20 * 7/(pi h^3)
  T rho0, tait_k;     // rho0 c0^2 / gamma (gamma = 7)
  T eps;              // 0.1 h^2
  T visc_unit;        // h c0 (artificial viscosity factor without alpha)
  T alpha, nu;        // artificial and laminar (kinematic) viscosity
  T diff_k;           // h delta c0 (MOG)
  T gx, gy;           // constant gravity
  int point_source;
  T point_mag, cx, cy;
  int mog;
};

template <typename S>
struct PairOut {
  S ax, ay, dp;
  S vx, vy;  // artificial viscosity part without alpha (for d/d alpha)
};

template <typename S, typename T>
__device__ __forceinline__ S tait7(const S& rt, const DropParams<T>& P) {
  const S r2 = rt * rt;
  const S r4 = r2 * r2;
  return P.tait_k * (r4 * r2 * rt - T(1));
}

// Row i's terms from neighbor j (x_i - x_j nonzero).  Reference formulas: pressure.py:31-38,
// diffusion.py:30-44, laminar.py:30-46 (its index choices), momentum.py:31-38,
// densityDiffusion.py:74-82, kernels.py:20-33.
template <typename S, typename T>
__device__ __forceinline__ PairOut<S> pair_terms(const S& xix, const S& xiy, const S& vix, const S& viy,
                                                 const S& rti, const S& xjx, const S& xjy, const S& vjx,
                                                 const S& vjy, const S& rtj, T Aj, const DropParams<T>& P) {
  const S dx = xix - xjx, dy = xiy - xjy;          // x_i - x_j
  const S r2 = dx * dx + dy * dy;
  const S r = sqrt_(r2);
  const S q = r * P.inv_h;
  const S a = T(1) - q;
  const S gwr = -(P.cg20 * q * a * a * a) / r;   // gradW = gwr * (x_i - x_j)
  const S gx = gwr * dx, gy = gwr * dy;
  const S rhoi = rti * P.rho0, rhoj = rtj * P.rho0;
  const S Vj = Aj / rtj;
  const S pi = tait7(rti, P), pj = tait7(rtj, P);
  const S ux = vjx - vix, uy = vjy - viy;          // u_j - u_i
  const S rx = -dx, ry = -dy;                      // x_j - x_i
  const S R2 = r2 + P.eps;
  const S rg = rx * gx + ry * gy;
  PairOut<S> o;
  const S pf = (pi + pj) * Vj / rhoi;
  o.ax = -(pf * gx);
  o.ay = -(pf * gy);
  S pij = ux * rx + uy * ry;
  if (val(pij) > T(0)) pij = make_const(T(0), pij);
  const S vf = P.visc_unit * pij / R2 * Vj * rhoj / (rhoi + rhoj);
  o.vx = vf * gx;
  o.vy = vf * gy;
  o.ax = o.ax + P.alpha * o.vx;
  o.ay = o.ay + P.alpha * o.vy;
  const S rs = rhoi + rhoj;
  const S term = T(8) * rhoj * Vj * rhoi * P.nu * rg / (rs * rs * R2);   // 4 m_j (mu_i + mu_j), mu = rho_i nu
  o.ax = o.ax - term * (vix - vjx);
  o.ay = o.ay - term * (viy - vjy);
  o.dp = -((ux * gx + uy * gy) * Vj * rhoj);
  if (P.mog) o.dp = o.dp + P.diff_k * T(2) * (rhoj - rhoi) / R2 * rg * Vj;
  return o;
}

template <typename T>
__device__ __forceinline__ bool apart(T xix, T xiy, T xjx, T xjy) {
  const T dx = xix - xjx, dy = xiy - xjy;
  return dx * dx + dy * dy >= T(1e-14);   // the reference's e_ij is 0 below r = 1e-7
}

template <typename T, typename V2>
__global__ void __launch_bounds__(128) k_drop_rhs(int n, const int32_t* __restrict__ offsets,
                                                  const int64_t* __restrict__ cols, const V2* __restrict__ x,
                                                  const V2* __restrict__ v, const T* __restrict__ rt,
                                                  const T* __restrict__ area, DropParams<T> P, V2* __restrict__ acc,
                                                  T* __restrict__ dpdt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V2 xi = x[i], vi = v[i];
  const T ri = rt[i];
  T ax = 0, ay = 0, dp = 0;
  for (int k = offsets[i]; k < offsets[i + 1]; ++k) {
    const int j = (int)cols[k];
    const V2 xj = x[j], vj = v[j];
    if (!apart(xi.x, xi.y, xj.x, xj.y)) continue;
    const PairOut<T> o = pair_terms<T, T>(xi.x, xi.y, vi.x, vi.y, ri, xj.x, xj.y, vj.x, vj.y, rt[j], area[j], P);
    ax += o.ax;
    ay += o.ay;
    dp += o.dp;
  }
  if (P.point_source) {
    T dx = xi.x - P.cx, dy = xi.y - P.cy;
    const T d = sqrt(dx * dx + dy * dy);
    if (d > T(1e-7)) {
      dx /= d;
      dy /= d;
    }
    ax += -P.point_mag * dx * d;
    ay += -P.point_mag * dy * d;
  } else {
    ax += P.gx;
    ay += P.gy;
  }
  acc[i].x = ax;
  acc[i].y = ay;
  dpdt[i] = dp;
}

template <typename T, typename V2>
__global__ void k_drop_sie(int n, V2* __restrict__ x, V2* __restrict__ v, T* __restrict__ rt,
                           const V2* __restrict__ acc, const T* __restrict__ dpdt, T dt, T rho0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V2 a = acc[i], vi = v[i], xi = x[i];
  V2 vn, xn;
  vn.x = vi.x + dt * a.x;
  vn.y = vi.y + dt * a.y;
  xn.x = xi.x + dt * (vi.x + dt * a.x);
  xn.y = xi.y + dt * (vi.y + dt * a.y);
  x[i] = xn;
  v[i] = vn;
  rt[i] = rt[i] + dt * dpdt[i] / rho0;
}

// One step of the adjoint: from (lx', lv', lr') of step k+1 and the state of step k, the
// adjoint of step k and particle i's share of dL/d alpha.
template <typename T, typename V2>
__global__ void __launch_bounds__(128) k_drop_adjoint(int n, const int32_t* __restrict__ offsets,
                                                      const int64_t* __restrict__ cols, const V2* __restrict__ x,
                                                      const V2* __restrict__ v, const T* __restrict__ rt,
                                                      const T* __restrict__ area, DropParams<T> P, T dt,
                                                      const V2* __restrict__ lx1, const V2* __restrict__ lv1,
                                                      const T* __restrict__ lr1, V2* __restrict__ lx0,
                                                      V2* __restrict__ lv0, T* __restrict__ lr0,
                                                      T* __restrict__ dalpha) {
  using D = Dual<T, 5>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T dt2 = dt * dt, sdp = dt / P.rho0;
  const V2 xi = x[i], vi = v[i];
  const T ri = rt[i];
  // lambda of row i's outputs: acc via v' = v + dt a and x' = x + dt v + dt^2 a; dpdt via rho'
  const V2 lxi1 = lx1[i], lvi1 = lv1[i];
  const T lai_x = dt * lvi1.x + dt2 * lxi1.x, lai_y = dt * lvi1.y + dt2 * lxi1.y, ldi = sdp * lr1[i];
  D Xx, Xy, Vx, Vy, R;   // particle i's inputs, seeded
  Xx = make_const(xi.x, Xx);
  Xy = make_const(xi.y, Xy);
  Vx = make_const(vi.x, Vx);
  Vy = make_const(vi.y, Vy);
  R = make_const(ri, R);
  Xx.d[0] = T(1);
  Xy.d[1] = T(1);
  Vx.d[2] = T(1);
  Vy.d[3] = T(1);
  R.d[4] = T(1);
  T g[5] = {0, 0, 0, 0, 0};
  T da = 0;
  for (int k = offsets[i]; k < offsets[i + 1]; ++k) {
    const int j = (int)cols[k];
    const V2 xj = x[j], vj = v[j];
    if (!apart(xi.x, xi.y, xj.x, xj.y)) continue;
    const T rj = rt[j];
    const D Jx = make_const(xj.x, Xx), Jy = make_const(xj.y, Xx), Jvx = make_const(vj.x, Xx),
            Jvy = make_const(vj.y, Xx), Jr = make_const(rj, Xx);
    // row i, derivatives with respect to i
    const PairOut<D> o = pair_terms<D, T>(Xx, Xy, Vx, Vy, R, Jx, Jy, Jvx, Jvy, Jr, area[j], P);
#pragma unroll
    for (int c = 0; c < 5; ++c) g[c] += o.ax.d[c] * lai_x + o.ay.d[c] * lai_y + o.dp.d[c] * ldi;
    da += o.vx.v * lai_x + o.vy.v * lai_y;
    // row j, derivatives with respect to i (its column)
    const V2 lxj1 = lx1[j], lvj1 = lv1[j];
    const T laj_x = dt * lvj1.x + dt2 * lxj1.x, laj_y = dt * lvj1.y + dt2 * lxj1.y, ldj = sdp * lr1[j];
    const PairOut<D> w = pair_terms<D, T>(Jx, Jy, Jvx, Jvy, Jr, Xx, Xy, Vx, Vy, R, area[i], P);
#pragma unroll
    for (int c = 0; c < 5; ++c) g[c] += w.ax.d[c] * laj_x + w.ay.d[c] * laj_y + w.dp.d[c] * ldj;
  }
  if (P.point_source) {  // a = -mag (x - c) away from the centre
    const T dx = xi.x - P.cx, dy = xi.y - P.cy;
    if (dx * dx + dy * dy > T(1e-14)) {
      g[0] += -P.point_mag * lai_x;
      g[1] += -P.point_mag * lai_y;
    }
  }
  V2 ox, ov;
  ox.x = lxi1.x + g[0];
  ox.y = lxi1.y + g[1];
  ov.x = lvi1.x + dt * lxi1.x + g[2];
  ov.y = lvi1.y + dt * lxi1.y + g[3];
  lx0[i] = ox;
  lv0[i] = ov;
  lr0[i] = lr1[i] + g[4];
  dalpha[i] = da;
}

template <typename T>
DropParams<T> drop_params(const sph_params* p, int mog) {
  DropParams<T> P;
  const double h = p->support;
  P.inv_h = T(1.0 / h);
  P.cg20 = T(20.0 * 7.0 / 3.14159265358979323846 / (h * h * h));
  P.rho0 = T(p->rest_density);
  P.tait_k = T((double)p->rest_density * p->c0 * p->c0 / p->gamma);
  P.eps = T(h * h * 0.1);
  P.visc_unit = T(h * p->c0);
  P.alpha = T(p->alpha);
  P.nu = T(p->kinematic);
  P.diff_k = T(h * p->delta * p->c0);
  P.gx = T(p->gravity[0]);
  P.gy = T(p->gravity[1]);
  P.point_source = p->point_source;
  P.point_mag = T(p->point_magnitude);
  P.cx = T(p->point_center[0]);
  P.cy = T(p->point_center[1]);
  P.mog = mog;
  return P;
}

}  // namespace sph

using namespace sph;

extern "C" {

sph_status_t sph_drop_rhs(int32_t fp64, int64_t n, const int32_t* offsets, const int64_t* cols, const void* x,
                          const void* v, const void* rho, const void* area, const sph_params* params, void* acc,
                          void* dpdt, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && params && params->support > 0.f && params->gamma == 7.f &&
                  (params->density_diffusion == 0 || params->density_diffusion == 1) &&
                  (n == 0 || (offsets && cols && x && v && rho && area && acc && dpdt)),
              "drop_rhs: bad arguments (gamma 7, MOG or no density diffusion)");
  if (n == 0) return SPH_OK;
  const int mog = params->density_diffusion == 1;
  cudaStream_t st = as_stream(stream);
  if (fp64) {
    k_drop_rhs<double, double2><<<grid_for(n, 128), 128, 0, st>>>(
        (int)n, offsets, cols, static_cast<const double2*>(x), static_cast<const double2*>(v),
        static_cast<const double*>(rho), static_cast<const double*>(area), drop_params<double>(params, mog),
        static_cast<double2*>(acc), static_cast<double*>(dpdt));
  } else {
    k_drop_rhs<float, float2><<<grid_for(n, 128), 128, 0, st>>>(
        (int)n, offsets, cols, static_cast<const float2*>(x), static_cast<const float2*>(v),
        static_cast<const float*>(rho), static_cast<const float*>(area), drop_params<float>(params, mog),
        static_cast<float2*>(acc), static_cast<float*>(dpdt));
  }
  SPH_CHECK_LAUNCH("drop_rhs");
  return SPH_OK;
}

sph_status_t sph_drop_integrate(int32_t fp64, int64_t n, void* x, void* v, void* rho, const void* acc,
                                const void* dpdt, double dt, double rest_density, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && (n == 0 || (x && v && rho && acc && dpdt)) && rest_density > 0,
              "drop_integrate: bad arguments");
  if (n == 0) return SPH_OK;
  cudaStream_t st = as_stream(stream);
  if (fp64)
    k_drop_sie<double, double2><<<grid_for(n, 256), 256, 0, st>>>(
        (int)n, static_cast<double2*>(x), static_cast<double2*>(v), static_cast<double*>(rho),
        static_cast<const double2*>(acc), static_cast<const double*>(dpdt), dt, rest_density);
  else
    k_drop_sie<float, float2><<<grid_for(n, 256), 256, 0, st>>>(
        (int)n, static_cast<float2*>(x), static_cast<float2*>(v), static_cast<float*>(rho),
        static_cast<const float2*>(acc), static_cast<const float*>(dpdt), (float)dt, (float)rest_density);
  SPH_CHECK_LAUNCH("drop_integrate");
  return SPH_OK;
}

sph_status_t sph_drop_adjoint(int32_t fp64, int64_t n, const int32_t* offsets, const int64_t* cols, const void* x,
                              const void* v, const void* rho, const void* area, const sph_params* params, double dt,
                              const void* lx1, const void* lv1, const void* lr1, void* lx0, void* lv0, void* lr0,
                              void* dalpha, void* stream) {
  SPH_REQUIRE(n >= 0 && n < (1LL << 31) && params && params->support > 0.f && params->gamma == 7.f &&
                  (params->density_diffusion == 0 || params->density_diffusion == 1) &&
                  (n == 0 || (offsets && cols && x && v && rho && area && lx1 && lv1 && lr1 && lx0 && lv0 && lr0 &&
                              dalpha)),
              "drop_adjoint: bad arguments (gamma 7, MOG or no density diffusion)");
  SPH_REQUIRE(lx0 != lx1 && lv0 != lv1 && lr0 != lr1, "drop_adjoint: outputs must not alias inputs");
  if (n == 0) return SPH_OK;
  const int mog = params->density_diffusion == 1;
  cudaStream_t st = as_stream(stream);
  if (fp64)
    k_drop_adjoint<double, double2><<<grid_for(n, 128), 128, 0, st>>>(
        (int)n, offsets, cols, static_cast<const double2*>(x), static_cast<const double2*>(v),
        static_cast<const double*>(rho), static_cast<const double*>(area), drop_params<double>(params, mog), dt,
        static_cast<const double2*>(lx1), static_cast<const double2*>(lv1), static_cast<const double*>(lr1),
        static_cast<double2*>(lx0), static_cast<double2*>(lv0), static_cast<double*>(lr0),
        static_cast<double*>(dalpha));
  else
    k_drop_adjoint<float, float2><<<grid_for(n, 128), 128, 0, st>>>(
        (int)n, offsets, cols, static_cast<const float2*>(x), static_cast<const float2*>(v),
        static_cast<const float*>(rho), static_cast<const float*>(area), drop_params<float>(params, mog), (float)dt,
        static_cast<const float2*>(lx1), static_cast<const float2*>(lv1), static_cast<const float*>(lr1),
        static_cast<float2*>(lx0), static_cast<float2*>(lv0), static_cast<float*>(lr0), static_cast<float*>(dalpha));
  SPH_CHECK_LAUNCH("drop_adjoint");
  return SPH_OK;
}

}  // extern "C"
