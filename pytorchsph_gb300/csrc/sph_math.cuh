// Device math of the SPH summations: Wendland C2 / spiky kernels (src/kernels.py:20-33),
// pair geometry (src/modules/neighborSearch.py:218-223), the reference's closed-form 2x2
// pseudo-inverse (src/util.py:386-433) and a 3x3 pseudo-inverse for mDBC.
#pragma once

#include "sph_common.cuh"

namespace sph {

// Parameters shared by every summation kernel (by value in the launch).
struct SphParams {
  float h, inv_h;
  float thr;        // sq_threshold(h): the pair test v <= thr for support h
  float c_w;        // 7 / (pi h^2)           Wendland W
  float c_g;        // 7 / (pi h^3)           Wendland gradient (times 20 q (1-q)^3)
  float c_s;        // 30 / (pi h^3)          spiky gradient
  float gk;         // -20 c_g / h: gradW = gk (1 - q)^3 (x_i - x_j)
  float eps;        // 0.1 h^2
  float rho0, c0, gamma;
  float tait_k;     // rho0 c0^2 / gamma
  float visc_k;     // h alpha c0
  float diff_k;     // h delta c0
  float kinematic;
  float gx, gy;     // constant gravity
  int point_source; // gravity = -g (x - c)  (potential field)
  float point_mag, point_cx, point_cy;
  int diffusion;    // 0 none, 1 MOG, 2 deltaSPH
  int boundary_diffusion;
  int search_radius;
  int cell_capacity;
};

// Wall particles, sorted by their cell in the fluid grid; quantities per sorted wall.
struct WallView {
  const float2* x;         // wall positions
  const float2* xg;        // ghost positions
  const float* area;       // boundaryVolume (pi r^2)
  const int32_t* cell_start;  // wall cell table in the fluid grid (cells+2)
  int n;
  float* rho;              // relative wall density
  float* vol;              // A_b / rho_b
  float* p;                // wall pressure
};

__device__ __forceinline__ float kW(float q, float c_w) {
  float a = 1.0f - q;
  float a2 = a * a;
  return a2 * a2 * (1.0f + 4.0f * q) * c_w;
}

// gradW = e * kGW(q): Wendland gradient magnitude factor -C/h^3 * 20 q (1-q)^3.
__device__ __forceinline__ float kGW(float q, float c_g) {
  float a = 1.0f - q;
  return -c_g * 20.0f * q * a * a * a;
}

// spikyGrad = e * kGS(q): -30/(pi h^3) (1-q)^2.
__device__ __forceinline__ float kGS(float q, float c_s) {
  float a = 1.0f - q;
  return -c_s * a * a;
}

// Approximate reciprocal square root and reciprocal of a positive NORMAL float (every caller
// passes a value >= 1e-30): the same hardware approximation as rsqrtf(x) and
// __fdividef(1, x), in their .ftz forms, which skip the scaling that the default forms wrap
// around it for subnormal inputs.  For normal inputs the results are the same.
__device__ __forceinline__ float rsqrt_normal(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rcp_normal(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

struct Geo {
  float dx, dy;   // x_row - x_col
  float r, q;
  float ex, ey;   // unit vector, 0 when r < 1e-7
};

__device__ __forceinline__ Geo geo(float xi, float yi, float xj, float yj, float inv_h) {
  Geo g;
  g.dx = xi - xj;
  g.dy = yi - yj;
  g.r = sqrtf(g.dx * g.dx + g.dy * g.dy);
  if (g.r >= 1e-7f) {
    float ir = 1.0f / g.r;
    g.ex = g.dx * ir;
    g.ey = g.dy * ir;
  } else {
    g.ex = 0.f;
    g.ey = 0.f;
  }
  g.q = g.r * inv_h;
  return g;
}

__device__ __forceinline__ float tait(float rho_rel, const SphParams& P) {
  float r7;
  if (P.gamma == 7.0f) {
    float r2 = rho_rel * rho_rel;
    float r4 = r2 * r2;
    r7 = r4 * r2 * rho_rel;
  } else {
    r7 = powf(rho_rel, P.gamma);
  }
  return P.tait_k * (r7 - 1.0f);
}

// pinv2x2, src/util.py:386-433: closed-form SVD pseudo-inverse, singular values <= 1e-5
// dropped.  M = [[a, b], [c, d]]; returns [[o00, o01], [o10, o11]] in a float4 (row major).
__device__ __forceinline__ float4 pinv2x2(float a, float b, float c, float d) {
  float theta = 0.5f * atan2f(2 * a * c + 2 * b * d, a * a + b * b - c * c - d * d);
  float ct = cosf(theta), st = sinf(theta);
  float S1 = a * a + b * b + c * c + d * d;
  float t = a * a + b * b - c * c - d * d;
  float u = a * c + b * d;
  float S2 = sqrtf(t * t + 4 * u * u);
  float o1 = sqrtf((S1 + S2) * 0.5f);
  float o2 = sqrtf((S1 - S2) * 0.5f);
  float phi = 0.5f * atan2f(2 * a * b + 2 * c * d, a * a - b * b + c * c - d * d);
  float cp = cosf(phi), sp = sinf(phi);
  float v1 = (a * ct + c * st) * cp + (b * ct + d * st) * sp;
  float v2 = (a * st - c * ct) * sp + (-b * st + d * ct) * cp;
  float s11 = (v1 > 0.f) ? 1.f : ((v1 < 0.f) ? -1.f : 0.f);
  float s22 = (v2 > 0.f) ? 1.f : ((v2 < 0.f) ? -1.f : 0.f);
  // V = [[cp s11, -sp s22], [sp s11, cp s22]]; U = [[ct, -st], [st, ct]]
  float i1 = fabsf(o1) > 1e-5f ? 1.0f / o1 : 0.f;
  float i2 = fabsf(o2) > 1e-5f ? 1.0f / o2 : 0.f;
  // V S^-1 = [[cp s11 i1, -sp s22 i2], [sp s11 i1, cp s22 i2]]; times U^T = [[ct, st], [-st, ct]]
  float m00 = cp * s11 * i1, m01 = -sp * s22 * i2, m10 = sp * s11 * i1, m11 = cp * s22 * i2;
  return make_float4(m00 * ct - m01 * st, m00 * st + m01 * ct, m10 * ct - m11 * st, m10 * st + m11 * ct);
}

// pinv2x2 of a well-conditioned M: there the pseudo-inverse is the inverse adj(M) / det, a
// few operations instead of the closed form's atan2 / cos / sin.  With S1 = |M|_F^2 and
// sigma_max^2 = (S1 + sqrt(S1^2 - 4 det^2)) / 2 (no cancellation), sigma_min^2 = det^2 /
// sigma_max^2.  Taken when sigma_min > 0.1 sigma_max and sigma_min > 2e-5 (twice the 1e-5
// cutoff): there the closed form in float32 is itself within ~1e-5 of the inverse (its small
// singular value carries a relative error of ~FLT_EPSILON (sigma_max / sigma_min)^2).  Any
// other M (free-surface particles, non-finite input) goes through pinv2x2.
__device__ __forceinline__ float4 pinv2x2_fast(float a, float b, float c, float d) {
  const float det = a * d - b * c;
  const float S1 = a * a + b * b + c * c + d * d;
  const float s1sq = 0.5f * (S1 + sqrtf(fmaxf(S1 * S1 - 4.0f * det * det, 0.0f)));
  const float d2 = det * det;
  if (d2 > 0.01f * s1sq * s1sq && d2 > 4e-10f * s1sq && isfinite(d2)) {
    const float id = 1.0f / det;
    return make_float4(d * id, -b * id, -c * id, a * id);
  }
  return pinv2x2(a, b, c, d);
}

// x = pinv(A) b for a 3x3 A in double (torch.linalg.pinv semantics: singular values below
// 3 * FLT_EPSILON * sigma_max are dropped).  Eigen-decomposition of A^T A by cyclic Jacobi
// rotations (at most 16 sweeps), then pinv(A) b = sum_k v_k ((A v_k) . b) / sigma_k^2.
// Kept out of line: its arrays would otherwise set the register count of every caller's
// common path (pinv3_solve below).
static __device__ __noinline__ void pinv3_solve_jacobi(const double A[3][3], const double b[3], double x[3]) {
  double S[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) S[r][c] = A[0][r] * A[0][c] + A[1][r] * A[1][c] + A[2][r] * A[2][c];
  double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 16; ++sweep) {
    double off = fabs(S[0][1]) + fabs(S[0][2]) + fabs(S[1][2]);
    double diag = fabs(S[0][0]) + fabs(S[1][1]) + fabs(S[2][2]);
    if (off <= 1e-300 || off <= 1e-17 * diag) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = S[p][q];
        if (fabs(apq) <= 1e-300) continue;
        double tau = (S[q][q] - S[p][p]) / (2.0 * apq);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < 3; ++k) {  // S = J^T S J
          double skp = S[k][p], skq = S[k][q];
          S[k][p] = c * skp - s * skq;
          S[k][q] = s * skp + c * skq;
        }
        for (int k = 0; k < 3; ++k) {
          double spk = S[p][k], sqk = S[q][k];
          S[p][k] = c * spk - s * sqk;
          S[q][k] = s * spk + c * sqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  double lmax = fmax(fmax(S[0][0], S[1][1]), S[2][2]);
  double smax = sqrt(fmax(lmax, 0.0));
  double tol = 3.0 * 1.1920928955078125e-07 * smax;
  x[0] = x[1] = x[2] = 0.0;
  for (int k = 0; k < 3; ++k) {
    double sig = sqrt(fmax(S[k][k], 0.0));
    if (!(sig > tol)) continue;
    double av[3];
    for (int r = 0; r < 3; ++r) av[r] = A[r][0] * V[0][k] + A[r][1] * V[1][k] + A[r][2] * V[2][k];
    double coef = (av[0] * b[0] + av[1] * b[1] + av[2] * b[2]) / (sig * sig);
    for (int r = 0; r < 3; ++r) x[r] += V[r][k] * coef;
  }
}

__device__ inline void pinv3_solve(const double A[3][3], const double b[3], double x[3]) {
  // Well-conditioned A (Frobenius condition bound ||A|| ||A^-1|| below 1e5, far under the
  // 1/(3 FLT_EPSILON) at which a singular value would be dropped): pinv(A) = A^-1, applied
  // through the adjugate.  This is the common case and costs ~50 double operations instead
  // of the Jacobi sweeps (GB300's FP64 rate is low).
  {
    // cofactors a*b - c*d as fma(a, b, -(c*d)): two double operations each
    const auto cof = [](double a, double b, double c, double d) { return fma(a, b, -(c * d)); };
    const double c00 = cof(A[1][1], A[2][2], A[1][2], A[2][1]), c01 = cof(A[1][2], A[2][0], A[1][0], A[2][2]),
                 c02 = cof(A[1][0], A[2][1], A[1][1], A[2][0]);
    const double c10 = cof(A[0][2], A[2][1], A[0][1], A[2][2]), c11 = cof(A[0][0], A[2][2], A[0][2], A[2][0]),
                 c12 = cof(A[0][1], A[2][0], A[0][0], A[2][1]);
    const double c20 = cof(A[0][1], A[1][2], A[0][2], A[1][1]), c21 = cof(A[0][2], A[1][0], A[0][0], A[1][2]),
                 c22 = cof(A[0][0], A[1][1], A[0][1], A[1][0]);
    const double det = fma(A[0][0], c00, fma(A[0][1], c01, A[0][2] * c02));
    // The bound only decides between two exact-enough paths: its norms run in float, on A
    // scaled by its largest entry (cofactors by its square, det by its cube), so that the
    // squares neither underflow nor overflow whatever the matrix's scale (MLS moment
    // matrices with volumes A / rho0 have entries near 1e-12).
    double amax = 0.0;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) amax = fmax(amax, fabs(A[r][c]));
    const double is = amax > 0.0 ? 1.0 / amax : 0.0, is2 = is * is;
    float na = 0.f;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const float v = (float)(A[r][c] * is);
        na += v * v;
      }
    const float f00 = (float)(c00 * is2), f01 = (float)(c01 * is2), f02 = (float)(c02 * is2),
                f10 = (float)(c10 * is2), f11 = (float)(c11 * is2), f12 = (float)(c12 * is2),
                f20 = (float)(c20 * is2), f21 = (float)(c21 * is2), f22 = (float)(c22 * is2);
    const float nc = f00 * f00 + f01 * f01 + f02 * f02 + f10 * f10 + f11 * f11 + f12 * f12 + f20 * f20 +
                     f21 * f21 + f22 * f22;
    const double ds = det * is2 * is;
    // ||A^-1||_F = ||adj A||_F / |det|, all three scaled alike
    if (det != 0.0 && amax > 0.0 && (double)na * (double)nc < 1e10 * ds * ds) {
      const double id = 1.0 / det;  // A^-1 = adj(A) / det, adj(A)[r][c] = cofactor c_cr
      x[0] = fma(c00, b[0], fma(c10, b[1], c20 * b[2])) * id;
      x[1] = fma(c01, b[0], fma(c11, b[1], c21 * b[2])) * id;
      x[2] = fma(c02, b[0], fma(c12, b[1], c22 * b[2])) * id;
      return;
    }
  }
  pinv3_solve_jacobi(A, b, x);
}

// Iterate the wall particles whose cell is within +-r of fluid cell (cx, cy) and that pass
// the wall-side predicate sqrtf(fmaf(dx,dx,dy*dy)) < h_b with dx = x_b - x_f: exactly the
// wall->fluid pairs of searchExisting (src/modules/neighborSearch.py:231-252).
// `coff` is the scene's first slot in the (batched) cell tables; 0 for a single scene.
template <typename F>
__device__ __forceinline__ void for_each_wall(const WallView& W, const sph_grid& g, int r, int cx, int cy, float xf,
                                              float yf, float thr_b, F&& f, int coff = 0) {
  const int x0 = max(cx - r, 0), x1 = min(cx + r, g.cells_x - 1);
  if (x0 > x1) return;
  const int y0 = max(cy - r, 0), y1 = min(cy + r, g.cells_y - 1);
  const int32_t* cs = W.cell_start + coff;
  for (int yy = y0; yy <= y1; ++yy) {
    const int row = yy * g.cells_x;
    const int b0 = __ldg(cs + row + x0), b1 = __ldg(cs + row + x1 + 1);
    for (int b = b0; b < b1; ++b) {
      const float2 xb = __ldg(W.x + b);
      if (dist2_ref(xb.x, xb.y, xf, yf) <= thr_b) f(b, xb);
    }
  }
}

// ---------------------------------------------------------------- candidate segments
// The candidates of a particle in one cell row are a contiguous sorted range; it is tested
// in segments of 32 candidates into bit masks (bit t: candidate c + t passes the pair test),
// and a particle keeps its non-empty segments, at most kMaxSegments, as (start, mask) pairs.
constexpr int kMaxSegments = 8;

// One candidate per step (the force passes' rare fallback for a particle whose segments
// did not fit).
__device__ __forceinline__ uint32_t segment_mask_scalar(const float2* __restrict__ x, int c, int e, float xi,
                                                        float yi, float thr) {
  const int len = min(e - c, 32);
  uint32_t m = 0;
  for (int t = 0; t < len; ++t) {
    const float2 pj = __ldg(x + c + t);
    m |= (uint32_t)(dist2_ref(xi, yi, pj.x, pj.y) <= thr) << t;
  }
  return m;
}

// Two candidates per step with the paired float32 instructions (per component the same
// round-to-nearest operations as dist2_ref: x_i - x_j as x_i + (-x_j), which IEEE
// arithmetic makes identical, so the pair test is unchanged bit for bit).
__device__ __forceinline__ uint32_t segment_mask(const float2* __restrict__ x, int c, int e, float xi, float yi,
                                                 float thr) {
  const int len = min(e - c, 32);
  uint32_t m = 0;
  const float2 qx = make_float2(xi, xi), qy = make_float2(yi, yi);
  // unrolled over the segment's 16 candidate pairs, each guarded by the length: every bit
  // position is a constant, so a candidate costs its test and one predicated OR
#pragma unroll
  for (int t = 0; t < 32; t += 2) {
    if (t + 1 < len) {
      const float2 a = __ldg(x + c + t), b = __ldg(x + c + t + 1);
      const float2 dx = __fadd2_rn(qx, make_float2(-a.x, -b.x));
      const float2 dy = __fadd2_rn(qy, make_float2(-a.y, -b.y));
      const float2 v = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
      if (v.x <= thr) m |= 1u << t;
      if (v.y <= thr) m |= 2u << t;
    } else if (t < len) {
      const float2 a = __ldg(x + c + t);
      if (dist2_ref(xi, yi, a.x, a.y) <= thr) m |= 1u << t;
    }
  }
  return m;
}

// segment_mask when c + 32 <= n (the array's length): every candidate load is in bounds, so
// all 32 candidates are tested without per-pair guards (all loads can be in flight
// together) and the bits past the range are cleared; the bits inside it are segment_mask's.
__device__ __forceinline__ uint32_t segment_mask_full(const float2* __restrict__ x, int c, int e, float xi,
                                                      float yi, float thr) {
  const int len = min(e - c, 32);
  uint32_t m = 0;
  const float2 qx = make_float2(xi, xi), qy = make_float2(yi, yi);
#pragma unroll
  for (int t = 0; t < 32; t += 2) {
    const float2 a = __ldg(x + c + t), b = __ldg(x + c + t + 1);
    const float2 dx = __fadd2_rn(qx, make_float2(-a.x, -b.x));
    const float2 dy = __fadd2_rn(qy, make_float2(-a.y, -b.y));
    const float2 v = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
    if (v.x <= thr) m |= 1u << t;
    if (v.y <= thr) m |= 2u << t;
  }
  return len >= 32 ? m : m & ((1u << len) - 1u);
}

// The bits of a stored segment that name a particle: none for a start outside [0, n),
// none at index n or past it.
__device__ __forceinline__ uint32_t clip_segment(uint32_t w, int b, int n) {
  if ((unsigned)b >= (unsigned)n) return 0;
  return n - b < 32 ? w & ((1u << (n - b)) - 1) : w;
}

struct FluidView {
  const float2* x;
  const float2* v;
  const float* rho;
  const float* area;
  const uint32_t* keys;
  const int32_t* offsets;
  const int32_t* cols;
  const int32_t* cell_start;
  int n;
  int pair_cap;  // 0: cols holds every row
};

// End of particle i's CSR row [offsets[i], end): a row that ends past the column buffer was
// not filled and reads as empty, so no kernel reads a column that was never written.
__device__ __forceinline__ int row_end(const FluidView& F, int i, int k0) {
  const int k1 = F.offsets[i + 1];
  return (F.pair_cap > 0 && k1 > F.pair_cap) ? k0 : k1;
}

// Cell coordinates of a grid key.  A key past the grid (a particle outside its grid) gives a
// row far below the grid, so that every +-r cell window around it is empty.
__device__ __forceinline__ void cell_of(uint32_t key, const sph_grid& g, int* cx, int* cy) {
  if (key >= (uint32_t)g.num_cells) {
    *cx = 0;
    *cy = -(1 << 20);
    return;
  }
  *cx = (int)(key % (uint32_t)g.cells_x);
  *cy = (int)(key / (uint32_t)g.cells_x);
}

}  // namespace sph

// Host-side conversions of the C-ABI views into the kernels' views.
namespace sph {
// One scene of a batch as the kernels see it: derived parameters, its search grid, its
// first slot in the concatenated cell tables and its time step.
struct SceneDev {
  SphParams P;
  sph_grid g;
  int coff;
  float dt;
};

static inline SphParams to_params(const sph_params* p) {
  SphParams P;
  P.h = p->support;
  P.inv_h = 1.0f / p->support;
  P.thr = sq_threshold(p->support);
  const double h = p->support;
  P.c_w = (float)(7.0 / 3.14159265358979323846 / (h * h));
  P.c_g = (float)(7.0 / 3.14159265358979323846 / (h * h * h));
  P.c_s = (float)(30.0 / 3.14159265358979323846 / (h * h * h));
  P.gk = (float)(-20.0 * 7.0 / 3.14159265358979323846 / (h * h * h * h));
  P.eps = (float)(h * h * 0.1);
  P.rho0 = p->rest_density;
  P.c0 = p->c0;
  P.gamma = p->gamma;
  P.tait_k = (float)((double)p->rest_density * p->c0 * p->c0 / p->gamma);
  P.visc_k = (float)(h * p->alpha * p->c0);
  P.diff_k = (float)(h * p->delta * p->c0);
  P.kinematic = p->kinematic;
  P.gx = p->gravity[0];
  P.gy = p->gravity[1];
  P.point_source = p->point_source;
  P.point_mag = p->point_magnitude;
  P.point_cx = p->point_center[0];
  P.point_cy = p->point_center[1];
  P.diffusion = p->density_diffusion;
  P.boundary_diffusion = p->boundary_diffusion;
  P.search_radius = p->search_radius;
  P.cell_capacity = p->cell_capacity;
  return P;
}

static inline FluidView to_fluid(const sph_fluid_view* f) {
  FluidView F;
  F.x = reinterpret_cast<const float2*>(f->x);
  F.v = reinterpret_cast<const float2*>(f->v);
  F.rho = f->rho;
  F.area = f->area;
  F.keys = f->keys;
  F.offsets = f->offsets;
  F.cols = f->cols;
  F.cell_start = f->cell_start;
  F.n = (int)f->n;
  F.pair_cap = f->pair_capacity > 0x7fffffff ? 0x7fffffff : (int)f->pair_capacity;
  return F;
}

static inline WallView to_walls(const sph_wall_view* w) {
  WallView W;
  W.x = reinterpret_cast<const float2*>(w->x);
  W.xg = reinterpret_cast<const float2*>(w->ghost);
  W.area = w->area;
  W.cell_start = w->cell_start;
  W.n = (int)w->n;
  W.rho = w->rho;
  W.vol = w->volume;
  W.p = w->pressure;
  return W;
}

}  // namespace sph

#define SPH_VIEW_CHECK(f) SPH_REQUIRE((f) && (f)->n >= 0 && (f)->n < (1LL << 31), "bad particle view")
