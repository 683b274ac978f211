/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the reference's
 * hashed-grid neighbor search and density summation (wi-re/pytorchSPH), used by the
 * tests as the checker for the CUDA path and by bench.py as the timed CPU baseline.
 * Nothing in the product links or calls this file.
 *
 * Functions and the reference code each one restates:
 *   oracle_sort_positions   src/modules/neighborSearch.py:30-55   (sortPositions)
 *   oracle_hash_map         src/modules/neighborSearch.py:58-88   (constructHashMap)
 *   query_cell              cppSrc/neighSearch.cpp:93-114         (queryHashMap)
 *   oracle_nl_cells         cppSrc/neighSearch.cpp:172-259        (buildNeighborList)
 *   oracle_nl_query         cppSrc/neighSearch.cpp:261-331        (buildNeighborListUnsortedPerParticle;
 *                           the CUDA path cppSrc/neighSearch_cuda.cu:101-209 has the same pair set)
 *   oracle_nl_asym          cppSrc/neighSearch.cpp:333-410        (buildNeighborListAsymmetric)
 *   oracle_canonical_csr    src/modules/neighborSearch.py:153-157 (finalize: pairs ordered by (i, j))
 *   oracle_density          src/modules/density.py:26-30 with src/kernels.py:20-24 (Wendland C2)
 *
 * Pair predicate.  The reference tests `sqrt(dx*dx + dy*dy) < h_i` on floats with
 * dx = x_i - x_j (i = query).  Compiled with the reference's flags
 * (-O3 -march=native, GCC, FMA-capable host) GCC contracts the sum into
 * fmaf(dx, dx, dy*dy); the CUDA path spells exactly that form out.  The oracle keeps
 * the alternative spellings selectable (`pred`) so the tests can show which one the
 * compiled reference follows.  This file is compiled with -ffp-contract=off so that
 * each spelling means what it says.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { PRED_FMA_XX = 0, PRED_FMA_YY = 1, PRED_UNFUSED = 2, PRED_DOUBLE_SQRT = 3 };

static inline int pair_pred(float xi0, float xi1, float xj0, float xj1, float hi, int pred) {
  float dx = xi0 - xj0;
  float dy = xi1 - xj1;
  switch (pred) {
    case PRED_FMA_YY: return sqrtf(fmaf(dy, dy, dx * dx)) < hi;
    case PRED_UNFUSED: { float a = dx * dx; float b = dy * dy; return sqrtf(a + b) < hi; }
    case PRED_DOUBLE_SQRT: { float a = dx * dx; float b = dy * dy; return sqrt((double)(a + b)) < (double)hi; }
    default: return sqrtf(fmaf(dx, dx, dy * dy)) < hi;
  }
}

/* ---------------------------------------------------------------- sortPositions */
/* hMax = max(h); qMin = (minCoord or min(pos)) - hMax; qMax = (maxCoord or max(pos)) + 2 hMax;
 * cellCount = ceil((qMax - qMin) / hMax); idx = ceil((x - qMin) / hMax); lin = ix + cellsX * iy;
 * order = stable argsort(lin).  All arithmetic in float32 like the torch code. */
int oracle_sort_positions(const float* pos, const float* h, int64_t n, const float* min_coord,
                          const float* max_coord, float* qmin_out, float* hmax_out,
                          int32_t* cells_out, int32_t* lin_out, int64_t* order_out) {
  if (n <= 0) return -1;
  float hmax = h[0];
  float mn[2] = {pos[0], pos[1]}, mx[2] = {pos[0], pos[1]};
  for (int64_t i = 0; i < n; ++i) {
    if (h[i] > hmax) hmax = h[i];
    for (int d = 0; d < 2; ++d) {
      float v = pos[2 * i + d];
      if (v < mn[d]) mn[d] = v;
      if (v > mx[d]) mx[d] = v;
    }
  }
  float hs = hmax * 1.0f;     /* hMax * supportScale (supportScale = 1.0) */
  float two_hs = 2.0f * hmax; /* 2 * hMax * supportScale */
  two_hs = two_hs * 1.0f;
  float qmin[2], qmax[2];
  for (int d = 0; d < 2; ++d) {
    qmin[d] = (min_coord ? min_coord[d] : mn[d]) - hs;
    qmax[d] = (max_coord ? max_coord[d] : mx[d]) + two_hs;
    float ext = qmax[d] - qmin[d];
    cells_out[d] = (int32_t)ceilf(ext / hs);
    qmin_out[d] = qmin[d];
  }
  *hmax_out = hmax;
  int32_t cx = cells_out[0];
  for (int64_t i = 0; i < n; ++i) {
    int32_t ix = (int32_t)ceilf((pos[2 * i] - qmin[0]) / hmax);
    int32_t iy = (int32_t)ceilf((pos[2 * i + 1] - qmin[1]) / hmax);
    lin_out[i] = ix + cx * iy;
  }
  /* stable counting-free argsort: LSD radix on (lin + 2^31) in 4 byte passes */
  int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * n);
  uint32_t* key = (uint32_t*)malloc(sizeof(uint32_t) * n);
  if (!tmp || !key) { free(tmp); free(key); return -2; }
  for (int64_t i = 0; i < n; ++i) { order_out[i] = i; }
  for (int64_t i = 0; i < n; ++i) key[i] = (uint32_t)lin_out[i] ^ 0x80000000u;
  for (int pass = 0; pass < 4; ++pass) {
    int64_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    int sh = pass * 8;
    for (int64_t i = 0; i < n; ++i) cnt[((key[order_out[i]] >> sh) & 255u) + 1]++;
    for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
    for (int64_t i = 0; i < n; ++i) {
      int64_t o = order_out[i];
      tmp[cnt[(key[o] >> sh) & 255u]++] = o;
    }
    memcpy(order_out, tmp, sizeof(int64_t) * n);
  }
  free(tmp);
  free(key);
  return 0;
}

/* ---------------------------------------------------------------- constructHashMap */
/* cells = unique_consecutive(sortedLin) with counts; begins = exclusive cumsum of counts;
 * hash = (3*ix + 5*iy) % L with ix = lin % cellsX, iy = lin / cellsX (trunc);
 * cells re-ordered by a stable argsort of hash; table[hash] = (first slot, #cells). */
int64_t oracle_hash_map(const int32_t* sorted_lin, int64_t n, int32_t cells_x, int32_t L,
                        int32_t* table /*[L,2]*/, int32_t* cell_indices, int32_t* cum_cell,
                        int32_t* cell_span) {
  int64_t C = 0;
  int32_t* ci = (int32_t*)malloc(sizeof(int32_t) * (n + 1));
  int32_t* cc = (int32_t*)malloc(sizeof(int32_t) * (n + 1));
  int32_t* cs = (int32_t*)malloc(sizeof(int32_t) * (n + 1));
  int64_t* hs = (int64_t*)malloc(sizeof(int64_t) * (n + 1));
  if (!ci || !cc || !cs || !hs) return -1;
  for (int64_t i = 0; i < n; ++i) {
    if (i == 0 || sorted_lin[i] != sorted_lin[i - 1]) {
      ci[C] = sorted_lin[i];
      cc[C] = 0;
      cs[C] = (int32_t)i;
      ++C;
    }
    cc[C - 1]++;
  }
  for (int64_t c = 0; c < C; ++c) {
    /* torch integer % and div(rounding_mode='trunc') on non-negative ids */
    int64_t x = ci[c] % cells_x, y = ci[c] / cells_x;
    int64_t hv = (x * 3 + y * 5) % L;
    if (hv < 0) hv += L;
    hs[c] = hv;
  }
  /* stable sort of cells by hash (insertion into buckets) */
  int64_t* cnt = (int64_t*)calloc((size_t)L + 1, sizeof(int64_t));
  int64_t* ord = (int64_t*)malloc(sizeof(int64_t) * (C + 1));
  if (!cnt || !ord) return -1;
  for (int64_t c = 0; c < C; ++c) cnt[hs[c] + 1]++;
  for (int64_t b = 0; b < L; ++b) cnt[b + 1] += cnt[b];
  for (int64_t b = 0; b < L; ++b) { table[2 * b] = -1; table[2 * b + 1] = 0; }
  for (int64_t b = 0; b < L; ++b) {
    int64_t k = cnt[b + 1] - cnt[b];
    if (k > 0) { table[2 * b] = (int32_t)cnt[b]; table[2 * b + 1] = (int32_t)k; }
  }
  int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * ((size_t)L + 1));
  memcpy(pos, cnt, sizeof(int64_t) * ((size_t)L + 1));
  for (int64_t c = 0; c < C; ++c) ord[pos[hs[c]]++] = c;
  for (int64_t k = 0; k < C; ++k) {
    int64_t c = ord[k];
    cell_indices[k] = ci[c];
    cum_cell[k] = cc[c];   /* counts (reference name: cumCell) */
    cell_span[k] = cs[c];  /* begins (reference name: cellSpan) */
  }
  free(ci); free(cc); free(cs); free(hs); free(cnt); free(ord); free(pos);
  return C;
}

/* queryHashMap: (ix,iy) -> [begin,end) or (-1,-1) */
static inline void query_cell(int32_t qx, int32_t qy, const int32_t* table, const int32_t* cell_indices,
                              const int32_t* cum_cell, const int32_t* cell_span, int32_t cells_x,
                              int32_t L, int32_t* b, int32_t* e) {
  *b = -1; *e = -1;
  if (qx < 0 || qy < 0) return;
  int32_t qlin = qx + cells_x * qy;
  int32_t qh = (qx * 3 + qy * 5) % L;
  int32_t first = table[2 * qh];
  if (first == -1) return;
  int32_t last = first + table[2 * qh + 1];
  for (int32_t k = first; k < last; ++k) {
    if (cell_indices[k] == qlin) { *b = cell_span[k]; *e = cell_span[k] + cum_cell[k]; return; }
  }
}

/* growable per-thread pair buffer */
typedef struct { int32_t* r; int32_t* c; int64_t n, cap; } pairbuf;
static int pb_push(pairbuf* p, int32_t r, int32_t c) {
  if (p->n == p->cap) {
    int64_t nc = p->cap ? p->cap * 2 : 4096;
    int32_t* nr = (int32_t*)realloc(p->r, sizeof(int32_t) * nc);
    int32_t* ncc = (int32_t*)realloc(p->c, sizeof(int32_t) * nc);
    if (!nr || !ncc) return -1;
    p->r = nr; p->c = ncc; p->cap = nc;
  }
  p->r[p->n] = r; p->c[p->n] = c; p->n++;
  return 0;
}

static int64_t merge_bufs(pairbuf* bufs, int nb, int32_t** rows, int32_t** cols) {
  int64_t tot = 0;
  for (int t = 0; t < nb; ++t) tot += bufs[t].n;
  *rows = (int32_t*)malloc(sizeof(int32_t) * (tot > 0 ? tot : 1));
  *cols = (int32_t*)malloc(sizeof(int32_t) * (tot > 0 ? tot : 1));
  int64_t off = 0;
  for (int t = 0; t < nb; ++t) {
    if (bufs[t].n) {
      memcpy(*rows + off, bufs[t].r, sizeof(int32_t) * bufs[t].n);
      memcpy(*cols + off, bufs[t].c, sizeof(int32_t) * bufs[t].n);
    }
    off += bufs[t].n;
    free(bufs[t].r); free(bufs[t].c);
  }
  free(bufs);
  return tot;
}

static int n_threads(int req) {
#ifdef _OPENMP
  return req > 0 ? req : omp_get_max_threads();
#else
  (void)req; return 1;
#endif
}

/* buildNeighborList: for every occupied cell (hash order), every neighbor cell, every i, j. */
int64_t oracle_nl_cells(const float* sorted_pos, const float* sorted_h, const int32_t* table,
                        const int32_t* cell_indices, const int32_t* cum_cell, const int32_t* cell_span,
                        const int32_t* sort, int64_t C, int32_t cells_x, int32_t L, int32_t radius,
                        int pred, int threads, int32_t** rows, int32_t** cols) {
  int nt = n_threads(threads);
  pairbuf* bufs = (pairbuf*)calloc(nt, sizeof(pairbuf));
  int fail = 0;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    pairbuf* pb = &bufs[t];
#pragma omp for schedule(static)
    for (int64_t b = 0; b < C; ++b) {
      int32_t cell = cell_indices[b];
      int32_t qx = cell % cells_x, qy = cell / cells_x;
      int32_t ib, ie;
      query_cell(qx, qy, table, cell_indices, cum_cell, cell_span, cells_x, L, &ib, &ie);
      for (int32_t xx = -radius; xx <= radius; ++xx)
        for (int32_t yy = -radius; yy <= radius; ++yy) {
          int32_t jb, je;
          query_cell(qx + xx, qy + yy, table, cell_indices, cum_cell, cell_span, cells_x, L, &jb, &je);
          if (jb == -1) continue;
          for (int32_t i = ib; i < ie; ++i) {
            float xi0 = sorted_pos[2 * i], xi1 = sorted_pos[2 * i + 1], hi = sorted_h[i];
            for (int32_t j = jb; j < je; ++j)
              if (pair_pred(xi0, xi1, sorted_pos[2 * j], sorted_pos[2 * j + 1], hi, pred))
                if (pb_push(pb, sort[i], sort[j])) fail = 1;
          }
        }
    }
  }
  int64_t tot = merge_bufs(bufs, nt, rows, cols);
  return fail ? -1 : tot;
}

/* buildNeighborListUnsortedPerParticle (and the CUDA path's pair set): query points vs grid. */
int64_t oracle_nl_query(const float* qpos, const float* qh, int64_t m, const float* sorted_pos,
                        const int32_t* table, const int32_t* cell_indices, const int32_t* cum_cell,
                        const int32_t* cell_span, const int32_t* sort, int32_t cells_x, int32_t L,
                        const float* qmin, float hmax, int32_t radius, int pred, int threads,
                        int32_t** rows, int32_t** cols) {
  int nt = n_threads(threads);
  pairbuf* bufs = (pairbuf*)calloc(nt, sizeof(pairbuf));
  int fail = 0;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    pairbuf* pb = &bufs[t];
#pragma omp for schedule(static)
    for (int64_t b = 0; b < m; ++b) {
      float xi0 = qpos[2 * b], xi1 = qpos[2 * b + 1], hi = qh[b];
      int32_t qx = (int32_t)ceilf((xi0 - qmin[0]) / hmax);
      int32_t qy = (int32_t)ceilf((xi1 - qmin[1]) / hmax);
      for (int32_t xx = -radius; xx <= radius; ++xx)
        for (int32_t yy = -radius; yy <= radius; ++yy) {
          int32_t jb, je;
          query_cell(qx + xx, qy + yy, table, cell_indices, cum_cell, cell_span, cells_x, L, &jb, &je);
          if (jb == -1) continue;
          for (int32_t j = jb; j < je; ++j)
            if (pair_pred(xi0, xi1, sorted_pos[2 * j], sorted_pos[2 * j + 1], hi, pred))
              if (pb_push(pb, (int32_t)b, sort[j])) fail = 1;
        }
    }
  }
  int64_t tot = merge_bufs(bufs, nt, rows, cols);
  return fail ? -1 : tot;
}

/* buildNeighborListAsymmetric: cells of set A (query) against the grid of set B, radius 1. */
int64_t oracle_nl_asym(const float* pos_a, const float* h_a, const int32_t* table_a,
                       const int32_t* ci_a, const int32_t* cc_a, const int32_t* cs_a, const int32_t* sort_a,
                       int64_t C_a, const float* pos_b, const int32_t* table_b, const int32_t* ci_b,
                       const int32_t* cc_b, const int32_t* cs_b, const int32_t* sort_b, int32_t cells_x,
                       int32_t L, int pred, int threads, int32_t** rows, int32_t** cols) {
  int nt = n_threads(threads);
  pairbuf* bufs = (pairbuf*)calloc(nt, sizeof(pairbuf));
  int fail = 0;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    pairbuf* pb = &bufs[t];
#pragma omp for schedule(static)
    for (int64_t b = 0; b < C_a; ++b) {
      int32_t cell = ci_a[b];
      int32_t qx = cell % cells_x, qy = cell / cells_x;
      int32_t ib, ie;
      query_cell(qx, qy, table_a, ci_a, cc_a, cs_a, cells_x, L, &ib, &ie);
      for (int32_t xx = -1; xx <= 1; ++xx)
        for (int32_t yy = -1; yy <= 1; ++yy) {
          int32_t jb, je;
          query_cell(qx + xx, qy + yy, table_b, ci_b, cc_b, cs_b, cells_x, L, &jb, &je);
          if (jb == -1) continue;
          for (int32_t i = ib; i < ie; ++i) {
            float xi0 = pos_a[2 * i], xi1 = pos_a[2 * i + 1], hi = h_a[i];
            for (int32_t j = jb; j < je; ++j)
              if (pair_pred(xi0, xi1, pos_b[2 * j], pos_b[2 * j + 1], hi, pred))
                if (pb_push(pb, sort_a[i], sort_b[j])) fail = 1;
          }
        }
    }
  }
  int64_t tot = merge_bufs(bufs, nt, rows, cols);
  return fail ? -1 : tot;
}

void oracle_free(void* p) { free(p); }

/* Pairs -> CSR over rows with columns ascending inside each row (the (i, j) order that the
 * reference's CUDA finalize produces with two stable sorts). */
int oracle_canonical_csr(const int32_t* rows, const int32_t* cols, int64_t P, int64_t n_rows,
                         int64_t* offsets /*[n_rows+1]*/, int32_t* cols_out /*[P]*/) {
  memset(offsets, 0, sizeof(int64_t) * (n_rows + 1));
  for (int64_t k = 0; k < P; ++k) {
    if (rows[k] < 0 || rows[k] >= n_rows) return -1;
    offsets[rows[k] + 1]++;
  }
  for (int64_t r = 0; r < n_rows; ++r) offsets[r + 1] += offsets[r];
  int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (n_rows + 1));
  memcpy(cur, offsets, sizeof(int64_t) * (n_rows + 1));
  for (int64_t k = 0; k < P; ++k) cols_out[cur[rows[k]]++] = cols[k];
  free(cur);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < n_rows; ++r) {
    int32_t* c = cols_out + offsets[r];
    int64_t len = offsets[r + 1] - offsets[r];
    for (int64_t a = 1; a < len; ++a) {
      int32_t v = c[a];
      int64_t b = a - 1;
      while (b >= 0 && c[b] > v) { c[b + 1] = c[b]; --b; }
      c[b + 1] = v;
    }
  }
  return 0;
}

/* Wendland C2 in 2D, src/kernels.py:20-24: W = 7/pi * (1-q)^4 (1+4q) / h^2 (float32 ops). */
static inline float wendland_f(float q, float h) {
  const float C = (float)(7.0 / 3.14159265358979323846);
  float a = 1.0f - q;
  float b1 = (a * a) * (a * a);
  float b2 = 1.0f + 4.0f * q;
  return b1 * b2 * C / (h * h);
}

/* density: rho_i = sum_j W(|x_i - x_j| / support) * A_j over the CSR rows (ascending j),
 * in float32 (reference) or float64 (error reference) accumulation. */
int oracle_density(const int64_t* offsets, const int32_t* cols, int64_t n, const float* pos,
                   const float* area, float support, int use_double, double* rho_out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    if (use_double) {
      double acc = 0.0;
      const double C = 7.0 / 3.14159265358979323846;
      double h = support;
      for (int64_t k = offsets[i]; k < offsets[i + 1]; ++k) {
        int32_t j = cols[k];
        double dx = (double)pos[2 * i] - pos[2 * j], dy = (double)pos[2 * i + 1] - pos[2 * j + 1];
        double q = sqrt(dx * dx + dy * dy) / h;
        double a = 1.0 - q;
        acc += a * a * a * a * (1.0 + 4.0 * q) * C / (h * h) * area[j];
      }
      rho_out[i] = acc;
    } else {
      float acc = 0.0f;
      for (int64_t k = offsets[i]; k < offsets[i + 1]; ++k) {
        int32_t j = cols[k];
        float dx = pos[2 * i] - pos[2 * j], dy = pos[2 * i + 1] - pos[2 * j + 1];
        float q = sqrtf(dx * dx + dy * dy) / support;
        acc += wendland_f(q, support) * area[j];
      }
      rho_out[i] = acc;
    }
  }
  return 0;
}
