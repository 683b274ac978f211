/* A C host of the search path through the C ABI only (no Python, no torch): device buffers
 * from cudaMalloc, the reference's pipeline of grid, keys, counting sort, gather, count,
 * scan and fill on one stream, then the pair set and the densities checked against a
 * brute-force host evaluation of the reference's predicate sqrtf(fmaf(dx,dx,dy*dy)) < h and
 * of the Wendland C2 sum.  Prints "ok <pairs>" and returns 0 when everything agrees.
 * Build: gcc -O2 search_host.c -I include -I $CUDA/include -L <lib dir> -lsph_gb300
 *        -L $CUDA/lib64 -lcudart -lm */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sph_gb300.h"

#define CK(x)                                                                     \
  do {                                                                            \
    if ((x) != cudaSuccess) {                                                     \
      fprintf(stderr, "CUDA error %s at line %d\n", cudaGetErrorString(x), __LINE__); \
      return 2;                                                                   \
    }                                                                             \
  } while (0)
#define SK(x)                                                                     \
  do {                                                                            \
    if ((x) != SPH_OK) {                                                          \
      fprintf(stderr, "sph error at line %d: %s\n", __LINE__, sph_last_error());  \
      return 3;                                                                   \
    }                                                                             \
  } while (0)

static float urand(uint64_t* s) {
  *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
  return (float)((*s >> 40) & 0xFFFFFF) / 16777216.0f;
}

static int cmp64(const void* a, const void* b) {
  const int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return x < y ? -1 : x > y;
}

int main(void) {
  const int side = 64, n = side * side;
  const float dx = 1.0f / side, h = 3.0f * dx;
  float* pos = (float*)malloc(sizeof(float) * 2 * n);
  float* sup = (float*)malloc(sizeof(float) * n);
  float* area = (float*)malloc(sizeof(float) * n);
  uint64_t seed = 12345;
  for (int i = 0; i < side; ++i)
    for (int j = 0; j < side; ++j) {
      const int k = i * side + j;
      pos[2 * k] = (i + 0.5f) * dx + (urand(&seed) - 0.5f) * 0.2f * dx;
      pos[2 * k + 1] = (j + 0.5f) * dx + (urand(&seed) - 0.5f) * 0.2f * dx;
      sup[k] = h;
      area[k] = dx * dx;
    }
  const float mn[2] = {0.0f, 0.0f}, mx[2] = {1.0f, 1.0f};
  cudaStream_t st;
  CK(cudaStreamCreate(&st));
  float *d_pos, *d_sup, *d_area, *d_xy, *d_ssup, *d_sarea, *d_rho;
  uint32_t *d_keys, *d_order, *d_skeys;
  int32_t *d_count, *d_start, *d_counts, *d_off, *d_cols, *d_status;
  sph_grid* d_grid;
  void *d_gs, *d_ss, *d_scan;
  const int32_t cap = 1 << 16;
  const int64_t pcap = (int64_t)n * 64;
  CK(cudaMalloc((void**)&d_pos, sizeof(float) * 2 * n));
  CK(cudaMalloc((void**)&d_sup, sizeof(float) * n));
  CK(cudaMalloc((void**)&d_area, sizeof(float) * n));
  CK(cudaMalloc((void**)&d_xy, sizeof(float) * 2 * n));
  CK(cudaMalloc((void**)&d_ssup, sizeof(float) * n));
  CK(cudaMalloc((void**)&d_sarea, sizeof(float) * n));
  CK(cudaMalloc((void**)&d_rho, sizeof(float) * n));
  CK(cudaMalloc((void**)&d_keys, sizeof(uint32_t) * n));
  CK(cudaMalloc((void**)&d_order, sizeof(uint32_t) * n));
  CK(cudaMalloc((void**)&d_skeys, sizeof(uint32_t) * n));
  CK(cudaMalloc((void**)&d_count, sizeof(int32_t) * (cap + 1)));
  CK(cudaMalloc((void**)&d_start, sizeof(int32_t) * (cap + 2)));
  CK(cudaMalloc((void**)&d_counts, sizeof(int32_t) * n));
  CK(cudaMalloc((void**)&d_off, sizeof(int32_t) * (n + 1)));
  CK(cudaMalloc((void**)&d_cols, sizeof(int32_t) * pcap));
  CK(cudaMalloc((void**)&d_status, sizeof(int32_t)));
  CK(cudaMalloc((void**)&d_grid, sizeof(sph_grid)));
  CK(cudaMalloc(&d_gs, sph_grid_scratch_bytes(n)));
  CK(cudaMalloc(&d_ss, sph_counting_sort_scratch_bytes(n, cap)));
  CK(cudaMalloc(&d_scan, sph_scan_scratch_bytes(n)));
  CK(cudaMemcpy(d_pos, pos, sizeof(float) * 2 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_sup, sup, sizeof(float) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_area, area, sizeof(float) * n, cudaMemcpyHostToDevice));
  CK(cudaMemset(d_count, 0, sizeof(int32_t) * (cap + 1)));
  CK(cudaMemset(d_status, 0, sizeof(int32_t)));
  CK(cudaMemset(d_counts, 0, sizeof(int32_t) * n));

  SK(sph_grid_build(d_pos, d_sup, n, mn, mx, cap, d_grid, d_status, d_gs, sph_grid_scratch_bytes(n), st));
  SK(sph_cell_keys(d_pos, n, d_grid, cap, d_keys, NULL, d_count, d_status, st));
  SK(sph_counting_sort(d_keys, n, cap, d_count, d_start, d_order, d_skeys, d_status, d_ss,
                       sph_counting_sort_scratch_bytes(n, cap), st));
  SK(sph_gather_sorted(d_order, n, d_pos, d_sup, d_area, d_xy, d_ssup, d_sarea, st));
  SK(sph_nl_count(d_xy, d_ssup, d_sarea, n, d_skeys, d_start, d_grid, cap, 1, h, d_counts, d_rho, st));
  SK(sph_exclusive_scan_i32(d_counts, d_off, n, d_scan, sph_scan_scratch_bytes(n), st));
  SK(sph_nl_fill(d_xy, d_ssup, n, d_skeys, d_start, d_grid, cap, 1, d_off, pcap, d_cols, d_status, st));
  CK(cudaStreamSynchronize(st));

  int32_t status = 0;
  int32_t* off = (int32_t*)malloc(sizeof(int32_t) * (n + 1));
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * n);
  float* rho = (float*)malloc(sizeof(float) * n);
  CK(cudaMemcpy(&status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(off, d_off, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(order, d_order, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(rho, d_rho, sizeof(float) * n, cudaMemcpyDeviceToHost));
  if (status != 0) {
    fprintf(stderr, "status flags %d\n", status);
    return 4;
  }
  const int64_t P = off[n];
  int32_t* cols = (int32_t*)malloc(sizeof(int32_t) * (P > 0 ? P : 1));
  CK(cudaMemcpy(cols, d_cols, sizeof(int32_t) * P, cudaMemcpyDeviceToHost));

  /* GPU pairs in original indices */
  int64_t* got = (int64_t*)malloc(sizeof(int64_t) * (P > 0 ? P : 1));
  for (int s = 0; s < n; ++s)
    for (int k = off[s]; k < off[s + 1]; ++k) got[k] = (int64_t)order[s] * n + order[cols[k]];
  qsort(got, P, sizeof(int64_t), cmp64);
  /* brute force on the host: the reference's predicate, Wendland C2 densities in double */
  int64_t* ref = (int64_t*)malloc(sizeof(int64_t) * (size_t)n * 64);
  int64_t R = 0;
  double max_err = 0.0, max_rho = 0.0;
  const double c_w = 7.0 / (M_PI * (double)h * (double)h);
  float* rho_sorted_by_orig = (float*)malloc(sizeof(float) * n);
  for (int s = 0; s < n; ++s) rho_sorted_by_orig[order[s]] = rho[s];
  for (int i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) {
      const float ddx = pos[2 * i] - pos[2 * j], ddy = pos[2 * i + 1] - pos[2 * j + 1];
      const float r = sqrtf(fmaf(ddx, ddx, ddy * ddy));
      if (r < sup[i]) {
        if (R < (int64_t)n * 64) ref[R] = (int64_t)i * n + j;
        ++R;
        const double q = (double)r / h, a = 1.0 - q;
        acc += c_w * a * a * a * a * (1.0 + 4.0 * q) * area[j];
      }
    }
    const double e = fabs(acc - rho_sorted_by_orig[i]);
    if (e > max_err) max_err = e;
    if (acc > max_rho) max_rho = acc;
  }
  qsort(ref, R, sizeof(int64_t), cmp64);
  if (R != P || memcmp(ref, got, sizeof(int64_t) * P) != 0) {
    fprintf(stderr, "pair sets differ: %lld vs %lld\n", (long long)P, (long long)R);
    return 5;
  }
  if (max_err > 1e-5 * max_rho) {
    fprintf(stderr, "density error %g of %g\n", max_err, max_rho);
    return 6;
  }
  printf("ok %lld\n", (long long)P);
  return 0;
}
