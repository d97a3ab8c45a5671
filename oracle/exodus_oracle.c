/*
 * CPU restatement of sif's exodus void-finder path (see exodus_oracle.h).
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 *
 * Compiled with -ffp-contract=off: every float expression below is evaluated
 * in the written order with one rounding per operation, which is what the
 * reference computes in a strict IEEE build. Where the reference's order of
 * evaluation is part of the answer (the filter table, the distance, the skip
 * and crossing tests) the expression is written in that order and cited.
 */
#include "exodus_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw_shim/fftw3.h"

#ifdef _OPENMP
#  include <omp.h>
#endif

#define PI_F ((float)3.14159265358979323846)

/* ------------------------------------------------------------------------ */
/* Box folding and the chain mesh                                           */
/* ------------------------------------------------------------------------ */

/* sif__box_fold, src/structures/field_internal.h:58-64. */
static inline float box_fold(float v, float box) {
  if (v >= box)
    v -= box;
  else if (v < 0)
    v += box;
  return v >= box ? 0.0f : v;
}

/* chain_mesh_flat_idx, src/structures/chain_mesh.c:316-331. */
static inline uint64_t mesh_cell_of(
  float x, float y, float z, float inv_l, uint32_t n, float box) {
  int32_t ix = (int32_t)(box_fold(x, box) * inv_l);
  int32_t iy = (int32_t)(box_fold(y, box) * inv_l);
  int32_t iz = (int32_t)(box_fold(z, box) * inv_l);
  const int32_t hi = (int32_t)n - 1;
  ix = ix < 0 ? 0 : (ix > hi ? hi : ix);
  iy = iy < 0 ? 0 : (iy > hi ? hi : iy);
  iz = iz < 0 ? 0 : (iz > hi ? hi : iz);
  return (uint64_t)ix * n * n + (uint64_t)iy * n + (uint64_t)iz;
}

/* The mesh of chain_mesh_create + chain_mesh_canonicalise
 * (src/structures/chain_mesh.c:680-832, 420-542), with their parallel
 * structure: counts per cell by run-length-batched atomic adds over one
 * chunk of particles per thread, a serial prefix, a scatter that claims each
 * run's slots with one atomic, then every cell put in ascending source index
 * (a sort of (index, slot) records, insertion sort up to 32 entries), which
 * makes the result independent of the threads: each cell in source order.
 * The box check of chain_mesh_new (field.c:889-935) is the caller's;
 * coordinates are folded as the scatter folds them. */
#define CANON_INSERTION_MAX 32u

typedef struct {
  uint64_t key, slot;
} canon_t;

static int canon_cmp(const void* a, const void* b) {
  const uint64_t x = ((const canon_t*)a)->key, y = ((const canon_t*)b)->key;
  return (x > y) - (x < y);
}

int orc_chain_mesh(const float* x, const float* y, const float* z, uint64_t n,
  uint32_t n_cells, float box, float* ox, float* oy, float* oz,
  uint64_t* offsets, uint64_t* orig) {
  if (n_cells == 0 || !(box > 0.0f))
    return -2;
  const uint64_t total = (uint64_t)n_cells * n_cells * n_cells;
  const float cell_length = box / (float)n_cells;
  const float inv_l = 1.0f / cell_length;
  uint64_t* idx = orig ? orig : malloc(n * sizeof(uint64_t));
  uint64_t* cursor = malloc(total * sizeof(uint64_t));
  if (!idx || !cursor) {
    if (!orig)
      free(idx);
    free(cursor);
    return -1;
  }
#pragma omp parallel for schedule(static)
  for (uint64_t c = 0; c <= total; c++)
    offsets[c] = 0;
#pragma omp parallel
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const uint64_t chunk = n / (uint64_t)nt;
    const uint64_t a = (uint64_t)t * chunk, e = t == nt - 1 ? n : a + chunk;
    uint64_t i = a;
    while (i < e) {
      const uint64_t c = mesh_cell_of(x[i], y[i], z[i], inv_l, n_cells, box);
      uint64_t run = 1;
      while (i + run < e && mesh_cell_of(x[i + run], y[i + run], z[i + run], inv_l, n_cells,
                              box) == c)
        run++;
#pragma omp atomic
      offsets[c] += run;
      i += run;
    }
  }
  uint64_t acc = 0;
  for (uint64_t c = 0; c < total; c++) {
    const uint64_t v = offsets[c];
    offsets[c] = acc;
    acc += v;
  }
  offsets[total] = acc;
#pragma omp parallel for schedule(static)
  for (uint64_t c = 0; c < total; c++)
    cursor[c] = offsets[c];
#pragma omp parallel
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const uint64_t chunk = n / (uint64_t)nt;
    const uint64_t a = (uint64_t)t * chunk, e = t == nt - 1 ? n : a + chunk;
    uint64_t i = a;
    while (i < e) {
      const uint64_t c = mesh_cell_of(x[i], y[i], z[i], inv_l, n_cells, box);
      uint64_t run = 1;
      while (i + run < e && mesh_cell_of(x[i + run], y[i + run], z[i + run], inv_l, n_cells,
                              box) == c)
        run++;
      uint64_t base;
#pragma omp atomic capture
      {
        base = cursor[c];
        cursor[c] += run;
      }
      for (uint64_t j = 0; j < run; j++) {
        idx[base + j] = i + j;
        ox[base + j] = box_fold(x[i + j], box);
        oy[base + j] = box_fold(y[i + j], box);
        oz[base + j] = box_fold(z[i + j], box);
      }
      i += run;
    }
  }
  free(cursor);
#pragma omp parallel
  {
    canon_t* order = NULL;
    float* tmp = NULL;
    uint64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (uint64_t c = 0; c < total; c++) {
      const uint64_t lo = offsets[c], hi = offsets[c + 1], m = hi - lo;
      if (m < 2)
        continue;
      uint64_t run = 1;
      while (run < m && idx[lo + run - 1] < idx[lo + run])
        run++;
      if (run == m)
        continue;
      if (m > cap) {
        cap = m + (m >> 1) + 8;
        order = realloc(order, cap * sizeof(canon_t));
        tmp = realloc(tmp, cap * sizeof(float));
      }
      for (uint64_t i = 0; i < m; i++) {
        order[i].key = idx[lo + i];
        order[i].slot = i;
      }
      if (m <= CANON_INSERTION_MAX) {
        for (uint64_t i = 1; i < m; i++) {
          const canon_t v = order[i];
          uint64_t j = i;
          while (j > 0 && order[j - 1].key > v.key) {
            order[j] = order[j - 1];
            j--;
          }
          order[j] = v;
        }
      } else {
        qsort(order, (size_t)m, sizeof(canon_t), canon_cmp);
      }
      float* cols[3] = {ox, oy, oz};
      for (int k = 0; k < 3; k++) {
        for (uint64_t i = 0; i < m; i++)
          tmp[i] = cols[k][lo + order[i].slot];
        memcpy(cols[k] + lo, tmp, m * sizeof(float));
      }
      for (uint64_t i = 0; i < m; i++)
        idx[lo + i] = order[i].key;
    }
    free(order);
    free(tmp);
  }
  if (!orig)
    free(idx);
  return 0;
}

/* The mesh's weight columns, chain_mesh.c:800-801 (a tracer's weight moves
 * with it, so in mesh order it is the field's at the source index) and
 * chain_mesh_sum_weights, 624-672: per cell a double sum in mesh order,
 * stored as float; the total over 64 fixed blocks of cells, each a serial
 * double sum of its cells', added in block order. */
void orc_mesh_weights(const float* field_w, const uint64_t* orig, uint64_t n,
  const uint64_t* offsets, uint32_t n_cells, float* out_w, float* out_cell_w,
  double* total) {
  for (uint64_t p = 0; p < n; p++)
    out_w[p] = field_w[orig[p]];
  enum { WEIGHT_BLOCKS = 64 };
  const uint64_t cells = (uint64_t)n_cells * n_cells * n_cells;
  const uint64_t block = (cells + WEIGHT_BLOCKS - 1) / WEIGHT_BLOCKS;
  double bt[WEIGHT_BLOCKS];
#pragma omp parallel for schedule(static, 1)
  for (int b = 0; b < WEIGHT_BLOCKS; b++) {
    const uint64_t c0 = (uint64_t)b * block;
    const uint64_t c1 = c0 + block < cells ? c0 + block : cells;
    double sum = 0.0;
    for (uint64_t c = c0; c < c1; c++) {
      double cell = 0.0;
      for (uint64_t p = offsets[c]; p < offsets[c + 1]; p++)
        cell += (double)out_w[p];
      out_cell_w[c] = (float)cell;
      sum += cell;
    }
    bt[b] = sum;
  }
  double t = 0.0;
  for (int b = 0; b < WEIGHT_BLOCKS; b++)
    t += bt[b];
  *total = t;
}

/* ------------------------------------------------------------------------ */
/* CIC and the density contrast                                             */
/* ------------------------------------------------------------------------ */

/* The CIC deposit of grid_compute_cic (src/structures/grid.c:455-746) in
 * double: base cell (uint32)(fold(x) * N/L) with the >= N fallback to 0,
 * weights (1 - t, t), periodic upper neighbours, divided by the cell volume.
 * The particles are bucketed by their base x plane; a plane's bucket writes
 * planes x and x + 1 only, so the even planes' buckets run in parallel, then
 * the odd ones' (and, for an odd N, the last plane, which wraps onto plane 0,
 * alone). The sums are double: their order moves only the last bits. */
static void cic_f64_base(float v, float box, double idx, uint32_t N, uint32_t* i0,
  uint32_t* i1, double* w0, double* w1) {
  const double u = (double)box_fold(v, box) * idx;
  const uint32_t raw = (uint32_t)u;
  *i0 = raw >= N ? 0u : raw;
  *i1 = *i0 + 1 == N ? 0u : *i0 + 1;
  const double t = u - (double)raw;
  *w0 = 1.0 - t;
  *w1 = t;
}

void orc_cic_f64(const float* x, const float* y, const float* z, uint64_t n,
  uint32_t N, float box, double* out) {
  orc_cic_f64_w(x, y, z, NULL, n, N, box, out);
}

void orc_cic_f64_w(const float* x, const float* y, const float* z, const float* ws,
  uint64_t n, uint32_t N, float box, double* out) {
  const uint64_t total = (uint64_t)N * N * N;
  const uint64_t plane = (uint64_t)N * N;
  const double idx = (double)N / (double)box;
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < total; i++)
    out[i] = 0.0;
  if (n == 0 || n >= (1ull << 32))
    return;
  /* Bucketed by base plane, counted per thread chunk and placed in order. */
  const int nt = omp_get_max_threads();
  uint64_t* counts = calloc((size_t)nt * N + 1, sizeof(uint64_t));
  uint32_t* order = malloc(n * sizeof(uint32_t));
  uint64_t* start = malloc(((size_t)N + 1) * sizeof(uint64_t));
  if (!counts || !order || !start) {
    free(counts);
    free(order);
    free(start);
    return;
  }
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const uint64_t a = n * (uint64_t)t / (uint64_t)nt, e = n * (uint64_t)(t + 1) / (uint64_t)nt;
    uint64_t* c = counts + (uint64_t)t * N;
    for (uint64_t p = a; p < e; p++) {
      uint32_t i0, i1;
      double w0, w1;
      cic_f64_base(x[p], box, idx, N, &i0, &i1, &w0, &w1);
      c[i0]++;
    }
#pragma omp barrier
#pragma omp single
    {
      uint64_t run = 0;
      for (uint32_t ix = 0; ix < N; ix++) {
        start[ix] = run;
        for (int u = 0; u < nt; u++) {
          const uint64_t v = counts[(uint64_t)u * N + ix];
          counts[(uint64_t)u * N + ix] = run;
          run += v;
        }
      }
      start[N] = run;
    }
    for (uint64_t p = a; p < e; p++) {
      uint32_t i0, i1;
      double w0, w1;
      cic_f64_base(x[p], box, idx, N, &i0, &i1, &w0, &w1);
      order[c[i0]++] = (uint32_t)p;
    }
  }
  free(counts);
  for (int phase = 0; phase < 3; phase++) {
    /* Phase 0: even planes, 1: odd planes, 2: an odd N's last plane. */
    const uint32_t last = (N & 1u) ? N - 1 : N;
#pragma omp parallel for schedule(dynamic, 1)
    for (uint32_t ix = 0; ix < N; ix++) {
      const int mine = phase == 2 ? ix == last : (ix != last && (int)(ix & 1u) == phase);
      if (!mine)
        continue;
      for (uint64_t q = start[ix]; q < start[ix + 1]; q++) {
        const uint64_t p = order[q];
        uint32_t i0[3], i1[3];
        double w0[3], w1[3];
        cic_f64_base(x[p], box, idx, N, &i0[0], &i1[0], &w0[0], &w1[0]);
        cic_f64_base(y[p], box, idx, N, &i0[1], &i1[1], &w0[1], &w1[1]);
        cic_f64_base(z[p], box, idx, N, &i0[2], &i1[2], &w0[2], &w1[2]);
        for (int a = 0; a < 2; a++)
          for (int b = 0; b < 2; b++)
            for (int c = 0; c < 2; c++) {
              const uint64_t cell = (uint64_t)(a ? i1[0] : i0[0]) * plane +
                                    (uint64_t)(b ? i1[1] : i0[1]) * N + (c ? i1[2] : i0[2]);
              out[cell] += (a ? w1[0] : w0[0]) * (b ? w1[1] : w0[1]) * (c ? w1[2] : w0[2]) *
                           (ws ? (double)ws[p] : 1.0);
            }
      }
    }
  }
  free(order);
  free(start);
  const double cl = (double)box / (double)N;
  const double inv_vol = 1.0 / (cl * cl * cl);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < total; i++)
    out[i] *= inv_vol;
}

/* The reference's own float CIC deposit, grid_compute_cic with
 * grid_cic_deposit_tile for SIF_ASSIGNMENT_CIC (src/structures/grid.c:
 * 180-345, 455-746): slabs of N/16 planes' width (the last takes the rest),
 * each with one ghost plane above; the particles taken in tiles of 64Mi
 * (the cic_tile_particles default), each tile counting-sorted by slab over
 * 256 fixed chunks (counts per chunk and slab, offsets slab-major, a scatter
 * of indices) and deposited a slab per thread in that order; the ghost planes
 * folded into the next slab serially; the slabs copied out times the
 * inverse cell volume. The order of every float addition is the reference's,
 * so the density is its bit for bit. */
#define CIC_CHUNKS 256
#define CIC_SLAB_WIDTH 16u
#define CIC_TILE_PARTICLES 67108864ull

void orc_cic_float(const float* xs, const float* ys, const float* zs, uint64_t n,
  uint32_t N, float box, float* grid) {
  orc_cic_float_w(xs, ys, zs, NULL, n, N, box, grid);
}

/* The same with per-particle weights (NULL: 1 each), which enter as the
 * reference's do (grid.c:635-639): the weight times each z factor, then the
 * (x, y) products times those. */
void orc_cic_float_w(const float* xs, const float* ys, const float* zs, const float* ws,
  uint64_t n, uint32_t N, float box, float* grid) {
  const float idx = (float)N / (float)box;
  int32_t n_slabs = (int32_t)(N / CIC_SLAB_WIDTH);
  if (n_slabs < 1)
    n_slabs = 1;
  const uint64_t plane = (uint64_t)N * N;
  uint64_t* slab_off = malloc(((size_t)n_slabs + 1) * sizeof(uint64_t));
  uint32_t* slab_x0 = malloc((size_t)n_slabs * sizeof(uint32_t));
  uint32_t* slab_w = malloc((size_t)n_slabs * sizeof(uint32_t));
  slab_off[0] = 0;
  for (int t = 0; t < n_slabs; t++) {
    slab_x0[t] = (uint32_t)t * (N / (uint32_t)n_slabs);
    const uint32_t end = t == n_slabs - 1 ? N : (uint32_t)(t + 1) * (N / (uint32_t)n_slabs);
    slab_w[t] = end - slab_x0[t];
    uint64_t cells = (uint64_t)(slab_w[t] + 1) * plane;
    cells = (cells + 15) & ~(uint64_t)15; /* a 64-byte line of floats */
    slab_off[t + 1] = slab_off[t] + cells;
  }
  float* arena = calloc(slab_off[n_slabs], sizeof(float));
  const uint32_t base_width = N / (uint32_t)n_slabs;
  uint64_t tile_n = CIC_TILE_PARTICLES < n ? CIC_TILE_PARTICLES : n;
  if (tile_n == 0)
    tile_n = 1;
  uint64_t* counts = malloc((size_t)CIC_CHUNKS * n_slabs * sizeof(uint64_t));
  uint64_t* sorted = malloc(tile_n * sizeof(uint64_t));
  for (uint64_t lo = 0; lo < n; lo += tile_n) {
    const uint64_t hi = lo + tile_n > n ? n : lo + tile_n;
    const uint64_t chunk = (hi - lo + CIC_CHUNKS - 1) / CIC_CHUNKS;
    memset(counts, 0, (size_t)CIC_CHUNKS * n_slabs * sizeof(uint64_t));
#pragma omp parallel for schedule(static, 1)
    for (int c = 0; c < CIC_CHUNKS; c++) {
      const uint64_t a = lo + (uint64_t)c * chunk, e = a + chunk > hi ? hi : a + chunk;
      for (uint64_t p = a; p < e; p++) {
        uint32_t ix = (uint32_t)(box_fold(xs[p], box) * idx);
        ix = ix >= N ? ix - N : ix;
        const uint32_t sl = ix / base_width < (uint32_t)(n_slabs - 1) ? ix / base_width
                                                                      : (uint32_t)(n_slabs - 1);
        counts[(uint64_t)c * n_slabs + sl]++;
      }
    }
    uint64_t run = 0;
    for (int32_t sl = 0; sl < n_slabs; sl++)
      for (int c = 0; c < CIC_CHUNKS; c++) {
        const uint64_t k = (uint64_t)c * n_slabs + sl, v = counts[k];
        counts[k] = run;
        run += v;
      }
#pragma omp parallel for schedule(static, 1)
    for (int c = 0; c < CIC_CHUNKS; c++) {
      const uint64_t a = lo + (uint64_t)c * chunk, e = a + chunk > hi ? hi : a + chunk;
      for (uint64_t p = a; p < e; p++) {
        uint32_t ix = (uint32_t)(box_fold(xs[p], box) * idx);
        ix = ix >= N ? ix - N : ix;
        const uint32_t sl = ix / base_width < (uint32_t)(n_slabs - 1) ? ix / base_width
                                                                      : (uint32_t)(n_slabs - 1);
        sorted[counts[(uint64_t)c * n_slabs + sl]++] = p;
      }
    }
#pragma omp parallel for schedule(static, 1)
    for (int32_t sl = 0; sl < n_slabs; sl++) {
      const uint64_t s0 = sl == 0 ? 0 : counts[(uint64_t)(CIC_CHUNKS - 1) * n_slabs + sl - 1];
      const uint64_t s1 = counts[(uint64_t)(CIC_CHUNKS - 1) * n_slabs + sl];
      float* v = arena + slab_off[sl];
      const uint32_t x0 = slab_x0[sl];
      for (uint64_t q = s0; q < s1; q++) {
        const uint64_t p = sorted[q];
        const float cx = box_fold(xs[p], box) * idx;
        const float cy = box_fold(ys[p], box) * idx;
        const float cz = box_fold(zs[p], box) * idx;
        const uint32_t rx = (uint32_t)cx, ry = (uint32_t)cy, rz = (uint32_t)cz;
        const uint32_t ix = rx >= N ? 0 : rx, iy = ry >= N ? 0 : ry, iz = rz >= N ? 0 : rz;
        const uint32_t iy1 = iy + 1 == N ? 0 : iy + 1, iz1 = iz + 1 == N ? 0 : iz + 1;
        const uint64_t l0 = (uint64_t)(ix - x0) * plane, l1 = l0 + plane;
        const float tx = cx - (float)rx, ty = cy - (float)ry, tz = cz - (float)rz;
        const float wx0 = 1.0f - tx, wx1 = tx, wy0 = 1.0f - ty, wy1 = ty;
        const float wz0 = 1.0f - tz, wz1 = tz;
        const float w00 = wx0 * wy0, w01 = wx0 * wy1, w10 = wx1 * wy0, w11 = wx1 * wy1;
        const float pw = ws ? ws[p] : 1.0f;
        const float mz0 = pw * wz0, mz1 = pw * wz1;
        v[l0 + (uint64_t)iy * N + iz] += w00 * mz0;
        v[l0 + (uint64_t)iy * N + iz1] += w00 * mz1;
        v[l0 + (uint64_t)iy1 * N + iz] += w01 * mz0;
        v[l0 + (uint64_t)iy1 * N + iz1] += w01 * mz1;
        v[l1 + (uint64_t)iy * N + iz] += w10 * mz0;
        v[l1 + (uint64_t)iy * N + iz1] += w10 * mz1;
        v[l1 + (uint64_t)iy1 * N + iz] += w11 * mz0;
        v[l1 + (uint64_t)iy1 * N + iz1] += w11 * mz1;
      }
    }
  }
  /* grid_cic_reduce_ghost_cells: slab t's ghost plane into slab t+1's first. */
  for (int32_t t = 0; t < n_slabs; t++) {
    const float* ghost = arena + slab_off[t] + (uint64_t)slab_w[t] * plane;
    float* first = arena + slab_off[(t + 1) % n_slabs];
    for (uint64_t i = 0; i < plane; i++)
      first[i] += ghost[i];
  }
  const float cl = box / (float)N;
  const float inv_vol = 1.0f / (float)(cl * cl * cl);
#pragma omp parallel for schedule(static)
  for (int32_t t = 0; t < n_slabs; t++) {
    const float* v = arena + slab_off[t];
    float* out = grid + (uint64_t)slab_x0[t] * plane;
    for (uint64_t i = 0; i < (uint64_t)slab_w[t] * plane; i++)
      out[i] = v[i] * inv_vol;
  }
  free(sorted);
  free(counts);
  free(arena);
  free(slab_w);
  free(slab_x0);
  free(slab_off);
}

/* The density contrast of an FP64 density, all in double: the mean by the
 * same 64 fixed blocks, then v / mean - 1. */
int orc_density_contrast_f64(double* v, uint64_t n) {
  const int blocks = 64;
  const uint64_t block = (n + blocks - 1) / blocks;
  double part[64];
#pragma omp parallel for schedule(static, 1)
  for (int b = 0; b < blocks; b++) {
    const uint64_t s = (uint64_t)b * block;
    const uint64_t e = s + block < n ? s + block : n;
    double sum = 0.0;
    for (uint64_t i = s; i < e; i++)
      sum += v[i];
    part[b] = sum;
  }
  double total = 0.0;
  for (int b = 0; b < blocks; b++)
    total += part[b];
  const double mean = total / (double)n;
  if (!(mean > 0.0))
    return -3;
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < n; i++)
    v[i] = v[i] / mean - 1.0;
  return 0;
}

/* sif_grid_to_density_contrast, src/structures/grid.c:1177-1244: the mean in
 * 64 fixed blocks of double, then v * (float)(1/mean) - 1 in float. */
int orc_density_contrast(float* v, uint64_t n) {
  const int blocks = 64;
  const uint64_t block = (n + blocks - 1) / blocks;
  double part[64];
#pragma omp parallel for schedule(static, 1)
  for (int b = 0; b < blocks; b++) {
    const uint64_t s = (uint64_t)b * block;
    const uint64_t e = s + block < n ? s + block : n;
    double sum = 0.0;
    for (uint64_t i = s; i < e; i++)
      sum += (double)v[i];
    part[b] = sum;
  }
  double total = 0.0;
  for (int b = 0; b < blocks; b++)
    total += part[b];
  const double mean = total / (double)n;
  if (!(mean > 0.0))
    return -3;
  const float inv = (float)(1.0 / mean);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < n; i++)
    v[i] = v[i] * inv - 1.0f;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Smoothing                                                                */
/* ------------------------------------------------------------------------ */

struct orc_spectrum {
  uint32_t n;
  float box;
  int mode;
  fftw_complex* spec;   /* mode 0: n * n * (n/2+1), double */
  fftwf_complex* specf; /* mode 1: the same modes in float, plane-major */
  double* window;       /* per-axis factor, or NULL */
};

/* The float mode's transforms are laid out as the reference lays out its own
 * (src/math/fft.c:269-434, 790-888): a 2-D transform of every x plane and a
 * 1-D transform along x of every (y, kz) pencil, FFT_PENCIL_BLOCK pencils at
 * a time, each through one single-threaded plan, in parallel over the planes
 * and the pencil blocks. Through the same FFTW-API calls on the same plans
 * the spectrum and the smoothed fields are the reference's bit for bit. */
#define PENCIL_BLOCK 16

static uint64_t plane_modes(uint32_t n) { return (uint64_t)n * (n / 2 + 1); }

/* fft_pencils (src/math/fft.c:378-434), sif__fft_grid_forward (790-818) and
 * sif__fft_grid_backward (820-888) for a precision: X the FFTW-API prefix,
 * R its real type. The float pair is the reference's transform; the double
 * pair runs the FP64 oracle's transforms the same way (plane by plane, pencil
 * block by pencil block), which keeps them in cache at large grids. */
#define ORC_TRANSFORMS(X, R, SUFFIX)                                              \
  static void pencils_##SUFFIX(X##_complex* c, uint32_t n, int sign) {            \
    const int len[1] = {(int)n};                                                  \
    const uint64_t n_pencils = plane_modes(n);                                    \
    const uint64_t n_blocks = (n_pencils + PENCIL_BLOCK - 1) / PENCIL_BLOCK;      \
    X##_complex* scratch = X##_malloc((size_t)n * PENCIL_BLOCK * sizeof(X##_complex)); \
    X##_plan plan = X##_plan_many_dft(1, len, PENCIL_BLOCK, scratch, NULL,        \
      PENCIL_BLOCK, 1, scratch, NULL, PENCIL_BLOCK, 1, sign, FFTW_ESTIMATE);      \
    X##_free(scratch);                                                            \
    _Pragma("omp parallel")                                                       \
    {                                                                             \
      X##_complex* g = X##_malloc((size_t)n * PENCIL_BLOCK * sizeof(X##_complex)); \
      _Pragma("omp for schedule(static)")                                         \
      for (uint64_t b = 0; b < n_blocks; b++) {                                   \
        const uint64_t j0 = b * PENCIL_BLOCK;                                     \
        const uint64_t w = n_pencils - j0 < PENCIL_BLOCK ? n_pencils - j0 : PENCIL_BLOCK; \
        for (uint32_t x = 0; x < n; x++) {                                        \
          X##_complex* row = g + (uint64_t)x * PENCIL_BLOCK;                      \
          memcpy(row, c + x * n_pencils + j0, w * sizeof(X##_complex));           \
          if (w < PENCIL_BLOCK)                                                   \
            memset(row + w, 0, (PENCIL_BLOCK - w) * sizeof(X##_complex));        \
        }                                                                         \
        X##_execute_dft(plan, g, g);                                              \
        for (uint32_t x = 0; x < n; x++)                                          \
          memcpy(c + x * n_pencils + j0, g + (uint64_t)x * PENCIL_BLOCK,          \
            w * sizeof(X##_complex));                                             \
      }                                                                           \
      X##_free(g);                                                                \
    }                                                                             \
    X##_destroy_plan(plan);                                                       \
  }                                                                               \
                                                                                  \
  static void forward_##SUFFIX(const R* in, X##_complex* spec, uint32_t n) {      \
    const uint64_t reals = (uint64_t)n * n, modes = plane_modes(n);               \
    R* pr = X##_malloc(reals * sizeof(R));                                        \
    X##_complex* pc = X##_malloc(modes * sizeof(X##_complex));                    \
    X##_plan plane = X##_plan_dft_r2c_2d((int)n, (int)n, pr, pc, FFTW_ESTIMATE);  \
    X##_free(pr);                                                                 \
    X##_free(pc);                                                                 \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (uint32_t x = 0; x < n; x++)                                              \
      X##_execute_dft_r2c(plane, (R*)in + x * reals, spec + x * modes);           \
    X##_destroy_plan(plane);                                                      \
    pencils_##SUFFIX(spec, n, FFTW_FORWARD);                                      \
  }                                                                               \
                                                                                  \
  static void backward_##SUFFIX(X##_complex* c, R* out, uint32_t n) {             \
    pencils_##SUFFIX(c, n, FFTW_BACKWARD);                                        \
    const uint64_t reals = (uint64_t)n * n, modes = plane_modes(n);               \
    const R norm = (R)1.0 / (R)((uint64_t)n * n * n);                             \
    R* pr = X##_malloc(reals * sizeof(R));                                        \
    X##_complex* pc = X##_malloc(modes * sizeof(X##_complex));                    \
    X##_plan plane = X##_plan_dft_c2r_2d((int)n, (int)n, pc, pr, FFTW_ESTIMATE);  \
    X##_free(pr);                                                                 \
    X##_free(pc);                                                                 \
    _Pragma("omp parallel")                                                       \
    {                                                                             \
      R* buf = X##_malloc(reals * sizeof(R));                                     \
      _Pragma("omp for schedule(static)")                                         \
      for (uint32_t x = 0; x < n; x++) {                                          \
        X##_execute_dft_c2r(plane, c + x * modes, buf);                           \
        R* o = out + x * reals;                                                   \
        for (uint64_t i = 0; i < reals; i++)                                      \
          o[i] = buf[i] * norm;                                                   \
      }                                                                           \
      X##_free(buf);                                                              \
    }                                                                             \
    X##_destroy_plan(plane);                                                      \
  }

ORC_TRANSFORMS(fftwf, float, f)
ORC_TRANSFORMS(fftw, double, d)

/* x = pi k / N for index i (src/math/fft.c:939-943), with the reference's
 * float pi in the float mode. */
static double axis_x(uint32_t i, uint32_t n, int mode) {
  const uint32_t h = n >> 1;
  const int32_t k = i > h ? (int32_t)i - (int32_t)n : (int32_t)i;
  const double pi = mode ? (double)PI_F : M_PI;
  return pi * (double)k / (double)n;
}

static orc_spectrum_t* spectrum_new(const float* delta_f, const double* delta_d, uint32_t n,
  float box, int window_mode, int mode) {
  orc_spectrum_t* s = calloc(1, sizeof(*s));
  s->n = n;
  s->box = box;
  s->mode = mode;
  const uint64_t total = (uint64_t)n * n * n;
  const uint64_t modes = (uint64_t)n * n * (n / 2 + 1);
  if (mode) {
    s->specf = fftwf_malloc(modes * sizeof(fftwf_complex));
    forward_f(delta_f, s->specf, n);
  } else {
    s->spec = fftw_malloc(modes * sizeof(fftw_complex));
    if (delta_d) {
      forward_d(delta_d, s->spec, n);
    } else {
      double* in = malloc(total * sizeof(double));
#pragma omp parallel for schedule(static)
      for (uint64_t i = 0; i < total; i++)
        in[i] = (double)delta_f[i];
      forward_d(in, s->spec, n);
      free(in);
    }
  }
  if (window_mode) {
    /* fft_build_window_axis, src/math/fft.c:958-975, order 2 (CIC):
     * W = sinc^2, factor 1/W (full) or W/S with S = 1 - 2 sin^2/3. */
    s->window = malloc(n * sizeof(double));
    for (uint32_t i = 0; i < n; i++) {
      const double x = axis_x(i, n, mode);
      const double sc = (x < 1e-9 && x > -1e-9) ? 1.0 : sin(x) / x;
      double w = 1.0;
      w *= sc;
      w *= sc;
      if (window_mode == 2) {
        const double s2 = sin(x) * sin(x);
        s->window[i] = w / (1.0 - 2.0 * s2 / 3.0);
      } else {
        s->window[i] = 1.0 / w;
      }
    }
  }
  return s;
}

orc_spectrum_t* orc_spectrum_new(
  const float* delta, uint32_t n, float box, int window_mode, int mode) {
  return spectrum_new(delta, NULL, n, box, window_mode, mode);
}

orc_spectrum_t* orc_spectrum_new_f64(
  const double* delta, uint32_t n, float box, int window_mode) {
  return spectrum_new(NULL, delta, n, box, window_mode, 0);
}

/* fft_build_filter_lut + sif__fft_apply_filter_smoothed + the backward
 * transform's 1/N^3 (src/math/fft.c:521-568, 703-788, 820-888). filter 0 is
 * SIF__FILTER_NONE: the spectrum as it is, no window (the reference's restore
 * of the grid at the end of a run, exodus_finder.c:2430-2453). */
void orc_spectrum_smooth(orc_spectrum_t* s, int filter, float r, float sigma,
  float* out_f, double* out_d) {
  const uint32_t n = s->n;
  const uint32_t h = n >> 1;
  const uint32_t zd = n / 2 + 1;
  const uint32_t max_k2 = 3 * h * h;
  const uint64_t modes = (uint64_t)n * n * zd;
  const uint64_t total = (uint64_t)n * n * n;
  double* lut = malloc(((size_t)max_k2 + 1) * sizeof(double));
  if (s->mode) {
    const float factor = (float)((double)r * 2.0 * (double)PI_F / (double)s->box);
    const float factor2 = factor * factor;
    const float gfactor = (float)((double)sigma * 2.0 * (double)PI_F / (double)s->box);
    const float gfactor2 = gfactor * gfactor;
#pragma omp parallel for schedule(static)
    for (uint32_t k2 = 0; k2 <= max_k2; k2++) {
      float v;
      if (k2 == 0) {
        v = 1.0f;
      } else if (filter == 1) {
        const float kr = factor * sqrtf((float)k2);
        v = kr > 1e-4f ? 3.0f * (sinf(kr) - kr * cosf(kr)) / (kr * kr * kr) : 1.0f;
      } else {
        v = expf(-0.5f * factor2 * (float)k2);
      }
      if (sigma > 0.0f && k2 > 0)
        v *= expf(-0.5f * gfactor2 * (float)k2);
      lut[k2] = v;
    }
  } else {
    const double factor = (double)r * 2.0 * M_PI / (double)s->box;
    const double gfactor = (double)sigma * 2.0 * M_PI / (double)s->box;
#pragma omp parallel for schedule(static)
    for (uint32_t k2 = 0; k2 <= max_k2; k2++) {
      double v;
      if (k2 == 0) {
        v = 1.0;
      } else if (filter == 1) {
        const double kr = factor * sqrt((double)k2);
        v = kr > 1e-4 ? 3.0 * (sin(kr) - kr * cos(kr)) / (kr * kr * kr) : 1.0;
      } else {
        v = exp(-0.5 * factor * factor * (double)k2);
      }
      if (sigma > 0.0f && k2 > 0)
        v *= exp(-0.5 * gfactor * gfactor * (double)k2);
      lut[k2] = v;
    }
  }
  const double* win = filter ? s->window : NULL;
  if (s->mode) {
    fftwf_complex* work = fftwf_malloc(modes * sizeof(fftwf_complex));
    const fftwf_complex* spec = s->specf;
#pragma omp parallel for schedule(static)
    for (uint32_t ix = 0; ix < n; ix++) {
      const int32_t kx = ix > h ? (int32_t)ix - (int32_t)n : (int32_t)ix;
      const uint32_t kx2 = (uint32_t)(kx * kx);
      const double cx = win ? win[ix] : 1.0;
      for (uint32_t iy = 0; iy < n; iy++) {
        const int32_t ky = iy > h ? (int32_t)iy - (int32_t)n : (int32_t)iy;
        const uint32_t kxy2 = kx2 + (uint32_t)(ky * ky);
        const double cxy = cx * (win ? win[iy] : 1.0);
        for (uint32_t iz = 0; iz < zd; iz++) {
          const uint64_t i = ((uint64_t)ix * n + iy) * zd + iz;
          if (!filter) {
            work[i][0] = spec[i][0];
            work[i][1] = spec[i][1];
            continue;
          }
          float smf = (float)lut[kxy2 + iz * iz];
          if (win)
            smf = (float)((double)smf * cxy * win[iz]);
          work[i][0] = spec[i][0] * smf;
          work[i][1] = spec[i][1] * smf;
        }
      }
    }
    free(lut);
    float* f = out_f ? out_f : malloc(total * sizeof(float));
    backward_f(work, f, n);
    fftwf_free(work);
    if (out_d)
#pragma omp parallel for schedule(static)
      for (uint64_t i = 0; i < total; i++)
        out_d[i] = (double)f[i];
    if (!out_f)
      free(f);
    return;
  }
  fftw_complex* work = fftw_malloc(modes * sizeof(fftw_complex));
#pragma omp parallel for schedule(static)
  for (uint32_t ix = 0; ix < n; ix++) {
    const int32_t kx = ix > h ? (int32_t)ix - (int32_t)n : (int32_t)ix;
    const uint32_t kx2 = (uint32_t)(kx * kx);
    const double cx = win ? win[ix] : 1.0;
    for (uint32_t iy = 0; iy < n; iy++) {
      const int32_t ky = iy > h ? (int32_t)iy - (int32_t)n : (int32_t)iy;
      const uint32_t kxy2 = kx2 + (uint32_t)(ky * ky);
      const double cxy = cx * (win ? win[iy] : 1.0);
      for (uint32_t iz = 0; iz < zd; iz++) {
        const uint32_t k2 = kxy2 + iz * iz;
        const uint64_t i = ((uint64_t)ix * n + iy) * zd + iz;
        double sm = filter ? lut[k2] : 1.0;
        if (win)
          sm = sm * cxy * win[iz];
        work[i][0] = s->spec[i][0] * sm;
        work[i][1] = s->spec[i][1] * sm;
      }
    }
  }
  free(lut);
  double* real = out_d ? out_d : malloc(total * sizeof(double));
  backward_d(work, real, n);
  fftw_free(work);
  if (out_f)
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < total; i++)
      out_f[i] = (float)real[i];
  if (!out_d)
    free(real);
}

void orc_spectrum_free(orc_spectrum_t* s) {
  if (!s)
    return;
  fftw_free(s->spec);
  fftwf_free(s->specf);
  free(s->window);
  free(s);
}

/* ------------------------------------------------------------------------ */
/* Candidate order                                                          */
/* ------------------------------------------------------------------------ */

/* The reference sorts candidates with a three-way (Dijkstra) quicksort whose
 * pivot is the middle element of the range (include/sif/utils/sort.h:56-98),
 * and its parallel form reproduces the serial permutation (108-145). Equal
 * depths are common, and their order is part of the answer, so the same
 * partition steps are taken here: scan left to right; a smaller key moves to
 * the low end, a larger one is exchanged with the high end and re-examined,
 * an equal one stays. Ranges are kept on an explicit stack; the two sides of a
 * partition are disjoint, so the order they are processed in is immaterial. */
static void partition3_cand(orc_candidate_t* a, int64_t lo, int64_t hi, int64_t* lt_out,
  int64_t* gt_out) {
  const float pivot = a[lo + (hi - lo) / 2].delta;
  int64_t lt = lo, i = lo, gt = hi;
  while (i <= gt) {
    const float v = a[i].delta;
    if (v < pivot) {
      const orc_candidate_t t = a[lt];
      a[lt] = a[i];
      a[i] = t;
      lt++;
      i++;
    } else if (pivot < v) {
      const orc_candidate_t t = a[i];
      a[i] = a[gt];
      a[gt] = t;
      gt--;
    } else {
      i++;
    }
  }
  *lt_out = lt;
  *gt_out = gt;
}

static void sort_serial(orc_candidate_t* a, uint64_t count);

/* SIF_DEFINE_QUICKSORT_PARALLEL (include/sif/utils/sort.h:100-145): the two
 * sides of a partition of more than SIF_QUICKSORT_TASK_CUTOFF (65536)
 * elements sorted as OpenMP tasks; the same permutation as the serial sort. */
#define SORT_TASK_CUTOFF 65536
static void sort_tasks(orc_candidate_t* a, int64_t lo, int64_t hi) {
  if (hi - lo < SORT_TASK_CUTOFF) {
    if (hi > lo)
      sort_serial(a + lo, (uint64_t)(hi - lo + 1));
    return;
  }
  int64_t lt, gt;
  partition3_cand(a, lo, hi, &lt, &gt);
#pragma omp task untied
  sort_tasks(a, lo, lt - 1);
  sort_tasks(a, gt + 1, hi);
}

void orc_sort_candidates(orc_candidate_t* a, uint64_t count) {
  if (count <= SORT_TASK_CUTOFF) {
    sort_serial(a, count);
    return;
  }
#pragma omp parallel
#pragma omp single nowait
  sort_tasks(a, 0, (int64_t)count - 1);
}

static void sort_serial(orc_candidate_t* a, uint64_t count) {
  if (count < 2)
    return;
  int64_t* stack = malloc(sizeof(int64_t) * 2 * 128);
  size_t cap = 128, top = 0;
  stack[top * 2] = 0;
  stack[top * 2 + 1] = (int64_t)count - 1;
  top++;
  while (top > 0) {
    top--;
    const int64_t lo = stack[top * 2], hi = stack[top * 2 + 1];
    if (lo >= hi)
      continue;
    const float pivot = a[lo + (hi - lo) / 2].delta;
    int64_t lt = lo, i = lo, gt = hi;
    while (i <= gt) {
      const float v = a[i].delta;
      if (v < pivot) {
        const orc_candidate_t t = a[lt];
        a[lt] = a[i];
        a[i] = t;
        lt++;
        i++;
      } else if (pivot < v) {
        const orc_candidate_t t = a[i];
        a[i] = a[gt];
        a[gt] = t;
        gt--;
      } else {
        i++;
      }
    }
    if (top + 2 > cap) {
      cap *= 2;
      stack = realloc(stack, sizeof(int64_t) * 2 * cap);
    }
    stack[top * 2] = lo;
    stack[top * 2 + 1] = lt - 1;
    top++;
    stack[top * 2] = gt + 1;
    stack[top * 2 + 1] = hi;
    top++;
  }
  free(stack);
}

/* ------------------------------------------------------------------------ */
/* The rescaling                                                            */
/* ------------------------------------------------------------------------ */

#define CELL_CORE   1
#define CELL_STRADDLE 2
#define CELL_EDGE   3
#define CELL_SHELL  4

/* sif__exodus_template_build, src/finder/exodus_rescale.c:175-283. */
int orc_template_build(orc_template_t* t, uint32_t mesh_n, float cell_length,
  float rmin, float r_search) {
  memset(t, 0, sizeof(*t));
  const int32_t cr = (int32_t)(r_search / cell_length) + 1;
  if (cr >= (int32_t)mesh_n)
    return -3;
  const uint64_t max = (uint64_t)(2 * cr + 1) * (2 * cr + 1) * (2 * cr + 1);
  t->dx = malloc(max * sizeof(int32_t));
  t->dy = malloc(max * sizeof(int32_t));
  t->dz = malloc(max * sizeof(int32_t));
  t->type = malloc(max);
  t->min_d2 = malloc(max * sizeof(float));
  t->max_d2 = malloc(max * sizeof(float));
  const float rs2 = r_search * r_search;
  const float rc2 = rmin * rmin;
  for (int32_t dx = -cr; dx <= cr; dx++)
    for (int32_t dy = -cr; dy <= cr; dy++)
      for (int32_t dz = -cr; dz <= cr; dz++) {
        const float mnx = dx == 0 ? 0.0f : (fabsf((float)dx) - 1.0f) * cell_length;
        const float mny = dy == 0 ? 0.0f : (fabsf((float)dy) - 1.0f) * cell_length;
        const float mnz = dz == 0 ? 0.0f : (fabsf((float)dz) - 1.0f) * cell_length;
        const float mn = mnx * mnx + mny * mny + mnz * mnz;
        if (mn > rs2)
          continue;
        const float mxx = (fabsf((float)dx) + 1.0f) * cell_length;
        const float mxy = (fabsf((float)dy) + 1.0f) * cell_length;
        const float mxz = (fabsf((float)dz) + 1.0f) * cell_length;
        const float mx = mxx * mxx + mxy * mxy + mxz * mxz;
        const uint32_t k = t->count++;
        t->dx[k] = dx;
        t->dy[k] = dy;
        t->dz[k] = dz;
        t->min_d2[k] = mn;
        t->max_d2[k] = mx;
        if (mx <= rc2)
          t->type[k] = CELL_CORE;
        else if (mn > rc2)
          t->type[k] = mx <= rs2 ? CELL_SHELL : CELL_EDGE;
        else
          t->type[k] = CELL_STRADDLE;
      }
  return 0;
}

void orc_template_free(orc_template_t* t) {
  free(t->dx);
  free(t->dy);
  free(t->dz);
  free(t->type);
  free(t->min_d2);
  free(t->max_d2);
  memset(t, 0, sizeof(*t));
}

typedef struct {
  const orc_mesh_t* m;
  const orc_template_t* t;
  float cx, cy, cz;
  int32_t ix, iy, iz;
} query_t;

/* query_cell, src/finder/exodus_rescale.c:295-342: the wrapped cell and the
 * periodic image of the centre its particles are measured against. */
static inline int query_cell(const query_t* q, uint32_t i, uint64_t* s,
  uint64_t* e, float* ex, float* ey, float* ez) {
  const int32_t N = (int32_t)q->m->n_cells;
  const float L = q->m->box_length;
  int32_t ix = q->ix + q->t->dx[i];
  float cx = q->cx;
  if (ix < 0) {
    ix += N;
    cx += L;
  } else if (ix >= N) {
    ix -= N;
    cx -= L;
  }
  int32_t iy = q->iy + q->t->dy[i];
  float cy = q->cy;
  if (iy < 0) {
    iy += N;
    cy += L;
  } else if (iy >= N) {
    iy -= N;
    cy -= L;
  }
  int32_t iz = q->iz + q->t->dz[i];
  float cz = q->cz;
  if (iz < 0) {
    iz += N;
    cz += L;
  } else if (iz >= N) {
    iz -= N;
    cz -= L;
  }
  const uint64_t flat = (uint64_t)ix * N * N + (uint64_t)iy * N + (uint64_t)iz;
  *s = q->m->offsets[flat];
  *e = q->m->offsets[flat + 1];
  *ex = cx;
  *ey = cy;
  *ez = cz;
  return *e > *s;
}

/* The flat index of the cell query_cell() wraps template entry i into. */
static inline uint64_t query_flat(const query_t* q, uint32_t i) {
  const int32_t N = (int32_t)q->m->n_cells;
  int32_t a[3] = {q->ix + q->t->dx[i], q->iy + q->t->dy[i], q->iz + q->t->dz[i]};
  for (int k = 0; k < 3; k++)
    a[k] = a[k] < 0 ? a[k] + N : (a[k] >= N ? a[k] - N : a[k]);
  return (uint64_t)a[0] * N * N + (uint64_t)a[1] * N + (uint64_t)a[2];
}

/* dist2, src/finder/exodus_rescale.c:349-355. */
static inline float dist2(float px, float py, float pz, float cx, float cy, float cz) {
  const float dx = px - cx;
  const float dy = py - cy;
  const float dz = pz - cz;
  return dx * dx + dy * dy + dz * dz;
}

/* bin_of, src/finder/exodus_rescale.c:360-369. */
static inline uint32_t bin_of(float d2, float rc2, float inv_w, uint32_t nb) {
  const int32_t b = (int32_t)((d2 - rc2) * inv_w);
  if (b < 0)
    return 0;
  if ((uint32_t)b >= nb)
    return nb - 1;
  return (uint32_t)b;
}

static int cmp_float(const void* a, const void* b) {
  const float x = *(const float*)a, y = *(const float*)b;
  return (x > y) - (x < y);
}

/* A weighted refinement entry (exodus_internal.h:84-88) and the reference's
 * three-way quicksort over them by d2 ascending (sort_pairs_asc,
 * exodus_rescale.c:29, the SIF_DEFINE_QUICKSORT of include/sif/utils/
 * sort.h:56-98): middle pivot, the same swaps, so ties of d2 come out in the
 * reference's order and the double walk subtracts their weights in its order. */
typedef struct {
  float d2;
  float w;
} pair_t;

static void pairs_partition(pair_t* a, int64_t lo, int64_t hi, int64_t* lt_out,
  int64_t* gt_out) {
  int64_t lt = lo, gt = hi, i = lo;
  const pair_t pivot = a[lo + (hi - lo) / 2];
  while (i <= gt) {
    if (a[i].d2 < pivot.d2) {
      const pair_t t = a[lt];
      a[lt] = a[i];
      a[i] = t;
      lt++;
      i++;
    } else if (pivot.d2 < a[i].d2) {
      const pair_t t = a[i];
      a[i] = a[gt];
      a[gt] = t;
      gt--;
    } else {
      i++;
    }
  }
  *lt_out = lt;
  *gt_out = gt;
}

static void pairs_sort(pair_t* a, int64_t lo, int64_t hi) {
  if (lo >= hi)
    return;
  int64_t lt, gt;
  pairs_partition(a, lo, hi, &lt, &gt);
  pairs_sort(a, lo, lt - 1);
  pairs_sort(a, gt + 1, hi);
}

/* resolve_bin, src/finder/exodus_rescale.c:391-507. Unweighted, the
 * collected distances are equal values wherever they tie, so any ascending
 * sort gives the reference's sequence; weighted, the pairs are sorted as the
 * reference sorts them. cur_w is the weight at or below the window's top. */
static int resolve(const query_t* q, uint32_t blo, uint32_t bhi, float lo,
  float hi, float rc2, float rs2, float inv_w, uint32_t nb, uint64_t cur_n,
  double cur_w, float K2, float* out, void** buf, uint64_t* cap, int weighted) {
  const orc_template_t* t = q->t;
  const size_t esz = weighted ? sizeof(pair_t) : sizeof(float);
  uint64_t count = 0;
  for (uint32_t i = 0; i < t->count; i++) {
    const uint8_t type = t->type[i];
    if (type == CELL_CORE || t->max_d2[i] < lo || t->min_d2[i] > hi)
      continue;
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(q, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (count + (e - s) > *cap) {
      while (count + (e - s) > *cap)
        *cap *= 2;
      *buf = realloc(*buf, *cap * esz);
    }
    for (uint64_t p = s; p < e; p++) {
      const float d2 = dist2(q->m->x[p], q->m->y[p], q->m->z[p], ex, ey, ez);
      if (type != CELL_SHELL && !(d2 > rc2 && d2 <= rs2))
        continue;
      const uint32_t bi = bin_of(d2, rc2, inv_w, nb);
      if (bi < blo || bi > bhi)
        continue;
      if (weighted)
        ((pair_t*)*buf)[count++] = (pair_t){d2, q->m->w[p]};
      else
        ((float*)*buf)[count++] = d2;
    }
  }
  if (weighted) {
    pair_t* pr = (pair_t*)*buf;
    if (count > 1)
      pairs_sort(pr, 0, (int64_t)count - 1);
    for (int64_t k = (int64_t)count - 1; k >= 0; k--) {
      const float d2 = pr[k].d2;
      const double wt = (double)pr[k].w;
      if (d2 == 0.0f) {
        cur_w -= wt;
        continue;
      }
      const float w_in = (float)(cur_w - wt);
      const float d2c = d2 * d2 * d2;
      if (w_in * w_in <= K2 * d2c) {
        *out = sqrtf(d2);
        return 1;
      }
      cur_w -= wt;
    }
    return 0;
  }
  float* fb = (float*)*buf;
  if (count > 1)
    qsort(fb, count, sizeof(float), cmp_float);
  for (int64_t k = (int64_t)count - 1; k >= 0; k--) {
    const float d2 = fb[k];
    if (d2 == 0.0f) {
      cur_n--;
      continue;
    }
    const uint64_t n_in = cur_n - 1;
    const float d2c = d2 * d2 * d2;
    const float rn = (float)n_in;
    if (rn * rn <= K2 * d2c) {
      *out = sqrtf(d2);
      return 1;
    }
    cur_n--;
  }
  return 0;
}

/* find_exact_radius_impl, src/finder/exodus_rescale.c:642-1012. Weighted
 * (the mesh's w set), every count is a double sum of weights taken in the
 * reference's order -- whole cells from cell_w, the rest tracer by tracer --
 * and the density tests use mass_factor; vol_factor still sizes the
 * histogram. */
static float find_radius_impl(const orc_mesh_t* m, const orc_template_t* t, float cx,
  float cy, float cz, float r_search, float threshold, float vol_factor, float mass_factor,
  float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum, uint64_t* span_count,
  int weighted) {
  *reason = ORC_RESCALE_OK;
  const float inv_l = 1.0f / m->cell_length;
  const query_t q = {m, t, cx, cy, cz, (int32_t)(cx * inv_l),
    (int32_t)(cy * inv_l), (int32_t)(cz * inv_l)};
  const float rs2 = r_search * r_search;
  const float rc2 = rmin * rmin;
  const float* mw = m->w;
  const float* cw = m->cell_w;

  const float span = rs2 - rc2;
  uint32_t nb = 2048u;
  {
    const float expected_shell =
      vol_factor * (r_search * r_search * r_search - rmin * rmin * rmin);
    const float want = expected_shell / 16.0f;
    if (!(want >= 64.0f))
      nb = 64u;
    else if (want < 2048.0f)
      nb = (uint32_t)want;
  }
  if (!(span > 0.0f)) {
    *reason = ORC_RESCALE_DEGENERATE;
    return -1.0f;
  }

  /* The early refusal, 738-782. */
  {
    const float expected = mass_factor * r_search * r_search * r_search;
    uint64_t within = 0;
    double w_within = 0.0;
    for (uint32_t i = 0; i < t->count; i++) {
      const uint8_t type = t->type[i];
      uint64_t s, e;
      float ex, ey, ez;
      if (!query_cell(&q, i, &s, &e, &ex, &ey, &ez))
        continue;
      if (type == CELL_CORE || type == CELL_SHELL) {
        if (weighted) {
          w_within += (double)cw[query_flat(&q, i)];
        } else {
          within += e - s;
        }
        continue;
      }
      if (weighted) {
        for (uint64_t p = s; p < e; p++)
          if (dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez) <= rs2)
            w_within += (double)mw[p];
      } else {
        for (uint64_t p = s; p < e; p++)
          within += dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez) <= rs2;
      }
    }
    if (weighted ? !(w_within > 0.0) : within == 0) {
      *reason = ORC_RESCALE_EMPTY;
      return -1.0f;
    }
    const float wf = weighted ? (float)w_within : (float)within;
    if ((wf / expected) - 1.0f <= threshold) {
      *reason = ORC_RESCALE_BEYOND_SEARCH;
      return -1.0f;
    }
  }

  const float inv_w = (float)nb / span;
  const float bin_w = span / (float)nb;
  uint32_t* bins = calloc(nb, sizeof(uint32_t));
  double* wbins = calloc(nb, sizeof(double));
  uint64_t n_core = 0, n_shell = 0;
  double w_core = 0.0, w_shell = 0.0;
  for (uint32_t i = 0; i < t->count; i++) {
    const uint8_t type = t->type[i];
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(&q, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (type == CELL_CORE) {
      if (weighted) {
        w_core += (double)cw[query_flat(&q, i)];
      } else {
        n_core += e - s;
      }
    } else if (type == CELL_SHELL) {
      for (uint64_t p = s; p < e; p++) {
        const uint32_t b = bin_of(dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez), rc2, inv_w, nb);
        if (weighted) {
          wbins[b] += (double)mw[p];
          w_shell += (double)mw[p];
        } else {
          bins[b]++;
        }
      }
      if (!weighted)
        n_shell += e - s;
    } else {
      for (uint64_t p = s; p < e; p++) {
        const float d2 = dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez);
        if (weighted) {
          const double wt = (double)mw[p];
          if (d2 <= rc2) {
            w_core += wt;
          } else if (d2 <= rs2) {
            wbins[bin_of(d2, rc2, inv_w, nb)] += wt;
            w_shell += wt;
          }
        } else {
          n_core += d2 <= rc2;
          if (d2 > rc2 && d2 <= rs2) {
            bins[bin_of(d2, rc2, inv_w, nb)]++;
            n_shell++;
          }
        }
      }
    }
  }

  const uint64_t total = n_core + n_shell;
  const double total_w = w_core + w_shell;
  if (weighted ? !(total_w > 0.0) : total == 0) {
    free(bins);
    free(wbins);
    *reason = ORC_RESCALE_EMPTY;
    return -1.0f;
  }
  {
    const float expected = mass_factor * r_search * r_search * r_search;
    const float tf = weighted ? (float)total_w : (float)total;
    if ((tf / expected) - 1.0f <= threshold) {
      free(bins);
      free(wbins);
      *reason = ORC_RESCALE_BEYOND_SEARCH;
      return -1.0f;
    }
  }

  const float K = (threshold + 1.0f) * mass_factor;
  const float K2 = K * K;
  uint64_t above = 0;
  double above_w = 0.0;
  int32_t b_first = -1;
  uint64_t cap = 4096;
  void* buf = malloc(cap * (weighted ? sizeof(pair_t) : sizeof(float)));
  float result = -1.0f;
  *reason = ORC_RESCALE_BELOW_RUNG;
  for (int32_t b = (int32_t)nb - 1; b >= 0; b--) {
    const uint32_t count = weighted ? 0u : bins[b];
    const double count_w = weighted ? wbins[b] : 0.0;
    if (weighted ? !(count_w > 0.0) : count == 0)
      continue;
    float hi = rc2 + (float)(b + 1) * bin_w;
    if (b == (int32_t)nb - 1)
      hi = rs2 * (1.0f + 1e-6f);
    const float n_in_min =
      weighted ? (float)(total_w - above_w - count_w) : (float)(total - above - count);
    if (n_in_min * n_in_min > K2 * hi * hi * hi) {
      if (weighted)
        above_w += count_w;
      else
        above += count;
      continue;
    }
    if (b_first < 0)
      b_first = b;
    int32_t b_lo = b - (int32_t)(window - 1);
    if (b_lo < 0)
      b_lo = 0;
    uint64_t wcount = 0;
    double wsum = 0.0;
    for (int32_t bb = b_lo; bb <= b; bb++) {
      if (weighted)
        wsum += wbins[bb];
      else
        wcount += bins[bb];
    }
    const float win_lo = rc2 + (float)b_lo * bin_w;
    float r = -1.0f;
    if (resolve(&q, (uint32_t)b_lo, (uint32_t)b, win_lo, hi, rc2, rs2, inv_w, nb,
          total - above, total_w - above_w, K2, &r, &buf, &cap, weighted)) {
      const int32_t b_found = (int32_t)bin_of(r * r, rc2, inv_w, nb);
      int32_t reached = b_first - b_found + 1;
      if (reached < 1)
        reached = 1;
      if (span_sum)
        *span_sum += (uint64_t)reached;
      if (span_count)
        (*span_count)++;
      result = r;
      *reason = ORC_RESCALE_OK;
      break;
    }
    if (weighted)
      above_w += wsum;
    else
      above += wcount;
    b = b_lo;
  }
  free(buf);
  free(bins);
  free(wbins);
  return result;
}

float orc_find_radius(const orc_mesh_t* m, const orc_template_t* t, float cx,
  float cy, float cz, float r_search, float threshold, float vol_factor,
  float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum,
  uint64_t* span_count) {
  return find_radius_impl(m, t, cx, cy, cz, r_search, threshold, vol_factor, vol_factor,
    rmin, window, reason, span_sum, span_count, 0);
}

float orc_find_radius_weighted(const orc_mesh_t* m, const orc_template_t* t, float cx,
  float cy, float cz, float r_search, float threshold, float vol_factor,
  float mass_factor, float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum,
  uint64_t* span_count) {
  return find_radius_impl(m, t, cx, cy, cz, r_search, threshold, vol_factor, mass_factor,
    rmin, window, reason, span_sum, span_count, 1);
}

static int cmp_double(const void* a, const void* b) {
  const double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* The radius by definition, over every particle in the box: the outermost
 * distance d in (rung, r_search] at which the particles strictly inside are at
 * most (1 + threshold) times the mean count of a sphere of radius d; -1 when
 * none qualifies. The definition tests/test_finders.c:419-459 checks the
 * finder against; nothing here shares code with the histogram walk. */
double orc_brute_force_radius(const float* x, const float* y, const float* z,
  uint64_t n, float box, double cx, double cy, double cz, double rung,
  double r_search, double threshold) {
  const double L = (double)box, half = 0.5 * L;
  uint64_t n_core = 0, n_shell = 0;
  double* d = malloc((n ? n : 1) * sizeof(double));
  for (uint64_t p = 0; p < n; p++) {
    double dx = fabs((double)x[p] - cx), dy = fabs((double)y[p] - cy),
           dz = fabs((double)z[p] - cz);
    dx = dx > half ? L - dx : dx;
    dy = dy > half ? L - dy : dy;
    dz = dz > half ? L - dz : dz;
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (r <= rung)
      n_core++;
    else if (r <= r_search)
      d[n_shell++] = r;
  }
  qsort(d, n_shell, sizeof(double), cmp_double);
  const double k = (1.0 + threshold) * (double)n / (L * L * L) * 4.0 / 3.0 * M_PI;
  double out = -1.0;
  for (uint64_t i = n_shell; i-- > 0;) {
    if ((double)(n_core + i) <= k * d[i] * d[i] * d[i]) {
      out = d[i];
      break;
    }
  }
  free(d);
  return out;
}

/* ------------------------------------------------------------------------ */
/* Overlap tests, the mask, the void index                                  */
/* ------------------------------------------------------------------------ */

/* sif__wrap_pbc, src/finder/utils.h:25-31, for any n. */
static inline uint32_t wrap_pbc(int32_t v, uint32_t n) {
  int32_t w = v % (int32_t)n;
  return (uint32_t)(w < 0 ? w + (int32_t)n : w);
}

static inline int mask_get(const uint64_t* words, uint64_t i) {
  return (words[i >> 6] >> (i & 63)) & 1u;
}

static inline void mask_set(uint64_t* words, uint64_t i) {
  words[i >> 6] |= 1ull << (i & 63);
}

/* sif__overlap_quick, src/finder/utils.c:819-848: the six axis poles. */
static int overlap_quick(const uint64_t* mask, uint32_t n, uint32_t ix,
  uint32_t iy, uint32_t iz, uint32_t r) {
  const uint64_t nn = n;
  if (mask_get(mask, ((uint64_t)wrap_pbc((int32_t)(ix + r), n) * nn + iy) * nn + iz))
    return 1;
  if (mask_get(mask, ((uint64_t)wrap_pbc((int32_t)ix - (int32_t)r, n) * nn + iy) * nn + iz))
    return 1;
  if (mask_get(mask, ((uint64_t)ix * nn + wrap_pbc((int32_t)(iy + r), n)) * nn + iz))
    return 1;
  if (mask_get(mask, ((uint64_t)ix * nn + wrap_pbc((int32_t)iy - (int32_t)r, n)) * nn + iz))
    return 1;
  if (mask_get(mask, ((uint64_t)ix * nn + iy) * nn + wrap_pbc((int32_t)(iz + r), n)))
    return 1;
  if (mask_get(mask, ((uint64_t)ix * nn + iy) * nn + wrap_pbc((int32_t)iz - (int32_t)r, n)))
    return 1;
  return 0;
}

/* The accepted voids and their 32^3 periodic cell index
 * (src/structures/cell_linked_list.c, VOID_CLL_CELLS exodus_finder.c:219). */
#define VOID_CELLS 32
typedef struct {
  float *cx, *cy, *cz, *r;
  uint64_t n, cap;
  int32_t head[VOID_CELLS * VOID_CELLS * VOID_CELLS];
  int32_t* next;
  float inv_cell; /* (float)32 / box */
} voids_t;

static uint32_t void_axis(const voids_t* v, float c) {
  int32_t i = (int32_t)floorf(c * v->inv_cell);
  i %= VOID_CELLS;
  if (i < 0)
    i += VOID_CELLS;
  return (uint32_t)i;
}

static void voids_init(voids_t* v, float box) {
  memset(v, 0, sizeof(*v));
  memset(v->head, 0xFF, sizeof(v->head));
  v->inv_cell = (float)VOID_CELLS / box;
}

static void voids_add(voids_t* v, float cx, float cy, float cz, float r) {
  if (v->n == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 1024;
    v->cx = realloc(v->cx, v->cap * sizeof(float));
    v->cy = realloc(v->cy, v->cap * sizeof(float));
    v->cz = realloc(v->cz, v->cap * sizeof(float));
    v->r = realloc(v->r, v->cap * sizeof(float));
    v->next = realloc(v->next, v->cap * sizeof(int32_t));
  }
  const uint64_t i = v->n++;
  v->cx[i] = cx;
  v->cy[i] = cy;
  v->cz[i] = cz;
  v->r[i] = r;
  const uint64_t cell = ((uint64_t)void_axis(v, cx) * VOID_CELLS + void_axis(v, cy)) *
                          VOID_CELLS +
                        void_axis(v, cz);
  v->next[i] = v->head[cell];
  v->head[cell] = (int32_t)i;
}

static void paint_sphere(uint64_t* mask, float cx, float cy, float cz, float r,
  uint32_t n, float cell_length, int set);

static uint64_t void_cell(const voids_t* v, float cx, float cy, float cz) {
  return ((uint64_t)void_axis(v, cx) * VOID_CELLS + void_axis(v, cy)) * VOID_CELLS +
         void_axis(v, cz);
}

/* sif_cell_linked_list_remove, src/structures/cell_linked_list.c:212-232. */
static void voids_unlink(voids_t* v, uint64_t i) {
  int32_t* link = &v->head[void_cell(v, v->cx[i], v->cy[i], v->cz[i])];
  while (*link != -1 && *link != (int32_t)i)
    link = &v->next[*link];
  if (*link != -1)
    *link = v->next[i];
}

/* compact_catalogue, src/finder/exodus_finder.c:1043-1078: the displaced
 * voids (radius negated) dropped, the rest re-indexed in order. */
static void voids_compact(voids_t* v) {
  uint64_t j = 0;
  for (uint64_t i = 0; i < v->n; i++) {
    if (!(v->r[i] > 0.0f))
      continue;
    v->cx[j] = v->cx[i];
    v->cy[j] = v->cy[i];
    v->cz[j] = v->cz[i];
    v->r[j] = v->r[i];
    j++;
  }
  memset(v->head, 0xFF, sizeof(v->head));
  v->n = 0;
  for (uint64_t i = 0; i < j; i++) {
    const uint64_t cell = void_cell(v, v->cx[i], v->cy[i], v->cz[i]);
    v->next[i] = v->head[cell];
    v->head[cell] = (int32_t)i;
  }
  v->n = j;
}

/* find_conflicts, src/finder/exodus_finder.c:696-756: the accepted voids a
 * sphere at r collides with (the exact overlap's pair test, minimum image),
 * in the order the index walks them; returns their count, the largest
 * radius among them in *largest (-1 for none). */
static uint64_t find_conflicts(const voids_t* v, float max_r, float scale, float cx, float cy,
  float cz, float r, float f, float box, uint64_t** list, uint64_t* cap, float* largest) {
  const float half = 0.5f * box;
  const float reach = scale * (r + max_r - f * (r < max_r ? r : max_r));
  const float x[3] = {cx, cy, cz};
  int32_t lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = (int32_t)floorf((x[a] - reach) * v->inv_cell);
    hi[a] = (int32_t)floorf((x[a] + reach) * v->inv_cell);
    if (hi[a] - lo[a] >= VOID_CELLS) {
      lo[a] = 0;
      hi[a] = VOID_CELLS - 1;
    }
  }
  uint64_t k = 0;
  *largest = -1.0f;
  for (int32_t a = lo[0]; a <= hi[0]; a++) {
    const int32_t wa = ((a % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
    for (int32_t b = lo[1]; b <= hi[1]; b++) {
      const int32_t wb = ((b % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
      for (int32_t c = lo[2]; c <= hi[2]; c++) {
        const int32_t wc = ((c % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
        for (int32_t i = v->head[(wa * VOID_CELLS + wb) * VOID_CELLS + wc]; i != -1;
             i = v->next[i]) {
          float dx = fabsf(cx - v->cx[i]);
          float dy = fabsf(cy - v->cy[i]);
          float dz = fabsf(cz - v->cz[i]);
          dx = dx > half ? box - dx : dx;
          dy = dy > half ? box - dy : dy;
          dz = dz > half ? box - dz : dz;
          const float ri = v->r[i];
          const float tot = scale * (r + ri - f * (r < ri ? r : ri));
          if (dx * dx + dy * dy + dz * dz >= tot * tot)
            continue;
          if (k == *cap) {
            *cap = *cap ? 2 * *cap : 64;
            *list = realloc(*list, *cap * sizeof(uint64_t));
          }
          (*list)[k++] = (uint64_t)i;
          if (ri > *largest)
            *largest = ri;
        }
      }
    }
  }
  return k;
}

/* displace_void, src/finder/exodus_finder.c:946-1037: void i leaves the
 * index, its radius is negated, its sphere cleared from the mask, and the
 * spheres of the voids still indexed that intersect it painted back. */
static void displace_void(voids_t* v, uint64_t* mask, uint64_t i, float max_r, float scale,
  uint32_t n, float cell, float box) {
  const float cx = v->cx[i], cy = v->cy[i], cz = v->cz[i], r = v->r[i];
  voids_unlink(v, i);
  v->r[i] = -r;
  paint_sphere(mask, cx, cy, cz, scale * r, n, cell, 0);
  const float half = 0.5f * box;
  const float reach = scale * (r + max_r);
  const float x[3] = {cx, cy, cz};
  int32_t lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = (int32_t)floorf((x[a] - reach) * v->inv_cell);
    hi[a] = (int32_t)floorf((x[a] + reach) * v->inv_cell);
    if (hi[a] - lo[a] >= VOID_CELLS) {
      lo[a] = 0;
      hi[a] = VOID_CELLS - 1;
    }
  }
  for (int32_t a = lo[0]; a <= hi[0]; a++)
    for (int32_t b = lo[1]; b <= hi[1]; b++)
      for (int32_t c = lo[2]; c <= hi[2]; c++) {
        const int32_t wa = ((a % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
        const int32_t wb = ((b % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
        const int32_t wc = ((c % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
        for (int32_t j = v->head[(wa * VOID_CELLS + wb) * VOID_CELLS + wc]; j != -1;
             j = v->next[j]) {
          float dx = fabsf(cx - v->cx[j]);
          float dy = fabsf(cy - v->cy[j]);
          float dz = fabsf(cz - v->cz[j]);
          dx = dx > half ? box - dx : dx;
          dy = dy > half ? box - dy : dy;
          dz = dz > half ? box - dz : dz;
          const float t = scale * (r + v->r[j]);
          if (dx * dx + dy * dy + dz * dz < t * t)
            paint_sphere(mask, v->cx[j], v->cy[j], v->cz[j], scale * v->r[j], n, cell, 1);
        }
      }
}

static void voids_free(voids_t* v) {
  free(v->cx);
  free(v->cy);
  free(v->cz);
  free(v->r);
  free(v->next);
}

/* sif__overlap_exact, src/finder/utils.c:850-960. */
static int overlap_exact(const voids_t* v, float cx, float cy, float cz,
  float r, float max_r, float box, float f, float scale) {
  const float half = box * 0.5f;
  const float search = scale * (r + max_r - f * (r < max_r ? r : max_r));
  const float inv = v->inv_cell;
  const int32_t x0 = (int32_t)floorf((cx - search) * inv);
  const int32_t x1 = (int32_t)floorf((cx + search) * inv);
  const int32_t y0 = (int32_t)floorf((cy - search) * inv);
  const int32_t y1 = (int32_t)floorf((cy + search) * inv);
  const int32_t z0 = (int32_t)floorf((cz - search) * inv);
  const int32_t z1 = (int32_t)floorf((cz + search) * inv);
  const int interior = (cx - search >= 0.0f) && (cx + search < box) &&
                       (cy - search >= 0.0f) && (cy + search < box) &&
                       (cz - search >= 0.0f) && (cz + search < box);
  for (int32_t ix = x0; ix <= x1; ix++) {
    const uint32_t wx = (uint32_t)ix & (VOID_CELLS - 1);
    for (int32_t iy = y0; iy <= y1; iy++) {
      const uint32_t wy = (uint32_t)iy & (VOID_CELLS - 1);
      for (int32_t iz = z0; iz <= z1; iz++) {
        const uint32_t wz = (uint32_t)iz & (VOID_CELLS - 1);
        int32_t j = v->head[(wx * VOID_CELLS + wy) * VOID_CELLS + wz];
        while (j != -1) {
          const float rj = v->r[j];
          const float mn = r < rj ? r : rj;
          const float tot = scale * (r + rj - f * mn);
          const float tot2 = tot * tot;
          if (interior) {
            const float dx = cx - v->cx[j];
            const float dy = cy - v->cy[j];
            const float dz = cz - v->cz[j];
            if (dx * dx + dy * dy + dz * dz < tot2)
              return 1;
          } else {
            float dx = fabsf(cx - v->cx[j]);
            dx = dx > half ? box - dx : dx;
            const float dx2 = dx * dx;
            if (dx2 < tot2) {
              float dy = fabsf(cy - v->cy[j]);
              dy = dy > half ? box - dy : dy;
              const float dy2 = dy * dy;
              if (dx2 + dy2 < tot2) {
                float dz = fabsf(cz - v->cz[j]);
                dz = dz > half ? box - dz : dz;
                if (dx2 + dy2 + dz * dz < tot2)
                  return 1;
              }
            }
          }
          j = v->next[j];
        }
      }
    }
  }
  return 0;
}

/* paint_sphere with set = 1, src/finder/utils.c:965-1027. */
static inline void mask_clear(uint64_t* words, uint64_t i) {
  words[i >> 6] &= ~(1ull << (i & 63));
}

static void mark_sphere(uint64_t* mask, float cx, float cy, float cz, float r,
  uint32_t n, float cell_length) {
  paint_sphere(mask, cx, cy, cz, r, n, cell_length, 1);
}

/* paint_sphere, src/finder/utils.c:965-1027: set (sif__mark_sphere) or
 * clear (sif__clear_sphere) every node within r. */
static void paint_sphere(uint64_t* mask, float cx, float cy, float cz, float r,
  uint32_t n, float cell_length, int set) {
  const float r2 = r * r;
  const float inv = 1.0f / cell_length;
  const float box = (float)n * cell_length;
  const float half = box * 0.5f;
  const int32_t cr = (int32_t)(r * inv) + 1;
  const int32_t ci = (int32_t)(cx * inv), cj = (int32_t)(cy * inv),
                ck = (int32_t)(cz * inv);
  for (int32_t dx = -cr; dx <= cr; dx++) {
    const int32_t gx = ci + dx;
    float ddx = fabsf((float)gx * cell_length - cx);
    ddx = ddx > half ? box - ddx : ddx;
    const float dx2 = ddx * ddx;
    if (dx2 > r2)
      continue;
    const uint32_t wx = wrap_pbc(gx, n);
    for (int32_t dy = -cr; dy <= cr; dy++) {
      const int32_t gy = cj + dy;
      float ddy = fabsf((float)gy * cell_length - cy);
      ddy = ddy > half ? box - ddy : ddy;
      const float dxy2 = dx2 + ddy * ddy;
      if (dxy2 > r2)
        continue;
      const uint32_t wy = wrap_pbc(gy, n);
      for (int32_t dz = -cr; dz <= cr; dz++) {
        const int32_t gz = ck + dz;
        float ddz = fabsf((float)gz * cell_length - cz);
        ddz = ddz > half ? box - ddz : ddz;
        if (dxy2 + ddz * ddz <= r2) {
          const uint64_t cell = ((uint64_t)wx * n + wy) * n + wrap_pbc(gz, n);
          if (set)
            mask_set(mask, cell);
          else
            mask_clear(mask, cell);
        }
      }
    }
  }
}

/* collision_radius, src/finder/exodus_finder.c:780-845: voids smaller than
 * min_rj left out (under displacement only a larger void refuses). */
#define COLLISION_SLACK 1e-5
static double collision_radius(const voids_t* v, float max_acc, float scale_f,
  float cx, float cy, float cz, float r_hi, float min_rj, float f, float box) {
  const double L = (double)box, half = 0.5 * L, ff = (double)f,
               scale = (double)scale_f;
  const float reach = scale_f * (r_hi + max_acc);
  const float x[3] = {cx, cy, cz};
  int32_t lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = (int32_t)floorf((x[a] - reach) * v->inv_cell);
    hi[a] = (int32_t)floorf((x[a] + reach) * v->inv_cell);
    if (hi[a] - lo[a] >= VOID_CELLS) {
      lo[a] = 0;
      hi[a] = VOID_CELLS - 1;
    }
  }
  double best = INFINITY;
  for (int32_t a = lo[0]; a <= hi[0]; a++) {
    const int32_t wa = ((a % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
    for (int32_t b = lo[1]; b <= hi[1]; b++) {
      const int32_t wb = ((b % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
      for (int32_t c = lo[2]; c <= hi[2]; c++) {
        const int32_t wc = ((c % VOID_CELLS) + VOID_CELLS) % VOID_CELLS;
        for (int32_t i = v->head[(wa * VOID_CELLS + wb) * VOID_CELLS + wc]; i != -1;
             i = v->next[i]) {
          const double rj = (double)v->r[i];
          if (v->r[i] < min_rj)
            continue;
          double dx = fabs((double)cx - (double)v->cx[i]);
          double dy = fabs((double)cy - (double)v->cy[i]);
          double dz = fabs((double)cz - (double)v->cz[i]);
          dx = dx > half ? L - dx : dx;
          dy = dy > half ? L - dy : dy;
          dz = dz > half ? L - dz : dz;
          const double D = (sqrt(dx * dx + dy * dy + dz * dz) +
                             COLLISION_SLACK * (L + (double)r_hi + rj)) /
                           scale;
          double rs;
          if (D <= rj)
            rs = 0.0;
          else if (D <= (2.0 - ff) * rj)
            rs = (D - rj) / (1.0 - ff);
          else
            rs = D - (1.0 - ff) * rj;
          if (rs < best)
            best = rs;
        }
      }
    }
  }
  return best;
}

/* sif__exodus_witness, src/finder/exodus_rescale.c:1074-1167 (closed = 0). */
#define WITNESS_SLACK 1e-5f
static int witness(const orc_mesh_t* m, const orc_template_t* t, float cx,
  float cy, float cz, float rho2, float r_search, float threshold,
  float vol_factor, int closed) {
  const float inv_l = 1.0f / m->cell_length;
  const query_t q = {m, t, cx, cy, cz, (int32_t)(cx * inv_l),
    (int32_t)(cy * inv_l), (int32_t)(cz * inv_l)};
  const float rs2 = r_search * r_search;
  if (!(rho2 < rs2))
    return 0;
  const float K = (threshold + 1.0f) * vol_factor;
  const float K2 = K * K;
  const float bound = K2 * (rho2 * rho2 * rho2) * (1.0f - WITNESS_SLACK);
  const double n_cap = sqrt((double)bound) + 2.0;
  const float whole_in = rho2 * (1.0f - WITNESS_SLACK);
  const float whole_out = rho2 * (1.0f + WITNESS_SLACK);
  uint64_t n = 0, within = 0;
  int beyond = 0;
  for (uint32_t i = 0; i < t->count; i++) {
    const uint8_t type = t->type[i];
    if (!closed && beyond && t->min_d2[i] > whole_out)
      continue;
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(&q, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (type == CELL_CORE || t->max_d2[i] <= whole_in) {
      n += e - s;
      within += e - s;
    } else if (type == CELL_SHELL && t->min_d2[i] > whole_out) {
      within += e - s;
      beyond = 1;
    } else {
      for (uint64_t p = s; p < e; p++) {
        const float d2 = dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez);
        if (d2 <= rho2) {
          n++;
          within++;
        } else if (type == CELL_SHELL || d2 <= rs2) {
          within++;
          beyond = 1;
        }
      }
    }
    if ((double)n > n_cap)
      return 0;
  }
  const float rn = (float)n;
  if (!beyond || !(rn * rn <= bound))
    return 0;
  if (closed) {
    /* The search sphere must not be underdense out to r_search (the
     * rescaling's refusal is within / expected - 1 <= threshold). */
    const double expected = (double)vol_factor * (double)r_search * (double)r_search *
                            (double)r_search;
    if (!((double)within > (1.0 + (double)threshold) * expected * (1.0 + WITNESS_SLACK)))
      return 0;
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* The run                                                                  */
/* ------------------------------------------------------------------------ */

#define BATCH_MAX 4096u
#define BATCH_PER_THREAD 8u
#define BATCH_FLOOR 32u
#define RESOLVE_INITIAL 8u

#define ST_PROXY 1
#define ST_MESH 2
#define ST_RESCALE 3
#define ST_ACCEPTED 4
#define ST_WITNESS 5

typedef struct {
  uint8_t status;
  float r;
  float cx, cy, cz;
  uint32_t ix, iy, iz;
} result_t;

static int cmp_desc(const void* a, const void* b) {
  const float x = *(const float*)a, y = *(const float*)b;
  return (x < y) - (x > y);
}

/* is_minimum of src/finder/utils.c:243-259 over the 27-node stencil of
 * load_stencil (utils.c:221-241): the node is strictly below every neighbour
 * at a lower flat index and not above any at a higher one, so of a run of
 * equal values exactly the lowest-indexed is a minimum. */
static int is_minimum_node(const float* f, uint32_t n, uint64_t i) {
  const uint32_t ix = (uint32_t)(i / ((uint64_t)n * n)), iy = (uint32_t)((i / n) % n),
                 iz = (uint32_t)(i % n);
  const uint32_t xs[3] = {(ix + n - 1) % n, ix, (ix + 1) % n};
  const uint32_t ys[3] = {(iy + n - 1) % n, iy, (iy + 1) % n};
  const uint32_t zs[3] = {(iz + n - 1) % n, iz, (iz + 1) % n};
  const float v = f[i];
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) {
        const uint64_t j = ((uint64_t)xs[a] * n + ys[b]) * n + zs[c];
        if (a == 1 && b == 1 && c == 1)
          continue;
        if (j < i ? !(v < f[j]) : !(v <= f[j]))
          return 0;
      }
  return 1;
}

/* A refined candidate's offset off its node, in cells (sif_offset_t,
 * src/finder/utils.h:164-172). */
typedef struct {
  float dx, dy, dz;
} orc_offset_t;

/* newton_step, src/finder/utils.c:261-313: gradient and Hessian by central
 * differences on the 27-node stencil (cross terms included), d = -H^-1 g by
 * cofactors, in double; 0 unless H is positive definite (Sylvester's leading
 * minors) and the step is within MINIMUM_MAX_STEP (one cell) on every axis.
 * s[(a+1)*9 + (b+1)*3 + (c+1)] holds the value at offset (a, b, c). */
static int newton_step(const float s[27], double d[3], double* depth) {
#define S(a, b, c) ((double)s[((a) + 1) * 9 + ((b) + 1) * 3 + ((c) + 1)])
  const double c0 = S(0, 0, 0);
  const double g0 = 0.5 * (S(1, 0, 0) - S(-1, 0, 0));
  const double g1 = 0.5 * (S(0, 1, 0) - S(0, -1, 0));
  const double g2 = 0.5 * (S(0, 0, 1) - S(0, 0, -1));
  const double h00 = S(1, 0, 0) - 2.0 * c0 + S(-1, 0, 0);
  const double h11 = S(0, 1, 0) - 2.0 * c0 + S(0, -1, 0);
  const double h22 = S(0, 0, 1) - 2.0 * c0 + S(0, 0, -1);
  const double h01 = 0.25 * (S(1, 1, 0) - S(1, -1, 0) - S(-1, 1, 0) + S(-1, -1, 0));
  const double h02 = 0.25 * (S(1, 0, 1) - S(1, 0, -1) - S(-1, 0, 1) + S(-1, 0, -1));
  const double h12 = 0.25 * (S(0, 1, 1) - S(0, 1, -1) - S(0, -1, 1) + S(0, -1, -1));
#undef S
  const double k00 = h11 * h22 - h12 * h12;
  const double k01 = h02 * h12 - h01 * h22;
  const double k02 = h01 * h12 - h02 * h11;
  const double k11 = h00 * h22 - h02 * h02;
  const double k12 = h01 * h02 - h00 * h12;
  const double k22 = h00 * h11 - h01 * h01;
  const double det = h00 * k00 + h01 * k01 + h02 * k02;
  if (!(h00 > 0.0 && k22 > 0.0 && det > 0.0))
    return 0;
  d[0] = -(k00 * g0 + k01 * g1 + k02 * g2) / det;
  d[1] = -(k01 * g0 + k11 * g1 + k12 * g2) / det;
  d[2] = -(k02 * g0 + k12 * g1 + k22 * g2) / det;
  if (!(fabs(d[0]) <= 1.0 && fabs(d[1]) <= 1.0 && fabs(d[2]) <= 1.0))
    return 0;
  *depth = c0 + 0.5 * (g0 * d[0] + g1 * d[1] + g2 * d[2]);
  return 1;
}

/* The 27 values around node i (load_stencil, utils.c:227-241). */
static void load_stencil27(const float* f, uint32_t n, uint64_t i, float s[27]) {
  const uint32_t ix = (uint32_t)(i / ((uint64_t)n * n)), iy = (uint32_t)((i / n) % n),
                 iz = (uint32_t)(i % n);
  const uint32_t xs[3] = {(ix + n - 1) % n, ix, (ix + 1) % n};
  const uint32_t ys[3] = {(iy + n - 1) % n, iy, (iy + 1) % n};
  const uint32_t zs[3] = {(iz + n - 1) % n, iz, (iz + 1) % n};
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++)
        s[a * 9 + b * 3 + c] = f[((uint64_t)xs[a] * n + ys[b]) * n + zs[c]];
}

/* step_cells, utils.c:317-319: a step of exactly half a cell stays. */
static int32_t step_cells(double d) { return d > 0.5 ? 1 : (d < -0.5 ? -1 : 0); }

/* candidate_centre, exodus_finder.c:371-393: node plus offset, in cells,
 * times the cell length, wrapped into the box. */
static void cand_centre(const orc_candidate_t* c, const orc_offset_t* offs, uint32_t N,
  float cell, float box, float out[3]) {
  const uint32_t node[3] = {(uint32_t)(c->flat / ((uint64_t)N * N)),
    (uint32_t)((c->flat / N) % N), (uint32_t)(c->flat % N)};
  float off[3] = {0.0f, 0.0f, 0.0f};
  if (c->refined) {
    const orc_offset_t* o = &offs[c->refined - 1];
    off[0] = o->dx;
    off[1] = o->dy;
    off[2] = o->dz;
  }
  for (int a = 0; a < 3; a++) {
    float x = ((float)node[a] + off[a]) * cell;
    if (x < 0.0f)
      x += box;
    if (x >= box)
      x -= box;
    out[a] = x;
  }
}

/* masked_overlap, exodus_finder.c:440-452: the node's mask bit; for a
 * centre refined off its node, only while the offset is within
 * scale * r * (1 - f). */
static int cand_masked(const uint64_t* mask, const orc_candidate_t* c, const orc_offset_t* offs,
  float r, float f, float scale, float cell) {
  if (!mask_get(mask, c->flat))
    return 0;
  if (!c->refined)
    return 1;
  const orc_offset_t* o = &offs[c->refined - 1];
  const float off = sqrtf(o->dx * o->dx + o->dy * o->dy + o->dz * o->dz) * cell;
  return off < scale * r * (1.0f - f);
}

/* The rung loop of sif__exodus_run (src/finder/exodus_finder.c:1585-2492)
 * for a box, unweighted, seeds on their nodes: per rung the
 * top-hat smoothing, the scan and sort, the reach, the template, the
 * pre-filter at the rung, then speculative batches -- phase 0 (masked skip),
 * phase 1 (pole probe, exact overlap, collision witness, rescaling; in
 * parallel), phase 2 (the sequential commit with its re-checks at the
 * rescaled radius) -- and the batch and window retuning between them. */
/* The rescaling a run calls for a candidate (exodus_finder.c:2046-2072):
 * weighted on a weighted mesh. */
/* ---------------------------------------------------------------------------
 * Surveys: the footprint the randoms mark out, the field scanned against
 * them, the radius grown against them, and how much of each void was
 * observed (src/finder/exodus_survey.c; exodus_rescale.c:1944-2317).
 * ------------------------------------------------------------------------- */

/* SIF__FINDER_UNOBSERVED, src/finder/utils.h:161-166. */
#define SURVEY_OUTSIDE 1e30f
/* CLOSING_MIN_RANDOMS, CLOSING_MAX_RADIUS, exodus_survey.c:59-60. */
#define CLOSING_MIN_RANDOMS 128.0
#define CLOSING_MAX_RADIUS 4
/* RESCALE_NO_RANDOMS, src/finder/exodus_internal.h:174. */
#define ORC_RESCALE_NO_RANDOMS 6

/* survey_node, exodus_survey.c:41-44: the node nearest a position. */
static inline uint32_t survey_node(float p, float inv_l, uint32_t n) {
  const uint32_t i = (uint32_t)(p * inv_l + 0.5f);
  return i < n ? i : n - 1;
}

/* survey_randoms_per_node, exodus_survey.c:68-80: lambda from m = lambda /
 * (1 - exp(-lambda)) by 64 bisections. */
static double survey_randoms_per_node(double m) {
  if (!(m > 1.0))
    return 0.0;
  double lo = 0.0, hi = m;
  for (int i = 0; i < 64; i++) {
    const double mid = 0.5 * (lo + hi);
    if (mid < m * (1.0 - exp(-mid)))
      lo = mid;
    else
      hi = mid;
  }
  return 0.5 * (lo + hi);
}

/* survey_close_pass, exodus_survey.c:89-120: along `axis`, a node is set when
 * its window of 2k + 1 nodes (those past the faces unset) holds any set node
 * (dilate) or only set nodes (erode). */
static void survey_close_pass(const uint64_t* src, uint64_t* dst, uint32_t n, int axis,
  int32_t k, int erode) {
  const uint64_t n2 = (uint64_t)n * n;
  const uint64_t stride = axis == 0 ? n2 : (axis == 1 ? n : 1);
  const uint64_t step_a = axis == 0 ? n : n2;
  const uint64_t step_b = axis == 2 ? n : 1;
  const int32_t len = (int32_t)n, full = 2 * k + 1;
  memset(dst, 0, ((n2 * n + 63) / 64) * sizeof(uint64_t));
  for (uint64_t line = 0; line < n2; line++) {
    const uint64_t base = (line / n) * step_a + (line % n) * step_b;
    for (int32_t i = 0; i < len; i++) {
      int32_t count = 0;
      for (int32_t j = i - k; j <= i + k; j++)
        if (j >= 0 && j < len)
          count += mask_get(src, base + (uint64_t)j * stride);
      if (erode ? count == full : count > 0)
        mask_set(dst, base + (uint64_t)i * stride);
    }
  }
}

uint64_t orc_survey_occupancy(const orc_mesh_t* rm, uint32_t n, float box, uint64_t* occ,
  int32_t* k_out) {
  /* sif__exodus_survey_occupancy, exodus_survey.c:159-201: every node a
   * random is nearest to, then closed (dilated, then eroded) over a box of
   * 2k + 1 nodes, k the smallest that expects CLOSING_MIN_RANDOMS at the
   * randoms' density over the marked nodes, at most CLOSING_MAX_RADIUS. */
  const uint64_t total = (uint64_t)n * n * n;
  const uint64_t words = (total + 63) / 64;
  memset(occ, 0, words * sizeof(uint64_t));
  const float cell = box / (float)n;
  const float inv_l = 1.0f / cell;
  for (uint64_t p = 0; p < rm->n_particles; p++) {
    const uint64_t ix = survey_node(rm->x[p], inv_l, n), iy = survey_node(rm->y[p], inv_l, n),
                   iz = survey_node(rm->z[p], inv_l, n);
    mask_set(occ, (ix * n + iy) * n + iz);
  }
  uint64_t marked = 0;
  for (uint64_t w = 0; w < words; w++)
    marked += (uint64_t)__builtin_popcountll(occ[w]);
  *k_out = 0;
  if (marked == 0)
    return 0;
  const double lambda = survey_randoms_per_node((double)rm->n_particles / (double)marked);
  int32_t k = 1;
  while (k < CLOSING_MAX_RADIUS &&
         lambda * (2 * k + 1) * (2 * k + 1) * (2 * k + 1) < CLOSING_MIN_RANDOMS)
    k++;
  *k_out = k;
  uint64_t* tmp = malloc(words * sizeof(uint64_t));
  survey_close_pass(occ, tmp, n, 0, k, 0);
  survey_close_pass(tmp, occ, n, 1, k, 0);
  survey_close_pass(occ, tmp, n, 2, k, 0);
  survey_close_pass(tmp, occ, n, 0, k, 1);
  survey_close_pass(occ, tmp, n, 1, k, 1);
  survey_close_pass(tmp, occ, n, 2, k, 1);
  free(tmp);
  uint64_t observed = 0;
  for (uint64_t w = 0; w < words; w++)
    observed += (uint64_t)__builtin_popcountll(occ[w]);
  return observed;
}

/* sif__exodus_survey_contrast, exodus_survey.c:215-227: the smoothed data
 * over alpha times the smoothed randoms, less 1, on observed nodes with an
 * expectation; SURVEY_OUTSIDE elsewhere. */
static void survey_contrast(float* data, const float* randoms, const uint64_t* occ,
  float alpha, uint64_t total) {
  for (uint64_t c = 0; c < total; c++) {
    const float expected = alpha * randoms[c];
    data[c] = (mask_get(occ, c) && expected > 0.0f) ? data[c] / expected - 1.0f : SURVEY_OUTSIDE;
  }
}

static inline double survey_w(const float* w, uint64_t p) { return w ? (double)w[p] : 1.0; }

/* survey_sphere_total, exodus_rescale.c:1957-1993: the weight and the tracers
 * within r_search, whole core and shell cells from the cell table (or their
 * counts), the rest tracer by tracer. */
static void survey_sphere_total(const query_t* q, float rs2, double* w_out, uint64_t* n_out) {
  const orc_mesh_t* m = q->m;
  double w = 0.0;
  uint64_t n = 0;
  for (uint32_t i = 0; i < q->t->count; i++) {
    const uint8_t type = q->t->type[i];
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(q, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (type == CELL_CORE || type == CELL_SHELL) {
      w += m->cell_w ? (double)m->cell_w[query_flat(q, i)] : (double)(e - s);
      n += e - s;
      continue;
    }
    for (uint64_t p = s; p < e; p++)
      if (dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez) <= rs2) {
        w += survey_w(m->w, p);
        n++;
      }
  }
  *w_out = w;
  *n_out = n;
}

/* survey_histogram, exodus_rescale.c:2000-2056: one mesh's weight per bin of
 * the annulus, in its core and in the annulus. */
static void survey_histogram(const query_t* q, double* bins, uint32_t nb, float rc2, float rs2,
  float inv_w, double* core_out, double* shell_out) {
  const orc_mesh_t* m = q->m;
  double core = 0.0, shell = 0.0;
  memset(bins, 0, nb * sizeof(double));
  for (uint32_t i = 0; i < q->t->count; i++) {
    const uint8_t type = q->t->type[i];
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(q, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (type == CELL_CORE) {
      core += m->cell_w ? (double)m->cell_w[query_flat(q, i)] : (double)(e - s);
    } else if (type == CELL_SHELL) {
      for (uint64_t p = s; p < e; p++) {
        const float d2 = dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez);
        const double w = survey_w(m->w, p);
        bins[bin_of(d2, rc2, inv_w, nb)] += w;
        shell += w;
      }
    } else {
      for (uint64_t p = s; p < e; p++) {
        const float d2 = dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez);
        const double w = survey_w(m->w, p);
        if (d2 <= rc2) {
          core += w;
        } else if (d2 <= rs2) {
          bins[bin_of(d2, rc2, inv_w, nb)] += w;
          shell += w;
        }
      }
    }
  }
  *core_out = core;
  *shell_out = shell;
}

/* survey_resolve, exodus_rescale.c:2058-2146: the data tracers in bins
 * [blo, bhi], sorted (the reference's pair quicksort) and walked outside-in
 * against the random weight interpolated at each one's distance. */
static int survey_resolve(const query_t* dq, uint32_t blo, uint32_t bhi, float lo, float hi,
  float rc2, float rs2, float inv_w, float bin_w, uint32_t nb, double d_top, double r_top,
  const double* rbins, float K, float* out, pair_t** buf, uint64_t* cap) {
  const orc_mesh_t* m = dq->m;
  uint64_t count = 0;
  for (uint32_t i = 0; i < dq->t->count; i++) {
    const uint8_t type = dq->t->type[i];
    if (type == CELL_CORE || dq->t->max_d2[i] < lo || dq->t->min_d2[i] > hi)
      continue;
    uint64_t s, e;
    float ex, ey, ez;
    if (!query_cell(dq, i, &s, &e, &ex, &ey, &ez))
      continue;
    if (count + (e - s) > *cap) {
      while (count + (e - s) > *cap)
        *cap *= 2;
      *buf = realloc(*buf, *cap * sizeof(pair_t));
    }
    for (uint64_t p = s; p < e; p++) {
      const float d2 = dist2(m->x[p], m->y[p], m->z[p], ex, ey, ez);
      if (type != CELL_SHELL && !(d2 > rc2 && d2 <= rs2))
        continue;
      const uint32_t bi = bin_of(d2, rc2, inv_w, nb);
      if (bi < blo || bi > bhi)
        continue;
      (*buf)[count++] = (pair_t){d2, (float)survey_w(m->w, p)};
    }
  }
  pair_t* pr = *buf;
  if (count > 1)
    pairs_sort(pr, 0, (int64_t)count - 1);
  uint32_t cur = bhi;
  double r_below = r_top - rbins[bhi];
  double d_cur = d_top;
  for (int64_t k = (int64_t)count - 1; k >= 0; k--) {
    const float d2 = pr[k].d2;
    const double wt = (double)pr[k].w;
    if (d2 == 0.0f) {
      d_cur -= wt;
      continue;
    }
    const uint32_t bi = bin_of(d2, rc2, inv_w, nb);
    while (cur > bi) {
      cur--;
      r_below -= rbins[cur];
    }
    float frac = (d2 - (rc2 + (float)cur * bin_w)) * inv_w;
    frac = frac < 0.0f ? 0.0f : (frac > 1.0f ? 1.0f : frac);
    const float r_in = (float)(r_below + rbins[cur] * (double)frac);
    const float d_in = (float)(d_cur - wt);
    if (r_in > 0.0f && d_in <= K * r_in) {
      *out = sqrtf(d2);
      return 1;
    }
    d_cur -= wt;
  }
  return 0;
}

/* sif__exodus_find_radius_survey, exodus_rescale.c:2154-2317: the largest
 * data distance at which D(<d) <= K R(<d), data and randoms each on its own
 * mesh and template. */
float orc_find_radius_survey(const orc_mesh_t* dm, const orc_template_t* dt,
  const orc_mesh_t* rm, const orc_template_t* rt, float cx, float cy, float cz,
  float r_search, float K, float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum,
  uint64_t* span_count) {
  *reason = ORC_RESCALE_OK;
  const float dinv = 1.0f / dm->cell_length, rinv = 1.0f / rm->cell_length;
  const query_t dq = {dm, dt, cx, cy, cz, (int32_t)(cx * dinv), (int32_t)(cy * dinv),
    (int32_t)(cz * dinv)};
  const query_t rq = {rm, rt, cx, cy, cz, (int32_t)(cx * rinv), (int32_t)(cy * rinv),
    (int32_t)(cz * rinv)};
  const float rs2 = r_search * r_search, rc2 = rmin * rmin, span = rs2 - rc2;
  if (!(span > 0.0f)) {
    *reason = ORC_RESCALE_DEGENERATE;
    return -1.0f;
  }
  double d_within, r_within;
  uint64_t n_d, n_r;
  survey_sphere_total(&dq, rs2, &d_within, &n_d);
  survey_sphere_total(&rq, rs2, &r_within, &n_r);
  if (!(r_within > 0.0)) {
    *reason = ORC_RESCALE_NO_RANDOMS;
    return -1.0f;
  }
  if ((float)d_within <= K * (float)r_within) {
    *reason = ORC_RESCALE_BEYOND_SEARCH;
    return -1.0f;
  }
  uint32_t nb = 2048u;
  {
    const float core_fraction = (rmin * rmin * rmin) / (r_search * r_search * r_search);
    const float want = (float)n_d * (1.0f - core_fraction) / 16.0f;
    if (!(want >= 64.0f))
      nb = 64u;
    else if (want < 2048.0f)
      nb = (uint32_t)want;
  }
  const float inv_w = (float)nb / span, bin_w = span / (float)nb;
  double* dbins = malloc(nb * sizeof(double));
  double* rbins = malloc(nb * sizeof(double));
  double d_core, d_shell, r_core, r_shell;
  survey_histogram(&dq, dbins, nb, rc2, rs2, inv_w, &d_core, &d_shell);
  survey_histogram(&rq, rbins, nb, rc2, rs2, inv_w, &r_core, &r_shell);
  const double d_total = d_core + d_shell, r_total = r_core + r_shell;
  float result = -1.0f;
  uint64_t cap = 4096;
  pair_t* buf = malloc(cap * sizeof(pair_t));
  if (!(r_total > 0.0)) {
    *reason = ORC_RESCALE_NO_RANDOMS;
  } else if ((float)d_total <= K * (float)r_total) {
    *reason = ORC_RESCALE_BEYOND_SEARCH;
  } else {
    *reason = ORC_RESCALE_BELOW_RUNG;
    double d_above = 0.0, r_above = 0.0;
    int32_t b_first = -1;
    for (int32_t b = (int32_t)nb - 1; b >= 0; b--) {
      const double bd = dbins[b], br = rbins[b];
      if (!(bd > 0.0)) {
        r_above += br;
        continue;
      }
      float hi = rc2 + (float)(b + 1) * bin_w;
      if (b == (int32_t)nb - 1)
        hi = rs2 * (1.0f + 1e-6f);
      const float d_in_min = (float)(d_total - d_above - bd);
      const float r_in_max = (float)(r_total - r_above);
      if (!(r_in_max > 0.0f) || d_in_min > K * r_in_max) {
        d_above += bd;
        r_above += br;
        continue;
      }
      if (b_first < 0)
        b_first = b;
      int32_t b_lo = b - (int32_t)(window - 1);
      if (b_lo < 0)
        b_lo = 0;
      double win_d = 0.0, win_r = 0.0;
      for (int32_t bb = b_lo; bb <= b; bb++) {
        win_d += dbins[bb];
        win_r += rbins[bb];
      }
      const float win_lo = rc2 + (float)b_lo * bin_w;
      float radius = -1.0f;
      if (survey_resolve(&dq, (uint32_t)b_lo, (uint32_t)b, win_lo, hi, rc2, rs2, inv_w, bin_w,
            nb, d_total - d_above, r_total - r_above, rbins, K, &radius, &buf, &cap)) {
        const int32_t b_found = (int32_t)bin_of(radius * radius, rc2, inv_w, nb);
        int32_t reached = b_first - b_found + 1;
        if (reached < 1)
          reached = 1;
        *span_sum += (uint64_t)reached;
        (*span_count)++;
        *reason = ORC_RESCALE_OK;
        result = radius;
        break;
      }
      d_above += win_d;
      r_above += win_r;
      b = b_lo;
    }
  }
  free(buf);
  free(dbins);
  free(rbins);
  return result;
}

/* survey_void_footprint, exodus_survey.c:240-296: the observed fraction of a
 * lattice of points through the sphere and through the shell out to twice its
 * radius, spaced a sixteenth of the diameter (half a cell at least). */
static void survey_void_footprint(const uint64_t* occ, uint32_t n, float box, float cx,
  float cy, float cz, float r, float* inside, float* shell) {
  const float l = box / (float)n;
  const float inv_l = 1.0f / l;
  float h = 0.125f * r;
  if (h < 0.5f * l)
    h = 0.5f * l;
  const int32_t half = (int32_t)(2.0f * r / h) + 1;
  const float r2 = r * r, r2_out = 4.0f * r2;
  uint64_t n_in = 0, occ_in = 0, n_sh = 0, occ_sh = 0;
  for (int32_t a = -half; a < half; a++) {
    const float dx = ((float)a + 0.5f) * h;
    for (int32_t b = -half; b < half; b++) {
      const float dy = ((float)b + 0.5f) * h;
      for (int32_t c = -half; c < half; c++) {
        const float dz = ((float)c + 0.5f) * h;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > r2_out)
          continue;
        const float px = cx + dx, py = cy + dy, pz = cz + dz;
        int o = 0;
        if (px >= 0.0f && px < box && py >= 0.0f && py < box && pz >= 0.0f && pz < box) {
          const uint64_t ix = survey_node(px, inv_l, n), iy = survey_node(py, inv_l, n),
                         iz = survey_node(pz, inv_l, n);
          o = mask_get(occ, (ix * n + iy) * n + iz);
        }
        if (d2 <= r2) {
          n_in++;
          occ_in += (uint64_t)o;
        } else {
          n_sh++;
          occ_sh += (uint64_t)o;
        }
      }
    }
  }
  *inside = n_in ? (float)((double)occ_in / (double)n_in) : 0.0f;
  *shell = n_sh ? (float)((double)occ_sh / (double)n_sh) : 0.0f;
}

static float grow_one(const orc_mesh_t* m, const orc_template_t* t, float cx, float cy,
  float cz, float r_search, float threshold, float vol_factor, float mass_factor, float rmin,
  uint32_t window, uint8_t* reason, uint64_t* span_sum, uint64_t* span_count) {
  return find_radius_impl(m, t, cx, cy, cz, r_search, threshold, vol_factor, mass_factor,
    rmin, window, reason, span_sum, span_count, m->w != NULL);
}

int orc_exodus(const float* delta, const orc_mesh_t* mesh, const float* radii_in,
  uint32_t n_radii, const orc_exodus_params_t* p, orc_catalogue_t* out,
  orc_rung_stats_t* stats_out) {
  memset(out, 0, sizeof(*out));
  const uint32_t N = p->grid_n;
  const float box = p->box_length;
  const float cell = box / (float)N;
  const uint64_t total = (uint64_t)N * N * N;
  const float threshold = p->threshold, f = p->overlap_fraction;
  const uint32_t opt = p->options;
  if (!(threshold > -1.0f && threshold < 0.0f) || !(f >= 0.0f && f <= 1.0f) ||
      n_radii == 0 || mesh->box_length != box)
    return -2;
  /* SIF_FINDER_REFINE_GAUSSIAN (utils.c:406-552, exodus_finder.c:1362-1380,
   * 1740-1760): the minima found on the rung's top-hat times a Gaussian of
   * 0.15 of the rung (one more transform), placed between the nodes by a
   * Newton step; the candidates ordered on that field; the threshold still
   * tested on the top-hat. The tracer and hill refinements are not here. */
  const uint32_t refine = opt & (3u << 19);
  if (refine && refine != (1u << 19))
    return -5;
  const int gaussian = refine == (1u << 19);
  /* SIF_FINDER_DISPLACE (exodus_finder.c:696-756, 946-1078, 2239-2275): a
   * void is refused only by a larger one and displaces the smaller ones it
   * collides with. The reference's catalogue does not depend on where its
   * batches fall (a displacement ends one), so it is restated here as the
   * sequential pass that defines it: each candidate in order against the
   * catalogue as it then stands. */
  const int displace = (opt & (1u << 22)) != 0;
  /* SIF_FINDER_EXTEND_REACH (exodus_finder.c:1664-1702, 2060-2072): a
   * crossing past the rung's reach is measured again at the levels of an
   * extended reach, from the first level EXT_SLACK past the rung's own. */
  const int extend_reach = (opt & (1u << 21)) != 0;
  /* SIF_FINDER_SEEDS_MINIMA without refinement: the candidates are the
   * below-threshold, unmasked nodes that are local minima of the rung's field
   * (sif__finder_scan_refined with minima_only, utils.c:406-552); nothing
   * else of the run changes (exodus_finder.c:287-292). */
  const int minima = (opt & (1u << 9)) != 0;
  /* A survey (exodus_survey.c:401-545, exodus_finder.c:1114-1137): cell
   * seeds on their nodes only. */
  const int survey = p->random_mesh != NULL;
  if (survey && (refine || displace || extend_reach || minima || !p->random_grid))
    return -2;

  float* radii = malloc(n_radii * sizeof(float));
  memcpy(radii, radii_in, n_radii * sizeof(float));
  qsort(radii, n_radii, sizeof(float), cmp_desc);

  const float scale = (opt & (1u << 18)) ? (float)cbrt(1.0 + (double)threshold) : 1.0f;
  static const float factors[4] = {1.5f, 1.25f, 1.75f, 2.0f};
  const float search_factor = factors[(opt >> 12) & 3u];
  const int window_mode = (opt & (1u << 14)) ? 0 : ((opt & (1u << 8)) ? 2 : 1);

  /* A weighted mesh (exodus_finder.c:1316-1319, 1076-1106, 1634-1642): its
   * weights finite and non-negative (by their bits; a negative zero passes),
   * their total positive, and the density tests against the mean weight
   * density. No collision witness on it (1868). */
  const int weighted = mesh->w != NULL;
  if (weighted) {
    if (!mesh->cell_w) {
      free(radii);
      return -2;
    }
    for (uint64_t i = 0; i < mesh->n_particles; i++) {
      uint32_t b;
      memcpy(&b, &mesh->w[i], 4);
      if (((b >> 23) & 0xFFu) == 0xFFu || ((b >> 31) && (b << 1))) {
        free(radii);
        return -2;
      }
    }
    if (!(mesh->total_weight > 0.0)) {
      free(radii);
      return -2;
    }
  }
  if (survey) {
    const orc_mesh_t* rm = p->random_mesh;
    for (uint64_t i = 0; rm->w && i < rm->n_particles; i++) {
      uint32_t b;
      memcpy(&b, &rm->w[i], 4);
      if (((b >> 23) & 0xFFu) == 0xFFu || ((b >> 31) && (b << 1))) {
        free(radii);
        return -2;
      }
    }
    if ((rm->w && !rm->cell_w) || !(rm->total_weight > 0.0) || !(mesh->total_weight > 0.0) ||
        rm->box_length != box) {
      free(radii);
      return -2;
    }
  }

  orc_spectrum_t* spec = NULL;
  orc_spectrum_t* rspec = NULL;
  if (!p->inject) {
    spec = orc_spectrum_new(delta, N, box, window_mode, p->smoothing_mode);
    if (survey)
      rspec = orc_spectrum_new(p->random_grid, N, box, window_mode, p->smoothing_mode);
  }
  /* The survey's footprint and normalisation (exodus_finder.c:630-644,
   * 1649-1653): the observed nodes, how much data weight each unit of random
   * weight stands for, and the rescaling's K. */
  uint64_t* occ = NULL;
  float survey_alpha = 0.0f, survey_K = 0.0f;
  if (survey) {
    int32_t k_close;
    occ = calloc((total + 63) / 64, sizeof(uint64_t));
    orc_survey_occupancy(p->random_mesh, N, box, occ, &k_close);
    survey_alpha = (float)(mesh->total_weight / p->random_mesh->total_weight);
    survey_K = (1.0f + threshold) * survey_alpha;
  }
  float* rfield = survey ? malloc(total * sizeof(float)) : NULL;

  const float box_volume = box * box * box;
  const float mean_density = (float)mesh->n_particles / box_volume;
  const float vol_factor = (4.0f / 3.0f) * PI_F * mean_density;
  const float mass_factor =
    weighted ? (4.0f / 3.0f) * PI_F * ((float)mesh->total_weight / box_volume) : vol_factor;

  int n_threads = p->n_threads > 0 ? p->n_threads : 1;

  /* The extended reach's levels (exodus_finder.c:1675-1702, 242-244, 1342-
   * 1353): from the top rung's reach down by EXT_GROWTH to below the bottom
   * rung, level k measuring [ext_rmin[k], ext_reach[k]] with template etpl[k]. */
  enum { EXT_MAX_LEVELS = 32 };
  const float EXT_GROWTH = 1.5f, EXT_SLACK = 1.2f;
  uint32_t n_ext = 0;
  float ext_reach[EXT_MAX_LEVELS], ext_rmin[EXT_MAX_LEVELS];
  orc_template_t etpl[EXT_MAX_LEVELS];
  memset(etpl, 0, sizeof(etpl));
  if (extend_reach) {
    const float r_ext = radii[0] + fmaxf((search_factor - 1.0f) * radii[0], 3.0f * cell);
    const float r_low = radii[n_radii - 1];
    while (n_ext < EXT_MAX_LEVELS &&
           (n_ext == 0 || r_ext / powf(EXT_GROWTH, (float)(n_ext - 1)) > r_low))
      n_ext++;
    for (uint32_t k = 0; k < n_ext; k++)
      ext_reach[k] = r_ext / powf(EXT_GROWTH, (float)(n_ext - 1 - k));
    for (uint32_t k = 0; k < n_ext; k++) {
      ext_rmin[k] = (k ? ext_reach[k - 1] : ext_reach[0] / EXT_GROWTH) / EXT_SLACK;
      if (orc_template_build(&etpl[k], mesh->n_cells, mesh->cell_length, ext_rmin[k],
            ext_reach[k])) {
        for (uint32_t j = 0; j < k; j++)
          orc_template_free(&etpl[j]);
        free(radii);
        return -3;
      }
    }
  }

  uint64_t* mask = calloc((total + 63) / 64, sizeof(uint64_t));
  float* field = malloc(total * sizeof(float));
  /* The field the minima are found and the candidates ordered on: the
   * refinement's own smoothing, or the top-hat itself. */
  float* fmin = gaussian ? malloc(total * sizeof(float)) : field;
  orc_offset_t* offs = NULL;
  uint64_t offs_cap = 0;
  uint64_t inj_k = 0;  /* the next injected field */
  voids_t V;
  voids_init(&V, box);
  float max_acc = 0.0f;
  /* The prior voids, put back as accept_void() puts a void in
   * (exodus_finder.c:1614-1622, 656-683): the catalogue, the mask at
   * scale * r, the largest radius. */
  for (uint64_t v = 0; v < p->n_prior; v++) {
    voids_add(&V, p->prior_cx[v], p->prior_cy[v], p->prior_cz[v], p->prior_r[v]);
    mark_sphere(mask, p->prior_cx[v], p->prior_cy[v], p->prior_cz[v], scale * p->prior_r[v], N,
      cell);
    if (p->prior_r[v] > max_acc)
      max_acc = p->prior_r[v];
  }
  orc_candidate_t* cand = NULL;
  uint64_t cand_cap = 0;
  uint64_t* conflicts = NULL;
  uint64_t conf_cap = 0;
  result_t* res = malloc(2 * BATCH_MAX * sizeof(result_t));
  uint64_t* bidx = malloc(2 * BATCH_MAX * sizeof(uint64_t));
  int status = 0;

  for (uint32_t ri = 0; ri < n_radii && status == 0; ri++) {
    const float radius = radii[ri];
    orc_rung_stats_t st;
    memset(&st, 0, sizeof(st));
    /* Injected fields are taken in the order the run's transforms return
     * them (each backward transform the next field): the rung's top-hat,
     * then, refined, the top-hat times the Gaussian -- which the reference
     * runs only for a rung with cells to refine (utils.c:441-453). */
    if (p->inject)
      memcpy(field, p->inject + inj_k++ * total, total * sizeof(float));
    else
      orc_spectrum_smooth(spec, 1, radius, 0.0f, field, NULL);
    /* A survey's rung (exodus_finder.c:1729-1737): the randoms smoothed the
     * same way, then the field scanned is the data against them. */
    if (survey) {
      if (p->inject)
        memcpy(rfield, p->inject + inj_k++ * total, total * sizeof(float));
      else
        orc_spectrum_smooth(rspec, 1, radius, 0.0f, rfield, NULL);
      survey_contrast(field, rfield, occ, survey_alpha, total);
    }

    /* The scan, src/finder/utils.c:130-213: 256 fixed chunks counted, their
     * offsets, each chunk written in flat order; then the sort. */
    uint64_t nc = 0;
    if (gaussian) {
      /* sif__finder_scan_refined, utils.c:406-552: the cells at or below the
       * threshold on the top-hat and unmasked, in flat order; each one's
       * stencil on the refinement's field; a minimum (its own test, ties to
       * the lower index) gets a Newton step and, if that lands on a node
       * that is itself a candidate, moves there at the step's depth with the
       * rest of the step as its offset (place_candidate, 331-365); every
       * candidate goes by its depth on the refinement's field. A minimum
       * takes the next offset slot whether or not it moves. */
      uint64_t count = 0, n_min = 0;
      for (uint64_t i = 0; i < total; i++)
        count += field[i] <= threshold && !mask_get(mask, i);
      if (count > 0) {
        if (p->inject)
          memcpy(fmin, p->inject + inj_k++ * total, total * sizeof(float));
        else
          orc_spectrum_smooth(spec, 1, radius, 0.15f * radius, fmin, NULL);
        for (uint64_t i = 0; i < total; i++)
          n_min += field[i] <= threshold && !mask_get(mask, i) && is_minimum_node(fmin, N, i);
      }
      if (count > cand_cap) {
        cand_cap = count;
        cand = realloc(cand, cand_cap * sizeof(orc_candidate_t));
      }
      if (n_min > offs_cap) {
        offs_cap = n_min;
        offs = realloc(offs, offs_cap * sizeof(orc_offset_t));
      }
      uint64_t slot = 0;
      for (uint64_t i = 0; i < total; i++) {
        if (!(field[i] <= threshold && !mask_get(mask, i)))
          continue;
        const int minimum = is_minimum_node(fmin, N, i);
        if (minima && !minimum)
          continue;
        orc_candidate_t* c = &cand[nc++];
        c->delta = fmin[i];
        c->refined = 0;
        c->flat = i;
        if (minimum) {
          float s27[27];
          double d[3], depth;
          load_stencil27(fmin, N, i, s27);
          if (newton_step(s27, d, &depth)) {
            const int32_t sx = step_cells(d[0]), sy = step_cells(d[1]), sz = step_cells(d[2]);
            const uint32_t ix = (uint32_t)(i / ((uint64_t)N * N)), iy = (uint32_t)((i / N) % N),
                           iz = (uint32_t)(i % N);
            const uint32_t jx = (uint32_t)(((int64_t)ix + sx + N) % N);
            const uint32_t jy = (uint32_t)(((int64_t)iy + sy + N) % N);
            const uint32_t jz = (uint32_t)(((int64_t)iz + sz + N) % N);
            const uint64_t j = ((uint64_t)jx * N + jy) * N + jz;
            if (field[j] <= threshold && !mask_get(mask, j)) {
              c->delta = (float)depth;
              c->flat = j;
              c->refined = (uint32_t)(slot + 1);
              offs[slot].dx = (float)(d[0] - sx);
              offs[slot].dy = (float)(d[1] - sy);
              offs[slot].dz = (float)(d[2] - sz);
            }
          }
          slot++;
        }
      }
    } else {
      enum { SCAN_CHUNKS = 256 };
      uint64_t chunk_off[SCAN_CHUNKS];
      const uint64_t scan_chunk = total / SCAN_CHUNKS;
#pragma omp parallel for schedule(static, 1) num_threads(n_threads)
      for (int c = 0; c < SCAN_CHUNKS; c++) {
        const uint64_t a = (uint64_t)c * scan_chunk, e = c == SCAN_CHUNKS - 1 ? total : a + scan_chunk;
        uint64_t k = 0;
        for (uint64_t i = a; i < e; i++)
          k += field[i] <= threshold && !mask_get(mask, i) && (!minima || is_minimum_node(field, N, i));
        chunk_off[c] = k;
      }
      for (int c = 0; c < SCAN_CHUNKS; c++) {
        const uint64_t k = chunk_off[c];
        chunk_off[c] = nc;
        nc += k;
      }
      if (nc > cand_cap) {
        cand_cap = nc;
        cand = realloc(cand, cand_cap * sizeof(orc_candidate_t));
      }
#pragma omp parallel for schedule(static, 1) num_threads(n_threads)
      for (int c = 0; c < SCAN_CHUNKS; c++) {
        const uint64_t a = (uint64_t)c * scan_chunk, e = c == SCAN_CHUNKS - 1 ? total : a + scan_chunk;
        uint64_t w = chunk_off[c];
        for (uint64_t i = a; i < e; i++)
          if (field[i] <= threshold && !mask_get(mask, i) &&
              (!minima || is_minimum_node(field, N, i))) {
            cand[w].delta = field[i];
            cand[w].refined = 0;
            cand[w].flat = i;
            w++;
          }
      }
    }
    orc_sort_candidates(cand, nc);
    st.n_candidates = nc;

    const float rmin = 1.0f * radius;
    float r_search = radius + fmaxf((search_factor - 1.0f) * radius, 3.0f * cell);
    if (ri > 0 && radii[ri - 1] > r_search)
      r_search = radii[ri - 1];
    orc_template_t tpl, rtpl;
    memset(&rtpl, 0, sizeof(rtpl));
    if (orc_template_build(&tpl, mesh->n_cells, mesh->cell_length, rmin, r_search)) {
      status = -3;
      break;
    }
    /* The random mesh's own template (exodus_finder.c:1834-1845). */
    if (survey && orc_template_build(&rtpl, p->random_mesh->n_cells,
                    p->random_mesh->cell_length, rmin, r_search)) {
      orc_template_free(&tpl);
      status = -3;
      break;
    }
    const int32_t proxy_pole = (int32_t)(scale * radius * (1.0f - f) / cell) - 1;
    const float rc2 = rmin * rmin;
    /* The first level of the extended reach this rung enters (1826-1832). */
    uint32_t ext0 = n_ext;
    for (uint32_t e = 0; e < n_ext && ext0 == n_ext; e++)
      if (ext_reach[e] >= EXT_SLACK * r_search)
        ext0 = e;
    if (ext0 == n_ext && n_ext > 0 && ext_reach[n_ext - 1] > r_search)
      ext0 = n_ext - 1;

    /* prefilter_cells, src/finder/exodus_finder.c:871-944: 16 chunks a
     * thread, each compacted by one thread, then closed up in order. Not
     * under displacement: a void refusing a candidate now may be gone by its
     * turn (exodus_finder.c:1873-1875). */
    if (nc > 0 && !displace) {
      uint64_t n_chunks = 16u * (uint64_t)n_threads;
      if (n_chunks > nc)
        n_chunks = nc;
      uint64_t* kept = malloc(n_chunks * sizeof(uint64_t));
      uint64_t n_masked = 0, n_proxy = 0, n_overlap = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads) \
  reduction(+ : n_masked, n_proxy, n_overlap)
      for (uint64_t c = 0; c < n_chunks; c++) {
        const uint64_t lo = nc * c / n_chunks, hi = nc * (c + 1) / n_chunks;
        uint64_t w = lo;
        for (uint64_t k = lo; k < hi; k++) {
          const uint64_t flat = cand[k].flat;
          if (cand_masked(mask, &cand[k], offs, radius, f, scale, cell)) {
            n_masked++;
            continue;
          }
          const uint32_t ix = (uint32_t)(flat / ((uint64_t)N * N)),
                         iy = (uint32_t)((flat / N) % N), iz = (uint32_t)(flat % N);
          if (proxy_pole > 0 && overlap_quick(mask, N, ix, iy, iz, (uint32_t)proxy_pole)) {
            n_proxy++;
            continue;
          }
          float cc[3];
          cand_centre(&cand[k], offs, N, cell, box, cc);
          if (overlap_exact(&V, cc[0], cc[1], cc[2], radius, max_acc, box, f, scale)) {
            n_overlap++;
            continue;
          }
          cand[w++] = cand[k];
        }
        kept[c] = w - lo;
      }
      uint64_t w = 0;
      for (uint64_t c = 0; c < n_chunks; c++) {
        const uint64_t lo = nc * c / n_chunks;
        if (lo != w && kept[c] > 0)
          memmove(&cand[w], &cand[lo], kept[c] * sizeof(orc_candidate_t));
        w += kept[c];
      }
      free(kept);
      nc = w;
      st.rejected_masked += n_masked;
      st.rejected_proxy += n_proxy;
      st.rejected_overlap += n_overlap;
    }

    if (displace) {
      /* The witness under displacement: only a void larger than anything the
       * search sphere can return refuses (min_rj), and with an extended reach
       * the sphere must be closed (exodus_finder.c:1868-1871, 2019-2030). */
      const float witness_min_rj = r_search * (1.0f + (float)COLLISION_SLACK);
      uint64_t removed = 0;
      for (uint64_t k = 0; k < nc && status == 0; k++) {
        const uint64_t flat = cand[k].flat;
        if (cand_masked(mask, &cand[k], offs, radius, f, scale, cell)) {
          st.rejected_masked++;
          continue;
        }
        const uint32_t ix = (uint32_t)(flat / ((uint64_t)N * N)),
                       iy = (uint32_t)((flat / N) % N), iz = (uint32_t)(flat % N);
        if (proxy_pole > 0 && overlap_quick(mask, N, ix, iy, iz, (uint32_t)proxy_pole)) {
          st.rejected_proxy++;
          continue;
        }
        float cc[3];
        cand_centre(&cand[k], offs, N, cell, box, cc);
        const float cx = cc[0], cy = cc[1], cz = cc[2];
        if (overlap_exact(&V, cx, cy, cz, radius, max_acc, box, f, scale)) {
          st.rejected_overlap++;
          continue;
        }
        const double rho =
          collision_radius(&V, max_acc, scale, cx, cy, cz, r_search, witness_min_rj, f, box);
        if (!weighted && rho < (double)r_search) {
          float rho2 = (float)(rho * rho * (1.0 + COLLISION_SLACK));
          if (rho2 < rc2)
            rho2 = rc2;
          if (witness(mesh, &tpl, cx, cy, cz, rho2, r_search, threshold, vol_factor,
                extend_reach)) {
            st.rejected_witness++;
            continue;
          }
        }
        uint8_t reason;
        uint64_t ss = 0, sc = 0;
        float rr = grow_one(mesh, &tpl, cx, cy, cz, r_search, threshold, vol_factor, mass_factor, rmin,
          p->window > 0 ? (uint32_t)p->window : RESOLVE_INITIAL, &reason, &ss, &sc);
        for (uint32_t e = ext0; e < n_ext && rr < 0.0f && reason == ORC_RESCALE_BEYOND_SEARCH;
             e++)
          rr = grow_one(mesh, &etpl[e], cx, cy, cz, ext_reach[e], threshold, vol_factor, mass_factor,
            ext_rmin[e], p->window > 0 ? (uint32_t)p->window : RESOLVE_INITIAL, &reason, &ss, &sc);
        st.n_rescaled++;
        if (rr < 0.0f) {
          st.rejected_rescale++;
          continue;
        }
        float largest;
        const uint64_t nconf =
          find_conflicts(&V, max_acc, scale, cx, cy, cz, rr, f, box, &conflicts, &conf_cap,
            &largest);
        if (largest >= rr) {
          st.rejected_exact++;
          continue;
        }
        for (uint64_t j = 0; j < nconf; j++)
          displace_void(&V, mask, conflicts[j], max_acc, scale, N, cell, box);
        removed += nconf;
        voids_add(&V, cx, cy, cz, rr);
        mark_sphere(mask, cx, cy, cz, scale * rr, N, cell);
        if (rr > max_acc)
          max_acc = rr;
        st.accepted++;
      }
      if (removed)
        voids_compact(&V);
      orc_template_free(&tpl);
      if (stats_out)
        stats_out[ri] = st;
      continue;
    }

    uint64_t floor_ = (uint64_t)BATCH_PER_THREAD * (uint64_t)n_threads;
    if (floor_ < BATCH_FLOOR)
      floor_ = BATCH_FLOOR;
    if (floor_ > BATCH_MAX)
      floor_ = BATCH_MAX;
    uint64_t batch_cap = floor_;
    uint32_t window = p->window > 0 ? (uint32_t)p->window : RESOLVE_INITIAL;

    uint64_t k = 0;
    while (k < nc && status == 0) {
      uint64_t nb = 0;
      while (k < nc && nb < batch_cap) {
        if (cand_masked(mask, &cand[k], offs, radius, f, scale, cell))
          st.rejected_masked++;
        else
          bidx[nb++] = k;
        k++;
      }
      if (nb == 0)
        break;
      uint64_t span_sum = 0, span_count = 0;
      const float max_acc_frozen = max_acc;
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads) \
  reduction(+ : span_sum, span_count)
      for (uint64_t b = 0; b < nb; b++) {
        const uint64_t flat = cand[bidx[b]].flat;
        result_t* r = &res[b];
        r->ix = (uint32_t)(flat / ((uint64_t)N * N));
        r->iy = (uint32_t)((flat / N) % N);
        r->iz = (uint32_t)(flat % N);
        if (proxy_pole > 0 &&
            overlap_quick(mask, N, r->ix, r->iy, r->iz, (uint32_t)proxy_pole)) {
          r->status = ST_PROXY;
          continue;
        }
        float cc[3];
        cand_centre(&cand[bidx[b]], offs, N, cell, box, cc);
        r->cx = cc[0];
        r->cy = cc[1];
        r->cz = cc[2];
        if (overlap_exact(&V, r->cx, r->cy, r->cz, radius, max_acc_frozen, box, f,
              scale)) {
          r->status = ST_MESH;
          continue;
        }
        /* No witness on a weighted mesh or a survey (1868). */
        const double rho = (weighted || survey) ? INFINITY
                                                : collision_radius(&V, max_acc_frozen, scale,
                                                    r->cx, r->cy, r->cz, r_search, 0.0f, f, box);
        if (rho < (double)r_search) {
          float rho2 = (float)(rho * rho * (1.0 + COLLISION_SLACK));
          if (rho2 < rc2)
            rho2 = rc2;
          if (witness(mesh, &tpl, r->cx, r->cy, r->cz, rho2, r_search, threshold,
                vol_factor, 0)) {
            r->status = ST_WITNESS;
            continue;
          }
        }
        uint8_t reason;
        uint64_t ss = 0, sc = 0;
        if (survey)
          r->r = orc_find_radius_survey(mesh, &tpl, p->random_mesh, &rtpl, r->cx, r->cy, r->cz,
            r_search, survey_K, rmin, window, &reason, &ss, &sc);
        else
          r->r = grow_one(mesh, &tpl, r->cx, r->cy, r->cz, r_search, threshold,
            vol_factor, mass_factor, rmin, window, &reason, &ss, &sc);
        span_sum += ss;
        span_count += sc;
        for (uint32_t e = ext0; e < n_ext && r->r < 0.0f && reason == ORC_RESCALE_BEYOND_SEARCH;
             e++) {
          ss = sc = 0;
          r->r = grow_one(mesh, &etpl[e], r->cx, r->cy, r->cz, ext_reach[e], threshold,
            vol_factor, mass_factor, ext_rmin[e], window, &reason, &ss, &sc);
          span_sum += ss;
          span_count += sc;
        }
        r->status = r->r < 0.0f ? ST_RESCALE : ST_ACCEPTED;
      }

      const uint64_t acc_before = st.accepted;
      for (uint64_t b = 0; b < nb; b++) {
        const result_t* r = &res[b];
        if (r->status == ST_PROXY) {
          st.rejected_proxy++;
          continue;
        }
        if (r->status == ST_MESH) {
          st.rejected_overlap++;
          continue;
        }
        if (r->status == ST_RESCALE) {
          st.rejected_rescale++;
          st.n_rescaled++;
          continue;
        }
        if (r->status == ST_WITNESS) {
          st.rejected_witness++;
          continue;
        }
        st.n_rescaled++;
        if (cand_masked(mask, &cand[bidx[b]], offs, r->r, f, scale, cell)) {
          st.rejected_masked++;
          continue;
        }
        const int32_t exact_pole = (int32_t)(scale * r->r * (1.0f - f) / cell) - 1;
        if (exact_pole > 0 &&
            overlap_quick(mask, N, r->ix, r->iy, r->iz, (uint32_t)exact_pole)) {
          st.rejected_proxy_recheck++;
          continue;
        }
        if (overlap_exact(&V, r->cx, r->cy, r->cz, r->r, max_acc, box, f, scale)) {
          st.rejected_exact++;
          continue;
        }
        voids_add(&V, r->cx, r->cy, r->cz, r->r);
        mark_sphere(mask, r->cx, r->cy, r->cz, scale * r->r, N, cell);
        if (r->r > max_acc)
          max_acc = r->r;
        st.accepted++;
      }

      const uint64_t n_acc = st.accepted - acc_before;
      if (n_acc == 0) {
        batch_cap += floor_;
        if (batch_cap > BATCH_MAX)
          batch_cap = BATCH_MAX;
      } else {
        batch_cap /= (n_acc + 1);
        if (batch_cap < floor_)
          batch_cap = floor_;
      }
      if (p->window <= 0 && span_count > 0) {
        uint64_t w = (span_sum * 2u + span_count - 1) / span_count;
        if (w < 1)
          w = 1;
        if (w > 64)
          w = 64;
        window = (uint32_t)w;
      }
    }
    orc_template_free(&tpl);
    orc_template_free(&rtpl);
    if (stats_out)
      stats_out[ri] = st;
  }

  /* The grid handed back restored: an unfiltered backward transform of its
   * spectrum, as the reference runs one unless SIF_FINDER_CONSUME_GRID
   * (exodus_finder.c:2430-2453); here the values are discarded, since the
   * oracle never changes the caller's contrast. */
  if (spec && status == 0)
    orc_spectrum_smooth(spec, 0, 0.0f, 0.0f, field, NULL);
  if (rspec && status == 0)
    orc_spectrum_smooth(rspec, 0, 0.0f, 0.0f, field, NULL);
  /* The footprint of every void, once the catalogue is final
   * (sif__exodus_survey_footprint, exodus_survey.c:299-311). */
  if (survey && status == 0) {
    out->footprint = malloc((V.n ? V.n : 1) * sizeof(float));
    out->footprint_shell = malloc((V.n ? V.n : 1) * sizeof(float));
    for (uint64_t v = 0; v < V.n; v++)
      survey_void_footprint(occ, N, box, V.cx[v], V.cy[v], V.cz[v], V.r[v], &out->footprint[v],
        &out->footprint_shell[v]);
  }
  free(occ);
  free(rfield);
  orc_spectrum_free(rspec);
  for (uint32_t k = 0; k < n_ext; k++)
    orc_template_free(&etpl[k]);
  free(bidx);
  free(res);
  free(cand);
  free(offs);
  free(conflicts);
  if (fmin != field)
    free(fmin);
  free(field);
  free(mask);
  free(radii);
  orc_spectrum_free(spec);
  if (status == 0) {
    out->n_voids = V.n;
    out->cx = V.cx;
    out->cy = V.cy;
    out->cz = V.cz;
    out->r = V.r;
    free(V.next);
  } else {
    voids_free(&V);
  }
  return status;
}

void orc_catalogue_free(orc_catalogue_t* c) {
  free(c->cx);
  free(c->cy);
  free(c->cz);
  free(c->r);
  free(c->footprint);
  free(c->footprint_shell);
  memset(c, 0, sizeof(*c));
}
