// The survey finder's own stages (src/finder/exodus_survey.c): the footprint
// the randoms mark on the grid, closed over its chance holes; the field the
// candidates are scanned on, the smoothed data over the smoothed randoms;
// each void's observed fractions; and the bounding box the margin checks read.
//
// The footprint is a bit per grid node, flat (x-major) order, 32 to a word.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "finder.cuh"

namespace sifg {

namespace {

constexpr double kClosingMinRandoms = 128.0;  // CLOSING_MIN_RANDOMS, exodus_survey.c:59
constexpr int32_t kClosingMaxRadius = 4;      // CLOSING_MAX_RADIUS, exodus_survey.c:60

// survey_node, exodus_survey.c:41-44: the node nearest a position.
template <class R>
__device__ __forceinline__ uint32_t survey_node(R p, R inv_l, uint32_t n) {
  const uint32_t i = (uint32_t)fadd(fmul(p, inv_l), R(0.5f));
  return i < n ? i : n - 1;
}

__device__ __forceinline__ bool occ_get(const uint32_t* occ, uint64_t i) {
  return (__ldg(occ + (i >> 5)) >> (i & 31)) & 1u;
}

template <class R>
__global__ void survey_mark_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                   const R* __restrict__ z, uint64_t n_randoms, uint32_t n,
                                   R inv_l, uint32_t* __restrict__ occ) {
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_randoms;
       p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t flat =
        ((uint64_t)survey_node(x[p], inv_l, n) * n + survey_node(y[p], inv_l, n)) * n +
        survey_node(z[p], inv_l, n);
    atomicOr(occ + (flat >> 5), 1u << (flat & 31));
  }
}

__global__ void popcount_kernel(const uint32_t* __restrict__ w, uint64_t words,
                                unsigned long long* __restrict__ out) {
  unsigned long long c = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words;
       i += (uint64_t)gridDim.x * blockDim.x)
    c += (unsigned)__popc(w[i]);
  for (int d = 16; d > 0; d >>= 1) c += __shfl_down_sync(0xffffffffu, c, d);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// One pass of the closing (survey_close_pass, exodus_survey.c:89-120): along
// `axis`, node i is set when the window [i - k, i + k] (nodes past the faces
// unset) holds any set node (dilate) or only set nodes (erode). A thread per
// node, a warp per output word.
__global__ void close_pass_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                  uint32_t n, int axis, int32_t k, int erode, uint64_t words) {
  const uint64_t total = (uint64_t)n * n * n;
  const uint64_t stride = axis == 0 ? (uint64_t)n * n : (axis == 1 ? n : 1);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words * 32;
       i += (uint64_t)gridDim.x * blockDim.x) {
    bool set = false;
    if (i < total) {
      const int32_t c = (int32_t)(axis == 0 ? i / ((uint64_t)n * n) : (axis == 1 ? (i / n) % n : i % n));
      int32_t count = 0;
      for (int32_t j = -k; j <= k; j++) {
        const int32_t cj = c + j;
        if (cj >= 0 && cj < (int32_t)n) count += occ_get(src, i + (int64_t)j * (int64_t)stride);
      }
      set = erode ? count == 2 * k + 1 : count > 0;
    }
    const unsigned word = __ballot_sync(0xffffffffu, set);
    if ((threadIdx.x & 31) == 0) dst[i >> 5] = word;
  }
}

template <class R>
__global__ void survey_contrast_kernel(R* __restrict__ data, const R* __restrict__ randoms,
                                       const uint32_t* __restrict__ occ, R alpha, uint64_t cells) {
  // SIF__FINDER_UNOBSERVED, src/finder/utils.h:161-166.
  const R outside = R(1e30);
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
       c += (uint64_t)gridDim.x * blockDim.x) {
    const R expected = fmul(alpha, randoms[c]);
    data[c] = (occ_get(occ, c) && expected > R(0.0f)) ? fsub(fdiv(data[c], expected), R(1.0f))
                                                      : outside;
  }
}

// survey_void_footprint, exodus_survey.c:240-296: a CTA per void over a
// lattice of points through the cube of side 4r around it, spaced an eighth
// of the radius (half a grid cell at least); a point outside the box is
// outside the footprint.
template <class R>
__global__ void __launch_bounds__(256) survey_footprint_kernel(
    const R* __restrict__ cx, const R* __restrict__ cy, const R* __restrict__ cz,
    const R* __restrict__ rr, uint32_t n_voids, const uint32_t* __restrict__ occ, uint32_t n,
    R box, R* __restrict__ inside, R* __restrict__ shell) {
  __shared__ unsigned long long red[4][8];
  const R l = fdiv(box, (R)n);
  const R inv_l = fdiv(R(1.0f), l);
  for (uint32_t v = blockIdx.x; v < n_voids; v += gridDim.x) {
    const R r = rr[v], x0 = cx[v], y0 = cy[v], z0 = cz[v];
    R h = fmul(R(0.125f), r);
    if (h < fmul(R(0.5f), l)) h = fmul(R(0.5f), l);
    const int32_t half = (int32_t)fdiv(fmul(R(2.0f), r), h) + 1;
    const R r2 = fmul(r, r), r2_out = fmul(R(4.0f), r2);
    const uint32_t side = 2u * (uint32_t)half;
    const uint64_t points = (uint64_t)side * side * side;
    unsigned long long n_in = 0, o_in = 0, n_sh = 0, o_sh = 0;
    for (uint64_t q = threadIdx.x; q < points; q += blockDim.x) {
      const int32_t a = (int32_t)(q / ((uint64_t)side * side)) - half;
      const int32_t b = (int32_t)((q / side) % side) - half;
      const int32_t c = (int32_t)(q % side) - half;
      const R dx = fmul(fadd((R)a, R(0.5f)), h);
      const R dy = fmul(fadd((R)b, R(0.5f)), h);
      const R dz = fmul(fadd((R)c, R(0.5f)), h);
      const R d2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
      if (d2 > r2_out) continue;
      const R px = fadd(x0, dx), py = fadd(y0, dy), pz = fadd(z0, dz);
      bool o = false;
      if (px >= R(0.0f) && px < box && py >= R(0.0f) && py < box && pz >= R(0.0f) && pz < box)
        o = occ_get(occ, ((uint64_t)survey_node(px, inv_l, n) * n + survey_node(py, inv_l, n)) * n +
                             survey_node(pz, inv_l, n));
      if (d2 <= r2) {
        n_in++;
        o_in += o;
      } else {
        n_sh++;
        o_sh += o;
      }
    }
    unsigned long long t[4] = {n_in, o_in, n_sh, o_sh};
    for (int j = 0; j < 4; j++)
      for (int d = 16; d > 0; d >>= 1) t[j] += __shfl_down_sync(0xffffffffu, t[j], d);
    if ((threadIdx.x & 31) == 0)
      for (int j = 0; j < 4; j++) red[j][threadIdx.x >> 5] = t[j];
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long s[4] = {0, 0, 0, 0};
      for (int j = 0; j < 4; j++)
        for (int w = 0; w < 8; w++) s[j] += red[j][w];
      inside[v] = s[0] ? (R)__ddiv_rn((double)s[1], (double)s[0]) : R(0.0f);
      shell[v] = s[2] ? (R)__ddiv_rn((double)s[3], (double)s[2]) : R(0.0f);
    }
    __syncthreads();
  }
}

// Per block: the least and largest of each coordinate (lo[3], hi[3] per
// block in out).
template <class R>
__global__ void __launch_bounds__(256) extent_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                                     const R* __restrict__ z, uint64_t n,
                                                     R* __restrict__ out) {
  __shared__ R red[6][8];
  R v[6] = {real_inf<R>(), real_inf<R>(), real_inf<R>(), -real_inf<R>(), -real_inf<R>(),
            -real_inf<R>()};
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (uint64_t)gridDim.x * blockDim.x) {
    const R c[3] = {x[p], y[p], z[p]};
    for (int a = 0; a < 3; a++) {
      v[a] = c[a] < v[a] ? c[a] : v[a];
      v[3 + a] = c[a] > v[3 + a] ? c[a] : v[3 + a];
    }
  }
  for (int a = 0; a < 6; a++)
    for (int d = 16; d > 0; d >>= 1) {
      const R o = __shfl_down_sync(0xffffffffu, v[a], d);
      v[a] = a < 3 ? (o < v[a] ? o : v[a]) : (o > v[a] ? o : v[a]);
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 6; a++) red[a][threadIdx.x >> 5] = v[a];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int a = 0; a < 6; a++) {
      R t = red[a][0];
      for (int w = 1; w < 8; w++) t = a < 3 ? (red[a][w] < t ? red[a][w] : t) : (red[a][w] > t ? red[a][w] : t);
      out[6 * blockIdx.x + a] = t;
    }
}

}  // namespace

template <class R>
uint64_t survey_mark(const R* x, const R* y, const R* z, uint64_t n_randoms, uint32_t n, R box,
                     uint32_t* occ, unsigned long long* d_count, cudaStream_t st) {
  const uint64_t cells = (uint64_t)n * n * n;
  const uint64_t words = (cells + 31) / 32;
  SIFG_CUDA(cudaMemsetAsync(occ, 0, words * sizeof(uint32_t), st));
  // inv_l as the reference takes it: 1 over the grid's cell length.
  const R inv_l = (R)1.0f / (box / (R)n);
  if (n_randoms)
    survey_mark_kernel<R><<<grid_for(n_randoms, 256), 256, 0, st>>>(x, y, z, n_randoms, n, inv_l, occ);
  SIFG_LAUNCH_CHECK();
  SIFG_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
  popcount_kernel<<<grid_for(words, 256), 256, 0, st>>>(occ, words, d_count);
  SIFG_LAUNCH_CHECK();
  unsigned long long h = 0;
  SIFG_CUDA(cudaMemcpyAsync(&h, d_count, sizeof(h), cudaMemcpyDeviceToHost, st));
  SIFG_CUDA(cudaStreamSynchronize(st));
  return h;
}

// survey_randoms_per_node, exodus_survey.c:68-80: lambda from the randoms
// per marked node m = lambda / (1 - exp(-lambda)), by 64 bisections.
static double randoms_per_node(double m) {
  if (!(m > 1.0)) return 0.0;
  double lo = 0.0, hi = m;
  for (int i = 0; i < 64; i++) {
    const double mid = 0.5 * (lo + hi);
    if (mid < m * (1.0 - std::exp(-mid)))
      lo = mid;
    else
      hi = mid;
  }
  return 0.5 * (lo + hi);
}

int32_t survey_closing_k(uint64_t n_randoms, uint64_t marked) {
  const double lambda = randoms_per_node((double)n_randoms / (double)marked);
  int32_t k = 1;
  while (k < kClosingMaxRadius && lambda * (2 * k + 1) * (2 * k + 1) * (2 * k + 1) < kClosingMinRandoms)
    k++;
  return k;
}

void survey_close(uint32_t* occ, uint32_t* tmp, uint32_t n, int32_t k, cudaStream_t st) {
  const uint64_t cells = (uint64_t)n * n * n;
  const uint64_t words = (cells + 31) / 32;
  const unsigned grid = grid_for(words * 32, 256);
  // Dilate along x, y, z, then erode, the masks taking turns (survey_close,
  // exodus_survey.c:130-144).
  uint32_t* a = occ;
  uint32_t* b = tmp;
  for (int pass = 0; pass < 6; pass++) {
    close_pass_kernel<<<grid, 256, 0, st>>>(a, b, n, pass % 3, k, pass >= 3, words);
    SIFG_LAUNCH_CHECK();
    std::swap(a, b);
  }
}

template <class R>
void survey_contrast(R* data, const R* randoms, const uint32_t* occ, R alpha, uint64_t cells,
                     cudaStream_t st) {
  survey_contrast_kernel<R><<<grid_for(cells, 256), 256, 0, st>>>(data, randoms, occ, alpha, cells);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void survey_footprint(const R* cx, const R* cy, const R* cz, const R* r, uint32_t n_voids,
                      const uint32_t* occ, uint32_t n, R box, R* inside, R* shell,
                      cudaStream_t st) {
  if (n_voids == 0) return;
  const unsigned g = n_voids < 152u * 8u ? n_voids : 152u * 8u;
  survey_footprint_kernel<R><<<g, 256, 0, st>>>(cx, cy, cz, r, n_voids, occ, n, box, inside, shell);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void extent(const R* x, const R* y, const R* z, uint64_t n, R lo[3], R hi[3], cudaStream_t st) {
  const unsigned g = grid_for(n ? n : 1, 256, 152u * 4u);
  thread_local DevBuf buf;
  R* d = (R*)buf.ensure((size_t)g * 6 * sizeof(R));
  extent_kernel<R><<<g, 256, 0, st>>>(x, y, z, n, d);
  SIFG_LAUNCH_CHECK();
  std::vector<R> h((size_t)g * 6);
  SIFG_CUDA(cudaMemcpyAsync(h.data(), d, h.size() * sizeof(R), cudaMemcpyDeviceToHost, st));
  SIFG_CUDA(cudaStreamSynchronize(st));
  for (int a = 0; a < 3; a++) {
    lo[a] = h[a];
    hi[a] = h[3 + a];
    for (unsigned b = 1; b < g; b++) {
      lo[a] = std::min(lo[a], h[6 * b + a]);
      hi[a] = std::max(hi[a], h[6 * b + 3 + a]);
    }
  }
}

#define SIFG_SURVEY_INST(R)                                                                        \
  template uint64_t survey_mark<R>(const R*, const R*, const R*, uint64_t, uint32_t, R, uint32_t*, \
                                   unsigned long long*, cudaStream_t);                            \
  template void survey_contrast<R>(R*, const R*, const uint32_t*, R, uint64_t, cudaStream_t);      \
  template void survey_footprint<R>(const R*, const R*, const R*, const R*, uint32_t,              \
                                    const uint32_t*, uint32_t, R, R*, R*, cudaStream_t);           \
  template void extent<R>(const R*, const R*, const R*, uint64_t, R*, R*, cudaStream_t);
SIFG_SURVEY_INST(float)
SIFG_SURVEY_INST(double)

}  // namespace sifg
