// CIC deposit of particles onto the density grid, and the density contrast.
//
// Replaces grid_compute_cic / grid_cic_deposit_tile (src/structures/grid.c:
// 455-746) and sif_grid_to_density_contrast (grid.c:1177-1244).
//
// The reference sums float weights in a fixed slab/chunk order so its grid is
// deterministic. Here every corner weight is quantised to 2^-24 of a particle
// and summed as int64, so the sum is exact and independent of the order the
// GPU happens to add in. The eight quantised weights of a particle sum to
// exactly 2^24: each corner is rounded, and what rounding left over goes to
// the particle's largest corner.
//
// Layout of the work:
//   1. tile_count:   each particle's tile (16^3 base cells), histogram with
//                    warp-aggregated atomics;
//   2. exclusive scan of the tile counts;
//   3. tile_scatter: each particle's base cell and fractions, found once, as
//                    a 16-byte record in tile order (one atomic per group of
//                    lanes bound for the same tile);
//   4. tile_deposit: one CTA per tile accumulates a 17^3 tile of 64-bit sums
//                    (32-bit words plus carries) in shared memory with one
//                    shared atomic per corner; the 15^3 cells no other tile touches
//                    are written straight to the grid as float density, the
//                    faces shared with neighbouring tiles go to int64 face
//                    buffers with global atomics;
//   5. face_fixup:   the face buffers converted to float density.
//
// Weighted (sif_field_t::weights), a particle's corners carry its weight as
// the reference's products do (grid.c:635-639: the weight times each z
// factor, then the (x, y) products times those), quantised to 2^-24 of the
// binade of the largest weight magnitude: the same integers as unweighted
// when every weight is that power of two, so weights of 1 or 4 give the
// unweighted density times the weight, bit for bit. Negative weights sum as
// two's complement; a non-finite weight deposits nothing in the sums and
// its products are added to its eight cells afterwards, so those cells go
// non-finite as the reference's do.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.cuh"

namespace sifg {

constexpr int TB = kCicTile;  // base cells per tile side
constexpr int TS = TB + 1;    // tile extent including the upper neighbours

struct CicGeom {
  uint32_t n;       // grid cells per side
  uint32_t nt;      // tiles per side
  float box;
  float idx_hi;     // n / box in double, as a pair of floats
  float idx_lo;
};

// A coordinate in cell units, u = fold(v) * n / box, and its base cell and
// fraction (grid.c:585-620: cell = floor(u), wrapped into [0, n); t = u -
// floor(u)). The reference rounds u to a float, which moves t by up to an
// ulp of u -- 1e-5 of a cell at u ~ 128; here the product is kept exact as
// hi + lo (lo from the fused multiply-add's residual), so t is good to an ulp
// of 1 and the deposit's error is the 2^-24 quantum.
__device__ __forceinline__ void cic_axis(float v, const CicGeom& g, uint32_t& cell, float& t) {
  const float x = box_fold(v, g.box);
  const float hi = fmul(x, g.idx_hi);
  const float lo = fadd(__fmaf_rn(x, g.idx_hi, -hi), fmul(x, g.idx_lo));
  float r = floorf(hi);
  float f = fadd(fsub(hi, r), lo);
  if (f < 0.0f) {
    r -= 1.0f;
    f = fadd(f, 1.0f);
  } else if (f >= 1.0f) {
    r += 1.0f;
    f = fsub(f, 1.0f);
  }
  int32_t c = (int32_t)r;
  if (c < 0) c += (int32_t)g.n;
  if (c >= (int32_t)g.n) c -= (int32_t)g.n;
  // In range for every position in the box; the clamp only keeps a position
  // far outside it (which the box check reports) from indexing past the grid.
  cell = min((uint32_t)c, g.n - 1);
  t = f;
}

__device__ __forceinline__ uint32_t tile_of(float x, float y, float z, const CicGeom& g) {
  uint32_t cx, cy, cz;
  float t;
  cic_axis(x, g, cx, t);
  cic_axis(y, g, cy, t);
  cic_axis(z, g, cz, t);
  return ((cx / TB) * g.nt + cy / TB) * g.nt + cz / TB;
}

// With `outside` set, also counts the particles outside [lo, hi] on any axis
// (NaN included): the box check, from the same reads.
__global__ void tile_count_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                  const float* __restrict__ z, uint64_t n, CicGeom g,
                                  uint32_t* __restrict__ counts, float lo, float hi,
                                  unsigned long long* __restrict__ outside) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long bad = 0;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    uint32_t tile = 0xffffffffu;
    if (valid) {
      const float px = x[p], py = y[p], pz = z[p];
      tile = tile_of(px, py, pz, g);
      bad += (px >= lo && px <= hi && py >= lo && py <= hi && pz >= lo && pz <= hi) ? 0u : 1u;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, tile);
    if (valid && (threadIdx.x & 31u) == (unsigned)(__ffs(peers) - 1))
      atomicAdd(counts + tile, (uint32_t)__popc(peers));
  }
  if (outside) {
    for (int d = 16; d > 0; d >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, d);
    if ((threadIdx.x & 31u) == 0 && bad) atomicAdd(outside, bad);
  }
}

// A particle's deposit record: its fractions along x, y, z and, in the
// fourth word's bits, its base cell within its tile (x << 8 | y << 4 | z).
static_assert(TB == 16, "4 bits per axis of the cell within its tile");

__global__ void tile_scatter_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                    const float* __restrict__ z, uint64_t n, CicGeom g,
                                    uint32_t* __restrict__ cursor, float4* __restrict__ rec,
                                    const float* __restrict__ w, float* __restrict__ wrec) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31u;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t tile = 0xffffffffu;
    if (valid) {
      uint32_t cx, cy, cz;
      cic_axis(x[p], g, cx, r.x);
      cic_axis(y[p], g, cy, r.y);
      cic_axis(z[p], g, cz, r.z);
      tile = ((cx / TB) * g.nt + cy / TB) * g.nt + cz / TB;
      r.w = __uint_as_float((cx % TB) << 8 | (cy % TB) << 4 | (cz % TB));
    }
    const unsigned peers = __match_any_sync(0xffffffffu, tile);
    const unsigned leader = __ffs(peers) - 1;
    uint32_t slot0 = 0;
    if (valid && lane == leader) slot0 = atomicAdd(cursor + tile, (uint32_t)__popc(peers));
    slot0 = __shfl_sync(0xffffffffu, slot0, leader);
    if (valid) {
      const uint32_t slot = slot0 + __popc(peers & ((1u << lane) - 1u));
      rec[slot] = r;
      if (w) wrec[slot] = w[p];
    }
  }
}

// The largest finite weight magnitude, as its bits (which order as the
// magnitudes do), and the count of non-finite weights.
__global__ void weight_max_kernel(const float* __restrict__ w, uint64_t n,
                                  unsigned* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned m = 0, bad = 0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    const unsigned b = __float_as_uint(w[p]) & 0x7fffffffu;
    if (b >= 0x7f800000u)
      bad++;
    else
      m = max(m, b);
  }
  m = __reduce_max_sync(0xffffffffu, m);
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31u) == 0) {
    if (m) atomicMax(out, m);
    if (bad) atomicAdd(out + 1, bad);
  }
}

// The weighted quantum from the largest weight's binade [2^E, 2^(E+1)):
// corners quantised at 2^(E-24) (scale 2^(24-E)), clamped to keep both the
// scale and its inverse normal floats.
__device__ __forceinline__ int weight_scale_exp(const unsigned* wmax) {
  const int e = (int)(*wmax >> 23) - 127;
  return min(100, max(-100, 24 - e));
}

// Each non-finite weight's eight products, added to its cells after the
// deposit (the reference's float sums carry them into those cells).
__global__ void nonfinite_weights_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                         const float* __restrict__ z,
                                         const float* __restrict__ w, uint64_t n, CicGeom g,
                                         const unsigned* __restrict__ wmax,
                                         float* __restrict__ grid) {
  if (wmax[1] == 0) return;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    const float pw = w[p];
    if ((__float_as_uint(pw) & 0x7fffffffu) < 0x7f800000u) continue;
    uint32_t c[3];
    float t[3];
    cic_axis(x[p], g, c[0], t[0]);
    cic_axis(y[p], g, c[1], t[1]);
    cic_axis(z[p], g, c[2], t[2]);
    for (int k = 0; k < 8; k++) {
      uint32_t q[3];
      float f = 1.0f;
      for (int a = 0; a < 3; a++) {
        const int up = (k >> (2 - a)) & 1;
        q[a] = up ? (c[a] + 1 == g.n ? 0u : c[a] + 1) : c[a];
        f = fmul(f, up ? t[a] : fsub(1.0f, t[a]));
      }
      float* cell = grid + ((uint64_t)q[0] * g.n + q[1]) * g.n + q[2];
      *cell = fadd(*cell, fmul(pw, f));
    }
  }
}

// Face buffers: cells on a tile boundary in x (x % TB == 0), else in y, else
// in z, each laid out densely over its own boundary planes.
struct FaceBufs {
  unsigned long long* fx;  // [nt][n][n]
  unsigned long long* fy;  // [n][nt][n]
  unsigned long long* fz;  // [n][n][nt]
};

__device__ __forceinline__ unsigned long long* face_slot(const FaceBufs& f, uint32_t gx,
                                                        uint32_t gy, uint32_t gz,
                                                        const CicGeom& g) {
  const uint64_t n = g.n, nt = g.nt;
  if (gx % TB == 0) return f.fx + ((uint64_t)(gx / TB) * n + gy) * n + gz;
  if (gy % TB == 0) return f.fy + ((uint64_t)gx * nt + gy / TB) * n + gz;
  return f.fz + ((uint64_t)gx * n + gy) * nt + gz / TB;
}

__global__ void __launch_bounds__(256) tile_deposit_kernel(
    const float4* __restrict__ rec, const uint32_t* __restrict__ offsets, CicGeom g,
    float inv_cell_vol, float* __restrict__ grid, FaceBufs faces,
    const float* __restrict__ wrec, const unsigned* __restrict__ wmax) {
  // The tile's sums as two 32-bit words a cell: a 32-bit shared atomic add is
  // one instruction, a 64-bit one a compare-and-swap loop (measured: the
  // 512^3 deposit with one 64-bit add per corner took 3.4 ms, against 1.7). A tile with fewer
  // than 2^16 particles adds each quantum's low 16 bits to the first word and
  // its high bits (arithmetic shift) to the second, neither of which can wrap
  // (a cell takes one add per particle), with adds that return nothing; a
  // denser tile adds the whole quantum to the first word and counts its wraps
  // in the second (each add is below 2^32, so it wraps at most once), which
  // needs the old value back. Either pair is the exact 64-bit sum whatever the
  // order of the adds.
  extern __shared__ uint32_t acc_lo[];  // TS^3 words, then TS^3 carries
  uint32_t* acc_hi = acc_lo + TS * TS * TS;
  const uint32_t nt = g.nt;
  const uint32_t n_tiles = nt * nt * nt;
  // The quantum: 2^-24 of a particle, or of the largest weight's binade.
  float qscale = 16777216.0f, qinv = 1.0f / 16777216.0f;
  if (wrec) {
    const int e = weight_scale_exp(wmax);
    qscale = __uint_as_float((uint32_t)(127 + e) << 23);
    qinv = __uint_as_float((uint32_t)(127 - e) << 23);
  }
  // Cleared once; each flush leaves the cells it reads cleared for the next tile.
  for (int i = threadIdx.x; i < 2 * TS * TS * TS; i += blockDim.x) acc_lo[i] = 0u;
  __syncthreads();
  for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const uint32_t tx = tile / (nt * nt), ty = (tile / nt) % nt, tz = tile % nt;
    const uint32_t ox = tx * TB, oy = ty * TB, oz = tz * TB;

    const uint32_t s = offsets[tile], e = offsets[tile + 1];
    const bool split = e - s < (1u << 16);
    for (uint32_t base = s; base < e; base += blockDim.x) {
      const uint32_t p = base + threadIdx.x;
      const bool valid = p < e;
      uint32_t cell = 0xffffffffu;
      uint32_t q[8];
      if (valid) {
        const float4 r = __ldg(rec + p);
        const float tx_ = r.x, ty_ = r.y, tz_ = r.z;
        const uint32_t local = __float_as_uint(r.w);
        float wz0 = fsub(1.0f, tz_), wz1 = tz_;
        float pw = 1.0f;
        if (wrec) {
          // A non-finite weight is added afterwards, outside the sums.
          pw = __ldg(wrec + p);
          if ((__float_as_uint(pw) & 0x7fffffffu) >= 0x7f800000u) pw = 0.0f;
          wz0 = fmul(pw, wz0);
          wz1 = fmul(pw, wz1);
        }
        const float wx0 = fsub(1.0f, tx_), wy0 = fsub(1.0f, ty_);
        // The reference's eight products (grid.c:627-650): (x,y) pairs times
        // z (times the weight).
        const float w00 = fmul(wx0, wy0), w01 = fmul(wx0, ty_);
        const float w10 = fmul(tx_, wy0), w11 = fmul(tx_, ty_);
        const float w[8] = {fmul(w00, wz0), fmul(w00, wz1), fmul(w01, wz0), fmul(w01, wz1),
                            fmul(w10, wz0), fmul(w10, wz1), fmul(w11, wz0), fmul(w11, wz1)};
        // w times a power of two is exact in float, so rounding it to an
        // integer in float is the quantisation itself; GB300's FP64 rate is
        // no place for it.
        int sum = 0;
        int big = 0;
        float wbig = fabsf(w[0]);
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int qk = __float2int_rn(fmul(w[k], qscale));
          q[k] = (uint32_t)qk;
          sum += qk;
          if (fabsf(w[k]) > wbig) {  // the first largest, as a scan from corner 0 finds it
            wbig = fabsf(w[k]);
            big = k;
          }
        }
        // The eight sum to the particle's own quantised weight.
        const int fix = (wrec ? __float2int_rn(fmul(pw, qscale)) : 16777216) - sum;
#pragma unroll
        for (int k = 0; k < 8; k++) q[k] = (uint32_t)((int)q[k] + (k == big ? fix : 0));
        cell = ((local >> 8) * TS + ((local >> 4) & 15u)) * TS + (local & 15u);
      }
      // One shared atomic per corner. (Reducing lanes bound for the same cell
      // first with __reduce_add_sync over each lane group's own mask costs a
      // serialised pass per distinct group: eight per corner per cell in the
      // warp, far more than the atomics it saves.)
      if (valid && split) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const uint32_t c =
              cell + (uint32_t)(((k >> 2) & 1) * TS * TS + ((k >> 1) & 1) * TS + (k & 1));
          atomicAdd(acc_lo + c, q[k] & 0xffffu);
          const int hi16 = (int)q[k] >> 16;
          if (hi16) atomicAdd(acc_hi + c, (uint32_t)hi16);
        }
      } else if (valid) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const uint32_t v = q[k];
          const uint32_t c =
              cell + (uint32_t)(((k >> 2) & 1) * TS * TS + ((k >> 1) & 1) * TS + (k & 1));
          const uint32_t old = atomicAdd(acc_lo + c, v);
          // The carry, and for a negative value its sign extension.
          const uint32_t hi = (old + v < old ? 1u : 0u) + ((int)v < 0 ? 0xffffffffu : 0u);
          if (hi) atomicAdd(acc_hi + c, hi);
        }
      }
    }
    __syncthreads();

    // Flush. Cells 1..TB-1 of this tile (within the grid) are touched by no
    // other tile; the rest are shared with a neighbour.
    const uint32_t ex = min((uint32_t)TB, g.n - ox), ey = min((uint32_t)TB, g.n - oy),
                   ez = min((uint32_t)TB, g.n - oz);
    for (int i = threadIdx.x; i < TS * TS * TS; i += blockDim.x) {
      const uint32_t a = i / (TS * TS), b = (i / TS) % TS, c = i % TS;
      if (a > ex || b > ey || c > ez) continue;
      const unsigned long long v =
          split ? (unsigned long long)((long long)(int)acc_hi[i] * 65536ll + (long long)acc_lo[i])
                : ((unsigned long long)acc_hi[i] << 32) | acc_lo[i];
      acc_lo[i] = 0u;
      acc_hi[i] = 0u;
      const uint32_t gx = ox + a == g.n ? 0u : ox + a;
      const uint32_t gy = oy + b == g.n ? 0u : oy + b;
      const uint32_t gz = oz + c == g.n ? 0u : oz + c;
      const bool interior = a >= 1 && a < ex && b >= 1 && b < ey && c >= 1 && c < ez;
      if (interior) {
        grid[((uint64_t)gx * g.n + gy) * g.n + gz] =
            fmul(fmul(__ll2float_rn((long long)v), qinv), inv_cell_vol);
      } else if (v != 0ull) {
        atomicAdd(face_slot(faces, gx, gy, gz, g), v);
      }
    }
    __syncthreads();
  }
}

__global__ void face_fixup_kernel(CicGeom g, float inv_cell_vol, float* __restrict__ grid,
                                  FaceBufs faces, const unsigned* __restrict__ wmax) {
  float qinv = 1.0f / 16777216.0f;
  if (wmax) qinv = __uint_as_float((uint32_t)(127 - weight_scale_exp(wmax)) << 23);
  const uint64_t n = g.n, nt = g.nt;
  const uint64_t nfx = nt * n * n;
  const uint64_t total = 3 * nfx;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const uint64_t which = i / nfx, j = i % nfx;
    uint64_t gx, gy, gz;
    unsigned long long v;
    if (which == 0) {
      gx = (j / (n * n)) * TB;
      gy = (j / n) % n;
      gz = j % n;
      if (gx >= n) continue;
      v = faces.fx[j];
    } else if (which == 1) {
      gx = j / (nt * n);
      gy = ((j / n) % nt) * TB;
      gz = j % n;
      if (gy >= n || gx % TB == 0) continue;
      v = faces.fy[j];
    } else {
      gx = j / (n * nt);
      gy = (j / nt) % n;
      gz = (j % nt) * TB;
      if (gz >= n || gx % TB == 0 || gy % TB == 0) continue;
      v = faces.fz[j];
    }
    grid[(gx * n + gy) * n + gz] = fmul(fmul(__ll2float_rn((long long)v), qinv), inv_cell_vol);
  }
}

// ---------------------------------------------------------------------------
// The FP64 form's deposit (the reference's SIF_USE_DOUBLE build): the cell
// coordinate u = fold(x) * (N / L), its base cell and fraction, and the eight
// weights in double as grid.c:585-650 computes them. Each weight is rounded to
// a multiple of 2^-40 of a particle (the remainder to the largest, so the
// eight sum to exactly one particle) and summed as int64 with global atomics:
// the grid is exact to 2^-40 per particle and independent of the order the
// additions land in. One thread per particle, no tiling: this is the plain
// form the float path is measured against.
// ---------------------------------------------------------------------------
constexpr double kQ64 = 1099511627776.0;  // 2^40

__device__ __forceinline__ void cic_axis_f64(double v, uint32_t n, double box, double idx,
                                             uint32_t& c0, uint32_t& c1, double& t) {
  const double u = fmul(box_fold(v, box), idx);
  const uint32_t raw = (uint32_t)u;
  c0 = raw >= n ? 0u : raw;
  c1 = c0 + 1 == n ? 0u : c0 + 1;
  t = fsub(u, (double)raw);
}

// Weighted: the largest finite weight magnitude's bits and the count of
// non-finite weights, as weight_max_kernel in float.
__global__ void weight_max_f64_kernel(const double* __restrict__ w, uint64_t n,
                                      unsigned long long* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long m = 0, bad = 0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(w[p]) & 0x7fffffffffffffffull;
    if (b >= 0x7ff0000000000000ull)
      bad++;
    else
      m = b > m ? b : m;
  }
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_down_sync(0xffffffffu, m, d);
    m = o > m ? o : m;
    bad += __shfl_down_sync(0xffffffffu, bad, d);
  }
  if ((threadIdx.x & 31u) == 0) {
    if (m) atomicMax(out, m);
    if (bad) atomicAdd(out + 1, bad);
  }
}

// The FP64 quantum: 2^-40 of a particle, or of the largest weight's binade
// (clamped to keep the scale and its inverse normal).
__device__ __forceinline__ int weight_scale_exp_f64(const unsigned long long* wmax) {
  const int e = (int)(wmax[0] >> 52) - 1023;
  return min(900, max(-900, 40 - e));
}

__global__ void cic_f64_kernel(const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, uint64_t np, uint32_t n, double box,
                               double idx, unsigned long long* __restrict__ acc,
                               const double* __restrict__ wts,
                               const unsigned long long* __restrict__ wmax) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double qs = kQ64;
  if (wts) qs = __longlong_as_double((long long)(1023 + weight_scale_exp_f64(wmax)) << 52);
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    uint32_t x0, x1, y0, y1, z0, z1;
    double tx, ty, tz;
    cic_axis_f64(x[p], n, box, idx, x0, x1, tx);
    cic_axis_f64(y[p], n, box, idx, y0, y1, ty);
    cic_axis_f64(z[p], n, box, idx, z0, z1, tz);
    double wz0 = fsub(1.0, tz), wz1 = tz, pw = 1.0;
    if (wts) {
      pw = wts[p];
      // A non-finite weight is added afterwards, outside the sums.
      if (((unsigned long long)__double_as_longlong(pw) & 0x7fffffffffffffffull) >=
          0x7ff0000000000000ull)
        continue;
      wz0 = fmul(pw, wz0);
      wz1 = fmul(pw, wz1);
    }
    const double wx0 = fsub(1.0, tx), wy0 = fsub(1.0, ty);
    const double w00 = fmul(wx0, wy0), w01 = fmul(wx0, ty), w10 = fmul(tx, wy0),
                 w11 = fmul(tx, ty);
    const double w[8] = {fmul(w00, wz0), fmul(w00, wz1), fmul(w01, wz0), fmul(w01, wz1),
                         fmul(w10, wz0), fmul(w10, wz1), fmul(w11, wz0), fmul(w11, wz1)};
    long long q[8];
    long long sum = 0;
    int big = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      q[k] = __double2ll_rn(fmul(w[k], qs));
      sum += q[k];
      if (fabs(w[k]) > fabs(w[big])) big = k;
    }
    const long long fix = (wts ? __double2ll_rn(fmul(pw, qs)) : (long long)kQ64) - sum;
    const uint32_t xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const long long v = q[k] + (k == big ? fix : 0);
      if (v == 0) continue;
      const uint64_t c = ((uint64_t)xs[k >> 2] * n + ys[(k >> 1) & 1]) * n + zs[k & 1];
      atomicAdd(acc + c, (unsigned long long)v);
    }
  }
}

__global__ void cic_f64_finish_kernel(const unsigned long long* __restrict__ acc, uint64_t cells,
                                      double inv_cell_vol, double* __restrict__ grid,
                                      const unsigned long long* __restrict__ wmax) {
  double qinv = 1.0 / kQ64;
  if (wmax) qinv = __longlong_as_double((long long)(1023 - weight_scale_exp_f64(wmax)) << 52);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cells; i += stride)
    grid[i] = fmul(fmul(__ll2double_rn((long long)acc[i]), qinv), inv_cell_vol);
}

// Each non-finite weight's eight products added to its cells (see the float
// form's nonfinite_weights_kernel).
__global__ void nonfinite_weights_f64_kernel(const double* __restrict__ x,
                                             const double* __restrict__ y,
                                             const double* __restrict__ z,
                                             const double* __restrict__ w, uint64_t np, uint32_t n,
                                             double box, double idx,
                                             const unsigned long long* __restrict__ wmax,
                                             double* __restrict__ grid) {
  if (wmax[1] == 0) return;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    const double pw = w[p];
    if (((unsigned long long)__double_as_longlong(pw) & 0x7fffffffffffffffull) <
        0x7ff0000000000000ull)
      continue;
    uint32_t c0[3], c1[3];
    double t[3];
    cic_axis_f64(x[p], n, box, idx, c0[0], c1[0], t[0]);
    cic_axis_f64(y[p], n, box, idx, c0[1], c1[1], t[1]);
    cic_axis_f64(z[p], n, box, idx, c0[2], c1[2], t[2]);
    for (int k = 0; k < 8; k++) {
      uint32_t q[3];
      double f = 1.0;
      for (int a = 0; a < 3; a++) {
        const int up = (k >> (2 - a)) & 1;
        q[a] = up ? c1[a] : c0[a];
        f = fmul(f, up ? t[a] : fsub(1.0, t[a]));
      }
      double* cell = grid + ((uint64_t)q[0] * n + q[1]) * n + q[2];
      *cell = fadd(*cell, fmul(pw, f));
    }
  }
}

size_t cic_f64_scratch_bytes(uint32_t n) { return (size_t)n * n * n * sizeof(unsigned long long) + 512; }

void cic_deposit_f64(const double* x, const double* y, const double* z, uint64_t n_particles,
                     uint32_t n, double box, double* grid, void* scratch, cudaStream_t st,
                     KernelTimer* timer, const double* w) {
  const uint64_t cells = (uint64_t)n * n * n;
  unsigned long long* acc = (unsigned long long*)scratch;
  unsigned long long* wmax = w ? acc + cells : nullptr;
  SIFG_CUDA(cudaMemsetAsync(acc, 0, (cells + (w ? 2 : 0)) * sizeof(unsigned long long), st));
  // grid.c:684 and 735-737 in double.
  const double idx = (double)n / box;
  const double cl = box / (double)n;
  const double inv_cell_vol = 1.0f / (double)(cl * cl * cl);
  if (w) {
    weight_max_f64_kernel<<<grid_for(n_particles, 256, 152u * 16u), 256, 0, st>>>(w, n_particles,
                                                                                  wmax);
    SIFG_LAUNCH_CHECK();
  }
  if (timer) timer->begin(st);
  cic_f64_kernel<<<grid_for(n_particles, 256), 256, 0, st>>>(x, y, z, n_particles, n, box, idx, acc,
                                                             w, wmax);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
  cic_f64_finish_kernel<<<grid_for(cells, 256), 256, 0, st>>>(acc, cells, inv_cell_vol, grid, wmax);
  SIFG_LAUNCH_CHECK();
  if (w) {
    nonfinite_weights_f64_kernel<<<grid_for(n_particles, 256, 152u * 16u), 256, 0, st>>>(
        x, y, z, w, n_particles, n, box, idx, wmax, grid);
    SIFG_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// Density contrast: the mean in double over fixed blocks (a fixed launch, so
// the summation order and the result never change), then v * inv - 1.
// ---------------------------------------------------------------------------
constexpr int kMeanBlocks = 1024;
constexpr int kMeanThreads = 256;

template <class R>
__global__ void __launch_bounds__(kMeanThreads) mean_partial_kernel(const R* __restrict__ v,
                                                                    uint64_t n,
                                                                    double* __restrict__ partial) {
  __shared__ double s[kMeanThreads];
  const uint64_t chunk = (n + kMeanBlocks - 1) / kMeanBlocks;
  const uint64_t lo = (uint64_t)blockIdx.x * chunk;
  const uint64_t hi = lo + chunk < n ? lo + chunk : n;
  double acc = 0.0;
  // Four loads in flight, added in the same order as one at a time.
  uint64_t i = lo + threadIdx.x;
  for (; i + 3 * kMeanThreads < hi; i += 4 * kMeanThreads) {
    const R a = v[i], b = v[i + kMeanThreads], c = v[i + 2 * kMeanThreads],
            d = v[i + 3 * kMeanThreads];
    acc += (double)a;
    acc += (double)b;
    acc += (double)c;
    acc += (double)d;
  }
  for (; i < hi; i += kMeanThreads) acc += (double)v[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kMeanThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// The float form's partial sums without a double operation per value: this
// GPU's FP64 rate would bound the pass (a conversion and an add per cell),
// not its 4 bytes a cell. Each thread keeps its running sum as a float pair
// by Knuth's TwoSum (the rounding error of every add kept in the low part),
// at least as exact as a double chain over the same values, in the same
// fixed order; the block's 256 pairs are then added in double as above.
template <>
__global__ void __launch_bounds__(kMeanThreads) mean_partial_kernel<float>(
    const float* __restrict__ v, uint64_t n, double* __restrict__ partial) {
  __shared__ double s[kMeanThreads];
  const uint64_t chunk = (n + kMeanBlocks - 1) / kMeanBlocks;
  const uint64_t lo = (uint64_t)blockIdx.x * chunk;
  const uint64_t hi = lo + chunk < n ? lo + chunk : n;
  float sh = 0.0f, sl = 0.0f;
  auto add = [&](float x) {
    const float t = __fadd_rn(sh, x);
    const float b = __fsub_rn(t, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, b)), __fsub_rn(x, b));
    sh = t;
    sl = __fadd_rn(sl, e);
  };
  uint64_t i = lo + threadIdx.x;
  for (; i + 3 * kMeanThreads < hi; i += 4 * kMeanThreads) {
    const float a = v[i], b = v[i + kMeanThreads], c = v[i + 2 * kMeanThreads],
                d = v[i + 3 * kMeanThreads];
    add(a);
    add(b);
    add(c);
    add(d);
  }
  for (; i < hi; i += kMeanThreads) add(v[i]);
  s[threadIdx.x] = (double)sh + (double)sl;
  __syncthreads();
  for (int w = kMeanThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void mean_final_kernel(const double* __restrict__ partial, uint64_t n,
                                  double* __restrict__ mean_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < kMeanBlocks; b++) t += partial[b];
    mean_out[0] = t / (double)n;
  }
}

template <class R>
__global__ void contrast_kernel(R* __restrict__ v, uint64_t n, const double* __restrict__ mean) {
  // The double division once a block (this GPU's FP64 rate is low).
  __shared__ R inv_s;
  if (threadIdx.x == 0) inv_s = (R)(1.0 / mean[0]);
  __syncthreads();
  const R inv = inv_s;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    v[i] = fsub(fmul(v[i], inv), R(1.0f));
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

static CicGeom make_geom(uint32_t n, float box) {
  CicGeom g;
  g.n = n;
  g.nt = (n + TB - 1) / TB;
  g.box = box;
  const double idx = (double)n / (double)box;
  g.idx_hi = (float)idx;
  g.idx_lo = (float)(idx - (double)g.idx_hi);
  return g;
}

size_t cic_scratch_bytes(uint64_t n_particles, uint32_t n, bool weighted) {
  const uint64_t nt = (n + TB - 1) / TB;
  const uint64_t tiles = nt * nt * nt;
  const uint64_t face = 3 * nt * (uint64_t)n * n * sizeof(unsigned long long);
  return n_particles * (sizeof(float4) + (weighted ? sizeof(float) : 0)) +
         (2 * tiles + 2) * sizeof(uint32_t) + face + 16 * 256 + 512;
}

void cic_deposit(const float* x, const float* y, const float* z, uint64_t n_particles,
                 uint32_t n, float box, float* grid, void* scratch, cudaStream_t st,
                 KernelTimer* timer, const float* bounds, unsigned long long* outside,
                 cudaEvent_t sorted, const float* w, KernelTimer* stage) {
  const CicGeom g = make_geom(n, box);
  const uint64_t nt = g.nt, tiles = nt * nt * nt;
  char* p = (char*)scratch;
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return (void*)r;
  };
  float4* rec = (float4*)take(n_particles * sizeof(float4));
  uint32_t* counts = (uint32_t*)take((tiles + 1) * sizeof(uint32_t));
  uint32_t* cursor = (uint32_t*)take((tiles + 1) * sizeof(uint32_t));
  const size_t face_elems = nt * (uint64_t)n * n;
  FaceBufs faces;
  faces.fx = (unsigned long long*)take(face_elems * 8);
  faces.fy = (unsigned long long*)take(face_elems * 8);
  faces.fz = (unsigned long long*)take(face_elems * 8);
  float* wrec = w ? (float*)take(n_particles * sizeof(float)) : nullptr;
  unsigned* wmax = w ? (unsigned*)take(2 * sizeof(unsigned)) : nullptr;

  // The stage: the tile sort, the deposit proper and the faces' fix-up.
  if (stage) stage->begin(st);
  SIFG_CUDA(cudaMemsetAsync(counts, 0, (tiles + 1) * sizeof(uint32_t), st));
  SIFG_CUDA(cudaMemsetAsync(faces.fx, 0, face_elems * 8, st));
  SIFG_CUDA(cudaMemsetAsync(faces.fy, 0, face_elems * 8, st));
  SIFG_CUDA(cudaMemsetAsync(faces.fz, 0, face_elems * 8, st));
  const unsigned blk = 256;
  const unsigned grd = grid_for(n_particles, blk, 152u * 16u);
  if (w) {
    SIFG_CUDA(cudaMemsetAsync(wmax, 0, 2 * sizeof(unsigned), st));
    weight_max_kernel<<<grd, blk, 0, st>>>(w, n_particles, wmax);
    SIFG_LAUNCH_CHECK();
  }
  tile_count_kernel<<<grd, blk, 0, st>>>(x, y, z, n_particles, g, counts,
                                         bounds ? bounds[0] : 0.f, bounds ? bounds[1] : 0.f,
                                         bounds ? outside : nullptr);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_u32(counts, (uint32_t)(tiles + 1), st);
  SIFG_CUDA(cudaMemcpyAsync(cursor, counts, (tiles + 1) * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, st));
  tile_scatter_kernel<<<grd, blk, 0, st>>>(x, y, z, n_particles, g, cursor, rec, w, wrec);
  SIFG_LAUNCH_CHECK();
  if (sorted) SIFG_CUDA(cudaEventRecord(sorted, st));
  const float cl = box / (float)n;
  const float inv_cell_vol = 1.0f / (float)(cl * cl * cl);
  const size_t smem = (size_t)2 * TS * TS * TS * sizeof(uint32_t);
  thread_local bool attr = false;  // a per-thread flag: the attribute is set once per thread
  if (!attr) {
    SIFG_CUDA(cudaFuncSetAttribute(tile_deposit_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const unsigned dgrid = (unsigned)(tiles < 152u * 5u ? tiles : 152u * 5u);
  if (timer) timer->begin(st);
  tile_deposit_kernel<<<dgrid, 256, smem, st>>>(rec, counts, g, inv_cell_vol, grid, faces,
                                                 wrec, wmax);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
  face_fixup_kernel<<<grid_for(3 * face_elems, 256), 256, 0, st>>>(g, inv_cell_vol, grid, faces,
                                                                  wmax);
  SIFG_LAUNCH_CHECK();
  if (stage) stage->end(st);
  if (w) {
    nonfinite_weights_kernel<<<grd, blk, 0, st>>>(x, y, z, w, n_particles, g, wmax, grid);
    SIFG_LAUNCH_CHECK();
  }
}

template <class R>
void density_contrast(R* v, uint64_t n, double* d_scratch, cudaStream_t st, bool mean_only) {
  // d_scratch: kMeanBlocks + 1 doubles.
  mean_partial_kernel<R><<<kMeanBlocks, kMeanThreads, 0, st>>>(v, n, d_scratch);
  SIFG_LAUNCH_CHECK();
  mean_final_kernel<<<1, 32, 0, st>>>(d_scratch, n, d_scratch + kMeanBlocks);
  SIFG_LAUNCH_CHECK();
  if (!mean_only) apply_contrast(v, n, d_scratch + kMeanBlocks, st);
}
template void density_contrast<float>(float*, uint64_t, double*, cudaStream_t, bool);
template void density_contrast<double>(double*, uint64_t, double*, cudaStream_t, bool);

template <class R>
void apply_contrast(R* v, uint64_t n, const double* mean, cudaStream_t st) {
  contrast_kernel<R><<<grid_for(n, 256), 256, 0, st>>>(v, n, mean);
  SIFG_LAUNCH_CHECK();
}
template void apply_contrast<float>(float*, uint64_t, const double*, cudaStream_t);
template void apply_contrast<double>(double*, uint64_t, const double*, cudaStream_t);

const double* contrast_mean(const double* d_scratch) { return d_scratch + kMeanBlocks; }

size_t density_contrast_scratch_bytes() { return (kMeanBlocks + 1) * sizeof(double); }

double read_mean(const double* d_scratch, cudaStream_t st) {
  // On the stream that computed it: the library's streams do not wait for
  // the legacy default stream, nor it for them.
  double m = 0.0;
  SIFG_CUDA(cudaMemcpyAsync(&m, d_scratch + kMeanBlocks, sizeof(double), cudaMemcpyDeviceToHost, st));
  SIFG_CUDA(cudaStreamSynchronize(st));
  return m;
}

}  // namespace sifg
