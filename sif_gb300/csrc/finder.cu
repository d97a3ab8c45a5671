// The per-rung finder stages of the exodus path on the GPU.
//
// scan_candidates  sif__finder_scan_candidates (src/finder/utils.c:130-213),
//                  the flat-order compaction; the depth order itself is
//                  the host's replay of the reference's quicksort.
// prefilter        prefilter_cells (src/finder/exodus_finder.c:871-944):
//                  mask bit, pole probe and exact overlap at the rung radius,
//                  against the catalogue as the rung begins.
// grow             sif__exodus_find_radius (src/finder/exodus_rescale.c:
//                  642-1027): early refusal, d^2 histogram in shared memory,
//                  bin walk, exact resolution of a window of bins.
// commit_round     the sequential commit of exodus_finder.c:2181-2329 as
//                  rounds: a survivor is decided once every survivor ranked
//                  before it that it could interact with is decided.
// paint_new        sif__mark_sphere (src/finder/utils.c:965-1033).
//
// Every R expression that decides a candidate is written with _rn
// intrinsics in the reference's order, so it rounds as the strict CPU build.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "common.cuh"
#include "finder.cuh"

namespace sifg {

// ---------------------------------------------------------------------------
// Candidate scan
// ---------------------------------------------------------------------------
// Each thread takes 4 consecutive cells per round with one 16-byte load (the
// field is 256-byte aligned, cells 4k..4k+3 never straddle it) and their 4
// mask bits from one word; a block covers kScanChunk cells.
constexpr int kScanT = 256;
constexpr int kScanRounds = 8;
constexpr uint64_t kScanChunk = (uint64_t)kScanT * 4 * kScanRounds;

uint32_t scan_blocks(uint64_t n_cells) { return (uint32_t)((n_cells + kScanChunk - 1) / kScanChunk); }

// Four consecutive cells in one 16-byte load (two for double).
__device__ __forceinline__ void load4(const float* __restrict__ f, uint64_t c0, float* v) {
  const float4 q = __ldg(reinterpret_cast<const float4*>(f + c0));
  v[0] = q.x;
  v[1] = q.y;
  v[2] = q.z;
  v[3] = q.w;
}
__device__ __forceinline__ void load4(const double* __restrict__ f, uint64_t c0, double* v) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(f + c0));
  const double2 b = __ldg(reinterpret_cast<const double2*>(f + c0 + 2));
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
  v[3] = b.y;
}

// is_minimum of src/finder/utils.c:243-259 on the 27-node stencil of
// load_stencil (utils.c:221-241): strictly below every neighbour at a lower
// flat index, not above any at a higher one, so of a run of equal values
// exactly the lowest-indexed node is a minimum.
template <class R>
__device__ bool is_minimum(const R* __restrict__ f, uint32_t n, uint64_t i) {
  const uint64_t nn = (uint64_t)n * n;
  const uint32_t ix = (uint32_t)(i / nn), iy = (uint32_t)((i / n) % n), iz = (uint32_t)(i % n);
  const uint32_t xs[3] = {(ix + n - 1) % n, ix, (ix + 1) % n};
  const uint32_t ys[3] = {(iy + n - 1) % n, iy, (iy + 1) % n};
  const uint32_t zs[3] = {(iz + n - 1) % n, iz, (iz + 1) % n};
  const R v = __ldg(f + i);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) {
        if (a == 1 && b == 1 && c == 1) continue;
        const uint64_t j = (uint64_t)xs[a] * nn + (uint64_t)ys[b] * n + zs[c];
        const R w = __ldg(f + j);
        if (j < i ? !(v < w) : !(v <= w)) return false;
      }
  return true;
}

// The candidate bits of cells c0..c0+3 (bit j for c0 + j), and their depths.
// With `minima` (SIF_FINDER_SEEDS_MINIMA, no refinement) a cell must also be
// a local minimum of the field (sif__finder_scan_refined with minima_only,
// utils.c:406-552); grid_n is the grid's side.
template <class R>
__device__ __forceinline__ uint32_t quad_candidates(const R* __restrict__ f,
                                                    const uint32_t* __restrict__ mask,
                                                    uint64_t c0, uint64_t n, R thr, R* v,
                                                    uint32_t grid_n, bool minima) {
  if (c0 + 3 < n) {
    load4(f, c0, v);
  } else {
    for (int k = 0; k < 4; k++) v[k] = c0 + k < n ? f[c0 + k] : R(1);
  }
  if (c0 >= n) return 0u;
  const uint32_t m = __ldg(mask + (c0 >> 5)) >> (c0 & 31);
  uint32_t bits = 0;
#pragma unroll
  for (int k = 0; k < 4; k++)
    bits |= (v[k] <= thr && !(m & (1u << k)) && c0 + k < n) ? (1u << k) : 0u;
  if (minima)
    for (uint32_t b = bits; b; b &= b - 1) {
      const int k = __ffs(b) - 1;
      if (!is_minimum(f, grid_n, c0 + k)) bits &= ~(1u << k);
    }
  return bits;
}

// Exclusive scan of one value per thread across the block; *total the sum.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* ws, uint32_t* total) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= (unsigned)d) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  uint32_t before = 0, t = 0;
#pragma unroll
  for (int w = 0; w < kScanT / 32; w++) {
    const uint32_t s = ws[w];
    before += (w < (int)warp) ? s : 0u;
    t += s;
  }
  __syncthreads();
  *total = t;
  return before + x - v;
}

template <class R>
__global__ void __launch_bounds__(kScanT) scan_count_kernel(const R* __restrict__ f,
                                                            const uint32_t* __restrict__ mask,
                                                            uint64_t n, R thr,
                                                            uint32_t* __restrict__ counts,
                                                            uint32_t grid_n, bool minima) {
  __shared__ uint32_t ws[kScanT / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
  uint32_t c = 0;
#pragma unroll
  for (int j = 0; j < kScanRounds; j++) {
    R v[4];
    c += __popc(quad_candidates(f, mask, base + ((uint64_t)j * kScanT + threadIdx.x) * 4, n, thr, v,
                                grid_n, minima));
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanT / 32; w++) t += ws[w];
    counts[blockIdx.x] = t;
  }
}

template <class R>
__global__ void __launch_bounds__(kScanT) scan_write_kernel(
    const R* __restrict__ f, const uint32_t* __restrict__ mask, uint64_t n, R thr,
    const uint32_t* __restrict__ offsets, R* __restrict__ cdelta, uint32_t* __restrict__ cflat,
    uint32_t grid_n, bool minima) {
  __shared__ uint32_t ws[kScanT / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
  uint32_t out = offsets[blockIdx.x];
  for (int j = 0; j < kScanRounds; j++) {
    const uint64_t c0 = base + ((uint64_t)j * kScanT + threadIdx.x) * 4;
    R v[4];
    const uint32_t bits = quad_candidates(f, mask, c0, n, thr, v, grid_n, minima);
    uint32_t total;
    uint32_t pos = out + block_scan_excl(__popc(bits), ws, &total);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (bits & (1u << k)) {
        cdelta[pos] = v[k];
        cflat[pos] = (uint32_t)(c0 + k);
        pos++;
      }
    }
    out += total;
  }
}

// One pass over the field: each CTA writes its candidates, in flat order, to
// the start of its own region of kScanChunk slots and its count to
// counts[block]; the compaction then moves only the candidates.
template <class R>
__global__ void __launch_bounds__(kScanT) scan_regions_kernel(
    const R* __restrict__ f, const uint32_t* __restrict__ mask, uint64_t n, R thr,
    uint32_t* __restrict__ counts, R* __restrict__ rdelta, uint32_t* __restrict__ rflat,
    uint32_t grid_n, bool minima) {
  __shared__ uint32_t ws[kScanT / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
  uint32_t out = 0;
  for (int j = 0; j < kScanRounds; j++) {
    const uint64_t c0 = base + ((uint64_t)j * kScanT + threadIdx.x) * 4;
    R v[4];
    const uint32_t bits = quad_candidates(f, mask, c0, n, thr, v, grid_n, minima);
    uint32_t total;
    uint32_t pos = out + block_scan_excl(__popc(bits), ws, &total);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (bits & (1u << k)) {
        rdelta[base + pos] = v[k];
        rflat[base + pos] = (uint32_t)(c0 + k);
        pos++;
      }
    }
    out += total;
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = out;
}

// A warp per region: its candidates to their place in the compacted list.
template <class R>
__global__ void scan_compact_kernel(const uint32_t* __restrict__ offsets, uint32_t nb,
                                    const R* __restrict__ rdelta, const uint32_t* __restrict__ rflat,
                                    R* __restrict__ cdelta, uint32_t* __restrict__ cflat) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += warps) {
    const uint32_t o = offsets[b], cnt = offsets[b + 1] - o;
    const uint64_t src = (uint64_t)b * kScanChunk;
    for (uint32_t i = lane; i < cnt; i += 32) {
      cdelta[o + i] = rdelta[src + i];
      cflat[o + i] = rflat[src + i];
    }
  }
}

uint64_t scan_region_slots(uint64_t n_cells) { return (uint64_t)scan_blocks(n_cells) * kScanChunk; }

// The candidates from a below-threshold list made by the smoothing (blocks
// of `block` cells, block b's entries at the start of its region): the
// listed cells whose mask bit is clear, in the list's order. A warp per block.
__global__ void below_count_kernel(const uint32_t* __restrict__ counts,
                                   const uint32_t* __restrict__ flat, uint32_t nb, uint32_t block,
                                   const uint32_t* mask, uint32_t* __restrict__ kept) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += warps) {
    const uint32_t cnt = counts[b];
    const uint32_t* f = flat + (uint64_t)b * block;
    uint32_t k = 0;
    for (uint32_t i = lane; i < cnt; i += 32) k += mask_get_rw(mask, f[i]) ? 0u : 1u;
    k = __reduce_add_sync(0xffffffffu, k);
    if (lane == 0) kept[b] = k;
  }
}

__global__ void below_write_kernel(const uint32_t* __restrict__ counts,
                                   const float* __restrict__ delta,
                                   const uint32_t* __restrict__ flat, uint32_t nb, uint32_t block,
                                   const uint32_t* mask, const uint32_t* __restrict__ offsets,
                                   float* __restrict__ cdelta, uint32_t* __restrict__ cflat) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += warps) {
    const uint32_t cnt = counts[b];
    const uint64_t src = (uint64_t)b * block;
    uint32_t out = offsets[b];
    for (uint32_t i0 = 0; i0 < cnt; i0 += 32) {
      const uint32_t i = i0 + lane;
      uint32_t c = 0;
      bool keep = false;
      if (i < cnt) {
        c = flat[src + i];
        keep = !mask_get_rw(mask, c);
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const uint32_t pos = out + __popc(ballot & ((1u << lane) - 1u));
        cdelta[pos] = delta[src + i];
        cflat[pos] = c;
      }
      out += __popc(ballot);
    }
  }
}

void below_count_pass(const uint32_t* counts, const uint32_t* flat, uint32_t nb, uint32_t block,
                      const uint32_t* mask, uint32_t* block_counts, uint32_t* d_count,
                      cudaStream_t st) {
  const uint32_t warps = nb < 152u * 64u ? nb : 152u * 64u;
  below_count_kernel<<<(warps + 7) / 8, 256, 0, st>>>(counts, flat, nb, block, mask, block_counts);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_total(block_counts, nb, d_count, st);
}

void below_write_pass(const uint32_t* counts, const float* delta, const uint32_t* flat,
                      uint32_t nb, uint32_t block, const uint32_t* mask,
                      const uint32_t* block_offsets, float* cand_delta, uint32_t* cand_flat,
                      cudaStream_t st) {
  const uint32_t warps = nb < 152u * 64u ? nb : 152u * 64u;
  below_write_kernel<<<(warps + 7) / 8, 256, 0, st>>>(counts, delta, flat, nb, block, mask,
                                                      block_offsets, cand_delta, cand_flat);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void scan_fused_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     uint32_t* block_counts, uint32_t* d_count, R* region_delta,
                     uint32_t* region_flat, cudaStream_t st, uint32_t grid_n, bool minima) {
  const uint32_t nb = scan_blocks(n_cells);
  scan_regions_kernel<R><<<nb, kScanT, 0, st>>>(field, mask, n_cells, threshold, block_counts,
                                                region_delta, region_flat, grid_n, minima);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_total(block_counts, nb, d_count, st);
}

template <class R>
void scan_compact(const uint32_t* block_counts, uint64_t n_cells, const R* region_delta,
                  const uint32_t* region_flat, R* cand_delta, uint32_t* cand_flat,
                  cudaStream_t st) {
  const uint32_t nb = scan_blocks(n_cells);
  const uint32_t warps = nb < 152u * 64u ? nb : 152u * 64u;
  scan_compact_kernel<R><<<(warps + 7) / 8, 256, 0, st>>>(block_counts, nb, region_delta,
                                                           region_flat, cand_delta, cand_flat);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void scan_count_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     uint32_t* block_counts, uint32_t* d_count, cudaStream_t st, uint32_t grid_n,
                     bool minima) {
  const uint32_t nb = scan_blocks(n_cells);
  scan_count_kernel<<<nb, kScanT, 0, st>>>(field, mask, n_cells, threshold, block_counts, grid_n,
                                           minima);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_total(block_counts, nb, d_count, st);
}

template <class R>
void scan_write_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     const uint32_t* block_counts, R* cand_delta, uint32_t* cand_flat,
                     cudaStream_t st, uint32_t grid_n, bool minima) {
  scan_write_kernel<<<scan_blocks(n_cells), kScanT, 0, st>>>(field, mask, n_cells, threshold,
                                                             block_counts, cand_delta, cand_flat,
                                                             grid_n, minima);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Overlap tests
// ---------------------------------------------------------------------------

// sif__overlap_quick, src/finder/utils.c:819-848.
__device__ bool overlap_quick(const uint32_t* mask, uint32_t n, uint32_t ix, uint32_t iy,
                              uint32_t iz, uint32_t r) {
  const uint64_t nn = n;
  if (mask_get_rw(mask, ((uint64_t)wrap_pbc((int32_t)(ix + r), n) * nn + iy) * nn + iz)) return true;
  if (mask_get_rw(mask, ((uint64_t)wrap_pbc((int32_t)ix - (int32_t)r, n) * nn + iy) * nn + iz)) return true;
  if (mask_get_rw(mask, ((uint64_t)ix * nn + wrap_pbc((int32_t)(iy + r), n)) * nn + iz)) return true;
  if (mask_get_rw(mask, ((uint64_t)ix * nn + wrap_pbc((int32_t)iy - (int32_t)r, n)) * nn + iz)) return true;
  if (mask_get_rw(mask, ((uint64_t)ix * nn + iy) * nn + wrap_pbc((int32_t)(iz + r), n))) return true;
  if (mask_get_rw(mask, ((uint64_t)ix * nn + iy) * nn + wrap_pbc((int32_t)iz - (int32_t)r, n))) return true;
  return false;
}

// The pair test of sif__overlap_exact (src/finder/utils.c:904-955): the
// interior form when the query's search box lies inside the box, the
// minimum-image form otherwise.
template <class R>
__device__ __forceinline__ bool collide(R cx, R cy, R cz, R r, R vx, R vy,
                                        R vz, R rj, R f, R scale, R box,
                                        R half, bool interior) {
  const R mn = r < rj ? r : rj;
  const R tot = fmul(scale, fsub(fadd(r, rj), fmul(f, mn)));
  const R tot2 = fmul(tot, tot);
  if (interior) {
    const R dx = fsub(cx, vx), dy = fsub(cy, vy), dz = fsub(cz, vz);
    return fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)) < tot2;
  }
  R dx = fabs_(fsub(cx, vx));
  dx = dx > half ? fsub(box, dx) : dx;
  const R dx2 = fmul(dx, dx);
  if (dx2 >= tot2) return false;
  R dy = fabs_(fsub(cy, vy));
  dy = dy > half ? fsub(box, dy) : dy;
  const R dy2 = fmul(dy, dy);
  const R dxy2 = fadd(dx2, dy2);
  if (dxy2 >= tot2) return false;
  R dz = fabs_(fsub(cz, vz));
  dz = dz > half ? fsub(box, dz) : dz;
  return fadd(dxy2, fmul(dz, dz)) < tot2;
}

template <class R>
__device__ __forceinline__ R search_radius(R r, R max_r, R f, R scale) {
  const R mn = r < max_r ? r : max_r;
  return fmul(scale, fsub(fadd(r, max_r), fmul(f, mn)));
}

template <class R>
__device__ __forceinline__ bool is_interior(R cx, R cy, R cz, R s, R box) {
  return fsub(cx, s) >= 0.0f && fadd(cx, s) < box && fsub(cy, s) >= 0.0f && fadd(cy, s) < box &&
         fsub(cz, s) >= 0.0f && fadd(cz, s) < box;
}

// sif__overlap_exact (src/finder/utils.c:850-960) over the void index.
template <class R>
__device__ bool overlap_exact(const VoidViewT<R>& v, R cx, R cy, R cz, R r, R f,
                              R scale, R box) {
  if (v.n == 0) return false;
  const R half = fmul(box, R(0.5f));
  const R s = search_radius(r, v.max_r, f, scale);
  const int32_t x0 = (int32_t)ffloor(fmul(fsub(cx, s), v.inv_cell));
  const int32_t x1 = (int32_t)ffloor(fmul(fadd(cx, s), v.inv_cell));
  const int32_t y0 = (int32_t)ffloor(fmul(fsub(cy, s), v.inv_cell));
  const int32_t y1 = (int32_t)ffloor(fmul(fadd(cy, s), v.inv_cell));
  const int32_t z0 = (int32_t)ffloor(fmul(fsub(cz, s), v.inv_cell));
  const int32_t z1 = (int32_t)ffloor(fmul(fadd(cz, s), v.inv_cell));
  const bool interior = is_interior(cx, cy, cz, s, box);
  for (int32_t ix = x0; ix <= x1; ix++) {
    const uint32_t wx = (uint32_t)ix & (kVoidCells - 1);
    for (int32_t iy = y0; iy <= y1; iy++) {
      const uint32_t wy = (uint32_t)iy & (kVoidCells - 1);
      for (int32_t iz = z0; iz <= z1; iz++) {
        const uint32_t wz = (uint32_t)iz & (kVoidCells - 1);
        const uint32_t c = (wx * kVoidCells + wy) * kVoidCells + wz;
        for (uint32_t k = v.start[c]; k < v.start[c + 1]; k++) {
          const uint32_t j = v.ids[k];
          if (collide(cx, cy, cz, r, v.cx[j], v.cy[j], v.cz[j], v.r[j], f, scale, box, half,
                      interior))
            return true;
        }
      }
    }
  }
  return false;
}

// overlap_exact by a warp: the same cells and the same pair tests, the
// lanes taking the cells 32 at a time (a thread alone walks them one load
// after another). Every lane returns the answer.
template <class R>
__device__ bool overlap_exact_warp(const VoidViewT<R>& v, R cx, R cy, R cz, R r, R f, R scale,
                                   R box) {
  if (v.n == 0) return false;
  const unsigned lane = threadIdx.x & 31u;
  const R half = fmul(box, R(0.5f));
  const R s = search_radius(r, v.max_r, f, scale);
  const int32_t x0 = (int32_t)ffloor(fmul(fsub(cx, s), v.inv_cell));
  const int32_t x1 = (int32_t)ffloor(fmul(fadd(cx, s), v.inv_cell));
  const int32_t y0 = (int32_t)ffloor(fmul(fsub(cy, s), v.inv_cell));
  const int32_t y1 = (int32_t)ffloor(fmul(fadd(cy, s), v.inv_cell));
  const int32_t z0 = (int32_t)ffloor(fmul(fsub(cz, s), v.inv_cell));
  const int32_t z1 = (int32_t)ffloor(fmul(fadd(cz, s), v.inv_cell));
  const bool interior = is_interior(cx, cy, cz, s, box);
  const uint32_t ny = (uint32_t)(y1 - y0 + 1), nz = (uint32_t)(z1 - z0 + 1);
  const uint32_t cells = (uint32_t)(x1 - x0 + 1) * ny * nz;
  for (uint32_t k0 = 0; k0 < cells; k0 += 32) {
    bool hit = false;
    const uint32_t k = k0 + lane;
    if (k < cells) {
      const uint32_t wx = (uint32_t)(x0 + (int32_t)(k / (ny * nz))) & (kVoidCells - 1);
      const uint32_t wy = (uint32_t)(y0 + (int32_t)((k / nz) % ny)) & (kVoidCells - 1);
      const uint32_t wz = (uint32_t)(z0 + (int32_t)(k % nz)) & (kVoidCells - 1);
      const uint32_t c = (wx * kVoidCells + wy) * kVoidCells + wz;
      for (uint32_t q = v.start[c]; q < v.start[c + 1] && !hit; q++) {
        const uint32_t j = v.ids[q];
        hit = collide(cx, cy, cz, r, v.cx[j], v.cy[j], v.cz[j], v.r[j], f, scale, box, half, interior);
      }
    }
    if (__any_sync(0xffffffffu, hit)) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// SIF_FINDER_REFINE_GAUSSIAN: the candidates' placing (sif__finder_scan_refined,
// src/finder/utils.c:406-552; place_candidate 331-365; newton_step 261-313)
// ---------------------------------------------------------------------------

// One Newton step from the node on the stencil of the refinement's field,
// in double and in the reference's operation order: the gradient and the
// Hessian by central differences, d = -H^-1 g by cofactors; false unless H
// is positive definite and the step stays within a cell on every axis.
template <class R>
__device__ bool newton_step(const R (&s)[27], double (&d)[3], double& depth) {
  auto S = [&](int a, int b, int c) { return (double)s[(a + 1) * 9 + (b + 1) * 3 + (c + 1)]; };
  const double c0 = S(0, 0, 0);
  const double g0 = __dmul_rn(0.5, __dsub_rn(S(1, 0, 0), S(-1, 0, 0)));
  const double g1 = __dmul_rn(0.5, __dsub_rn(S(0, 1, 0), S(0, -1, 0)));
  const double g2 = __dmul_rn(0.5, __dsub_rn(S(0, 0, 1), S(0, 0, -1)));
  const double two_c0 = __dmul_rn(2.0, c0);
  const double h00 = __dadd_rn(__dsub_rn(S(1, 0, 0), two_c0), S(-1, 0, 0));
  const double h11 = __dadd_rn(__dsub_rn(S(0, 1, 0), two_c0), S(0, -1, 0));
  const double h22 = __dadd_rn(__dsub_rn(S(0, 0, 1), two_c0), S(0, 0, -1));
  const double h01 = __dmul_rn(
      0.25, __dadd_rn(__dsub_rn(__dsub_rn(S(1, 1, 0), S(1, -1, 0)), S(-1, 1, 0)), S(-1, -1, 0)));
  const double h02 = __dmul_rn(
      0.25, __dadd_rn(__dsub_rn(__dsub_rn(S(1, 0, 1), S(1, 0, -1)), S(-1, 0, 1)), S(-1, 0, -1)));
  const double h12 = __dmul_rn(
      0.25, __dadd_rn(__dsub_rn(__dsub_rn(S(0, 1, 1), S(0, 1, -1)), S(0, -1, 1)), S(0, -1, -1)));
  const double k00 = __dsub_rn(__dmul_rn(h11, h22), __dmul_rn(h12, h12));
  const double k01 = __dsub_rn(__dmul_rn(h02, h12), __dmul_rn(h01, h22));
  const double k02 = __dsub_rn(__dmul_rn(h01, h12), __dmul_rn(h02, h11));
  const double k11 = __dsub_rn(__dmul_rn(h00, h22), __dmul_rn(h02, h02));
  const double k12 = __dsub_rn(__dmul_rn(h01, h02), __dmul_rn(h00, h12));
  const double k22 = __dsub_rn(__dmul_rn(h00, h11), __dmul_rn(h01, h01));
  const double det =
      __dadd_rn(__dadd_rn(__dmul_rn(h00, k00), __dmul_rn(h01, k01)), __dmul_rn(h02, k02));
  if (!(h00 > 0.0 && k22 > 0.0 && det > 0.0)) return false;
  d[0] = __ddiv_rn(-__dadd_rn(__dadd_rn(__dmul_rn(k00, g0), __dmul_rn(k01, g1)), __dmul_rn(k02, g2)),
                   det);
  d[1] = __ddiv_rn(-__dadd_rn(__dadd_rn(__dmul_rn(k01, g0), __dmul_rn(k11, g1)), __dmul_rn(k12, g2)),
                   det);
  d[2] = __ddiv_rn(-__dadd_rn(__dadd_rn(__dmul_rn(k02, g0), __dmul_rn(k12, g1)), __dmul_rn(k22, g2)),
                   det);
  if (!(fabs(d[0]) <= 1.0 && fabs(d[1]) <= 1.0 && fabs(d[2]) <= 1.0)) return false;
  depth = __dadd_rn(c0, __dmul_rn(0.5, __dadd_rn(__dadd_rn(__dmul_rn(g0, d[0]), __dmul_rn(g1, d[1])),
                                                __dmul_rn(g2, d[2]))));
  return true;
}

__device__ __forceinline__ int32_t step_cells(double d) { return d > 0.5 ? 1 : (d < -0.5 ? -1 : 0); }

// Each candidate (a cell at or below the threshold on the top-hat fa, not
// masked, in flat order) placed on the refinement's field fb: its depth
// there; a minimum of fb moved by its Newton step to the node it lands on,
// if that node is a candidate too, at the step's depth and with the rest of
// the step as its offset. keep[k]: whether it stays a candidate (all, or
// under SIF_FINDER_SEEDS_MINIMA the minima).
template <class R>
__global__ void refine_kernel(const R* __restrict__ fa, const R* __restrict__ fb,
                              const uint32_t* __restrict__ mask, R thr, uint32_t n, R cell,
                              const uint32_t* __restrict__ cflat, uint32_t m, bool minima_only,
                              R* __restrict__ d_out, uint32_t* __restrict__ f_out,
                              CandOffT<R>* __restrict__ o_out, uint32_t* __restrict__ keep) {
  const uint64_t nn = (uint64_t)n * n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint32_t i = cflat[k];
    const bool minimum = is_minimum(fb, n, i);
    keep[k] = (!minima_only || minimum) ? 1u : 0u;
    R delta = __ldg(fb + i);
    uint32_t flat = i;
    CandOffT<R> o{R(0), R(0), R(0), R(-1.0f)};
    if (minimum) {
      const uint32_t ix = (uint32_t)(i / nn), iy = (uint32_t)((i / n) % n), iz = (uint32_t)(i % n);
      const uint32_t xs[3] = {(ix + n - 1) % n, ix, (ix + 1) % n};
      const uint32_t ys[3] = {(iy + n - 1) % n, iy, (iy + 1) % n};
      const uint32_t zs[3] = {(iz + n - 1) % n, iz, (iz + 1) % n};
      R st[27];
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
          for (int c = 0; c < 3; c++) st[a * 9 + b * 3 + c] = __ldg(fb + xs[a] * nn + (uint64_t)ys[b] * n + zs[c]);
      double d[3], depth;
      if (newton_step(st, d, depth)) {
        const int32_t sx = step_cells(d[0]), sy = step_cells(d[1]), sz = step_cells(d[2]);
        const uint32_t jx = (uint32_t)(((int64_t)ix + sx + n) % n);
        const uint32_t jy = (uint32_t)(((int64_t)iy + sy + n) % n);
        const uint32_t jz = (uint32_t)(((int64_t)iz + sz + n) % n);
        const uint32_t j = (uint32_t)(((uint64_t)jx * n + jy) * n + jz);
        if (__ldg(fa + j) <= thr && !mask_get(mask, j)) {
          delta = (R)depth;
          flat = j;
          o.dx = (R)__dsub_rn(d[0], (double)sx);
          o.dy = (R)__dsub_rn(d[1], (double)sy);
          o.dz = (R)__dsub_rn(d[2], (double)sz);
          // masked_overlap's off (exodus_finder.c:449-451).
          o.len = fmul(fsqrt(fadd(fadd(fmul(o.dx, o.dx), fmul(o.dy, o.dy)), fmul(o.dz, o.dz))), cell);
        }
      }
    }
    d_out[k] = delta;
    f_out[k] = flat;
    o_out[k] = o;
  }
}

// The kept entries in order; pos the exclusive scan of keep (m + 1 entries).
template <class R>
__global__ void refine_compact_kernel(const uint32_t* __restrict__ pos, uint32_t m,
                                      const R* __restrict__ d_in, const uint32_t* __restrict__ f_in,
                                      const CandOffT<R>* __restrict__ o_in, R* __restrict__ d_out,
                                      uint32_t* __restrict__ f_out, CandOffT<R>* __restrict__ o_out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint32_t p = pos[k];
    if (pos[k + 1] == p) continue;
    d_out[p] = d_in[k];
    f_out[p] = f_in[k];
    o_out[p] = o_in[k];
  }
}

template <class R>
uint32_t refine_candidates(const R* fa, const R* fb, const uint32_t* mask, R thr, uint32_t n,
                           R cell, uint32_t m, bool minima_only, R*& cdelta, uint32_t*& cflat,
                           R* d_tmp, uint32_t* f_tmp, CandOffT<R>* o_tmp, CandOffT<R>*& coff,
                           CandOffT<R>* o_out, uint32_t* keep, uint32_t* h_count,
                           cudaStream_t st) {
  if (m == 0) return 0;
  refine_kernel<R><<<grid_for(m, 128), 128, 0, st>>>(fa, fb, mask, thr, n, cell, cflat, m,
                                                      minima_only, d_tmp, f_tmp, o_tmp, keep);
  SIFG_LAUNCH_CHECK();
  if (!minima_only) {
    // Every candidate stays, in order: the placed arrays are the list.
    std::swap(cdelta, d_tmp);
    std::swap(cflat, f_tmp);
    coff = o_tmp;
    return m;
  }
  SIFG_CUDA(cudaMemsetAsync(keep + m, 0, sizeof(uint32_t), st));
  exclusive_scan_u32(keep, m + 1, st);
  refine_compact_kernel<R><<<grid_for(m, 256), 256, 0, st>>>(keep, m, d_tmp, f_tmp, o_tmp, cdelta,
                                                              cflat, o_out);
  SIFG_LAUNCH_CHECK();
  coff = o_out;
  SIFG_CUDA(cudaMemcpyAsync(h_count, keep + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SIFG_CUDA(cudaStreamSynchronize(st));
  return *h_count;
}

// candidate_centre (exodus_finder.c:371-393): node plus offset, times the
// cell length, wrapped into the box; on its node, node times the cell.
template <class R>
__device__ __forceinline__ R cand_axis(uint32_t node, R off, const RungConstsT<R>& rc) {
  R x = fmul(fadd((R)node, off), rc.cell);
  if (x < R(0)) x = fadd(x, rc.box);
  if (x >= rc.box) x = fsub(x, rc.box);
  return x;
}

// masked_overlap (exodus_finder.c:440-452): the node's mask bit; a centre
// off its node (len >= 0) only while len < scale * r * (1 - f).
template <class R>
__device__ __forceinline__ bool cand_masked(const uint32_t* mask, uint32_t node, R len, R r,
                                            const RungConstsT<R>& rc) {
  if (!mask_get_rw(mask, node)) return false;
  if (len < R(0)) return true;
  return len < fmul(fmul(rc.scale, r), fsub(R(1.0f), rc.f));
}

// ---------------------------------------------------------------------------
// Pre-filter
// ---------------------------------------------------------------------------

template <class R>
__global__ void prefilter_kernel(const uint32_t* __restrict__ cflat, uint32_t m,
                                 const uint32_t* __restrict__ mask, VoidViewT<R> voids, RungConstsT<R> rc,
                                 uint8_t* __restrict__ alive, bool keep_all,
                                 const CandOffT<R>* __restrict__ coff) {
  const uint32_t n = rc.grid_n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint32_t flat = cflat[k];
    const CandOffT<R> o = coff ? coff[k] : CandOffT<R>{R(0), R(0), R(0), R(-1.0f)};
    uint8_t ok = 1;
    if (keep_all) {
      // Under displacement a void refusing a candidate now may be gone by
      // its turn (exodus_finder.c:1873-1875): nothing is refused here.
    } else if (cand_masked(mask, flat, o.len, rc.radius, rc)) {
      ok = 0;
    } else {
      const uint32_t ix = flat / (n * n), iy = (flat / n) % n, iz = flat % n;
      if (rc.proxy_pole > 0 && overlap_quick(mask, n, ix, iy, iz, (uint32_t)rc.proxy_pole)) {
        ok = 0;
      } else {
        const R cx = cand_axis(ix, o.dx, rc), cy = cand_axis(iy, o.dy, rc),
                cz = cand_axis(iz, o.dz, rc);
        if (overlap_exact(voids, cx, cy, cz, rc.radius, rc.f, rc.scale, rc.box)) ok = 0;
      }
    }
    alive[k] = ok;
  }
}

constexpr int kCompactT = 256;
constexpr int kCompactRounds = 8;
constexpr uint32_t kCompactChunk = kCompactT * kCompactRounds;

__global__ void __launch_bounds__(kCompactT) flag_count_kernel(const uint8_t* __restrict__ flags,
                                                               uint32_t m,
                                                               uint32_t* __restrict__ counts) {
  __shared__ uint32_t ws[kCompactT / 32];
  const uint32_t base = blockIdx.x * kCompactChunk;
  uint32_t c = 0;
  for (int j = 0; j < kCompactRounds; j++) {
    const uint32_t i = base + j * kCompactT + threadIdx.x;
    c += (i < m && flags[i]) ? 1u : 0u;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kCompactT / 32; w++) t += ws[w];
    counts[blockIdx.x] = t;
  }
}

template <class R>
__global__ void __launch_bounds__(kCompactT) survivor_write_kernel(
    const uint8_t* __restrict__ flags, uint32_t m, const uint32_t* __restrict__ offsets,
    const uint32_t* __restrict__ cflat, RungConstsT<R> rc, uint32_t* __restrict__ surv_cand,
    uint32_t* __restrict__ sflat, R* __restrict__ scx, R* __restrict__ scy,
    R* __restrict__ scz, const CandOffT<R>* __restrict__ coff, R* __restrict__ soff) {
  __shared__ uint32_t wsum[kCompactT / 32];
  const uint32_t base = blockIdx.x * kCompactChunk;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t out = offsets[blockIdx.x];
  const uint32_t n = rc.grid_n;
  for (int j = 0; j < kCompactRounds; j++) {
    const uint32_t i = base + j * kCompactT + threadIdx.x;
    const bool p = i < m && flags[i];
    const unsigned bal = __ballot_sync(0xffffffffu, p);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kCompactT / 32; w++) {
      const uint32_t v = wsum[w];
      before += (w < (int)warp) ? v : 0u;
      total += v;
    }
    if (p) {
      const uint32_t pos = out + before + __popc(bal & ((1u << lane) - 1u));
      const uint32_t flat = cflat[i];
      surv_cand[pos] = i;
      sflat[pos] = flat;
      // candidate_centre (exodus_finder.c:366-388): its node, and its
      // offset off the node where the refinement moved it.
      const CandOffT<R> o = coff ? coff[i] : CandOffT<R>{R(0), R(0), R(0), R(-1.0f)};
      scx[pos] = cand_axis(flat / (n * n), o.dx, rc);
      scy[pos] = cand_axis((flat / n) % n, o.dy, rc);
      scz[pos] = cand_axis(flat % n, o.dz, rc);
      if (soff) soff[pos] = o.len;
    }
    out += total;
    __syncthreads();
  }
}

template <class R>
void prefilter(const uint32_t* cand_flat, uint32_t m, const uint32_t* mask, VoidViewT<R> voids,
               RungConstsT<R> rc, uint8_t* alive, uint32_t* block_counts, uint32_t* surv_cand,
               uint32_t* surv_flat, R* scx, R* scy, R* scz, uint32_t* d_surv_count,
               cudaStream_t st, bool keep_all, const CandOffT<R>* coff, R* soff) {
  if (m == 0) {
    SIFG_CUDA(cudaMemsetAsync(d_surv_count, 0, sizeof(uint32_t), st));
    return;
  }
  prefilter_kernel<<<grid_for(m, 128), 128, 0, st>>>(cand_flat, m, mask, voids, rc, alive, keep_all,
                                                      coff);
  SIFG_LAUNCH_CHECK();
  const uint32_t nb = (m + kCompactChunk - 1) / kCompactChunk;
  flag_count_kernel<<<nb, kCompactT, 0, st>>>(alive, m, block_counts);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_total(block_counts, nb, d_surv_count, st);
  survivor_write_kernel<<<nb, kCompactT, 0, st>>>(alive, m, block_counts, cand_flat, rc,
                                                  surv_cand, surv_flat, scx, scy, scz, coff, soff);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Sphere growth
// ---------------------------------------------------------------------------
// One CTA per survivor. A warp takes the template 32 cells at a time: each
// lane looks up one cell's particle range and periodic image at once, then
// the warp walks the cells that need distances with every lane on a particle.
// The reference's three stages (exodus_rescale.c:738-1007) in two passes over
// the particles: pass 1 reads only the cells that cross a boundary of the
// annulus -- enough for the early refusal, and binning the annulus particles
// they hold on the way; pass 2, for a survivor not refused, bins the cells
// wholly inside the annulus. The counts and the histogram are the reference's
// exactly: the same distances, the same bin_of, the same classification.
constexpr int kGrowT = 256;
constexpr int kGrowWarps = kGrowT / 32;
constexpr uint32_t kMaxBins = 2048;
constexpr uint32_t kSmemBuf = 2048;
constexpr int kWalkUnroll = 4;  // particle loads in flight per lane

unsigned growth_grid() { return 152u * 4u; }

template <class R>
struct CellRange {
  uint32_t s, e;
  R ex, ey, ez;
  uint32_t flat;  // the wrapped cell's flat index
};

// query_cell, src/finder/exodus_rescale.c:295-342.
template <class R>
__device__ __forceinline__ CellRange<R> query_cell(const MeshViewT<R>& m, const TemplateViewT<R>& t,
                                                uint32_t i, int32_t ci, int32_t cj, int32_t ck,
                                                R cx, R cy, R cz) {
  const int32_t N = m.n;
  int32_t ix = ci + __ldg(t.dx + i), iy = cj + __ldg(t.dy + i), iz = ck + __ldg(t.dz + i);
  CellRange<R> r;
  r.ex = cx;
  r.ey = cy;
  r.ez = cz;
  if (ix < 0) { ix += N; r.ex = fadd(cx, m.box); } else if (ix >= N) { ix -= N; r.ex = fsub(cx, m.box); }
  if (iy < 0) { iy += N; r.ey = fadd(cy, m.box); } else if (iy >= N) { iy -= N; r.ey = fsub(cy, m.box); }
  if (iz < 0) { iz += N; r.ez = fadd(cz, m.box); } else if (iz >= N) { iz -= N; r.ez = fsub(cz, m.box); }
  const uint64_t flat = ((uint64_t)ix * N + iy) * N + iz;
  r.s = __ldg(m.offsets + flat);
  r.e = __ldg(m.offsets + flat + 1);
  r.flat = (uint32_t)flat;
  return r;
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v,
                                                            unsigned long long* red) {
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long t = 0;
  for (int w = 0; w < kGrowWarps; w++) t += red[w];
  __syncthreads();
  return t;
}

// Two sums at once: one set of barriers instead of two.
__device__ __forceinline__ void block_sum2_u64(unsigned long long& a, unsigned long long& b,
                                               unsigned long long* red) {
  for (int d = 16; d > 0; d >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, d);
    b += __shfl_down_sync(0xffffffffu, b, d);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = a;
    red[kGrowWarps + (threadIdx.x >> 5)] = b;
  }
  __syncthreads();
  unsigned long long ta = 0, tb = 0;
  for (int w = 0; w < kGrowWarps; w++) {
    ta += red[w];
    tb += red[kGrowWarps + w];
  }
  __syncthreads();
  a = ta;
  b = tb;
}

// Ascending sort of 256 values held by one warp, v[j] at index j * 32 + lane:
// a bitonic network, partners in other lanes through shuffles, in other
// registers of the same lane directly. No block barrier.
template <class R>
__device__ __forceinline__ void warp_sort256(R (&v)[8]) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (int k = 2; k <= 256; k <<= 1) {
#pragma unroll
    for (int d = k >> 1; d > 0; d >>= 1) {
      if (d >= 32) {
        const int dj = d >> 5;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          if (j & dj) continue;
          const int jj = j | dj;
          const bool up = (((j << 5) | (int)lane) & k) == 0;
          const R a = v[j], b = v[jj];
          if ((a > b) == up) {
            v[j] = b;
            v[jj] = a;
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const R o = __shfl_xor_sync(0xffffffffu, v[j], d);
          const bool up = (((j << 5) | (int)lane) & k) == 0;
          const bool lower = (lane & (unsigned)d) == 0;
          const R lo = v[j] < o ? v[j] : o, hi = v[j] < o ? o : v[j];
          v[j] = (lower == up) ? lo : hi;
        }
      }
    }
  }
}

__device__ __forceinline__ int block_max_int(int v, int* red) {
  for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, d));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = red[0];
  for (int w = 1; w < kGrowWarps; w++) t = max(t, red[w]);
  __syncthreads();
  return t;
}

// Top edge of bin b (exodus_rescale.c:905-913).
template <class R>
__device__ __forceinline__ R bin_hi(const RungConstsT<R>& rc, int32_t b) {
  if (b == (int32_t)rc.nb - 1) return fmul(rc.rs2, R(1.0f + 1e-6f));
  return fadd(rc.rc2, fmul((R)(b + 1), rc.bin_w));
}

// Ascending bitonic sort of buf[0, p), p a power of two.
template <class R>
__device__ void bitonic_sort(R* buf, uint32_t p) {
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < p; i += kGrowT) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const R a = buf[i], b = buf[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// The cells of the template a warp walks, 32 at a time: `want(type, i)` says
// whether a cell's range is looked up, `whole(type, count)` (or
// `whole(type, count, flat)`, for a per-cell table) is then called on the
// lane holding it (for counts), `particles(type)` whether its particles
// are read, and `each(type, d2, p, i)` runs per particle read (i: its cell's
// template index). `visited` and `read` count the lookups and the particles.
template <class R, class Want, class Whole, class Particles, class Each>
__device__ __forceinline__ void walk_cells(const MeshViewT<R>& mesh, const TemplateViewT<R>& tpl,
                                           int32_t ci, int32_t cj, int32_t ck, R cx, R cy,
                                           R cz, Want want, Whole whole, Particles particles,
                                           Each each, unsigned long long& visited,
                                           unsigned long long& read, bool whole_warp = false) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // A CTA's warps share the template's chunks; a warp on its own takes all.
  const uint32_t first = whole_warp ? 0u : warp * 32;
  const uint32_t step = whole_warp ? 32u : kGrowWarps * 32;
  for (uint32_t c0 = first; c0 < tpl.count; c0 += step) {
    const uint32_t i = c0 + lane;
    CellRange<R> c{0, 0, 0.f, 0.f, 0.f, 0};
    uint8_t type = 0;
    bool need = false;
    if (i < tpl.count) {
      type = __ldg(tpl.type + i);
      if (want(type, i)) {
        c = query_cell(mesh, tpl, i, ci, cj, ck, cx, cy, cz);
        if constexpr (std::is_invocable_v<Whole, uint8_t, uint32_t, uint32_t>)
          whole(type, c.e - c.s, c.flat);
        else
          whole(type, c.e - c.s);
        need = c.e > c.s && particles(type);
        visited++;
      }
    }
    // The chunk's particles as one stream: each lane takes every 32nd item,
    // finds the cell it falls in by a binary search over the cells' starts
    // (shuffles), and keeps kWalkUnroll items' loads in flight.
    const uint32_t cnt = need ? c.e - c.s : 0u;
    uint32_t incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= (unsigned)d) incl += y;
    }
    const uint32_t start = incl - cnt;  // this lane's cell's first item
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (lane == 0) read += total;
    for (uint32_t base = 0; base < total; base += 32 * kWalkUnroll) {
      uint32_t pp[kWalkUnroll];
      int own[kWalkUnroll];
#pragma unroll
      for (int u = 0; u < kWalkUnroll; u++) {
        const uint32_t idx = base + (uint32_t)u * 32 + lane;
        // The last cell (lane) whose start is <= idx owns item idx (cells
        // without items share a start with the next one).
        int j = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const uint32_t st = __shfl_sync(0xffffffffu, start, j + step);
          if (st <= idx) j += step;
        }
        const uint32_t s_j = __shfl_sync(0xffffffffu, c.s, j);
        const uint32_t st_j = __shfl_sync(0xffffffffu, start, j);
        own[u] = j;
        pp[u] = idx < total ? s_j + (idx - st_j) : 0xffffffffu;
      }
      R px[kWalkUnroll], py[kWalkUnroll], pz[kWalkUnroll];
#pragma unroll
      for (int u = 0; u < kWalkUnroll; u++) {
        // Past the stream's end a lane loads particle 0 (there is one: the
        // stream is not empty) and drops it.
        const uint32_t q = pp[u] != 0xffffffffu ? pp[u] : 0u;
        if constexpr (sizeof(R) == 4) {
          if (mesh.xyzw) {
            const float4 v = __ldg(mesh.xyzw + q);
            px[u] = v.x;
            py[u] = v.y;
            pz[u] = v.z;
            continue;
          }
        }
        px[u] = __ldg(mesh.x + q);
        py[u] = __ldg(mesh.y + q);
        pz[u] = __ldg(mesh.z + q);
      }
#pragma unroll
      for (int u = 0; u < kWalkUnroll; u++) {
        const R qx = __shfl_sync(0xffffffffu, c.ex, own[u]);
        const R qy = __shfl_sync(0xffffffffu, c.ey, own[u]);
        const R qz = __shfl_sync(0xffffffffu, c.ez, own[u]);
        const uint8_t t = (uint8_t)__shfl_sync(0xffffffffu, (int)type, own[u]);
        if (pp[u] != 0xffffffffu)
          each(t, dist2(px[u], py[u], pz[u], qx, qy, qz), pp[u], c0 + (uint32_t)own[u]);
      }
    }
  }
}

// The next survivor for the calling warp (CTA) from a work counter zeroed
// before the launch: survivors go to whichever warp (CTA) is free, so a
// survivor that takes long delays only its own warp, not a fixed share of
// survivors behind it. A survivor's result does not depend on which warp
// takes it, or when.
__device__ __forceinline__ uint32_t next_warp_item(uint32_t* work) {
  uint32_t s = 0;
  if ((threadIdx.x & 31u) == 0) s = atomicAdd(work, 1u);
  return __shfl_sync(0xffffffffu, s, 0);
}

__device__ __forceinline__ uint32_t next_cta_item(uint32_t* work, uint32_t* slot) {
  if (threadIdx.x == 0) *slot = atomicAdd(work, 1u);
  __syncthreads();
  const uint32_t s = *slot;
  __syncthreads();
  return s;
}

// traffic[0] counts the particles whose positions a pass read (12 bytes
// each), traffic[1] the template cells a pass visited (a range lookup, 8
// bytes, plus the template entry, 8 bytes): the gathered bytes of the
// sphere growth.
template <class R>
__global__ void __launch_bounds__(kGrowT, 4) growth_kernel(MeshViewT<R> mesh, TemplateViewT<R> tpl,
                                                           RungConstsT<R> rc, SurvivorsT<R> sv,
                                                           R* __restrict__ gbuf, uint32_t gcap,
                                                           unsigned long long* __restrict__ traffic,
                                                           uint8_t only, uint32_t* work,
                                                           const uint32_t* __restrict__ list = nullptr,
                                                           const uint32_t* __restrict__ list_count = nullptr) {
  __shared__ uint32_t bins[kMaxBins];
  __shared__ uint32_t below[kMaxBins];  // particles inside bin b's lower edge
  __shared__ R sbuf[kSmemBuf];
  __shared__ unsigned long long red64[2 * kGrowWarps];
  __shared__ R found_d2;
  __shared__ int found_k;
  __shared__ int redi[kGrowWarps];
  __shared__ uint32_t collected;

  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t n_surv = *sv.count;
  R* my_gbuf = gbuf + (uint64_t)blockIdx.x * gcap;
  __shared__ uint32_t s_item;

  // With a list, only the survivors it names (the warp kernel's leftovers).
  const uint32_t n_items = list ? *list_count : n_surv;
  for (uint32_t k = next_cta_item(work, &s_item); k < n_items; k = next_cta_item(work, &s_item)) {
    const uint32_t s = list ? list[k] : k;
    if (only != kAllSurvivors ? sv.reason[s] != only : sv.reason[s] == kRescaleWitness) continue;
    const R cx = sv.cx[s], cy = sv.cy[s], cz = sv.cz[s];
    const int32_t ci = (int32_t)fmul(cx, mesh.inv_l), cj = (int32_t)fmul(cy, mesh.inv_l),
                  ck = (int32_t)fmul(cz, mesh.inv_l);
    uint8_t reason = kRescaleOk;
    R radius = -1.0f;
    unsigned long long read = 0, visited = 0;

    for (uint32_t b = threadIdx.x; b < rc.nb; b += kGrowT) bins[b] = 0;
    __syncthreads();

    // 1. Every cell: core and shell cells by their counts, the boundary
    //    cells particle by particle -- the early refusal's count
    //    (exodus_rescale.c:738-782) and their share of the histogram
    //    (794-865) from the same distances.
    unsigned long long within = 0, n_core = 0, n_shell = 0;
    walk_cells(
        mesh, tpl, ci, cj, ck, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
        [&](uint8_t type, uint32_t cnt) {
          if (type == kCellCore) {
            within += cnt;
            n_core += cnt;
          } else if (type == kCellShell) {
            within += cnt;
            n_shell += cnt;
          }
        },
        [](uint8_t type) { return type == kCellStraddle || type == kCellEdge; },
        [&](uint8_t, R d2, uint32_t, uint32_t) {
          if (d2 <= rc.rs2) within++;
          if (d2 <= rc.rc2) {
            n_core++;
          } else if (d2 <= rc.rs2) {
            atomicAdd(bins + bin_of(d2, rc.rc2, rc.inv_w, rc.nb), 1u);
            n_shell++;
          }
        },
        visited, read);
    within = block_sum_u64(within, red64);
    if (within == 0) {
      reason = kRescaleEmpty;
    } else if (fsub(fdiv(from_u64<R>(within), rc.expected), R(1.0f)) <= rc.threshold) {
      reason = kRescaleBeyondSearch;
    }

    if (reason == kRescaleOk) {
      // 2. The cells wholly inside the annulus, every particle binned.
      walk_cells(
          mesh, tpl, ci, cj, ck, cx, cy, cz,
          [](uint8_t type, uint32_t) { return type == kCellShell; }, [](uint8_t, uint32_t) {},
          [](uint8_t) { return true; },
          [&](uint8_t, R d2, uint32_t, uint32_t) {
            atomicAdd(bins + bin_of(d2, rc.rc2, rc.inv_w, rc.nb), 1u);
          },
          visited, read);
      block_sum2_u64(n_core, n_shell, red64);
      const unsigned long long total = n_core + n_shell;
      if (total == 0) {
        reason = kRescaleEmpty;
      } else if (fsub(fdiv(from_u64<R>(total), rc.expected), R(1.0f)) <= rc.threshold) {
        reason = kRescaleBeyondSearch;
      }
      if (reason == kRescaleOk) {
        // below[b] = core + bins < b: the interior count of bin b's skip test.
        if (warp == 0) {
          uint32_t carry = (uint32_t)n_core;
          for (uint32_t b0 = 0; b0 < rc.nb; b0 += 32) {
            const uint32_t b = b0 + lane;
            const uint32_t v = b < rc.nb ? bins[b] : 0u;
            uint32_t x = v;
            for (int d = 1; d < 32; d <<= 1) {
              const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
              if (lane >= (unsigned)d) x += y;
            }
            if (b < rc.nb) below[b] = carry + x - v;
            carry += __shfl_sync(0xffffffffu, x, 31);
          }
        }
        __syncthreads();

        // 3. The walk (exodus_rescale.c:914-1007): the highest bin its skip
        //    test does not rule out, resolved with the bins below it.
        int32_t cursor = (int32_t)rc.nb - 1;
        reason = kRescaleBelowRung;
        while (cursor >= 0) {
          int best = -1;
          for (int32_t b = threadIdx.x; b <= cursor; b += kGrowT) {
            if (bins[b] == 0) continue;
            const R hi = bin_hi(rc, b);
            const R nm = from_u32<R>(below[b]);
            if (!(fmul(nm, nm) > fmul(fmul(fmul(rc.K2, hi), hi), hi))) best = max(best, b);
          }
          best = block_max_int(best, redi);
          if (best < 0) break;
          const int32_t b_hi = best;
          int32_t b_lo = b_hi - (int32_t)rc.window + 1;
          if (b_lo < 0) b_lo = 0;
          const uint32_t top = below[b_hi] + bins[b_hi];
          while (b_lo < b_hi && top - below[b_lo] > kSmemBuf) b_lo++;
          const uint32_t want = top - below[b_lo];
          R* buf = sbuf;
          uint32_t cap = kSmemBuf;
          if (want > kSmemBuf) {
            buf = my_gbuf;
            cap = gcap;
          }
          if (want > cap) {
            reason = kRescaleOverflow;
            break;
          }
          const R lo = fadd(rc.rc2, fmul((R)b_lo, rc.bin_w));
          const R hi = bin_hi(rc, b_hi);
          if (threadIdx.x == 0) collected = 0;
          __syncthreads();
          walk_cells(
              mesh, tpl, ci, cj, ck, cx, cy, cz,
              [&](uint8_t type, uint32_t i) {
                return type != kCellCore && !(__ldg(tpl.max_d2 + i) < lo) &&
                       !(__ldg(tpl.min_d2 + i) > hi);
              },
              [](uint8_t, uint32_t) {}, [](uint8_t) { return true; },
              [&](uint8_t type, R d2, uint32_t, uint32_t) {
                if (type != kCellShell && !(d2 > rc.rc2 && d2 <= rc.rs2)) return;
                const uint32_t bi = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
                if (bi < (uint32_t)b_lo || bi > (uint32_t)b_hi) return;
                const uint32_t slot = atomicAdd(&collected, 1u);
                if (slot < cap) buf[slot] = d2;
              },
              visited, read);
          __syncthreads();
          const uint32_t m = collected < cap ? collected : cap;
          // Outside-in: the k-th smallest encloses top - m + k particles;
          // the answer is the largest k that passes (exodus_rescale.c:405-438).
          int found = -1;
          R found_val = 0;
          if (m <= 256) {
            // One warp sorts and tests the window in registers.
            if (warp == 0) {
              R v[8];
#pragma unroll
              for (int j = 0; j < 8; j++) {
                const uint32_t i = (uint32_t)j * 32 + lane;
                v[j] = i < m ? buf[i] : real_inf<R>();
              }
              warp_sort256(v);
              int f = -1;
              R fv = 0;
#pragma unroll
              for (int j = 0; j < 8; j++) {
                const uint32_t k = (uint32_t)j * 32 + lane;
                const R d2 = v[j];
                if (k < m && d2 != R(0)) {
                  const R rn = from_u32<R>(top - m + k);
                  const R d2c = fmul(fmul(d2, d2), d2);
                  if (fmul(rn, rn) <= fmul(rc.K2, d2c)) {
                    f = (int)k;
                    fv = d2;
                  }
                }
              }
              const int best_k = __reduce_max_sync(0xffffffffu, f + 1) - 1;
              if (best_k >= 0 && f == best_k) {
                found_k = best_k;
                found_d2 = fv;
              }
              if (lane == 0 && best_k < 0) found_k = -1;
            }
            __syncthreads();
            found = found_k;
            found_val = found_d2;
          } else {
            uint32_t p2 = 1;
            while (p2 < m) p2 <<= 1;
            for (uint32_t i = m + threadIdx.x; i < p2; i += kGrowT) buf[i] = real_inf<R>();
            __syncthreads();
            bitonic_sort(buf, p2);
            for (uint32_t k = threadIdx.x; k < m; k += kGrowT) {
              const R d2 = buf[k];
              if (d2 == 0.0f) continue;
              const R rn = from_u32<R>(top - m + k);
              const R d2c = fmul(fmul(d2, d2), d2);
              if (fmul(rn, rn) <= fmul(rc.K2, d2c)) found = max(found, (int)k);
            }
            found = block_max_int(found, redi);
            if (found >= 0) found_val = buf[found];
          }
          if (found >= 0) {
            radius = fsqrt(found_val);
            reason = kRescaleOk;
            break;
          }
          cursor = b_lo - 1;
          __syncthreads();
        }
      }
    }
    if (traffic) {
      // walk_cells counts particles on lane 0 and the cells each lane looked up.
      const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
      if (lane == 0) {
        if (read) atomicAdd(traffic, read);
        if (v) atomicAdd(traffic + 1, v);
      }
    }
    if (threadIdx.x == 0) {
      sv.r[s] = reason == kRescaleOk ? radius : -1.0f;
      sv.reason[s] = reason;
    }
    __syncthreads();
  }
}

// The same growth with a warp per survivor and no block barrier: the warp
// walks the whole template, keeps the survivor's histogram and prefix in its
// own slice of shared memory, and resolves windows of up to 256 distances in
// registers. A survivor whose window is wider is left kRescalePending for the
// per-CTA kernel. Every count, bin and test is the per-CTA kernel's, so the
// radius is the same bits.
//
// With shell_cap > 0 the warp also keeps, as the first two walks meet them,
// the distances of the particles the windows can collect -- the boundary
// cells' particles inside the shell and every particle of the shell cells --
// with their cells' template indices, up to shell_cap of them. A window then
// takes its distances from that list, with the walk's own cell test (the
// cell's bounds against the window) and bin test: the same distances as a
// walk over the cells, without reading a particle again. A survivor with
// more is resolved by walks, as without the list.
constexpr int kWarpSort = 256;

// Bytes of one warp's slice: bins, prefix, the window's distances, two
// counters (and padding), the shell list's distances and template indices.
template <class R>
__host__ __device__ constexpr size_t warp_slice_bytes(uint32_t nb_stride, uint32_t shell_cap) {
  return 2 * (size_t)nb_stride * sizeof(uint32_t) + kWarpSort * sizeof(R) + 16 +
         (size_t)shell_cap * (sizeof(R) + sizeof(uint32_t));
}

template <class R>
__global__ void __launch_bounds__(kGrowT, 4) growth_warp_kernel(MeshViewT<R> mesh,
                                                             TemplateViewT<R> tpl,
                                                             RungConstsT<R> rc, SurvivorsT<R> sv,
                                                             uint32_t nb_stride, uint32_t shell_cap,
                                                             uint8_t only,
                                                             unsigned long long* __restrict__ traffic,
                                                             uint32_t* work, uint32_t* __restrict__ pend) {
  extern __shared__ unsigned char warp_smem[];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  unsigned char* base = warp_smem + warp * warp_slice_bytes<R>(nb_stride, shell_cap);
  uint32_t* bins = (uint32_t*)base;
  uint32_t* below = bins + nb_stride;
  R* wbuf = (R*)(below + nb_stride);
  uint32_t* collected = (uint32_t*)(wbuf + kWarpSort);
  uint32_t* listed = collected + 1;  // entries offered to the shell list (may pass shell_cap)
  R* sd2 = (R*)(collected + 16 / sizeof(uint32_t));
  uint32_t* scell = (uint32_t*)(sd2 + shell_cap);
  // One entry of the shell list, for as long as there is room.
  auto keep = [&](R d2, uint32_t cell) {
    if (shell_cap == 0) return;
    const uint32_t slot = atomicAdd(listed, 1u);
    if (slot < shell_cap) {
      sd2[slot] = d2;
      scell[slot] = cell;
    }
  };
  const uint32_t n_surv = *sv.count;
  for (uint32_t s = next_warp_item(work); s < n_surv; s = next_warp_item(work)) {
    if (only != kAllSurvivors ? sv.reason[s] != only : sv.reason[s] == kRescaleWitness) continue;
    const R cx = sv.cx[s], cy = sv.cy[s], cz = sv.cz[s];
    const int32_t ci = (int32_t)fmul(cx, mesh.inv_l), cj = (int32_t)fmul(cy, mesh.inv_l),
                  ck = (int32_t)fmul(cz, mesh.inv_l);
    uint8_t reason = kRescaleOk;
    R radius = -1.0f;
    unsigned long long read = 0, visited = 0;
    for (uint32_t b = lane; b < rc.nb; b += 32) bins[b] = 0;
    if (lane == 0) *listed = 0;
    __syncwarp();
    // 1. Early refusal and the boundary cells' share of the histogram.
    unsigned long long within = 0, n_core = 0, n_shell = 0;
    walk_cells(
        mesh, tpl, ci, cj, ck, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
        [&](uint8_t type, uint32_t cnt) {
          if (type == kCellCore) {
            within += cnt;
            n_core += cnt;
          } else if (type == kCellShell) {
            within += cnt;
            n_shell += cnt;
          }
        },
        [](uint8_t type) { return type == kCellStraddle || type == kCellEdge; },
        [&](uint8_t, R d2, uint32_t, uint32_t cell) {
          if (d2 <= rc.rs2) within++;
          if (d2 <= rc.rc2) {
            n_core++;
          } else if (d2 <= rc.rs2) {
            atomicAdd(bins + bin_of(d2, rc.rc2, rc.inv_w, rc.nb), 1u);
            n_shell++;
            keep(d2, cell);
          }
        },
        visited, read, true);
    within = __reduce_add_sync(0xffffffffu, (unsigned)within);
    if (within == 0) {
      reason = kRescaleEmpty;
    } else if (fsub(fdiv(from_u64<R>(within), rc.expected), R(1.0f)) <= rc.threshold) {
      reason = kRescaleBeyondSearch;
    }
    if (reason == kRescaleOk) {
      // 2. The shell cells.
      walk_cells(
          mesh, tpl, ci, cj, ck, cx, cy, cz,
          [](uint8_t type, uint32_t) { return type == kCellShell; }, [](uint8_t, uint32_t) {},
          [](uint8_t) { return true; },
          [&](uint8_t, R d2, uint32_t, uint32_t cell) {
            atomicAdd(bins + bin_of(d2, rc.rc2, rc.inv_w, rc.nb), 1u);
            keep(d2, cell);
          },
          visited, read, true);
      n_core = __reduce_add_sync(0xffffffffu, (unsigned)n_core);
      n_shell = __reduce_add_sync(0xffffffffu, (unsigned)n_shell);
      const unsigned long long total = n_core + n_shell;
      if (total == 0) {
        reason = kRescaleEmpty;
      } else if (fsub(fdiv(from_u64<R>(total), rc.expected), R(1.0f)) <= rc.threshold) {
        reason = kRescaleBeyondSearch;
      }
      if (reason == kRescaleOk) {
        __syncwarp();
        uint32_t carry = (uint32_t)n_core;
        for (uint32_t b0 = 0; b0 < rc.nb; b0 += 32) {
          const uint32_t b = b0 + lane;
          const uint32_t v = b < rc.nb ? bins[b] : 0u;
          uint32_t x = v;
          for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= (unsigned)d) x += y;
          }
          if (b < rc.nb) below[b] = carry + x - v;
          carry += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        // 3. The walk and the resolution.
        int32_t cursor = (int32_t)rc.nb - 1;
        reason = kRescaleBelowRung;
        while (cursor >= 0) {
          int best = -1;
          for (int32_t b = lane; b <= cursor; b += 32) {
            if (bins[b] == 0) continue;
            const R hi = bin_hi(rc, b);
            const R nm = from_u32<R>(below[b]);
            if (!(fmul(nm, nm) > fmul(fmul(fmul(rc.K2, hi), hi), hi))) best = max(best, b);
          }
          best = __reduce_max_sync(0xffffffffu, best + 1) - 1;
          if (best < 0) break;
          const int32_t b_hi = best;
          int32_t b_lo = b_hi - (int32_t)rc.window + 1;
          if (b_lo < 0) b_lo = 0;
          const uint32_t top = below[b_hi] + bins[b_hi];
          while (b_lo < b_hi && top - below[b_lo] > (uint32_t)kWarpSort) b_lo++;
          if (top - below[b_lo] > (uint32_t)kWarpSort) {
            reason = kRescalePending;  // one bin wider than the registers hold
            break;
          }
          const R lo = fadd(rc.rc2, fmul((R)b_lo, rc.bin_w));
          const R hi = bin_hi(rc, b_hi);
          if (lane == 0) *collected = 0;
          __syncwarp();
          const uint32_t n_listed = *listed;
          if (shell_cap > 0 && n_listed <= shell_cap) {
            // From the shell list: its entries are the particles the walk
            // below reads and keeps (shell cells whole, the others' inside
            // the shell), so the same cell and bin tests leave the same set.
            for (uint32_t e = lane; e < n_listed; e += 32) {
              const uint32_t i = scell[e];
              if (__ldg(tpl.max_d2 + i) < lo || __ldg(tpl.min_d2 + i) > hi) continue;
              const R d2 = sd2[e];
              const uint32_t bi = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
              if (bi < (uint32_t)b_lo || bi > (uint32_t)b_hi) continue;
              const uint32_t slot = atomicAdd(collected, 1u);
              if (slot < (uint32_t)kWarpSort) wbuf[slot] = d2;
            }
          } else {
            walk_cells(
                mesh, tpl, ci, cj, ck, cx, cy, cz,
                [&](uint8_t type, uint32_t i) {
                  return type != kCellCore && !(__ldg(tpl.max_d2 + i) < lo) &&
                         !(__ldg(tpl.min_d2 + i) > hi);
                },
                [](uint8_t, uint32_t) {}, [](uint8_t) { return true; },
                [&](uint8_t type, R d2, uint32_t, uint32_t) {
                  if (type != kCellShell && !(d2 > rc.rc2 && d2 <= rc.rs2)) return;
                  const uint32_t bi = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
                  if (bi < (uint32_t)b_lo || bi > (uint32_t)b_hi) return;
                  const uint32_t slot = atomicAdd(collected, 1u);
                  if (slot < (uint32_t)kWarpSort) wbuf[slot] = d2;
                },
                visited, read, true);
          }
          __syncwarp();
          const uint32_t m = *collected;  // = top - below[b_lo] <= kWarpSort
          R v[8];
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const uint32_t i = (uint32_t)j * 32 + lane;
            v[j] = i < m ? wbuf[i] : real_inf<R>();
          }
          warp_sort256(v);
          int f = -1;
          R fv = 0;
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const uint32_t k = (uint32_t)j * 32 + lane;
            const R d2 = v[j];
            if (k < m && d2 != R(0)) {
              const R rn = from_u32<R>(top - m + k);
              const R d2c = fmul(fmul(d2, d2), d2);
              if (fmul(rn, rn) <= fmul(rc.K2, d2c)) {
                f = (int)k;
                fv = d2;
              }
            }
          }
          const int best_k = __reduce_max_sync(0xffffffffu, f + 1) - 1;
          if (best_k >= 0) {
            const int owner = best_k & 31;
            radius = fsqrt(__shfl_sync(0xffffffffu, fv, owner));
            reason = kRescaleOk;
            break;
          }
          cursor = b_lo - 1;
          __syncwarp();
        }
      }
    }
    if (traffic) {
      const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
      if (lane == 0) {
        if (read) atomicAdd(traffic, read);
        if (v) atomicAdd(traffic + 1, v);
      }
    }
    if (lane == 0) {
      sv.r[s] = reason == kRescaleOk ? radius : -1.0f;
      sv.reason[s] = reason;
      // A leftover for the per-CTA pass, listed (work[2] counts them).
      if (reason == kRescalePending && pend) pend[atomicAdd(work + 2, 1u)] = s;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// The collision witness
// ---------------------------------------------------------------------------
// One warp per survivor. First the collision radius rho: over the void-index
// cells within scale * (r_search + largest radius) of the centre, the
// smallest radius past which the survivor's sphere is certain to collide
// with an accepted void, in IEEE double as collision_radius computes it
// (exodus_finder.c:780-845; the separation padded by 1e-5 of the lengths).
// Then, where rho < r_search, the witness (exodus_rescale.c:1074-1167): the
// particles at or inside rho^2 (whole cells counted where their bounds clear
// rho^2 by the 1e-5 slack, the rest by distance) must satisfy the crossing
// test already, n^2 <= K^2 rho^6 (1 - 1e-5), with a particle beyond rho^2 in
// the search shell: the crossing then lies past rho and the commit would
// refuse the void. The reference walks the cells in order and stops early
// (past n_cap inside, or skipping cells wholly beyond rho^2 once one
// particle is); the warp counts every cell, which gives the same answer: n
// only grows, and a cell whose bound lies beyond rho^2 by the slack holds no
// particle at or inside it. Cells wholly beyond rho^2 are read only while no
// non-empty shell cell beyond it has been seen.
constexpr double kCollisionSlack = 1e-5;

template <class R>
__device__ __forceinline__ double collision_radius_warp(const VoidViewT<R>& v, R cx, R cy, R cz,
                                                         R r_hi, R f, R scale, R box) {
  const unsigned lane = threadIdx.x & 31u;
  if (v.n == 0) return CUDART_INF;
  const double L = (double)box, half = __dmul_rn(0.5, L), ff = (double)f, sc = (double)scale;
  const R reach = fmul(scale, fadd(r_hi, v.max_r));
  const R xs[3] = {cx, cy, cz};
  int32_t lo[3], span[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = (int32_t)ffloor(fmul(fsub(xs[a], reach), v.inv_cell));
    int32_t hi = (int32_t)ffloor(fmul(fadd(xs[a], reach), v.inv_cell));
    if (hi - lo[a] >= (int32_t)kVoidCells) {
      lo[a] = 0;
      hi = (int32_t)kVoidCells - 1;
    }
    span[a] = hi - lo[a] + 1;
  }
  const uint32_t cells = (uint32_t)(span[0] * span[1] * span[2]);
  // Only a void whose r* is below r_hi can decide anything (the caller
  // compares the result with r_hi), and r* grows with the separation: it
  // reaches r_hi at D0 = tot(r_hi) = r_hi + rj - f min(r_hi, rj), and D is at
  // least d / scale. A float separation past scale * D0 by 1e-4 of it and
  // 1e-5 of the box (far more than float rounding, of the positions too)
  // rules the void out before any double arithmetic;
  // the minimum over the rest is the same double whenever it is below r_hi.
  const float halff = 0.5f * (float)box, boxf = (float)box, rhf = (float)r_hi, ff32 = (float)f;
  const float scf = (float)scale;
  double best = CUDART_INF;
  for (uint32_t k = lane; k < cells; k += 32) {
    const int32_t a = lo[0] + (int32_t)(k / (uint32_t)(span[1] * span[2]));
    const int32_t b = lo[1] + (int32_t)((k / (uint32_t)span[2]) % (uint32_t)span[1]);
    const int32_t c = lo[2] + (int32_t)(k % (uint32_t)span[2]);
    const int32_t n = (int32_t)kVoidCells;
    const uint32_t cell = (uint32_t)(((((a % n) + n) % n) * n + (((b % n) + n) % n)) * n +
                                     (((c % n) + n) % n));
    for (uint32_t q = __ldg(v.start + cell); q < __ldg(v.start + cell + 1); q++) {
      const uint32_t i = __ldg(v.ids + q);
      {
        float ex = fabsf((float)cx - (float)v.cx[i]), ey = fabsf((float)cy - (float)v.cy[i]),
              ez = fabsf((float)cz - (float)v.cz[i]);
        ex = ex > halff ? boxf - ex : ex;
        ey = ey > halff ? boxf - ey : ey;
        ez = ez > halff ? boxf - ez : ez;
        const float rjf = (float)v.r[i];
        const float d0 = (rhf + rjf - ff32 * fminf(rhf, rjf)) * scf * 1.0001f + 1e-5f * boxf;
        if (ex * ex + ey * ey + ez * ez > d0 * d0) continue;
      }
      const double rj = (double)v.r[i];
      double dx = fabs(__dsub_rn((double)cx, (double)v.cx[i]));
      double dy = fabs(__dsub_rn((double)cy, (double)v.cy[i]));
      double dz = fabs(__dsub_rn((double)cz, (double)v.cz[i]));
      dx = dx > half ? __dsub_rn(L, dx) : dx;
      dy = dy > half ? __dsub_rn(L, dy) : dy;
      dz = dz > half ? __dsub_rn(L, dz) : dz;
      const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                            __dmul_rn(dz, dz)));
      const double pad = __dmul_rn(kCollisionSlack, __dadd_rn(__dadd_rn(L, (double)r_hi), rj));
      const double D = __ddiv_rn(__dadd_rn(d, pad), sc);
      double r_star;
      if (D <= rj)
        r_star = 0.0;
      else if (D <= __dmul_rn(__dsub_rn(2.0, ff), rj))
        r_star = __ddiv_rn(__dsub_rn(D, rj), __dsub_rn(1.0, ff));
      else
        r_star = __dsub_rn(D, __dmul_rn(__dsub_rn(1.0, ff), rj));
      best = r_star < best ? r_star : best;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, best, o);
    best = other < best ? other : best;
  }
  return best;
}

template <class R>
__global__ void __launch_bounds__(kGrowT) witness_kernel(MeshViewT<R> mesh, TemplateViewT<R> tpl,
                                                         RungConstsT<R> rc, SurvivorsT<R> sv,
                                                         VoidViewT<R> voids,
                                                         unsigned long long* __restrict__ traffic,
                                                         uint32_t* work) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t n_surv = *sv.count;
  const R slack_lo = R(1.0f - 1e-5f), slack_hi = R(1.0f + 1e-5f);
  for (uint32_t s = next_warp_item(work); s < n_surv; s = next_warp_item(work)) {
    const R cx = sv.cx[s], cy = sv.cy[s], cz = sv.cz[s];
    bool refused = false;
    unsigned long long read = 0, visited = 0;
    const double rho = collision_radius_warp(voids, cx, cy, cz, rc.r_search, rc.f, rc.scale, rc.box);
    if (rho < (double)rc.r_search) {
      R rho2 = (R)__dmul_rn(__dmul_rn(rho, rho), 1.0 + kCollisionSlack);
      if (rho2 < rc.rc2) rho2 = rc.rc2;
      if (rho2 < rc.rs2) {
        const R bound = fmul(fmul(rc.K2, fmul(fmul(rho2, rho2), rho2)), slack_lo);
        const double n_cap = __dadd_rn(__dsqrt_rn((double)bound), 2.0);
        const R whole_in = fmul(rho2, slack_lo), whole_out = fmul(rho2, slack_hi);
        const int32_t ci = (int32_t)fmul(cx, mesh.inv_l), cj = (int32_t)fmul(cy, mesh.inv_l),
                      ck = (int32_t)fmul(cz, mesh.inv_l);
        // Whole cells: inside rho^2, or non-empty shell cells beyond it.
        unsigned long long n = 0;
        bool beyond = false;
        for (uint32_t i = lane; i < tpl.count; i += 32) {
          const uint8_t type = __ldg(tpl.type + i);
          const bool in = type == kCellCore || !(__ldg(tpl.max_d2 + i) > whole_in);
          const bool out = type == kCellShell && __ldg(tpl.min_d2 + i) > whole_out;
          if (!in && !out) continue;
          const CellRange<R> c = query_cell(mesh, tpl, i, ci, cj, ck, cx, cy, cz);
          visited++;
          if (in)
            n += c.e - c.s;
          else if (c.e > c.s)
            beyond = true;
        }
        beyond = __any_sync(0xffffffffu, beyond);
        // n only grows: whole cells alone past n_cap already fail the test.
        const unsigned n_whole = __reduce_add_sync(0xffffffffu, (unsigned)n);
        if ((double)n_whole > n_cap) {
          if (traffic) {
            const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
            if (lane == 0 && v) atomicAdd(traffic + 1, v);
          }
          if (lane == 0) sv.reason[s] = kRescaleOk;
          __syncwarp();
          continue;
        }
        // The cells that need distances.
        walk_cells(
            mesh, tpl, ci, cj, ck, cx, cy, cz,
            [&](uint8_t type, uint32_t i) {
              if (type == kCellCore || !(__ldg(tpl.max_d2 + i) > whole_in)) return false;
              const bool far = __ldg(tpl.min_d2 + i) > whole_out;
              if (type == kCellShell && far) return false;
              return !(beyond && far);  // such a cell can only show what is already shown
            },
            [](uint8_t, uint32_t) {}, [](uint8_t) { return true; },
            [&](uint8_t type, R d2, uint32_t, uint32_t) {
              if (!(d2 > rho2))
                n++;
              else if (type == kCellShell || !(d2 > rc.rs2))
                beyond = true;
            },
            visited, read, true);
        n = __reduce_add_sync(0xffffffffu, (unsigned)n);
        beyond = __any_sync(0xffffffffu, beyond);
        const R rn = from_u64<R>(n);
        refused = beyond && !((double)n > n_cap) && !(fmul(rn, rn) > bound);
      }
    }
    if (traffic) {
      const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
      if (lane == 0) {
        if (read) atomicAdd(traffic, read);
        if (v) atomicAdd(traffic + 1, v);
      }
    }
    if (lane == 0) {
      sv.reason[s] = refused ? kRescaleWitness : kRescaleOk;
      if (refused) sv.r[s] = -1.0f;
    }
    __syncwarp();
  }
}

// Off unless switched on: at 512^3 it refuses about 1.5% of the survivors
// (2,340 of 155,497 a step) and costs 2.1 ms a step for 0.2 ms of growth it
// saves; the catalogue is the same either way.
static int g_witness = 0;
void set_witness(int on) { g_witness = on; }

template <class R>
void witness(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s,
             VoidViewT<R> voids, uint32_t max_survivors, unsigned long long* traffic,
             cudaStream_t st, KernelTimer* timer, uint32_t* work) {
  if (max_survivors == 0) return;
  if (!g_witness) {
    // Every survivor to be grown (kRescaleOk is 0).
    SIFG_CUDA(cudaMemsetAsync(s.reason, 0, max_survivors, st));
    return;
  }
  // As many CTAs as the GPU keeps resident (four an SM at 64 registers),
  // taking survivors from the counter.
  const uint32_t ctas_needed = (max_survivors + kGrowWarps - 1) / kGrowWarps;
  SIFG_CUDA(cudaMemsetAsync(work, 0, sizeof(uint32_t), st));
  if (timer) timer->begin(st);
  witness_kernel<R><<<std::min<uint32_t>(ctas_needed, 152u * 4u), kGrowT, 0, st>>>(
      mesh, tpl, rc, s, voids, traffic, work);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
}

static int g_growth_mode = 0;
void set_growth_mode(int mode) { g_growth_mode = mode; }
static int g_shell_list = -1;
void set_shell_list(int entries) { g_shell_list = entries; }

// A warp per survivor pays once survivors outnumber the CTAs the per-CTA
// kernel keeps resident several times over.
constexpr uint32_t kWarpGrowthMin = 2048;
constexpr uint32_t kShellListMax = 512;  // entries of a warp's shell list, at most (4 CTAs an SM)

template <class R>
void grow(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s, uint32_t max_survivors,
          R* gbuf, uint32_t gcap, unsigned long long* traffic, cudaStream_t st,
          KernelTimer* timer, uint8_t only, uint32_t* work, uint32_t* pend) {
  if (max_survivors == 0) return;
  // work[0] for the first launch, work[1] for the per-CTA pass after the
  // warp kernel, work[2] the warp kernel's leftovers listed in pend.
  SIFG_CUDA(cudaMemsetAsync(work, 0, 3 * sizeof(uint32_t), st));
  const bool by_warp = g_growth_mode == 2 || (g_growth_mode == 0 && max_survivors >= kWarpGrowthMin);
  const unsigned g = max_survivors < growth_grid() ? max_survivors : growth_grid();
  if (timer) timer->begin(st);
  if (by_warp) {
    const uint32_t nb_stride = (rc.nb + 31) & ~31u;
    // The shell list: room for the particles a shell of the mean density
    // holds (and 64), at most kShellListMax, where that shell holds at most
    // twice kShellListMax -- survivors sit in voids, and most of their shells
    // hold well under the mean; none for the larger spheres of the early
    // rungs, whose lists would overflow and only cost occupancy.
    const double rr = (double)rc.rc2 / (double)rc.rs2;
    const double shell = (double)rc.expected * (1.0 - rr * std::sqrt(rr));
    uint32_t shell_cap =
        shell <= 2.0 * kShellListMax
            ? std::min<uint32_t>(kShellListMax, ((uint32_t)shell + 64u + 31u) & ~31u)
            : 0u;
    if (g_shell_list >= 0)
      shell_cap = std::min<uint32_t>(kShellListMax, ((uint32_t)g_shell_list + 31u) & ~31u);
    const size_t smem = warp_slice_bytes<R>(nb_stride, shell_cap) * kGrowWarps;
    thread_local size_t attr_bytes = 0;  // the attribute is per thread's view of the function
    if (smem > attr_bytes) {
      SIFG_CUDA(cudaFuncSetAttribute(growth_warp_kernel<R>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr_bytes = smem;
    }
    int per_sm = 0;
    SIFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, growth_warp_kernel<R>, kGrowT, smem));
    const uint32_t warps_needed = (max_survivors + kGrowWarps - 1) / kGrowWarps;
    const uint32_t cap = 152u * (uint32_t)std::max(per_sm, 1);
    growth_warp_kernel<R><<<std::min(warps_needed, cap), kGrowT, smem, st>>>(mesh, tpl, rc, s,
                                                                            nb_stride, shell_cap,
                                                                            only, traffic, work, pend);
    SIFG_LAUNCH_CHECK();
    // The survivors whose windows were too wide for a warp: from the warp
    // kernel's list when there is one (a CTA taking every survivor in turn
    // to find the few left over cost a round trip each), else by their state.
    growth_kernel<<<g, kGrowT, 0, st>>>(mesh, tpl, rc, s, gbuf, gcap, traffic, kRescalePending,
                                        work + 1, pend, pend ? work + 2 : nullptr);
    SIFG_LAUNCH_CHECK();
  } else {
    growth_kernel<<<g, kGrowT, 0, st>>>(mesh, tpl, rc, s, gbuf, gcap, traffic, only, work);
    SIFG_LAUNCH_CHECK();
  }
  if (timer) timer->end(st);
}

// ---------------------------------------------------------------------------
// Weighted sphere growth (sif__exodus_find_radius_weighted,
// exodus_rescale.c:642-1037 with weighted set; resolve_bin 391-507).
//
// The same three stages as growth_kernel with every count a sum of weights:
// whole core and shell cells from the mesh's per-cell sums in the early
// refusal, whole core cells from them in the histogram, every other tracer by
// its own weight; the density tests against mass_factor (rc.expected and
// rc.K2 are built from it). The reference accumulates in double; here every
// weight is a fixed-point integer (MeshViewT::wscale), so each sum is exact
// and independent of the order the CTA adds in. Where the reference's double
// sums are exact -- its weights' smallest unit times 2^53 above the total,
// which the 63-bit sums here cover with room to spare -- the two agree bit
// for bit; only a mesh whose weights span more than that could differ, and
// then in the last bit of a sum. A window's tracers are sorted by distance
// with their weights and tested outside-in through suffix sums of the
// weights: the tracer at k encloses the window's top weight less everything
// from k up, as the reference's walk has it when it reaches k. Tracers at the
// same distance may sort in another order than the reference's quicksort
// puts them; the radius is the same (the group passes where its last tracer
// would, whose enclosed weight does not depend on the order).
// ---------------------------------------------------------------------------
constexpr uint32_t kWBuf = 1024;  // a window's pairs held in shared memory

template <class R>
__device__ __forceinline__ long long wfix(R w, R scale) {
  if constexpr (sizeof(R) == 4)
    return __float2ll_rn(__fmul_rn(w, scale));
  else
    return __double2ll_rn(__dmul_rn(w, scale));
}

// A weight sum as the reference's double accumulator holds it (exactly,
// while that sum is exact), then rounded to the form's precision as its
// (sif_real) casts do.
template <class R>
__device__ __forceinline__ R wreal(long long q, double winv) {
  return (R)__dmul_rn(__ll2double_rn(q), winv);
}

// Ascending bitonic sort of key[0, p) carrying val, p a power of two.
template <class R>
__device__ void bitonic_sort_pairs(R* key, long long* val, uint32_t p) {
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < p; i += kGrowT) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const R a = key[i], b = key[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            key[i] = b;
            key[l] = a;
            const long long t = val[i];
            val[i] = val[l];
            val[l] = t;
          }
        }
      }
      __syncthreads();
    }
  }
}

// v[k] = v[k] + v[k + 1] + ... + v[p - 1], in place, by the block: a
// contiguous chunk per thread, the chunks' totals combined by warp 0.
__device__ void suffix_sums(long long* v, uint32_t p, long long* tsum) {
  static_assert(kGrowT == 256, "warp 0 combines 8 chunk totals per lane");
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t per = (p + kGrowT - 1) / kGrowT;
  const uint32_t a = min(p, threadIdx.x * per), e = min(p, a + per);
  long long t = 0;
  for (uint32_t k = a; k < e; k++) t += v[k];
  tsum[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x < 32) {
    long long loc[8], ls = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      loc[j] = tsum[threadIdx.x * 8 + j];
      ls += loc[j];
    }
    long long incl = ls;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const long long y = __shfl_down_sync(0xffffffffu, incl, d);
      if (lane + d < 32) incl += y;
    }
    long long after = incl - ls;
#pragma unroll
    for (int j = 7; j >= 0; j--) {
      tsum[threadIdx.x * 8 + j] = after;
      after += loc[j];
    }
  }
  __syncthreads();
  long long run = tsum[threadIdx.x];  // everything past this thread's chunk
  for (uint32_t k = e; k > a; k--) {
    run += v[k - 1];
    v[k - 1] = run;
  }
  __syncthreads();
}

template <class R>
constexpr size_t weighted_smem_bytes() {
  return (2 * (size_t)kMaxBins + kWBuf) * sizeof(long long) + 2 * (size_t)kMaxBins * sizeof(uint32_t) +
         kWBuf * sizeof(R);
}

template <class R>
__global__ void __launch_bounds__(kGrowT) growth_weighted_kernel(
    MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> sv,
    R* __restrict__ gbuf, long long* __restrict__ gwbuf, uint32_t gcap,
    unsigned long long* __restrict__ traffic, uint8_t only, uint32_t* work) {
  extern __shared__ __align__(16) unsigned char wsm[];
  long long* bw = (long long*)wsm;           // weight per bin
  long long* belw = bw + kMaxBins;           // weight inside bin b's lower edge
  long long* pwv = belw + kMaxBins;          // a window's weights (then their suffix sums)
  uint32_t* bn = (uint32_t*)(pwv + kWBuf);   // tracers per bin (sizes the windows)
  uint32_t* beln = bn + kMaxBins;            // tracers in the bins below b
  R* pd2 = (R*)(beln + kMaxBins);            // a window's distances
  __shared__ unsigned long long red64[2 * kGrowWarps];
  __shared__ long long tsum[kGrowT];
  __shared__ int redi[kGrowWarps];
  __shared__ uint32_t collected;

  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t n_surv = *sv.count;
  const R ws = mesh.wscale;
  const double winv = mesh.winv;
  __shared__ uint32_t s_item;

  for (uint32_t s = next_cta_item(work, &s_item); s < n_surv; s = next_cta_item(work, &s_item)) {
    if (only != kAllSurvivors ? sv.reason[s] != only : sv.reason[s] == kRescaleWitness) continue;
    const R cx = sv.cx[s], cy = sv.cy[s], cz = sv.cz[s];
    const int32_t ci = (int32_t)fmul(cx, mesh.inv_l), cj = (int32_t)fmul(cy, mesh.inv_l),
                  ck = (int32_t)fmul(cz, mesh.inv_l);
    uint8_t reason = kRescaleOk;
    R radius = -1.0f;
    unsigned long long read = 0, visited = 0;

    for (uint32_t b = threadIdx.x; b < rc.nb; b += kGrowT) {
      bw[b] = 0;
      bn[b] = 0;
    }
    __syncthreads();

    // 1. The early refusal's weight (exodus_rescale.c:738-782) and the
    //    boundary cells' share of the histogram (794-865), from the same
    //    distances; whole core and shell cells from the per-cell sums.
    long long within = 0, core = 0, shell = 0;
    walk_cells(
        mesh, tpl, ci, cj, ck, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
        [&](uint8_t type, uint32_t cnt, uint32_t flat) {
          if (cnt == 0) return;  // an empty cell is skipped (query_cell)
          if (type == kCellCore) {
            const long long q = wfix(__ldg(mesh.cell_w + flat), ws);
            within += q;
            core += q;
          } else if (type == kCellShell) {
            within += wfix(__ldg(mesh.cell_w + flat), ws);
          }
        },
        [](uint8_t type) { return type == kCellStraddle || type == kCellEdge; },
        [&](uint8_t, R d2, uint32_t p, uint32_t) {
          const long long q = wfix(__ldg(mesh.w + p), ws);
          if (d2 <= rc.rs2) within += q;
          if (d2 <= rc.rc2) {
            core += q;
          } else if (d2 <= rc.rs2) {
            const uint32_t b = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
            atomicAdd((unsigned long long*)(bw + b), (unsigned long long)q);
            atomicAdd(bn + b, 1u);
            shell += q;
          }
        },
        visited, read);
    within = (long long)block_sum_u64((unsigned long long)within, red64);
    if (!(within > 0)) {
      reason = kRescaleEmpty;
    } else if (fsub(fdiv(wreal<R>(within, winv), rc.expected), R(1.0f)) <= rc.threshold) {
      reason = kRescaleBeyondSearch;
    }

    if (reason == kRescaleOk) {
      // 2. The shell cells, tracer by tracer.
      walk_cells(
          mesh, tpl, ci, cj, ck, cx, cy, cz,
          [](uint8_t type, uint32_t) { return type == kCellShell; }, [](uint8_t, uint32_t) {},
          [](uint8_t) { return true; },
          [&](uint8_t, R d2, uint32_t p, uint32_t) {
            const long long q = wfix(__ldg(mesh.w + p), ws);
            const uint32_t b = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
            atomicAdd((unsigned long long*)(bw + b), (unsigned long long)q);
            atomicAdd(bn + b, 1u);
            shell += q;
          },
          visited, read);
      unsigned long long uc = (unsigned long long)core, us = (unsigned long long)shell;
      block_sum2_u64(uc, us, red64);
      const long long total = (long long)uc + (long long)us;
      if (!(total > 0)) {
        reason = kRescaleEmpty;
      } else if (fsub(fdiv(wreal<R>(total, winv), rc.expected), R(1.0f)) <= rc.threshold) {
        reason = kRescaleBeyondSearch;
      }
      if (reason == kRescaleOk) {
        // belw[b]: the core and the bins below b -- total less the bins from
        // b up, the weight the skip test measures (914-957).
        if (warp == 0) {
          long long carry = (long long)uc;
          uint32_t carry_n = 0;
          for (uint32_t b0 = 0; b0 < rc.nb; b0 += 32) {
            const uint32_t b = b0 + lane;
            const long long v = b < rc.nb ? bw[b] : 0;
            const uint32_t vn = b < rc.nb ? bn[b] : 0u;
            long long x = v;
            uint32_t xn = vn;
            for (int d = 1; d < 32; d <<= 1) {
              const long long y = __shfl_up_sync(0xffffffffu, x, d);
              const uint32_t yn = __shfl_up_sync(0xffffffffu, xn, d);
              if (lane >= (unsigned)d) {
                x += y;
                xn += yn;
              }
            }
            if (b < rc.nb) {
              belw[b] = carry + x - v;
              beln[b] = carry_n + xn - vn;
            }
            carry += __shfl_sync(0xffffffffu, x, 31);
            carry_n += __shfl_sync(0xffffffffu, xn, 31);
          }
        }
        __syncthreads();

        // 3. The walk: the highest bin with weight that the skip test does
        //    not rule out, resolved with the bins below it.
        int32_t cursor = (int32_t)rc.nb - 1;
        reason = kRescaleBelowRung;
        while (cursor >= 0) {
          int best = -1;
          for (int32_t b = threadIdx.x; b <= cursor; b += kGrowT) {
            if (!(bw[b] > 0)) continue;  // no weight: skipped like an empty bin
            const R hi = bin_hi(rc, b);
            const R nm = wreal<R>(belw[b], winv);
            if (!(fmul(nm, nm) > fmul(fmul(fmul(rc.K2, hi), hi), hi))) best = max(best, b);
          }
          best = block_max_int(best, redi);
          if (best < 0) break;
          const int32_t b_hi = best;
          int32_t b_lo = b_hi - (int32_t)rc.window + 1;
          if (b_lo < 0) b_lo = 0;
          const uint32_t top_n = beln[b_hi] + bn[b_hi];
          while (b_lo < b_hi && top_n - beln[b_lo] > kWBuf) b_lo++;
          const uint32_t want = top_n - beln[b_lo];
          R* kb = pd2;
          long long* vb = pwv;
          uint32_t cap = kWBuf;
          if (want > kWBuf) {
            kb = gbuf + (uint64_t)blockIdx.x * gcap;
            vb = gwbuf + (uint64_t)blockIdx.x * gcap;
            cap = gcap;
          }
          if (want > cap) {
            reason = kRescaleOverflow;
            break;
          }
          const R lo = fadd(rc.rc2, fmul((R)b_lo, rc.bin_w));
          const R hi = bin_hi(rc, b_hi);
          if (threadIdx.x == 0) collected = 0;
          __syncthreads();
          walk_cells(
              mesh, tpl, ci, cj, ck, cx, cy, cz,
              [&](uint8_t type, uint32_t i) {
                return type != kCellCore && !(__ldg(tpl.max_d2 + i) < lo) &&
                       !(__ldg(tpl.min_d2 + i) > hi);
              },
              [](uint8_t, uint32_t) {}, [](uint8_t) { return true; },
              [&](uint8_t type, R d2, uint32_t p, uint32_t) {
                if (type != kCellShell && !(d2 > rc.rc2 && d2 <= rc.rs2)) return;
                const uint32_t bi = bin_of(d2, rc.rc2, rc.inv_w, rc.nb);
                if (bi < (uint32_t)b_lo || bi > (uint32_t)b_hi) return;
                const uint32_t slot = atomicAdd(&collected, 1u);
                if (slot < cap) {
                  kb[slot] = d2;
                  vb[slot] = wfix(__ldg(mesh.w + p), ws);
                }
              },
              visited, read);
          __syncthreads();
          const uint32_t m = collected < cap ? collected : cap;
          uint32_t p2 = 1;
          while (p2 < m) p2 <<= 1;
          for (uint32_t i = m + threadIdx.x; i < p2; i += kGrowT) {
            kb[i] = real_inf<R>();
            vb[i] = 0;
          }
          __syncthreads();
          bitonic_sort_pairs(kb, vb, p2);
          suffix_sums(vb, p2, tsum);
          // Outside-in (405-438): the tracer at k encloses the window's top
          // weight less its own and everything beyond it.
          const long long top_w = belw[b_hi] + bw[b_hi];
          int found = -1;
          for (uint32_t k = threadIdx.x; k < m; k += kGrowT) {
            const R d2 = kb[k];
            if (d2 == R(0)) continue;
            const R wi = wreal<R>(top_w - vb[k], winv);
            const R d2c = fmul(fmul(d2, d2), d2);
            if (fmul(wi, wi) <= fmul(rc.K2, d2c)) found = max(found, (int)k);
          }
          found = block_max_int(found, redi);
          if (found >= 0) {
            radius = fsqrt(kb[found]);
            reason = kRescaleOk;
            break;
          }
          cursor = b_lo - 1;
          __syncthreads();
        }
      }
    }
    if (traffic) {
      const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
      if (lane == 0) {
        if (read) atomicAdd(traffic, read);
        if (v) atomicAdd(traffic + 1, v);
      }
    }
    if (threadIdx.x == 0) {
      sv.r[s] = reason == kRescaleOk ? radius : -1.0f;
      sv.reason[s] = reason;
    }
    __syncthreads();
  }
}

template <class R>
void grow_weighted(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s,
                   uint32_t max_survivors, R* gbuf, long long* gwbuf, uint32_t gcap,
                   unsigned long long* traffic, cudaStream_t st, KernelTimer* timer, uint8_t only,
                   uint32_t* work) {
  if (max_survivors == 0) return;
  SIFG_CUDA(cudaMemsetAsync(work, 0, sizeof(uint32_t), st));
  constexpr size_t smem = weighted_smem_bytes<R>();
  thread_local bool attr = false;  // the attribute is per thread's view of the function
  if (!attr) {
    SIFG_CUDA(cudaFuncSetAttribute(growth_weighted_kernel<R>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const unsigned g = max_survivors < growth_grid() ? max_survivors : growth_grid();
  if (timer) timer->begin(st);
  growth_weighted_kernel<R><<<g, kGrowT, smem, st>>>(mesh, tpl, rc, s, gbuf, gwbuf, gcap, traffic,
                                                    only, work);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
}

// ---------------------------------------------------------------------------
// Survey sphere growth (sif__exodus_find_radius_survey, exodus_rescale.c:
// 2154-2317; survey_sphere_total 1957-1993, survey_histogram 2000-2056,
// survey_resolve 2058-2146).
//
// The largest data distance d at which the data weight inside d is at most K
// times the random weight inside it, K = (1 + threshold) alpha: the data and
// the randoms each on its own mesh and template, both in the fixed point of
// the weighted growth (a mesh without weights counts each tracer 1). One CTA
// per survivor: the two sphere totals (the cheap refusal), the bin count from
// the data's tracers, the two histograms, then the walk down the bins with
// the skip test, resolving a window of bins at a time: its data tracers
// sorted by distance with their weights, each tested against the data weight
// it encloses (the window's top less the suffix sum of the weights from it
// up) and the random weight interpolated at its distance inside its bin, in
// the reference's double expression. Every sum is exact, so the bins below
// each edge stand for the reference's running r_below and d_current wherever
// its double sums are exact.
// ---------------------------------------------------------------------------
template <class R>
constexpr size_t survey_smem_bytes() {
  return (4 * (size_t)kMaxBins + kWBuf) * sizeof(long long) + 2 * (size_t)kMaxBins * sizeof(uint32_t) +
         kWBuf * sizeof(R);
}

// A tracer's or a whole cell's weight in the mesh's fixed point: its own
// weight, or 1 a tracer where the mesh has none.
template <class R>
__device__ __forceinline__ long long tracer_w(const MeshViewT<R>& m, uint32_t p) {
  return m.w ? wfix(__ldg(m.w + p), m.wscale) : 1ll;
}
template <class R>
__device__ __forceinline__ long long cell_wt(const MeshViewT<R>& m, uint32_t flat, uint32_t cnt) {
  return m.cell_w ? wfix(__ldg(m.cell_w + flat), m.wscale) : (long long)cnt;
}

template <class R>
__global__ void __launch_bounds__(kGrowT) growth_survey_kernel(
    MeshViewT<R> dm, TemplateViewT<R> dt, MeshViewT<R> rm, TemplateViewT<R> rt, RungConstsT<R> rc,
    R K, SurvivorsT<R> sv, R* __restrict__ gbuf, long long* __restrict__ gwbuf, uint32_t gcap,
    unsigned long long* __restrict__ traffic, uint32_t* work) {
  extern __shared__ __align__(16) unsigned char ssm[];
  long long* dbin = (long long*)ssm;       // data weight per bin
  long long* rbin = dbin + kMaxBins;       // random weight per bin
  long long* dbel = rbin + kMaxBins;       // data weight inside bin b's lower edge
  long long* rbel = dbel + kMaxBins;       // random weight inside it
  long long* pwv = rbel + kMaxBins;        // a window's weights (then their suffix sums)
  uint32_t* bn = (uint32_t*)(pwv + kWBuf);  // data tracers per bin (sizes the windows)
  uint32_t* beln = bn + kMaxBins;           // data tracers in the bins below b
  R* pd2 = (R*)(beln + kMaxBins);           // a window's distances
  __shared__ unsigned long long red64[2 * kGrowWarps];
  __shared__ long long tsum[kGrowT];
  __shared__ int redi[kGrowWarps];
  __shared__ uint32_t collected;
  __shared__ uint32_t s_item;

  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t n_surv = *sv.count;
  const double dinv = dm.winv, rinv = rm.winv;
  const R rs2 = rc.rs2, rc2 = rc.rc2, span = fsub(rs2, rc2);
  // exodus_rescale.c:2192-2204, the same for every survivor of the rung but
  // its tracer count.
  const R core_fraction = fdiv(fmul(fmul(rc.rmin, rc.rmin), rc.rmin),
                               fmul(fmul(rc.r_search, rc.r_search), rc.r_search));

  for (uint32_t s = next_cta_item(work, &s_item); s < n_surv; s = next_cta_item(work, &s_item)) {
    const R cx = sv.cx[s], cy = sv.cy[s], cz = sv.cz[s];
    const int32_t di = (int32_t)fmul(cx, dm.inv_l), dj = (int32_t)fmul(cy, dm.inv_l),
                  dk = (int32_t)fmul(cz, dm.inv_l);
    const int32_t ri_ = (int32_t)fmul(cx, rm.inv_l), rj = (int32_t)fmul(cy, rm.inv_l),
                  rk = (int32_t)fmul(cz, rm.inv_l);
    uint8_t reason = kRescaleOk;
    R radius = -1.0f;
    unsigned long long read = 0, visited = 0;

    // 1. The weight inside r_search on both meshes, and the data's tracers.
    long long dw = 0, rw = 0;
    unsigned long long dn = 0;
    walk_cells(
        dm, dt, di, dj, dk, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
        [&](uint8_t type, uint32_t cnt, uint32_t flat) {
          if (cnt == 0 || !(type == kCellCore || type == kCellShell)) return;
          dw += cell_wt(dm, flat, cnt);
          dn += cnt;
        },
        [](uint8_t type) { return type == kCellStraddle || type == kCellEdge; },
        [&](uint8_t, R d2, uint32_t p, uint32_t) {
          if (d2 <= rs2) {
            dw += tracer_w(dm, p);
            dn++;
          }
        },
        visited, read);
    walk_cells(
        rm, rt, ri_, rj, rk, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
        [&](uint8_t type, uint32_t cnt, uint32_t flat) {
          if (cnt == 0 || !(type == kCellCore || type == kCellShell)) return;
          rw += cell_wt(rm, flat, cnt);
        },
        [](uint8_t type) { return type == kCellStraddle || type == kCellEdge; },
        [&](uint8_t, R d2, uint32_t p, uint32_t) {
          if (d2 <= rs2) rw += tracer_w(rm, p);
        },
        visited, read);
    unsigned long long udw = (unsigned long long)dw, urw = (unsigned long long)rw;
    block_sum2_u64(udw, urw, red64);
    dn = block_sum_u64(dn, red64);
    if (!((long long)urw > 0)) {
      reason = kRescaleNoRandoms;
    } else if (wreal<R>((long long)udw, dinv) <= fmul(K, wreal<R>((long long)urw, rinv))) {
      reason = kRescaleBeyondSearch;
    }

    if (reason == kRescaleOk) {
      // 2. The bins, sized by the data's tracers, and both histograms.
      uint32_t nb = kMaxBins;
      {
        const R want = fdiv(fmul((R)dn, fsub(R(1.0f), core_fraction)), R(16.0f));
        if (!(want >= R(64.0f)))
          nb = 64u;
        else if (want < R(2048.0f))
          nb = (uint32_t)want;
      }
      const R inv_w = fdiv((R)nb, span), bin_w = fdiv(span, (R)nb);
      for (uint32_t b = threadIdx.x; b < nb; b += kGrowT) {
        dbin[b] = 0;
        rbin[b] = 0;
        bn[b] = 0;
      }
      __syncthreads();
      long long dcore = 0, dshell = 0, rcore = 0, rshell = 0;
      walk_cells(
          dm, dt, di, dj, dk, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
          [&](uint8_t type, uint32_t cnt, uint32_t flat) {
            if (cnt && type == kCellCore) dcore += cell_wt(dm, flat, cnt);
          },
          [](uint8_t type) { return type != kCellCore; },
          [&](uint8_t type, R d2, uint32_t p, uint32_t) {
            const long long q = tracer_w(dm, p);
            if (type != kCellShell && d2 <= rc2) {
              dcore += q;
            } else if (type == kCellShell || d2 <= rs2) {
              const uint32_t b = bin_of(d2, rc2, inv_w, nb);
              atomicAdd((unsigned long long*)(dbin + b), (unsigned long long)q);
              atomicAdd(bn + b, 1u);
              dshell += q;
            }
          },
          visited, read);
      walk_cells(
          rm, rt, ri_, rj, rk, cx, cy, cz, [](uint8_t, uint32_t) { return true; },
          [&](uint8_t type, uint32_t cnt, uint32_t flat) {
            if (cnt && type == kCellCore) rcore += cell_wt(rm, flat, cnt);
          },
          [](uint8_t type) { return type != kCellCore; },
          [&](uint8_t type, R d2, uint32_t p, uint32_t) {
            const long long q = tracer_w(rm, p);
            if (type != kCellShell && d2 <= rc2) {
              rcore += q;
            } else if (type == kCellShell || d2 <= rs2) {
              atomicAdd((unsigned long long*)(rbin + bin_of(d2, rc2, inv_w, nb)),
                        (unsigned long long)q);
              rshell += q;
            }
          },
          visited, read);
      unsigned long long ua = (unsigned long long)dcore, ub = (unsigned long long)dshell;
      block_sum2_u64(ua, ub, red64);
      const long long d_core = (long long)ua, d_total = (long long)ua + (long long)ub;
      ua = (unsigned long long)rcore;
      ub = (unsigned long long)rshell;
      block_sum2_u64(ua, ub, red64);
      const long long r_core = (long long)ua, r_total = (long long)ua + (long long)ub;
      // The backstops (2226-2237).
      if (!(r_total > 0)) {
        reason = kRescaleNoRandoms;
      } else if (wreal<R>(d_total, dinv) <= fmul(K, wreal<R>(r_total, rinv))) {
        reason = kRescaleBeyondSearch;
      }
      if (reason == kRescaleOk) {
        // Below each bin's lower edge: the core and the bins under it.
        if (warp == 0) {
          long long cd = d_core, cr = r_core;
          uint32_t cn = 0;
          for (uint32_t b0 = 0; b0 < nb; b0 += 32) {
            const uint32_t b = b0 + lane;
            const long long vd = b < nb ? dbin[b] : 0, vr = b < nb ? rbin[b] : 0;
            const uint32_t vn = b < nb ? bn[b] : 0u;
            long long xd = vd, xr = vr;
            uint32_t xn = vn;
            for (int d = 1; d < 32; d <<= 1) {
              const long long yd = __shfl_up_sync(0xffffffffu, xd, d);
              const long long yr = __shfl_up_sync(0xffffffffu, xr, d);
              const uint32_t yn = __shfl_up_sync(0xffffffffu, xn, d);
              if (lane >= (unsigned)d) {
                xd += yd;
                xr += yr;
                xn += yn;
              }
            }
            if (b < nb) {
              dbel[b] = cd + xd - vd;
              rbel[b] = cr + xr - vr;
              beln[b] = cn + xn - vn;
            }
            cd += __shfl_sync(0xffffffffu, xd, 31);
            cr += __shfl_sync(0xffffffffu, xr, 31);
            cn += __shfl_sync(0xffffffffu, xn, 31);
          }
        }
        __syncthreads();

        // 3. The walk (2239-2312): the highest bin with data weight whose
        //    skip test fails -- the least data a tracer in it could enclose
        //    against the most randoms, everything to the bin's top -- then
        //    its window resolved.
        int32_t cursor = (int32_t)nb - 1;
        reason = kRescaleBelowRung;
        while (cursor >= 0) {
          int best = -1;
          for (int32_t b = threadIdx.x; b <= cursor; b += kGrowT) {
            if (!(dbin[b] > 0)) continue;
            const R d_in_min = wreal<R>(dbel[b], dinv);
            const R r_in_max = wreal<R>(rbel[b] + rbin[b], rinv);
            if (!(r_in_max > R(0.0f)) || d_in_min > fmul(K, r_in_max)) continue;
            best = max(best, b);
          }
          best = block_max_int(best, redi);
          if (best < 0) break;
          const int32_t b_hi = best;
          int32_t b_lo = b_hi - (int32_t)rc.window + 1;
          if (b_lo < 0) b_lo = 0;
          const uint32_t top_n = beln[b_hi] + bn[b_hi];
          while (b_lo < b_hi && top_n - beln[b_lo] > kWBuf) b_lo++;
          const uint32_t want = top_n - beln[b_lo];
          R* kb = pd2;
          long long* vb = pwv;
          uint32_t cap = kWBuf;
          if (want > kWBuf) {
            kb = gbuf + (uint64_t)blockIdx.x * gcap;
            vb = gwbuf + (uint64_t)blockIdx.x * gcap;
            cap = gcap;
          }
          if (want > cap) {
            reason = kRescaleOverflow;
            break;
          }
          const R lo = fadd(rc2, fmul((R)b_lo, bin_w));
          const R hi = b_hi == (int32_t)nb - 1 ? fmul(rs2, R(1.0f + 1e-6f))
                                               : fadd(rc2, fmul((R)(b_hi + 1), bin_w));
          if (threadIdx.x == 0) collected = 0;
          __syncthreads();
          walk_cells(
              dm, dt, di, dj, dk, cx, cy, cz,
              [&](uint8_t type, uint32_t i) {
                return type != kCellCore && !(__ldg(dt.max_d2 + i) < lo) &&
                       !(__ldg(dt.min_d2 + i) > hi);
              },
              [](uint8_t, uint32_t) {}, [](uint8_t) { return true; },
              [&](uint8_t type, R d2, uint32_t p, uint32_t) {
                if (type != kCellShell && !(d2 > rc2 && d2 <= rs2)) return;
                const uint32_t bi = bin_of(d2, rc2, inv_w, nb);
                if (bi < (uint32_t)b_lo || bi > (uint32_t)b_hi) return;
                const uint32_t slot = atomicAdd(&collected, 1u);
                if (slot < cap) {
                  kb[slot] = d2;
                  vb[slot] = tracer_w(dm, p);
                }
              },
              visited, read);
          __syncthreads();
          const uint32_t m = collected < cap ? collected : cap;
          uint32_t p2 = 1;
          while (p2 < m) p2 <<= 1;
          for (uint32_t i = m + threadIdx.x; i < p2; i += kGrowT) {
            kb[i] = real_inf<R>();
            vb[i] = 0;
          }
          __syncthreads();
          bitonic_sort_pairs(kb, vb, p2);
          suffix_sums(vb, p2, tsum);
          // Outside-in: the tracer at k encloses the data to the window's
          // top less its own weight and everything beyond it, against the
          // randoms below its bin's lower edge and the share of its bin's
          // randoms up to it.
          const long long d_top = dbel[b_hi] + dbin[b_hi];
          int found = -1;
          for (uint32_t k = threadIdx.x; k < m; k += kGrowT) {
            const R d2 = kb[k];
            if (d2 == R(0)) continue;
            const uint32_t bi = bin_of(d2, rc2, inv_w, nb);
            R frac = fmul(fsub(d2, fadd(rc2, fmul((R)bi, bin_w))), inv_w);
            frac = frac < R(0.0f) ? R(0.0f) : (frac > R(1.0f) ? R(1.0f) : frac);
            const double rb = __dmul_rn(__ll2double_rn(rbel[bi]), rinv);
            const double rn = __dmul_rn(__ll2double_rn(rbin[bi]), rinv);
            const R r_in = (R)__dadd_rn(rb, __dmul_rn(rn, (double)frac));
            const R d_in = wreal<R>(d_top - vb[k], dinv);
            if (r_in > R(0.0f) && d_in <= fmul(K, r_in)) found = max(found, (int)k);
          }
          found = block_max_int(found, redi);
          if (found >= 0) {
            radius = fsqrt(kb[found]);
            reason = kRescaleOk;
            break;
          }
          cursor = b_lo - 1;
          __syncthreads();
        }
      }
    }
    if (traffic) {
      const unsigned long long v = __reduce_add_sync(0xffffffffu, (unsigned)visited);
      if (lane == 0) {
        if (read) atomicAdd(traffic, read);
        if (v) atomicAdd(traffic + 1, v);
      }
    }
    if (threadIdx.x == 0) {
      sv.r[s] = reason == kRescaleOk ? radius : -1.0f;
      sv.reason[s] = reason;
    }
    __syncthreads();
  }
}

template <class R>
void grow_survey(MeshViewT<R> dm, TemplateViewT<R> dt, MeshViewT<R> rm, TemplateViewT<R> rt,
                 RungConstsT<R> rc, R K, SurvivorsT<R> s, uint32_t max_survivors, R* gbuf,
                 long long* gwbuf, uint32_t gcap, unsigned long long* traffic, cudaStream_t st,
                 KernelTimer* timer, uint32_t* work) {
  if (max_survivors == 0) return;
  SIFG_CUDA(cudaMemsetAsync(work, 0, sizeof(uint32_t), st));
  constexpr size_t smem = survey_smem_bytes<R>();
  thread_local bool attr = false;  // the attribute is per thread's view of the function
  if (!attr) {
    SIFG_CUDA(cudaFuncSetAttribute(growth_survey_kernel<R>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const unsigned g = max_survivors < growth_grid() ? max_survivors : growth_grid();
  if (timer) timer->begin(st);
  growth_survey_kernel<R><<<g, kGrowT, smem, st>>>(dm, dt, rm, rt, rc, K, s, gbuf, gwbuf, gcap,
                                                  traffic, work);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
}

// sif__exodus_check_weights (exodus_finder.c:1039-1106): by the bits, so a
// NaN or an infinity is caught whatever the compiler assumes; a negative
// zero is a zero.
template <class R>
__global__ void check_weights_kernel(const R* __restrict__ w, uint64_t n,
                                     unsigned long long* __restrict__ counts) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned neg = 0, bad = 0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    if constexpr (sizeof(R) == 4) {
      const uint32_t b = __float_as_uint(w[p]);
      bad += ((b >> 23) & 0xffu) == 0xffu;
      neg += ((b >> 23) & 0xffu) != 0xffu && (b >> 31) && (b << 1);
    } else {
      const uint64_t b = (uint64_t)__double_as_longlong(w[p]);
      bad += ((b >> 52) & 0x7ffu) == 0x7ffu;
      neg += ((b >> 52) & 0x7ffu) != 0x7ffu && (b >> 63) && (b << 1);
    }
  }
  neg = __reduce_add_sync(0xffffffffu, neg);
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31u) == 0) {
    if (neg) atomicAdd(counts, (unsigned long long)neg);
    if (bad) atomicAdd(counts + 1, (unsigned long long)bad);
  }
}

template <class R>
void check_weights(const R* w, uint64_t n, unsigned long long* counts, cudaStream_t st) {
  SIFG_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), st));
  check_weights_kernel<R><<<grid_for(n, 256, 152u * 16u), 256, 0, st>>>(w, n, counts);
  SIFG_LAUNCH_CHECK();
}

void weight_fixed_point(double bound, double* wscale, double* winv) {
  int e = 0;
  std::frexp(bound > 0.0 ? bound : 1.0, &e);  // bound < 2^e
  const int s = std::min(100, std::max(-100, 58 - e));
  *wscale = std::ldexp(1.0, s);
  *winv = std::ldexp(1.0, -s);
}

template void grow_survey<float>(MeshViewT<float>, TemplateViewT<float>, MeshViewT<float>,
                                 TemplateViewT<float>, RungConstsT<float>, float, SurvivorsT<float>,
                                 uint32_t, float*, long long*, uint32_t, unsigned long long*,
                                 cudaStream_t, KernelTimer*, uint32_t*);
template void grow_survey<double>(MeshViewT<double>, TemplateViewT<double>, MeshViewT<double>,
                                  TemplateViewT<double>, RungConstsT<double>, double,
                                  SurvivorsT<double>, uint32_t, double*, long long*, uint32_t,
                                  unsigned long long*, cudaStream_t, KernelTimer*, uint32_t*);
template void grow_weighted<float>(MeshViewT<float>, TemplateViewT<float>, RungConstsT<float>,
                                   SurvivorsT<float>, uint32_t, float*, long long*, uint32_t,
                                   unsigned long long*, cudaStream_t, KernelTimer*, uint8_t,
                                   uint32_t*);
template void grow_weighted<double>(MeshViewT<double>, TemplateViewT<double>, RungConstsT<double>,
                                    SurvivorsT<double>, uint32_t, double*, long long*, uint32_t,
                                    unsigned long long*, cudaStream_t, KernelTimer*, uint8_t,
                                    uint32_t*);
template void check_weights<float>(const float*, uint64_t, unsigned long long*, cudaStream_t);
template void check_weights<double>(const double*, uint64_t, unsigned long long*, cudaStream_t);

// ---------------------------------------------------------------------------
// Survivor hash
// ---------------------------------------------------------------------------

template <class R>
__device__ __forceinline__ int32_t hash_axis(R c, R inv, int32_t ng) {
  int32_t i = (int32_t)fmul(c, inv);
  return i < 0 ? 0 : (i >= ng ? ng - 1 : i);
}

template <class R>
__global__ void sgrid_count_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                   const R* __restrict__ z, const uint32_t* __restrict__ cnt,
                                   int32_t ng, R inv, uint32_t* __restrict__ counts,
                                   uint32_t* __restrict__ cell_of) {
  const uint32_t n = *cnt;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t c = ((uint32_t)hash_axis(x[i], inv, ng) * ng + hash_axis(y[i], inv, ng)) * ng +
                       hash_axis(z[i], inv, ng);
    cell_of[i] = c;
    atomicAdd(counts + c, 1u);
  }
}

__global__ void scatter_ids_kernel(const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ cnt,
                                   uint32_t fixed_n, uint32_t* __restrict__ cursor,
                                   uint32_t* __restrict__ ids) {
  const uint32_t n = cnt ? *cnt : fixed_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    ids[atomicAdd(cursor + cell_of[i], 1u)] = i;
}

template <class R>
__global__ void scatter_survivors_kernel(const uint32_t* __restrict__ cell_of,
                                         const uint32_t* __restrict__ cnt,
                                         uint32_t* __restrict__ cursor, uint32_t* __restrict__ ids,
                                         const R* __restrict__ x, const R* __restrict__ y,
                                         const R* __restrict__ z, const R* __restrict__ r,
                                         SurvPackT<R>* __restrict__ pack) {
  const uint32_t n = *cnt;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t k = atomicAdd(cursor + cell_of[i], 1u);
    ids[k] = i;
    pack[k] = SurvPackT<R>{x[i], y[i], z[i], r[i]};
  }
}

template <class R>
__global__ void survivor_ranks_kernel(SurvivorsT<R> sv, const uint32_t* __restrict__ rank,
                                      const uint32_t* __restrict__ ids,
                                      uint32_t* __restrict__ hrank) {
  const uint32_t n = *sv.count;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    hrank[k] = rank[sv.cand[ids[k]]];
}

template <class R>
void survivor_grid_ranks(SurvivorsT<R> s, const uint32_t* rank, const uint32_t* ids,
                         uint32_t* hrank, uint32_t max_survivors, cudaStream_t st) {
  if (max_survivors == 0) return;
  survivor_ranks_kernel<R><<<grid_for(max_survivors, 256), 256, 0, st>>>(s, rank, ids, hrank);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void build_survivor_grid(const R* scx, const R* scy, const R* scz, const R* sr,
                         const uint32_t* d_count, uint32_t max_survivors, int32_t ng, R box,
                         uint32_t* start, uint32_t* ids, uint32_t* cell_of, SurvPackT<R>* pack,
                         cudaStream_t st) {
  const uint32_t cells = (uint32_t)(ng * ng * ng);
  SIFG_CUDA(cudaMemsetAsync(start, 0, (cells + 1) * sizeof(uint32_t), st));
  if (max_survivors == 0) return;
  const R inv = (R)ng / box;
  sgrid_count_kernel<<<grid_for(max_survivors, 256), 256, 0, st>>>(scx, scy, scz, d_count, ng, inv,
                                                                   start, cell_of);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_u32(start, cells + 1, st);
  thread_local DevBuf cursor;  // one per host thread driving a stream
  uint32_t* cur = (uint32_t*)cursor.ensure((cells + 1) * sizeof(uint32_t));
  SIFG_CUDA(cudaMemcpyAsync(cur, start, (cells + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  scatter_survivors_kernel<R><<<grid_for(max_survivors, 256), 256, 0, st>>>(
      cell_of, d_count, cur, ids, scx, scy, scz, sr, pack);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Commit rounds
// ---------------------------------------------------------------------------

// The largest accepted radius: positive values order as their bit patterns.
__device__ __forceinline__ void store_rmax(uint32_t* counters, float r) {
  atomicMax((int*)(counters + 3), __float_as_int(r));
}
__device__ __forceinline__ void store_rmax(uint32_t* counters, double r) {
  atomicMax((unsigned long long*)(counters + 6), (unsigned long long)__double_as_longlong(r));
}

// Two survivors can interact -- one's acceptance change the other's fate --
// only if their centres are closer than the largest distance any of the
// commit's tests reaches: the mask and pole probes reach scale * (r_i + r_j)
// plus a cell, the overlap scale * (r_i + r_j); two cells of slack cover
// every rounding.
template <class R>
__device__ __forceinline__ bool interacts(R ax, R ay, R az, R ar, R bx,
                                          R by, R bz, R br, const RungConstsT<R>& rc) {
  const R half = 0.5f * rc.box;
  R dx = fabs_(ax - bx), dy = fabs_(ay - by), dz = fabs_(az - bz);
  dx = dx > half ? rc.box - dx : dx;
  dy = dy > half ? rc.box - dy : dy;
  dz = dz > half ? rc.box - dz : dz;
  const R reach = rc.scale * (ar + br) + 2.0f * rc.cell;
  return dx * dx + dy * dy + dz * dz < reach * reach;
}

// One round of the commit over every survivor: state st_in -> st_out. The
// states, the acceptance list, the counters and the mask are read past L1
// (__ldcg): the persistent form runs rounds in one kernel, where another SM
// wrote them since the last barrier.
// A survivor's outcome for the round: state, the accepted list, counters.
template <class R>
__device__ __forceinline__ void commit_outcome(uint32_t i, R r, bool reject, bool ready,
                                               const RungConstsT<R>& rc, uint8_t* st_out,
                                               uint32_t* acc, uint32_t* counters, uint32_t slot) {
  uint8_t out = kUndecided;
  if (reject) {
    out = kRejected;
  } else if (ready) {
    out = kAccepted;
    acc[atomicAdd(counters, 1u)] = i;
    store_rmax(counters, r);
    // More than MISMATCH_RATIO (2) times the rung (exodus_finder.c:233,
    // 2324-2328): counted for the checkpoint and the run's warning.
    if (fdiv(r, rc.radius) > R(2.0f)) atomicAdd(counters + 9, 1u);
  } else {
    atomicAdd(counters + kRoundUndecided + slot, 1u);
  }
  st_out[i] = out;
}

// The commit's re-checks (exodus_finder.c:2286-2317) that read the mask: the
// node's bit, the poles at the rescaled radius. (The exact overlap with the
// catalogue as the rung began is decided once, before the rounds, by
// commit_init; with the rung's own voids, from the survivor hash.)
template <class R>
__device__ __forceinline__ bool commit_mask_reject(const SurvivorsT<R>& sv, uint32_t i, R r,
                                                   const uint32_t* mask, const RungConstsT<R>& rc) {
  const uint32_t nn = rc.grid_n;
  const uint32_t node = sv.flat[i];
  if (cand_masked(mask, node, sv.off ? sv.off[i] : R(-1.0f), r, rc)) return true;
  const uint32_t ix = node / (nn * nn), iy = (node / nn) % nn, iz = node % nn;
  const int32_t pole = (int32_t)(fdiv(fmul(fmul(rc.scale, r), fsub(R(1.0f), rc.f)), rc.cell)) - 1;
  return pole > 0 && overlap_quick(mask, nn, ix, iy, iz, (uint32_t)pole);
}

// Cell q (0..26) of the 3^3 hash cells around (hx, hy, hz): its slots.
template <class R>
__device__ __forceinline__ void hash_range(const SurvivorGridT<R>& g, int32_t hx, int32_t hy,
                                           int32_t hz, int q, uint32_t& lo, uint32_t& hi) {
  const int32_t ng = g.ng;
  lo = hi = 0;
  const bool one = ng < 3;  // a hash coarser than 3 cells is one cell
  if (one && q != 13) return;
  const int32_t ax = q / 9 - 1, ay = (q / 3) % 3 - 1, az = q % 3 - 1;
  const uint32_t c = one ? 0u
                         : (uint32_t)(((hx + ax + ng) % ng) * ng + (hy + ay + ng) % ng) * ng +
                               (uint32_t)((hz + az + ng) % ng);
  lo = g.start[c];
  hi = g.start[c + 1];
}

// Neighbour k of survivor i in the hash: sets reject on a collision with an
// accepted void of this rung, clears ready on an undecided lower-ranked
// survivor within reach. Only a neighbour within reach -- the reach of every
// test, the exact overlap's included -- has its state read.
template <class R>
__device__ __forceinline__ void commit_neighbour(const SurvivorGridT<R>& g, const SurvPackT<R>& p,
                                                 uint32_t k, uint32_t i, R cx, R cy, R cz, R r,
                                                 uint32_t my_rank, R half, const RungConstsT<R>& rc,
                                                 const uint8_t* st_in, bool& reject, bool& ready) {
  if (!interacts(cx, cy, cz, r, p.x, p.y, p.z, p.r, rc)) return;
  const uint32_t j = g.ids[k];
  if (j == i) return;
  const uint8_t sj = __ldcg(st_in + j);
  if (sj == kRejected) return;
  if (sj == kAccepted) {
    // A same-rung void: the exact pair test (its search box is the
    // reference's at the rung's largest radius; the minimum image form
    // agrees with the interior one wherever it applies, since neither
    // reaches half the box).
    if (collide(cx, cy, cz, r, p.x, p.y, p.z, p.r, rc.f, rc.scale, rc.box, half, false))
      reject = true;
  } else if (ready && g.hrank[k] < my_rank) {
    ready = false;
  }
}

// One round over the undecided survivors: a thread each, reading the 27 hash
// cells' ranges together and then the neighbours' records kBatch at a time.
// A survivor inside a crowd (more than kCrowd records in its 27 cells) goes
// to its block's queue instead, and after the block's pass a warp takes it,
// the lanes sharing its records: one thread walking a long list held every
// other block at the barrier that follows the pass. st_in / st_out: the
// states before and after the round; states, acceptances and the mask are
// read past L1, since other SMs wrote them since the last barrier.
constexpr uint32_t kCrowd = 96;
constexpr uint32_t kCrowdQueue = 512;
template <class R>
__device__ __forceinline__ void commit_pass(const SurvivorsT<R>& sv, const uint32_t* __restrict__ rank,
                                            const SurvivorGridT<R>& g, const VoidViewT<R>& voids,
                                            const uint32_t* mask, const RungConstsT<R>& rc,
                                            const uint8_t* st_in, uint8_t* st_out, uint32_t* acc,
                                            uint32_t* counters, uint32_t slot) {
  __shared__ uint32_t crowd[kCrowdQueue];
  __shared__ uint32_t n_crowd;
  if (threadIdx.x == 0) n_crowd = 0;
  __syncthreads();
  const uint32_t n = *sv.count;
  const R half = fmul(rc.box, R(0.5f));
  const unsigned lane = threadIdx.x & 31u;
  // Warps take 32 consecutive survivors at a time from the round's counter
  // (counters[kCommitWork], zeroed by the paint that ends each round):
  // survivors next to one another in the list are next to one another in
  // space, and a fixed share per block left the blocks over the crowded
  // voids to finish the pass alone.
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counters + kCommitWork, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t i = base + lane;
    if (i >= n) continue;
    const uint8_t s0 = __ldcg(st_in + i);
    if (s0 != kUndecided) {
      st_out[i] = s0;
      continue;
    }
    const R cx = sv.cx[i], cy = sv.cy[i], cz = sv.cz[i], r = sv.r[i];
    bool reject = commit_mask_reject(sv, i, r, mask, rc);
    bool ready = true;
    if (!reject) {
      const uint32_t my_rank = rank[sv.cand[i]];
      const int32_t hx = hash_axis(cx, g.inv_cell, g.ng), hy = hash_axis(cy, g.inv_cell, g.ng),
                    hz = hash_axis(cz, g.inv_cell, g.ng);
      uint32_t lo[27], hi[27], total = 0;
#pragma unroll
      for (int q = 0; q < 27; q++) {
        hash_range(g, hx, hy, hz, q, lo[q], hi[q]);
        total += hi[q] - lo[q];
      }
      if (total > kCrowd) {
        const uint32_t at = atomicAdd(&n_crowd, 1u);
        if (at < kCrowdQueue) {
          crowd[at] = i;
          continue;
        }
      }
      constexpr uint32_t kBatch = 8;
#pragma unroll 1
      for (int q = 0; q < 27 && !reject; q++) {
        const uint32_t e = hi[q];
        for (uint32_t k0 = lo[q]; k0 < e && !reject; k0 += kBatch) {
          SurvPackT<R> pb[kBatch];
#pragma unroll
          for (uint32_t u = 0; u < kBatch; u++)
            if (k0 + u < e) pb[u] = g.pack[k0 + u];
#pragma unroll
          for (uint32_t u = 0; u < kBatch; u++) {
            if (k0 + u >= e || reject) break;
            commit_neighbour(g, pb[u], k0 + u, i, cx, cy, cz, r, my_rank, half, rc, st_in, reject,
                             ready);
          }
        }
      }
    }
    commit_outcome(i, r, reject, ready, rc, st_out, acc, counters, slot);
  }
  __syncthreads();
  // The crowded survivors, a warp each.
  const uint32_t queued = min(n_crowd, kCrowdQueue);
  for (uint32_t w = threadIdx.x >> 5; w < queued; w += blockDim.x >> 5) {
    const uint32_t i = crowd[w];
    const R cx = sv.cx[i], cy = sv.cy[i], cz = sv.cz[i], r = sv.r[i];
    const uint32_t my_rank = rank[sv.cand[i]];
    const int32_t hx = hash_axis(cx, g.inv_cell, g.ng), hy = hash_axis(cy, g.inv_cell, g.ng),
                  hz = hash_axis(cz, g.inv_cell, g.ng);
    uint32_t lo = 0, hi = 0;
    if (lane < 27) hash_range(g, hx, hy, hz, (int)lane, lo, hi);
    bool reject = false, ready = true;
    for (int q = 0; q < 27; q++) {
      const uint32_t clo = __shfl_sync(0xffffffffu, lo, q), chi = __shfl_sync(0xffffffffu, hi, q);
      for (uint32_t k = clo + lane; k < chi && !reject; k += 32)
        commit_neighbour(g, g.pack[k], k, i, cx, cy, cz, r, my_rank, half, rc, st_in, reject, ready);
    }
    const bool any_reject = __any_sync(0xffffffffu, reject);
    const bool all_ready = __all_sync(0xffffffffu, ready);
    if (lane == 0) commit_outcome(i, r, any_reject, all_ready, rc, st_out, acc, counters, slot);
  }
}

template <class R>
__global__ void commit_round_kernel(SurvivorsT<R> sv, const uint32_t* __restrict__ rank,
                                    SurvivorGridT<R> g, VoidViewT<R> voids, const uint32_t* mask,
                                    RungConstsT<R> rc, const uint8_t* st_in, uint8_t* st_out,
                                    uint32_t* acc, uint32_t* counters, uint32_t slot) {
  commit_pass(sv, rank, g, voids, mask, rc, st_in, st_out, acc, counters, slot);
}

// Before the rounds: a survivor whose rescaling failed is rejected, and so
// is one whose sphere at its rescaled radius overlaps a void of the
// catalogue as the rung began (the re-check's exact overlap, whose answer no
// round can change; a warp per survivor); the rest start undecided.
template <class R>
__global__ void commit_init_kernel(SurvivorsT<R> sv, VoidViewT<R> voids, RungConstsT<R> rc,
                                   uint8_t* __restrict__ state, uint32_t* __restrict__ counters) {
  const uint32_t n = *sv.count;
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const R r = sv.r[i];
    const bool ok = r >= 0.0f;
    const bool overlaps =
        ok && overlap_exact_warp(voids, sv.cx[i], sv.cy[i], sv.cz[i], r, rc.f, rc.scale, rc.box);
    if (lane == 0) {
      state[i] = ok && !overlaps ? kUndecided : kRejected;
      if (!ok) atomicAdd(counters + 4, 1u);
      if (sv.reason[i] == kRescaleOverflow) atomicAdd(counters + 5, 1u);
      if (sv.reason[i] == kRescaleWitness) atomicAdd(counters + 8, 1u);
    }
  }
}

template <class R>
void commit_init(SurvivorsT<R> s, VoidViewT<R> voids, RungConstsT<R> rc, uint8_t* state,
                 uint32_t* counters, uint32_t max_survivors, cudaStream_t st) {
  if (max_survivors == 0) return;
  commit_init_kernel<<<grid_for((uint64_t)max_survivors * 32, 256), 256, 0, st>>>(s, voids, rc, state,
                                                                                counters);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void commit_round(SurvivorsT<R> s, const uint32_t* rank, SurvivorGridT<R> g, VoidViewT<R> voids,
                  const uint32_t* mask, RungConstsT<R> rc, const uint8_t* state_in, uint8_t* state_out,
                  uint32_t* acc, uint32_t* counters, uint32_t round, uint32_t max_survivors,
                  cudaStream_t st) {
  commit_round_kernel<<<grid_for(max_survivors, 128), 128, 0, st>>>(s, rank, g, voids, mask, rc,
                                                                     state_in, state_out, acc,
                                                                     counters, round % kRoundRing);
  SIFG_LAUNCH_CHECK();
}

// paint_sphere with set = 1 (src/finder/utils.c:965-1027) by one warp: every
// node whose centre lies within scale * r, measured as the reference
// measures it.
// part / parts: the warp paints every parts-th 32 of the sphere's columns,
// from the part-th (several warps share a large sphere).
template <class R>
__device__ __forceinline__ void paint_one(R cx, R cy, R cz, R r, uint32_t* mask,
                                          const RungConstsT<R>& rc, unsigned lane,
                                          uint32_t part = 0, uint32_t parts = 1) {
  const uint32_t n = rc.grid_n;
  {
    const R rt = fmul(rc.scale, r);
    const R r2 = fmul(rt, rt);
    const R inv = fdiv(R(1.0f), rc.cell);
    const R half = fmul(rc.gbox, R(0.5f));
    const int32_t cr = (int32_t)fmul(rt, inv) + 1;
    const int32_t ci = (int32_t)fmul(cx, inv), cj = (int32_t)fmul(cy, inv), ck = (int32_t)fmul(cz, inv);
    const int32_t side = 2 * cr + 1;
    for (int32_t q = lane + 32 * (int32_t)part; q < side * side; q += 32 * (int32_t)parts) {
      const int32_t gx = ci + q / side - cr, gy = cj + q % side - cr;
      R ddx = fabs_(fsub(fmul((R)gx, rc.cell), cx));
      ddx = ddx > half ? fsub(rc.gbox, ddx) : ddx;
      const R dx2 = fmul(ddx, ddx);
      if (dx2 > r2) continue;
      R ddy = fabs_(fsub(fmul((R)gy, rc.cell), cy));
      ddy = ddy > half ? fsub(rc.gbox, ddy) : ddy;
      const R dxy2 = fadd(dx2, fmul(ddy, ddy));
      if (dxy2 > r2) continue;
      const uint64_t row = ((uint64_t)wrap_pbc(gx, n) * n + wrap_pbc(gy, n)) * n;
      for (int32_t dz = -cr; dz <= cr; dz++) {
        const int32_t gz = ck + dz;
        R ddz = fabs_(fsub(fmul((R)gz, rc.cell), cz));
        ddz = ddz > half ? fsub(rc.gbox, ddz) : ddz;
        if (fadd(dxy2, fmul(ddz, ddz)) <= r2) {
          const uint64_t cell = row + wrap_pbc(gz, n);
          atomicOr(mask + (cell >> 5), 1u << (cell & 31));
        }
      }
    }
  }
}

// The voids the rounds accepted, one warp each.
template <class R>
__device__ __forceinline__ void paint_pass(const SurvivorsT<R>& sv, const uint32_t* acc,
                                           uint32_t* counters, uint32_t slot, uint32_t* mask,
                                           const RungConstsT<R>& rc) {
  const uint32_t lo = __ldcg(counters + kRoundBegin + slot), hi = __ldcg(counters);
  // No round accepts while a paint runs: hi is where the next round begins,
  // and the next round's pass takes its survivors from a counter at zero.
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    counters[kRoundBegin + (slot + 1) % kRoundRing] = hi;
    counters[kCommitWork] = 0;
  }
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t nv = hi - lo;
  if (nv == 0) return;
  // Fewer voids than warps: each void's columns shared by warps / nv warps
  // (a large sphere painted by one warp held every other block at the
  // barrier after the paint).
  const uint32_t parts = nv < warps ? min(warps / nv, 64u) : 1u;
  for (uint32_t item = w; item < nv * parts; item += warps) {
    const uint32_t i = __ldcg(acc + lo + item / parts);
    paint_one(sv.cx[i], sv.cy[i], sv.cz[i], sv.r[i], mask, rc, lane, item % parts, parts);
  }
}

// Voids given before the first rung (a prior catalogue), one warp each.
template <class R>
__global__ void paint_voids_kernel(const R* __restrict__ cx, const R* __restrict__ cy,
                                   const R* __restrict__ cz, const R* __restrict__ r, uint32_t n_voids,
                                   uint32_t* mask, RungConstsT<R> rc) {
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n_voids; v += warps)
    paint_one(cx[v], cy[v], cz[v], r[v], mask, rc, threadIdx.x & 31u);
}

template <class R>
void paint_voids(const R* cx, const R* cy, const R* cz, const R* r, uint32_t n_voids,
                 uint32_t* mask, RungConstsT<R> rc, cudaStream_t st) {
  if (n_voids == 0) return;
  paint_voids_kernel<R><<<grid_for((uint64_t)n_voids * 32, 256), 256, 0, st>>>(cx, cy, cz, r, n_voids,
                                                                              mask, rc);
  SIFG_LAUNCH_CHECK();
}

// paint_sphere with set = 1 (src/finder/utils.c:965-1027), one warp per void:
// every node whose centre lies within scale * r, measured as the reference
// measures it.
template <class R>
__global__ void paint_kernel(SurvivorsT<R> sv, const uint32_t* acc, uint32_t* counters,
                             uint32_t slot, uint32_t* mask, RungConstsT<R> rc) {
  paint_pass(sv, acc, counters, slot, mask, rc);
}

template <class R>
void paint_new(SurvivorsT<R> s, const uint32_t* acc, uint32_t* counters, uint32_t round,
               uint32_t* mask, RungConstsT<R> rc, uint32_t max_survivors, cudaStream_t st) {
  const uint32_t warps = max_survivors < 152u * 16u ? (max_survivors ? max_survivors : 1) : 152u * 16u;
  paint_kernel<<<(warps + 3) / 4, 128, 0, st>>>(s, acc, counters, round % kRoundRing, mask, rc);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// The commit's rounds in one cooperative launch
// ---------------------------------------------------------------------------

// A grid-wide barrier for a cooperative launch (every block resident):
// bar[0] counts arrivals, bar[1] is the generation, bar[2] the error flag.
// A wait that outlasts kBarrierSpins naps (about a second) sets the flag; a
// block that sees it returns false and the kernel ends.
constexpr unsigned kBarrierSpins = 1u << 22;
constexpr int kCommitT = 256;
__device__ __forceinline__ bool grid_barrier(unsigned* bar) {
  __shared__ bool ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = true;
    volatile unsigned* vgen = bar + 1;
    const unsigned gen = *vgen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (*vgen == gen) {
        if (++spins > kBarrierSpins) {
          atomicExch(bar + 2, 1u);
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
    if (*(volatile unsigned*)(bar + 2)) ok = false;
  }
  __syncthreads();
  return ok;
}

// Rounds round0, round0 + 1, ... until one leaves no survivor undecided or
// max_rounds have run: each a commit pass, a barrier, the paint of what it
// accepted, a barrier. Round k reads the states from sa (k even) or sb and
// writes the other. bar[3]: the rounds run.
template <class R>
__global__ void __launch_bounds__(kCommitT) commit_loop_kernel(
    SurvivorsT<R> sv, const uint32_t* __restrict__ rank, SurvivorGridT<R> g, VoidViewT<R> voids,
    uint32_t* mask, RungConstsT<R> rc, uint8_t* sa, uint8_t* sb, uint32_t* acc, uint32_t* counters,
    uint32_t round0, uint32_t max_rounds, unsigned* bar) {
  for (uint32_t k = 0; k < max_rounds; k++) {
    const uint32_t slot = (round0 + k) % kRoundRing;
    commit_pass(sv, rank, g, voids, mask, rc, (k & 1) ? sb : sa, (k & 1) ? sa : sb, acc, counters,
                slot);
    if (!grid_barrier(bar)) return;
    paint_pass(sv, acc, counters, slot, mask, rc);
    if (!grid_barrier(bar)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) bar[3] = k + 1;
    if (__ldcg(counters + kRoundUndecided + slot) == 0) return;
  }
}

static int g_commit_mode = 0;
void set_commit_mode(int mode) { g_commit_mode = mode; }

template <class R>
bool commit_rounds(SurvivorsT<R> s, const uint32_t* rank, SurvivorGridT<R> g, VoidViewT<R> voids,
                   uint32_t* mask, RungConstsT<R> rc, uint8_t* sa, uint8_t* sb, uint32_t* acc,
                   uint32_t* counters, uint32_t round0, uint32_t max_rounds, unsigned* bar,
                   uint32_t max_survivors, cudaStream_t st) {
  if (g_commit_mode != 0) return false;
  thread_local int blocks = -1;  // co-resident blocks of the device, found once per thread
  if (blocks < 0) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    SIFG_CUDA(cudaGetDevice(&dev));
    SIFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SIFG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    SIFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, commit_loop_kernel<R>, kCommitT, 0));
    blocks = coop && per_sm > 0 ? sms : 0;  // one block per SM
  }
  if (blocks == 0) return false;
  // A block per kCommitT survivors: a small rung's grid barriers gather few
  // blocks, and its launch finds room beside other engines' kernels (all of
  // a cooperative launch's blocks must be resident at once).
  const unsigned want = (unsigned)std::max<uint64_t>(1, ((uint64_t)max_survivors + kCommitT - 1) / kCommitT);
  const unsigned grid = std::min<unsigned>((unsigned)blocks, want);
  SIFG_CUDA(cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), st));
  void* args[] = {&s, (void*)&rank, &g, &voids, &mask, &rc, &sa, &sb, &acc, &counters, &round0,
                  &max_rounds, &bar};
  SIFG_CUDA(cudaLaunchCooperativeKernel((const void*)commit_loop_kernel<R>, dim3(grid),
                                        dim3(kCommitT), args, 0, st));
  SIFG_LAUNCH_CHECK();
  return true;
}

// ---------------------------------------------------------------------------
// Appending the rung's voids in rank order
// ---------------------------------------------------------------------------

template <class R>
__global__ void mark_ranks_kernel(SurvivorsT<R> sv, const uint32_t* __restrict__ rank,
                                  const uint32_t* __restrict__ acc, const uint32_t* __restrict__ counters,
                                  uint32_t* __restrict__ slots) {
  const uint32_t n = counters[0];
  for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
    slots[rank[sv.cand[acc[a]]]] = 1;
}

template <class R>
__global__ void write_voids_kernel(SurvivorsT<R> sv, const uint32_t* __restrict__ rank,
                                   const uint32_t* __restrict__ acc,
                                   const uint32_t* __restrict__ counters,
                                   const uint32_t* __restrict__ pos, R* __restrict__ cx,
                                   R* __restrict__ cy, R* __restrict__ cz,
                                   R* __restrict__ cr, uint32_t base) {
  const uint32_t n = counters[0];
  for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const uint32_t i = acc[a];
    const uint32_t o = base + pos[rank[sv.cand[i]]];
    cx[o] = sv.cx[i];
    cy[o] = sv.cy[i];
    cz[o] = sv.cz[i];
    cr[o] = sv.r[i];
  }
}

template <class R>
void append_accepted(SurvivorsT<R> s, const uint32_t* rank, const uint32_t* acc,
                     const uint32_t* counters, uint32_t m_candidates, uint32_t* rank_slots,
                     R* cat_x, R* cat_y, R* cat_z, R* cat_r, uint32_t n_voids,
                     uint32_t max_survivors, cudaStream_t st) {
  SIFG_CUDA(cudaMemsetAsync(rank_slots, 0, (m_candidates + 1) * sizeof(uint32_t), st));
  mark_ranks_kernel<<<grid_for(max_survivors, 256), 256, 0, st>>>(s, rank, acc, counters, rank_slots);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_u32(rank_slots, m_candidates + 1, st);
  write_voids_kernel<<<grid_for(max_survivors, 256), 256, 0, st>>>(s, rank, acc, counters, rank_slots,
                                                                   cat_x, cat_y, cat_z, cat_r, n_voids);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Void index
// ---------------------------------------------------------------------------

// cll_axis_index, src/structures/cell_linked_list.c:40-58 (periodic).
template <class R>
__device__ __forceinline__ uint32_t void_axis(R c, R inv) {
  int32_t i = (int32_t)ffloor(fmul(c, inv));
  i %= (int32_t)kVoidCells;
  if (i < 0) i += kVoidCells;
  return (uint32_t)i;
}

template <class R>
__global__ void void_count_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                  const R* __restrict__ z, uint32_t n, R inv,
                                  uint32_t* __restrict__ counts, uint32_t* __restrict__ cell_of) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t c = (void_axis(x[i], inv) * kVoidCells + void_axis(y[i], inv)) * kVoidCells +
                       void_axis(z[i], inv);
    cell_of[i] = c;
    atomicAdd(counts + c, 1u);
  }
}

template <class R>
void build_void_index(const R* cx, const R* cy, const R* cz, uint32_t n, R box,
                      uint32_t* start, uint32_t* ids, uint32_t* cell_of, cudaStream_t st) {
  const uint32_t cells = kVoidCells * kVoidCells * kVoidCells;
  SIFG_CUDA(cudaMemsetAsync(start, 0, (cells + 1) * sizeof(uint32_t), st));
  if (n == 0) return;
  const R inv = (R)kVoidCells / box;
  void_count_kernel<<<grid_for(n, 256), 256, 0, st>>>(cx, cy, cz, n, inv, start, cell_of);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_u32(start, cells + 1, st);
  thread_local DevBuf cursor;  // one per host thread driving a stream
  uint32_t* cur = (uint32_t*)cursor.ensure((cells + 1) * sizeof(uint32_t));
  SIFG_CUDA(cudaMemcpyAsync(cur, start, (cells + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  scatter_ids_kernel<<<grid_for(n, 256), 256, 0, st>>>(cell_of, nullptr, n, cur, ids);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Displacement (SIF_FINDER_DISPLACE)
// ---------------------------------------------------------------------------
// Under displacement a void is refused only by a larger one, and displaces
// the smaller ones it collides with (find_conflicts, displace_void,
// exodus_finder.c:696-756, 946-1037, and the commit at 2239-2275). Voids
// leave the catalogue, so a test that fails now may pass later and the
// rounds above do not apply: one CTA takes the survivors in rank order and
// does what the reference's sequential pass does, against a linked void index
// like the reference's (each cell's chain in descending void index: the
// order its head insertions and compaction leave, which fixes the order the
// conflicts are displaced in and the spheres painted back). Thread 0 walks
// the index; the CTA paints.

// The void index as linked chains: head per cell of the 32^3 index, next per
// void, -1 ends a chain.
template <class R>
struct VoidListT {
  R* cx;
  R* cy;
  R* cz;
  R* r;  // negated once displaced (the index no longer holds it)
  int32_t* head;
  int32_t* next;
  R inv_cell;
};

// The chains from the compressed index (ids of a cell in any order): each
// cell's ids sorted descending and linked. A thread per cell.
__global__ void void_chains_kernel(const uint32_t* __restrict__ start, uint32_t* ids,
                                   int32_t* __restrict__ head, int32_t* __restrict__ next) {
  constexpr uint32_t cells = kVoidCells * kVoidCells * kVoidCells;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += gridDim.x * blockDim.x) {
    const uint32_t s = start[c], e = start[c + 1];
    for (uint32_t a = s + 1; a < e; a++) {
      const uint32_t v = ids[a];
      uint32_t b = a;
      while (b > s && ids[b - 1] < v) {
        ids[b] = ids[b - 1];
        b--;
      }
      ids[b] = v;
    }
    head[c] = s < e ? (int32_t)ids[s] : -1;
    for (uint32_t a = s; a < e; a++) next[ids[a]] = a + 1 < e ? (int32_t)ids[a + 1] : -1;
  }
}

template <class R>
__device__ __forceinline__ uint32_t void_cell_of(R cx, R cy, R cz, R inv) {
  return (void_axis(cx, inv) * kVoidCells + void_axis(cy, inv)) * kVoidCells + void_axis(cz, inv);
}

// The cell window of a search of `reach` about c (the reference's
// floor((x -+ reach) / cell), the whole index when it is as wide).
template <class R>
__device__ __forceinline__ void void_window(R cx, R cy, R cz, R reach, R inv, int32_t* lo,
                                            int32_t* hi) {
  const R xs[3] = {cx, cy, cz};
  for (int a = 0; a < 3; a++) {
    lo[a] = (int32_t)ffloor(fmul(fsub(xs[a], reach), inv));
    hi[a] = (int32_t)ffloor(fmul(fadd(xs[a], reach), inv));
    if (hi[a] - lo[a] >= (int32_t)kVoidCells) {
      lo[a] = 0;
      hi[a] = (int32_t)kVoidCells - 1;
    }
  }
}

__device__ __forceinline__ uint32_t wrap_void(int32_t a) {
  const int32_t n = (int32_t)kVoidCells;
  return (uint32_t)(((a % n) + n) % n);
}

// sif__overlap_exact (src/finder/utils.c:850-960) over the chains.
template <class R>
__device__ bool overlap_exact_chains(const VoidListT<R>& v, R max_r, R cx, R cy, R cz, R r, R f,
                                     R scale, R box) {
  const R half = fmul(box, R(0.5f));
  const R s = search_radius(r, max_r, f, scale);
  const int32_t x0 = (int32_t)ffloor(fmul(fsub(cx, s), v.inv_cell));
  const int32_t x1 = (int32_t)ffloor(fmul(fadd(cx, s), v.inv_cell));
  const int32_t y0 = (int32_t)ffloor(fmul(fsub(cy, s), v.inv_cell));
  const int32_t y1 = (int32_t)ffloor(fmul(fadd(cy, s), v.inv_cell));
  const int32_t z0 = (int32_t)ffloor(fmul(fsub(cz, s), v.inv_cell));
  const int32_t z1 = (int32_t)ffloor(fmul(fadd(cz, s), v.inv_cell));
  const bool interior = is_interior(cx, cy, cz, s, box);
  for (int32_t ix = x0; ix <= x1; ix++)
    for (int32_t iy = y0; iy <= y1; iy++)
      for (int32_t iz = z0; iz <= z1; iz++) {
        const uint32_t c = (((uint32_t)ix & (kVoidCells - 1)) * kVoidCells +
                            ((uint32_t)iy & (kVoidCells - 1))) * kVoidCells +
                           ((uint32_t)iz & (kVoidCells - 1));
        for (int32_t j = v.head[c]; j != -1; j = v.next[j])
          if (collide(cx, cy, cz, r, v.cx[j], v.cy[j], v.cz[j], v.r[j], f, scale, box, half,
                      interior))
            return true;
      }
  return false;
}

// The minimum-image distance test of find_conflicts and displace_void.
template <class R>
__device__ __forceinline__ R min_image_d2(R ax, R ay, R az, R bx, R by, R bz, R box) {
  const R half = fmul(R(0.5f), box);
  R dx = fabs_(fsub(ax, bx)), dy = fabs_(fsub(ay, by)), dz = fabs_(fsub(az, bz));
  dx = dx > half ? fsub(box, dx) : dx;
  dy = dy > half ? fsub(box, dy) : dy;
  dz = dz > half ? fsub(box, dz) : dz;
  return fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
}

// paint_sphere (set or clear) by the whole CTA: every node within r of c.
template <class R>
__device__ void paint_cta(R cx, R cy, R cz, R r, uint32_t* mask, const RungConstsT<R>& rc, bool set) {
  const uint32_t n = rc.grid_n;
  const R r2 = fmul(r, r);
  const R inv = fdiv(R(1.0f), rc.cell);
  const R half = fmul(rc.gbox, R(0.5f));
  const int32_t cr = (int32_t)fmul(r, inv) + 1;
  const int32_t ci = (int32_t)fmul(cx, inv), cj = (int32_t)fmul(cy, inv), ck = (int32_t)fmul(cz, inv);
  const int32_t side = 2 * cr + 1;
  for (int32_t q = threadIdx.x; q < side * side; q += blockDim.x) {
    const int32_t gx = ci + q / side - cr, gy = cj + q % side - cr;
    R ddx = fabs_(fsub(fmul((R)gx, rc.cell), cx));
    ddx = ddx > half ? fsub(rc.gbox, ddx) : ddx;
    const R dx2 = fmul(ddx, ddx);
    if (dx2 > r2) continue;
    R ddy = fabs_(fsub(fmul((R)gy, rc.cell), cy));
    ddy = ddy > half ? fsub(rc.gbox, ddy) : ddy;
    const R dxy2 = fadd(dx2, fmul(ddy, ddy));
    if (dxy2 > r2) continue;
    const uint64_t row = ((uint64_t)wrap_pbc(gx, n) * n + wrap_pbc(gy, n)) * n;
    for (int32_t dz = -cr; dz <= cr; dz++) {
      const int32_t gz = ck + dz;
      R ddz = fabs_(fsub(fmul((R)gz, rc.cell), cz));
      ddz = ddz > half ? fsub(rc.gbox, ddz) : ddz;
      if (fadd(dxy2, fmul(ddz, ddz)) <= r2) {
        const uint64_t cell = row + wrap_pbc(gz, n);
        if (set)
          atomicOr(mask + (cell >> 5), 1u << (cell & 31));
        else
          atomicAnd(mask + (cell >> 5), ~(1u << (cell & 31)));
      }
    }
  }
}

// The commit's state: [0] voids in the catalogue (displaced ones included
// until the compaction), [1] accepted this rung, [2] displaced this rung,
// [3] a list overflowed, [4..5] the largest accepted radius (R's bits), [6]
// accepted at more than twice the rung.
constexpr uint32_t kDispVoids = 0, kDispAccepted = 1, kDispRemoved = 2, kDispOverflow = 3,
                   kDispMaxR = 4, kDispMismatched = 6;
constexpr int kDispT = 512;

template <class R>
__device__ __forceinline__ R load_real(const uint32_t* p) {
  R v;
  memcpy(&v, (const void*)p, sizeof(R));
  return v;
}
template <class R>
__device__ __forceinline__ void store_real(uint32_t* p, R v) {
  memcpy((void*)p, &v, sizeof(R));
}

template <class R>
__global__ void __launch_bounds__(kDispT) displace_commit_kernel(
    SurvivorsT<R> sv, const uint32_t* __restrict__ order, uint32_t m, VoidListT<R> vl,
    uint32_t* mask, RungConstsT<R> rc, uint32_t* state, uint32_t* conflicts, uint32_t* paints,
    uint32_t cap) {
  __shared__ int s_accept;
  __shared__ uint32_t s_n, s_j;
  __shared__ R s_v[4];
  const uint32_t nn = rc.grid_n;
  for (uint32_t k = 0; k < m; k++) {
    if (threadIdx.x == 0) {
      s_accept = 0;
      s_n = 0;
      const uint32_t i = order[k];
      const R r = sv.r[i];
      const uint32_t node = sv.flat[i];
      const R cx = sv.cx[i], cy = sv.cy[i], cz = sv.cz[i];
      const R max_r = load_real<R>(state + kDispMaxR);
      const uint32_t ix = node / (nn * nn), iy = (node / nn) % nn, iz = node % nn;
      // The rescaling failed; the node's mask bit; the poles and the exact
      // overlap at the rung radius, against the catalogue as it now stands.
      bool ok = r >= R(0) && !cand_masked(mask, node, sv.off ? sv.off[i] : R(-1.0f), rc.radius, rc);
      if (ok && rc.proxy_pole > 0 && overlap_quick(mask, nn, ix, iy, iz, (uint32_t)rc.proxy_pole))
        ok = false;
      if (ok && overlap_exact_chains(vl, max_r, cx, cy, cz, rc.radius, rc.f, rc.scale, rc.box))
        ok = false;
      if (ok) {
        // find_conflicts at the rescaled radius: refused by a void at least
        // as large, else those it collides with are displaced.
        const R reach = search_radius(r, max_r, rc.f, rc.scale);
        int32_t lo[3], hi[3];
        void_window(cx, cy, cz, reach, vl.inv_cell, lo, hi);
        R largest = R(-1.0f);
        uint32_t nc = 0;
        for (int32_t a = lo[0]; a <= hi[0]; a++)
          for (int32_t b = lo[1]; b <= hi[1]; b++)
            for (int32_t c = lo[2]; c <= hi[2]; c++) {
              const uint32_t cell = (wrap_void(a) * kVoidCells + wrap_void(b)) * kVoidCells + wrap_void(c);
              for (int32_t j = vl.head[cell]; j != -1; j = vl.next[j]) {
                const R rj = vl.r[j];
                const R mn = r < rj ? r : rj;
                const R tot = fmul(rc.scale, fsub(fadd(r, rj), fmul(rc.f, mn)));
                if (!(min_image_d2(cx, cy, cz, vl.cx[j], vl.cy[j], vl.cz[j], rc.box) < fmul(tot, tot)))
                  continue;
                if (nc < cap) conflicts[nc] = (uint32_t)j;
                nc++;
                if (rj > largest) largest = rj;
              }
            }
        if (nc > cap) state[kDispOverflow] = 1;
        if (largest < r && nc <= cap) {
          s_accept = 1;
          s_n = nc;
          s_v[0] = cx;
          s_v[1] = cy;
          s_v[2] = cz;
          s_v[3] = r;
        }
      }
    }
    __syncthreads();
    if (!s_accept) continue;
    const uint32_t nconf = s_n;
    const R ncx = s_v[0], ncy = s_v[1], ncz = s_v[2], nr = s_v[3];
    for (uint32_t q = 0; q < nconf; q++) {
      // displace_void: out of the index, radius negated, its sphere cleared,
      // the spheres of the voids still indexed that intersect it painted back.
      __shared__ R d[4];
      if (threadIdx.x == 0) {
        const uint32_t j = conflicts[q];
        d[0] = vl.cx[j];
        d[1] = vl.cy[j];
        d[2] = vl.cz[j];
        d[3] = vl.r[j];
        int32_t* link = vl.head + void_cell_of(d[0], d[1], d[2], vl.inv_cell);
        while (*link != -1 && *link != (int32_t)j) link = vl.next + *link;
        if (*link != -1) *link = vl.next[j];
        vl.r[j] = -d[3];
        state[kDispRemoved]++;
      }
      __syncthreads();
      paint_cta(d[0], d[1], d[2], fmul(rc.scale, d[3]), mask, rc, false);
      __syncthreads();
      if (threadIdx.x == 0) {
        const R max_r = load_real<R>(state + kDispMaxR);
        const R reach = fmul(rc.scale, fadd(d[3], max_r));
        int32_t lo[3], hi[3];
        void_window(d[0], d[1], d[2], reach, vl.inv_cell, lo, hi);
        uint32_t np = 0;
        for (int32_t a = lo[0]; a <= hi[0]; a++)
          for (int32_t b = lo[1]; b <= hi[1]; b++)
            for (int32_t c = lo[2]; c <= hi[2]; c++) {
              const uint32_t cell = (wrap_void(a) * kVoidCells + wrap_void(b)) * kVoidCells + wrap_void(c);
              for (int32_t j = vl.head[cell]; j != -1; j = vl.next[j]) {
                const R t = fmul(rc.scale, fadd(d[3], vl.r[j]));
                if (min_image_d2(d[0], d[1], d[2], vl.cx[j], vl.cy[j], vl.cz[j], rc.box) < fmul(t, t)) {
                  if (np < cap) paints[np] = (uint32_t)j;
                  np++;
                }
              }
            }
        if (np > cap) state[kDispOverflow] = 1;
        s_j = np < cap ? np : cap;
      }
      __syncthreads();
      // Painting sets bits only: the spheres in any order, a warp each.
      const uint32_t warps = blockDim.x >> 5;
      for (uint32_t p = threadIdx.x >> 5; p < s_j; p += warps) {
        const uint32_t j = paints[p];
        paint_one(vl.cx[j], vl.cy[j], vl.cz[j], vl.r[j], mask, rc, threadIdx.x & 31u);
      }
      __syncthreads();
    }
    // accept_void: appended, indexed at the head of its chain, painted.
    if (threadIdx.x == 0) {
      const uint32_t v = state[kDispVoids];
      vl.cx[v] = ncx;
      vl.cy[v] = ncy;
      vl.cz[v] = ncz;
      vl.r[v] = nr;
      const uint32_t cell = void_cell_of(ncx, ncy, ncz, vl.inv_cell);
      vl.next[v] = vl.head[cell];
      vl.head[cell] = (int32_t)v;
      state[kDispVoids] = v + 1;
      state[kDispAccepted]++;
      if (fdiv(nr, rc.radius) > R(2.0f)) state[kDispMismatched]++;
      if (nr > load_real<R>(state + kDispMaxR)) store_real<R>(state + kDispMaxR, nr);
    }
    paint_cta(ncx, ncy, ncz, fmul(rc.scale, nr), mask, rc, true);
    __syncthreads();
  }
}

// Survivor order from the ranks: order[rank[cand[i]]] = i (every candidate
// is a survivor under displacement).
template <class R>
__global__ void order_by_rank_kernel(SurvivorsT<R> sv, const uint32_t* __restrict__ rank,
                                     uint32_t* __restrict__ order) {
  const uint32_t n = *sv.count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    order[rank[sv.cand[i]]] = i;
}

// compact_catalogue (exodus_finder.c:1043-1078): the voids still standing
// (radius > 0) closed up in order, by one CTA in chunks.
template <class R>
__global__ void __launch_bounds__(1024) compact_voids_kernel(R* cx, R* cy, R* cz, R* r,
                                                             uint32_t* state) {
  __shared__ uint32_t ws[32];
  __shared__ uint32_t base;
  const uint32_t n = state[kDispVoids];
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (uint32_t c0 = 0; c0 < n; c0 += blockDim.x) {
    const uint32_t i = c0 + threadIdx.x;
    R v[4] = {0, 0, 0, 0};
    bool keep = false;
    if (i < n) {
      v[0] = cx[i];
      v[1] = cy[i];
      v[2] = cz[i];
      v[3] = r[i];
      keep = v[3] > R(0);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (uint32_t w = 0; w < blockDim.x / 32; w++) {
      before += w < (threadIdx.x >> 5) ? ws[w] : 0u;
      total += ws[w];
    }
    const uint32_t pos = base + before + __popc(bal & ((1u << (threadIdx.x & 31)) - 1u));
    __syncthreads();  // every read of this chunk is done before any write
    if (keep) {
      cx[pos] = v[0];
      cy[pos] = v[1];
      cz[pos] = v[2];
      r[pos] = v[3];
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) state[kDispVoids] = base;
}

template <class R>
void displace_commit(SurvivorsT<R> s, const uint32_t* rank, uint32_t m, uint32_t* order,
                     const uint32_t* vstart, uint32_t* vids, int32_t* head, int32_t* next,
                     R* cat_x, R* cat_y, R* cat_z, R* cat_r, R box, uint32_t* mask,
                     RungConstsT<R> rc, uint32_t* state, uint32_t* conflicts, uint32_t* paints,
                     uint32_t cap, cudaStream_t st) {
  void_chains_kernel<<<grid_for((uint64_t)kVoidCells * kVoidCells * kVoidCells, 256), 256, 0, st>>>(
      vstart, vids, head, next);
  SIFG_LAUNCH_CHECK();
  if (m == 0) return;
  order_by_rank_kernel<R><<<grid_for(m, 256), 256, 0, st>>>(s, rank, order);
  SIFG_LAUNCH_CHECK();
  VoidListT<R> vl{cat_x, cat_y, cat_z, cat_r, head, next, (R)kVoidCells / box};
  displace_commit_kernel<R><<<1, kDispT, 0, st>>>(s, order, m, vl, mask, rc, state, conflicts, paints,
                                                 cap);
  SIFG_LAUNCH_CHECK();
}

template <class R>
void compact_voids(R* cx, R* cy, R* cz, R* r, uint32_t* state, cudaStream_t st) {
  compact_voids_kernel<R><<<1, 1024, 0, st>>>(cx, cy, cz, r, state);
  SIFG_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// The two forms: the reference's float build and its SIF_USE_DOUBLE build.
// ---------------------------------------------------------------------------
#define SIFG_FINDER_FORM(R)                                                                        \
  template void scan_count_pass<R>(const R*, const uint32_t*, uint64_t, R, uint32_t*, uint32_t*,   \
                                   cudaStream_t, uint32_t, bool);                                  \
  template void scan_write_pass<R>(const R*, const uint32_t*, uint64_t, R, const uint32_t*, R*,    \
                                   uint32_t*, cudaStream_t, uint32_t, bool);                       \
  template void scan_fused_pass<R>(const R*, const uint32_t*, uint64_t, R, uint32_t*, uint32_t*,   \
                                   R*, uint32_t*, cudaStream_t, uint32_t, bool);                   \
  template void scan_compact<R>(const uint32_t*, uint64_t, const R*, const uint32_t*, R*,          \
                                uint32_t*, cudaStream_t);                                          \
  template void prefilter<R>(const uint32_t*, uint32_t, const uint32_t*, VoidViewT<R>,             \
                             RungConstsT<R>, uint8_t*, uint32_t*, uint32_t*, uint32_t*, R*, R*,    \
                             R*, uint32_t*, cudaStream_t, bool, const CandOffT<R>*, R*);          \
  template uint32_t refine_candidates<R>(const R*, const R*, const uint32_t*, R, uint32_t, R,      \
                                         uint32_t, bool, R*&, uint32_t*&, R*, uint32_t*,           \
                                         CandOffT<R>*, CandOffT<R>*&, CandOffT<R>*, uint32_t*,     \
                                         uint32_t*, cudaStream_t);                                 \
  template void witness<R>(MeshViewT<R>, TemplateViewT<R>, RungConstsT<R>, SurvivorsT<R>,         \
                           VoidViewT<R>, uint32_t, unsigned long long*, cudaStream_t, KernelTimer*, \
                           uint32_t*);                                                              \
  template void grow<R>(MeshViewT<R>, TemplateViewT<R>, RungConstsT<R>, SurvivorsT<R>, uint32_t,   \
                        R*, uint32_t, unsigned long long*, cudaStream_t, KernelTimer*, uint8_t,    \
                        uint32_t*, uint32_t*);                                                     \
  template void build_survivor_grid<R>(const R*, const R*, const R*, const R*, const uint32_t*,    \
                                       uint32_t, int32_t, R, uint32_t*, uint32_t*, uint32_t*,      \
                                       SurvPackT<R>*, cudaStream_t);                               \
  template void survivor_grid_ranks<R>(SurvivorsT<R>, const uint32_t*, const uint32_t*, uint32_t*, \
                                       uint32_t, cudaStream_t);                                    \
  template void commit_init<R>(SurvivorsT<R>, VoidViewT<R>, RungConstsT<R>, uint8_t*, uint32_t*,     \
                              uint32_t, cudaStream_t);                                              \
  template void commit_round<R>(SurvivorsT<R>, const uint32_t*, SurvivorGridT<R>, VoidViewT<R>,    \
                                const uint32_t*, RungConstsT<R>, const uint8_t*, uint8_t*,         \
                                uint32_t*, uint32_t*, uint32_t, uint32_t, cudaStream_t);           \
  template void paint_new<R>(SurvivorsT<R>, const uint32_t*, uint32_t*, uint32_t, uint32_t*,       \
                             RungConstsT<R>, uint32_t, cudaStream_t);                              \
  template void paint_voids<R>(const R*, const R*, const R*, const R*, uint32_t, uint32_t*,        \
                               RungConstsT<R>, cudaStream_t);                                      \
  template bool commit_rounds<R>(SurvivorsT<R>, const uint32_t*, SurvivorGridT<R>, VoidViewT<R>,   \
                                 uint32_t*, RungConstsT<R>, uint8_t*, uint8_t*, uint32_t*,         \
                                 uint32_t*, uint32_t, uint32_t, unsigned*, uint32_t, cudaStream_t);\
  template void append_accepted<R>(SurvivorsT<R>, const uint32_t*, const uint32_t*,                \
                                   const uint32_t*, uint32_t, uint32_t*, R*, R*, R*, R*, uint32_t, \
                                   uint32_t, cudaStream_t);                                        \
  template void build_void_index<R>(const R*, const R*, const R*, uint32_t, R, uint32_t*,          \
                                    uint32_t*, uint32_t*, cudaStream_t);                           \
  template void displace_commit<R>(SurvivorsT<R>, const uint32_t*, uint32_t, uint32_t*,            \
                                   const uint32_t*, uint32_t*, int32_t*, int32_t*, R*, R*, R*, R*, \
                                   R, uint32_t*, RungConstsT<R>, uint32_t*, uint32_t*, uint32_t*,  \
                                   uint32_t, cudaStream_t);                                        \
  template void compact_voids<R>(R*, R*, R*, R*, uint32_t*, cudaStream_t);

SIFG_FINDER_FORM(float)
SIFG_FINDER_FORM(double)

}  // namespace sifg
