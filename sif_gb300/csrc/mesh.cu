// Chain-mesh build: the particles grouped by mesh cell, cells in flat order,
// each cell's particles in source order.
//
// Replaces chain_mesh_create + chain_mesh_canonicalise
// (src/structures/chain_mesh.c:680-832, 420-542). The cell of a particle is
// the reference's: (int32)(fold(x) * (1/cell_length)) clamped into the mesh
// (chain_mesh.c:316-331), so the mesh is the reference's bit for bit.
//
//   1. cell_count:  per-cell counts, warp-aggregated atomics;
//   2. exclusive scan into the cell offsets;
//   3. cell_scatter: (source index, x, y, z) into each cell's range, in the
//      order the atomics hand out slots;
//   4. cell_canon:  per cell, each entry's rank among the cell's source
//      indices (a count over the cell, with every lane reading the same
//      shared word at once), and the entry written to that rank -- the
//      canonical order, which no atomic race can change.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.cuh"

namespace sifg {

template <class R>
struct MeshGeom {
  uint32_t n;
  R box;
  R inv_l;  // 1 / cell_length
};

// A scatter record: source index and folded position.
template <class R>
struct alignas(16) MeshRec {
  uint32_t i;
  R x, y, z;
};
static_assert(sizeof(MeshRec<float>) == 16, "float records are 16 bytes");
static_assert(sizeof(MeshRec<double>) == 32, "double records are 32 bytes");

template <class R>
__device__ __forceinline__ uint32_t mesh_cell(R x, R y, R z, const MeshGeom<R>& g) {
  int32_t ix = (int32_t)fmul(box_fold(x, g.box), g.inv_l);
  int32_t iy = (int32_t)fmul(box_fold(y, g.box), g.inv_l);
  int32_t iz = (int32_t)fmul(box_fold(z, g.box), g.inv_l);
  const int32_t hi = (int32_t)g.n - 1;
  ix = ix < 0 ? 0 : (ix > hi ? hi : ix);
  iy = iy < 0 ? 0 : (iy > hi ? hi : iy);
  iz = iz < 0 ? 0 : (iz > hi ? hi : iz);
  return ((uint32_t)ix * g.n + (uint32_t)iy) * g.n + (uint32_t)iz;
}

template <class R>
__global__ void cell_count_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                  const R* __restrict__ z, uint64_t n, MeshGeom<R> g,
                                  uint32_t* __restrict__ counts) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    const uint32_t c = valid ? mesh_cell(x[p], y[p], z[p], g) : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    if (valid && (threadIdx.x & 31u) == (unsigned)(__ffs(peers) - 1))
      atomicAdd(counts + c, (uint32_t)__popc(peers));
  }
}

template <class R>
__global__ void cell_scatter_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                    const R* __restrict__ z, uint64_t n, MeshGeom<R> g,
                                    uint32_t* __restrict__ cursor, MeshRec<R>* __restrict__ tmp) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31u;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    R px = 0, py = 0, pz = 0;
    uint32_t c = 0xffffffffu;
    if (valid) {
      px = box_fold(x[p], g.box);
      py = box_fold(y[p], g.box);
      pz = box_fold(z[p], g.box);
      c = mesh_cell(x[p], y[p], z[p], g);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const unsigned leader = __ffs(peers) - 1;
    uint32_t slot0 = 0;
    if (valid && lane == leader) slot0 = atomicAdd(cursor + c, (uint32_t)__popc(peers));
    slot0 = __shfl_sync(0xffffffffu, slot0, leader);
    if (valid) {
      const uint32_t slot = slot0 + __popc(peers & ((1u << lane) - 1u));
      MeshRec<R> rec;
      rec.i = (uint32_t)p;
      rec.x = px;
      rec.y = py;
      rec.z = pz;
      tmp[slot] = rec;
    }
  }
}

// The float form's scatter straight into 16-byte position records, for a
// build that leaves each cell in scatter order.
__global__ void cell_scatter_xyzw_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                         const float* __restrict__ z, uint64_t n,
                                         MeshGeom<float> g, uint32_t* __restrict__ cursor,
                                         float4* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31u;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    float px = 0, py = 0, pz = 0;
    uint32_t c = 0xffffffffu;
    if (valid) {
      px = x[p];
      py = y[p];
      pz = z[p];
      c = mesh_cell(px, py, pz, g);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const unsigned leader = __ffs(peers) - 1;
    uint32_t slot0 = 0;
    if (valid && lane == leader) slot0 = atomicAdd(cursor + c, (uint32_t)__popc(peers));
    slot0 = __shfl_sync(0xffffffffu, slot0, leader);
    if (valid)
      out[slot0 + __popc(peers & ((1u << lane) - 1u))] =
          make_float4(box_fold(px, g.box), box_fold(py, g.box), box_fold(pz, g.box), 0.f);
  }
}

// The FP64 form's: straight into the mesh's position arrays.
template <class R>
__global__ void cell_scatter_soa_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                        const R* __restrict__ z, uint64_t n, MeshGeom<R> g,
                                        uint32_t* __restrict__ cursor, R* __restrict__ ox,
                                        R* __restrict__ oy, R* __restrict__ oz) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31u;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t p = base + threadIdx.x;
    const bool valid = p < n;
    R px = 0, py = 0, pz = 0;
    uint32_t c = 0xffffffffu;
    if (valid) {
      px = x[p];
      py = y[p];
      pz = z[p];
      c = mesh_cell(px, py, pz, g);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const unsigned leader = __ffs(peers) - 1;
    uint32_t slot0 = 0;
    if (valid && lane == leader) slot0 = atomicAdd(cursor + c, (uint32_t)__popc(peers));
    slot0 = __shfl_sync(0xffffffffu, slot0, leader);
    if (valid) {
      const uint32_t slot = slot0 + __popc(peers & ((1u << lane) - 1u));
      ox[slot] = box_fold(px, g.box);
      oy[slot] = box_fold(py, g.box);
      oz[slot] = box_fold(pz, g.box);
    }
  }
}

constexpr int kCanonThreads = 128;
constexpr int kCanonSmem = 2048;  // entries a CTA ranks in shared memory

// One warp per cell. A cell of up to kCanonSmem/4 entries per warp is ranked
// from shared memory; a larger one is ranked straight from global memory.
template <class R>
__global__ void __launch_bounds__(kCanonThreads) cell_canon_kernel(
    const MeshRec<R>* __restrict__ tmp, const uint32_t* __restrict__ offsets,
    uint32_t n_cells_total, R* __restrict__ ox, R* __restrict__ oy, R* __restrict__ oz,
    uint32_t* __restrict__ orig) {
  __shared__ uint32_t keys[kCanonSmem];
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const unsigned warps = kCanonThreads / 32;
  const uint32_t per_warp = kCanonSmem / warps;
  uint32_t* wk = keys + warp * per_warp;
  for (uint32_t cell = blockIdx.x * warps + warp; cell < n_cells_total;
       cell += gridDim.x * warps) {
    const uint32_t s = offsets[cell], e = offsets[cell + 1], cnt = e - s;
    if (cnt == 0) continue;
    const bool in_smem = cnt <= per_warp;
    if (in_smem) {
      for (uint32_t i = lane; i < cnt; i += 32) wk[i] = tmp[s + i].i;
      __syncwarp();
    }
    for (uint32_t i = lane; i < cnt + (32 - cnt % 32) % 32; i += 32) {
      const bool mine = i < cnt;
      MeshRec<R> v;
      v.i = 0;
      if (mine) v = tmp[s + i];
      uint32_t rank = 0;
      if (in_smem) {
        for (uint32_t j = 0; j < cnt; j++) rank += wk[j] < v.i;
      } else {
        for (uint32_t j = 0; j < cnt; j++) rank += tmp[s + j].i < v.i;
      }
      if (mine) {
        const uint32_t dst = s + rank;
        ox[dst] = v.x;
        oy[dst] = v.y;
        oz[dst] = v.z;
        if (orig) orig[dst] = v.i;
      }
    }
    __syncwarp();
  }
}

size_t mesh_scratch_bytes(uint64_t n_particles, uint32_t n_cells) {
  const uint64_t cells = (uint64_t)n_cells * n_cells * n_cells;
  return n_particles * sizeof(MeshRec<float>) + (cells + 1) * sizeof(uint32_t) + 1024;
}

template <class R>
void mesh_build(const R* x, const R* y, const R* z, uint64_t n_particles, DeviceMeshT<R>& m,
                void* scratch, cudaStream_t st, KernelTimer* timer, uint32_t* scan_sums,
                bool canonical) {
  MeshGeom<R> g;
  g.n = m.n_cells;
  g.box = m.box_length;
  g.inv_l = R(1.0f) / m.cell_length;
  const uint64_t cells = (uint64_t)m.n_cells * m.n_cells * m.n_cells;
  MeshRec<R>* tmp = (MeshRec<R>*)scratch;
  uint32_t* cursor = (uint32_t*)((char*)scratch +
                                 ((n_particles * sizeof(MeshRec<R>) + 255) & ~(size_t)255));
  SIFG_CUDA(cudaMemsetAsync(m.offsets, 0, (cells + 1) * sizeof(uint32_t), st));
  const unsigned grd = grid_for(n_particles, 256, 152u * 16u);
  if (timer) timer->begin(st);
  cell_count_kernel<R><<<grd, 256, 0, st>>>(x, y, z, n_particles, g, m.offsets);
  SIFG_LAUNCH_CHECK();
  exclusive_scan_u32(m.offsets, (uint32_t)(cells + 1), st, scan_sums);
  SIFG_CUDA(cudaMemcpyAsync(cursor, m.offsets, cells * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, st));
  if (!canonical) {
    if constexpr (sizeof(R) == 4)
      cell_scatter_xyzw_kernel<<<grd, 256, 0, st>>>(x, y, z, n_particles, g, cursor, m.xyzw);
    else
      cell_scatter_soa_kernel<R><<<grd, 256, 0, st>>>(x, y, z, n_particles, g, cursor, m.x, m.y,
                                                      m.z);
    SIFG_LAUNCH_CHECK();
    if (timer) timer->end(st);
    m.n_particles = n_particles;
    return;
  }
  cell_scatter_kernel<R><<<grd, 256, 0, st>>>(x, y, z, n_particles, g, cursor, tmp);
  SIFG_LAUNCH_CHECK();
  const unsigned cgrid = grid_for(cells, kCanonThreads / 32 * 1, 152u * 16u);
  cell_canon_kernel<R><<<cgrid, kCanonThreads, 0, st>>>(tmp, m.offsets, (uint32_t)cells, m.x, m.y,
                                                        m.z, m.orig);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(st);
  m.n_particles = n_particles;
}

// ---------------------------------------------------------------------------
// A weighted mesh's columns (chain_mesh.c:800-801, 624-672): each entry's
// weight is the field's at its source index; each cell's weights summed in
// double in mesh order and stored in the form's precision; the total over 64
// fixed blocks of cells, each block's cell sums added in order, the blocks
// then added in order. Every sum in the reference's order, so every bit is
// the reference's.
// ---------------------------------------------------------------------------
template <class R>
__global__ void gather_weights_kernel(const R* __restrict__ fw, const uint32_t* __restrict__ orig,
                                      uint64_t n, R* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride)
    out[p] = fw[orig[p]];
}

template <class R>
__global__ void cell_weight_kernel(const uint32_t* __restrict__ offsets, const R* __restrict__ w,
                                   uint64_t cells, double* __restrict__ csum, R* __restrict__ cw) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += stride) {
    double s = 0.0;
    for (uint32_t p = offsets[c]; p < offsets[c + 1]; p++) s = __dadd_rn(s, (double)w[p]);
    csum[c] = s;
    cw[c] = (R)s;
  }
}

constexpr int kWeightBlocks = 64;  // WEIGHT_BLOCKS, chain_mesh.c:642

__global__ void weight_total_kernel(const double* __restrict__ csum, uint64_t cells,
                                    double* __restrict__ total) {
  __shared__ double bt[kWeightBlocks];
  const uint64_t block = (cells + kWeightBlocks - 1) / kWeightBlocks;
  const uint64_t c0 = (uint64_t)threadIdx.x * block;
  const uint64_t c1 = c0 + block < cells ? c0 + block : cells;
  double s = 0.0;
  for (uint64_t c = c0; c < c1; c++) s = __dadd_rn(s, csum[c]);
  bt[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < kWeightBlocks; b++) t = __dadd_rn(t, bt[b]);
    *total = t;
  }
}

size_t mesh_weights_scratch_bytes(uint32_t n_cells) {
  return (size_t)n_cells * n_cells * n_cells * sizeof(double) + 256;
}

template <class R>
void mesh_weights(const R* field_w, DeviceMeshT<R>& m, void* scratch, double* d_total,
                  cudaStream_t st) {
  const uint64_t cells = (uint64_t)m.n_cells * m.n_cells * m.n_cells;
  gather_weights_kernel<R><<<grid_for(m.n_particles, 256, 152u * 16u), 256, 0, st>>>(
      field_w, m.orig, m.n_particles, m.w);
  SIFG_LAUNCH_CHECK();
  double* csum = (double*)scratch;
  cell_weight_kernel<R><<<grid_for(cells, 128, 152u * 32u), 128, 0, st>>>(m.offsets, m.w, cells,
                                                                         csum, m.cell_w);
  SIFG_LAUNCH_CHECK();
  weight_total_kernel<<<1, kWeightBlocks, 0, st>>>(csum, cells, d_total);
  SIFG_LAUNCH_CHECK();
}

template void mesh_weights<float>(const float*, DeviceMeshT<float>&, void*, double*, cudaStream_t);
template void mesh_weights<double>(const double*, DeviceMeshT<double>&, void*, double*,
                                   cudaStream_t);

template void mesh_build<float>(const float*, const float*, const float*, uint64_t,
                                DeviceMeshT<float>&, void*, cudaStream_t, KernelTimer*, uint32_t*,
                                bool);
template void mesh_build<double>(const double*, const double*, const double*, uint64_t,
                                 DeviceMeshT<double>&, void*, cudaStream_t, KernelTimer*,
                                 uint32_t*, bool);

}  // namespace sifg
