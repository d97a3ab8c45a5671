// Host-side entry points of the kernel modules, and the small helpers they
// share (device buffers, the event timer). Internal to the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace sifg {

constexpr int kCicTile = 16;  // CIC tile side, in grid cells

// The largest chain mesh side the GPU builds and reads: its cell ids and
// offsets are 32-bit, and 1625^3 + 1 is the last cube (plus the end offset)
// below 2^32. The reference's 64-bit offsets have no such bound; a larger
// mesh is refused with SIF_ERR_RANGE before anything is cubed.
constexpr uint32_t kMaxMeshSide = 1625;

// Destroys the timing events kept for reuse (before a device reset).
void event_pool_clear();

// Times a kernel with events on the stream it is launched on; accumulates.
// Its events come from, and go back to, a pool kept per device.
struct KernelTimer {
  std::vector<cudaEvent_t> starts, stops;
  int open = -1;
  void begin(cudaStream_t st);
  void end(cudaStream_t st);
  double total_ms();  // synchronises; sums every begin/end pair recorded
  int launches() const { return (int)stops.size(); }
  void reset();
  void swap(KernelTimer& o) {
    starts.swap(o.starts);
    stops.swap(o.stops);
    std::swap(open, o.open);
  }
  ~KernelTimer();
};

// A device allocation that grows on demand and is freed with its owner.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  void* ensure(size_t want);
  void release();
  ~DevBuf() { release(); }
  template <class T>
  T* as() const { return (T*)ptr; }
};

// --- hostpool.cu ---
// Host blocks for the library's structs: page-locked where possible, reused
// after host_block_put. host_block_put of a pointer the pool did not hand
// out frees it with free().
void* host_block_get(size_t bytes);
void host_block_put(void* ptr);
void host_pool_trim();
// The live block holding p (its start and size), if p lies in one.
bool host_block_find(const void* p, const void** start, size_t* bytes);

// --- mirror.cu ---
// Device mirrors of host arrays inside the library's blocks (off until
// mirror_enable(true)). mirror_acquire: the device buffer a call uses for host
// array `host` (host_bytes on the host, dev_bytes in its device form) --
// the array's mirror, or `scratch` when mirrors are off, the array is not in
// a library block, or the mirrors' cap is reached -- and whether it already
// holds the array's content (*holds). The mirror stands again only after
// mirror_commit(host), called once the two sides agree (the copy either way
// done or ordered before any later use). mirror_forget: the mirrors within
// the live block holding p (every mirror for NULL); mirror_forget_block: those
// within [start, start + bytes).
void mirror_enable(bool on);
bool mirror_enabled();
void* mirror_acquire(const void* host, size_t host_bytes, size_t dev_bytes, DevBuf& scratch,
                     bool* holds);
void mirror_commit(const void* host);
void mirror_forget(const void* p);
void mirror_forget_block(const void* start, size_t bytes);
void mirror_clear();

// --- scan.cu ---
// In-place exclusive prefix sum of n uint32 values (n < 2^31). The chunk
// totals go to `sums_scratch` (scan_sums_needed(n) entries) when given, else
// to a buffer the scan keeps.
uint32_t scan_sums_needed(uint32_t n);
void exclusive_scan_u32(uint32_t* data, uint32_t n, cudaStream_t st,
                        uint32_t* sums_scratch = nullptr);
// data[0..nb) scanned exclusively in place, data[nb] set to their total and
// *total (device) too; data[nb] need not be initialised. One launch up to
// 32,767 entries.
void exclusive_scan_total(uint32_t* data, uint32_t nb, uint32_t* total, cudaStream_t st);

// --- cic.cu ---
size_t cic_scratch_bytes(uint64_t n_particles, uint32_t n, bool weighted = false);
// bounds (lo, hi) and outside, when given: the deposit also adds to
// *outside the particles outside [lo, hi] (the box check from its own reads).
// sorted, when given, is recorded once the particles are in tile order: what
// follows (the deposit proper) is bound by shared-memory atomics, not by HBM.
// w: per-particle weights (device), or NULL for 1 each; the scratch is then
// cic_scratch_bytes(n_particles, n, true).
void cic_deposit(const float* x, const float* y, const float* z, uint64_t n_particles,
                 uint32_t n, float box, float* grid, void* scratch, cudaStream_t st,
                 KernelTimer* timer, const float* bounds = nullptr,
                 unsigned long long* outside = nullptr, cudaEvent_t sorted = nullptr,
                 const float* w = nullptr, KernelTimer* stage = nullptr);
// The FP64 form's deposit: scratch is cic_f64_scratch_bytes(n).
size_t cic_f64_scratch_bytes(uint32_t n);
void cic_deposit_f64(const double* x, const double* y, const double* z, uint64_t n_particles,
                     uint32_t n, double box, double* grid, void* scratch, cudaStream_t st,
                     KernelTimer* timer, const double* w = nullptr);
size_t density_contrast_scratch_bytes();
// The mean (a fixed summation order) into d_scratch, then v * (1 / mean) - 1
// in place unless mean_only; contrast_mean() is where the mean sits.
template <class R>
void density_contrast(R* v, uint64_t n, double* d_scratch, cudaStream_t st, bool mean_only = false);
template <class R>
void apply_contrast(R* v, uint64_t n, const double* mean, cudaStream_t st);
const double* contrast_mean(const double* d_scratch);
double read_mean(const double* d_scratch, cudaStream_t st);

// --- adjoint.cu ---
// dL/dx, dL/dy, dL/dz of every particle for g = dL/d(delta) on the grid,
// delta the CIC density contrast of the particles (the deposit's transpose).
template <class R>
void cic_contrast_vjp(const R* x, const R* y, const R* z, uint64_t np, uint32_t n, R box,
                      const R* g, R* gx, R* gy, R* gz, cudaStream_t st);

// --- mesh.cu ---
template <class R>
struct DeviceMeshT {
  uint32_t n_cells = 0;
  R box_length = 0, cell_length = 0;
  uint64_t n_particles = 0;
  R *x = nullptr, *y = nullptr, *z = nullptr;
  uint32_t* offsets = nullptr;  // n_cells^3 + 1
  uint32_t* orig = nullptr;     // source index of each entry
  // The float form's positions as 16-byte records (x, y, z, unused), one
  // load per particle, in place of x, y, z: the unordered build writes them.
  float4* xyzw = nullptr;
  // A weighted mesh (sif_chain_mesh_t::weights, cell_weights, total_weight):
  // weights in mesh order, per-cell sums; w NULL when unweighted.
  R* w = nullptr;
  R* cell_w = nullptr;
  double total_weight = 0.0;
};
using DeviceMesh = DeviceMeshT<float>;
// Scratch bytes of a mesh build in either form (the larger records).
size_t mesh_scratch_bytes(uint64_t n_particles, uint32_t n_cells);
// Builds into caller buffers (x, y, z, offsets, orig sized for the mesh).
// scratch: mesh_scratch_bytes(); scan_sums: NULL, or scan_sums_needed(cells
// + 1) entries the scan uses instead of a buffer of its own. With
// canonical false the cells' entries are left in the order the scatter
// placed them (no orig) and, in the float form, the positions go to m.xyzw:
// the same cells and counts, for a mesh only the sphere growth reads -- a
// radius depends on which particles a cell holds, not on their order.
template <class R>
void mesh_build(const R* x, const R* y, const R* z, uint64_t n_particles, DeviceMeshT<R>& m,
                void* scratch, cudaStream_t st, KernelTimer* timer, uint32_t* scan_sums = nullptr,
                bool canonical = true);
// A canonical mesh's weight columns from the field's weights (device, source
// order): m.w (n_particles) and m.cell_w (n_cells^3) written, the total to
// *d_total (device). scratch: mesh_weights_scratch_bytes(n_cells).
size_t mesh_weights_scratch_bytes(uint32_t n_cells);
template <class R>
void mesh_weights(const R* field_w, DeviceMeshT<R>& m, void* scratch, double* d_total,
                  cudaStream_t st);

}  // namespace sifg
