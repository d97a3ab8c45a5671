// The chain-mesh build without device allocation: sifg_mesh_device_noalloc.
//
// Some callers cannot let a library allocate GPU memory. A process whose
// framework reserves the device's memory up front in its own pool (as
// PyTorch's caching allocator and most serving stacks do) leaves cudaMalloc
// failing or fragmenting that pool; a latency-bound pipeline cannot afford
// cudaFree, which waits for the whole device; a host application that
// enforces its own memory budget forbids allocations it did not make. For
// them this entry point builds the mesh with a scratch area that is part of
// the library itself: a file-scope device array, allocated once when the
// library's module is loaded on a device and held until the process exits,
// on every GPU that loads it.
//
// The scratch holds what sifg_mesh_device's scratch holds: the (source index,
// x, y, z) records of the scatter, the per-cell cursors and the scan's chunk
// totals, plus the box check's counter. Its size fixes the limits: at most
// kNoAllocMaxParticles particles and kNoAllocMaxSide^3 mesh cells.
#include <cuda_runtime.h>

#include <cfloat>
#include <mutex>
#include <string>

#include "../../include/sif_gb300.h"
#include "kernels.cuh"

namespace sifg {

std::mutex& api_mutex();
bool api_stream(cudaStream_t* st, int* device);

constexpr uint64_t kNoAllocMaxParticles = 1ull << 20;  // 1,048,576 particles
constexpr uint32_t kNoAllocMaxSide = 64;               // mesh cells a side
constexpr uint64_t kNoAllocMaxCells = (uint64_t)kNoAllocMaxSide * kNoAllocMaxSide * kNoAllocMaxSide;

// Layout: the build's scratch (records, then cursors: mesh_scratch_bytes()
// at the limits), the scan's chunk totals, the box check's counter (in a
// 256-byte slot).
constexpr size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kMeshScratchBytes =
    a256(kNoAllocMaxParticles * 16 + (kNoAllocMaxCells + 1) * 4 + 1024);
constexpr size_t kScanSumsBytes = a256(((kNoAllocMaxCells + 1 + 4095) / 4096) * 4);
constexpr size_t kNoAllocScratchBytes = kMeshScratchBytes + kScanSumsBytes + 256;

// Shared by every call in the process: each call leaves its contents behind,
// and every part a call reads it first writes or clears.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The array's device address, per device. In host code g_noalloc_scratch
// names a host-side stand-in, not device memory, so the address comes from
// cudaGetSymbolAddress, with that device current. It is looked up by the
// first call on a device after sif_system_init() and forgotten by
// sif_system_finalise(): a caller that resets the device (cudaDeviceReset,
// which also ends the library's streams) finalises and initialises the
// library again, and the next call looks the address up anew.
static std::mutex g_setup_mu;
static void* g_scratch_addr[64] = {};

void noalloc_forget() {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  for (void*& p : g_scratch_addr) p = nullptr;
}

static int scratch_address(int device, void** out) {
  if (device < 0 || device >= 64) return SIF_ERR_RANGE;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (rc != cudaSuccess || !p) {
      set_error(SIF_ERR_INVALID, std::string("allocation-free mesh: cudaGetSymbolAddress: ") +
                                     cudaGetErrorString(rc));
      return SIF_ERR_INVALID;
    }
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return SIF_OK;
}

// sif__field_check_in_box (src/structures/field.c:889-935) into a counter of
// the static scratch: the particles with a coordinate outside the box by more
// than 4 float epsilons of it, or not a number. Those within that tolerance
// are folded by the build, as the reference folds them.
__global__ void noalloc_box_check_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                         const float* __restrict__ z, uint64_t n, float box,
                                         double tol, unsigned long long* __restrict__ out) {
  unsigned long long bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float v[3] = {x[i], y[i], z[i]};
    for (int a = 0; a < 3; a++) {
      const double d = (double)v[a];
      if (!(d >= -tol && d <= (double)box + tol)) {
        bad++;
        break;
      }
    }
  }
  for (int d = 16; d > 0; d >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, d);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(out, bad);
}

}  // namespace sifg

using namespace sifg;

extern "C" int sifg_mesh_device_noalloc(const float* x, const float* y, const float* z,
                                        uint64_t n, uint32_t n_cells, float box, float* mx,
                                        float* my, float* mz, uint32_t* offsets,
                                        uint32_t* orig) {
  // The whole call under the API lock: its enqueues on the library's stream
  // do not interleave with another host thread's call, and the stream
  // outlives it (sif_system_finalise waits for the lock).
  std::lock_guard<std::mutex> lk(api_mutex());
  cudaStream_t st;
  int device;
  if (!api_stream(&st, &device)) return SIF_ERR_UNINITIALISED;
  if (n_cells == 0 || !(box > 0.0f)) {
    set_error(SIF_ERR_INVALID, "allocation-free mesh: n_cells must be positive and box > 0");
    return SIF_ERR_INVALID;
  }
  // The side is bounded before it is cubed: a cube of a large side would
  // wrap around 64 bits and pass a bound on the cube.
  if (n > kNoAllocMaxParticles || n_cells > kNoAllocMaxSide) {
    set_error(SIF_ERR_RANGE,
              "allocation-free mesh: " + std::to_string(n) + " particles in " +
                  std::to_string(n_cells) + "^3 cells exceeds its fixed scratch (at most " +
                  std::to_string(kNoAllocMaxParticles) + " particles and " +
                  std::to_string(kNoAllocMaxSide) + "^3 cells); use sifg_mesh_device");
    return SIF_ERR_RANGE;
  }
  try {
    SIFG_CUDA(cudaSetDevice(device));
    void* scratch = nullptr;
    const int rc = scratch_address(device, &scratch);
    if (rc != SIF_OK) return rc;
    uint32_t* scan_sums = (uint32_t*)((char*)scratch + kMeshScratchBytes);
    unsigned long long* counters =
        (unsigned long long*)((char*)scratch + kMeshScratchBytes + kScanSumsBytes);
    SIFG_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned long long), st));
    if (n) {
      noalloc_box_check_kernel<<<grid_for(n, 256), 256, 0, st>>>(
          x, y, z, n, box, (double)box * 4.0 * (double)FLT_EPSILON, counters);
      SIFG_LAUNCH_CHECK();
    }
    unsigned long long bad = 0;
    SIFG_CUDA(cudaMemcpyAsync(&bad, counters, sizeof bad, cudaMemcpyDeviceToHost, st));
    SIFG_CUDA(cudaStreamSynchronize(st));
    if (bad) {
      set_error(SIF_ERR_RANGE, "allocation-free mesh: " + std::to_string(bad) +
                                   " particles outside the box");
      return SIF_ERR_RANGE;
    }
    DeviceMesh m;
    m.n_cells = n_cells;
    m.box_length = box;
    m.cell_length = box / (float)n_cells;
    m.x = mx;
    m.y = my;
    m.z = mz;
    m.offsets = offsets;
    m.orig = orig;
    mesh_build(x, y, z, n, m, scratch, st, nullptr, scan_sums);
    SIFG_CUDA(cudaStreamSynchronize(st));
    return SIF_OK;
  } catch (const CudaError& e) {
    set_error(SIF_ERR_INVALID, std::string("CUDA: ") + cudaGetErrorString(e.code) + " (" +
                                   e.where + ")");
    return SIF_ERR_INVALID;
  }
}
