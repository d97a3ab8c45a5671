// Exclusive prefix sums, and the small host helpers of kernels.cuh.
//
// The scan is the usual three phases: every CTA reduces its chunk, one CTA
// scans the chunk totals, every CTA rescans its chunk from its total. Up to
// kSmallChunks chunks (most of the path's scans: block totals, cell indexes)
// it is one CTA walking the chunks with a carry: one launch instead of three.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace sifg {

std::atomic<uint64_t> g_kernel_launches{0};

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint32_t kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums,
                                                         uint32_t& total) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= (unsigned)d) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t w = lane < (unsigned)nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= (unsigned)d) w += y;
    }
    if (lane < (unsigned)nw) warp_sums[lane] = w;
  }
  __syncthreads();
  total = warp_sums[(blockDim.x >> 5) - 1];
  const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ d,
                                                                   uint32_t n,
                                                                   uint32_t* __restrict__ sums) {
  __shared__ uint32_t ws[32];
  const uint32_t base = blockIdx.x * kScanChunk;
  uint32_t acc = 0;
  for (int k = 0; k < kScanItems; k++) {
    const uint32_t i = base + k * kScanThreads + threadIdx.x;
    if (i < n) acc += d[i];
  }
  uint32_t total;
  block_exclusive_scan(acc, ws, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(uint32_t* __restrict__ sums,
                                                                 uint32_t m) {
  __shared__ uint32_t ws[32];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < m; base += kScanThreads) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < m ? sums[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, ws, total);
    if (i < m) sums[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(uint32_t* __restrict__ d,
                                                                  uint32_t n,
                                                                  const uint32_t* __restrict__ sums) {
  __shared__ uint32_t ws[32];
  const uint32_t base = blockIdx.x * kScanChunk;
  // Each thread owns kScanItems consecutive entries.
  const uint32_t first = base + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint32_t i = first + k;
    v[k] = i < n ? d[i] : 0u;
    acc += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(acc, ws, total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint32_t i = first + k;
    if (i < n) d[i] = run;
    run += v[k];
  }
}

constexpr uint32_t kSmallChunks = 8;

// Every chunk is loaded before the first is scanned: the loads of all
// kSmallChunks chunks are in flight at once (the scans of the path's block
// totals sit between dependent launches, so this CTA's latency is theirs).
// last_zero: d[n - 1] is taken as 0 (not read); total, when set, receives the
// sum of all n.
__global__ void __launch_bounds__(kScanThreads) scan_small_kernel(uint32_t* __restrict__ d,
                                                                  uint32_t n, bool last_zero,
                                                                  uint32_t* __restrict__ total_out) {
  __shared__ uint32_t ws[32];
  uint32_t v[kSmallChunks][kScanItems];
#pragma unroll
  for (uint32_t c = 0; c < kSmallChunks; c++) {
    const uint32_t first = c * kScanChunk + threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
      v[c][k] = first + k < n && !(last_zero && first + k == n - 1) ? d[first + k] : 0u;
  }
  uint32_t carry = 0;
#pragma unroll
  for (uint32_t c = 0; c < kSmallChunks; c++) {
    if (c * kScanChunk >= n) break;  // uniform across the CTA
    const uint32_t first = c * kScanChunk + threadIdx.x * kScanItems;
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) acc += v[c][k];
    uint32_t total;
    uint32_t run = block_exclusive_scan(acc, ws, total) + carry;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      if (first + k < n) d[first + k] = run;
      run += v[c][k];
    }
    carry += total;
  }
  if (total_out && threadIdx.x == 0) *total_out = carry;
}

__global__ void store_last_kernel(const uint32_t* __restrict__ d, uint32_t i,
                                  uint32_t* __restrict__ out) {
  *out = d[i];
}

uint32_t scan_sums_needed(uint32_t n) { return (n + kScanChunk - 1) / kScanChunk; }

void exclusive_scan_u32(uint32_t* data, uint32_t n, cudaStream_t st, uint32_t* sums_scratch) {
  if (n == 0) return;
  const uint32_t blocks = (n + kScanChunk - 1) / kScanChunk;
  if (blocks <= kSmallChunks) {
    scan_small_kernel<<<1, kScanThreads, 0, st>>>(data, n, false, nullptr);
    SIFG_LAUNCH_CHECK();
    return;
  }
  thread_local DevBuf sums;  // chunk totals; small; one per host thread driving a stream
  uint32_t* s = sums_scratch ? sums_scratch
                             : (uint32_t*)sums.ensure((size_t)blocks * sizeof(uint32_t));
  scan_reduce_kernel<<<blocks, kScanThreads, 0, st>>>(data, n, s);
  SIFG_LAUNCH_CHECK();
  scan_sums_kernel<<<1, kScanThreads, 0, st>>>(s, blocks);
  SIFG_LAUNCH_CHECK();
  scan_apply_kernel<<<blocks, kScanThreads, 0, st>>>(data, n, s);
  SIFG_LAUNCH_CHECK();
}

void exclusive_scan_total(uint32_t* data, uint32_t nb, uint32_t* total, cudaStream_t st) {
  const uint32_t n = nb + 1;
  if ((n + kScanChunk - 1) / kScanChunk <= kSmallChunks) {
    // One launch: data[nb] taken as zero, the total written as the scan ends.
    scan_small_kernel<<<1, kScanThreads, 0, st>>>(data, n, true, total);
    SIFG_LAUNCH_CHECK();
    return;
  }
  SIFG_CUDA(cudaMemsetAsync(data + nb, 0, sizeof(uint32_t), st));
  exclusive_scan_u32(data, n, st);
  store_last_kernel<<<1, 1, 0, st>>>(data, nb, total);
  SIFG_LAUNCH_CHECK();
}

// --- helpers ---

void* DevBuf::ensure(size_t want) {
  if (want <= bytes && ptr) return ptr;
  release();
  size_t b = want < 256 ? 256 : want;
  SIFG_CUDA(cudaMalloc(&ptr, b));
  bytes = b;
  return ptr;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

// Timing events are kept for reuse, per device, instead of being created and
// destroyed for every span (a run records a few hundred). The pool and its
// lock are never destroyed: timers held by static objects return their
// events at exit, in no fixed order with other files' statics.
static std::mutex& event_mu() {
  static std::mutex* m = new std::mutex;
  return *m;
}
static std::map<int, std::vector<cudaEvent_t>>& event_pool() {
  static auto* p = new std::map<int, std::vector<cudaEvent_t>>;
  return *p;
}

static cudaEvent_t take_event() {
  int dev = 0;
  SIFG_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(event_mu());
    auto& pool = event_pool()[dev];
    if (!pool.empty()) {
      const cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
  }
  cudaEvent_t e;
  SIFG_CUDA(cudaEventCreate(&e));
  return e;
}

static void give_event(cudaEvent_t e) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaEventDestroy(e);
    return;
  }
  std::lock_guard<std::mutex> lk(event_mu());
  event_pool()[dev].push_back(e);
}

void event_pool_clear() {
  std::lock_guard<std::mutex> lk(event_mu());
  for (auto& [dev, pool] : event_pool())
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  event_pool().clear();
}

void KernelTimer::begin(cudaStream_t st) {
  const cudaEvent_t e = take_event();
  starts.push_back(e);
  open = (int)starts.size() - 1;
  SIFG_CUDA(cudaEventRecord(e, st));
}

void KernelTimer::end(cudaStream_t st) {
  const cudaEvent_t e = take_event();
  stops.push_back(e);
  open = -1;
  SIFG_CUDA(cudaEventRecord(e, st));
}

double KernelTimer::total_ms() {
  double t = 0.0;
  for (size_t i = 0; i < stops.size() && i < starts.size(); i++) {
    SIFG_CUDA(cudaEventSynchronize(stops[i]));
    float ms = 0.f;
    SIFG_CUDA(cudaEventElapsedTime(&ms, starts[i], stops[i]));
    t += ms;
  }
  return t;
}

void KernelTimer::reset() {
  for (auto e : starts) give_event(e);
  for (auto e : stops) give_event(e);
  starts.clear();
  stops.clear();
  open = -1;
}

KernelTimer::~KernelTimer() { reset(); }

}  // namespace sifg
