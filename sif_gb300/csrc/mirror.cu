// Device mirrors of the library's host blocks.
//
// sif's C API keeps every result in host arrays of its structs (a grid's
// values, a field's positions, a chain mesh's columns), and each call reads
// its inputs from them. Through that API the GPU path copies each input up
// and each result down on every call: a 512^3 pipeline moves the positions up
// twice, and the grid and the mesh it has just copied down up again.
//
// With mirrors on, the device copy an API call made of a host array (copied
// up as an input, or written on the device and copied down as a result) is
// kept, keyed by the array's address, and a later call that reads the same
// array uses it instead of copying again. That is only sound while the host
// array still holds what was copied, which the library cannot see when the
// caller writes through the struct's pointers. So mirrors are off unless the
// caller switches them on (sifg_set_host_mirrors, or SIFG_HOST_MIRRORS=1 at
// sif_system_init), and a caller that writes an array itself declares it with
// sifg_host_modified. As a net for writes that were not declared, each mirror
// keeps a sample of the host array's words taken when the two last agreed
// (kSamples words, evenly spaced, the first and the last among them); a call
// that finds any of them changed copies the array again. A write that misses
// every sampled word is not seen.
//
// Only arrays inside the library's own host blocks (host_block_get) are
// mirrored; a block returned to the pool forgets its mirrors. Device buffers
// of forgotten mirrors are kept for reuse up to kSpareBytes; all mirrors
// together hold at most kMirrorBytes (an array past it is copied as without
// mirrors).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace sifg {

namespace {

constexpr int kSamples = 1024;
constexpr size_t kMirrorBytes = 96ull << 30;
constexpr size_t kSpareBytes = 16ull << 30;

struct Mirror {
  size_t host_bytes = 0;
  size_t dev_bytes = 0;
  DevBuf dev;
  bool valid = false;
  std::vector<uint32_t> sample;
};

struct Registry {
  std::mutex mu;
  bool on = false;
  std::map<const void*, Mirror> live;  // by the host array's address
  std::vector<std::pair<void*, size_t>> spare;  // device buffers kept for reuse
  size_t live_bytes = 0, spare_bytes = 0;
};

Registry& reg() {
  static Registry* r = new Registry();  // outlives the static destructors that free blocks
  return *r;
}

void take_sample(const void* host, size_t bytes, std::vector<uint32_t>& out) {
  const uint32_t* w = (const uint32_t*)host;
  const size_t n = bytes / 4;
  out.resize(n ? kSamples : 0);
  for (int k = 0; n && k < kSamples; k++) {
    const size_t i = (size_t)((uint64_t)(n - 1) * (uint64_t)k / (kSamples - 1));
    out[k] = w[i];
  }
}

bool sample_holds(const void* host, size_t bytes, const std::vector<uint32_t>& s) {
  const uint32_t* w = (const uint32_t*)host;
  const size_t n = bytes / 4;
  if (s.size() != (n ? (size_t)kSamples : 0)) return false;
  for (int k = 0; n && k < kSamples; k++) {
    const size_t i = (size_t)((uint64_t)(n - 1) * (uint64_t)k / (kSamples - 1));
    if (w[i] != s[k]) return false;
  }
  return true;
}

// A mirror's buffer goes back to the spare list (or is freed past its cap).
void retire(Registry& r, Mirror& m) {
  r.live_bytes -= m.dev.bytes;
  if (m.dev.ptr && r.spare_bytes + m.dev.bytes <= kSpareBytes) {
    r.spare_bytes += m.dev.bytes;
    r.spare.emplace_back(m.dev.ptr, m.dev.bytes);
    m.dev.ptr = nullptr;  // handed to the spare list, not freed
    m.dev.bytes = 0;
  }
  m.dev.release();
}

void free_spares(Registry& r) {
  for (auto& b : r.spare) cudaFree(b.first);
  r.spare.clear();
  r.spare_bytes = 0;
}

void forget_range(Registry& r, const void* start, size_t bytes) {
  const char* lo = (const char*)start;
  auto it = r.live.lower_bound(start);
  while (it != r.live.end() && (const char*)it->first < lo + bytes) {
    retire(r, it->second);
    it = r.live.erase(it);
  }
}

// A device buffer of at least `bytes` into `out` (empty): the smallest spare
// one that does not waste more than a quarter, else a new one.
void take_buffer(Registry& r, DevBuf& out, size_t bytes) {
  int best = -1;
  for (int i = 0; i < (int)r.spare.size(); i++) {
    const size_t b = r.spare[i].second;
    if (b >= bytes && b - bytes <= b / 4 && (best < 0 || b < r.spare[best].second)) best = i;
  }
  if (best >= 0) {
    out.ptr = r.spare[best].first;
    out.bytes = r.spare[best].second;
    r.spare_bytes -= out.bytes;
    r.spare.erase(r.spare.begin() + best);
    return;
  }
  out.ensure(bytes);
}

}  // namespace

void mirror_enable(bool on) {
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  r.on = on;
  if (!on) {
    for (auto& kv : r.live) retire(r, kv.second);
    r.live.clear();
    free_spares(r);
  }
}

bool mirror_enabled() {
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  return r.on;
}

void* mirror_acquire(const void* host, size_t host_bytes, size_t dev_bytes, DevBuf& scratch,
                     bool* holds) {
  *holds = false;
  Registry& r = reg();
  const void* block = nullptr;
  size_t block_bytes = 0;
  {
    std::lock_guard<std::mutex> lk(r.mu);
    if (!r.on) return scratch.ensure(dev_bytes);
  }
  if (!host || !host_block_find(host, &block, &block_bytes) ||
      (const char*)host + host_bytes > (const char*)block + block_bytes)
    return scratch.ensure(dev_bytes);
  std::lock_guard<std::mutex> lk(r.mu);
  auto found = r.live.find(host);
  // A new mirror past the cap: this call's scratch instead (mirrors go only
  // when their blocks do, never while a call may be using them).
  if (found == r.live.end() && r.live_bytes + dev_bytes > kMirrorBytes) return scratch.ensure(dev_bytes);
  Mirror& m = found != r.live.end() ? found->second : r.live[host];
  if (m.valid && m.host_bytes == host_bytes && m.dev_bytes == dev_bytes && m.dev.ptr &&
      sample_holds(host, host_bytes, m.sample))
    *holds = true;
  m.valid = false;  // until mirror_commit: the call may write either side
  m.host_bytes = host_bytes;
  m.dev_bytes = dev_bytes;
  if (!m.dev.ptr || m.dev.bytes < dev_bytes) {
    retire(r, m);
    take_buffer(r, m.dev, dev_bytes);
    r.live_bytes += m.dev.bytes;
  }
  return m.dev.ptr;
}

void mirror_commit(const void* host) {
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  auto it = r.live.find(host);
  if (it == r.live.end() || !it->second.dev.ptr) return;
  take_sample(host, it->second.host_bytes, it->second.sample);
  it->second.valid = true;
}

void mirror_forget(const void* p) {
  Registry& r = reg();
  if (!p) {
    std::lock_guard<std::mutex> lk(r.mu);
    for (auto& kv : r.live) retire(r, kv.second);
    r.live.clear();
    return;
  }
  const void* block = nullptr;
  size_t bytes = 0;
  const bool in_block = host_block_find(p, &block, &bytes);
  std::lock_guard<std::mutex> lk(r.mu);
  if (in_block) {
    forget_range(r, block, bytes);
    return;
  }
  // Not a live block: the mirror whose array holds p, if any.
  auto it = r.live.upper_bound(p);
  if (it == r.live.begin()) return;
  --it;
  if ((const char*)p < (const char*)it->first + it->second.host_bytes) {
    retire(r, it->second);
    r.live.erase(it);
  }
}

void mirror_forget_block(const void* start, size_t bytes) {
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  forget_range(r, start, bytes);
}

void mirror_clear() {
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  for (auto& kv : r.live) retire(r, kv.second);
  r.live.clear();
  free_spares(r);
  r.live_bytes = 0;
}

}  // namespace sifg
