// Host blocks of the library's own structs (field positions, grid values,
// chain-mesh arrays, catalogues), kept for reuse.
//
// The reference allocates these with malloc and frees them with free
// (src/structures/field.c, grid.c:64-108, chain_mesh.c:49-215). Here they
// are the staging ends of host<->device copies, so they are page-locked
// where the driver allows it, and a freed block is kept for the next
// allocation of a similar size instead of being returned: a fresh block of
// gigabytes costs a page fault per page on first touch, more than the copy
// into it. At most kPoolBlocks free blocks and kPoolBytes free bytes are kept
// (oldest first out); every free block is released by host_pool_trim().
#include <cuda_runtime.h>
#include <stdlib.h>

#include <deque>
#include <mutex>
#include <unordered_map>

#include "kernels.cuh"

namespace sifg {

namespace {

constexpr size_t kPoolBlocks = 8;
constexpr size_t kPoolBytes = 24ull << 30;

struct Block {
  size_t bytes;
  bool pinned;
};

struct Pool {
  std::mutex mu;
  std::unordered_map<void*, Block> live;  // every block handed out
  std::deque<std::pair<void*, Block>> spare;
  size_t spare_bytes = 0;
};

Pool& pool() {
  static Pool* p = new Pool();  // outlives every static destructor that might free into it
  return *p;
}

void release(void* ptr, const Block& b) {
  if (b.pinned)
    cudaFreeHost(ptr);
  else
    free(ptr);
}

}  // namespace

void* host_block_get(size_t bytes) {
  if (bytes == 0) bytes = 1;
  Pool& p = pool();
  {
    std::lock_guard<std::mutex> lk(p.mu);
    // The smallest spare block that fits without wasting more than a quarter.
    auto best = p.spare.end();
    for (auto it = p.spare.begin(); it != p.spare.end(); ++it)
      if (it->second.bytes >= bytes && it->second.bytes - bytes <= it->second.bytes / 4 &&
          (best == p.spare.end() || it->second.bytes < best->second.bytes))
        best = it;
    if (best != p.spare.end()) {
      void* ptr = best->first;
      const Block b = best->second;
      p.spare_bytes -= b.bytes;
      p.spare.erase(best);
      p.live[ptr] = b;
      return ptr;
    }
  }
  void* ptr = nullptr;
  Block b{bytes, true};
  if (cudaMallocHost(&ptr, bytes) != cudaSuccess) {
    cudaGetLastError();  // no device, or no page-locked memory left: plain memory
    ptr = malloc(bytes);
    b.pinned = false;
    if (!ptr) return nullptr;
  }
  std::lock_guard<std::mutex> lk(p.mu);
  p.live[ptr] = b;
  return ptr;
}

void host_block_put(void* ptr) {
  if (!ptr) return;
  Pool& p = pool();
  std::lock_guard<std::mutex> lk(p.mu);
  auto it = p.live.find(ptr);
  if (it == p.live.end()) {
    free(ptr);  // not one of ours: the caller's own malloc
    return;
  }
  const Block b = it->second;
  // The block's content is gone for whoever takes it next: its device
  // mirrors with it (the registry's own lock, taken inside the pool's).
  mirror_forget_block(ptr, b.bytes);
  p.live.erase(it);
  p.spare.emplace_back(ptr, b);
  p.spare_bytes += b.bytes;
  while (!p.spare.empty() && (p.spare.size() > kPoolBlocks || p.spare_bytes > kPoolBytes)) {
    release(p.spare.front().first, p.spare.front().second);
    p.spare_bytes -= p.spare.front().second.bytes;
    p.spare.pop_front();
  }
}

bool host_block_find(const void* p, const void** start, size_t* bytes) {
  Pool& pl = pool();
  std::lock_guard<std::mutex> lk(pl.mu);
  const char* c = (const char*)p;
  for (const auto& kv : pl.live) {
    const char* s = (const char*)kv.first;
    if (c >= s && c < s + kv.second.bytes) {
      *start = kv.first;
      *bytes = kv.second.bytes;
      return true;
    }
  }
  return false;
}

void host_pool_trim() {
  Pool& p = pool();
  std::lock_guard<std::mutex> lk(p.mu);
  for (auto& s : p.spare) release(s.first, s.second);
  p.spare.clear();
  p.spare_bytes = 0;
}

}  // namespace sifg
