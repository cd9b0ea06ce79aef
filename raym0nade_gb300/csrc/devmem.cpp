// Device memory of render batches, kept for reuse.
//
// Every rmn_render call builds a batch whose worker pool, queues and unit
// partials take up to a few GB; allocating and freeing them per call made
// cudaMalloc / cudaFree (which can synchronise the device) a visible part of
// a render. Blocks returned by a batch are kept per device and handed to the
// next batch that asks for a size between the block's half and its size, up
// to kCacheLimit bytes per device; rmn_release_cached_memory frees them.
#include <map>
#include <mutex>
#include <unordered_map>

#include "rmn_host.h"

namespace rmn {
namespace {

constexpr size_t kCacheLimit = size_t(16) << 30;

struct DeviceCache {
  std::multimap<size_t, void*> free_blocks;  // size -> block
  size_t cached = 0;
};

std::mutex g_mu;
std::unordered_map<int, DeviceCache> g_cache;
std::unordered_map<void*, std::pair<int, size_t>> g_live;  // block -> (device, size)

void release_all(DeviceCache& c) {
  for (auto& kv : c.free_blocks) cudaFree(kv.second);
  c.free_blocks.clear();
  c.cached = 0;
}

}  // namespace

cudaError_t cached_malloc(void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) / 256 * 256;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceCache& c = g_cache[dev];
  auto it = c.free_blocks.lower_bound(bytes);
  if (it != c.free_blocks.end() && it->first <= 2 * bytes) {
    *p = it->second;
    c.cached -= it->first;
    g_live[*p] = {dev, it->first};
    c.free_blocks.erase(it);
    return cudaSuccess;
  }
  e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation && !c.free_blocks.empty()) {
    cudaGetLastError();
    release_all(c);
    e = cudaMalloc(p, bytes);
  }
  if (e == cudaSuccess) g_live[*p] = {dev, bytes};
  return e;
}

void cached_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_live.find(p);
  if (it == g_live.end()) return;
  const int dev = it->second.first;
  const size_t bytes = it->second.second;
  g_live.erase(it);
  DeviceCache& c = g_cache[dev];
  if (c.cached + bytes > kCacheLimit) {
    cudaFree(p);
    return;
  }
  c.free_blocks.emplace(bytes, p);
  c.cached += bytes;
}

void release_cached_memory() {
  std::lock_guard<std::mutex> lock(g_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  for (auto& kv : g_cache) {
    if (kv.first != dev) cudaSetDevice(kv.first);
    release_all(kv.second);
  }
  cudaSetDevice(dev);
}

}  // namespace rmn
