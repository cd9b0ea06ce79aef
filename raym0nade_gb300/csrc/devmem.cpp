// Device memory of render batches, kept for reuse.
//
// Every rmn_render call builds a batch whose worker pool, queues and unit
// partials take up to a few GB; allocating and freeing them per call made
// cudaMalloc / cudaFree (which can synchronise the device) a visible part of
// a render. Blocks returned by a batch are kept per device and handed to the
// next batch that asks for a size between the block's half and its size, up
// to kCacheLimit bytes per device; rmn_release_cached_memory frees them.
//
// The calls' short-lived buffers (host arrays staged through the device,
// intermediate images, status words) are stream-ordered allocations from a
// memory pool of the library's own per device, which keeps up to
// kStagingKeep bytes across stream synchronisations. The device's default
// pool gives its memory back at every synchronisation (release threshold
// 0), so each call of a loop such as one rmn_compose per image mapped its
// buffers anew: about 0.2 ms a call.
#include <map>
#include <mutex>
#include <unordered_map>

#include "rmn_host.h"

namespace rmn {
namespace {

constexpr size_t kCacheLimit = size_t(16) << 30;
constexpr uint64_t kStagingKeep = uint64_t(1) << 30;

std::mutex g_pool_mu;
std::unordered_map<int, cudaMemPool_t> g_pools;

// The library's staging pool of the current device (created on first use).
cudaError_t staging_pool(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  e = cudaMemPoolCreate(&pool, &props);
  if (e != cudaSuccess) return e;
  uint64_t keep = kStagingKeep;
  e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) {
    cudaMemPoolDestroy(pool);
    return e;
  }
  g_pools[dev] = pool;
  *out = pool;
  return cudaSuccess;
}

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

cudaError_t staging_malloc(void** p, size_t bytes, cudaStream_t st) {
  cudaMemPool_t pool = nullptr;
  cudaError_t e = staging_pool(&pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, st);
}

void release_cached_memory() {
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (auto& kv : g_pools) cudaMemPoolTrimTo(kv.second, 0);
  }
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
