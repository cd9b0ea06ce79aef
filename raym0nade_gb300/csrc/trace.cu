// Ray-query kernels: closest hit (Model::rayHit, src/model.cpp:332-341) and
// occlusion (Model::rayHit_test, src/model.cpp:343-354) over ray batches in
// HBM.
//
// Work distribution: a persistent grid (a multiple of the SM count) whose
// warps claim 32-ray batches from a global counter, so warps that drew short
// rays move on instead of idling while long rays of a static partition
// finish.
#include "rmn_host.h"
#include "trace.cuh"

namespace {

__device__ __forceinline__ float int_float(int i) { return __int_as_float(i); }

template <bool SHADOW>
__global__ void __launch_bounds__(128) trace_kernel(DevScene s, const float4* __restrict__ rays, int64_t n,
                                                    float4* __restrict__ hits, uint8_t* __restrict__ occ,
                                                    unsigned long long* __restrict__ next, int* status) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(next, 32ULL);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned long long)n) return;
    int64_t i = (int64_t)base + lane;
    if (i >= n) continue;
    float4 r0 = __ldg(rays + 2 * i), r1 = __ldg(rays + 2 * i + 1);
    TRay r = make_tray(f3(r0.x, r0.y, r0.z), f3(r1.x, r1.y, r1.z));
    if (SHADOW) {
      // HitRecord(eps, aimDepth + eps); occluded iff the hit is nearer than aimDepth.
      float aim = r1.w;
      float tmax = aim + RMN_EPS;
      int h = trace<true, false>(s, r, RMN_EPS, tmax, aim, nullptr);
      if (h == -2) atomicExch(status, (int)rmn::kDevStackOverflow);
      occ[i] = (tmax >= aim) ? 0 : 1;
    } else {
      float tmax = r1.w;
      int h = trace<false, false>(s, r, r0.w, tmax, 0.0f, nullptr);
      if (h == -2) atomicExch(status, (int)rmn::kDevStackOverflow);
      if (h < 0) {
        hits[i] = make_float4(int_float(-1), tmax, 0.0f, 0.0f);
      } else {
        const float4* t = s.tri + 3 * h;
        float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
        float3 bc = bary(f3(a), f3(b), f3(c), r.o + r.d * tmax);
        hits[i] = make_float4(a.w, tmax, bc.y, bc.z);
      }
    }
  }
}

int persistent_blocks(const void* kernel, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

cudaError_t launch(bool shadow, const DevScene& s, const rmn_ray* rays, int64_t n, rmn_hit* hits, uint8_t* occ,
                   int* status, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  unsigned long long* next = nullptr;
  cudaError_t e = cudaMallocAsync(&next, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), stream);
  if (e == cudaSuccess) {
    const int threads = 128;
    if (shadow) {
      int blocks = persistent_blocks((const void*)trace_kernel<true>, threads);
      int64_t need = (n + threads - 1) / threads;
      if (need < blocks) blocks = (int)need;
      trace_kernel<true><<<blocks, threads, 0, stream>>>(s, reinterpret_cast<const float4*>(rays), n, nullptr, occ,
                                                         next, status);
    } else {
      int blocks = persistent_blocks((const void*)trace_kernel<false>, threads);
      int64_t need = (n + threads - 1) / threads;
      if (need < blocks) blocks = (int)need;
      trace_kernel<false><<<blocks, threads, 0, stream>>>(s, reinterpret_cast<const float4*>(rays), n,
                                                          reinterpret_cast<float4*>(hits), nullptr, next, status);
    }
    e = cudaGetLastError();
  }
  cudaError_t f = cudaFreeAsync(next, stream);
  return e != cudaSuccess ? e : f;
}

}  // namespace

namespace rmn {
cudaError_t launch_trace_closest(const DevScene& s, const rmn_ray* rays, int64_t n, rmn_hit* hits, int* status,
                                 cudaStream_t stream) {
  return launch(false, s, rays, n, hits, nullptr, status, stream);
}
cudaError_t launch_trace_shadow(const DevScene& s, const rmn_ray* rays, int64_t n, uint8_t* occluded, int* status,
                                cudaStream_t stream) {
  return launch(true, s, rays, n, nullptr, occluded, status, stream);
}
}  // namespace rmn
