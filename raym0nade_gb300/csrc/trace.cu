// Ray-query kernels: closest hit (Model::rayHit, src/model.cpp:332-341) and
// occlusion (Model::rayHit_test, src/model.cpp:343-354) over ray batches in
// HBM. In scenes with alpha-tested materials, occlusion queries and closest
// queries over (eps, inf) -- Model::rayHit's interval -- retry past cut-away
// hits as the reference does; other intervals are bare BVH queries.
//
// Work distribution: a persistent grid (a multiple of the SM count). Each
// lane owns one ray at a time; after every round of inner-node steps and
// warp-cooperative leaf tests (trace.cuh, coop_nodes / coop_leaves) the
// lanes whose ray is answered take new rays from a global counter (one
// warp-aggregated atomic), so a warp no longer waits for its longest ray
// (Aila & Laine, "Understanding the efficiency of ray traversal on GPUs",
// HPG 2009: persistent threads with dynamic ray fetch).
#include "rmn_host.h"
#include "trace.cuh"

namespace {

// STACK: shared stack entries (RMN_STACK_SMALL for trees that fit it: one
// more block per SM).
template <bool SHADOW, int STACK>
__global__ void __launch_bounds__(128, RMN_COOP_BLOCKS(STACK)) trace_kernel(DevScene s, const float4* __restrict__ rays, int64_t n,
                                                    float4* __restrict__ hits, uint8_t* __restrict__ occ,
                                                    unsigned long long* __restrict__ next, int* status) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  bool active = false, retired = false;
  int64_t i = 0;
  TRay r;
  float tmin = 0.0f, aim = 0.0f, restart = 0.0f;
  int searches = 0;
  bool retry = false;
  // the deferred-child stack in shared memory (launched with 128 threads)
  // and the leaf-phase keys of each warp
  __shared__ int2 sstack[STACK * 128];
  __shared__ unsigned long long skeys[128];
  TravT<SharedStackN<STACK>> t;
  t.stack.base = sstack + threadIdx.x;
  t.ti = t.te = 0;
  unsigned long long* keys = skeys + (threadIdx.x & ~31);
  for (;;) {
    // lanes without a ray take the next ones from the batch
    unsigned need = __ballot_sync(0xffffffffu, !active && !retired);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !retired) {
        i = (int64_t)(base + __popc(need & lt));
        if (i < n) {
          float4 r0 = __ldg(rays + 2 * i), r1 = __ldg(rays + 2 * i + 1);
          r = make_tray(f3(r0.x, r0.y, r0.z), f3(r1.x, r1.y, r1.z));
          if (SHADOW) {
            // HitRecord(eps, aimDepth + eps); occluded iff nearer than aimDepth.
            tmin = RMN_EPS;
            aim = r1.w;
            restart = aim + RMN_EPS;
            retry = s.has_alpha != 0;
          } else {
            tmin = r0.w;
            restart = r1.w;
            retry = s.has_alpha && r0.w == RMN_EPS && isinf(r1.w) && r1.w > 0.0f;
          }
          trav_begin(s, t, restart);
          searches = 0;
          active = true;
        } else {
          retired = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, active) == 0) return;
    int st = coop_nodes<false>(s.nodes, r, tmin, t, active, kCoopSteps, nullptr);
    if (coop_leaves<SHADOW, true>(s.tri, r, tmin, aim, t, !retry, keys)) st = 1;
    if (!active || st == 0) continue;
    if (st == -2) atomicExch(status, (int)rmn::kDevStackOverflow);
    else if (retry && !(SHADOW && t.tmax >= aim) && alpha_again(s, r, t, tmin, restart, searches, !SHADOW)) continue;
    if (SHADOW) {
      occ[i] = (t.tmax >= aim) ? 0 : 1;
    } else if (t.hit < 0) {
      hits[i] = make_float4(__int_as_float(-1), t.tmax, 0.0f, 0.0f);
    } else {
      const float4* tp = s.tri + 3 * t.hit;
      float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
      float3 bc = bary(f3(a), f3(b), f3(c), r.o + r.d * t.tmax);
      hits[i] = make_float4(a.w, t.tmax, bc.y, bc.z);
    }
    active = false;
  }
}

// Occlusion queries of a scene without alpha-tested materials: pending
// leaves, order-free (trace.cuh, occ_nodes / occ_leaves).
template <int STACK>
__global__ void __launch_bounds__(128, RMN_OCC_BLOCKS) occ_kernel(DevScene s, const float4* __restrict__ rays,
                                                                          int64_t n, uint8_t* __restrict__ occ,
                                                                          unsigned long long* __restrict__ next,
                                                                          int* status) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  bool active = false, retired = false;
  int64_t i = 0;
  TRay r;
  float aim = 0.0f;
  __shared__ int sstack[STACK * 128];  // node references: occlusion pops skip nothing
  __shared__ OccExchange xch;
  OccT<SharedStackRefN<STACK>> t;
  t.stack.base = sstack + threadIdx.x;
  t.c0 = t.c1 = 0;
  for (;;) {
    unsigned need = __ballot_sync(0xffffffffu, !active && !retired);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !retired) {
        i = (int64_t)(base + __popc(need & lt));
        if (i < n) {
          float4 r0 = __ldg(rays + 2 * i), r1 = __ldg(rays + 2 * i + 1);
          r = make_tray(f3(r0.x, r0.y, r0.z), f3(r1.x, r1.y, r1.z));
          aim = r1.w;
          occ_begin(s.root, t);
          active = true;
        } else {
          retired = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, active) == 0) return;
    // HitRecord(eps, aimDepth + eps); occluded iff a hit is nearer than aimDepth
    const int st = occ_nodes<false>(s.nodes, r, RMN_EPS, aim + RMN_EPS, t, active, kOccSteps, nullptr);
    const bool o = occ_leaves<true>(s.tri, r, RMN_EPS, aim, t, xch);
    if (!active || (st == 0 && !o)) continue;
    if (st == -2) atomicExch(status, (int)rmn::kDevStackOverflow);
    occ[i] = (o && st != -2) ? 1 : 0;
    active = false;
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

template <bool SHADOW, int STACK>
void launch_kernel(const DevScene& s, const float4* rays, int64_t n, float4* hits, uint8_t* occ,
                   unsigned long long* next, int* status, cudaStream_t stream) {
  const int threads = 128;
  const bool order_free = SHADOW && !s.has_alpha;
  int blocks = order_free ? persistent_blocks((const void*)occ_kernel<STACK>, threads)
                          : persistent_blocks((const void*)trace_kernel<SHADOW, STACK>, threads);
  int64_t need = (n + threads - 1) / threads;
  if (need < blocks) blocks = (int)need;
  if (order_free) occ_kernel<STACK><<<blocks, threads, 0, stream>>>(s, rays, n, occ, next, status);
  else trace_kernel<SHADOW, STACK><<<blocks, threads, 0, stream>>>(s, rays, n, hits, occ, next, status);
}

cudaError_t launch(bool shadow, const DevScene& s, const rmn_ray* rays, int64_t n, rmn_hit* hits, uint8_t* occ,
                   int* status, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  unsigned long long* next = nullptr;
  cudaError_t e = rmn::staging_malloc(reinterpret_cast<void**>(&next), sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), stream);
  if (e == cudaSuccess) {
    const float4* r = reinterpret_cast<const float4*>(rays);
    float4* h = reinterpret_cast<float4*>(hits);
    const bool shallow = s.depth + 1 <= RMN_STACK_SMALL;
    if (shadow) {
      if (shallow) launch_kernel<true, RMN_STACK_SMALL>(s, r, n, nullptr, occ, next, status, stream);
      else launch_kernel<true, RMN_STACK>(s, r, n, nullptr, occ, next, status, stream);
    } else {
      if (shallow) launch_kernel<false, RMN_STACK_SMALL>(s, r, n, h, nullptr, next, status, stream);
      else launch_kernel<false, RMN_STACK>(s, r, n, h, nullptr, next, status, stream);
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
