// Integrator: the per-pixel work of render_multiThread (src/render.cpp:
// 448-551 renderPixel, with sampleDirectLightFromFirstIntersection :425-437,
// sampleIndirectLightFromFirstIntersection :314-423 and sampleRay :121-312).
//
// Two kernels on one stream:
//  1. primary_kernel -- one thread per pixel: camera ray (no jitter, as the
//     reference), closest hit, hit shading, the +0.04-red demodulation tweak
//     of grey base colours (:492-495), G-buffer written to HBM.
//  2. path_kernel -- persistent warps claim groups of 32/K pixels from a
//     global counter; the K lanes of a pixel split its spp_direct +
//     spp_indirect sample slots round-robin. Slot j < spp_direct is light
//     sample j of the first vertex; slot spp_direct + k is indirect path k,
//     run iteratively (the reference's recursion keeps one throughput
//     product and a product of 1/(1+fails) weights). Every slot draws from
//     its own counter-based stream keyed (seed, pixel, slot), so results do
//     not depend on K or on scheduling.
//     The lanes of a pixel then reduce with warp shuffles. The reference's
//     per-pixel firefly clamp (:532-547) drops sample i iff
//     Clum_i > 16 (S - Clum_i + 1e-4) with S the sum over all samples; with
//     non-negative luminances only the largest sample can satisfy that, so
//     each lane keeps its sums without its largest sample plus that sample's
//     contribution, and the reduction merges these pairs; the surviving
//     largest sample is dropped or added at the end. No per-sample storage.
#include <algorithm>
#include <vector>

#include "rmn_host.h"
#include "shade.cuh"

namespace {

struct Params {
  float3 pos, dir, up, right;
  float acc, exposure, p_direct;
  int W, H, spp, maxd, K, spp_d;
  int tasks;
  uint64_t seed;
};

// One render of a batch: a scene, its arguments, its output buffers and its
// place in the batch's pixel and task numbering.
struct Job {
  DevScene s;
  Params p;
  float* gbuf;
  float4 *dd, *ds, *id, *is;
  int pix_begin;   // first pixel of this job in the batch's pixel numbering
  int task_begin;  // first path task (group of 32/K pixels) of this job
};

// Batch-wide counters of the counting build.
struct Counters {
  unsigned long long closest, shadow, inner, leaves, tris, slots;
};

__device__ __forceinline__ int find_job(const Job* jobs, int n, int v, bool by_task) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    int b = by_task ? __ldg(&jobs[mid].task_begin) : __ldg(&jobs[mid].pix_begin);
    if (b <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// renderPixel's demodulation tweak, src/render.cpp:492-495: a faint red is
// added to black or grey base colours (double-precision literals as there).
__device__ __forceinline__ float3 tweak_base(float3 b) {
  float c0 = dot3(b, RMN_LUM);
  if ((double)c0 < 2e-2 || (c0 < 0.8f && (double)len3(b / c0 - f3(1.0f)) < 2e-2)) b.x = (float)((double)b.x + 4e-2);
  return b;
}

__device__ __forceinline__ Surf default_surf() {
  Surf g;
  g.shapeN = f3(NAN);
  g.surfN = f3(NAN);
  g.emis = f3(0.0f);
  g.base = f3(0.0f);
  g.pos = f3(NAN);
  g.specular = 0.04f;
  g.roughness = 0.8f;
  g.metallic = 0.0f;
  g.opacity = 1.0f;
  g.eta = 1.0f;
  g.id = 0;
  g.entering = true;
  return g;
}

// G-buffer record (RMN_GBUFFER_FLOATS = 20): base[3] emission[3] position[3]
// shapeN[3] surfN[3] roughness metallic opacity eta material-id. The base
// colour is stored untweaked; path_kernel applies renderPixel's tweak for its
// own use and writes the tweaked colour back where the reference leaves it.
template <bool COUNT>
__global__ void __launch_bounds__(128) primary_kernel(const Job* __restrict__ jobs, int njobs, int total_pix,
                                                      int* status, Counters* ctr) {
  int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= total_pix) return;
  const Job& J = jobs[find_job(jobs, njobs, gi, false)];
  const DevScene& s = J.s;
  const Params& p = J.p;
  int i = gi - J.pix_begin;
  int x = i % p.W, y = i / p.W;
  float rx = float(x) - float(p.W) / 2.0f, ry = float(y) - float(p.H) / 2.0f;
  float3 d = p.dir + p.acc * (rx * p.right + ry * p.up);
  float3 D = norm3(d);
  TRay r = make_tray(p.pos, D);
  float tmax = INFINITY;
  TraceCounters tc = {0, 0, 0, 0, 0};
  int h = trace<false, COUNT>(s, r, RMN_EPS, tmax, 0.0f, &tc);
  if (h == -2) atomicExch(status, 1);
  Surf g = default_surf();
  if (h < 0) {
    if (s.sky_w) g.emis = sky_get(s, D);
  } else {
    g.pos = p.pos + tmax * D;
    hit_info(s, h, D, g);
  }
  float* o = J.gbuf + (size_t)RMN_GBUFFER_FLOATS * i;
  float v[RMN_GBUFFER_FLOATS] = {g.base.x, g.base.y, g.base.z, g.emis.x, g.emis.y, g.emis.z, g.pos.x,
                                 g.pos.y, g.pos.z, g.shapeN.x, g.shapeN.y, g.shapeN.z, g.surfN.x, g.surfN.y,
                                 g.surfN.z, g.roughness, g.metallic, g.opacity, g.eta, (float)g.id};
#pragma unroll
  for (int k = 0; k < RMN_GBUFFER_FLOATS; ++k) o[k] = v[k];
  if (COUNT) {
    atomicAdd(&ctr->closest, (unsigned long long)tc.closest);
    atomicAdd(&ctr->inner, (unsigned long long)tc.inner);
    atomicAdd(&ctr->leaves, (unsigned long long)tc.leaves);
    atomicAdd(&ctr->tris, (unsigned long long)tc.tris);
  }
}

struct Rad4 {
  float3 c;
  float v;
};
__device__ __forceinline__ Rad4 rad0() { return {f3(0.0f), 0.0f}; }
__device__ __forceinline__ void radd(Rad4& a, const Rad4& b) { a.c += b.c; a.v += b.v; }

// accumulateInwardRadiance(_basic), src/image.cpp:615-659, as the two
// contributions (diffuse part, specular part) of one sample.
__device__ __forceinline__ bool basic(float3 in, float w, Rad4& out) {
  if (!any_finite3(in) || !finite1(w)) return false;
  out.c = in * w;
  out.v = dot3(in, in) * w;
  return true;
}
__device__ __forceinline__ void demodulate(float3 base, float3 bsdf, float3 light, float w, Rad4& d, Rad4& sp) {
  d = rad0();
  sp = rad0();
  if (len3(light) < RMN_EPS) return;
  float3 b0 = norm3(base);
  if (len3(base) < RMN_EPS) {
    basic(light * bsdf, w, sp);
    return;
  }
  const float3 white = norm3(f3(1.0f));
  float xy = dot3(b0, white);
  if (xy > 0.99f) {
    basic(light * bsdf / base, w, d);
    return;
  }
  float3 perp = norm3(cross3(b0, white));
  float3 bp = bsdf - perp * dot3(perp, bsdf);
  float d1 = dot3(bp, white), d2 = dot3(bp, b0);
  float apb = (d1 + d2) / (1 + xy), amb = (d1 - d2) / (1 - xy);
  float B = (apb - amb) / 2.0f;
  float3 bb = B * b0;
  basic(light * B / len3(base), w, d);
  basic(light * (bsdf - bb), w, sp);
}

struct Acc {
  Rad4 dd, ds;    // direct diffuse / specular sums
  Rad4 id, is;    // indirect sums without the largest sample
  Rad4 mid, mis;  // the largest indirect sample's contributions
  float mclum;    // its luminance (-1: none yet)
  float S;        // luminance sum of all indirect samples
  int n;          // indirect sample count
};

__device__ __forceinline__ void acc_indirect(Acc& a, const Rad4& d, const Rad4& s, float clum) {
  a.S += clum;
  a.n += 1;
  if (clum > a.mclum) {
    if (a.mclum >= 0.0f) {
      radd(a.id, a.mid);
      radd(a.is, a.mis);
    }
    a.mid = d;
    a.mis = s;
    a.mclum = clum;
  } else {
    radd(a.id, d);
    radd(a.is, s);
  }
}

struct PathCtx {
  float3 base;   // G-buffer base colour (tweaked), demodulation reference
  float3 w0;     // first-vertex bsdf/pdf factor (LightSample::bsdfPdf)
  float3 thr;    // product of the deeper vertices' factors
  float wf;      // product of 1/(1+fails) factors
  float inv_spp; // 1 / spp_indirect
};

__device__ __forceinline__ void emit(Acc& a, const PathCtx& c, const LSample& ls) {
  float3 light = (ls.light * ls.bsdf) * c.thr;
  float w = ls.weight * c.wf * c.inv_spp;
  Rad4 d, s;
  demodulate(c.base, c.w0, light, w, d, s);
  float clum = dot3(c.w0 * light, RMN_LUM) * w;
  acc_indirect(a, d, s, clum);
}

// One indirect sample from the first vertex (sampleIndirectLightFrom-
// FirstIntersection + the sampleRay recursion) for an opaque first vertex.
template <bool COUNT>
__device__ void indirect_path(const DevScene& s, const Params& p, const Surf& g, RmnRng& rng, Acc& a, float inv_spp,
                              int* status, TraceCounters* tc) {
  if (len3(g.emis) > 0.0f) return;
  float3 in = norm3(g.pos - p.pos);
  Surf v0 = g;
  v0.eta = 1.0f / v0.eta;
  float rf = g.roughness * 1.0f;
  if (!(rng.next() < 1.0f)) return;
  PathCtx c;
  c.base = g.base;
  c.inv_spp = inv_spp;
  float3 dir;
  int f0 = 0;
  sample_reflect(v0, -in, rng, dir, c.w0, f0);
  if (!any_finite3(dir)) return;
  c.wf = f0 > 0 ? 1.0f / (float)(1 + f0) : 1.0f;
  c.thr = f3(1.0f);
  float3 o = g.pos;
  bool exclude = true;
  for (int depth = 1;; ++depth) {
    TRay r = make_tray(o, dir);
    float tmax = INFINITY;
    int h = trace<false, COUNT>(s, r, RMN_EPS, tmax, 0.0f, tc);
    if (h == -2) {
      atomicExch(status, 1);
      return;
    }
    if (h < 0) {
      if (!exclude && s.sky_w) emit(a, c, {f3(1.0f), sky_get(s, dir), 1.0f});
      return;
    }
    Surf sf = default_surf();
    sf.pos = o + dir * tmax;
    hit_info(s, h, dir, sf);
    rf = fmaxf(rf, 1.0f * sf.roughness);
    sf.roughness = fmaxf(sf.roughness, rf);
    const float p_rr = 1.0f + (0.5f - 1.0f) * sqrtf(sf.roughness);
    bool nee = p_rr < 0.9f;
    if (len3(sf.emis) > RMN_EPS) {
      if (!exclude) emit(a, c, {f3(1.0f), sf.emis, 1.0f});
      return;
    }
    if (!(rng.next() <= 1.0f)) return;
    nee = nee && sf.entering;
    const float3 V = -dir;
    if (nee && (depth >= p.maxd || rng.next() > p_rr)) {
      int cnt = c_sample_count[depth < 16 ? depth : 16];
      float k = 1.0f / 1.0f;
      if (depth < p.maxd) k /= (1.0f - p_rr);
      float lw[8];
      float tot = 0.0f;
      if (s.sky_w == 0 && !light_weights(s, sf, V, lw, tot)) return;
      for (int T = 0; T < cnt; ++T) {
        LSample ls;
        if (light_sample<COUNT>(s, sf, V, lw, tot, cnt, rng, ls, status, tc)) {
          ls.bsdf *= k;
          emit(a, c, ls);
        }
      }
      return;
    }
    float3 nd, w;
    int nf = 0;
    sample_reflect(sf, V, rng, nd, w, nf);
    w = w / 1.0f;
    if (nee) w = w / p_rr;
    if (!any_finite3(nd) || depth == p.maxd) return;
    c.thr = c.thr * w;
    if (nf > 0) c.wf = c.wf * (1.0f / (float)(1 + nf));
    o = sf.pos;
    dir = nd;
    exclude = nee;
  }
}

__device__ __forceinline__ float shfl(float v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ Rad4 shfl4(const Rad4& r, int off) {
  return {f3(shfl(r.c.x, off), shfl(r.c.y, off), shfl(r.c.z, off)), shfl(r.v, off)};
}

__device__ __forceinline__ void calc_var(Rad4& r, float e) {  // renderPixel's calcVar, src/render.cpp:510-516
  r.c *= e;
  r.v *= e * e;
  r.v -= dot3(r.c, r.c);
  if (r.v < 0.0f) r.v = 0.0f;
}

template <bool COUNT>
__global__ void __launch_bounds__(128) path_kernel(const Job* __restrict__ jobs, int njobs, int total_tasks,
                                                   unsigned int* __restrict__ next, int* status, Counters* ctr) {
  const int lane = threadIdx.x & 31;
  TraceCounters tc = {0, 0, 0, 0, 0};
  unsigned long long slots_done = 0;
  for (;;) {
    unsigned int task = 0;
    if (lane == 0) task = atomicAdd(next, 1u);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= (unsigned)total_tasks) break;
    const Job& J = jobs[find_job(jobs, njobs, (int)task, true)];
    const DevScene& s = J.s;
    const Params& p = J.p;
    const int K = p.K, P = 32 / K;
    const int sub = lane % K, grp = lane / K;
    const int npix = p.W * p.H;
    const int pixel = ((int)task - J.task_begin) * P + grp;
    const bool valid = pixel < npix;
    Acc a;
    a.dd = a.ds = a.id = a.is = a.mid = a.mis = rad0();
    a.mclum = -1.0f;
    a.S = 0.0f;
    a.n = 0;
    bool hit = false;
    Surf g = default_surf();
    if (valid) {
      const float* gb = J.gbuf + (size_t)RMN_GBUFFER_FLOATS * pixel;
      g.base = f3(gb[0], gb[1], gb[2]);
      g.emis = f3(gb[3], gb[4], gb[5]);
      g.pos = f3(gb[6], gb[7], gb[8]);
      g.shapeN = f3(gb[9], gb[10], gb[11]);
      g.surfN = f3(gb[12], gb[13], gb[14]);
      g.roughness = gb[15];
      g.metallic = gb[16];
      g.opacity = gb[17];
      g.eta = gb[18];
      g.id = (int)gb[19];
      hit = any_finite3(g.pos);
      if (hit) g.base = tweak_base(g.base);
    }
    if (hit) {
      const int spp_d = p.spp_d;
      const int spp_i = (p.spp - spp_d) * 1;  // opaque first vertex
      const int slots = spp_d + spp_i;
      const float inv_spp = 1.0f / (float)spp_i;
      const bool direct_ok = !(len3(g.emis) > 0.0f);
      float3 Vd = -norm3(g.pos - p.pos);
      float lw[8];
      float tot = 0.0f;
      bool have_w = false, w_done = false;
      for (int j = sub; j < slots; j += K) {
        RmnRng rng = rmn_rng(p.seed, (uint32_t)pixel, (uint32_t)j);
        if (COUNT) slots_done++;
        if (j < spp_d) {
          if (!direct_ok) continue;
          if (!w_done) {
            have_w = s.sky_w != 0 || light_weights(s, g, Vd, lw, tot);
            w_done = true;
          }
          if (!have_w) continue;
          LSample ls;
          if (light_sample<COUNT>(s, g, Vd, lw, tot, spp_d, rng, ls, status, &tc)) {
            Rad4 d, sp;
            demodulate(g.base, ls.bsdf, ls.light, ls.weight, d, sp);
            radd(a.dd, d);
            radd(a.ds, sp);
          }
        } else {
          indirect_path<COUNT>(s, p, g, rng, a, inv_spp, status, &tc);
        }
      }
    }
    // reduce over the K lanes of each pixel
    for (int off = K >> 1; off >= 1; off >>= 1) {
      radd(a.dd, shfl4(a.dd, off));
      radd(a.ds, shfl4(a.ds, off));
      radd(a.id, shfl4(a.id, off));
      radd(a.is, shfl4(a.is, off));
      Rad4 omid = shfl4(a.mid, off), omis = shfl4(a.mis, off);
      float om = shfl(a.mclum, off);
      a.S += shfl(a.S, off);
      a.n += __shfl_xor_sync(0xffffffffu, a.n, off);
      if (om > a.mclum) {
        if (a.mclum >= 0.0f) {
          radd(a.id, a.mid);
          radd(a.is, a.mis);
        }
        a.mid = omid;
        a.mis = omis;
        a.mclum = om;
      } else if (om >= 0.0f) {
        radd(a.id, omid);
        radd(a.is, omis);
      }
    }
    if (valid && sub == 0) {
      if (hit) {
        calc_var(a.dd, p.exposure);
        calc_var(a.ds, p.exposure);
        if (a.n > 0) {
          if (!(a.mclum / (a.S - a.mclum + RMN_EPS) > 16.0f)) {
            radd(a.id, a.mid);
            radd(a.is, a.mis);
          }
          calc_var(a.id, p.exposure);
          calc_var(a.is, p.exposure);
        } else {
          // renderPixel restores the untweaked base colour only after
          // accumulating indirect samples; with none it returns early
          // (src/render.cpp:517-518) and the tweak stays in the G-buffer.
          J.gbuf[(size_t)RMN_GBUFFER_FLOATS * pixel] = g.base.x;
        }
      }
      J.dd[pixel] = make_float4(a.dd.c.x, a.dd.c.y, a.dd.c.z, a.dd.v);
      J.ds[pixel] = make_float4(a.ds.c.x, a.ds.c.y, a.ds.c.z, a.ds.v);
      J.id[pixel] = make_float4(a.id.c.x, a.id.c.y, a.id.c.z, a.id.v);
      J.is[pixel] = make_float4(a.is.c.x, a.is.c.y, a.is.c.z, a.is.v);
    }
  }
  if (COUNT) {
    atomicAdd(&ctr->closest, (unsigned long long)tc.closest);
    atomicAdd(&ctr->shadow, (unsigned long long)tc.shadow);
    atomicAdd(&ctr->inner, (unsigned long long)tc.inner);
    atomicAdd(&ctr->leaves, (unsigned long long)tc.leaves);
    atomicAdd(&ctr->tris, (unsigned long long)tc.tris);
    atomicAdd(&ctr->slots, slots_done);
  }
}

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

int path_blocks_per_sm() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, path_kernel<false>, 128, 0);
  return per_sm < 1 ? 1 : per_sm;
}

}  // namespace

namespace rmn {

// Lanes per pixel: the fewest (each lane then owns more of the pixel's
// sample slots, which balances the warp and amortises per-pixel set-up) that
// still yield about four waves of warps over the whole batch.
int default_lanes_per_pixel(int64_t batch_pixels, int spp) {
  const int64_t resident_warps = (int64_t)device_sms() * path_blocks_per_sm() * 4;
  int k = 1;
  while (k < 32 && k * 2 <= (spp > 0 ? spp : 1) && batch_pixels * k / 32 < 4 * resident_warps) k *= 2;
  return k;
}

struct JobTable {
  std::vector<Job> jobs;
  int total_pix = 0, total_tasks = 0;
};

struct BatchState {
  JobTable table;
  Job* d_jobs = nullptr;
  unsigned int* d_next = nullptr;
  int* d_status = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static Params make_params(const rmn_render_args& a, int K) {
  Params p;
  p.pos = f3(a.position[0], a.position[1], a.position[2]);
  p.dir = f3(a.direction[0], a.direction[1], a.direction[2]);
  p.up = f3(a.up[0], a.up[1], a.up[2]);
  p.right = f3(a.right[0], a.right[1], a.right[2]);
  p.acc = a.accuracy;
  p.exposure = a.exposure;
  p.p_direct = a.P_Direct;
  p.W = a.width;
  p.H = a.height;
  p.spp = a.spp;
  p.maxd = a.max_depth;
  p.spp_d = (int)((float)a.spp * a.P_Direct);  // renderPixel, src/render.cpp:497
  p.K = K;
  p.seed = a.seed;
  const int npix = p.W * p.H;
  p.tasks = (npix + (32 / K) - 1) / (32 / K);
  return p;
}

// Jobs ordered by decreasing cost per task (spp x depth), so the persistent
// warps finish on the cheap tasks; the result does not depend on the order.
static void build_jobs(const RenderItem* items, int n, JobTable* t) {
  int64_t batch_pixels = 0;
  for (int i = 0; i < n; ++i) batch_pixels += (int64_t)items[i].args.width * items[i].args.height;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  auto cost = [&](int i) {
    const rmn_render_args& a = items[i].args;
    int K = a.lanes_per_pixel > 0 ? a.lanes_per_pixel : default_lanes_per_pixel(batch_pixels, a.spp);
    return (double)a.spp * a.max_depth * (32 / K);
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
  t->jobs.clear();
  t->total_pix = t->total_tasks = 0;
  for (int i : order) {
    const RenderItem& it = items[i];
    int K = it.args.lanes_per_pixel > 0 ? it.args.lanes_per_pixel : default_lanes_per_pixel(batch_pixels, it.args.spp);
    Job j;
    j.s = it.scene->dev;
    j.p = make_params(it.args, K);
    j.gbuf = it.gbuf;
    j.dd = reinterpret_cast<float4*>(it.dd);
    j.ds = reinterpret_cast<float4*>(it.ds);
    j.id = reinterpret_cast<float4*>(it.id);
    j.is = reinterpret_cast<float4*>(it.is);
    j.pix_begin = t->total_pix;
    j.task_begin = t->total_tasks;
    t->total_pix += j.p.W * j.p.H;
    t->total_tasks += j.p.tasks;
    t->jobs.push_back(j);
  }
}

// Launch sequence of a batch: reset the task counter, primary kernel over
// every pixel of every job, then the persistent path kernel. With `ctr`
// the counting build runs (same images, plus visit counters).
static cudaError_t launch_jobs(const void* d_jobs, int njobs, int total_pix, int total_tasks, unsigned int* d_next,
                        int* d_status, void* d_ctr, cudaStream_t stream, cudaEvent_t* ev) {
  const Job* jobs = static_cast<const Job*>(d_jobs);
  Counters* ctr = static_cast<Counters*>(d_ctr);
  cudaError_t e = cudaMemsetAsync(d_next, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[0], stream);
  if (ctr) primary_kernel<true><<<(total_pix + 127) / 128, 128, 0, stream>>>(jobs, njobs, total_pix, d_status, ctr);
  else primary_kernel<false><<<(total_pix + 127) / 128, 128, 0, stream>>>(jobs, njobs, total_pix, d_status, ctr);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[1], stream);
  int blocks = device_sms() * path_blocks_per_sm();
  int need = (total_tasks + 3) / 4;
  if (need < blocks) blocks = need < 1 ? 1 : need;
  if (ctr) path_kernel<true><<<blocks, 128, 0, stream>>>(jobs, njobs, total_tasks, d_next, d_status, ctr);
  else path_kernel<false><<<blocks, 128, 0, stream>>>(jobs, njobs, total_tasks, d_next, d_status, ctr);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[2], stream);
  return cudaSuccess;
}

rmn_status batch_create(const RenderItem* items, int n, bool use_graph, cudaStream_t st, BatchState** out) {
  *out = nullptr;
  BatchState* b = new BatchState();
  build_jobs(items, n, &b->table);
  const size_t jb = sizeof(Job) * b->table.jobs.size();
  cudaError_t e = cudaMalloc(&b->d_jobs, jb);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_next, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_jobs, b->table.jobs.data(), jb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(int));
  if (e == cudaSuccess && use_graph) {
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
      e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t le = launch_jobs(b->d_jobs, (int)b->table.jobs.size(), b->table.total_pix, b->table.total_tasks,
                                     b->d_next, b->d_status, nullptr, cs, nullptr);
        e = cudaStreamEndCapture(cs, &b->graph);
        if (e == cudaSuccess) e = le;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
      cudaStreamDestroy(cs);
    }
  }
  if (e != cudaSuccess) {
    batch_destroy(b);
    return cuda_fail(e, "batch setup");
  }
  (void)st;
  *out = b;
  return RMN_OK;
}

rmn_status batch_launch(BatchState* b, cudaStream_t st) {
  cudaError_t e;
  if (b->exec) e = cudaGraphLaunch(b->exec, st);
  else
    e = launch_jobs(b->d_jobs, (int)b->table.jobs.size(), b->table.total_pix, b->table.total_tasks, b->d_next,
                    b->d_status, nullptr, st, nullptr);
  return e == cudaSuccess ? RMN_OK : cuda_fail(e, "batch launch");
}

rmn_status batch_status(BatchState* b, cudaStream_t st) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "render");
  if (h) return fail(RMN_ERR_DEVICE_LIMIT, "render: traversal stack bound reached");
  return RMN_OK;
}

// Counting run (visit counters) followed by a timed run with CUDA events
// around each kernel on `st`. Both produce the same images as batch_launch.
rmn_status batch_profile(BatchState* b, cudaStream_t st, RenderProfileData* prof) {
  Counters* d_ctr = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  cudaError_t e = cudaMalloc(&d_ctr, sizeof(Counters));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, sizeof(Counters), st);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaEventCreate(&ev[k]);
  const int nj = (int)b->table.jobs.size();
  if (e == cudaSuccess)
    e = launch_jobs(b->d_jobs, nj, b->table.total_pix, b->table.total_tasks, b->d_next, b->d_status, d_ctr, st,
                    nullptr);
  if (e == cudaSuccess)
    e = launch_jobs(b->d_jobs, nj, b->table.total_pix, b->table.total_tasks, b->d_next, b->d_status, nullptr, st, ev);
  Counters h{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    float a = 0.0f, c = 0.0f;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&c, ev[1], ev[2]);
    prof->primary_ms = a;
    prof->path_ms = c;
    prof->closest = h.closest;
    prof->shadow = h.shadow;
    prof->inner = h.inner;
    prof->leaves = h.leaves;
    prof->tris = h.tris;
    prof->slots = h.slots;
    prof->pixels = (unsigned long long)b->table.total_pix;
  }
  for (int k = 0; k < 3; ++k)
    if (ev[k]) cudaEventDestroy(ev[k]);
  if (d_ctr) cudaFree(d_ctr);
  return e == cudaSuccess ? RMN_OK : cuda_fail(e, "render profile");
}

void batch_destroy(BatchState* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_jobs) cudaFree(b->d_jobs);
  if (b->d_next) cudaFree(b->d_next);
  if (b->d_status) cudaFree(b->d_status);
  delete b;
}

}  // namespace rmn
