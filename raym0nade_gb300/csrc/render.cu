// Integrator: the per-pixel work of render_multiThread (src/render.cpp:
// 448-551 renderPixel, with sampleDirectLightFromFirstIntersection :425-437,
// sampleIndirectLightFromFirstIntersection :314-423 and sampleRay :121-312),
// as a wavefront over a batch of renders ("jobs").
//
// Work. A pixel's spp_direct + spp_indirect sample slots (slot j <
// spp_direct: light sample j of the first vertex; slot spp_direct + k:
// indirect path k) are cut into units of up to S consecutive slots. Every
// slot draws from its own counter-based stream keyed (seed, pixel, slot), so
// results do not depend on how slots are grouped or scheduled.
//
// Kernels, on one stream:
//  1. primary_kernel  -- one thread per pixel of every job: camera ray (no
//     jitter, as the reference), closest hit, hit shading -> G-buffer.
//  2. per iteration, until no worker is left, over a pool of W workers
//     (path state in HBM, structure of arrays):
//     shade_kernel, bounce_kernel, nee_kernel, slot_kernel, light_kernel,
//     path_kernel --
//                        the integrator's logic, split by phase so that each
//                        kernel runs over a compacted list of the workers in
//                        its phase (see below); a worker ends the iteration
//                        with a ray queued, retired, or (rarely) handed to
//                        the next iteration's slot_kernel;
//     qtrace_kernel<closest>, qocc_kernel (qtrace_kernel<shadow> in batches
//                        with alpha-tested materials) -- persistent traversal
//                        of the ray queues with per-lane dynamic ray fetch.
//     Traversal thus runs at the occupancy of a 64-register kernel, and the
//     shading code runs on warps of one phase each.
//  3. finalize_kernel -- per pixel, merges its units' partial accumulators
//     in unit order and writes the four RadianceData buffers.
//
// Firefly clamp (:532-547): the reference drops sample i iff
// Clum_i > 16 (S - Clum_i + 1e-4), S the luminance sum over the pixel's
// indirect samples. With non-negative luminances only the largest sample can
// satisfy that, so every unit keeps its sums without its largest sample plus
// that sample's contributions; finalize merges these pairs and drops or adds
// the surviving largest sample. No per-sample storage.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "rmn_host.h"
#include "integrator.cuh"

namespace {


// One render of a batch: a scene, its arguments, its output buffers and its
// place in the batch's pixel and unit numbering.
struct Job {
  DevScene s;
  Params p;
  float* gbuf;
  float4 *dd, *ds, *id, *is;
  int* dropped;          // optional: per pixel, the sample the firefly clamp dropped
  int pix_begin;         // first pixel of this job in the batch
  long long unit_begin;  // first unit of this job in the batch
};

// Batch-wide counters of the counting build.
struct Counters {
  unsigned long long closest, shadow, inner, leaves, tris, slots;
};

// Queue lengths of one iteration parity; cleared when an iteration of that
// parity starts.
struct QLen {
  unsigned int c, sn;           // ray queues: closest, shadow
  unsigned int sd, nw;          // workers waiting for first-vertex / NEE shadow answers
  unsigned int nee, slot;       // hand-offs to nee_kernel / slot_kernel within the iteration
  unsigned int light, path;     // hand-offs from slot_kernel to light_kernel / path_kernel
  unsigned int bounce;          // hand-off from shade_kernel to bounce_kernel
  unsigned int c_next, s_next;  // fetch cursors of the trace kernels
};
// Control words of one lane (an independent wavefront over its own share of
// the worker pool; a batch runs its lanes concurrently).
struct Ctl {
  QLen q[2];
};
constexpr int kMaxLanes = 4;
struct CtlBlock {
  unsigned long long next_unit;  // unit cursor shared by all lanes, runs over the whole render
  unsigned long long pad;
  Ctl lane[kMaxLanes];
};

// Worker-id lists. The ray queues are double-buffered by iteration parity.
struct Queues {
  int* c[2];   // closest-hit rays (worker ids)
  int* sn[2];  // shadow rays (~ray ids, kDirectBatch per worker)
  int* sd[2];  // workers waiting for first-vertex light samples (and the first iteration's seed)
  int* nw[2];  // workers waiting for their terminating vertex's light samples
  int* nee;
  int* slot;
  int* light;
  int* path;
  int* bounce;
};

// Worker pool in HBM (structure of arrays).
struct Pool {
  int W;
  // the worker's header, 2 per worker in one 32-byte sector, read and
  // written whole by every logic kernel: (job, pixel, j = current slot, j1 =
  // end of unit), (rng counter, phase | depth << 4 | flags << 12, global
  // unit index = the partial record, low and high word)
  int4* hdr;
  float4* ro;      // ray origin, t_min
  float4* rd;      // ray direction, t_max (closest) or aim depth (shadow)
  float2* res;     // closest: (leaf-order triangle, t); shadow: (occluded, -)
  float4* pa;      // first-vertex factor w0, weight product wf
  float4* pb;      // throughput product, roughness factor
  float4* nv;      // 6 per worker: NEE vertex pos|kscale, shapeN|rough, surfN|metal, base|eta, V|tot, absorb|opacity
  float4* lw;      // 2 per worker: light weights 0..7
  int4* nk;        // NEE sample k, count
  // shadow rays, up to kDirectBatch per worker in flight: first-vertex or
  // terminating-vertex light samples (ray r of worker w at
  // w * kDirectBatch + r); origin in ro
  float4* drd;     // direction, aim depth
  float4* dpend;   // 2 per ray: bsdf|weight, light|sample index
  float* dres;     // 1: occluded
  int2* dk;        // slots the batch covers, rays it queued
  // the media a path is inside (scenes with transmissive materials)
  int* mn;         // count
  int* mid;        // RMN_MEDIA per worker: material id (air -1)
  float4* mval;    // RMN_MEDIA per worker: ior, absorb
  // the differential of the path's current ray (scenes with textures):
  // 3 per worker, (dPdx, dPdy.x), (dPdy.yz, dDdx.xy), (dDdx.z, dDdy)
  float4* rdiff;
};

__device__ __forceinline__ RayDiff load_diff(const Pool& P, int w) {
  const float4 a = P.rdiff[3 * (size_t)w], b = P.rdiff[3 * (size_t)w + 1], c = P.rdiff[3 * (size_t)w + 2];
  return {f3(a.x, a.y, a.z), f3(a.w, b.x, b.y), f3(b.z, b.w, c.x), f3(c.y, c.z, c.w)};
}
__device__ __forceinline__ void store_diff(const Pool& P, int w, const RayDiff& d) {
  P.rdiff[3 * (size_t)w] = make_float4(d.dPdx.x, d.dPdx.y, d.dPdx.z, d.dPdy.x);
  P.rdiff[3 * (size_t)w + 1] = make_float4(d.dPdy.y, d.dPdy.z, d.dDdx.x, d.dDdx.y);
  P.rdiff[3 * (size_t)w + 2] = make_float4(d.dDdx.z, d.dDdy.x, d.dDdy.y, d.dDdy.z);
}

// Partial accumulator of one unit: 7 float4.
//   [0] Dd  [1] Ds  [2] Id without the largest sample  [3] Is likewise
//   [4] Id of the largest  [5] Is of the largest
//   [6] (its Clum or -1, S, n, its sample id = slot * 8 + index in the path's samples)
#define RMN_PART_F4 7

enum Phase { PH_FETCH = 0, PH_SLOT, PH_WAIT_DIRECT, PH_WAIT_CLOSEST, PH_NEE, PH_WAIT_NEE, PH_DONE, PH_BOUNCE };

// First-vertex light samples a worker draws at once: consecutive direct
// slots of its unit, each with its own shadow ray in the same queue.
constexpr int kDirectBatch = 8;  // also holds a terminating vertex's samples (sampleCount <= 6)
enum Flags { FL_EXCLUDE = 1 };

__device__ __forceinline__ int find_job_pix(const Job* jobs, int n, int v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&jobs[mid].pix_begin) <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ int find_job_unit(const Job* jobs, int n, long long v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&jobs[mid].unit_begin) <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}



// G-buffer record (RMN_GBUFFER_FLOATS = 21): base[3] emission[3] position[3]
// shapeN[3] surfN[3] roughness metallic opacity eta material-id entering. The base
// colour is stored untweaked; the integrator applies renderPixel's tweak for
// its own use and finalize writes the tweaked colour back where the
// reference leaves it. TEX: the batch has textured scenes (a separate build,
// so untextured batches keep the lean kernel).
template <bool COUNT, bool TEX>
__global__ void __launch_bounds__(128) primary_kernel(const Job* __restrict__ jobs, int njobs, int total_pix,
                                                      int* status, Counters* ctr) {
  int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= total_pix) return;
  const Job& J = jobs[find_job_pix(jobs, njobs, gi)];
  const DevScene& s = J.s;
  const Params& p = J.p;
  int i = gi - J.pix_begin;
  int x = i % p.W, y = i / p.W;
  float3 d = pixel_dir(p, x, y);
  float3 D = norm3(d);
  TRay r = make_tray(p.pos, D);
  float tmax = INFINITY;
  TraceCounters tc = {0, 0, 0, 0, 0};
  int h = trace<false, COUNT, TEX>(s, r, RMN_EPS, tmax, 0.0f, &tc);
  if (h == -2) atomicExch(status, 1);
  Surf g = default_surf();
  if (h < 0) {
    if (s.sky_w) g.emis = sky_get(s, D);
  } else {
    g.pos = p.pos + tmax * D;
    if (TEX && s.has_tex) {
      float3 px, py;
      hit_info_tex(s, h, D, tmax, init_ray_diff(p, d), g, px, py);
    } else {
      hit_info(s, h, D, g);
    }
  }
  float* o = J.gbuf + (size_t)RMN_GBUFFER_FLOATS * i;
  float v[RMN_GBUFFER_FLOATS] = {g.base.x, g.base.y, g.base.z, g.emis.x, g.emis.y, g.emis.z, g.pos.x,
                                 g.pos.y, g.pos.z, g.shapeN.x, g.shapeN.y, g.shapeN.z, g.surfN.x, g.surfN.y,
                                 g.surfN.z, g.roughness, g.metallic, g.opacity, g.eta, (float)g.id,
                                 g.entering ? 1.0f : 0.0f};
#pragma unroll
  for (int k = 0; k < RMN_GBUFFER_FLOATS; ++k) o[k] = v[k];
  if (COUNT) {
    atomicAdd(&ctr->closest, (unsigned long long)tc.closest);
    atomicAdd(&ctr->inner, (unsigned long long)tc.inner);
    atomicAdd(&ctr->leaves, (unsigned long long)tc.leaves);
    atomicAdd(&ctr->tris, (unsigned long long)tc.tris);
  }
}


// The largest-sample bookkeeping shared by emit (one sample into a unit) and
// finalize (unit into pixel).
struct Ind {
  Rad4 id, is, mid, mis;
  float mclum, S;
  int n, mid_sample;
};
__device__ __forceinline__ void ind_add(Ind& a, const Rad4& d, const Rad4& s, float clum, float S, int n, int sid) {
  a.S += S;
  a.n += n;
  if (clum > a.mclum) {
    if (a.mclum >= 0.0f) {
      radd(a.id, a.mid);
      radd(a.is, a.mis);
    }
    a.mid = d;
    a.mis = s;
    a.mclum = clum;
    a.mid_sample = sid;
  } else if (clum >= 0.0f) {
    radd(a.id, d);
    radd(a.is, s);
  }
}

__device__ __forceinline__ const float* gbuf_of(const Job& J, int pixel) {
  return J.gbuf + (size_t)RMN_GBUFFER_FLOATS * pixel;
}
__device__ __forceinline__ float3 base_of(const Job& J, int pixel) {
  const float* gb = gbuf_of(J, pixel);
  return tweak_base(f3(gb[0], gb[1], gb[2]));
}
// The base colour indirect samples are demodulated against: none behind a
// transmissive first vertex (renderPixel, src/render.cpp:543-546).
__device__ __forceinline__ float3 indirect_base_of(const Job& J, int pixel) {
  const float* gb = gbuf_of(J, pixel);
  if (J.p.glass && gb[17] < RMN_EPS) return f3(0.0f);
  return tweak_base(f3(gb[0], gb[1], gb[2]));
}
// 1 / spp_indirect of the pixel: 16 times the samples behind a transmissive
// or half-opaque first vertex (src/render.cpp:497-499).
__device__ __forceinline__ float inv_spp_of(const Job& J, int pixel) {
  if (!J.p.glass) return J.p.inv_spp;
  return gbuf_of(J, pixel)[17] > 1.0f - RMN_EPS ? J.p.inv_spp : J.p.inv_spp16;
}

// The worker's media (scenes with transmissive materials only).
__device__ __forceinline__ void load_media(const Pool& P, int w, Media& m) {
  m.n = P.mn[w];
  m.ok = true;
  for (int i = 0; i < m.n && i < RMN_MEDIA; ++i) {
    m.id[i] = P.mid[(size_t)w * RMN_MEDIA + i];
    m.v[i] = P.mval[(size_t)w * RMN_MEDIA + i];
  }
}
__device__ __forceinline__ void store_media(const Pool& P, int w, const Media& m) {
  P.mn[w] = m.n;
  for (int i = 0; i < m.n; ++i) {
    P.mid[(size_t)w * RMN_MEDIA + i] = m.id[i];
    P.mval[(size_t)w * RMN_MEDIA + i] = m.v[i];
  }
}

__device__ __forceinline__ Surf load_first_vertex(const Job& J, int pixel) {
  const float* gb = gbuf_of(J, pixel);
  Surf g = default_surf();
  g.base = tweak_base(f3(gb[0], gb[1], gb[2]));
  g.emis = f3(gb[3], gb[4], gb[5]);
  g.pos = f3(gb[6], gb[7], gb[8]);
  g.shapeN = f3(gb[9], gb[10], gb[11]);
  g.surfN = f3(gb[12], gb[13], gb[14]);
  g.roughness = gb[15];
  g.metallic = gb[16];
  g.opacity = gb[17];
  g.eta = gb[18];
  g.id = (int)gb[19];
  g.entering = gb[20] != 0.0f;
  return g;
}

// One indirect light sample into the unit's partial record: light and
// weight finished as passBsdf/mulWeight would (src/render.cpp:101-116),
// demodulated against the first vertex's (tweaked) base colour with the
// first-vertex factor w0 as LightSample::bsdfPdf.
__device__ void emit(float4* part, float3 base, float4 pa, float3 thr, float inv_spp, const LSample& ls, int sid) {
  float3 w0 = f3(pa.x, pa.y, pa.z);
  float3 light = (ls.light * ls.bsdf) * thr;
  float w = ls.weight * pa.w * inv_spp;
  Rad4 d, s;
  demodulate(base, w0, light, w, d, s);
  float clum = dot3(w0 * light, RMN_LUM) * w;
  Ind a;
  a.id = r4(part[2]);
  a.is = r4(part[3]);
  a.mid = r4(part[4]);
  a.mis = r4(part[5]);
  float4 m = part[6];
  a.mclum = m.x;
  a.S = m.y;
  a.n = __float_as_int(m.z);
  a.mid_sample = __float_as_int(m.w);
  ind_add(a, d, s, clum, clum, 1, sid);
  part[2] = f4(a.id);
  part[3] = f4(a.is);
  part[4] = f4(a.mid);
  part[5] = f4(a.mis);
  part[6] = make_float4(a.mclum, a.S, __int_as_float(a.n), __int_as_float(a.mid_sample));
}

// Warp-aggregated increment: the lanes that reach the call together take
// consecutive values with one atomic (single-address atomics would otherwise
// serialise a million workers per iteration).
template <class T>
__device__ __forceinline__ T agg_inc(T* ctr) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  T base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(ctr, (T)g.size());
  base = g.shfl(base, 0);
  return base + (T)g.thread_rank();
}

__device__ __forceinline__ void push(int* q, unsigned int* qn, int w) { q[agg_inc(qn)] = w; }

// The logic of one iteration runs as six kernels, each over a compacted
// list of the workers in its phase, so a warp executes one phase's code:
//   shade_kernel  closest-hit answers (sampleRay's body): emit the sky or an
//                 emitter, start the terminating vertex's light samples, or
//                 sample the next bounce (closest-hit queue) -- on opaque,
//                 untextured surfaces handing that to
//   bounce_kernel the reflection sample and the next closest-hit ray;
//   nee_kernel    shadow answers of terminating-vertex light samples and the
//                 workers shade_kernel handed over: emit, then draw the next
//                 light sample (shadow queue) until the vertex is done;
//   slot_kernel   shadow answers of first-vertex light samples and the
//                 workers whose slot ended in the kernels before: fetch
//                 units until one has a slot left (or retire when no unit is
//                 left), and hand the worker on by the kind of that slot:
//   light_kernel  a batch of first-vertex light samples (shadow queue);
//   path_kernel   the first bounce of an indirect path (closest-hit queue).
// Ray queues are double-buffered by iteration parity: the queues filled in
// iteration i are traced in iteration i and consumed in iteration i + 1.

// The light samples of a terminating vertex, drawn in order from the
// path's stream: each that needs a shadow ray gets one of the worker's ray
// slots (its sample index kept beside it). Returns the number queued.
__device__ __forceinline__ int nee_draw(const Job* J, const Pool& P, int w, RmnRng& rng, int cnt) {
  const DevScene& s = J->s;
  const float4* nv = P.nv + 6 * (size_t)w;
  float4 a = nv[0], b = nv[1], c = nv[2], d = nv[3], e = nv[4], f = nv[5];
  const int4 nk = P.nk[w];
  Surf sf = default_surf();
  sf.pos = f3(a.x, a.y, a.z);
  sf.shapeN = f3(b.x, b.y, b.z);
  sf.roughness = b.w;
  sf.surfN = f3(c.x, c.y, c.z);
  sf.metallic = c.w;
  sf.base = f3(d.x, d.y, d.z);
  sf.eta = d.w;
  sf.opacity = f.w;
  sf.entering = nk.z != 0;
  float4 l0 = P.lw[2 * w], l1 = P.lw[2 * w + 1];
  float lwt[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
  int n = 0;
  for (int k = 0; k < cnt; ++k) {
    float3 dir;
    float aim;
    LSample ls;
    if (!light_gen(s, sf, f3(e.x, e.y, e.z), lwt, e.w, cnt, rng, dir, aim, ls)) continue;
    ls.bsdf *= a.w;  // scaling(samples, factor), src/render.cpp:101-104
    if (nk.w) ls.bsdf = ls.bsdf * f3(f.x, f.y, f.z);  // passBsdf(samples, absorb), :232
    const size_t rid = (size_t)w * kDirectBatch + n++;
    P.drd[rid] = make_float4(dir.x, dir.y, dir.z, aim);
    P.dpend[2 * rid] = make_float4(ls.bsdf.x, ls.bsdf.y, ls.bsdf.z, ls.weight);
    P.dpend[2 * rid + 1] = make_float4(ls.light.x, ls.light.y, ls.light.z, __int_as_float(k));
  }
  if (n > 0) P.ro[w] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, RMN_EPS);
  return n;
}

// Appends the n shadow rays of worker w (ids ~(w * kDirectBatch + k)) to the
// shadow queue with one atomic per warp.
__device__ __forceinline__ void push_rays(int* q, unsigned int* qn, int w, int n) {
  namespace cg = cooperative_groups;
  cg::coalesced_group grp = cg::coalesced_threads();
  int incl = n;
  for (int off = 1; off < (int)grp.size(); off <<= 1) {
    int v = grp.shfl_up(incl, off);
    if ((int)grp.thread_rank() >= off) incl += v;
  }
  unsigned base = 0;
  if (grp.thread_rank() == grp.size() - 1) base = atomicAdd(qn, (unsigned)incl);
  base = grp.shfl(base, grp.size() - 1);
  const unsigned first = base + (unsigned)(incl - n);
  for (int k = 0; k < n; ++k) q[first + k] = ~(w * kDirectBatch + k);
}

// The header in registers: un = (job, pixel, j, j1), ph = (phase, rng
// counter, depth, flags), uid = the unit's partial record.
__device__ __forceinline__ void load_worker(const Pool& P, int w, int4& ph, int4& un, long long& uid) {
  const int4 a = P.hdr[2 * (size_t)w], b = P.hdr[2 * (size_t)w + 1];
  un = a;
  ph = make_int4(b.y & 15, b.x, (b.y >> 4) & 255, b.y >> 12);
  uid = (long long)(((unsigned long long)(unsigned)b.w << 32) | (unsigned)b.z);
}
__device__ __forceinline__ int worker_job(const Pool& P, int w) { return P.hdr[2 * (size_t)w].x; }
__device__ __forceinline__ void store_worker(const Pool& P, int w, const int4& ph, int phase, const RmnRng& rng,
                                             const int4& un, long long uid) {
  P.hdr[2 * (size_t)w] = un;
  P.hdr[2 * (size_t)w + 1] = make_int4((int)rng.ctr, phase | (ph.z << 4) | (ph.w << 12),
                                       (int)(unsigned)(unsigned long long)uid,
                                       (int)(unsigned)((unsigned long long)uid >> 32));
}

// sampleRay's body at a hit (src/render.cpp:121-312) for worker w: emit an
// emitter, start the vertex's light samples, or sample the next bounce.
// Returns the worker's next phase. GLASS: scenes with transmissive or
// half-opaque materials (media, Fresnel split, refraction); without it the
// opaque path compiles alone.
template <bool GLASS>
RMN_D int shade_hit(const Job* J, const Pool& P, int w, RmnRng& rng, int4& ph, const int4& un, float4* part,
                    float2 res, float3 o, float3 dir, int* status) {
  const Params& p = J->p;
  const DevScene& s = J->s;
  const int h = __float_as_int(res.x);
  const int depth = ph.z;
  const bool exclude = (ph.w & FL_EXCLUDE) != 0;
  int phase = PH_SLOT;  // unless set below, the slot ends here
  float4 pb = P.pb[w];
  Surf sf = default_surf();
  sf.pos = o + dir * res.y;
  RayDiff diff;
  float3 hpx, hpy;  // the hit point's differential (scenes with textures)
  if (s.has_tex) {
    diff = load_diff(P, w);
    hit_info_tex(s, h, dir, res.y, diff, sf, hpx, hpy);
  } else {
    hit_info(s, h, dir, sf);
  }
  const float ior = sf.eta;  // absolute; calcEta makes sf.eta relative
  float rf = fmaxf(pb.w, 1.0f * sf.roughness);
  sf.roughness = fmaxf(sf.roughness, rf);
  const float p_rr = 1.0f + (0.5f - 1.0f) * sqrtf(sf.roughness);
  bool nee = p_rr < 0.9f;
  Media med;
  med.n = 1;
  float3 absorb = f3(1.0f);
  if (GLASS) {
    load_media(P, w, med);
    absorb = get_absorb(med.absorb(), res.y);  // getAbsorb over the segment just traced
  }
  if (len3(sf.emis) > RMN_EPS) {
    if (!exclude)
      emit(part, indirect_base_of(*J, un.y), P.pa[w], f3(pb.x, pb.y, pb.z), inv_spp_of(*J, un.y),
           {absorb, sf.emis, 1.0f}, un.z * 8);
    return phase;
  }
  float pr = 1.0f, F = 0.0f;  // P_reflect and the Fresnel term
  if (GLASS && sf.opacity < RMN_EPS) {
    calc_eta(med, sf);
    float3 rd;
    precise_refraction(sf, -dir, rd, F);
    pr = (med.n == 1) ? kP0Reflect + (1.0f - kP0Reflect) * F : F;
    pr = (pr - 1e-3f < 0.0f) ? 0.0f : pr - 1e-3f;  // std::max(P_reflect - 1e-3f, 0.0f)
  }
  const float3 V = -dir;
  const bool reflect = rng.next() <= pr;
  if (!GLASS && !reflect) return phase;  // never: pr = 1 on opaque surfaces
  // light sampling at this vertex: reflection in air, or refraction out of a
  // medium into air
  nee = nee && (reflect ? (sf.entering && med.n == 1) : (!sf.entering && med.n == 2));
  if (nee && (depth >= p.maxd || rng.next() > p_rr)) {
    int cnt = c_sample_count[depth < 16 ? depth : 16];
    float k = 1.0f / (reflect ? pr : 1.0f - pr);
    if (depth < p.maxd) k /= (1.0f - p_rr);
    float lwt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float tot = 0.0f;
    if (s.sky_w != 0 || light_weights(s, sf, V, lwt, tot)) {
      float4* nv = P.nv + 6 * (size_t)w;
      nv[0] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, k);
      nv[1] = make_float4(sf.shapeN.x, sf.shapeN.y, sf.shapeN.z, sf.roughness);
      nv[2] = make_float4(sf.surfN.x, sf.surfN.y, sf.surfN.z, sf.metallic);
      nv[3] = make_float4(sf.base.x, sf.base.y, sf.base.z, sf.eta);
      nv[4] = make_float4(V.x, V.y, V.z, tot);
      nv[5] = make_float4(absorb.x, absorb.y, absorb.z, sf.opacity);
      P.lw[2 * w] = make_float4(lwt[0], lwt[1], lwt[2], lwt[3]);
      P.lw[2 * w + 1] = make_float4(lwt[4], lwt[5], lwt[6], lwt[7]);
      P.nk[w] = make_int4(0, cnt, sf.entering ? 1 : 0, reflect ? 0 : 1);
      phase = PH_NEE;
    }
  } else if (!GLASS && !s.has_tex) {
    // the bounce of an opaque, untextured surface: bounce_kernel samples it
    // from this record (the NEE vertex's slots, free at a bounce)
    float4* nv = P.nv + 6 * (size_t)w;
    nv[0] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, p_rr);
    nv[1] = make_float4(sf.shapeN.x, sf.shapeN.y, sf.shapeN.z, sf.roughness);
    nv[2] = make_float4(sf.surfN.x, sf.surfN.y, sf.surfN.z, sf.metallic);
    nv[3] = make_float4(sf.base.x, sf.base.y, sf.base.z, sf.eta);
    nv[4] = make_float4(V.x, V.y, V.z, sf.specular);
    nv[5] = make_float4(rf, sf.opacity, nee ? 1.0f : 0.0f, 0.0f);
    phase = PH_BOUNCE;
  } else {
    float3 nd, wv;
    int nf = 0;
    if (reflect) {
      sample_reflect(sf, V, rng, nd, wv, nf);
      wv = wv / pr;
    } else if (GLASS) {
      if (fabsf(sf.eta - 1.0f) < RMN_EPS) {  // inside a medium: straight on
        nd = dir;
        wv = f3(1.0f);
      } else {
        sample_btdf(sf, V, rng, nd, wv, nf);
        wv = wv * (1.0f - F);
      }
      wv = wv / (1.0f - pr);
      if (sf.entering) med.insert(sf.id, ior, sf.base);
      else med.erase(sf.id);
    }
    if (nee) wv = wv / p_rr;
    if (any_finite3(nd) && depth != p.maxd) {
      wv = wv * absorb;
      float3 thr = f3(pb.x, pb.y, pb.z) * wv;
      P.pb[w] = make_float4(thr.x, thr.y, thr.z, rf);
      if (nf > 0) {
        float4 pa = P.pa[w];
        pa.w = pa.w * (1.0f / (float)(1 + nf));
        P.pa[w] = pa;
      }
      P.ro[w] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, RMN_EPS);
      P.rd[w] = make_float4(nd.x, nd.y, nd.z, INFINITY);
      if (s.has_tex && reflect) {  // a refracted ray keeps its differential
        RayDiff nx;
        nx.dPdx = hpx;
        nx.dPdy = hpy;
        calc_dDdxy(dir, sf.surfN, diff, nx.dDdx, nx.dDdy);
        store_diff(P, w, nx);
      }
      ph.z = depth + 1;
      ph.w = nee ? FL_EXCLUDE : 0;
      phase = PH_WAIT_CLOSEST;
    }
  }
  if (GLASS) {
    if (!med.ok) atomicExch(status, rmn::kDevMediaOverflow);
    store_media(P, w, med);
  }
  return phase;
}
__device__ __noinline__ int shade_hit_glass(const Job* J, const Pool& P, int w, RmnRng& rng, int4& ph,
                                            const int4& un, float4* part, float2 res, float3 o, float3 dir,
                                            int* status) {
  return shade_hit<true>(J, P, w, rng, ph, un, part, res, o, dir, status);
}

__global__ void __launch_bounds__(128, 8) shade_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                       int par, float4* __restrict__ parts, int* status) {
  const unsigned n = ctl->q[par ^ 1].c;
  const int* in = Q.c[par ^ 1];
  QLen* out = &ctl->q[par];
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = in[idx];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    const Job* J = &jobs[un.x];
    const Params& p = J->p;
    const DevScene& s = J->s;
    RmnRng rng;
    rng.key = rmn_stream_key(p.seed, (uint32_t)un.y, (uint32_t)un.z);
    rng.ctr = (unsigned)ph.y;
    float4* part = parts + (size_t)uid * RMN_PART_F4;
    // sampleRay's body, src/render.cpp:121-312
    float2 res = P.res[w];
    int h = __float_as_int(res.x);
    float4 o4 = P.ro[w], d4 = P.rd[w];
    float3 o = f3(o4.x, o4.y, o4.z), dir = f3(d4.x, d4.y, d4.z);
    const bool exclude = (ph.w & FL_EXCLUDE) != 0;
    int phase = PH_SLOT;  // unless set below, the slot ends here
    if (h == -2) {
      atomicExch(status, 1);
    } else if (h < 0) {
      float4 pb = P.pb[w];
      if (!exclude && s.sky_w)
        emit(part, indirect_base_of(*J, un.y), P.pa[w], f3(pb.x, pb.y, pb.z), inv_spp_of(*J, un.y),
             {f3(1.0f), sky_get(s, dir), 1.0f}, un.z * 8);
    } else {
      phase = p.glass ? shade_hit_glass(J, P, w, rng, ph, un, part, res, o, dir, status)
                      : shade_hit<false>(J, P, w, rng, ph, un, part, res, o, dir, status);
    }
    if (phase == PH_SLOT) un.z++;
    store_worker(P, w, ph, phase, rng, un, uid);
    if (phase == PH_WAIT_CLOSEST) push(Q.c[par], &out->c, w);
    else if (phase == PH_NEE) push(Q.nee, &out->nee, w);
    else if (phase == PH_BOUNCE) push(Q.bounce, &out->bounce, w);
    else push(Q.slot, &out->slot, w);
  }
}

// The bounces shade_kernel handed over (opaque, untextured surfaces): the
// reflection sample of sampleRay (src/render.cpp:238-250) and the next
// closest-hit ray, in the operations and order of shade_hit's own bounce
// (pr = 1 and no absorption on an opaque surface). A warp here runs the
// reflection sampler alone, not beside emission and light-sample starts.
__global__ void __launch_bounds__(128, 6) bounce_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                        int par) {
  QLen* out = &ctl->q[par];
  const unsigned n = out->bounce;
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = Q.bounce[idx];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    const Params& p = jobs[un.x].p;
    RmnRng rng;
    rng.key = rmn_stream_key(p.seed, (uint32_t)un.y, (uint32_t)un.z);
    rng.ctr = (unsigned)ph.y;
    const float4* nv = P.nv + 6 * (size_t)w;
    const float4 a = nv[0], b = nv[1], c = nv[2], d = nv[3], e = nv[4], f = nv[5];
    Surf sf = default_surf();
    sf.pos = f3(a.x, a.y, a.z);
    sf.shapeN = f3(b.x, b.y, b.z);
    sf.roughness = b.w;
    sf.surfN = f3(c.x, c.y, c.z);
    sf.metallic = c.w;
    sf.base = f3(d.x, d.y, d.z);
    sf.eta = d.w;
    sf.specular = e.w;
    sf.opacity = f.y;
    const float3 V = f3(e.x, e.y, e.z);
    const float p_rr = a.w, rf = f.x;
    const bool nee = f.z != 0.0f;
    const int depth = ph.z;
    float3 nd, wv;
    int nf = 0;
    sample_reflect(sf, V, rng, nd, wv, nf);
    wv = wv / 1.0f;  // / P_reflect (1 on an opaque surface)
    if (nee) wv = wv / p_rr;
    int phase = PH_SLOT;
    if (any_finite3(nd) && depth != p.maxd) {
      wv = wv * f3(1.0f);  // no absorption outside media
      const float4 pb = P.pb[w];
      float3 thr = f3(pb.x, pb.y, pb.z) * wv;
      P.pb[w] = make_float4(thr.x, thr.y, thr.z, rf);
      if (nf > 0) {
        float4 pa = P.pa[w];
        pa.w = pa.w * (1.0f / (float)(1 + nf));
        P.pa[w] = pa;
      }
      P.ro[w] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, RMN_EPS);
      P.rd[w] = make_float4(nd.x, nd.y, nd.z, INFINITY);
      ph.z = depth + 1;
      ph.w = nee ? FL_EXCLUDE : 0;
      phase = PH_WAIT_CLOSEST;
    }
    if (phase == PH_SLOT) un.z++;
    store_worker(P, w, ph, phase, rng, un, uid);
    if (phase == PH_WAIT_CLOSEST) push(Q.c[par], &out->c, w);
    else push(Q.slot, &out->slot, w);
  }
}

__global__ void __launch_bounds__(128, 8) nee_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                     int par, float4* __restrict__ parts) {
  QLen* out = &ctl->q[par];
  const unsigned a = ctl->q[par ^ 1].nw, n = a + out->nee;
  const int* in = Q.nw[par ^ 1];
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = idx < a ? in[idx] : Q.nee[idx - a];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    const Job* J = &jobs[un.x];
    RmnRng rng;
    rng.key = rmn_stream_key(J->p.seed, (uint32_t)un.y, (uint32_t)un.z);
    rng.ctr = (unsigned)ph.y;
    int queued = 0;
    if (ph.x == PH_WAIT_NEE) {
      // the answered samples, emitted in sample order
      const int2 dk = P.dk[w];
      const float4 pa = P.pa[w], pb = P.pb[w];
      const float3 base = indirect_base_of(*J, un.y);
      const float inv_spp = inv_spp_of(*J, un.y);
      float4* part = parts + (size_t)uid * RMN_PART_F4;
      for (int k = 0; k < dk.y; ++k) {
        const size_t rid = (size_t)w * kDirectBatch + k;
        if (P.dres[rid] != 0.0f) continue;
        float4 b0 = P.dpend[2 * rid], b1 = P.dpend[2 * rid + 1];
        emit(part, base, pa, f3(pb.x, pb.y, pb.z), inv_spp, {f3(b0.x, b0.y, b0.z), f3(b1.x, b1.y, b1.z), b0.w},
             un.z * 8 + __float_as_int(b1.w));
      }
    } else {
      const int cnt = P.nk[w].y;
      queued = nee_draw(J, P, w, rng, cnt);
      if (queued) P.dk[w] = make_int2(cnt, queued);
    }
    if (!queued) un.z++;
    store_worker(P, w, ph, queued ? PH_WAIT_NEE : PH_SLOT, rng, un, uid);
    if (queued) {
      push_rays(Q.sn[par], &out->sn, w, queued);
      push(Q.nw[par], &out->nw, w);
    } else {
      push(Q.slot, &out->slot, w);
    }
  }
}

// The first bounce of an indirect path from the first vertex g
// (sampleIndirectLightFromFirstIntersection, src/render.cpp:314-423): the
// reflection sample, or with GLASS the Fresnel split into reflection and
// refraction, the refraction sample and the path's fresh media.
// With textures (d0: the camera ray's differential) the path's ray
// differential is set too: the reflection's, or d0 for a refraction.
template <bool GLASS>
RMN_D void first_bounce(const Pool& P, int w, const Surf& g, float3 eye, RmnRng& rng, float3& dir, float3& w0,
                        int& f0, const RayDiff* d0) {
  float3 in0 = norm3(g.pos - eye);
  Surf v0 = g;
  const float ior0 = v0.eta;
  v0.eta = 1.0f / v0.eta;  // from air into the surface
  float p_reflect = 1.0f, F0 = 0.0f;
  if (GLASS && v0.opacity < RMN_EPS) {
    float3 rd;
    precise_refraction(v0, -in0, rd, F0);
    p_reflect = kP0Reflect + (1.0f - kP0Reflect) * F0;
  }
  if (rng.next() < p_reflect) {
    if (d0) {
      RayDiff nx;
      calc_dPdxy(in0, len3(g.pos - eye), v0.shapeN, *d0, nx.dPdx, nx.dPdy);
      calc_dDdxy(in0, v0.surfN, *d0, nx.dDdx, nx.dDdy);
      store_diff(P, w, nx);
    }
    sample_reflect(v0, -in0, rng, dir, w0, f0);
    w0 = w0 / p_reflect;
    if (GLASS) {
      Media med;
      med.init();  // Medium::Init: a fresh path starts in air
      store_media(P, w, med);
    }
  } else if (GLASS) {
    if (d0) store_diff(P, w, *d0);
    sample_btdf(v0, -in0, rng, dir, w0, f0);
    w0 = w0 * (1.0f - F0);
    w0 = w0 / (1.0f - p_reflect);
    Media med;
    med.init();
    if (v0.entering) med.insert(v0.id, ior0, v0.base);
    else med.erase(v0.id);
    store_media(P, w, med);
  } else {
    dir = f3(NAN);  // never: p_reflect = 1 on opaque surfaces
  }
}
__device__ __noinline__ void first_bounce_glass(const Pool& P, int w, const Surf& g, float3 eye, RmnRng& rng,
                                                float3& dir, float3& w0, int& f0, const RayDiff* d0) {
  first_bounce<true>(P, w, g, eye, rng, dir, w0, f0, d0);
}

// Fetch order of a job's units: tiles of kFetchTile pixels, within a tile
// first every pixel's units that start with a light-sample slot, then its
// path units, so the 32 lanes of a warp fetching together start the same
// kind of slot. The record of unit (pixel, sub) stays at pixel * K + sub:
// results do not depend on the order.
constexpr int kFetchTile = 32;
__device__ __forceinline__ void unit_of_fetch(const Params& p, long long local, int& pixel, int& sub) {
  const int K = p.K;
  // units starting with a light-sample slot
  const int Kd = p.Kd ? p.Kd : min(K, (p.spp_d + p.S - 1) / p.S);
  const long long per_tile = (long long)kFetchTile * K;
  const long long tile = local / per_tile;
  const int r = (int)(local - tile * per_tile);
  const int npx = p.W * p.H;
  const int first = (int)(tile * kFetchTile);
  const int pt = min(kFetchTile, npx - first);
  if (r < pt * Kd) {
    pixel = first + r / Kd;
    sub = r % Kd;
  } else {
    const int r2 = r - pt * Kd, Ki = K - Kd;
    pixel = first + r2 / Ki;
    sub = Kd + r2 % Ki;
  }
}

// The slot hand-off, in three kernels so that each warp runs one kind of
// work with the registers and code of that kind alone:
//  * slot_kernel: workers whose slot ended (from shade / nee) and workers
//    whose first-vertex light samples were answered (the iteration before)
//    -- adds the answers, fetches units until one has a slot left, and
//    hands the worker to light_kernel (its next slot is a light-sample slot)
//    or path_kernel;
//  * light_kernel: up to kDirectBatch light-sample slots of the unit (the
//    shadow rays queued, the worker waits for their answers);
//  * path_kernel: the first bounce of the unit's next path slot (a closest-
//    hit ray queued).
// A light batch that queues no ray, or path slots that all end at the first
// vertex, leave the worker to the next iteration's slot_kernel. Results do
// not depend on these hand-offs: every slot draws from its own stream and
// adds into its own unit's record.
__global__ void __launch_bounds__(128, 8) slot_kernel(const Job* __restrict__ jobs, int njobs, Pool P, Queues Q,
                                                      Ctl* ctl, unsigned long long* next_unit, int par,
                                                      long long total_units, float4* __restrict__ parts) {
  QLen* out = &ctl->q[par];
  const unsigned a = ctl->q[par ^ 1].sd, n = a + out->slot;
  const int* in = Q.sd[par ^ 1];
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = idx < a ? in[idx] : Q.slot[idx - a];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    int phase = ph.x;
    const Job* J = phase == PH_FETCH ? nullptr : &jobs[un.x];
    RmnRng rng;
    rng.key = 0;
    rng.ctr = (unsigned)ph.y;
    if (phase == PH_WAIT_DIRECT) {
      // the answered light samples of the batch, added in slot order
      const int2 dk = P.dk[w];
      const float3 base = base_of(*J, un.y);
      float4* part = parts + (size_t)uid * RMN_PART_F4;
      Rad4 dd = r4(part[0]), ds = r4(part[1]);
      for (int k = 0; k < dk.y; ++k) {
        const size_t rid = (size_t)w * kDirectBatch + k;
        if (P.dres[rid] == 0.0f) {
          float4 b0 = P.dpend[2 * rid], b1 = P.dpend[2 * rid + 1];
          Rad4 d, sp;
          demodulate(base, f3(b0.x, b0.y, b0.z), f3(b1.x, b1.y, b1.z), b0.w, d, sp);
          radd(dd, d);
          radd(ds, sp);
        }
      }
      part[0] = f4(dd);
      part[1] = f4(ds);
      un.z += dk.x;
      phase = PH_SLOT;
    }
    // fetch units until one has a slot left; every pass takes a new unit,
    // so the loop ends within the units of the batch
    for (;;) {
      if (phase == PH_FETCH) {
        unsigned long long u = agg_inc(next_unit);
        if ((long long)u >= total_units) {
          phase = PH_DONE;
          break;
        }
        uid = (long long)u;
        int jb = find_job_unit(jobs, njobs, uid);
        J = &jobs[jb];
        int pixel, sub;
        unit_of_fetch(J->p, uid - J->unit_begin, pixel, sub);
        uid = J->unit_begin + (long long)pixel * J->p.K + sub;  // the unit's record, in pixel order
        const float* gb0 = gbuf_of(*J, pixel);
        // 16 times the indirect samples behind a transmissive or half-opaque
        // first vertex (renderPixel, src/render.cpp:497-499); the units of a
        // scene with such materials are laid out for that many
        const int pix_slots = (J->p.glass && !(gb0[17] > 1.0f - RMN_EPS)) ? J->p.slots16 : J->p.slots;
        int j0, j1;
        unit_slots(J->p, sub, pix_slots, j0, j1);
        float4* part = parts + (size_t)uid * RMN_PART_F4;
#pragma unroll
        for (int k = 0; k < 6; ++k) part[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        part[6] = make_float4(-1.0f, 0.0f, __int_as_float(0), __int_as_float(-1));
        const float* gb = gbuf_of(*J, pixel);
        bool hit = any_finite3(f3(gb[6], gb[7], gb[8]));
        un = make_int4(jb, pixel, hit ? j0 : j1, j1);
        phase = PH_SLOT;
        continue;
      }
      if (un.z >= un.w) {
        phase = PH_FETCH;
        continue;
      }
      break;
    }
    store_worker(P, w, ph, phase, rng, un, uid);
    if (phase == PH_DONE) continue;
    if (un.z < J->p.spp_d) push(Q.light, &out->light, w);
    else push(Q.path, &out->path, w);
  }
}

// sampleDirectLightFromFirstIntersection, src/render.cpp:425-437: up to
// kDirectBatch consecutive light-sample slots of the worker's unit at once,
// each from its own stream; the samples without a shadow ray add nothing.
template <bool COUNT>
__global__ void __launch_bounds__(128, 8) light_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                       int par, Counters* ctr) {
  QLen* out = &ctl->q[par];
  const unsigned n = out->light;
  unsigned long long slots_done = 0;
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = Q.light[idx];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    const Job* J = &jobs[un.x];
    const Params& p = J->p;
    const DevScene& s = J->s;
    RmnRng rng;
    rng.key = 0;
    rng.ctr = (unsigned)ph.y;
    Surf g = load_first_vertex(*J, un.y);
    const int c = min(min(un.w, p.spp_d) - un.z, kDirectBatch);
    if (COUNT) slots_done += (unsigned long long)c;
    float3 Vd = -norm3(g.pos - p.pos);
    float lwt[8];
    float tot = 0.0f;
    int nr = 0;
    if (!(len3(g.emis) > 0.0f) && (s.sky_w != 0 || light_weights(s, g, Vd, lwt, tot))) {
      for (int k = 0; k < c; ++k) {
        RmnRng rk = rmn_rng(p.seed, (uint32_t)un.y, (uint32_t)(un.z + k));
        float3 dir;
        float aim;
        LSample ls;
        if (!light_gen(s, g, Vd, lwt, tot, p.spp_d, rk, dir, aim, ls)) continue;
        const size_t rid = (size_t)w * kDirectBatch + nr++;
        P.drd[rid] = make_float4(dir.x, dir.y, dir.z, aim);
        P.dpend[2 * rid] = make_float4(ls.bsdf.x, ls.bsdf.y, ls.bsdf.z, ls.weight);
        P.dpend[2 * rid + 1] = make_float4(ls.light.x, ls.light.y, ls.light.z, 0.0f);
      }
    }
    int phase;
    if (nr == 0) {
      un.z += c;  // nothing to wait for: the next iteration's slot_kernel goes on
      phase = PH_SLOT;
    } else {
      P.ro[w] = make_float4(g.pos.x, g.pos.y, g.pos.z, RMN_EPS);
      P.dk[w] = make_int2(c, nr);
      push_rays(Q.sn[par], &out->sn, w, nr);
      phase = PH_WAIT_DIRECT;
    }
    store_worker(P, w, ph, phase, rng, un, uid);
    push(Q.sd[par], &out->sd, w);
  }
  if (COUNT && slots_done) atomicAdd(&ctr->slots, slots_done);
}

// sampleIndirectLightFromFirstIntersection, src/render.cpp:314-423: the
// first bounce of the unit's next path slot that has one.
// 6 blocks per SM: the reflection sampler's registers (fewer spills) are
// worth more here than occupancy (measured against 8: +0.8 % on batch64).
template <bool COUNT>
__global__ void __launch_bounds__(128, 6) path_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                      int par, Counters* ctr) {
  QLen* out = &ctl->q[par];
  const unsigned n = out->path;
  unsigned long long slots_done = 0;
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int w = Q.path[idx];
    int4 ph, un;
    long long uid;
    load_worker(P, w, ph, un, uid);
    const Job* J = &jobs[un.x];
    const Params& p = J->p;
    const DevScene& s = J->s;
    RmnRng rng;
    rng.key = 0;
    rng.ctr = (unsigned)ph.y;
    int phase = PH_SLOT;
    while (un.z < un.w) {
      Surf g = load_first_vertex(*J, un.y);
      rng = rmn_rng(p.seed, (uint32_t)un.y, (uint32_t)un.z);
      if (COUNT) slots_done++;
      if (len3(g.emis) > 0.0f) {
        un.z++;
        continue;
      }
      float3 dir, w0;
      int f0 = 0;
      RayDiff d0;
      if (s.has_tex) d0 = init_ray_diff(p, pixel_dir(p, un.y % p.W, un.y / p.W));
      if (p.glass) first_bounce_glass(P, w, g, p.pos, rng, dir, w0, f0, s.has_tex ? &d0 : nullptr);
      else first_bounce<false>(P, w, g, p.pos, rng, dir, w0, f0, s.has_tex ? &d0 : nullptr);
      if (!any_finite3(dir)) {
        un.z++;
        continue;
      }
      P.pa[w] = make_float4(w0.x, w0.y, w0.z, f0 > 0 ? 1.0f / (float)(1 + f0) : 1.0f);
      P.pb[w] = make_float4(1.0f, 1.0f, 1.0f, g.roughness * 1.0f);
      P.ro[w] = make_float4(g.pos.x, g.pos.y, g.pos.z, RMN_EPS);
      P.rd[w] = make_float4(dir.x, dir.y, dir.z, INFINITY);
      ph.z = 1;           // depth of the vertex this ray will hit
      ph.w = FL_EXCLUDE;  // the first bounce excludes direct light
      phase = PH_WAIT_CLOSEST;
      break;
    }
    store_worker(P, w, ph, phase, rng, un, uid);
    if (phase == PH_WAIT_CLOSEST) push(Q.c[par], &out->c, w);
    else push(Q.sd[par], &out->sd, w);  // unit used up: the next iteration's slot_kernel fetches
  }
  if (COUNT && slots_done) atomicAdd(&ctr->slots, slots_done);
}

// Seeds the first iteration: every worker (in PH_FETCH) is listed as if it
// had queued a first-vertex shadow ray in the iteration before.
__global__ void seed_kernel(Queues Q, Ctl* ctl, int W) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < W) Q.sd[1][i] = i;
  if (i == 0) ctl->q[1].sd = (unsigned)W;
}

// Persistent traversal of one queue. Each lane owns one queued worker's ray;
// after every round of inner-node steps and warp-cooperative leaf tests
// (trace.cuh: coop_nodes, coop_leaves), lanes whose ray is answered take the
// next queue entries (one warp-aggregated atomic), so a warp does not wait
// for its longest ray. The rays of a batch belong to different scenes; each
// lane traverses its own job's BVH, and the leaf phase tests a triangle
// against its owner's scene. ALPHA: the batch has scenes with alpha-tested
// materials, whose queries retry past cut-away texels (a separate build, so
// the common case keeps its register budget). STACK: the shared stack's
// entries (RMN_STACK, or RMN_STACK_SMALL for batches of shallower trees, with
// 8 instead of 7 blocks per SM).
template <bool SHADOW, bool COUNT, bool ALPHA, int STACK>
__global__ void __launch_bounds__(128, RMN_COOP_BLOCKS(STACK)) qtrace_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                     int par, int* status, Counters* ctr) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  QLen* ql = &ctl->q[par];
  // shadow queue entries: a worker id (its NEE sample) or ~(first-vertex
  // light-sample ray id)
  const unsigned n = SHADOW ? ql->sn : ql->c;
  unsigned int* next = SHADOW ? &ql->s_next : &ql->c_next;
  const int* q = SHADOW ? Q.sn[par] : Q.c[par];
  bool active = false, retired = false;
  int w = 0;
  TRay r;
  float tmin = 0.0f, aim = 0.0f;
  int searches = 0;  // alpha-test searches finished for the lane's ray
  int jb = 0;        // the lane's job
  bool alpha = false;
  // the deferred-child stack in shared memory (launched with 128 threads)
  // and the leaf-phase keys of each warp
  __shared__ int2 sstack[STACK * 128];
  __shared__ unsigned long long skeys[128];
  TravT<SharedStackN<STACK>> t;
  t.stack.base = sstack + threadIdx.x;
  t.ti = t.te = 0;
  unsigned long long* keys = skeys + (threadIdx.x & ~31);
  const DevNode* nodes = nullptr;  // the lane's job's tree and triangles
  const float4* tri = nullptr;
  TraceCounters tc = {0, 0, 0, 0, 0};
  for (;;) {
    unsigned need = __ballot_sync(0xffffffffu, !active && !retired);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !retired) {
        unsigned i = base + __popc(need & lt);
        if (i < n) {
          w = q[i];
          const int wk = (!SHADOW || w >= 0) ? w : (~w) / kDirectBatch;
          float4 o = P.ro[wk], d = (!SHADOW || w >= 0) ? P.rd[wk] : P.drd[~w];
          jb = worker_job(P, wk);
          const DevScene& js = jobs[jb].s;
          nodes = js.nodes;
          tri = js.tri;
          alpha = ALPHA && js.has_alpha != 0;
          const int root = js.root;
          r = make_tray(f3(o.x, o.y, o.z), f3(d.x, d.y, d.z));
          tmin = o.w;
          if (SHADOW) {
            aim = d.w;
            trav_begin(root, t, aim + RMN_EPS);  // HitRecord(eps, aimDepth + eps)
            if (COUNT) tc.shadow++;
          } else {
            trav_begin(root, t, d.w);
            if (COUNT) tc.closest++;
          }
          searches = 0;
          active = true;
        } else {
          retired = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, active) == 0) break;
    int st = coop_nodes<COUNT>(nodes, r, tmin, t, active, kCoopSteps, &tc);
    if (coop_leaves<SHADOW, false>(tri, r, tmin, aim, t, !alpha, keys)) st = 1;
    if (!active || st == 0) continue;
    // Model::rayHit / rayHit_test retry past cut-away texels (the texture
    // tables are read through the job table, not kept in registers)
    if (ALPHA && st == 1 && alpha && !(SHADOW && t.tmax >= aim) &&
        alpha_again(jobs[jb].s, r, t, tmin, SHADOW ? aim + RMN_EPS : INFINITY, searches, !SHADOW))
      continue;
    if (SHADOW) {
      const float occluded = st == -2 ? 0.0f : ((t.tmax >= aim) ? 0.0f : 1.0f);
      if (w >= 0) P.res[w] = make_float2(occluded, 0.0f);
      else P.dres[~w] = occluded;
    } else {
      P.res[w] = make_float2(__int_as_float(st == -2 ? -2 : t.hit), t.tmax);
    }
    if (st == -2) atomicExch(status, 1);
    active = false;
  }
  if (COUNT) {
    atomicAdd(&ctr->closest, (unsigned long long)tc.closest);
    atomicAdd(&ctr->shadow, (unsigned long long)tc.shadow);
    atomicAdd(&ctr->inner, (unsigned long long)tc.inner);
    atomicAdd(&ctr->leaves, (unsigned long long)tc.leaves);
    atomicAdd(&ctr->tris, (unsigned long long)tc.tris);
  }
}

// The shadow queue of a batch without alpha-tested materials: occlusion
// with pending leaves (trace.cuh, occ_nodes / occ_leaves), the same answer
// as the ordered search of qtrace_kernel<true, ...> in fewer instructions.
template <bool COUNT, int STACK>
__global__ void __launch_bounds__(128, RMN_OCC_BLOCKS) qocc_kernel(const Job* __restrict__ jobs, Pool P,
                                                                           Queues Q, Ctl* ctl, int par,
                                                                           int* status, Counters* ctr) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  QLen* ql = &ctl->q[par];
  const unsigned n = ql->sn;
  unsigned int* next = &ql->s_next;
  const int* q = Q.sn[par];
  bool active = false, retired = false;
  int w = 0;
  TRay r;
  float tmin = 0.0f, aim = 0.0f;
  __shared__ int sstack[STACK * 128];  // node references: occlusion pops skip nothing
  __shared__ OccExchange xch;
  OccT<SharedStackRefN<STACK>> t;
  t.stack.base = sstack + threadIdx.x;
  t.c0 = t.c1 = 0;
  const DevNode* nodes = nullptr;
  const float4* tri = nullptr;
  TraceCounters tc = {0, 0, 0, 0, 0};
  for (;;) {
    unsigned need = __ballot_sync(0xffffffffu, !active && !retired);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !retired) {
        unsigned i = base + __popc(need & lt);
        if (i < n) {
          w = q[i];
          const int wk = w >= 0 ? w : (~w) / kDirectBatch;
          float4 o = P.ro[wk], d = w >= 0 ? P.rd[wk] : P.drd[~w];
          const DevScene& js = jobs[worker_job(P, wk)].s;
          nodes = js.nodes;
          tri = js.tri;
          r = make_tray(f3(o.x, o.y, o.z), f3(d.x, d.y, d.z));
          tmin = o.w;
          aim = d.w;
          occ_begin(js.root, t);
          if (COUNT) tc.shadow++;
          active = true;
        } else {
          retired = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, active) == 0) break;
    // boxes against HitRecord(eps, aimDepth + eps) throughout
    const int st = occ_nodes<COUNT>(nodes, r, tmin, aim + RMN_EPS, t, active, kOccSteps, &tc);
    const bool occ = occ_leaves<false>(tri, r, tmin, aim, t, xch);
    if (!active || (st == 0 && !occ)) continue;
    const float occluded = (occ && st != -2) ? 1.0f : 0.0f;
    if (w >= 0) P.res[w] = make_float2(occluded, 0.0f);
    else P.dres[~w] = occluded;
    if (st == -2) atomicExch(status, 1);
    active = false;
  }
  if (COUNT) {
    atomicAdd(&ctr->shadow, (unsigned long long)tc.shadow);
    atomicAdd(&ctr->inner, (unsigned long long)tc.inner);
    atomicAdd(&ctr->leaves, (unsigned long long)tc.leaves);
    atomicAdd(&ctr->tris, (unsigned long long)tc.tris);
  }
}


// Ray binning (batch option ray_order): before a traversal launch, its queue
// is reordered by a bucket key -- the ray's job, the octant of its direction
// and a cell of its origin in an 8 x 8 x 8 grid over the job's scene box --
// with a counting sort, so the lanes of a warp trace rays that start close
// together and head the same way: they fetch the same upper nodes and walk
// more alike. Only the order in which rays are taken from the queue changes;
// each ray's visits and answer are its own, so images are unchanged.
constexpr int kBins = 4096;

__device__ __forceinline__ unsigned ray_bin(const Job* __restrict__ jobs, const Pool& P, int w, bool shadow) {
  const int wk = (!shadow || w >= 0) ? w : (~w) / kDirectBatch;
  const float4 o = P.ro[wk];
  const float4 d = (!shadow || w >= 0) ? P.rd[wk] : P.drd[~w];
  const int jb = worker_job(P, wk);
  const DevNode* nodes = jobs[jb].s.nodes;
  const int root = jobs[jb].s.root;
  unsigned cell = 0;
  if (root >= 0) {
    const DevNode* n = nodes + root;
    const float4 A = __ldg(&n->a), B = __ldg(&n->b), C = __ldg(&n->c);
    const float lx = fminf(A.x, B.z), ly = fminf(A.y, B.w), lz = fminf(A.z, C.x);
    const float hx = fmaxf(A.w, C.y), hy = fmaxf(B.x, C.z), hz = fmaxf(B.y, C.w);
    auto q = [](float v, float lo, float hi) {
      const float f = (v - lo) / fmaxf(hi - lo, 1e-20f) * 8.0f;
      return (unsigned)fminf(fmaxf(f, 0.0f), 7.0f);
    };
    cell = q(o.x, lx, hx) | q(o.y, ly, hy) << 3 | q(o.z, lz, hz) << 6;
  }
  const unsigned oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
  return ((cell << 3) | oct) ^ (((unsigned)jb * 2654435761u) >> 20);
}

// Counts the queue's rays per bucket (block histograms in shared memory,
// added into `bins`) and keeps each entry's bucket.
template <bool SHADOW>
__global__ void __launch_bounds__(256) bin_count_kernel(const Job* __restrict__ jobs, Pool P, Queues Q, Ctl* ctl,
                                                        int par, unsigned* bins, uint16_t* qb) {
  __shared__ unsigned h[kBins];
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const unsigned n = SHADOW ? ctl->q[par].sn : ctl->q[par].c;
  const int* q = SHADOW ? Q.sn[par] : Q.c[par];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned b = ray_bin(jobs, P, q[i], SHADOW) & (kBins - 1);
    qb[i] = (uint16_t)b;
    atomicAdd(&h[b], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kBins; i += blockDim.x)
    if (h[i]) atomicAdd(&bins[i], h[i]);
}

// Exclusive prefix sum of the kBins bucket counts, in place (one block of
// 1024 threads, 4 buckets each).
__global__ void __launch_bounds__(1024) bin_scan_kernel(unsigned* bins) {
  __shared__ unsigned part[1024];
  const int t = threadIdx.x;
  unsigned v[4], s = 0;
  for (int k = 0; k < 4; ++k) {
    v[k] = bins[4 * t + k];
    s += v[k];
  }
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const unsigned x = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += x;
    __syncthreads();
  }
  unsigned run = part[t] - s;
  for (int k = 0; k < 4; ++k) {
    bins[4 * t + k] = run;
    run += v[k];
  }
}

// Writes each queue entry to the next free place of its bucket.
template <bool SHADOW>
__global__ void __launch_bounds__(256) bin_scatter_kernel(Queues Q, Ctl* ctl, int par, unsigned* bins,
                                                          const uint16_t* qb, int* out) {
  const unsigned n = SHADOW ? ctl->q[par].sn : ctl->q[par].c;
  const int* q = SHADOW ? Q.sn[par] : Q.c[par];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[atomicAdd(&bins[qb[i]], 1u)] = q[i];
}


// Per pixel: merge the partial records of its K units in unit order, apply
// the firefly clamp and calcVar, write the RadianceData buffers; write the
// tweaked base colour back where renderPixel leaves it tweaked.
__global__ void __launch_bounds__(128) finalize_kernel(const Job* __restrict__ jobs, int njobs, int total_pix,
                                                       const float4* __restrict__ parts) {
  int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= total_pix) return;
  const Job& J = jobs[find_job_pix(jobs, njobs, gi)];
  const Params& p = J.p;
  const int pixel = gi - J.pix_begin;
  float* gb = J.gbuf + (size_t)RMN_GBUFFER_FLOATS * pixel;
  bool hit = any_finite3(f3(gb[6], gb[7], gb[8]));
  Rad4 dd = rad0(), ds = rad0();
  Ind a;
  a.id = a.is = a.mid = a.mis = rad0();
  a.mclum = -1.0f;
  a.S = 0.0f;
  a.n = 0;
  a.mid_sample = -1;
  int dropped = -1;
  if (hit) {
    const float4* pr = parts + (size_t)(J.unit_begin + (long long)pixel * p.K) * RMN_PART_F4;
    for (int k = 0; k < p.K; ++k, pr += RMN_PART_F4) {
      radd(dd, r4(pr[0]));
      radd(ds, r4(pr[1]));
      float4 m = pr[6];
      radd(a.id, r4(pr[2]));
      radd(a.is, r4(pr[3]));
      ind_add(a, r4(pr[4]), r4(pr[5]), m.x, m.y, __float_as_int(m.z), __float_as_int(m.w));
    }
    calc_var(dd, p.exposure);
    calc_var(ds, p.exposure);
    if (a.n > 0) {
      if (!(a.mclum / (a.S - a.mclum + RMN_EPS) > 16.0f)) {
        radd(a.id, a.mid);
        radd(a.is, a.mis);
      } else {
        dropped = a.mid_sample;
      }
      calc_var(a.id, p.exposure);
      calc_var(a.is, p.exposure);
    } else {
      // renderPixel restores the untweaked base colour only after
      // accumulating indirect samples; with none it returns early
      // (src/render.cpp:517-518) and the tweak stays in the G-buffer.
      gb[0] = tweak_base(f3(gb[0], gb[1], gb[2])).x;
    }
  }
  J.dd[pixel] = f4(dd);
  J.ds[pixel] = f4(ds);
  J.id[pixel] = f4(a.id);
  J.is[pixel] = f4(a.is);
  if (J.dropped) J.dropped[pixel] = dropped;
}

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

template <class K>
int blocks_per_sm(K kernel) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
  return per_sm < 1 ? 1 : per_sm;
}

}  // namespace

namespace rmn {


constexpr int kDefaultLanes = 3;
constexpr int kIterationsPerChunk = 8;
constexpr long long kMaxIterations = 1LL << 22;  // bound on the iteration loop; a finite render never reaches it

struct JobTable {
  std::vector<Job> jobs;
  std::vector<int> item;  // job k renders item item[k] of the caller's list
  std::vector<int> slots; // slots per unit chosen for an item that left it to the library (else 0)
  int total_pix = 0;
  long long total_units = 0;
};

struct BatchState {
  JobTable table;
  Job* d_jobs = nullptr;
  CtlBlock* d_ctl = nullptr;
  int* d_status = nullptr;
  float4* d_parts = nullptr;
  int lanes = 1;
  bool alpha = false;         // some job's scene has alpha-tested materials
  bool tex = false;           // some job's scene has textures
  bool shallow = true;        // the traversal runs its RMN_STACK_SMALL-entry build
  Pool pool[kMaxLanes] = {};  // each lane's share of the worker arrays
  Queues q[kMaxLanes] = {};
  // ray binning (ray_order): per lane, the reordered closest and shadow
  // queues, each entry's bucket, and the two queues' bucket counters
  bool binned = false;
  struct Bins {
    int *sc = nullptr, *ss = nullptr;
    uint16_t* qb = nullptr;
    unsigned* bins = nullptr;
  } bin[kMaxLanes];
  std::vector<void*> allocs;
  cudaGraphExec_t init_exec = nullptr, chunk_exec = nullptr, fin_exec = nullptr;
  bool use_graph = false;
  // per-lane streams and fork/join events: graph capture, and direct
  // launches of the lanes side by side
  cudaStream_t ls[kMaxLanes] = {};
  cudaEvent_t fork = nullptr, join[kMaxLanes] = {};
  // rmn_batch_update: the job table's pinned host copy and the event after
  // its last upload
  Job* h_jobs = nullptr;
  cudaEvent_t upd = nullptr;
};


// Jobs ordered by decreasing depth (the longest paths start first), so the
// pool drains on cheap units; results do not depend on the order.
static void build_jobs(const RenderItem* items, int n, JobTable* t) {
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return items[a].args.max_depth > items[b].args.max_depth; });
  t->jobs.clear();
  t->item = order;
  t->total_pix = 0;
  t->total_units = 0;
  for (int i : order) {
    const RenderItem& it = items[i];
    Job j;
    j.s = it.scene->dev;
    j.p = make_params(it.args, it.scene->dev.has_glass != 0);
    j.gbuf = it.gbuf;
    j.dd = reinterpret_cast<float4*>(it.dd);
    j.ds = reinterpret_cast<float4*>(it.ds);
    j.id = reinterpret_cast<float4*>(it.id);
    j.is = reinterpret_cast<float4*>(it.is);
    j.dropped = it.dropped;
    j.pix_begin = t->total_pix;
    j.unit_begin = t->total_units;
    t->total_pix += j.p.W * j.p.H;
    t->total_units += (long long)j.p.W * j.p.H * j.p.K;
    t->jobs.push_back(j);
  }
}

static cudaError_t launch_init(BatchState* b, cudaStream_t st, Counters* ctr) {
  const int nj = (int)b->table.jobs.size(), tp = b->table.total_pix;
  cudaError_t e = cudaMemsetAsync(b->d_ctl, 0, sizeof(CtlBlock), st);
  for (int l = 0; l < b->lanes && e == cudaSuccess; ++l)
    e = cudaMemsetAsync(b->pool[l].hdr, 0, 2 * sizeof(int4) * (size_t)b->pool[l].W, st);
  if (e != cudaSuccess) return e;
  const int pb = (tp + 127) / 128;
  if (ctr) {
    if (b->tex) primary_kernel<true, true><<<pb, 128, 0, st>>>(b->d_jobs, nj, tp, b->d_status, ctr);
    else primary_kernel<true, false><<<pb, 128, 0, st>>>(b->d_jobs, nj, tp, b->d_status, ctr);
  } else {
    if (b->tex) primary_kernel<false, true><<<pb, 128, 0, st>>>(b->d_jobs, nj, tp, b->d_status, ctr);
    else primary_kernel<false, false><<<pb, 128, 0, st>>>(b->d_jobs, nj, tp, b->d_status, ctr);
  }
  for (int l = 0; l < b->lanes; ++l)
    seed_kernel<<<(b->pool[l].W + 127) / 128, 128, 0, st>>>(b->q[l], &b->d_ctl->lane[l], b->pool[l].W);
  return cudaGetLastError();
}

// The two traversal kernels of an iteration (closest, then shadow), on as
// many persistent blocks as fit, at most one lane's worth of rays.
template <bool COUNT, bool ALPHA, int STACK>
static void launch_qtrace(BatchState* b, const Pool& P, const Queues& Q, Ctl* ctl, int par, Counters* ctr, int lb,
                          cudaStream_t st) {
  int tb = device_sms() * blocks_per_sm(qtrace_kernel<false, COUNT, ALPHA, STACK>);
  if (tb > lb) tb = lb;
  qtrace_kernel<false, COUNT, ALPHA, STACK><<<tb, 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, b->d_status, ctr);
  // the shadow queue: ordered search with the alpha-test retry, else order-free occlusion
  if constexpr (ALPHA) {
    qtrace_kernel<true, COUNT, ALPHA, STACK><<<tb, 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, b->d_status, ctr);
  } else {
    int ob = device_sms() * blocks_per_sm(qocc_kernel<COUNT, STACK>);
    if (ob > lb) ob = lb;
    qocc_kernel<COUNT, STACK><<<ob, 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, b->d_status, ctr);
  }
}

// Iteration k of a chunk (parity k & 1) of one lane: the six logic
// kernels, then the two traversal kernels. ev (optional) records [0] before
// the logic, [1] after it and [3] after the traversal.
static cudaError_t launch_iteration(BatchState* b, int lane, cudaStream_t st, Counters* ctr, int k,
                                    cudaEvent_t* ev = nullptr) {
  const int nj = (int)b->table.jobs.size();
  const int par = k & 1;
  const Pool& P = b->pool[lane];
  const Queues& Q = b->q[lane];
  Ctl* ctl = &b->d_ctl->lane[lane];
  cudaError_t e = cudaMemsetAsync(&ctl->q[par], 0, sizeof(QLen), st);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[0], st);
  const int sms = device_sms();
  const int gs = sms * blocks_per_sm(shade_kernel), gn = sms * blocks_per_sm(nee_kernel);
  shade_kernel<<<gs, 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, b->d_parts, b->d_status);
  bounce_kernel<<<sms * blocks_per_sm(bounce_kernel), 128, 0, st>>>(b->d_jobs, P, Q, ctl, par);
  nee_kernel<<<gn, 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, b->d_parts);
  slot_kernel<<<sms * blocks_per_sm(slot_kernel), 128, 0, st>>>(
      b->d_jobs, nj, P, Q, ctl, &b->d_ctl->next_unit, par, b->table.total_units, b->d_parts);
  if (ctr) {
    light_kernel<true><<<sms * blocks_per_sm(light_kernel<true>), 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, ctr);
    path_kernel<true><<<sms * blocks_per_sm(path_kernel<true>), 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, ctr);
  } else {
    light_kernel<false><<<sms * blocks_per_sm(light_kernel<false>), 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, ctr);
    path_kernel<false><<<sms * blocks_per_sm(path_kernel<false>), 128, 0, st>>>(b->d_jobs, P, Q, ctl, par, ctr);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[1], st);
  const int lb = (P.W + 127) / 128;
  Queues QT = Q;  // the queues the traversal reads: reordered by bucket when binning
  if (b->binned) {
    const BatchState::Bins& bb = b->bin[lane];
    e = cudaMemsetAsync(bb.bins, 0, 2 * kBins * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const int gb = sms * 4;
    bin_count_kernel<false><<<gb, 256, 0, st>>>(b->d_jobs, P, Q, ctl, par, bb.bins, bb.qb);
    bin_scan_kernel<<<1, 1024, 0, st>>>(bb.bins);
    bin_scatter_kernel<false><<<gb, 256, 0, st>>>(Q, ctl, par, bb.bins, bb.qb, bb.sc);
    bin_count_kernel<true><<<gb, 256, 0, st>>>(b->d_jobs, P, Q, ctl, par, bb.bins + kBins, bb.qb);
    bin_scan_kernel<<<1, 1024, 0, st>>>(bb.bins + kBins);
    bin_scatter_kernel<true><<<gb, 256, 0, st>>>(Q, ctl, par, bb.bins + kBins, bb.qb, bb.ss);
    QT.c[par] = bb.sc;
    QT.sn[par] = bb.ss;
  }
  if (ctr) {
    if (b->alpha && b->shallow) launch_qtrace<true, true, RMN_STACK_SMALL>(b, P, QT, ctl, par, ctr, lb, st);
    else if (b->alpha) launch_qtrace<true, true, RMN_STACK>(b, P, QT, ctl, par, ctr, lb, st);
    else if (b->shallow) launch_qtrace<true, false, RMN_STACK_SMALL>(b, P, QT, ctl, par, ctr, lb, st);
    else launch_qtrace<true, false, RMN_STACK>(b, P, QT, ctl, par, ctr, lb, st);
  } else {
    if (b->alpha && b->shallow) launch_qtrace<false, true, RMN_STACK_SMALL>(b, P, QT, ctl, par, ctr, lb, st);
    else if (b->alpha) launch_qtrace<false, true, RMN_STACK>(b, P, QT, ctl, par, ctr, lb, st);
    else if (b->shallow) launch_qtrace<false, false, RMN_STACK_SMALL>(b, P, QT, ctl, par, ctr, lb, st);
    else launch_qtrace<false, false, RMN_STACK>(b, P, QT, ctl, par, ctr, lb, st);
  }
  if (ev) cudaEventRecord(ev[3], st);
  return cudaGetLastError();
}

static cudaError_t launch_finalize(BatchState* b, cudaStream_t st) {
  const int nj = (int)b->table.jobs.size(), tp = b->table.total_pix;
  finalize_kernel<<<(tp + 127) / 128, 128, 0, st>>>(b->d_jobs, nj, tp, b->d_parts);
  return cudaGetLastError();
}

template <class F>
static cudaError_t capture(cudaStream_t cs, F&& body, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = body();
  e = cudaStreamEndCapture(cs, &g);
  if (e == cudaSuccess) e = le;
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  return e;
}

// The whole render: init (counters, pool, G-buffer), iterations in chunks
// until every worker has retired, finalize. The host reads the live-worker
// count after each chunk; kMaxIterations bounds the loop.
// One chunk of iterations of every lane. Without counters or per-kernel
// events the lanes run side by side on their own streams (forked from and
// joined back into st); otherwise one after the other on st.
static cudaError_t launch_lanes(BatchState* b, cudaStream_t st, Counters* ctr, cudaEvent_t (*ev)[kMaxLanes][4]) {
  cudaError_t e = cudaSuccess;
  if (ctr || ev || b->lanes == 1) {
    for (int k = 0; k < kIterationsPerChunk && e == cudaSuccess; ++k)
      for (int l = 0; l < b->lanes && e == cudaSuccess; ++l)
        e = launch_iteration(b, l, st, ctr, k, ev ? ev[k][l] : nullptr);
    return e;
  }
  e = cudaEventRecord(b->fork, st);
  for (int l = 0; l < b->lanes && e == cudaSuccess; ++l) {
    cudaStream_t ls = l == 0 ? st : b->ls[l];
    if (l > 0) e = cudaStreamWaitEvent(ls, b->fork, 0);
    for (int k = 0; k < kIterationsPerChunk && e == cudaSuccess; ++k) e = launch_iteration(b, l, ls, nullptr, k);
    if (l > 0 && e == cudaSuccess) e = cudaEventRecord(b->join[l], ls);
  }
  for (int l = 1; l < b->lanes && e == cudaSuccess; ++l) e = cudaStreamWaitEvent(st, b->join[l], 0);
  return e;
}

struct KernelTimes {
  double logic_ms = 0.0, trace_ms = 0.0;
  long long iterations = 0;
  cudaEvent_t e[kIterationsPerChunk][kMaxLanes][4] = {};
};

static rmn_status run(BatchState* b, cudaStream_t st, Counters* ctr, cudaEvent_t* ev, KernelTimes* kt = nullptr) {
  const bool graph = b->use_graph && !ctr && !kt;
  cudaError_t e;
  if (ev) cudaEventRecord(ev[0], st);
  e = graph ? cudaGraphLaunch(b->init_exec, st) : launch_init(b, st, ctr);
  if (e != cudaSuccess) return cuda_fail(e, "render init");
  if (ev) cudaEventRecord(ev[1], st);
  // Rays queued by the last iteration of a chunk (parity 1): the workers
  // still alive. The chunk length is even, so parities repeat chunk to chunk.
  static_assert(kIterationsPerChunk % 2 == 0, "iteration parity must repeat across chunks");
  CtlBlock h{};
  unsigned int live = 1;
  unsigned int last_live = 0xffffffffu;
  unsigned long long last_next = 0;
  int stalled = 0;
  long long iters = 0;
  while (live) {
    if (graph) {
      e = cudaGraphLaunch(b->chunk_exec, st);
    } else {
      e = launch_lanes(b, st, ctr, kt ? kt->e : nullptr);
    }
    if (e != cudaSuccess) return cuda_fail(e, "render iteration");
    iters += kIterationsPerChunk;
    e = cudaMemcpyAsync(&h, b->d_ctl, sizeof(CtlBlock), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "render iteration");
    live = 0;
    for (int l = 0; l < b->lanes; ++l) live += h.lane[l].q[1].c + h.lane[l].q[1].sd + h.lane[l].q[1].nw;
    if (kt) {
      for (int k = 0; k < kIterationsPerChunk; ++k)
        for (int l = 0; l < b->lanes; ++l) {
          float a = 0.0f, c = 0.0f;
          cudaEventElapsedTime(&a, kt->e[k][l][0], kt->e[k][l][1]);
          cudaEventElapsedTime(&c, kt->e[k][l][1], kt->e[k][l][3]);
          kt->logic_ms += a;
          kt->trace_ms += c;
        }
      kt->iterations += kIterationsPerChunk;
    }
    // Every iteration answers every queued ray, so a chunk that neither
    // retires a worker nor hands out a unit is only possible while paths are
    // long; 4096 such chunks in a row (>32k bounces) means no progress.
    if (live == last_live && h.next_unit == last_next) {
      if (++stalled > 4096) return fail(RMN_ERR_DEVICE_LIMIT, "render: no progress over 32768 iterations");
    } else {
      stalled = 0;
    }
    last_live = live;
    last_next = h.next_unit;
    if (iters > kMaxIterations) return fail(RMN_ERR_DEVICE_LIMIT, "render: iteration bound reached");
  }
  e = graph ? cudaGraphLaunch(b->fin_exec, st) : launch_finalize(b, st);
  if (e != cudaSuccess) return cuda_fail(e, "render finalize");
  if (ev) cudaEventRecord(ev[2], st);
  return RMN_OK;
}

void batch_destroy(BatchState* b) {
  if (!b) return;
  if (b->init_exec) cudaGraphExecDestroy(b->init_exec);
  if (b->chunk_exec) cudaGraphExecDestroy(b->chunk_exec);
  if (b->fin_exec) cudaGraphExecDestroy(b->fin_exec);
  for (int l = 0; l < kMaxLanes; ++l) {
    if (b->ls[l]) cudaStreamDestroy(b->ls[l]);
    if (b->join[l]) cudaEventDestroy(b->join[l]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->upd) cudaEventDestroy(b->upd);
  // the blocks go back to the cache for the next batch: no work of this
  // batch may still run on them (cudaFree would have waited likewise)
  cudaDeviceSynchronize();
  if (b->h_jobs) cudaFreeHost(b->h_jobs);
  for (void* p : b->allocs) cached_free(p);
  delete b;
}

// Bytes of one worker's state, shadow-ray slots and queue entries (media and
// ray differentials where a scene needs them).
static size_t worker_bytes(bool glass, bool tex) {
  // header 32 B, ray origin and direction, path factors, answer, NEE
  // vertex and weights, light-sample rays, queue entries
  return 4 * sizeof(int4) + 2 * sizeof(float4) + sizeof(float2) + 8 * sizeof(float4) +
         sizeof(int4) + kDirectBatch * (3 * sizeof(float4) + sizeof(float)) + sizeof(int2) +
         sizeof(int) * (2 * (3 + kDirectBatch) + 5) + (glass ? RMN_MEDIA * 20 + 4 : 0) + (tex ? 3 * sizeof(float4) : 0);
}

static size_t free_device_bytes() {
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return f;
}

// Unit records one item may take under the library's default split.
constexpr long long kItemPartBytes = 1LL << 34;  // 16 GiB

// The library's unit split for the items that leave it open
// (slots_per_unit = lanes_per_pixel = 0; others get 0 in S): 2 slots per
// unit for an item of up to 2^26 sample slots, 4 above, doubled while that
// item's own unit records (112 B each) would exceed kItemPartBytes. The
// choice depends on the item alone -- not on the batch around it, nor on the
// device memory free at the call -- so an item's images, whose float sums
// run over its units in unit order, are the same wherever it is rendered.
// Short units drain the wavefront evenly; the records are the price. A
// batch whose records do not fit fails with RMN_ERR_OUT_OF_MEMORY rather
// than changing the split.
void default_slots_per_unit(const RenderItem* items, int n, int* S) {
  for (int i = 0; i < n; ++i) {
    S[i] = 0;
    if (items[i].args.slots_per_unit != 0 || items[i].args.lanes_per_pixel != 0) continue;
    rmn_render_args a = items[i].args;
    const bool glass = items[i].scene->dev.has_glass != 0;
    a.slots_per_unit = 1;
    const Params p1 = make_params(a, glass);
    const long long slots = (long long)p1.W * p1.H * (glass ? p1.slots16 : p1.slots);
    int s = slots <= (1LL << 26) ? 2 : 4;
    for (;; s *= 2) {
      a.slots_per_unit = s;
      const Params p = make_params(a, glass);
      if (s >= (1 << 20) ||
          (long long)p.W * p.H * p.K * (long long)(sizeof(float4) * RMN_PART_F4) <= kItemPartBytes)
        break;
    }
    S[i] = s;
  }
}

int default_stack_entries(const RenderItem* items, int n) {
  for (int i = 0; i < n; ++i)
    if (items[i].scene->dev.depth + 1 > RMN_STACK_SMALL) return RMN_STACK;
  return RMN_STACK_SMALL;
}

rmn_status batch_create(const RenderItem* items_in, int n, bool use_graph, int pool_workers, int lanes,
                        int stack_entries, int ray_order, cudaStream_t st, BatchState** out) {
  *out = nullptr;
  // the traversal stack must hold every item's deepest path of deferred
  // children; a larger one only costs occupancy
  const int stack_min = default_stack_entries(items_in, n);
  if (stack_entries == 0) stack_entries = stack_min;
  if (stack_entries < stack_min)
    return fail(RMN_ERR_INVALID_ARGUMENT, "a traversal stack of %d entries is too small for a tree of this batch",
                stack_entries);
  // items that leave the unit split to the library take its default
  std::vector<RenderItem> items_v(items_in, items_in + n);
  std::vector<int> S_def(n, 0);
  default_slots_per_unit(items_in, n, S_def.data());
  for (int i = 0; i < n; ++i)
    if (S_def[i]) items_v[i].args.slots_per_unit = S_def[i];
  const RenderItem* items = items_v.data();
  BatchState* b = new BatchState();
  build_jobs(items, n, &b->table);
  b->table.slots = S_def;
  b->use_graph = use_graph;
  b->binned = ray_order != 0;
  b->lanes = lanes > 0 ? std::min(lanes, kMaxLanes) : kDefaultLanes;
  // workers per lane; no more lanes and workers than there are units; the
  // default pool halves while the workers would take more than a quarter of
  // the free device memory
  long long per = pool_workers > 0 ? pool_workers : kDefaultPoolWorkers;
  if (pool_workers <= 0) {
    bool glass = false, tex = false;
    for (const Job& j : b->table.jobs) {
      glass = glass || j.p.glass;
      tex = tex || j.s.has_tex;
    }
    const size_t budget = free_device_bytes() / 4;
    while (per > 4096 && worker_bytes(glass, tex) * (size_t)per * b->lanes > budget) per /= 2;
  }
  while (b->lanes > 1 && (long long)b->lanes * 128 > b->table.total_units) --b->lanes;
  per = std::min<long long>(per, (b->table.total_units + b->lanes - 1) / b->lanes);
  if (per < 1) per = 1;
  per = (per + 127) / 128 * 128;
  const long long W = per * b->lanes;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cached_malloc(p, bytes);
    if (e == cudaSuccess) b->allocs.push_back(*p);
  };
  const size_t jb = sizeof(Job) * b->table.jobs.size();
  alloc((void**)&b->d_jobs, jb);
  alloc((void**)&b->d_ctl, sizeof(CtlBlock));
  alloc((void**)&b->d_status, sizeof(int));
  alloc((void**)&b->d_parts, sizeof(float4) * RMN_PART_F4 * (size_t)b->table.total_units);
  Pool P{};
  P.W = (int)W;
  alloc((void**)&P.hdr, 2 * sizeof(int4) * W);
  alloc((void**)&P.ro, sizeof(float4) * W);
  alloc((void**)&P.rd, sizeof(float4) * W);
  alloc((void**)&P.res, sizeof(float2) * W);
  alloc((void**)&P.pa, sizeof(float4) * W);
  alloc((void**)&P.pb, sizeof(float4) * W);
  alloc((void**)&P.nv, sizeof(float4) * 6 * W);
  alloc((void**)&P.lw, sizeof(float4) * 2 * W);
  alloc((void**)&P.nk, sizeof(int4) * W);
  alloc((void**)&P.drd, sizeof(float4) * kDirectBatch * W);
  alloc((void**)&P.dpend, sizeof(float4) * 2 * kDirectBatch * W);
  alloc((void**)&P.dres, sizeof(float) * kDirectBatch * W);
  alloc((void**)&P.dk, sizeof(int2) * W);
  bool glass = false;
  for (const Job& j : b->table.jobs) glass = glass || j.p.glass;
  if (glass) {
    alloc((void**)&P.mn, sizeof(int) * W);
    alloc((void**)&P.mid, sizeof(int) * RMN_MEDIA * W);
    alloc((void**)&P.mval, sizeof(float4) * RMN_MEDIA * W);
  }
  for (const Job& j : b->table.jobs) {
    b->tex = b->tex || j.s.has_tex;
    b->alpha = b->alpha || j.s.has_alpha;
  }
  b->shallow = stack_entries == RMN_STACK_SMALL;
  const bool tex = b->tex;
  if (tex) alloc((void**)&P.rdiff, sizeof(float4) * 3 * W);
  for (int l = 0; l < b->lanes; ++l) {
    const size_t o = (size_t)l * per;
    Pool& L = b->pool[l];
    L.W = (int)per;
    if (e == cudaSuccess) {
      L.hdr = P.hdr + 2 * o;
      L.ro = P.ro + o;
      L.rd = P.rd + o;
      L.res = P.res + o;
      L.pa = P.pa + o;
      L.pb = P.pb + o;
      L.nv = P.nv + 6 * o;
      L.lw = P.lw + 2 * o;
      L.nk = P.nk + o;
      L.drd = P.drd + kDirectBatch * o;
      L.dpend = P.dpend + 2 * kDirectBatch * o;
      L.dres = P.dres + kDirectBatch * o;
      L.dk = P.dk + o;
      if (glass) {
        L.mn = P.mn + o;
        L.mid = P.mid + RMN_MEDIA * o;
        L.mval = P.mval + RMN_MEDIA * o;
      }
      if (tex) L.rdiff = P.rdiff + 3 * o;
    }
    Queues& Q = b->q[l];
    for (int k = 0; k < 2; ++k) {
      alloc((void**)&Q.c[k], sizeof(int) * per);
      alloc((void**)&Q.sn[k], sizeof(int) * kDirectBatch * per);
      alloc((void**)&Q.sd[k], sizeof(int) * per);
      alloc((void**)&Q.nw[k], sizeof(int) * per);
    }
    alloc((void**)&Q.nee, sizeof(int) * per);
    alloc((void**)&Q.slot, sizeof(int) * per);
    alloc((void**)&Q.light, sizeof(int) * per);
    alloc((void**)&Q.path, sizeof(int) * per);
    alloc((void**)&Q.bounce, sizeof(int) * per);
    if (b->binned) {
      BatchState::Bins& bb = b->bin[l];
      alloc((void**)&bb.sc, sizeof(int) * per);
      alloc((void**)&bb.ss, sizeof(int) * kDirectBatch * per);
      alloc((void**)&bb.qb, sizeof(uint16_t) * kDirectBatch * per);
      alloc((void**)&bb.bins, sizeof(unsigned) * 2 * kBins);
    }
  }
  if (e == cudaSuccess) e = cudaMemcpy(b->d_jobs, b->table.jobs.data(), jb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(int));
  for (int l = 0; l < b->lanes && e == cudaSuccess; ++l) {
    e = cudaStreamCreateWithFlags(&b->ls[l], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[l], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess && use_graph) {
    // One chunk graph: the lanes' iterations as parallel branches (fork and
    // join through events between the lane streams), so their kernels overlap.
    cudaStream_t c0 = b->ls[0];
    e = capture(c0, [&] { return launch_init(b, c0, nullptr); }, &b->init_exec);
    if (e == cudaSuccess) e = capture(c0, [&] { return launch_lanes(b, c0, nullptr, nullptr); }, &b->chunk_exec);
    if (e == cudaSuccess) e = capture(c0, [&] { return launch_finalize(b, c0); }, &b->fin_exec);
  }
  if (e != cudaSuccess) {
    batch_destroy(b);
    return cuda_fail(e, "batch setup");
  }
  (void)st;
  *out = b;
  return RMN_OK;
}

rmn_status batch_launch(BatchState* b, cudaStream_t st) { return run(b, st, nullptr, nullptr); }

// New camera poses, seeds and exposures for the items of a batch: the job
// table is rewritten and uploaded (on `st`, before the next render on it).
// Everything that shapes the work -- image size, spp, P_Direct, max depth,
// the unit split -- must stay as the batch was built.
rmn_status batch_update(BatchState* b, const rmn_render_args* args, int n, cudaStream_t st) {
  const int nj = (int)b->table.jobs.size();
  if (n != nj) return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_batch_update: %d arguments for a batch of %d", n, nj);
  cudaError_t e = cudaSuccess;
  if (!b->h_jobs) {
    e = cudaMallocHost(&b->h_jobs, sizeof(Job) * nj);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->upd, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "rmn_batch_update (pinned job table)");
  } else {
    e = cudaEventSynchronize(b->upd);  // the previous upload has read the pinned copy
    if (e != cudaSuccess) return cuda_fail(e, "rmn_batch_update");
  }
  std::vector<Job> next = b->table.jobs;
  for (int k = 0; k < nj; ++k) {
    Job& j = next[k];
    rmn_render_args a = args[b->table.item[k]];
    const int S_def = b->table.slots[b->table.item[k]];
    if (S_def && a.slots_per_unit == 0 && a.lanes_per_pixel == 0) a.slots_per_unit = S_def;
    const Params q = make_params(a, j.p.glass != 0);
    const Params& p = j.p;
    if (q.W != p.W || q.H != p.H || q.spp != p.spp || q.maxd != p.maxd || q.spp_d != p.spp_d || q.S != p.S ||
        q.K != p.K || q.Sd != p.Sd || q.Kd != p.Kd || q.slots != p.slots || q.slots16 != p.slots16)
      return fail(RMN_ERR_INVALID_ARGUMENT,
                  "rmn_batch_update: item %d changes the image size, spp, P_Direct, max depth or unit split",
                  b->table.item[k]);
    j.p = q;
  }
  b->table.jobs = next;
  std::memcpy(b->h_jobs, next.data(), sizeof(Job) * nj);
  e = cudaMemcpyAsync(b->d_jobs, b->h_jobs, sizeof(Job) * nj, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(b->upd, st);
  if (e != cudaSuccess) return cuda_fail(e, "rmn_batch_update (upload)");
  return RMN_OK;
}

size_t batch_job_bytes() { return sizeof(Job); }

// Device bytes batch_create would take for these items: the unit partials,
// and per worker its state, shadow-ray slots and queue entries (media and
// ray differentials where a scene needs them).
size_t batch_device_bytes(const RenderItem* items_in, int n, int pool_workers, int lanes, int ray_order) {
  // items that leave the unit split open take the library's default
  std::vector<RenderItem> items(items_in, items_in + n);
  std::vector<int> S(n, 0);
  default_slots_per_unit(items_in, n, S.data());
  for (int i = 0; i < n; ++i)
    if (S[i]) items[i].args.slots_per_unit = S[i];
  JobTable t;
  build_jobs(items.data(), n, &t);
  bool glass = false, tex = false;
  for (const Job& j : t.jobs) {
    glass = glass || j.p.glass;
    tex = tex || j.s.has_tex;
  }
  const int nl = lanes > 0 ? std::min(lanes, kMaxLanes) : kDefaultLanes;
  long long per = pool_workers > 0 ? pool_workers : kDefaultPoolWorkers;
  per = std::min<long long>(per, (t.total_units + nl - 1) / nl);
  // binning: the reordered queues and each entry's bucket, per worker; the
  // bucket counters per lane
  const size_t bin_bytes =
      ray_order ? (sizeof(int) * (1 + kDirectBatch) + sizeof(uint16_t) * kDirectBatch) * (size_t)per * nl +
                      sizeof(unsigned) * 2 * kBins * nl
                : 0;
  return sizeof(float4) * RMN_PART_F4 * (size_t)t.total_units + worker_bytes(glass, tex) * (size_t)per * nl +
         bin_bytes;
}
int batch_items(const BatchState* b) { return (int)b->table.jobs.size(); }

rmn_status batch_status(BatchState* b, cudaStream_t st) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "render");
  if (h == kDevMediaOverflow) return fail(RMN_ERR_DEVICE_LIMIT, "render: a path entered more than %d nested media",
                                          RMN_MEDIA - 1);
  if (h) return fail(RMN_ERR_DEVICE_LIMIT, "render: traversal stack bound reached");
  return RMN_OK;
}

// Counting run (visit counters) followed by a timed run with CUDA events
// around the G-buffer kernel and around the iterations + finalize. Both
// produce the same images as batch_launch.
rmn_status batch_profile(BatchState* b, cudaStream_t st, RenderProfileData* prof) {
  Counters* d_ctr = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  cudaError_t e = cudaMalloc(&d_ctr, sizeof(Counters));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, sizeof(Counters), st);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaEventCreate(&ev[k]);
  rmn_status r = e == cudaSuccess ? RMN_OK : cuda_fail(e, "render profile");
  KernelTimes kt;
  for (int k = 0; k < kIterationsPerChunk && r == RMN_OK; ++k)
    for (int l = 0; l < b->lanes; ++l)
      for (int j = 0; j < 4 && r == RMN_OK; ++j)
        if (cudaEventCreate(&kt.e[k][l][j]) != cudaSuccess) r = fail(RMN_ERR_CUDA, "cudaEventCreate");
  if (r == RMN_OK) r = run(b, st, d_ctr, nullptr);
  if (r == RMN_OK) r = run(b, st, nullptr, ev, &kt);
  for (int k = 0; k < kIterationsPerChunk; ++k)
    for (int l = 0; l < kMaxLanes; ++l)
      for (int j = 0; j < 4; ++j)
        if (kt.e[k][l][j]) cudaEventDestroy(kt.e[k][l][j]);
  Counters h{};
  if (r == RMN_OK) {
    e = cudaMemcpyAsync(&h, d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) r = cuda_fail(e, "render profile");
  }
  if (r == RMN_OK) {
    float a = 0.0f, c = 0.0f;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&c, ev[1], ev[2]);
    prof->primary_ms = a;
    prof->path_ms = c;
    prof->logic_ms = kt.logic_ms;
    prof->trace_ms = kt.trace_ms;
    prof->iterations = kt.iterations;
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
  return r;
}

}  // namespace rmn
