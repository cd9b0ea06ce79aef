// Adjoint of the integrator (rmn_adjoint): the gradient of an image loss
// with respect to every material's base colour, roughness and emission
// scale, by path replay. The reference has no counterpart; what is
// differentiated is its estimator, renderPixel (src/render.cpp:448-551) with
// sampleRay (:121-312), composed by Photo::shade(Full) (src/image.cpp:
// 215-246) into I = base (*) (Dd + Id) + Ds + Is + emission * exposure.
//
// Input: the G-buffer and the per-pixel dropped-sample record of a forward
// rmn_render with the same scene and arguments, and dL/dI (3 floats per
// pixel). Every sample slot draws from the counter-based stream keyed
// (seed, pixel, slot), so one thread per slot replays exactly the forward's
// path -- same hits, same branches -- without anything stored per path.
//
// Per sample s of a path (a light sample at the terminating vertex, or the
// emitter or sky the path hits) the contribution S_s = dL/dI . dI_s is
// bilinear in the first-vertex factor w0 and in the sample's light (the
// product of the emitted radiance and every later path factor), so each
// multiplicative factor v of the path adds (A (*) dlog v) with A = dS/dv (*)
// v and sum(A) = S. The replay records, per bounce vertex, the factor's
// log-derivatives (factor_logd) and at the end applies the path's summed
// A to all of them; the first-vertex factor and the demodulation against the
// base colour (demod_adj) are differentiated directly.
//
// Sampling that depends on a parameter is handled by the score function
// (detached sampling): for the roughness, the GGX half vectors drawn and the
// choice between the cosine and the GGX candidate (sample_reflect's
// ReflectAD). Russian roulette and light selection divide by the
// probability of the decision they draw, so their score cancels their
// derivative and neither appears. The base colour and emission change no
// sampling probability except the light selection weights (cancelled the
// same way). Decisions taken by thresholds on the parameters (the
// luminance-clamp boundary, the firefly clamp of :532-547, the NEE switch at
// P_RR < 0.9) are held as the forward took them: the forward's record of
// the sample the firefly clamp dropped is skipped.
#include <vector>

#include "integrator.cuh"

namespace {

constexpr int kGradPerMat = 5;   // base colour r, g, b; roughness; emission scale
constexpr int kSharedMats = 2048;  // per-block gradient table in shared memory up to this many materials
constexpr int kMaxRecords = 16;  // bounce vertices of one path (max depth 16)

struct AdjJob {
  DevScene s;
  Params p;
  const float* gbuf;
  const int* dropped;
  const float* dimg;  // dL/dI, 3 per pixel
};

// Gradient accumulation: a block-wide table in shared memory, flushed to the
// double-precision global table when the block ends.
struct GradSink {
  float* sh;
  double* gl;
  bool use_sh;
  __device__ __forceinline__ void add(int m, int k, float v) {
    if (v == 0.0f || !finite1(v)) return;
    if (use_sh) atomicAdd(sh + m * kGradPerMat + k, v);
    else atomicAdd(gl + m * kGradPerMat + k, (double)v);
  }
  __device__ __forceinline__ void add_base(int m, float3 v) {
    add(m, 0, v.x);
    add(m, 1, v.y);
    add(m, 2, v.z);
  }
};

// S = dL/dI . (contribution of one sample to I) and its derivatives, for
// accumulateInwardRadiance (src/image.cpp:627-659) against the tweaked base
// colour bt, composed with the G-buffer's base colour sav, times calcVar's
// exposure E. f = the sample's bsdfPdf (the first-vertex factor), light =
// its light, w = its weight, g = dL/dI of the pixel. dbase is the
// derivative through bt and sav together (both move with the material's
// base colour; the tweak only shifts it).
struct DemodAdj {
  float S;
  float3 df, dlight, dbase;
};
__device__ __noinline__ DemodAdj demod_adj(float3 bt, float3 sav, float3 f, float3 light, float w, float3 g,
                                           float E) {
  DemodAdj r;
  r.S = 0.0f;
  r.df = r.dlight = r.dbase = f3(0.0f);
  if (len3(light) < RMN_EPS || !finite1(w)) return r;
  const float Ew = E * w;
  const float n = len3(bt);
  const float3 gl = g * light;
  if (n < RMN_EPS) {  // all specular
    if (!all_finite3(light * f)) return r;
    r.S = Ew * dot3(gl, f);
    r.df = Ew * gl;
    r.dlight = Ew * (g * f);
    return r;
  }
  const float3 b0 = norm3(bt);
  const float3 white = norm3(f3(1.0f));
  const float xy = dot3(b0, white);
  if (xy > 0.99f) {  // all diffuse: d = light f / bt
    float3 d = light * f / bt;
    if (!all_finite3(d)) return r;
    r.S = Ew * dot3(g * sav, d);
    r.df = Ew * (g * sav * light / bt);
    r.dlight = Ew * (g * sav * f / bt);
    r.dbase = Ew * (g * light * f / bt - g * sav * d / bt);
    return r;
  }
  // B = beta . f with beta = ((white + b0) / (1 + xy) - (white - b0) / (1 - xy)) / 2
  const float a = dot3(white, f), c = dot3(b0, f);
  const float ip = 1.0f / (1.0f + xy), im = 1.0f / (1.0f - xy);
  const float B = 0.5f * ((a + c) * ip - (a - c) * im);
  const float3 dpart = light * B / n, spart = light * (f - B * b0);
  const bool dok = all_finite3(dpart), sok = all_finite3(spart);
  const float Q = dot3(g * sav, light);
  const float kappa = (dok ? Q / n : 0.0f) - (sok ? dot3(gl, b0) : 0.0f);
  const float3 beta = 0.5f * ((white + b0) * ip - (white - b0) * im);
  r.S = Ew * ((dok ? B * Q / n : 0.0f) + (sok ? dot3(gl, f) - B * dot3(gl, b0) : 0.0f));
  r.df = Ew * (kappa * beta + (sok ? gl : f3(0.0f)));
  r.dlight = Ew * ((dok ? (B / n) * (g * sav) : f3(0.0f)) + (sok ? g * f - B * (g * b0) : f3(0.0f)));
  // through b0 (B and the projection), |bt| and sav
  const float dB_dc = 0.5f * (ip + im);
  const float dB_dxy = 0.5f * (-(a + c) * ip * ip - (a - c) * im * im);
  const float3 dB_db0 = dB_dc * f + dB_dxy * white;
  const float3 dS_db0 = Ew * (kappa * dB_db0 - (sok ? B * gl : f3(0.0f)));
  const float dS_dn = dok ? -Ew * B * Q / (n * n) : 0.0f;
  const float3 dS_dbt = (dS_db0 - b0 * dot3(b0, dS_db0)) / n + b0 * dS_dn;
  const float3 dS_dsav = dok ? Ew * (B / n) * gl : f3(0.0f);
  r.dbase = dS_dbt + dS_dsav;
  return r;
}

// Sums over the samples of one path.
struct PathAdj {
  float S;
  float3 A_light, A_w0, dbase;
};

// stk: the thread's deferred-child stack in shared memory. A real call, as
// are brdf_logd and demod_adj: inlined at each of their call sites they
// multiplied the replay's code, and its warps stalled on instruction fetch.
__device__ __noinline__ bool occluded(const DevScene& s, float3 pos, float3 dir, float aim, int* status,
                                         int2* stk) {
  float tm = aim + RMN_EPS;  // HitRecord(eps, aimDepth + eps), Model::rayHit_test
  int st = trace_shared<true>(s, make_tray(pos, dir), RMN_EPS, tm, aim, stk);  // no textured scenes here
  if (st == -2) {
    atomicExch(status, 1);
    return false;
  }
  return tm < aim;
}

// Log-derivatives of a factor clamp64(brdf(V, L)) * k of surface sf.
__device__ __noinline__ void brdf_logd(const Surf& sf, float3 V, float3 L, int clamp_mode, float3& l, float3& q,
                                          float3& lr) {
  float3 db, dr;
  float3 f = brdf_d(sf, V, L, db, dr);
  bool clamped = clamp_mode == 2 ? dot3(f, RMN_LUM) > 64.0f : clamp_mode == 1;
  factor_logd(f, db, dr, clamped, l, q, lr);
}

struct Record {
  int m, a;  // material of the vertex; material whose roughness the vertex used
  float3 l, q, lr;
};

__device__ void adjoint_slot(const AdjJob& J, int pixel, int j, GradSink& G, int* status, int2* stk) {
  const Params& p = J.p;
  const DevScene& s = J.s;
  const float* gb = J.gbuf + (size_t)RMN_GBUFFER_FLOATS * pixel;
  const float3 pos0 = f3(gb[6], gb[7], gb[8]);
  if (!any_finite3(pos0)) return;  // a miss: sky only, no material
  const int m0 = (int)gb[19];
  const float E = p.exposure;
  const float3 gpx = f3(J.dimg[3 * (size_t)pixel], J.dimg[3 * (size_t)pixel + 1], J.dimg[3 * (size_t)pixel + 2]);
  // The first vertex as the forward shades it: the material's base colour
  // with renderPixel's tweak (the G-buffer's copy is the composed one).
  Surf g = default_surf();
  g.base = tweak_base(f3(__ldg(&s.mats[m0].base)));
  g.emis = f3(gb[3], gb[4], gb[5]);
  g.pos = pos0;
  g.shapeN = f3(gb[9], gb[10], gb[11]);
  g.surfN = f3(gb[12], gb[13], gb[14]);
  g.roughness = gb[15];
  g.metallic = gb[16];
  g.opacity = gb[17];
  g.eta = gb[18];
  g.id = m0;
  const float3 sav = f3(gb[0], gb[1], gb[2]);
  if (j == 0) G.add(m0, 4, E * dot3(gpx, g.emis));  // Photo::shade's emission * exposure
  if (len3(g.emis) > 0.0f) return;
  RmnRng rng = rmn_rng(p.seed, (uint32_t)pixel, (uint32_t)j);

  if (j < p.spp_d) {  // a light sample of the first vertex
    const float3 Vd = -norm3(g.pos - p.pos);
    float lwt[8];
    float tot = 0.0f;
    if (s.sky_w == 0 && !light_weights(s, g, Vd, lwt, tot)) return;
    float3 dir;
    float aim;
    LSample ls;
    int li = -1;
    if (!light_gen(s, g, Vd, lwt, tot, p.spp_d, rng, dir, aim, ls, &li)) return;
    if (occluded(s, g.pos, dir, aim, status, stk)) return;
    DemodAdj d = demod_adj(g.base, sav, ls.bsdf, ls.light, ls.weight, gpx, E);
    if (!finite1(d.S) || d.S == 0.0f) return;
    float3 l, q, lr;
    brdf_logd(g, Vd, dir, 2, l, q, lr);
    const float3 A = d.df * ls.bsdf;
    G.add_base(m0, A * l - d.S * q + d.dbase);
    G.add(m0, 3, dot3(A, lr));
    if (li >= 0) G.add(__ldg(&s.lights[li].material), 4, d.S);
    return;
  }

  // an indirect path
  if (!(rng.next() < 1.0f)) return;
  const float3 in = norm3(g.pos - p.pos);
  Surf v0 = g;
  v0.eta = 1.0f / v0.eta;
  float3 dir, w0;
  int f0 = 0;
  ReflectAD ad0;
  sample_reflect(v0, -in, rng, dir, w0, f0, &ad0);
  if (!any_finite3(dir)) return;
  float3 l0, q0, lr0;
  brdf_logd(v0, -in, dir, ad0.clamped, l0, q0, lr0);
  lr0 = lr0 + f3(ad0.score);
  float paw = f0 > 0 ? 1.0f / (float)(1 + f0) : 1.0f;
  float3 thr = f3(1.0f);
  float rf = g.roughness;
  int rfm = m0;
  float3 o = g.pos;
  int depth = 1;
  bool exclude = true;
  const int drop = J.dropped ? J.dropped[pixel] : -1;
  const int sid0 = j * 8;
  Record rec[kMaxRecords];
  int nrec = 0;
  PathAdj acc;
  acc.S = 0.0f;
  acc.A_light = acc.A_w0 = acc.dbase = f3(0.0f);
  auto add_sample = [&](float3 light, float w) {
    DemodAdj d = demod_adj(g.base, sav, w0, light, w, gpx, E);
    if (!finite1(d.S) || d.S == 0.0f) {
      d.S = 0.0f;
      d.dlight = f3(0.0f);
      return d;
    }
    acc.S += d.S;
    acc.A_light += d.dlight * light;
    acc.A_w0 += d.df * w0;
    acc.dbase += d.dbase;
    return d;
  };
  for (;;) {
    float tm = INFINITY;
    int h = trace_shared<false>(s, make_tray(o, dir), RMN_EPS, tm, 0.0f, stk);
    if (h == -2) {
      atomicExch(status, 1);
      return;
    }
    if (h < 0) {
      if (!exclude && s.sky_w && drop != sid0) add_sample(sky_get(s, dir) * thr, paw * p.inv_spp);
      break;
    }
    Surf sf = default_surf();
    sf.pos = o + dir * tm;
    hit_info(s, h, dir, sf);
    const int mk = sf.id;
    const float own = sf.roughness;
    const float rfn = fmaxf(rf, 1.0f * own);
    const int am = own >= rf ? mk : rfm;
    sf.roughness = fmaxf(sf.roughness, rfn);
    rf = rfn;
    rfm = am;
    const float p_rr = 1.0f + (0.5f - 1.0f) * sqrtf(sf.roughness);
    bool nee = p_rr < 0.9f;
    if (len3(sf.emis) > RMN_EPS) {
      if (!exclude && drop != sid0) {
        DemodAdj d = add_sample(sf.emis * thr, paw * p.inv_spp);
        G.add(mk, 4, d.S);
      }
      break;
    }
    if (!(rng.next() <= 1.0f)) break;
    nee = nee && sf.entering;
    const float3 V = -dir;
    if (nee && (depth >= p.maxd || rng.next() > p_rr)) {
      const int cnt = c_sample_count[depth < 16 ? depth : 16];
      float k = 1.0f / 1.0f;
      if (depth < p.maxd) k /= (1.0f - p_rr);
      float lwt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      float tot = 0.0f;
      if (s.sky_w == 0 && !light_weights(s, sf, V, lwt, tot)) break;
      for (int n = 0; n < cnt; ++n) {
        float3 ld;
        float aim;
        LSample ls;
        int li = -1;
        if (!light_gen(s, sf, V, lwt, tot, cnt, rng, ld, aim, ls, &li)) continue;
        ls.bsdf *= k;
        if (occluded(s, sf.pos, ld, aim, status, stk)) continue;
        if (drop == sid0 + n) continue;
        const float3 light = (ls.light * ls.bsdf) * thr;
        DemodAdj d = add_sample(light, ls.weight * paw * p.inv_spp);
        if (d.S == 0.0f) continue;
        float3 l, q, lr;
        brdf_logd(sf, V, ld, 2, l, q, lr);
        const float3 A = d.dlight * light;
        G.add_base(mk, A * l - d.S * q);
        G.add(am, 3, dot3(A, lr));
        if (li >= 0) G.add(__ldg(&s.lights[li].material), 4, d.S);
      }
      break;
    }
    float3 nd, wv;
    int nf = 0;
    ReflectAD ad;
    sample_reflect(sf, V, rng, nd, wv, nf, &ad);
    wv = wv / 1.0f;
    if (nee) wv = wv / p_rr;
    if (!any_finite3(nd) || depth == p.maxd) break;
    thr = thr * wv;
    if (nrec < kMaxRecords) {
      Record& r = rec[nrec++];
      r.m = mk;
      r.a = am;
      brdf_logd(sf, V, nd, ad.clamped, r.l, r.q, r.lr);
      r.lr = r.lr + f3(ad.score);
    }
    if (nf > 0) paw = paw * (1.0f / (float)(1 + nf));
    o = sf.pos;
    dir = nd;
    depth++;
    exclude = nee;
  }
  if (acc.S == 0.0f) return;
  for (int i = 0; i < nrec; ++i) {
    const Record& r = rec[i];
    G.add_base(r.m, acc.A_light * r.l - acc.S * r.q);
    G.add(r.a, 3, dot3(acc.A_light, r.lr));
  }
  G.add_base(m0, acc.A_w0 * l0 - acc.S * q0 + acc.dbase);
  G.add(m0, 3, dot3(acc.A_w0, lr0));
}

__global__ void __launch_bounds__(128, 8) adjoint_kernel(AdjJob J, long long total, int nmats, double* gout,
                                                      int* status) {
  extern __shared__ float sg[];
  const bool use_sh = nmats <= kSharedMats;
  if (use_sh) {
    for (int i = threadIdx.x; i < nmats * kGradPerMat; i += blockDim.x) sg[i] = 0.0f;
    __syncthreads();
  }
  GradSink G{sg, gout, use_sh};
  __shared__ int2 sstack[RMN_STACK * 128];  // traversal stacks (launched with 128 threads)
  // Slot-major order: the lanes of a warp replay the same slot of 32
  // neighbouring pixels, so they run the same kind of work (a first-vertex
  // light sample or a path) on nearby surfaces.
  const long long npx = (long long)J.p.W * J.p.H;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    adjoint_slot(J, (int)(t % npx), (int)(t / npx), G, status, sstack + threadIdx.x);
  if (use_sh) {
    __syncthreads();
    for (int i = threadIdx.x; i < nmats * kGradPerMat; i += blockDim.x)
      if (sg[i] != 0.0f) atomicAdd(gout + i, (double)sg[i]);
  }
}

__global__ void to_float_kernel(const double* in, float* out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

}  // namespace

namespace rmn {

rmn_status launch_adjoint(const rmn_scene* scene, const rmn_render_args& args, const float* gbuf,
                          const int* dropped, const float* dimg, float* dmat, cudaStream_t st) {
  AdjJob J;
  J.s = scene->dev;
  J.p = make_params(args);
  J.gbuf = gbuf;
  J.dropped = dropped;
  J.dimg = dimg;
  const int nmats = scene->dev.num_mats;
  const int ng = nmats * kGradPerMat;
  double* acc = nullptr;
  int* status = nullptr;
  cudaError_t e = rmn::staging_malloc(reinterpret_cast<void**>(&acc), (size_t)ng * sizeof(double) + 16, st);
  if (e != cudaSuccess) return cuda_fail(e, "staging allocation (adjoint)");
  status = reinterpret_cast<int*>(acc + ng);
  e = cudaMemsetAsync(acc, 0, (size_t)ng * sizeof(double) + 16, st);
  const long long total = (long long)J.p.W * J.p.H * J.p.slots;
  const size_t smem = nmats <= kSharedMats ? (size_t)ng * sizeof(float) : 0;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel, 128, smem);
  if (per_sm < 1) per_sm = 1;
  long long want = (total + 127) / 128;
  long long grid = std::min<long long>(want, (long long)sms * per_sm * 8);
  if (e == cudaSuccess && total > 0) {
    adjoint_kernel<<<(unsigned)std::max<long long>(grid, 1), 128, smem, st>>>(J, total, nmats, acc, status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    to_float_kernel<<<(ng + 127) / 128, 128, 0, st>>>(acc, dmat, ng);
    e = cudaGetLastError();
  }
  int h_status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(acc, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
  if (h_status) return fail(RMN_ERR_CUDA, "traversal stack overflow in the adjoint");
  return RMN_OK;
}

}  // namespace rmn
