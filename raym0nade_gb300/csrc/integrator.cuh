// Pieces of renderPixel (src/render.cpp:448-551) shared by the forward
// integrator (render.cu) and its adjoint (adjoint.cu): the per-render
// parameters, the first-vertex base-colour tweak, the demodulation of a
// sample into diffuse and specular parts, and calcVar.
#pragma once
#include "rmn_host.h"
#include "shade.cuh"

namespace {

struct Params {
  float3 pos, dir, up, right;
  float acc, exposure, p_direct, inv_spp;
  int W, H, spp, maxd, spp_d, slots;
  int glass;      // the scene has transmissive or half-opaque materials
  int slots16;    // slots of a pixel behind such a first vertex
  float inv_spp16;
  int S;   // slots per path unit
  int K;   // units per pixel
  int Sd;  // slots per light-sample unit
  int Kd;  // light-sample units per pixel (0: every unit holds S consecutive slots)
  uint64_t seed;
};

// Slots per work unit. A unit is the work of one worker between two fetches;
// shorter units shorten the drain at the end of a render, longer ones need
// fewer partial records (112 B each).
constexpr int kDefaultSlotsPerUnit = 16;
// Slots of a light-sample unit at least: a worker draws a unit's first-vertex
// light samples up to 8 at a time, each with its shadow ray, in one round
// trip (a light sample is one shadow ray, so a long unit of them drains no
// slower than a short path unit).
constexpr int kLightSlotsPerUnit = 8;

inline Params make_params(const rmn_render_args& a, bool glass = false) {
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
  const int spp_i = (a.spp - p.spp_d) * 1;      // opaque first vertex
  p.inv_spp = 1.0f / (float)spp_i;
  p.slots = p.spp_d + spp_i;
  p.glass = glass ? 1 : 0;
  p.slots16 = p.spp_d + spp_i * 16;  // renderPixel's MultiSampleForRefraction
  p.inv_spp16 = 1.0f / (float)(spp_i * 16);
  const int layout = glass ? p.slots16 : p.slots;  // units are cut for the largest pixel
  // lanes_per_pixel > 0 fixes the number of units per pixel, each of S
  // consecutive slots; 0 cuts the light-sample slots into units of Sd =
  // max(S, kLightSlotsPerUnit) and the path slots into units of S =
  // slots_per_unit (kDefaultSlotsPerUnit if 0).
  if (a.lanes_per_pixel > 0) {
    p.K = a.lanes_per_pixel;
    p.S = (layout + p.K - 1) / p.K;
    if (p.S < 1) p.S = 1;
    p.Sd = p.S;
    p.Kd = 0;
  } else {
    p.S = a.slots_per_unit > 0 ? a.slots_per_unit : kDefaultSlotsPerUnit;
    p.Sd = p.S > kLightSlotsPerUnit ? p.S : kLightSlotsPerUnit;
    p.Kd = (p.spp_d + p.Sd - 1) / p.Sd;
    p.K = p.Kd + (layout - p.spp_d + p.S - 1) / p.S;
    if (p.K < 1) p.K = 1;
  }
  p.seed = a.seed;
  return p;
}

// Slots [j0, j1) of unit `sub` of a pixel with `pix_slots` sample slots:
// the first Kd units hold the light-sample slots, Sd each, the others the
// path slots, S each; with Kd = 0 unit k holds slots [k S, (k + 1) S).
__host__ __device__ __forceinline__ void unit_slots(const Params& p, int sub, int pix_slots, int& j0, int& j1) {
  if (sub < p.Kd) {
    j0 = sub * p.Sd;
    j1 = min(j0 + p.Sd, p.spp_d);
  } else {
    j0 = (p.Kd ? p.spp_d : 0) + (sub - p.Kd) * p.S;
    j1 = min(j0 + p.S, pix_slots);
  }
  if (j0 > j1) j0 = j1;
}

// The camera ray's unnormalised direction for pixel (x, y) (renderPixel,
// src/render.cpp:463-467; no jitter).
__device__ __forceinline__ float3 pixel_dir(const Params& p, int x, int y) {
  float rx = float(x) - float(p.W) / 2.0f, ry = float(y) - float(p.H) / 2.0f;
  return p.dir + p.acc * (rx * p.right + ry * p.up);
}

// initRayDiff, src/render.cpp:439-446: the camera ray's differential.
__device__ __forceinline__ RayDiff init_ray_diff(const Params& p, float3 d) {
  RayDiff r;
  r.dPdx = f3(0.0f);
  r.dPdy = f3(0.0f);
  const float3 ddx = p.acc * p.right, ddy = p.acc * p.up;
  float dd = dot3(d, d), dx = dot3(d, ddx), dy = dot3(d, ddy);
  r.dDdx = (dd * ddx - d * dx) / (sqrtf(dd) * dd);
  r.dDdy = (dd * ddy - d * dy) / (sqrtf(dd) * dd);
  return r;
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

struct Rad4 {
  float3 c;
  float v;
};
__device__ __forceinline__ Rad4 rad0() { return {f3(0.0f), 0.0f}; }
__device__ __forceinline__ void radd(Rad4& a, const Rad4& b) { a.c += b.c; a.v += b.v; }
__device__ __forceinline__ Rad4 r4(float4 v) { return {f3(v.x, v.y, v.z), v.w}; }
__device__ __forceinline__ float4 f4(const Rad4& r) { return make_float4(r.c.x, r.c.y, r.c.z, r.v); }

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

__device__ __forceinline__ void calc_var(Rad4& r, float e) {  // renderPixel's calcVar, src/render.cpp:510-516
  r.c *= e;
  r.v *= e * e;
  r.v -= dot3(r.c, r.c);
  if (r.v < 0.0f) r.v = 0.0f;
}

}  // namespace
