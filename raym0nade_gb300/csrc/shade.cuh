// Device-side hit shading, BSDF and light sampling of the integrator.
// Included by render.cu only. Each function restates the reference routine
// it cites; expression order follows the reference so that a path run on the
// same random numbers as the CPU oracle takes the same branches.
#pragma once
#include "rmn_internal.h"
#include "trace.cuh"

#define RMN_LUM f3(0.3f, 0.6f, 0.1f)  // RGB_Weight, include/geometry.h:16
// The three largest routines are real calls: inlined at their many call
// sites they multiply the integrator kernels' code, and warps in different
// phases then stall on instruction fetch. brdf takes its surface by value
// (in registers; a reference would make every caller keep the surface in
// local memory): 1 % faster on the benchmark batch. The samplers keep
// their by-reference outputs: by value, the 64-register kernels spilled
// more and ran 1 % slower.
#define RMN_CALL static __device__ __noinline__
#define RMN_MAX_TRYS 16                // src/sampling.cpp:201

__constant__ int c_sample_count[17] = {0, 1, 2, 2, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 5, 6};  // src/render.cpp:126

struct Surf {  // HitInfo, include/model.h:12-18 (defaults src/model.cpp:4-7)
  float3 shapeN, surfN, emis, base, pos;
  float specular, roughness, metallic, opacity, eta;
  int id;
  bool entering;
};

RMN_D float fmixf(float a, float b, float t) { return a * (1 - t) + b * t; }  // src/sampling.cpp:16-18

RMN_D bool flip_toward(float3& v, float3 dir) {  // reverseFix, src/model.cpp:232-238
  if (dot3(v, dir) < 0.0f) {
    v = v * -1.0f;
    return false;
  }
  return true;
}

// getHitNormals, src/model.cpp:240-270, for a triangle given by v0 + edges
// and its vertex normals.
RMN_D void hit_normals(float3 e1, float3 e2, bool smooth, float3 n0, float3 n1, float3 n2, float3 in, float3 b,
                       float3& shapeN, float3& surfN, bool& entering) {
  float3 c = cross3(e1, e2);
  shapeN = norm3(c);
  entering = flip_toward(shapeN, -in);
  surfN = shapeN;
  if (!smooth) return;
  flip_toward(n0, shapeN);
  flip_toward(n1, shapeN);
  flip_toward(n2, shapeN);
  surfN = norm3(b.x * (dot3(n0, shapeN) > 0.85f ? n0 : shapeN) + b.y * (dot3(n1, shapeN) > 0.85f ? n1 : shapeN) +
                b.z * (dot3(n2, shapeN) > 0.85f ? n2 : shapeN));
  if (!any_finite3(surfN)) surfN = shapeN;
}

// getHitInfo + getHitMaterial + calcSurfaceNormal for a closest hit at
// leaf-order triangle `i` (src/render.cpp:62-79, src/model.cpp:279-328).
// h.pos must hold the hit position.
RMN_D void hit_info(const DevScene& s, int i, float3 rd, Surf& h) {
  const float4* t = s.tri + 3 * i;
  float4 A = __ldg(t), B = __ldg(t + 1), C = __ldg(t + 2);
  int flags = __float_as_int(C.w);
  float3 v0 = f3(A), e1 = f3(B), e2 = f3(C);
  float3 b = bary(v0, e1, e2, h.pos);
  const float4* sh = s.shade + 3 * i;
  float4 N0 = __ldg(sh);
  int mat = __float_as_int(N0.w);
  float3 n0 = f3(N0), n1 = f3(0.0f), n2 = f3(0.0f);
  bool smooth = (flags & RMN_TRI_SMOOTH) != 0;
  if (smooth) {
    n1 = f3(__ldg(sh + 1));
    n2 = f3(__ldg(sh + 2));
  }
  hit_normals(e1, e2, smooth, n0, n1, n2, rd, b, h.shapeN, h.surfN, h.entering);
  float3 raw = h.surfN;
  const DevMat& m = s.mats[mat];
  float4 mb = __ldg(&m.base), me = __ldg(&m.emis), mm = __ldg(&m.misc);
  h.id = (int)mm.w;
  h.roughness = mb.w;
  h.metallic = me.w;
  h.opacity = mm.x;
  h.eta = mm.y;
  h.specular = 0.04f;
  if (h.opacity > 1.0f - RMN_EPS) h.entering = true;
  // getHitMaterial, src/model.cpp:320-323: a transmissive surface takes its
  // transmitting colour as base colour
  h.base = h.opacity < RMN_EPS ? f3(__ldg(&m.trans)) : f3(mb);
  h.emis = f3(me);
  if (flags & RMN_TRI_RENORM) {  // calcSurfaceNormal with a zero normal-map texel
    float3 keep = h.surfN;
    h.surfN = norm3(h.surfN + f3(0.0f));
    if (!any_finite3(h.surfN)) h.surfN = keep;
  }
  if (dot3(h.surfN, rd) >= 0.0f) h.surfN = raw;
  if (dot3(h.surfN, rd) >= 0.0f) h.surfN = h.shapeN;
}

// ---------------------------------------------------------- textures ------
// RayDifferential, include/render.h:29-33.
struct RayDiff {
  float3 dPdx, dPdy, dDdx, dDdy;
};

// calc_dPdxy, src/render.cpp:44-50: the hit point's differential for a ray
// of direction rd hitting a plane of normal n at distance t.
RMN_D void calc_dPdxy(float3 rd, float t, float3 n, const RayDiff& d, float3& px, float3& py) {
  float dtdx = -dot3(d.dPdx + t * d.dDdx, n) / dot3(rd, n);
  float dtdy = -dot3(d.dPdy + t * d.dDdy, n) / dot3(rd, n);
  px = d.dPdx + dtdx * rd + t * d.dDdx;
  py = d.dPdy + dtdy * rd + t * d.dDdy;
}
// calc_dDdxy, src/render.cpp:52-60: the reflected direction's differential
// (the normal's derivatives are zero).
RMN_D void calc_dDdxy(float3 rd, float3 n, const RayDiff& d, float3& dx, float3& dy) {
  const float3 dN = f3(0.0f);
  float dDNdx = dot3(dN, rd) + dot3(d.dDdx, n);
  float dDNdy = dot3(dN, rd) + dot3(d.dDdy, n);
  dx = d.dDdx - 2.0f * (dot3(rd, n) * dN + dDNdx * n);
  dy = d.dDdy - 2.0f * (dot3(rd, n) * dN + dDNdy * n);
}
// getDuv, src/model.cpp:272-277: the texture-space step of a surface step dP.
RMN_D float2 get_duv(float3 v0, float3 e1, float3 e2, float4 u01, float4 u2, float3 dP) {
  float3 b = bary(v0, e1, e2, v0 + dP);
  return make_float2((b.x - 1.0f) * u01.x + b.y * u01.z + b.z * u2.x, (b.x - 1.0f) * u01.y + b.y * u01.w + b.z * u2.y);
}
RMN_D bool any_finite2(float2 v) { return finite1(v.x) || finite1(v.y); }  // isfinite(vec2), any component
RMN_D float len2(float2 v) { return sqrtf(v.x * v.x + v.y * v.y); }

// getHitInfo + getHitMaterial + calcSurfaceNormal of a scene with textures
// (src/render.cpp:62-79, src/model.cpp:279-328) for a hit at distance t
// along rd on leaf-order triangle i, reached by a ray of differential d:
// texture coordinates, level of detail duv from the hit point's
// differential (returned in px, py), textured diffuse, emission and
// specular data, and the normal map in the uv tangent frame. Slots without
// a texture take the material's constant texel. h.pos must hold the hit.
RMN_CALL void hit_info_tex(const DevScene& s, int i, float3 rd, float t, const RayDiff& d, Surf& h, float3& px,
                           float3& py) {
  const float4* tp = s.tri + 3 * i;
  float4 A = __ldg(tp), B = __ldg(tp + 1), C = __ldg(tp + 2);
  int flags = __float_as_int(C.w);
  float3 v0 = f3(A), e1 = f3(B), e2 = f3(C);
  float3 b = bary(v0, e1, e2, h.pos);
  const float4* sh = s.shade + 3 * i;
  float4 N0 = __ldg(sh);
  int mat = __float_as_int(N0.w);
  float3 n0 = f3(N0), n1 = f3(0.0f), n2 = f3(0.0f);
  bool smooth = (flags & RMN_TRI_SMOOTH) != 0;
  if (smooth) {
    n1 = f3(__ldg(sh + 1));
    n2 = f3(__ldg(sh + 2));
  }
  hit_normals(e1, e2, smooth, n0, n1, n2, rd, b, h.shapeN, h.surfN, h.entering);
  float3 raw = h.surfN;
  calc_dPdxy(rd, t, h.shapeN, d, px, py);
  const float4 u01 = __ldg(s.uv + 2 * i), u2 = __ldg(s.uv + 2 * i + 1);
  const float u = b.x * u01.x + b.y * u01.z + b.z * u2.x;
  const float v = b.x * u01.y + b.y * u01.w + b.z * u2.y;
  const DevMat& m = s.mats[mat];
  float4 mb = __ldg(&m.base), me = __ldg(&m.emis), mm = __ldg(&m.misc);
  int4 tx = __ldg(&m.tex);
  h.id = (int)mm.w;
  if (tx.y >= 0) {  // getSurfaceData: level 0 of the specular texture
    float4 sd = tex_get<4>(s.texs[tx.y], s.texels, u, v, 0.0f);
    h.metallic = 0.99f < sd.z ? 0.99f : sd.z;
    h.roughness = sd.y < 1e-3f ? 1e-3f : sd.y;
  } else {
    h.roughness = mb.w;
    h.metallic = me.w;
  }
  h.opacity = mm.x;
  h.eta = mm.y;
  h.specular = 0.04f;
  if (h.opacity > 1.0f - RMN_EPS) h.entering = true;
  const float2 ux = get_duv(v0, e1, e2, u01, u2, px), uy = get_duv(v0, e1, e2, u01, u2, py);
  // the reference tests dUVdx twice (src/model.cpp:316)
  const float duv = (any_finite2(ux) && any_finite2(ux)) ? (len2(ux) + len2(uy)) / 2.0f : NAN;
  if (h.opacity < RMN_EPS) {
    h.base = f3(__ldg(&m.trans));
  } else if (tx.x >= 0) {
    const DevTex& tt = s.texs[tx.x];
    h.base = tex_gamma(tex_get<4>(tt, s.texels, u, v, tex_level(tt, duv)));
  } else {
    h.base = f3(mb);
  }
  if (tx.z >= 0) {
    const DevTex& tt = s.texs[tx.z];
    h.emis = tex_gamma(tex_get<4>(tt, s.texels, u, v, tex_level(tt, duv)));
  } else {
    h.emis = f3(me);
  }
  float3 nm = f3(0.0f);
  if (tx.w >= 0) {
    const DevTex& tt = s.texs[tx.w];
    nm = f3(tex_get<3>(tt, s.texels, u, v, tex_level(tt, duv))) * 2.0f - f3(1.0f);
  }
  // calcSurfaceNormal, src/model.cpp:279-298
  const float d1x = u01.z - u01.x, d1y = u01.w - u01.y, d2x = u2.x - u01.x, d2y = u2.y - u01.y;
  const float k = 1.0f / (d1x * d2y - d2x * d1y);
  const float3 tu = k * (d2y * e1 - d1y * e2), tv = k * (-d2x * e1 + d1x * e2);
  const float3 tg = norm3(tu - h.shapeN * dot3(h.shapeN, tu));
  const float3 bt = norm3(tv - h.shapeN * dot3(h.shapeN, tv) - tg * dot3(tg, tv));
  const float3 keep = h.surfN;
  h.surfN = norm3(tg * nm.x + bt * nm.y + h.surfN);
  if (!any_finite3(h.surfN)) h.surfN = keep;
  if (dot3(h.surfN, rd) >= 0.0f) h.surfN = raw;
  if (dot3(h.surfN, rd) >= 0.0f) h.surfN = h.shapeN;
}

// ------------------------------------------------------------------ BSDF --
RMN_D float pow5f(float x) { float x2 = x * x; return x2 * x2 * x; }
RMN_D float schlick(float u) {
  float m = 1 - u;
  m = m < 0 ? 0 : (m > 1 ? 1 : m);
  return pow5f(m);
}
RMN_D float gtr1(float c, float a) {
  if (a >= 1) return 1 / RMN_PI;
  float a2 = a * a;
  float t = 1 + (a2 - 1) * c * c;
  return (a2 - 1) / (RMN_PI * logf(a2) * t);
}
RMN_D float gtr2(float c, float a) {
  float a2 = a * a;
  float t = 1 + (a2 - 1) * c * c;
  return a2 / (RMN_PI * t * t);
}
RMN_D float smith_g(float c, float ag) {
  float a = ag * ag, b = c * c;
  return 1 / (c + sqrtf(a + b - a * b));
}
RMN_D void lum_clamp(float3& v) {  // clamp(vec3&), src/sampling.cpp:238-243
  float l = dot3(v, RMN_LUM);
  if (l > 64.0f) v = v / (l / 64.0f);
}

// BSDF::getBRDF, src/sampling.cpp:49-157 (subsurface, sheen, tints 0;
// clearcoat 1.5, gloss 0.2). V = in, N = surfN.
RMN_CALL float3 brdf(const Surf s, float3 V, float3 L) {
  const float3 N = s.surfN;
  float nl = dot3(N, L), nv = dot3(N, V);
  if (nl <= 0.0f || nv <= 0.0f) return f3(0.0f);
  float3 H = norm3(L + V);
  float nh = dot3(N, H), lh = dot3(L, H);
  float3 cd = s.base;
  float cdl = dot3(cd, RMN_LUM);
  float3 tint = cdl > 0.0f ? cd / cdl : f3(1.0f);
  float3 one_mix = mix3(f3(1.0f), tint, 0.0f);
  float3 spec0 = mix3(s.specular * one_mix, cd, s.metallic);
  float fl = schlick(nl), fv = schlick(nv);
  float fd90 = 0.5f + 2.0f * lh * lh * s.roughness;
  float fd = fmixf(1.0f, fd90, fl) * fmixf(1.0f, fd90, fv);
  float fss90 = lh * lh * s.roughness;
  float fss = fmixf(1.0f, fss90, fl) * fmixf(1.0f, fss90, fv);
  float ss = 1.25f * (fss * (1.0f / (nl + nv) - .5f) + .5f);
  float ds = gtr2(nh, s.roughness);
  float fh;
  if (s.eta <= 1.0f) {
    fh = schlick(lh);
  } else {
    float ci = fabsf(lh);
    float x = 1.0f - ci * ci;
    float si = x <= 0.0f ? 0.0f : sqrtf(x);
    float st = s.eta * si;
    if (st >= 1.0f) {
      fh = 1.0f;
    } else {
      float y = 1.0f - st * st;
      float ct = y <= 0.0f ? 0.0f : sqrtf(y);
      float r0 = (s.eta - 1.0f) / (s.eta + 1.0f);
      r0 = r0 * r0;
      fh = fmixf(r0, 1.0f, schlick(ct));
    }
  }
  float3 fs = mix3(spec0, f3(1.0f), fh);
  float gs = smith_g(nl, s.roughness);
  gs *= smith_g(nv, s.roughness);
  float3 fsheen = fh * 0.0f * one_mix;
  float dr = gtr1(nh, fmixf(.1f, .001f, 0.2f));
  float fr = fmixf(.04f, 1.0f, fh);
  float gr = smith_g(nl, .25f) * smith_g(nv, .25f);
  float3 ret = ((1.0f / RMN_PI) * fmixf(fd, ss, 0.0f) * cd + fsheen);
  ret *= (1.0f - s.metallic);
  ret += (0.25f * 1.5f * gr * fr * dr) * one_mix;
  ret *= s.opacity;
  ret += fs * ds * gs;
  return ret * nl;
}

// BSDF::getBTDF, src/sampling.cpp:159-192 (eta relative, V = in).
RMN_D float3 btdf(const Surf& s, float3 V, float3 L) {
  const float3 N = s.surfN;
  float nl = dot3(s.surfN, L);
  if (nl >= 0.0f) return f3(0.0f);
  float3 H = norm3(L + s.eta * V);
  float D = gtr2(dot3(N, H), s.roughness);
  float bt = D * (-nl);
  float lh = dot3(L, H), nv = dot3(N, V), hv = dot3(H, V);
  bt *= fabsf(lh * hv) / (fabsf(nl * nv) + RMN_EPS);
  float k = s.eta * hv + lh;
  bt /= k * k;
  return f3(bt);
}

// BSDF::getBSDF, :194-199: the BTDF on the far side of a transmissive or
// half-opaque surface, the BRDF otherwise.
RMN_D float3 bsdf_eval(const Surf& s, float3 V, float3 L) {
  if (s.opacity > 1.0f - RMN_EPS || s.entering) return brdf(s, V, L);
  return btdf(s, V, L);
}

// getTangentSpaceWithInDir, src/geometry.cpp:105-124.
RMN_D void frame(const Surf& s, float3 in, float3& t, float3& b) {
  float c = dot3(s.surfN, in);
  if (c < -1.0f + 1e-3f) {
    float3 v0 = fabsf(s.surfN.x) < 0.8f ? f3(1.0f, 0.0f, 0.0f) : f3(0.0f, 1.0f, 0.0f);
    t = norm3(cross3(v0, s.surfN));
    b = cross3(s.surfN, t);
    return;
  }
  b = norm3(cross3(s.surfN, in));
  t = cross3(b, s.surfN);
}

// BSDF::sampleReflection (src/sampling.cpp:310-340) with sampleCos (:245-269)
// and sampleBRDF (:203-236): both strategies are drawn in full, then one is
// kept with probability pdf_cos / (pdf_cos + pdf_ggx).
//
// With `ad`, the draw also reports what its adjoint needs (ReflectAD).
struct ReflectAD {
  int cos_branch;  // 1: the cosine sample was kept
  int clamped;     // the kept factor was luminance-clamped (cosine branch only)
  // d/dr of log(probability of the draws) + d/dr log(1 / kept pdf), r the
  // roughness the draw used: the score of every GGX half vector drawn
  // (accepted or not), the score of the branch choice (probability pc or
  // 1 - pc, pc depending on r through the GGX pdf), and, for the GGX
  // branch, the derivative of dividing by its pdf.
  float score;
};
// d/dr log GTR2(c, r) = 2/r - 4 r c^2 / (1 + (r^2 - 1) c^2): the roughness
// score of a GGX half vector with cos(theta_h) = c.
RMN_D float dlog_gtr2(float c, float r) {
  if (!(r > 1e-6f)) return 0.0f;
  float t = 1.0f + (r * r - 1.0f) * c * c;
  return 2.0f / r - 4.0f * r * c * c / t;
}
RMN_CALL void sample_reflect(const Surf& s, float3 in, RmnRng& rng, float3& dir, float3& w, int& fails,
                          ReflectAD* ad = nullptr) {
  float3 t, b;
  frame(s, in, t, b);
  float3 d1 = f3(NAN), w1 = f3(0.0f), d2 = f3(NAN), w2 = f3(0.0f);
  float p1 = 0.0f, p2 = 0.0f;
  int f1 = 0, f2 = 0;
  float sc = 0.0f, g2 = 0.0f;  // adjoint: GGX scores of all tries, of the kept try
  bool cl1 = false;
  for (int T = 1; T <= RMN_MAX_TRYS; ++T) {  // sampleCos
    float u = rng.next(), phi = rng.next() * 2.0f * RMN_PI;
    float d = sqrtf(u);
    float z = sqrtf(1 - d * d);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float x = d * cp, y = d * sp;
    float3 o = x * t + y * b + z * s.surfN;
    float pdf = dot3(o, s.surfN) / RMN_PI;
    if (dot3(o, s.shapeN) > 0.0f && pdf > 0.0f) {
      d1 = o;
      w1 = brdf(s, in, o) / pdf;
      if (ad) cl1 = dot3(w1, RMN_LUM) > 64.0f;
      lum_clamp(w1);
      p1 = pdf;
      break;
    }
    f1++;
  }
  for (int T = 1; T <= RMN_MAX_TRYS; ++T) {  // sampleBRDF (GGX half vector)
    float u = rng.next(), phi = rng.next() * 2.0f * RMN_PI;
    float ct = sqrtf((1.0f - u) / (1.0f + (s.roughness * s.roughness - 1.0f) * u));
    if (ad) sc += dlog_gtr2(ct, s.roughness);
    float st = sqrtf(1 - ct * ct);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float3 H = st * cp * t + st * sp * b + ct * s.surfN;
    float3 o = 2.0f * dot3(in, H) * H - in;
    float lh = dot3(o, H), ln = dot3(o, s.surfN);
    float pdf = (lh <= 0.0f || ln <= 0.0f) ? 0.0f : gtr2(ct, s.roughness) / (4.0f * lh);
    if (dot3(o, s.shapeN) > 0.0f && pdf > 0.0f) {
      d2 = o;
      w2 = brdf(s, in, o) / pdf;
      p2 = pdf;
      if (ad) g2 = dlog_gtr2(ct, s.roughness);
      break;
    }
    f2++;
  }
  float pc = p1 / (p1 + p2);
  if (rng.next() < pc) {
    dir = d1; w = w1; fails += f1;
    if (ad) {
      ad->cos_branch = 1;
      ad->clamped = cl1;
      ad->score = sc - (p2 > 0.0f ? (1.0f - pc) * g2 : 0.0f);
    }
  } else {
    dir = d2; w = w2; fails += f2;
    if (ad) {
      ad->cos_branch = 0;
      ad->clamped = 0;
      ad->score = sc + (p1 + p2 > 0.0f ? pc * g2 : 0.0f) - g2;
    }
  }
}

// ---------------------------------------------------------- light sampling
// RandomDistribution::operator() (src/component.cpp:20-24): lower_bound of
// total * u in the prefix sums.
RMN_D int prefix_draw(const float* p, int n, float x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(p + mid) < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// prefix_draw over the sky's prefix sums through its guide table: the same
// index (the lower_bound is monotone in x, and the table brackets it), in a
// few steps instead of log2(texels).
RMN_D int sky_draw(const DevScene& s, int n, float x) {
  const int K = s.sky_gk;
  if (K <= 0) return prefix_draw(s.sky_prefix, n, x);
  int k = (int)(x * s.sky_ginv);
  k = k < 0 ? 0 : (k > K - 1 ? K - 1 : k);
  while (k > 0 && __ldg(s.sky_gt + k) > x) --k;
  while (k < K - 1 && __ldg(s.sky_gt + k + 1) <= x) ++k;
  int lo = __ldg(s.sky_gi + k), hi = __ldg(s.sky_gi + k + 1);
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(s.sky_prefix + mid) < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// SkyBox::get, src/component.cpp:120-140.
RMN_D float3 sky_get(const DevScene& s, float3 dir) {
  if (s.sky_w == 0) return f3(0.0f);
  float th = atan2f(-dir.x, dir.z);
  float phi = acosf(dir.y);
  if (th < 0.0f) th += 2.0f * RMN_PI;
  int u = (int)(th / (2.0f * RMN_PI) * float(s.sky_w));
  int v = (int)(phi / RMN_PI * float(s.sky_h));
  u = u < 0 ? 0 : (u >= s.sky_w ? s.sky_w - 1 : u);
  v = v < 0 ? 0 : (v >= s.sky_h ? s.sky_h - 1 : v);
  phi = RMN_PI * (float(v) + 0.5f) / float(s.sky_h);
  float area = sinf(phi) * 2.0f * RMN_PI / float(s.sky_w * s.sky_h);
  return f3(__ldg(s.sky + (size_t)v * s.sky_w + u)) / area;
}

struct LSample {
  float3 bsdf, light;
  float weight;
};

// One sample T of sampleDirectLight (src/sampling.cpp:467-527), weights
// precomputed by light_weights. Returns false when the sample is dropped.
// pos = surface position, V = direction to the previous vertex.
RMN_D bool light_weights(const DevScene& s, const Surf& sf, float3 V, float* w, float& tot) {
  tot = 0.0f;
  for (int i = 0; i < s.num_lights && i < 8; ++i) {  // getLightObjectWeight, :406-417
    float4 c = __ldg(&s.lights[i].center);
    float3 ld = norm3(f3(c) - sf.pos);
    float dist = len3(f3(c) - sf.pos);
    float3 f = bsdf_eval(sf, V, ld);
    w[i] = dot3(f, RMN_LUM) * c.w / (dist * dist + 1e-3f);
  }
  for (int i = 0; i < s.num_lights && i < 8; ++i) tot += w[i];
  return tot != 0.0f;
}

// One sample T of sampleDirectLight (src/sampling.cpp:467-527) up to its
// shadow test: draws the light (or sky texel), the point and the rejection
// loop, and returns the shadow ray (from sf.pos along `dir`, occluded iff a
// hit lies nearer than `aim`) together with the sample the reference keeps
// if that ray is unoccluded (bsdf value clamped at luminance 64, light,
// weight). Returns false when the sample is dropped before any shadow test.
// Light weights `w` / `tot` come from light_weights (light mode only).
RMN_CALL bool light_gen(const DevScene& s, const Surf& sf, float3 V, const float* w, float tot, int cnt, RmnRng& rng,
                     float3& dir, float& aim, LSample& out, int* light_index = nullptr) {
  const float3 pos = sf.pos;
  if (s.sky_w == 0) {
    float rv = tot * rng.next();  // sample(), :396-404
    int li = -1;
    float acc = 0.0f;
    for (int i = 0; i < s.num_lights && i < 8; ++i) {
      acc += w[i];
      if (rv <= acc) { li = i; break; }
    }
    if (li < 0) return false;
    if (light_index) *light_index = li;
    float pl = w[li] / tot;
    const DevLight& L = s.lights[li];
    float4 lc = __ldg(&L.center), lcol = __ldg(&L.color);
    int nf = (int)lcol.w, first = L.first_face;
    const float* pre = s.light_prefix + first;
    float total = __ldg(pre + nf - 1);
    float3 lp = f3(NAN);
    int fails = 0;
    for (int T = 1; T <= RMN_MAX_TRYS; ++T) {  // sampleLightFace, :436-448
      int fi = prefix_draw(pre, nf, total * rng.next());
      if (fi >= nf) fi = nf - 1;
      const float4* F = s.light_faces + (size_t)(first + fi) * RMN_LIGHT_FACE_F4;
      float3 v0 = f3(__ldg(F)), v1 = f3(__ldg(F + 1)), v2 = f3(__ldg(F + 2));
      float a = rng.next(), b = rng.next();  // generateRandomPointInLightFace, :419-434
      if (a + b > 1.0f) { a = 1.0f - a; b = 1.0f - b; }
      float c = 1.0f - a - b;
      float3 p = a * v0 + b * v1 + c * v2;
      float3 ld = norm3(p - pos);
      float3 e1 = v1 - v0, e2 = v2 - v0;
      float area = len3(cross3(e1, e2)) / 2.0f;
      bool smooth = !(area > 1e-2f);
      float3 sn, un;
      bool ent;
      hit_normals(e1, e2, smooth, f3(__ldg(F + 3)), f3(__ldg(F + 4)), f3(__ldg(F + 5)), ld, f3(a, b, c), sn, un, ent);
      float cphi = dot3(un, -ld);
      if (cphi > 0.0f && rng.next() < cphi) { lp = p; break; }
      fails++;
    }
    if (!any_finite3(lp)) return false;
    dir = norm3(lp - pos);
    float dist = len3(lp - pos);
    aim = dist - RMN_EPS;
    float3 f = bsdf_eval(sf, V, dir);
    lum_clamp(f);
    out.bsdf = f;
    out.light = 2.0f * RMN_PI * lc.w * f3(lcol) / (dist * dist + 1e-3f) / pl;
    out.weight = 1.0f / (float)(cnt * (fails + 1));
    return true;
  }
  // sampleSkyBox, :450-465
  if (light_index) *light_index = -1;
  const int npx = s.sky_w * s.sky_h;
  const float total = __ldg(s.sky_prefix + npx - 1);
  for (int T = 1; T <= RMN_MAX_TRYS; ++T) {
    int p = sky_draw(s, npx, total * rng.next());
    if (p >= npx) p = npx - 1;
    int u = p % s.sky_w, v = p / s.sky_w;
    float phi = RMN_PI * (float(v) + 0.5f) / float(s.sky_h);
    float th = 2.0f * RMN_PI * (float(u) + 0.5f) / float(s.sky_w);
    float sp = sinf(phi), cp = cosf(phi), st = sinf(th), ct = cosf(th);
    float3 d = f3(-sp * st, cp, sp * ct);
    if (dot3(d, sf.surfN) > 0.0f) {
      float pr = __ldg(s.sky_prefix + p);
      if (p > 0) pr -= __ldg(s.sky_prefix + p - 1);
      float pdf = pr / total;
      dir = d;
      aim = INFINITY;
      float3 f = bsdf_eval(sf, V, d);
      lum_clamp(f);
      out.bsdf = f;
      out.light = f3(__ldg(s.sky + p)) / pdf;
      out.weight = 1.0f / (float)cnt;
      return true;
    }
  }
  return false;
}

// ------------------------------------------------------------ glass -------
// BSDF::preciseRefraction, src/sampling.cpp:285-308 (eta relative).
RMN_D void precise_refraction(const Surf& s, float3 V, float3& out, float& F) {
  const float3 N = s.surfN;
  const float eta = s.eta;
  float nv = dot3(N, V);
  if (nv < 0.0f) {
    F = 1.0f;
    out = f3(NAN);
    return;
  }
  float delta = 1.0f - eta * eta * (1.0f - nv * nv);
  if (delta < 0.0f) {
    F = 1.0f;
    out = f3(NAN);
    return;
  }
  float k = eta * nv - sqrtf(delta);
  out = k * N - eta * V;
  float ln = -dot3(out, N);
  float r0 = (1.0f - eta) / (1.0f + eta);
  r0 = r0 * r0;
  F = r0 + (1.0f - r0) * schlick(ln);
}

// refract, :342-349.
RMN_D float3 refract_dir(float3 V, float3 N, float eta) {
  float nv = dot3(N, V);
  float delta = 1.0f - eta * eta * (1.0f - nv * nv);
  if (delta < 0.0f) return f3(NAN);
  float k = eta * nv - sqrtf(delta);
  return k * N - eta * V;
}

// BSDF::sampleBTDF, :351-388: a GGX half vector, refracted (<= 16 tries).
RMN_CALL void sample_btdf(const Surf& s, float3 in, RmnRng& rng, float3& out, float3& w, int& fails) {
  if (fabsf(s.eta - 1.0f) < RMN_EPS) {
    out = -in;
    w = f3(1.0f);
    return;
  }
  float3 t, b;
  frame(s, in, t, b);
  const float3 V = in;
  for (int T = 1; T <= RMN_MAX_TRYS; ++T) {
    float u = rng.next(), phi = rng.next() * 2.0f * RMN_PI;
    float ct = sqrtf((1.0f - u) / (1.0f + (s.roughness * s.roughness - 1.0f) * u));
    float st = sqrtf(1 - ct * ct);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float3 H = st * cp * t + st * sp * b + ct * s.surfN;
    out = refract_dir(V, H, s.eta);
    float weight;
    if (!any_finite3(out)) {
      weight = 0.0f;
    } else {
      float vh = dot3(V, H), vn = dot3(V, s.surfN), hn = dot3(H, s.surfN);
      weight = fabsf(vh) / fabsf(vn * hn);
    }
    if (weight > 0.0f && dot3(out, s.shapeN) < 0.0f) {
      w = f3(weight);
      return;
    }
    fails++;
  }
  w = f3(0.0f);
  out = f3(NAN);
}

// getAbsorb, src/render.cpp:83-87, with pow_s (src/geometry.cpp:22-27).
RMN_D float3 get_absorb(float3 a, float dis) {
  float c = dot3(a, RMN_LUM);
  if (!(c < 1.0f - RMN_EPS)) return f3(1.0f);
  const float k = 32.0f * dis;
  a.x = a.x < 0.0f ? 0.0f : a.x;
  a.y = a.y < 0.0f ? 0.0f : a.y;
  a.z = a.z < 0.0f ? 0.0f : a.z;
  return f3(powf(a.x, k), powf(a.y, k), powf(a.z, k));
}

#define RMN_MEDIA 8  // media a path can be inside at once, air included
constexpr float kP0Reflect = 0.24f;  // P0_reflect, src/render.cpp:118

// Medium, src/render.cpp:11-42: the reference's multimap from material id
// (air: -1) to (ior, absorb), as a sorted array: equal ids keep insertion
// order, erase removes every entry of an id. ok turns false if a path would
// be inside more than RMN_MEDIA media.
struct Media {
  int n;
  bool ok;
  int id[RMN_MEDIA];
  float4 v[RMN_MEDIA];  // ior, absorb
  RMN_D void init() {
    n = 1;
    ok = true;
    id[0] = -1;
    v[0] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  }
  RMN_D void insert(int k, float ior, float3 ab) {
    if (n >= RMN_MEDIA) {
      ok = false;
      return;
    }
    int i = n;
    while (i > 0 && id[i - 1] > k) {
      id[i] = id[i - 1];
      v[i] = v[i - 1];
      --i;
    }
    id[i] = k;
    v[i] = make_float4(ior, ab.x, ab.y, ab.z);
    ++n;
  }
  RMN_D void erase(int k) {
    int j = 0;
    for (int i = 0; i < n; ++i)
      if (id[i] != k) {
        id[j] = id[i];
        v[j] = v[i];
        ++j;
      }
    n = j;
  }
  RMN_D float ior() const {
    float r = 1.0f;
    for (int i = 0; i < n; ++i) r = r < v[i].x ? v[i].x : r;  // std::max
    return r;
  }
  RMN_D float3 absorb() const {
    float3 a = f3(1.0f);
    for (int i = 0; i < n; ++i) a = a * f3(v[i].y, v[i].z, v[i].w);
    return a;
  }
};

// calcEta, src/render.cpp:89-99: sets s.eta to the relative index.
RMN_D void calc_eta(Media& m, Surf& s) {
  float eta1 = m.ior(), eta2;
  if (s.entering) {
    eta2 = eta1 < s.eta ? s.eta : eta1;  // std::max(eta1, eta)
  } else {
    m.erase(s.id);
    eta2 = m.ior();
    m.insert(s.id, s.eta, s.base);
  }
  s.eta = eta1 / eta2;
}

// ------------------------------------------------------------ derivatives --
// BSDF::getBRDF and its derivatives with respect to the base colour (one
// channel each: the BRDF is affine in it, tints being zero) and to the
// roughness, differentiated by hand from the expressions of brdf() above.
// The specular lobe's colour depends on the base colour only through
// metallic (Cspec0 = mix(0.04, base, metallic)).
RMN_D float3 brdf_d(const Surf& s, float3 V, float3 L, float3& d_base, float3& d_rough) {
  d_base = f3(0.0f);
  d_rough = f3(0.0f);
  const float3 N = s.surfN;
  float nl = dot3(N, L), nv = dot3(N, V);
  if (nl <= 0.0f || nv <= 0.0f) return f3(0.0f);
  float3 H = norm3(L + V);
  float nh = dot3(N, H), lh = dot3(L, H);
  const float r = s.roughness, m = s.metallic;
  float fl = schlick(nl), fv = schlick(nv);
  float fd90 = 0.5f + 2.0f * lh * lh * r;
  float ml = fmixf(1.0f, fd90, fl), mv = fmixf(1.0f, fd90, fv);
  float fd = ml * mv;
  float dfd = 2.0f * lh * lh * (fl * mv + ml * fv);
  float a2 = r * r, t = 1 + (a2 - 1) * nh * nh;
  float ds = a2 / (RMN_PI * t * t);
  float dds = (2.0f * r / (RMN_PI * t * t)) * (1.0f - 2.0f * a2 * nh * nh / t);
  float fh;
  if (s.eta <= 1.0f) {
    fh = schlick(lh);
  } else {
    float ci = fabsf(lh);
    float x = 1.0f - ci * ci;
    float si = x <= 0.0f ? 0.0f : sqrtf(x);
    float st = s.eta * si;
    if (st >= 1.0f) {
      fh = 1.0f;
    } else {
      float y = 1.0f - st * st;
      float ct = y <= 0.0f ? 0.0f : sqrtf(y);
      float r0 = (s.eta - 1.0f) / (s.eta + 1.0f);
      r0 = r0 * r0;
      fh = fmixf(r0, 1.0f, schlick(ct));
    }
  }
  float3 spec0 = f3(0.04f) * (1.0f - m) + s.base * m;
  float3 fs = spec0 * (1.0f - fh) + f3(fh);
  auto G = [](float c, float ag, float& dG) {
    float a = ag * ag, b = c * c;
    float q = sqrtf(a + b - a * b);
    float g = 1 / (c + q);
    dG = -(ag * (1.0f - b) / q) * g * g;
    return g;
  };
  float dgl, dgv;
  float gl = G(nl, r, dgl), gv = G(nv, r, dgv);
  float gs = gl * gv, dgs = dgl * gv + gl * dgv;
  float dr = gtr1(nh, fmixf(.1f, .001f, 0.2f));
  float fr = fmixf(.04f, 1.0f, fh);
  float gr = smith_g(nl, .25f) * smith_g(nv, .25f);
  float3 ret = (1.0f / RMN_PI) * fd * s.base * (1.0f - m) + f3(0.25f * 1.5f * gr * fr * dr);
  ret = ret * s.opacity + fs * ds * gs;
  d_base = f3(((1.0f / RMN_PI) * fd * (1.0f - m) * s.opacity + m * (1.0f - fh) * ds * gs) * nl);
  d_rough = ((1.0f / RMN_PI) * dfd * (1.0f - m) * s.opacity * s.base + fs * (dds * gs + ds * dgs)) * nl;
  return ret * nl;
}

// Log-derivatives of a path factor v = clamp64(f) * k, f = brdf_d's value,
// k a scalar that depends on neither the base colour nor the roughness of
// the brdf (clamp64: the luminance clamp of src/sampling.cpp:238-243).
// With A = dS/dv (*) v the factor's adjoint and S = sum(A) (the sample's
// contribution is linear in v), the factor adds
//   dS/dbase = A (*) l - S q,   dS/dr = A . lr.
// Unclamped: l = df_base / f, q = 0, lr = df_rough / f per channel. Clamped
// (v = f 64 / lum(f)): l as before, q = LUM (*) df_base / lum(f) and
// lr = df_rough / f - lum(df_rough) / lum(f).
RMN_D void factor_logd(float3 f, float3 df_base, float3 df_rough, bool clamped, float3& l, float3& q, float3& lr) {
  auto ratio = [](float a, float b) { return b != 0.0f ? a / b : 0.0f; };
  l = f3(ratio(df_base.x, f.x), ratio(df_base.y, f.y), ratio(df_base.z, f.z));
  lr = f3(ratio(df_rough.x, f.x), ratio(df_rough.y, f.y), ratio(df_rough.z, f.z));
  q = f3(0.0f);
  if (clamped) {
    float L = dot3(f, RMN_LUM);
    if (L > 0.0f) {
      q = f3(0.3f * df_base.x, 0.6f * df_base.y, 0.1f * df_base.z) / L;
      lr = lr - f3(dot3(df_rough, RMN_LUM) / L);
    }
  }
}
