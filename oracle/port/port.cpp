// Oracle test infrastructure -- not part of the shipped library.
//
// CPU restatement of the reference's hot path (lemonchu/Raym0nade), used only
// by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
// checker. It is pinned against the reference's own sources compiled with
// shims (oracle/ref -> oracle/_ref/libref.so, functions ref_*): the tests
// require identical BVH trees, identical closest-hit and shadow answers,
// bit-identical renders under the reference's mt19937 stream, and
// bit-identical FXAA. On machines without the reference sources the pin is
// carried by the committed fixtures in tests/golden/ (made by
// tests/golden/make_golden.py from the compiled reference).
//
// Scope of the restatement: the opaque path of the configs (constant-texel
// materials, area lights or a lat-long sky, no media). Glass/media, alpha
// testing and textured materials are not restated here.
//
// Every function cites the reference file:line it follows.
#include "oracle_api.h"

#include <glm/glm.hpp>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <random>
#include <thread>
#include <map>
#include <vector>

#include "../../raym0nade_gb300/csrc/rmn_rng.h"

namespace orc {

using vec2 = glm::vec<2, float>;
using vec3 = glm::vec<3, float>;
using vec4 = glm::vec<4, float>;
using glm::cross;
using glm::dot;
using glm::length;
using glm::normalize;

constexpr float kEps = 1e-4f;                       // include/geometry.h:13
const float kPi = 3.14159265358979323846f;          // include/geometry.h:14
const vec3 kLum(0.3f, 0.6f, 0.1f);                  // include/geometry.h:16
constexpr int kMaxTrys = 16;                        // src/sampling.cpp:201
constexpr float kLightRadius = 1e-3f;               // include/sampling.h:34
constexpr unsigned kLeafSize = 10;                  // src/bvh.cpp:16
constexpr int kSampleCount[17] = {0, 1, 2, 2, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 5, 6};  // src/render.cpp:126

// The reference's isfinite(vec) is true when ANY component is finite
// (src/geometry.cpp:4-10).
static bool any_finite(const vec3& v) { return std::isfinite(v.x) || std::isfinite(v.y) || std::isfinite(v.z); }

static float fmix(float a, float b, float t) { return a * (1 - t) + b * t; }  // src/sampling.cpp:16-18
static float fclampf(float x, float a, float b) { return x < a ? a : (x > b ? b : x); }  // :12-14

// ---------------------------------------------------------------- textures -
constexpr int kMipLevels = 8;  // MAX_MIPMAP_LEVEL, include/material.h:10

// ImageData, src/material.cpp:26-118: 8-bit texels, a mip chain of 2x2 box
// averages (integer division), bilinear lookups with wrap-around and a blend
// of two levels.
struct Image {
  int w = 0, h = 0, ch = 0, depth = 0;
  std::vector<uint8_t> lv[kMipLevels];

  void mips() {  // ImageData::generateMipmaps, :100-129
    depth = kMipLevels;
    for (int level = 1; level < kMipLevels; ++level) {
      int pw = w >> (level - 1), ph = h >> (level - 1), cw = w >> level, chh = h >> level;
      if (cw == 0 || chh == 0) { depth = level; break; }
      lv[level].resize((size_t)cw * chh * ch);
      for (int y = 0; y < chh; ++y)
        for (int x = 0; x < cw; ++x)
          for (int c = 0; c < ch; ++c) {
            int sum = 0;
            for (int dy = 0; dy < 2; ++dy)
              for (int dx = 0; dx < 2; ++dx) {
                int px = (x * 2 + dx) % pw, py = (y * 2 + dy) % ph;
                sum += lv[level - 1][((size_t)py * pw + px) * ch + c];
              }
            lv[level][((size_t)y * cw + x) * ch + c] = (uint8_t)(sum / 4);
          }
    }
  }
  // get_basic<vec3/vec4>: N bytes from index, / 255.
  template <int N>
  static vec4 basic(const std::vector<uint8_t>& d, int i) {
    vec4 v(static_cast<float>(d[i]), static_cast<float>(d[i + 1]), static_cast<float>(d[i + 2]),
           N == 4 ? static_cast<float>(d[i + 3]) : 0.0f);
    return v / 255.0f;
  }
  // get_bilinear, :48-80 (the element stride follows the requested type).
  template <int N>
  static vec4 bilinear(const std::vector<uint8_t>& d, int width, int height, float u, float v) {
    auto wrap = [](int& x, int m) {
      if (x < 0 || x >= m) {
        x %= m;
        if (x < 0) x += m;
      }
    };
    float x = u * float(width), y = v * float(height);
    int x0 = int(floorf(x)), y0 = int(floorf(y));
    float dx = x - float(x0), dy = y - float(y0);
    wrap(x0, width);
    wrap(y0, height);
    int x1 = (x0 + 1) % width, y1 = (y0 + 1) % height;
    vec4 c00 = basic<N>(d, (y0 * width + x0) * N), c01 = basic<N>(d, (y0 * width + x1) * N);
    vec4 c10 = basic<N>(d, (y1 * width + x0) * N), c11 = basic<N>(d, (y1 * width + x1) * N);
    vec4 c0 = c00 * (1.0f - dx) + c01 * dx;
    vec4 c1 = c10 * (1.0f - dx) + c11 * dx;
    return c0 * (1.0f - dy) + c1 * dy;
  }
  // ImageData::get, :82-94.
  template <int N>
  vec4 get(float u, float v, float dep) const {
    v = 1.0f - v;
    dep = std::max(std::min(dep, static_cast<float>(depth - 1)), 0.0f);
    int level = static_cast<int>(dep);
    int next = std::min(level + 1, depth - 1);
    float blend = dep - float(level);
    vec4 a = bilinear<N>(lv[level], w >> level, h >> level, u, v);
    vec4 b = bilinear<N>(lv[next], w >> next, h >> next, u, v);
    return a * (1.0f - blend) + b * blend;
  }
  bool has_transparent_part() const {  // ImageData::hasTransparentPart, :100-105
    for (size_t i = 3; i < lv[0].size(); i += 4)
      if (lv[0][i] < 255) return true;
    return false;
  }
};

static void gamma_pow(vec4& v) {  // gammaPow, src/material.cpp:335-346
  const float g = 2.2f;
  v[0] = std::pow(v[0], g);
  v[1] = std::pow(v[1], g);
  v[2] = std::pow(v[2], g);
}

// ---------------------------------------------------------------- scene ----
struct Mat {
  vec3 base, emis, trans;
  bool has_base, has_emis, has_surf;
  float roughness, metallic, opacity, ior;
  int id;
  const Image* tex[4] = {nullptr, nullptr, nullptr, nullptr};  // diffuse, specular, emissive, normal map
  bool transparent = false;  // Material::hasFullyTransparentPart
  // Material::getDiffuseColor / getNormal / getEmissiveColor /
  // getSurfaceData, src/material.cpp:349-383: a texture when the slot has
  // one (mip level log2(duv * width), duv = NaN: level 0), else the record's
  // constant texel.
  static float level_of(const Image* t, float duv) { return std::isnan(duv) ? 0.0f : std::log2(duv * float(t->w)); }
  vec4 diffuse4(float u, float v, float duv) const {
    if (!tex[0]) return has_base ? vec4(base.x, base.y, base.z, 1.0f) : vec4(1.0f);
    vec4 c = tex[0]->get<4>(u, v, level_of(tex[0], duv));
    gamma_pow(c);
    return c;
  }
  vec3 diffuse(float u = 0.0f, float v = 0.0f, float duv = NAN) const { return vec3(diffuse4(u, v, duv)); }
  vec3 normal_map(float u, float v, float duv) const {
    if (!tex[3]) return vec3(0.0f);
    return vec3(tex[3]->get<3>(u, v, level_of(tex[3], duv))) * 2.0f - 1.0f;
  }
  vec3 emission(float u = 0.0f, float v = 0.0f, float duv = NAN) const {
    if (!tex[2]) return has_emis ? emis : vec3(0.0f);
    vec4 c = tex[2]->get<4>(u, v, level_of(tex[2], duv));
    gamma_pow(c);
    return vec3(c);
  }
  bool emissive() const { return tex[2] != nullptr || has_emis; }
  void surface(float& r, float& m, float u = 0.0f, float v = 0.0f) const {
    if (tex[1]) {
      vec4 d = tex[1]->get<4>(u, v, 0);
      m = std::min(d[2], 0.99f);
      r = std::max(d[1], 1e-3f);
      return;
    }
    if (!has_surf) { m = 0.0f; r = roughness; return; }
    m = std::min(metallic, 0.99f);
    r = std::max(roughness, 1e-3f);
  }
};

struct Tri {
  vec3 v[3];
  int vid[3];  // vertex indices (normals, uvs)
  int mat;
  int id;      // index in the input triangle array
};

struct Box { vec3 lo, hi; };
static Box box_union(const Box& a, const Box& b) {  // src/geometry.cpp:30-35
  return {vec3(std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y), std::fmin(a.lo.z, b.lo.z)),
          vec3(std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y), std::fmax(a.hi.z, b.hi.z))};
}
static vec3 tri_center(const Tri& f) { return (f.v[0] + f.v[1] + f.v[2]) / 3.0f; }  // src/component.cpp:37-39
static Box tri_box(const Tri& f) {                                                    // :41-46
  return {glm::min(f.v[0], glm::min(f.v[1], f.v[2])), glm::max(f.v[0], glm::max(f.v[1], f.v[2]))};
}

struct Node {
  Box box;
  int faceL = 0, faceR = 0;
};

struct Light {  // LightObject, include/component.h:47-54
  vec3 center = vec3(0.0f), color = vec3(0.0f);
  float power = 0.0f;
  std::vector<Tri> faces;
  std::vector<float> prefix;
};

struct Sky {  // SkyBox, include/component.h:56-67
  int w = 0, h = 0;
  std::vector<vec3> data;  // premultiplied by texel solid angle (src/component.cpp:54-67)
  std::vector<float> prefix;
  bool empty() const { return data.empty(); }
};

struct Stats { uint64_t inner = 0, leaves = 0, tris = 0; };

struct Scene {
  std::vector<vec3> nrm;
  std::vector<vec2> uv;
  std::vector<Image> images;
  std::vector<Mat> mats;
  std::vector<Tri> tris;   // permuted in place by the builder, like Model::faces
  std::vector<Node> nodes; // heap-indexed, children 2u and 2u+1
  std::vector<Light> lights;
  Sky sky;
};

// RandomDistribution, src/component.cpp:12-31.
static void prefix_init(std::vector<float>& p, const std::vector<float>& w) {
  p.resize(w.size());
  p[0] = w[0];
  for (size_t i = 1; i < w.size(); ++i) p[i] = p[i - 1] + w[i];
}
template <class G>
static int prefix_draw(const std::vector<float>& p, G& gen) {
  float x = p.back() * gen();
  return (int)(std::lower_bound(p.begin(), p.end(), x) - p.begin());
}
static float prefix_pdf(const std::vector<float>& p, int i) {
  float now = p[i];
  if (i > 0) now -= p[i - 1];
  return now / p.back();
}

// --------------------------------------------------------------- builder ---
// BVH::dfs_build / nodeCount / build, src/bvh.cpp:18-54: median split on the
// axis of largest centroid variance, std::nth_element on the centroid
// coordinate, leaves of at most 10 triangles, heap-indexed nodes.
static void build_rec(Scene& s, int u, int l, int r) {
  if ((unsigned)(r - l) <= kLeafSize) {
    Node& n = s.nodes[u];
    n.faceL = l;
    n.faceR = r;
    n.box = {vec3(INFINITY), vec3(-INFINITY)};
    for (int i = l; i < r; ++i) n.box = box_union(n.box, tri_box(s.tris[i]));
    return;
  }
  vec3 sum = vec3(0), sum2 = vec3(0);
  for (int i = l; i < r; ++i) {
    vec3 c = tri_center(s.tris[i]);
    sum += c;
    sum2 += c * c;
  }
  vec3 var = sum2 - sum * sum / (float)(r - l);
  int axis = 0;
  if (var[1] > var[0]) axis = 1;
  if (var[2] > var[0] && var[2] > var[1]) axis = 2;
  int m = (r + l) / 2;
  std::nth_element(s.tris.begin() + l, s.tris.begin() + m, s.tris.begin() + r,
                   [axis](const Tri& a, const Tri& b) { return tri_center(a)[axis] < tri_center(b)[axis]; });
  build_rec(s, u << 1, l, m);
  build_rec(s, u << 1 | 1, m, r);
  s.nodes[u].box = box_union(s.nodes[u << 1].box, s.nodes[u << 1 | 1].box);
}
static int heap_slots(int u, int n) { return ((unsigned)n <= kLeafSize) ? u : heap_slots(u << 1 | 1, (n + 1) >> 1); }

// ------------------------------------------------------------- traversal ---
struct Ray { vec3 o, d; };
struct Hit { float tmin, tmax; int face; };

// rayInBox, src/geometry.cpp:40-61 (cumulative tR += eps per axis, early
// return once tL > tR, origin-inside rule for |d| < eps).
static void slab(const Ray& r, const Box& b, float& tL, float& tR) {
  for (int i = 0; i < 3; ++i) {
    if (std::abs(r.d[i]) < kEps) {
      if (r.o[i] < b.lo[i] || r.o[i] > b.hi[i]) { tR = -1.0f; return; }
      continue;
    }
    float inv = 1.0f / r.d[i];
    float lo = inv >= 0 ? b.lo[i] : b.hi[i];
    float hi = inv >= 0 ? b.hi[i] : b.lo[i];
    tL = std::fmax(tL, (lo - r.o[i]) * inv);
    tR = std::fmin(tR, (hi - r.o[i]) * inv);
    tR += kEps;
    if (tL > tR) return;
  }
}

// RayTriangleIntersection (Moller-Trumbore), src/geometry.cpp:63-87.
static float tri_t(const Ray& r, const vec3& v0, const vec3& v1, const vec3& v2) {
  vec3 e1 = v1 - v0, e2 = v2 - v0;
  vec3 h = cross(r.d, e2);
  float a = dot(e1, h);
  if (std::abs(a) / length(e1) < kEps) return INFINITY;
  float f = 1.0f / a;
  vec3 s = r.o - v0;
  float u = f * dot(s, h);
  if (u < 0.0f || u > 1.0f) return INFINITY;
  vec3 q = cross(s, e1);
  float v = f * dot(r.d, q);
  if (v < 0.0f || u + v > 1.0f) return INFINITY;
  return f * dot(e2, q);
}

// BVH::dfs_rayHit, src/bvh.cpp:56-88: near child first (ties go right), the
// far child only if its entry is still closer than the current hit.
static void visit(const Scene& s, int u, const Ray& r, Hit& h, Stats* st) {
  const Node& n = s.nodes[u];
  if (n.faceR) {
    if (st) { st->leaves++; st->tris += (uint64_t)(n.faceR - n.faceL); }
    for (int i = n.faceL; i < n.faceR; ++i) {
      const Tri& f = s.tris[i];
      float t = tri_t(r, f.v[0], f.v[1], f.v[2]);
      if (h.tmin < t && t < h.tmax) { h.tmax = t; h.face = i; }
    }
    return;
  }
  if (st) st->inner++;
  float a0 = h.tmin, b0 = h.tmax, a1 = h.tmin, b1 = h.tmax;
  slab(r, s.nodes[u << 1].box, a0, b0);
  slab(r, s.nodes[u << 1 | 1].box, a1, b1);
  if (a0 < a1) {
    if (a0 < b0) visit(s, u << 1, r, h, st);
    if (a1 < b1 && a1 < h.tmax) visit(s, u << 1 | 1, r, h, st);
  } else {
    if (a1 < b1) visit(s, u << 1 | 1, r, h, st);
    if (a0 < b0 && a0 < h.tmax) visit(s, u << 1, r, h, st);
  }
}
static void traverse(const Scene& s, const Ray& r, Hit& h, Stats* st) {
  if (s.tris.empty()) return;  // the reference indexes past its node array here
  visit(s, 1, r, h, st);
}
static vec3 bary(const vec3& v0, const vec3& v1, const vec3& v2, const vec3& p);
// TransparentTest, src/model.cpp:217-230: the hit is cut away when its
// material's diffuse texture has texels of alpha < 1 and the level-0 alpha at
// the hit is below eps.
static bool alpha_cut(const Scene& s, const Ray& r, const Hit& h) {
  const Tri& f = s.tris[h.face];
  const Mat& m = s.mats[f.mat];
  if (!m.transparent) return false;
  vec3 p = r.o + r.d * h.tmax;
  vec3 b = bary(f.v[0], f.v[1], f.v[2], p);
  vec2 uv = b[0] * s.uv[f.vid[0]] + b[1] * s.uv[f.vid[1]] + b[2] * s.uv[f.vid[2]];
  return m.diffuse4(uv[0], uv[1], NAN)[3] < kEps;
}
constexpr int kAlphaRetries = 8;  // maxRayDepth_hit, src/model.cpp:330
// Model::rayHit, src/model.cpp:332-341: a cut-away hit restarts the search
// eps beyond it, at most 8 times.
static Hit closest(const Scene& s, const Ray& r, Stats* st = nullptr) {
  Hit h{kEps, INFINITY, -1};
  for (int k = 0; k < kAlphaRetries; ++k) {
    traverse(s, r, h, st);
    if (h.tmax == INFINITY || !alpha_cut(s, r, h)) return h;
    h = Hit{h.tmax + kEps, INFINITY, -1};
  }
  return h;
}
// Model::rayHit_test, src/model.cpp:343-354.
static bool occluded(const Scene& s, const Ray& r, float aim, Stats* st = nullptr) {
  Hit h{kEps, aim + kEps, -1};
  for (int k = 0; k < kAlphaRetries; ++k) {
    traverse(s, r, h, st);
    if (h.tmax >= aim) return false;
    if (!alpha_cut(s, r, h)) return true;
    h = Hit{h.tmax + kEps, aim + kEps, -1};
  }
  return true;
}

// barycentric, src/geometry.cpp:89-103 -> (gamma, alpha, beta).
static vec3 bary(const vec3& v0, const vec3& v1, const vec3& v2, const vec3& p) {
  vec3 e1 = v1 - v0, e2 = v2 - v0;
  vec3 n = cross(e1, e2);
  float den = dot(n, n);
  vec3 vp = p - v0;
  float al = dot(cross(vp, e2), n) / den;
  float be = dot(cross(e1, vp), n) / den;
  float ga = 1.0f - al - be;
  return vec3(ga, al, be);
}

// ------------------------------------------------------------- shading -----
struct Surf {  // HitInfo, include/model.h:12-18 with defaults of src/model.cpp:4-7
  vec3 shapeN = vec3(NAN), surfN = vec3(NAN), emis = vec3(0.0f), base = vec3(0.0f), pos = vec3(NAN);
  float specular = 0.04f, roughness = 0.8f, metallic = 0.0f, opacity = 1.0f, eta = 1.0f;
  int id = 0;
  bool entering = true;
};

static bool flip_toward(vec3& v, const vec3& dir) {  // reverseFix, src/model.cpp:232-238
  if (dot(v, dir) < 0.0f) { v *= -1.0f; return false; }
  return true;
}

// getHitNormals, src/model.cpp:240-270.
static void hit_normals(const Scene& s, const Tri& f, const vec3& in, const vec3& b, vec3& shapeN, vec3& surfN,
                        bool& entering) {
  vec3 c = cross(f.v[1] - f.v[0], f.v[2] - f.v[0]);
  shapeN = normalize(c);
  entering = flip_toward(shapeN, -in);
  surfN = shapeN;
  float area = length(c) / 2.0f;
  if (area > 1e-2f) return;
  vec3 n0 = s.nrm[f.vid[0]], n1 = s.nrm[f.vid[1]], n2 = s.nrm[f.vid[2]];
  flip_toward(n0, shapeN);
  flip_toward(n1, shapeN);
  flip_toward(n2, shapeN);
  surfN = normalize(b[0] * (dot(n0, shapeN) > 0.85f ? n0 : shapeN) + b[1] * (dot(n1, shapeN) > 0.85f ? n1 : shapeN) +
                    b[2] * (dot(n2, shapeN) > 0.85f ? n2 : shapeN));
  if (!any_finite(surfN)) surfN = shapeN;
}

// calcSurfaceNormal, src/model.cpp:279-298: the normal-map texel (zero
// without a normal map) in the uv tangent frame.
static void surface_normal(const Scene& s, const Tri& f, const vec3& nm, const vec3& shapeN, vec3& surfN) {
  vec3 e1 = f.v[1] - f.v[0], e2 = f.v[2] - f.v[0];
  vec2 d1 = s.uv[f.vid[1]] - s.uv[f.vid[0]], d2 = s.uv[f.vid[2]] - s.uv[f.vid[0]];
  float k = 1.0f / (d1.x * d2.y - d2.x * d1.y);
  vec3 tu = k * (d2.y * e1 - d1.y * e2), tv = k * (-d2.x * e1 + d1.x * e2);
  vec3 t = normalize(tu - shapeN * dot(shapeN, tu));
  vec3 bt = normalize(tv - shapeN * dot(shapeN, tv) - t * dot(t, tv));
  vec3 keep = surfN;
  surfN = normalize(t * nm.x + bt * nm.y + surfN);
  if (!any_finite(surfN)) surfN = keep;
}

// RayDifferential, include/render.h:29-33.
struct Diff { vec3 dPdx = vec3(0.0f), dPdy = vec3(0.0f), dDdx = vec3(0.0f), dDdy = vec3(0.0f); };

// calc_dPdxy, src/render.cpp:44-50.
static void calc_dPdxy(const Ray& r, float t, const vec3& n, const Diff& d, vec3& px, vec3& py) {
  float dtdx = -dot(d.dPdx + t * d.dDdx, n) / dot(r.d, n);
  float dtdy = -dot(d.dPdy + t * d.dDdy, n) / dot(r.d, n);
  px = d.dPdx + dtdx * r.d + t * d.dDdx;
  py = d.dPdy + dtdy * r.d + t * d.dDdy;
}
// calc_dDdxy, src/render.cpp:52-60 (the normal's derivatives are zero).
static void calc_dDdxy(const Ray& r, const vec3& n, const Diff& d, vec3& dx, vec3& dy) {
  const vec3 dN(0.0f);
  float dDNdx = dot(dN, r.d) + dot(d.dDdx, n);
  float dDNdy = dot(dN, r.d) + dot(d.dDdy, n);
  dx = d.dDdx - 2.0f * (dot(r.d, n) * dN + dDNdx * n);
  dy = d.dDdy - 2.0f * (dot(r.d, n) * dN + dDNdy * n);
}
static bool any_finite2(const vec2& v) { return std::isfinite(v.x) || std::isfinite(v.y); }
// getDuv, src/model.cpp:272-277.
static vec2 get_duv(const Scene& s, const Tri& f, const vec3& dP) {
  vec3 b = bary(f.v[0], f.v[1], f.v[2], f.v[0] + dP);
  return (b[0] - 1.0f) * s.uv[f.vid[0]] + b[1] * s.uv[f.vid[1]] + b[2] * s.uv[f.vid[2]];
}

// getHitInfo + getHitMaterial, src/render.cpp:62-79 and src/model.cpp:
// 300-328: t is the hit distance along r, d the ray's differential (texture
// level of detail); hit_dPdx / hit_dPdy receive the hit point's.
static void hit_info(const Scene& s, const Tri& f, const Ray& r, float t, const Diff& d, Surf& h, vec3* hit_dPdx = nullptr,
                     vec3* hit_dPdy = nullptr) {
  vec3 b = bary(f.v[0], f.v[1], f.v[2], h.pos);
  hit_normals(s, f, r.d, b, h.shapeN, h.surfN, h.entering);
  vec3 raw = h.surfN;
  vec3 px, py;
  calc_dPdxy(r, t, h.shapeN, d, px, py);
  vec2 uv = b[0] * s.uv[f.vid[0]] + b[1] * s.uv[f.vid[1]] + b[2] * s.uv[f.vid[2]];
  const Mat& m = s.mats[f.mat];
  h.id = m.id;
  m.surface(h.roughness, h.metallic, uv[0], uv[1]);
  h.opacity = m.opacity;
  h.eta = m.ior;
  if (h.opacity > 1.0f - kEps) h.entering = true;
  vec2 ux = get_duv(s, f, px), uy = get_duv(s, f, py);
  float duv = (any_finite2(ux) && any_finite2(ux)) ? (length(ux) + length(uy)) / 2.0f : NAN;
  h.base = (h.opacity < kEps) ? m.trans : m.diffuse(uv[0], uv[1], duv);
  h.emis = m.emission(uv[0], uv[1], duv);
  vec3 nm = m.normal_map(uv[0], uv[1], duv);
  surface_normal(s, f, nm, h.shapeN, h.surfN);
  if (dot(h.surfN, r.d) >= 0.0f) h.surfN = raw;
  if (dot(h.surfN, r.d) >= 0.0f) h.surfN = h.shapeN;
  if (hit_dPdx) *hit_dPdx = px;
  if (hit_dPdy) *hit_dPdy = py;
}

// ---------------------------------------------------------------- BSDF -----
static float pow5(float x) { float x2 = x * x; return x2 * x2 * x; }           // src/sampling.cpp:20-23
static float schlick(float u) { return pow5(fclampf(1 - u, 0, 1)); }          // :25-28
static float gtr1(float c, float a) {                                          // :30-35
  if (a >= 1) return 1 / kPi;
  float a2 = a * a;
  float t = 1 + (a2 - 1) * c * c;
  return (a2 - 1) / (kPi * std::log(a2) * t);
}
static float gtr2(float c, float a) {                                          // :37-41
  float a2 = a * a;
  float t = 1 + (a2 - 1) * c * c;
  return a2 / (kPi * t * t);
}
static float smith_g(float c, float ag) {                                      // :43-47
  float a = ag * ag, b = c * c;
  return 1 / (c + std::sqrt(a + b - a * b));
}
static void lum_clamp(vec3& v) {                                               // :238-243
  float l = dot(v, kLum);
  if (l > 64.0f) v /= l / 64.0f;
}

struct Bsdf {
  vec3 in;  // direction towards the previous vertex
  Surf s;

  // BSDF::getBRDF, src/sampling.cpp:49-157 (subsurface, sheen and tints 0,
  // clearcoat 1.5, clearcoat gloss 0.2).
  vec3 brdf(const vec3& L) const {
    const vec3& V = in;
    const vec3& N = s.surfN;
    float nl = dot(N, L), nv = dot(N, V);
    if (nl <= 0.0f || nv <= 0.0f) return vec3(0);
    vec3 H = normalize(L + V);
    float nh = dot(N, H), lh = dot(L, H);
    vec3 cd = s.base;
    float cdl = dot(cd, kLum);
    vec3 tint = cdl > 0.0f ? cd / cdl : vec3(1.0f);
    vec3 spec0 = glm::mix(s.specular * glm::mix(vec3(1.0f), tint, 0.0f), cd, s.metallic);
    vec3 sheenc = glm::mix(vec3(1.0f), tint, 0.0f);
    float fl = schlick(nl), fv = schlick(nv);
    float fd90 = 0.5f + 2.0f * lh * lh * s.roughness;
    float fd = fmix(1.0f, fd90, fl) * fmix(1.0f, fd90, fv);
    float fss90 = lh * lh * s.roughness;
    float fss = fmix(1.0f, fss90, fl) * fmix(1.0f, fss90, fv);
    float ss = 1.25f * (fss * (1.0f / (nl + nv) - .5f) + .5f);
    float ds = gtr2(nh, s.roughness);
    float fh;
    if (s.eta <= 1.0f) {
      fh = schlick(lh);
    } else {
      float ci = std::fabs(lh);
      float si = ci * ci;
      si = (1.0f - si) <= 0.0f ? 0.0f : std::sqrt(1.0f - si);
      float st = s.eta * si;
      if (st >= 1.0f) {
        fh = 1.0f;
      } else {
        float ct = (1.0f - st * st) <= 0.0f ? 0.0f : std::sqrt(1.0f - st * st);
        float r0 = (s.eta - 1.0f) / (s.eta + 1.0f);
        r0 = r0 * r0;
        fh = fmix(r0, 1.0f, schlick(ct));
      }
    }
    vec3 fs = glm::mix(spec0, vec3(1.0f), fh);
    float gs = smith_g(nl, s.roughness);
    gs *= smith_g(nv, s.roughness);
    vec3 fsheen = fh * 0.0f * sheenc;
    float dr = gtr1(nh, fmix(.1f, .001f, 0.2f));
    float fr = fmix(.04f, 1.0f, fh);
    float gr = smith_g(nl, .25f) * smith_g(nv, .25f);
    vec3 ret = ((1.0f / kPi) * fmix(fd, ss, 0.0f) * cd + fsheen);
    ret *= (1.0f - s.metallic);
    ret += (0.25f * 1.5f * gr * fr * dr) * glm::mix(vec3(1.0f), tint, 0.0f);
    ret *= s.opacity;
    ret += fs * ds * gs;
    return ret * nl;
  }
  // BSDF::getBTDF, src/sampling.cpp:159-192.
  vec3 btdf(const vec3& L) const {
    const vec3& N = s.surfN;
    float nl = dot(s.surfN, L);
    if (nl >= 0.0f) return vec3(0.0f);
    const vec3& V = in;
    vec3 H = normalize(L + s.eta * V);
    float D = gtr2(dot(N, H), s.roughness);
    float bt = D * (-nl);
    float lh = dot(L, H), nv = dot(N, V), hv = dot(H, V);
    bt *= std::abs(lh * hv) / (std::abs(nl * nv) + kEps);
    float k = s.eta * hv + lh;
    bt /= k * k;
    return vec3(bt);
  }
  // BSDF::getBSDF, :194-199: the BTDF on the far side of a transmissive
  // surface, the BRDF otherwise.
  vec3 eval(const vec3& L) const {
    if (s.opacity > 1.0f - kEps || s.entering) return brdf(L);
    return btdf(L);
  }
  // BSDF::preciseRefraction, :285-308.
  void precise_refraction(vec3& out, float& F) const {
    const vec3& V = in;
    const vec3& N = s.surfN;
    float eta = s.eta;
    float nv = dot(N, V);
    if (nv < 0.0f) { F = 1.0f; out = vec3(NAN); return; }
    float delta = 1.0f - eta * eta * (1.0f - nv * nv);
    if (delta < 0.0f) { F = 1.0f; out = vec3(NAN); return; }
    float k = eta * nv - std::sqrt(delta);
    out = k * N - eta * V;
    float ln = -dot(out, N);
    float r0 = (1.0f - eta) / (1.0f + eta);
    r0 = r0 * r0;
    F = r0 + (1.0f - r0) * schlick(ln);
  }
  // refract, :342-349.
  static vec3 refract(const vec3& V, const vec3& N, float eta) {
    float nv = dot(N, V);
    float delta = 1.0f - eta * eta * (1.0f - nv * nv);
    if (delta < 0.0f) return vec3(NAN);
    float k = eta * nv - std::sqrt(delta);
    return k * N - eta * V;
  }
  // BSDF::sampleBTDF, :351-388 (GGX half vector, refracted; <= 16 tries).
  template <class G>
  void sample_btdf(G& gen, vec3& out, vec3& w, int& fails) const {
    if (std::abs(s.eta - 1.0f) < kEps) {
      out = -in;
      w = vec3(1.0f);
      return;
    }
    vec3 t, b;
    frame(t, b);
    const vec3& V = in;
    for (int T = 1; T <= kMaxTrys; ++T) {
      float u = gen(), phi = gen() * 2.0f * kPi;
      float ct = std::sqrt((1.0f - u) / (1.0f + (s.roughness * s.roughness - 1.0f) * u));
      float st = std::sqrt(1 - ct * ct);
      vec3 H = st * std::cos(phi) * t + st * std::sin(phi) * b + ct * s.surfN;
      out = refract(V, H, s.eta);
      float weight;
      if (!any_finite(out)) {
        weight = 0.0f;
      } else {
        float vh = dot(V, H), vn = dot(V, s.surfN), hn = dot(H, s.surfN);
        weight = std::abs(vh) / std::abs(vn * hn);
      }
      if (weight > 0.0f && dot(out, s.shapeN) < 0.0f) {
        w = vec3(weight);
        return;
      }
      fails++;
    }
    w = vec3(0.0f);
    out = vec3(NAN);
  }

  // getTangentSpaceWithInDir, src/geometry.cpp:114-124 (the fallback branch
  // needs dot(N, in) < -0.999, which hit shading rules out).
  void frame(vec3& t, vec3& b) const {
    float c = dot(s.surfN, in);
    if (c < -1.0f + 1e-3f) {
      vec3 v0 = std::fabs(s.surfN.x) < 0.8f ? vec3(1.0f, 0.0f, 0.0f) : vec3(0.0f, 1.0f, 0.0f);
      t = normalize(cross(v0, s.surfN));
      b = cross(s.surfN, t);
      return;
    }
    b = normalize(cross(s.surfN, in));
    t = cross(b, s.surfN);
  }

  // BSDF::sampleBRDF, :203-236 (GGX half-vector sampling, <= 16 tries).
  template <class G>
  void sample_ggx(G& gen, vec3& out, vec3& w, float& pdf, int& fails) const {
    vec3 t, b;
    frame(t, b);
    for (int T = 1; T <= kMaxTrys; ++T) {
      float u = gen(), phi = gen() * 2.0f * kPi;
      float ct = std::sqrt((1.0f - u) / (1.0f + (s.roughness * s.roughness - 1.0f) * u));
      float st = std::sqrt(1 - ct * ct);
      vec3 H = st * std::cos(phi) * t + st * std::sin(phi) * b + ct * s.surfN;
      out = 2.0f * dot(in, H) * H - in;
      float lh = dot(out, H), ln = dot(out, s.surfN);
      if (lh <= 0.0f || ln <= 0.0f) pdf = 0.0f;
      else pdf = gtr2(ct, s.roughness) / (4.0f * lh);
      if (dot(out, s.shapeN) > 0.0f && pdf > 0.0f) { w = brdf(out) / pdf; return; }
      fails++;
    }
    pdf = 0.0f;
    w = vec3(0.0f);
    out = vec3(NAN);
  }
  // BSDF::sampleCos, :245-269 (cosine sampling, luminance clamp 64).
  template <class G>
  void sample_cos(G& gen, vec3& out, vec3& w, float& pdf, int& fails) const {
    vec3 t, b;
    frame(t, b);
    for (int T = 1; T <= kMaxTrys; ++T) {
      float u = gen(), phi = gen() * 2.0f * kPi;
      float d = std::sqrt(u);
      float z = std::sqrt(1 - d * d);
      float x = d * std::cos(phi), y = d * std::sin(phi);
      out = x * t + y * b + z * s.surfN;
      pdf = dot(out, s.surfN) / kPi;
      if (dot(out, s.shapeN) > 0.0f && pdf > 0.0f) {
        w = brdf(out) / pdf;
        lum_clamp(w);
        return;
      }
      fails++;
    }
    pdf = 0.0f;
    w = vec3(0.0f);
    out = vec3(NAN);
  }
  // BSDF::sampleReflection, :310-340: draw both, keep one with p1 = pdf1/(pdf1+pdf2).
  template <class G>
  void sample_reflect(G& gen, vec3& dir, vec3& w, int& fails) const {
    vec3 d1, d2, w1, w2;
    int f1 = 0, f2 = 0;
    float p1, p2;
    sample_cos(gen, d1, w1, p1, f1);
    sample_ggx(gen, d2, w2, p2, f2);
    float pc = p1 / (p1 + p2);
    if (gen() < pc) { dir = d1; w = w1; fails += f1; }
    else { dir = d2; w = w2; fails += f2; }
  }
};

// --------------------------------------------------------- light sampling --
struct LSample {  // LightSample, include/sampling.h:28-32
  vec3 bsdf, light;
  float weight;
};

// generateRandomPointInLightFace + sampleLightFace, src/sampling.cpp:419-448.
template <class G>
static void light_point(const Scene& s, const Light& lo, const vec3& pos, G& gen, vec3& lp, int& fails) {
  for (int T = 1; T <= kMaxTrys; ++T) {
    int fi = prefix_draw(lo.prefix, gen);
    const Tri& f = lo.faces[fi];
    float a = gen(), b = gen();
    if (a + b > 1.0f) { a = 1.0f - a; b = 1.0f - b; }
    float c = 1.0f - a - b;
    lp = a * f.v[0] + b * f.v[1] + c * f.v[2];
    vec3 ld = normalize(lp - pos);
    vec3 sn, un;
    bool ent;
    hit_normals(s, f, ld, vec3(a, b, c), sn, un, ent);
    float cphi = dot(un, -ld);
    if (cphi > 0.0f && gen() < cphi) return;
    fails++;
  }
  lp = vec3(NAN);
}

// sampleSkyBox, src/sampling.cpp:450-465.
template <class G>
static void sky_dir(const Sky& k, const vec3& n, G& gen, vec3& dir, vec3& light) {
  for (int T = 1; T <= kMaxTrys; ++T) {
    int p = prefix_draw(k.prefix, gen);
    int u = p % k.w, v = p / k.w;
    float phi = kPi * (float(v) + 0.5f) / float(k.h);
    float th = 2.0f * kPi * (float(u) + 0.5f) / float(k.w);
    dir = vec3(-std::sin(phi) * std::sin(th), std::cos(phi), std::sin(phi) * std::cos(th));
    if (dot(dir, n) > 0.0f) { light = k.data[p] / prefix_pdf(k.prefix, p); return; }
  }
  dir = vec3(NAN);
}

// SkyBox::get, src/component.cpp:120-140.
static vec3 sky_get(const Sky& k, const vec3& dir) {
  if (k.empty()) return vec3(0.0f);
  float th = std::atan2(-dir.x, dir.z);
  float phi = std::acos(dir.y);
  if (th < 0.0f) th += 2.0f * kPi;
  int u = (int)(th / (2.0f * kPi) * float(k.w));
  int v = (int)(phi / kPi * float(k.h));
  u = u < 0 ? 0 : (u >= k.w ? k.w - 1 : u);
  v = v < 0 ? 0 : (v >= k.h ? k.h - 1 : v);
  phi = kPi * (float(v) + 0.5f) / float(k.h);
  float area = std::sin(phi) * 2.0f * kPi / float(k.w * k.h);
  return k.data[v * k.w + u] / area;
}

// sampleDirectLight, src/sampling.cpp:467-527. gen_of(T) yields the generator
// of light sample T (one stream for all T in the reference).
template <class GenOf>
static void direct_light(const Scene& s, const Bsdf& bs, int cnt, GenOf&& gen_of, std::vector<LSample>& out) {
  const vec3& pos = bs.s.pos;
  if (s.sky.empty()) {
    std::vector<float> w;
    w.reserve(s.lights.size());
    for (const Light& lo : s.lights) {  // getLightObjectWeight, :406-417
      vec3 ld = normalize(lo.center - pos);
      float dist = length(lo.center - pos);
      vec3 f = bs.eval(ld);
      w.push_back(dot(f, kLum) * lo.power / (dist * dist + kLightRadius));
    }
    float tot = 0.0f;
    for (float x : w) tot += x;
    if (tot == 0.0f) return;
    for (int T = 0; T < cnt; ++T) {
      auto& gen = gen_of(T);
      float rv = tot * gen();  // sample(), :396-404
      int li = -1;
      float acc = 0.0f;
      for (size_t i = 0; i < w.size(); ++i) {
        acc += w[i];
        if (rv <= acc) { li = (int)i; break; }
      }
      if (li == -1) continue;
      float pl = w[li] / tot;
      const Light& lo = s.lights[li];
      vec3 lp;
      int fails = 0;
      light_point(s, lo, pos, gen, lp, fails);
      if (!any_finite(lp)) continue;
      vec3 ld = normalize(lp - pos);
      float dist = length(lp - pos);
      if (occluded(s, {pos, ld}, dist - kEps)) continue;
      vec3 f = bs.eval(ld);
      lum_clamp(f);
      vec3 L = 2.0f * kPi * lo.power * lo.color / (dist * dist + kLightRadius) / pl;
      out.push_back({f, L, 1.0f / (float)(cnt * (fails + 1))});
    }
  } else {
    for (int T = 0; T < cnt; ++T) {
      auto& gen = gen_of(T);
      vec3 dir, L;
      sky_dir(s.sky, bs.s.surfN, gen, dir, L);
      if (!any_finite(dir)) continue;
      if (occluded(s, {pos, dir}, INFINITY)) continue;
      vec3 f = bs.eval(dir);
      lum_clamp(f);
      out.push_back({f, L, 1.0f / (float)cnt});
    }
  }
}

// ------------------------------------------------------------- media -------
// Medium, src/render.cpp:11-42: the media a path is inside, keyed by
// material id (air: -1), as the reference's multimap.
struct Medium {
  std::multimap<int, std::pair<float, vec3>> m;
  void init() {
    m.clear();
    m.emplace(-1, std::make_pair(1.0f, vec3(1.0f)));
  }
  void insert(int id, float ior, const vec3& absorb) { m.emplace(id, std::make_pair(ior, absorb)); }
  void erase(int id) { m.erase(id); }
  float ior() const {
    float r = 1.0f;
    for (const auto& e : m) r = std::max(r, e.second.first);
    return r;
  }
  vec3 absorb() const {
    vec3 a = vec3(1.0f);
    for (const auto& e : m) a *= e.second.second;
    return a;
  }
  int size() const { return (int)m.size(); }
};

static vec3 pow_s(vec3 v, float k) {  // src/geometry.cpp:22-27
  if (v.x < 0.0f) v.x = 0.0f;
  if (v.y < 0.0f) v.y = 0.0f;
  if (v.z < 0.0f) v.z = 0.0f;
  return vec3(std::pow(v.x, k), std::pow(v.y, k), std::pow(v.z, k));
}

// getAbsorb, src/render.cpp:83-87.
static vec3 get_absorb(const vec3& absorb, float dis) {
  const float omega = 32.0f;
  float c = dot(absorb, kLum);
  return (c < 1.0f - kEps) ? pow_s(absorb, omega * dis) : vec3(1.0f);
}

// calcEta, src/render.cpp:89-99: the relative index of refraction.
static void calc_eta(Medium& med, Surf& h) {
  float eta1 = med.ior(), eta2;
  if (h.entering) {
    eta2 = std::max(eta1, h.eta);
  } else {
    med.erase(h.id);
    eta2 = med.ior();
    med.insert(h.id, h.eta, h.base);
  }
  h.eta = eta1 / eta2;
}

constexpr float kP0Reflect = 0.24f;  // P0_reflect, src/render.cpp:118

// ---------------------------------------------------------- integrator -----
// One indirect sample from the first vertex: sampleIndirectLightFromFirst-
// Intersection (src/render.cpp:314-423) followed by the sampleRay recursion
// (:121-312), unrolled into a loop. The recursion hands samples back up and
// multiplies each vertex's factor into them innermost first (passBsdf,
// mulWeight, :101-116); the loop keeps the per-depth factors and applies them
// in that order so the float products match.
template <class G>
static void indirect_path(const Scene& s, const Surf& g, const vec3& eye, const Diff& d0, int maxd, G& gen,
                          std::vector<LSample>& out) {
  if (length(g.emis) > 0) return;
  Medium med;
  med.init();
  vec3 in = normalize(g.pos - eye);
  Bsdf b0{-in, g};
  float rf = g.roughness * 1.0f;
  const float ior0 = b0.s.eta;
  b0.s.eta = 1.0f / b0.s.eta;  // from air into the surface
  float p_reflect = 1.0f, F0 = 0.0f;
  if (b0.s.opacity < kEps) {
    vec3 rd;
    b0.precise_refraction(rd, F0);
    p_reflect = kP0Reflect + (1.0f - kP0Reflect) * F0;
  }
  vec3 dir, w0 = vec3(NAN);
  int f0 = 0;
  Diff diff = d0;  // the refracted ray keeps the camera ray's differential
  if (gen() < p_reflect) {
    const Ray cam{eye, in};
    calc_dPdxy(cam, length(g.pos - eye), b0.s.shapeN, d0, diff.dPdx, diff.dPdy);
    calc_dDdxy(cam, b0.s.surfN, d0, diff.dDdx, diff.dDdy);
    b0.sample_reflect(gen, dir, w0, f0);
    w0 /= p_reflect;
  } else {
    b0.sample_btdf(gen, dir, w0, f0);
    w0 *= (1.0f - F0);
    w0 /= (1.0f - p_reflect);
    if (b0.s.entering) med.insert(b0.s.id, ior0, b0.s.base);
    else med.erase(b0.s.id);
  }
  if (!any_finite(dir)) return;

  vec3 fac[18];
  int fails[18];
  Ray ray{b0.s.pos, dir};
  bool exclude = true;
  std::vector<LSample> term;
  int depth = 1;
  for (;; ++depth) {
    term.clear();
    Hit h = closest(s, ray);
    if (h.tmax == INFINITY) {
      if (!exclude && !s.sky.empty()) term.push_back({vec3(1.0f), sky_get(s.sky, ray.d), 1.0f});
      break;
    }
    Bsdf bs{-ray.d, Surf()};
    bs.s.pos = ray.o + ray.d * h.tmax;
    vec3 hpx, hpy;
    hit_info(s, s.tris[h.face], ray, h.tmax, diff, bs.s, &hpx, &hpy);
    const float ior = bs.s.eta;
    rf = std::max(rf, 1.0f * bs.s.roughness);
    bs.s.roughness = std::max(bs.s.roughness, rf);
    const float p_rr = 1.0f + (0.5f - 1.0f) * std::sqrt(bs.s.roughness);
    bool nee = p_rr < 0.9f;
    const vec3 absorb = get_absorb(med.absorb(), h.tmax);
    if (length(bs.s.emis) > kEps) {
      if (!exclude) term.push_back({absorb, bs.s.emis, 1.0f});
      break;
    }
    float pr = 1.0f, F = 0.0f;
    if (bs.s.opacity < kEps) {
      calc_eta(med, bs.s);
      vec3 rd;
      bs.precise_refraction(rd, F);
      pr = (med.size() == 1) ? kP0Reflect + (1.0f - kP0Reflect) * F : F;
      pr = std::max(pr - 1e-3f, 0.0f);
    }
    const int cnt = kSampleCount[std::min(depth, 16)];
    vec3 nd, w;
    int nf = 0;
    if (gen() <= pr) {  // reflection
      nee = nee && bs.s.entering && med.size() == 1;
      if (nee && (depth >= maxd || gen() > p_rr)) {
        direct_light(s, bs, cnt, [&](int) -> G& { return gen; }, term);
        float k = 1.0f / pr;
        if (depth < maxd) k /= (1.0f - p_rr);
        for (LSample& x : term) x.bsdf *= k;
        break;
      }
      bs.sample_reflect(gen, nd, w, nf);
      w /= pr;
      if (nee) w /= p_rr;
      vec3 ddx, ddy;
      calc_dDdxy(ray, bs.s.surfN, diff, ddx, ddy);
      diff = Diff{hpx, hpy, ddx, ddy};
    } else {  // refraction
      nee = nee && !bs.s.entering && med.size() == 2;
      if (nee && (depth >= maxd || gen() > p_rr)) {
        direct_light(s, bs, cnt, [&](int) -> G& { return gen; }, term);
        float k = 1.0f / (1.0f - pr);
        if (depth < maxd) k /= (1.0f - p_rr);
        for (LSample& x : term) x.bsdf *= k;
        for (LSample& x : term) { x.light *= x.bsdf; x.bsdf = absorb; }  // passBsdf(samples, absorb)
        break;
      }
      if (std::abs(bs.s.eta - 1.0f) < kEps) {
        nd = ray.d;
        w = vec3(1.0f);
      } else {
        bs.sample_btdf(gen, nd, w, nf);
        w *= (1.0f - F);
      }
      w /= (1.0f - pr);
      if (nee) w /= p_rr;
      if (bs.s.entering) med.insert(bs.s.id, ior, bs.s.base);
      else med.erase(bs.s.id);
    }
    if (!any_finite(nd) || depth == maxd) { term.clear(); break; }
    w *= absorb;
    fac[depth] = w;
    fails[depth] = nf;
    ray = {bs.s.pos, nd};
    exclude = nee;
  }
  for (int k = depth - 1; k >= 1; --k) {
    for (LSample& x : term) { x.light *= x.bsdf; x.bsdf = fac[k]; }
    if (fails[k] > 0)
      for (LSample& x : term) x.weight *= 1.0f / (float)(1 + fails[k]);
  }
  for (LSample& x : term) { x.light *= x.bsdf; x.bsdf = w0; }
  if (f0 > 0)
    for (LSample& x : term) x.weight *= 1.0f / (float)(1 + f0);
  out.insert(out.end(), term.begin(), term.end());
}

struct Rad { vec3 r = vec3(0.0f); float var = 0.0f; };  // RadianceData

// accumulateInwardRadiance(_basic), src/image.cpp:615-659: split into a
// part along normalize(baseColor) (demodulated by |baseColor|) and the rest.
static void acc_basic(Rad& r, const vec3& in, float w) {
  if (!any_finite(in)) return;
  if (!std::isfinite(w)) return;
  r.r += in * w;
  r.var += dot(in, in) * w;
}
static void accumulate(const vec3& base, const LSample& x, Rad& d, Rad& sp) {
  if (length(x.light) < kEps) return;
  vec3 b0 = normalize(base);
  if (length(base) < kEps) { acc_basic(sp, x.light * x.bsdf, x.weight); return; }
  static const vec3 white = normalize(vec3(1.0f));
  float xy = dot(b0, white);
  if (xy > 0.99f) { acc_basic(d, x.light * x.bsdf / base, x.weight); return; }
  vec3 perp = normalize(cross(b0, white));
  vec3 bp = x.bsdf - perp * dot(perp, x.bsdf);
  float d1 = dot(bp, white), d2 = dot(bp, b0);
  float apb = (d1 + d2) / (1 + xy), amb = (d1 - d2) / (1 - xy);
  float B = (apb - amb) / 2.0f;
  vec3 bb = B * b0;
  acc_basic(d, x.light * B / length(base), x.weight);
  acc_basic(sp, x.light * (x.bsdf - bb), x.weight);
}
static void calc_var(Rad& r, float e) {  // renderPixel's calcVar, src/render.cpp:510-516
  r.r *= e;
  r.var *= e * e;
  r.var -= dot(r.r, r.r);
  if (r.var < 0.0f) r.var = 0.0f;
}

struct Args {
  vec3 pos, dir, up, right;
  float accuracy, focus, coc, exposure, p_direct;
  int w, h, spp, threads, maxd;
};

// Generator, src/component.cpp:5-10.
struct MtGen {
  std::mt19937 mt;
  std::uniform_real_distribution<float> U;
  explicit MtGen(uint32_t seed) : mt(seed), U(1e-6f, 1.0f - 1e-6f) {}
  float operator()() { return U(mt); }
};
struct CtrGen {
  RmnRng r;
  float operator()() { return r.next(); }
};

// initRayDiff, src/render.cpp:439-446: the camera ray's differential for
// the unnormalised pixel direction d.
static Diff ray_diff(const vec3& d, const Args& a) {
  Diff r;
  const vec3 ddx = a.accuracy * a.right, ddy = a.accuracy * a.up;
  float dd = dot(d, d), dx = dot(d, ddx), dy = dot(d, ddy);
  r.dDdx = (dd * ddx - d * dx) / (std::sqrt(dd) * dd);
  r.dDdy = (dd * ddy - d * dy) / (std::sqrt(dd) * dd);
  return r;
}

// renderPixel, src/render.cpp:448-551. mode 0: one mt19937 per pixel seeded
// with orc_pixel_seed (reference stream); mode 1: the library's counter
// stream, one per (pixel, sample slot).
static void render_pixel(const Scene& s, const Args& a, uint64_t seed, int mode, int x, int y, float* rec) {
  std::memset(rec, 0, sizeof(float) * ORC_PIX_FLOATS);
  const int id = y * a.w + x;
  float rx = float(x) - float(a.w) / 2.0f, ry = float(y) - float(a.h) / 2.0f;
  vec3 d = a.dir + a.accuracy * (rx * a.right + ry * a.up);
  const Diff d0 = ray_diff(d, a);
  vec3 dir = normalize(d);
  Ray ray{a.pos, dir};
  Surf g;
  Rad Dd, Ds, Id, Is;
  int nsamples = 0, spp_i = 0;
  Hit h = closest(s, ray);
  vec3 base_out;
  if (h.tmax == INFINITY) {
    g.pos = vec3(NAN);
    if (!s.sky.empty()) g.emis = sky_get(s.sky, dir);
    base_out = g.base;
  } else {
    g.pos = ray.o + h.tmax * ray.d;
    hit_info(s, s.tris[h.face], ray, h.tmax, d0, g);
    bool opaque = g.opacity > 1.0f - kEps;
    vec3 keep = g.base;
    float c0 = dot(g.base, kLum);
    if (c0 < 2e-2 || (c0 < 0.8f && length(g.base / c0 - vec3(1.0f)) < 2e-2)) g.base[0] += 4e-2;
    const int spp_d = int(float(a.spp) * a.p_direct);
    spp_i = (a.spp - spp_d) * (opaque ? 1 : 16);

    MtGen mt(orc_pixel_seed(seed, (uint32_t)id));
    CtrGen ctr{rmn_rng(seed, (uint32_t)id, 0)};

    // sampleDirectLightFromFirstIntersection, :425-437.
    if (any_finite(g.pos) && !(length(g.emis) > 0)) {
      vec3 in = normalize(g.pos - a.pos);
      Bsdf bs{-in, g};
      std::vector<LSample> ds;
      if (mode == 0) {
        direct_light(s, bs, spp_d, [&](int) -> MtGen& { return mt; }, ds);
      } else {
        direct_light(s, bs, spp_d, [&](int T) -> CtrGen& { ctr = CtrGen{rmn_rng(seed, (uint32_t)id, (uint32_t)T)}; return ctr; }, ds);
      }
      for (const LSample& x : ds) accumulate(g.base, x, Dd, Ds);
    }
    calc_var(Dd, a.exposure);
    calc_var(Ds, a.exposure);

    std::vector<LSample> samples;
    for (int T = 0; T < spp_i; ++T) {
      if (mode == 0) {
        indirect_path(s, g, a.pos, d0, a.maxd, mt, samples);
      } else {
        CtrGen c{rmn_rng(seed, (uint32_t)id, (uint32_t)(spp_d + T))};
        indirect_path(s, g, a.pos, d0, a.maxd, c, samples);
      }
    }
    nsamples = (int)samples.size();
    if (!samples.empty()) {
      for (LSample& x : samples) x.weight *= 1.0f / (float)spp_i;
      float mean = 0.0f;
      for (const LSample& x : samples) mean += dot(x.bsdf * x.light, kLum) * x.weight;
      vec3 base_acc = g.opacity < kEps ? vec3(0.0f) : g.base;
      for (const LSample& x : samples) {  // per-pixel firefly clamp, :532-549
        float c = dot(x.bsdf * x.light, kLum) * x.weight;
        if (c / (mean - c + kEps) > 16.0f) continue;
        accumulate(base_acc, x, Id, Is);
      }
      calc_var(Id, a.exposure);
      calc_var(Is, a.exposure);
      g.base = keep;
    }
    base_out = g.base;
  }
  const Rad* rr[4] = {&Dd, &Ds, &Id, &Is};
  for (int k = 0; k < 4; ++k) {
    rec[4 * k + 0] = rr[k]->r.x; rec[4 * k + 1] = rr[k]->r.y; rec[4 * k + 2] = rr[k]->r.z; rec[4 * k + 3] = rr[k]->var;
  }
  auto put3 = [&](int o, const vec3& v) { rec[o] = v.x; rec[o + 1] = v.y; rec[o + 2] = v.z; };
  put3(16, base_out);
  put3(19, g.emis);
  put3(22, g.pos);
  put3(25, g.shapeN);
  put3(28, g.surfN);
  rec[31] = g.roughness; rec[32] = g.metallic; rec[33] = g.opacity; rec[34] = g.specular; rec[35] = g.eta;
  rec[36] = (float)g.id; rec[37] = g.entering ? 1.0f : 0.0f; rec[38] = (float)nsamples; rec[39] = (float)spp_i;
}

// ------------------------------------------------------------- post --------
// Photo::shade(Full) + gammaCorrection, src/image.cpp:215-246 and :454-468.
static vec3 compose(const float* rec, float exposure) {
  vec3 rd = vec3(0.0f), rs = vec3(0.0f);
  rd += vec3(rec[0], rec[1], rec[2]);
  rs += vec3(rec[4], rec[5], rec[6]);
  rd += vec3(rec[8], rec[9], rec[10]);
  rs += vec3(rec[12], rec[13], rec[14]);
  vec3 p = vec3(rec[16], rec[17], rec[18]) * rd + rs;
  p += vec3(rec[19], rec[20], rec[21]) * exposure;
  return p;
}
static vec3 gamma(vec3 p) {
  p = glm::max(p, 0.0f);
  float c = dot(p, kLum);
  if (c > 0.75f) p = p / c * (std::tanh(3.0f * (c - 0.75f)) / 3.0f + 0.75f);
  p = glm::min(p, 1.0f);
  return glm::pow(p, vec3(1.0f / 2.2f));
}

// Photo::FXAA, src/image.cpp:358-452.
static void fxaa(const float* in, float* out, int W, int H) {
  auto px = [&](int x, int y) { const float* p = in + 3 * ((size_t)y * W + x); return vec3(p[0], p[1], p[2]); };
  auto lum = [&](int x, int y) { return dot(px(x, y), kLum); };
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      vec3 c = px(x, y);
      vec3 o = c;
      float M = lum(x, y);
      float N = y > 0 ? lum(x, y - 1) : M, S = y < H - 1 ? lum(x, y + 1) : M;
      float E = x < W - 1 ? lum(x + 1, y) : M, Wl = x > 0 ? lum(x - 1, y) : M;
      float lo = std::min({N, S, E, Wl}), hi = std::max({N, S, E, Wl});
      float range = hi - lo;
      if (!(range < std::max(0.0312f, hi * 0.125f))) {
        float NW = (y > 0 && x > 0) ? lum(x - 1, y - 1) : M;
        float NE = (y > 0 && x < W - 1) ? lum(x + 1, y - 1) : M;
        float SW = (y < H - 1 && x > 0) ? lum(x - 1, y + 1) : M;
        float SE = (y < H - 1 && x < W - 1) ? lum(x + 1, y + 1) : M;
        float eh = std::abs((NW + Wl + SW) - (NE + E + SE)) * (1.0f / 3.0f);
        float ev = std::abs((NW + N + NE) - (SW + S + SE)) * (1.0f / 3.0f);
        bool horiz = eh >= ev;
        float step = horiz ? 1.0f / float(W) : 1.0f / float(H);
        float g = std::clamp((horiz ? eh : ev) / range, -2.0f, 2.0f);
        vec2 uv(float(x) / float(W), float(y) / float(H));
        vec3 best_c = c;
        float best = 0.0f;
        for (int i = 0; i < 12; ++i) {
          float off = g * step * float(i + 1);
          vec2 su = uv + vec2(horiz ? 0.0f : off, horiz ? off : 0.0f);
          if (su.x < 0.0f || su.x > 1.0f || su.y < 0.0f || su.y > 1.0f) continue;
          int sx = std::clamp(int(su.x * float(W)), 0, W - 1), sy = std::clamp(int(su.y * float(H)), 0, H - 1);
          vec3 sc = px(sx, sy);
          float dl = std::abs(dot(sc, kLum) - M);
          if (dl > best) { best = dl; best_c = sc; }
        }
        float sub = std::min((std::abs(N + S - 2.0f * M) * 2.0f + std::abs(E + Wl - 2.0f * M)) * 0.25f, 1.0f);
        o = glm::mix(c, best_c, sub * 0.75f);
      }
      float* q = out + 3 * ((size_t)y * W + x);
      q[0] = o.x; q[1] = o.y; q[2] = o.z;
    }
}

// ------------------------------------------------------ photo passes -----
// Photo's post passes (src/image.cpp:30-356, 454-479) on the records of a
// render: radiance buffers with their Var, the G-buffer, and the pixel array.
struct PhotoBuf {
  int w = 0, h = 0;
  float exposure = 1.0f, focus = 1.0f, coc = 0.0f;
  vec3 cam = vec3(0.0f);
  std::vector<Surf> g;
  std::vector<Rad> buf[4];  // Dd, Ds, Id, Is
  std::vector<vec3> px;
};

// clamp(RadianceData*, ...), src/image.cpp:30-75: luminance blurred by a
// separable 7-tap kernel (taps outside the image dropped); a pixel brighter
// than 36x its neighbourhood (its own tap removed) is scaled down to it.
static void spatial_clamp_buf(std::vector<Rad>& r, int W, int H) {
  const float h[7] = {0.03125f, 0.109375f, 0.21875f, 0.28125f, 0.21875f, 0.109375f, 0.03125f};
  const size_t n = (size_t)W * H;
  std::vector<float> lum(n), b1(n), b2(n);
  for (size_t i = 0; i < n; ++i) lum[i] = dot(r[i].r, kLum);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float sum = 0.0f;
      for (int dx = -3; dx <= 3; ++dx) {
        int nx = x + dx;
        if (nx >= 0 && nx < W) sum += lum[(size_t)y * W + nx] * h[dx + 3];
      }
      b1[(size_t)y * W + x] = sum;
    }
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float sum = 0.0f;
      for (int dy = -3; dy <= 3; ++dy) {
        int ny = y + dy;
        if (ny >= 0 && ny < H) sum += b1[(size_t)ny * W + x] * h[dy + 3];
      }
      b2[(size_t)y * W + x] = sum;
    }
  for (size_t i = 0; i < n; ++i) {
    float l = lum[i];
    float bl = b2[i] - h[3] * h[3] * l;
    if (l > 36.0f * bl) r[i].r *= bl / (l + kEps) / (1.0f - h[3] * h[3]);
  }
}

// filterVar, src/image.cpp:84-108: Var of a 3x3 binomial neighbourhood.
static void filter_var(std::vector<Rad>& r, int W, int H) {
  const float h[3] = {0.25f, 0.5f, 0.25f};
  std::vector<float> v((size_t)W * H);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      vec3 E(0.0f);
      float E2 = 0.0f, V = 0.0f;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          int nx = x + dx, ny = y + dy;
          if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
          const Rad& q = r[(size_t)ny * W + nx];
          float wt = h[dx + 1] * h[dy + 1];
          E += q.r * wt;
          E2 += dot(q.r, q.r) * wt;
          V += q.var * wt;
        }
      v[(size_t)y * W + x] = V + E2 - dot(E, E);
    }
  for (size_t i = 0; i < v.size(); ++i) r[i].var = v[i];
}

// getWeight, src/image.cpp:110-158: edge-stopping weight of tap q for p.
static float edge_weight(const Surf& P, const Surf& Q, const Rad& Lp, const Rad& Lq, bool specular) {
  if (!any_finite(Q.pos)) return 0.0f;
  float w = std::pow(std::max(0.0f, dot(P.surfN, Q.surfN)), 1024.0f);
  if (w < 1e-6f) return 0.0f;
  float k = 0.0f;
  vec3 dir = normalize(Q.pos - P.pos);
  float st = std::abs(dot(P.shapeN, dir));
  float tt = st / (std::sqrt(1.0f - st * st) + kEps);
  k += -tt / 1.0f;
  float rd = length(Lp.r - Lq.r) / (1.0f * std::sqrt(Lp.var) + 1e-2f);
  k += -rd;
  float md = length(vec3(P.metallic - Q.metallic, P.specular - Q.specular, P.opacity - Q.opacity));
  k += -md / 1.0f;
  if (k < -7.5f) return 0.0f;
  w *= std::exp(k);
  if (specular) w *= std::max(P.roughness, 4e-2f);
  if (!std::isfinite(w)) return 0.0f;
  return w;
}

// filterRadiance(..., step), src/image.cpp:160-199: one a-trous pass.
static void filter_pass(std::vector<Rad>& r, const std::vector<Surf>& G, int W, int H, bool specular, int step) {
  const float h[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  const size_t n = (size_t)W * H;
  std::vector<vec3> rb(n, vec3(0.0f));
  std::vector<float> vb(n, 0.0f);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = (size_t)y * W + x;
      float ws = 0.0f;
      const Rad& Lp = r[i];
      const Surf& P = G[i];
      if (!any_finite(P.pos)) continue;
      for (int dy = -2; dy <= 2; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
          int nx = x + dx * step, ny = y + dy * step;
          if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
          float wt = h[dx + 2] * h[dy + 2];
          const size_t j = (size_t)ny * W + nx;
          if (dx != 0 || dy != 0) wt *= edge_weight(P, G[j], Lp, r[j], specular);
          ws += wt;
          rb[i] += r[j].r * wt;
          vb[i] += r[j].var * wt * wt;
        }
      rb[i] /= ws;
      vb[i] /= ws * ws;
    }
  for (size_t i = 0; i < n; ++i) {
    r[i].r = rb[i];
    r[i].var = vb[i];
  }
}

// Photo::filter, src/image.cpp:201-213: filterVar, then passes of step 1, 2,
// 4, 8, 16; the specular buffers weight by roughness.
static void filter_photo(PhotoBuf& ph) {
  for (int b = 0; b < 4; ++b) {
    const bool spec = (b & 1) != 0;
    filter_var(ph.buf[b], ph.w, ph.h);
    for (int step = 1; step <= 16; step *= 2) filter_pass(ph.buf[b], ph.g, ph.w, ph.h, spec, step);
  }
}

// Photo::shade, src/image.cpp:215-246.
static void shade_photo(PhotoBuf& ph, int opt) {
  for (size_t i = 0; i < ph.px.size(); ++i) {
    const Surf& G = ph.g[i];
    if (opt & 64) { ph.px[i] = (G.shapeN + vec3(1.0f)) / 2.0f; continue; }
    if (opt & 128) { ph.px[i] = (G.surfN + vec3(1.0f)) / 2.0f; continue; }
    vec3 rd(0.0f), rs(0.0f);
    if (opt & 4) {
      if (opt & 16) rd += ph.buf[0][i].r;
      if (opt & 32) rs += ph.buf[1][i].r;
    }
    if (opt & 8) {
      if (opt & 16) rd += ph.buf[2][i].r;
      if (opt & 32) rs += ph.buf[3][i].r;
    }
    if (!(opt & (4 | 8))) rd = vec3(1.0f);
    vec3 dc = (opt & 1) ? G.base : vec3(1.0f);
    ph.px[i] = dc * rd + rs;
    if (opt & 2) ph.px[i] += G.emis * ph.exposure;
  }
}

// Photo::bloom, src/image.cpp:248-280: the part above luminance 1 (scaled
// by lum^-0.65, minus 1 per channel) blurred by five a-trous passes, each
// pass's result added at 1/6.
static void bloom_photo(PhotoBuf& ph) {
  const float h[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  const int W = ph.w, H = ph.h;
  std::vector<vec3> bc((size_t)W * H, vec3(0.0f));
  for (size_t i = 0; i < bc.size(); ++i) {
    float c = dot(ph.px[i], kLum);
    if (c < 1.0f) continue;
    bc[i] = ph.px[i] / std::pow(c, 0.65f);
    for (int k = 0; k < 3; ++k) bc[i][k] = std::max(bc[i][k] - 1.0f, 0.0f);
  }
  for (int step = 1; step <= 16; step *= 2) {
    std::vector<vec3> t = bc;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        vec3& col = bc[(size_t)y * W + x];
        col = vec3(0.0f);
        for (int ky = -2; ky <= 2; ++ky)
          for (int kx = -2; kx <= 2; ++kx) {
            int nx = x + kx * step, ny = y + ky * step;
            if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
            col += t[(size_t)ny * W + nx] * h[ky + 2] * h[kx + 2];
          }
      }
    for (size_t i = 0; i < bc.size(); ++i) ph.px[i] += bc[i] / 6.0f;
  }
}

// float -> int of the depth-of-field radii: truncation, 0 for NaN (what
// aarch64 and CUDA give; the conversion is undefined in C++ and x86 gives
// INT_MIN, on which the reference's loops run for 2^31 steps).
static int dof_int(float v) {
  if (v != v) return 0;
  if (v >= 2147483647.0f) return 2147483647;
  if (v <= -2147483648.0f) return (-2147483647 - 1);
  return (int)v;
}

// Photo::depthFeildBlur, src/image.cpp:282-356: pixels in stable depth
// order scatter their colour over a disc of radius CoC0 (weights normalised
// per pixel); a receiving pixel stops taking weight at 0.99.
static void dof_photo(PhotoBuf& ph) {
  struct PixelPos { int x, y; float depth; };
  const int W = ph.w, H = ph.h;
  std::vector<PixelPos> pix;
  pix.reserve((size_t)W * H);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) pix.push_back({x, y, length(ph.g[(size_t)y * W + x].pos - ph.cam)});
  std::stable_sort(pix.begin(), pix.end(), [](const PixelPos& a, const PixelPos& b) { return a.depth < b.depth; });
  std::vector<vec3> blur((size_t)W * H, vec3(0.0f));
  std::vector<float> gained((size_t)W * H, 0.0f);
  for (const PixelPos& p : pix) {
    const float coc0 = std::min(ph.coc * std::abs(1.0f - ph.focus / p.depth) + kEps, 96.0f);
    const int radius = dof_int(coc0);
    const vec3 color = ph.px[(size_t)p.y * W + p.x];
    float tw = 0.0f;
    for (int dy = -radius; dy <= radius; ++dy) {
      int xl, xr;
      const int xlen = dof_int(std::sqrt(coc0 * coc0 - dy * dy));
      for (xl = -xlen; xl <= 0; xl++) {
        float wt = std::min(coc0 - std::sqrt(float(xl * xl + dy * dy)), 1.0f);
        if (wt == 1.0f) break;
        tw += wt;
      }
      for (xr = xlen; xr > 0; xr--) {
        float wt = std::min(coc0 - std::sqrt(float(xr * xr + dy * dy)), 1.0f);
        if (wt == 1.0f) break;
        tw += wt;
      }
      tw += xr - xl + 1;
    }
    for (int dy = -radius; dy <= radius; ++dy) {
      const int xlen = dof_int(std::sqrt(coc0 * coc0 - dy * dy));
      for (int dx = -xlen; dx <= xlen; ++dx) {
        int nx = p.x + dx, ny = p.y + dy;
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        float wt = std::min(coc0 - std::sqrt(float(dx * dx + dy * dy)), 1.0f) / tw;
        if (wt < kEps) continue;
        const size_t id = (size_t)ny * W + nx;
        if (gained[id] + wt > 0.99f) wt = 0.99f - gained[id];
        if (wt < kEps) continue;
        blur[id] += color * wt;
        gained[id] += wt;
      }
    }
  }
  for (size_t i = 0; i < blur.size(); ++i) ph.px[i] = blur[i] / gained[i];
}

template <class F>
static void parallel_for(long n, int threads, F&& f, long chunk = 64) {
  if (threads <= 1 || n <= chunk) { for (long i = 0; i < n; ++i) f(i); return; }
  std::atomic<long> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&] {
      for (;;) {
        long i0 = next.fetch_add(chunk);
        if (i0 >= n) break;
        long i1 = std::min(n, i0 + chunk);
        for (long i = i0; i < i1; ++i) f(i);
      }
    });
  for (auto& t : pool) t.join();
}

}  // namespace orc

using namespace orc;

extern "C" {

// Model construction for the configs: Model::processMesh / checkLightObject /
// SkyBox::Init / BVH::build (src/model.cpp:44-123,172-215,
// src/component.cpp:54-67, src/bvh.cpp:48-54) on arrays instead of assimp.
void* port_scene_create(const orc_scene_in* in) {
  Scene* s = new Scene();
  s->nrm.resize(in->num_vertices);
  s->uv.resize(in->num_vertices);
  for (int i = 0; i < in->num_vertices; ++i) {
    s->nrm[i] = in->normals ? vec3(in->normals[3 * i], in->normals[3 * i + 1], in->normals[3 * i + 2]) : vec3(0.0f);
    s->uv[i] = in->uvs ? vec2(in->uvs[2 * i], in->uvs[2 * i + 1]) : vec2(0.0f);
  }
  s->images.resize(in->num_textures > 0 ? in->num_textures : 0);
  for (int i = 0; i < in->num_textures; ++i) {
    Image& im = s->images[i];
    im.w = in->tex_dims[3 * i];
    im.h = in->tex_dims[3 * i + 1];
    im.ch = in->tex_dims[3 * i + 2];
    im.lv[0].assign(in->tex_data[i], in->tex_data[i] + (size_t)im.w * im.h * im.ch);
    im.mips();
  }
  for (int m = 0; m < in->num_materials; ++m) {
    const float* p = in->materials + ORC_MAT_FLOATS * m;
    Mat q;
    for (int k = 0; k < 4; ++k) {
      int t = in->mat_tex ? in->mat_tex[4 * m + k] : -1;
      q.tex[k] = t >= 0 ? &s->images[t] : nullptr;
    }
    q.transparent = q.tex[0] && q.tex[0]->has_transparent_part();
    q.base = vec3(p[0], p[1], p[2]); q.has_base = p[3] != 0.0f;
    q.emis = vec3(p[4], p[5], p[6]); q.has_emis = p[7] != 0.0f;
    q.roughness = p[8]; q.metallic = p[9]; q.has_surf = p[10] != 0.0f;
    q.opacity = p[11]; q.ior = p[12]; q.trans = vec3(p[13], p[14], p[15]);
    q.id = m;
    s->mats.push_back(q);
  }
  s->tris.reserve(in->num_triangles);
  for (int mesh = 0; mesh < in->num_meshes; ++mesh) {
    int first = in->mesh_first[mesh], last = in->mesh_first[mesh + 1], mat = in->mesh_material[mesh];
    size_t off = s->tris.size();
    for (int t = first; t < last; ++t) {
      Tri f;
      for (int k = 0; k < 3; ++k) {
        int v = in->indices[3 * t + k];
        f.vid[k] = v;
        f.v[k] = vec3(in->positions[3 * v], in->positions[3 * v + 1], in->positions[3 * v + 2]);
      }
      f.mat = mat;
      f.id = t;
      s->tris.push_back(f);
    }
    const Mat& M = s->mats[mat];
    if (!M.emissive()) continue;
    // checkLightObject, src/model.cpp:44-82, with getAverageEmissiveColor
    // (:23-42): the emission averaged over an 8x8 grid of barycentric points.
    Light lo;
    vec3 col(0.0f);
    std::vector<float> fw;
    for (size_t j = off; j < s->tris.size(); ++j) {
      const Tri& f = s->tris[j];
      vec3 avg(0.0f);
      for (int gi = 0; gi < 8; ++gi)
        for (int gj = 0; gj < 8; ++gj) {
          float ga = static_cast<float>(gi) / 7.0f, gb = static_cast<float>(gj) / 7.0f;
          if (ga + gb > 1.0f) { ga = 1.0f - ga; gb = 1.0f - gb; }
          float gc = 1.0f - ga - gb;
          vec2 uv = ga * s->uv[f.vid[0]] + gb * s->uv[f.vid[1]] + gc * s->uv[f.vid[2]];
          avg += M.emission(uv[0], uv[1], NAN);
        }
      avg = avg / static_cast<float>(64);
      float cl = dot(avg, kLum), area = length(cross(f.v[1] - f.v[0], f.v[2] - f.v[0])) / 2.0f;
      if (cl < kEps || area < kEps) continue;
      col += avg * area;
      lo.faces.push_back(f);
      fw.push_back(area * cl);
    }
    if (lo.faces.empty()) continue;
    lo.color = col / dot(col, kLum);
    for (size_t j = 0; j < lo.faces.size(); ++j) {
      lo.power += fw[j];
      lo.center += tri_center(lo.faces[j]) * fw[j];
    }
    prefix_init(lo.prefix, fw);
    lo.center /= lo.power;
    s->lights.push_back(lo);
  }
  if (in->env_rgb && in->env_width > 0 && in->env_height > 0) {
    Sky& k = s->sky;
    k.w = in->env_width; k.h = in->env_height;
    k.data.resize((size_t)k.w * k.h);
    std::vector<float> wts;
    wts.reserve(k.data.size());
    for (int v = 0; v < k.h; ++v)
      for (int u = 0; u < k.w; ++u) {
        size_t i = (size_t)v * k.w + u;
        k.data[i] = vec3(in->env_rgb[3 * i], in->env_rgb[3 * i + 1], in->env_rgb[3 * i + 2]);
        float phi = kPi * (float(v) + 0.5f) / float(k.h);
        float area = std::sin(phi) * 2.0f * kPi / float(k.w * k.h);
        k.data[i] *= area;
        wts.push_back(dot(k.data[i], kLum));
      }
    prefix_init(k.prefix, wts);
  }
  int n = (int)s->tris.size();
  s->nodes.assign(heap_slots(1, n) + 1, Node());
  if (n > 0) build_rec(*s, 1, 0, n);
  return s;
}

void port_scene_destroy(void* h) { delete static_cast<Scene*>(h); }

int port_bvh_size(void* h) { return (int)static_cast<Scene*>(h)->nodes.size(); }

void port_bvh_export(void* h, float* boxes, int32_t* ranges, int32_t* order) {
  const Scene& s = *static_cast<Scene*>(h);
  for (size_t u = 0; u < s.nodes.size(); ++u) {
    const Node& n = s.nodes[u];
    float b[6] = {n.box.lo.x, n.box.lo.y, n.box.lo.z, n.box.hi.x, n.box.hi.y, n.box.hi.z};
    std::memcpy(boxes + 6 * u, b, sizeof b);
    ranges[2 * u] = n.faceL;
    ranges[2 * u + 1] = n.faceR;
  }
  for (size_t i = 0; i < s.tris.size(); ++i) order[i] = s.tris[i].id;
}

// Light objects: per light 8 floats (center, color, power, face count).
int port_light_count(void* h) { return (int)static_cast<Scene*>(h)->lights.size(); }
void port_light_export(void* h, float* out) {
  const Scene& s = *static_cast<Scene*>(h);
  for (size_t i = 0; i < s.lights.size(); ++i) {
    const Light& l = s.lights[i];
    float r[8] = {l.center.x, l.center.y, l.center.z, l.color.x, l.color.y, l.color.z, l.power, (float)l.faces.size()};
    std::memcpy(out + 8 * i, r, sizeof r);
  }
}

// rays: 8 floats each (origin, t_min, direction, t_max). Model::rayHit always
// uses t_min = 1e-4, t_max = inf; other bounds go straight to the BVH query.
// Output: input triangle index (-1 on a miss), t, barycentrics (gamma, alpha, beta).
void port_trace_closest(void* h, const float* rays, int64_t n, int32_t* face, float* t, float* bc, int threads) {
  const Scene& s = *static_cast<Scene*>(h);
  parallel_for(n, threads, [&](long i) {
    const float* r = rays + 8 * i;
    Ray ray{vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6])};
    Hit hh{r[3], r[7], -1};
    if (r[3] == kEps && std::isinf(r[7]) && r[7] > 0) hh = closest(s, ray);  // Model::rayHit, alpha test included
    else traverse(s, ray, hh, nullptr);
    if (hh.face < 0) {
      face[i] = -1; t[i] = hh.tmax; bc[3 * i] = bc[3 * i + 1] = bc[3 * i + 2] = 0.0f;
      return;
    }
    const Tri& f = s.tris[hh.face];
    face[i] = f.id;
    t[i] = hh.tmax;
    vec3 b = bary(f.v[0], f.v[1], f.v[2], ray.o + ray.d * hh.tmax);
    bc[3 * i] = b.x; bc[3 * i + 1] = b.y; bc[3 * i + 2] = b.z;
  });
}

// rays: 8 floats each (origin, unused, direction, aim depth) -> occluded.
void port_trace_shadow(void* h, const float* rays, int64_t n, uint8_t* occ, int threads) {
  const Scene& s = *static_cast<Scene*>(h);
  parallel_for(n, threads, [&](long i) {
    const float* r = rays + 8 * i;
    occ[i] = occluded(s, {vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6])}, r[7]) ? 1 : 0;
  });
}

// Node and triangle visit counts of the closest-hit (mode 0) or shadow
// (mode 1) queries of a ray batch: out = {inner nodes, leaves, triangles}.
void port_trace_stats(void* h, const float* rays, int64_t n, int mode, uint64_t* out) {
  const Scene& s = *static_cast<Scene*>(h);
  Stats st;
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 8 * i;
    Ray ray{vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6])};
    if (mode == 0) { Hit hh{r[3], r[7], -1}; traverse(s, ray, hh, &st); }
    else occluded(s, ray, r[7], &st);
  }
  out[0] = st.inner; out[1] = st.leaves; out[2] = st.tris;
}

static Args unpack_args(const float* p) {
  Args a;
  a.pos = vec3(p[0], p[1], p[2]); a.dir = vec3(p[3], p[4], p[5]); a.up = vec3(p[6], p[7], p[8]);
  a.right = vec3(p[9], p[10], p[11]);
  a.accuracy = p[12]; a.focus = p[13]; a.coc = p[14]; a.exposure = p[15]; a.p_direct = p[16];
  a.w = (int)p[17]; a.h = (int)p[18]; a.spp = (int)p[19]; a.threads = (int)p[20]; a.maxd = (int)p[21];
  if (a.maxd <= 0 || a.maxd > 16) a.maxd = 16;
  return a;
}

// Renders the pixel rectangle [x0,x1) x [y0,y1) of the image described by
// args; out holds ORC_PIX_FLOATS per pixel of the rectangle, row-major.
void port_render(void* h, const float* args, uint64_t seed, int mode, int x0, int y0, int x1, int y1, float* out,
                 int threads) {
  const Scene& s = *static_cast<Scene*>(h);
  Args a = unpack_args(args);
  int rw = x1 - x0;
  long n = (long)rw * (y1 - y0);
  parallel_for(n, threads, [&](long i) {
    int x = x0 + (int)(i % rw), y = y0 + (int)(i / rw);
    render_pixel(s, a, seed, mode, x, y, out + ORC_PIX_FLOATS * i);
  }, 1);
}

// Renders the listed pixels (row-major indices y * width + x) of the image
// described by args; out holds ORC_PIX_FLOATS per listed pixel.
void port_render_pixels(void* h, const float* args, uint64_t seed, int mode, const int32_t* pixels, int64_t n,
                        float* out, int threads) {
  const Scene& s = *static_cast<Scene*>(h);
  Args a = unpack_args(args);
  parallel_for((long)n, threads, [&](long i) {
    render_pixel(s, a, seed, mode, pixels[i] % a.w, pixels[i] / a.w, out + ORC_PIX_FLOATS * i);
  }, 1);
}

// Photo::shade(Full) [+ gammaCorrection] over pixel records -> rgb.
void port_compose(const float* recs, int64_t n, float exposure, int apply_gamma, float* rgb) {
  for (int64_t i = 0; i < n; ++i) {
    vec3 p = compose(recs + ORC_PIX_FLOATS * i, exposure);
    if (apply_gamma) p = gamma(p);
    rgb[3 * i] = p.x; rgb[3 * i + 1] = p.y; rgb[3 * i + 2] = p.z;
  }
}

void port_gamma(const float* in, int64_t n, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    vec3 p = gamma(vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
    out[3 * i] = p.x; out[3 * i + 1] = p.y; out[3 * i + 2] = p.z;
  }
}

void port_fxaa(const float* in, float* out, int w, int h) { fxaa(in, out, w, h); }

void port_photo(float* recs, int w, int h, int stages, int options, const float* post, float* rgb) {
  PhotoBuf ph;
  ph.w = w;
  ph.h = h;
  ph.exposure = post[0];
  ph.focus = post[1];
  ph.coc = post[2];
  ph.cam = vec3(post[3], post[4], post[5]);
  const size_t n = (size_t)w * h;
  ph.g.resize(n);
  ph.px.assign(n, vec3(0.0f));
  for (int b = 0; b < 4; ++b) ph.buf[b].resize(n);
  for (size_t i = 0; i < n; ++i) {
    const float* r = recs + ORC_PIX_FLOATS * i;
    for (int b = 0; b < 4; ++b) {
      ph.buf[b][i].r = vec3(r[4 * b], r[4 * b + 1], r[4 * b + 2]);
      ph.buf[b][i].var = r[4 * b + 3];
    }
    Surf& G = ph.g[i];
    G.base = vec3(r[16], r[17], r[18]);
    G.emis = vec3(r[19], r[20], r[21]);
    G.pos = vec3(r[22], r[23], r[24]);
    G.shapeN = vec3(r[25], r[26], r[27]);
    G.surfN = vec3(r[28], r[29], r[30]);
    G.roughness = r[31]; G.metallic = r[32]; G.opacity = r[33]; G.specular = r[34]; G.eta = r[35];
    G.id = (int)r[36]; G.entering = r[37] != 0.0f;
  }
  if (stages & 1)
    for (int b = 0; b < 4; ++b) spatial_clamp_buf(ph.buf[b], w, h);
  if (stages & 2) filter_photo(ph);
  if (stages & (4 | 8)) {  // Photo::postProcessing, src/image.cpp:470-479 (8: without gamma and FXAA)
    shade_photo(ph, options);
    if (options & 1024) dof_photo(ph);
    if (options & 256) bloom_photo(ph);
    if (stages & 4) {
      for (vec3& p : ph.px) p = gamma(p);
      if (options & 512) {
        std::vector<float> a(3 * n), o(3 * n);
        for (size_t i = 0; i < n; ++i) { a[3 * i] = ph.px[i].x; a[3 * i + 1] = ph.px[i].y; a[3 * i + 2] = ph.px[i].z; }
        fxaa(a.data(), o.data(), w, h);
        for (size_t i = 0; i < n; ++i) ph.px[i] = vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
      }
    }
    for (size_t i = 0; i < n; ++i) { rgb[3 * i] = ph.px[i].x; rgb[3 * i + 1] = ph.px[i].y; rgb[3 * i + 2] = ph.px[i].z; }
  }
  for (size_t i = 0; i < n; ++i) {
    float* r = recs + ORC_PIX_FLOATS * i;
    for (int b = 0; b < 4; ++b) {
      r[4 * b] = ph.buf[b][i].r.x; r[4 * b + 1] = ph.buf[b][i].r.y; r[4 * b + 2] = ph.buf[b][i].r.z;
      r[4 * b + 3] = ph.buf[b][i].var;
    }
  }
}

}  // extern "C"
