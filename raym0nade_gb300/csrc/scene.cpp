// Scene construction on the host and upload to HBM (rmn_scene_create).
//
// The BVH is the reference's own tree: BVH::dfs_build (src/bvh.cpp:18-42)
// splits at the median of the centroid coordinate of largest variance with
// std::nth_element and stops at <= 10 triangles. Running the same comparator
// through std::nth_element on an array of (centroid, index) items performs
// the same comparisons and swaps as the reference does on its Face array,
// so the tree, the leaf order and therefore every closest-hit id are the
// reference's. Disjoint subtrees are built on separate threads, which changes
// nothing in the result.
//
// The heap-indexed tree is then flattened depth-first into 64-byte two-child
// nodes (DevNode), and triangles are stored in leaf order with their edges
// precomputed (e1 = v1 - v0, e2 = v2 - v0 are exactly the differences that
// RayTriangleIntersection forms, src/geometry.cpp:65-66).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <vector>
#include <memory>
#include <utility>
#include <mutex>
#include <thread>

#include "rmn_host.h"
#include "texture.h"

namespace rmn {
namespace {

// fn(lo, hi) over [0, n) in contiguous ranges, one per hardware thread (16
// at most) once n is large; each index belongs to one range, so loops whose
// iterations write only their own slots give the same arrays on any number
// of threads. A worker's exception is rethrown here, after every worker has
// finished.
template <class F>
void parallel_ranges(size_t n, F fn) {
  const size_t parts = std::min(host_threads(), std::max<size_t>(1, n / 16384));
  run_threads(parts, [&](size_t k) { fn(n * k / parts, n * (k + 1) / parts); });
}

// An allocator whose default-inserted elements are left uninitialised
// (default- instead of value-initialised), for the large per-vertex and
// per-triangle arrays that a parallel loop then fills slot by slot: their
// pages are first touched by the threads that write them, not zeroed by one
// thread beforehand.
template <class T>
struct NoInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInit<U>;
  };
  NoInit() = default;
  template <class U>
  NoInit(const NoInit<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
template <class T>
using FillVec = std::vector<T, NoInit<T>>;

struct Item {
  float c[3];
  int32_t id;
};

struct HeapNode {
  float3 lo, hi;
  int32_t faceL = 0, faceR = 0;
};

struct Builder {
  const float3* pos;
  const int32_t* idx;
  FillVec<Item> items;
  std::vector<HeapNode> heap;

  float3 vtx(int tri, int k) const { return pos[idx[3 * tri + k]]; }

  void leaf(int u, int l, int r) {
    HeapNode& n = heap[u];
    n.faceL = l;
    n.faceR = r;
    n.lo = f3(INFINITY);
    n.hi = f3(-INFINITY);
    for (int i = l; i < r; ++i) {
      int t = items[i].id;
      float3 a = vtx(t, 0), b = vtx(t, 1), c = vtx(t, 2);
      float3 lo = min3(a, min3(b, c)), hi = max3(a, max3(b, c));
      n.lo = f3(std::fmin(n.lo.x, lo.x), std::fmin(n.lo.y, lo.y), std::fmin(n.lo.z, lo.z));
      n.hi = f3(std::fmax(n.hi.x, hi.x), std::fmax(n.hi.y, hi.y), std::fmax(n.hi.z, hi.z));
    }
  }

  void build(int u, int l, int r, int par_depth) {
    if ((unsigned)(r - l) <= (unsigned)RMN_LEAF_MAX) {
      leaf(u, l, r);
      return;
    }
    float3 s = f3(0.0f), s2 = f3(0.0f);
    for (int i = l; i < r; ++i) {
      float3 c = f3(items[i].c[0], items[i].c[1], items[i].c[2]);
      s += c;
      s2 += c * c;
    }
    float3 var = s2 - s * s / (float)(r - l);
    int axis = 0;
    if (var.y > var.x) axis = 1;
    if (var.z > var.x && var.z > var.y) axis = 2;
    int m = (r + l) / 2;
    std::nth_element(items.begin() + l, items.begin() + m, items.begin() + r,
                     [axis](const Item& a, const Item& b) { return a.c[axis] < b.c[axis]; });
    if (par_depth > 0 && r - l > 65536) {
      auto left = std::async(std::launch::async, [&] { build(u << 1, l, m, par_depth - 1); });
      build(u << 1 | 1, m, r, par_depth - 1);
      left.get();
    } else {
      build(u << 1, l, m, 0);
      build(u << 1 | 1, m, r, 0);
    }
    const HeapNode &a = heap[u << 1], &b = heap[u << 1 | 1];
    heap[u].lo = f3(std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y), std::fmin(a.lo.z, b.lo.z));
    heap[u].hi = f3(std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y), std::fmax(a.hi.z, b.hi.z));
  }
};

int heap_slots(int u, int n) { return ((unsigned)n <= (unsigned)RMN_LEAF_MAX) ? u : heap_slots(u << 1 | 1, (n + 1) >> 1); }

struct Flattener {
  const std::vector<HeapNode>& heap;
  std::vector<DevNode> out;
  int max_depth = 0;

  int ref_of(int u, int depth) {
    const HeapNode& n = heap[u];
    if (n.faceR) {
      max_depth = std::max(max_depth, depth);
      return leaf_ref(n.faceL, n.faceR - n.faceL);
    }
    int me = (int)out.size();
    out.emplace_back();
    int l = ref_of(u << 1, depth + 1);
    int r = ref_of(u << 1 | 1, depth + 1);
    const HeapNode &L = heap[u << 1], &R = heap[u << 1 | 1];
    DevNode& d = out[me];
    d.a = make_float4(L.lo.x, L.lo.y, L.lo.z, L.hi.x);
    d.b = make_float4(L.hi.y, L.hi.z, R.lo.x, R.lo.y);
    d.c = make_float4(R.lo.z, R.hi.x, R.hi.y, R.hi.z);
    d.d = make_int4(l, r, 0, 0);
    return me;
  }
};

float bits_float(int32_t i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}
int32_t float_bits(float f) {
  int32_t i;
  std::memcpy(&i, &f, 4);
  return i;
}

// The tangent frame of calcSurfaceNormal (src/model.cpp:279-298). With the
// zero normal-map texel of an untextured material its only effect is to
// renormalise the surface normal, and only when this frame is finite; the
// frame does not depend on which side the shape normal was flipped to.
bool tangent_frame_finite(float3 e1, float3 e2, const float* uv0, const float* uv1, const float* uv2) {
  float d1x = uv1[0] - uv0[0], d1y = uv1[1] - uv0[1];
  float d2x = uv2[0] - uv0[0], d2y = uv2[1] - uv0[1];
  float k = 1.0f / (d1x * d2y - d2x * d1y);
  float3 tu = k * (d2y * e1 - d1y * e2), tv = k * (-d2x * e1 + d1x * e2);
  float3 sn = norm3(cross3(e1, e2));
  float3 t = norm3(tu - sn * dot3(sn, tu));
  float3 b = norm3(tv - sn * dot3(sn, tv) - t * dot3(t, tv));
  return all_finite3(t) && all_finite3(b);
}

template <class T, class A>
rmn_status upload(rmn_scene* s, const std::vector<T, A>& v, const T** out) {
  *out = nullptr;
  if (v.empty()) return RMN_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, v.size() * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (scene)");
  s->device_allocations.push_back(p);
  e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (scene)");
  s->info.device_bytes += (int64_t)(v.size() * sizeof(T));
  *out = static_cast<const T*>(p);
  return RMN_OK;
}

// Sky tables shared between scenes. A batch typically lights many scenes
// with one environment; one copy of its texels, prefix sums and guide table
// then stays in L2 instead of one per scene. Entries are keyed by device
// and compared byte for byte; the last scene using an entry frees it.
struct SkyShare {
  int device = 0, w = 0, h = 0;
  uint64_t hash = 0;
  std::vector<float4> texels;  // host copy for the comparison
  void* dev[4] = {};           // texels, prefix, guide thresholds, guide indices
  int gk = 0;
  float ginv = 0.0f;
  int refs = 0;
  int64_t bytes = 0;
};
std::mutex g_sky_mu;
std::vector<SkyShare*> g_skies;

uint64_t hash_bytes(const void* p, size_t n) {  // FNV-1a, 64 bit
  const unsigned char* b = static_cast<const unsigned char*>(p);
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ULL;
  return h;
}

// Guide table for lower_bound over a prefix-sum array p (non-decreasing):
// K + 1 thresholds t_k = total * k / K and gi[k] = lower_bound(p, t_k).
void build_guide(const std::vector<float>& p, std::vector<float>& gt, std::vector<int>& gi, int& K, float& inv) {
  const int n = (int)p.size();
  K = std::max(1, n / 8);
  const float total = p[n - 1];
  gt.resize(K + 1);
  gi.resize(K + 1);
  for (int k = 0; k <= K; ++k) {
    gt[k] = (float)((double)total * k / K);
    gi[k] = (int)(std::lower_bound(p.begin(), p.end(), gt[k]) - p.begin());
    if (gi[k] > n - 1) gi[k] = n - 1;
  }
  inv = total > 0.0f ? (float)K / total : 0.0f;
}

rmn_status acquire_sky(rmn_scene* s, int W, int H, const std::vector<float4>& sky, const std::vector<float>& prefix) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t h = hash_bytes(sky.data(), sky.size() * sizeof(float4));
  std::lock_guard<std::mutex> lock(g_sky_mu);
  SkyShare* e = nullptr;
  for (SkyShare* c : g_skies)
    if (c->device == dev && c->w == W && c->h == H && c->hash == h &&
        std::memcmp(c->texels.data(), sky.data(), sky.size() * sizeof(float4)) == 0)
      e = c;
  if (!e) {
    std::unique_ptr<SkyShare> n(new SkyShare());
    n->device = dev;
    n->w = W;
    n->h = H;
    n->hash = h;
    n->texels = sky;
    std::vector<float> gt;
    std::vector<int> gi;
    build_guide(prefix, gt, gi, n->gk, n->ginv);
    const void* src[4] = {sky.data(), prefix.data(), gt.data(), gi.data()};
    const size_t bytes[4] = {sky.size() * sizeof(float4), prefix.size() * sizeof(float), gt.size() * sizeof(float),
                             gi.size() * sizeof(int)};
    for (int k = 0; k < 4; ++k) {
      cudaError_t err = cudaMalloc(&n->dev[k], bytes[k]);
      if (err == cudaSuccess) err = cudaMemcpy(n->dev[k], src[k], bytes[k], cudaMemcpyHostToDevice);
      if (err != cudaSuccess) {
        for (int j = 0; j <= k; ++j)
          if (n->dev[j]) cudaFree(n->dev[j]);
        return cuda_fail(err, "sky upload");
      }
      n->bytes += (int64_t)bytes[k];
    }
    e = n.release();
    g_skies.push_back(e);
  }
  e->refs++;
  s->sky_share = e;
  DevScene& g = s->dev;
  g.sky = static_cast<const float4*>(e->dev[0]);
  g.sky_prefix = static_cast<const float*>(e->dev[1]);
  g.sky_gt = static_cast<const float*>(e->dev[2]);
  g.sky_gi = static_cast<const int*>(e->dev[3]);
  g.sky_gk = e->gk;
  g.sky_ginv = e->ginv;
  s->info.device_bytes += e->bytes;
  return RMN_OK;
}

// ImageData after Material::loadImageFromFile and generateMipmaps
// (src/material.cpp:107-129): level l is (w >> l) x (h >> l) texels, until a
// side would reach 0, at most 8 levels; the levels of every texture are
// packed one after the other. Level 0 is the caller's array; the device
// builds the rest (mips.cu).
DevTex texture_layout(const rmn_texture& in, long long& bytes) {
  DevTex t{};
  t.w = in.width;
  t.h = in.height;
  t.depth = RMN_MIP_LEVELS;
  for (int l = 0; l < RMN_MIP_LEVELS; ++l) {
    if (l > 0 && ((t.w >> l) == 0 || (t.h >> l) == 0)) {
      t.depth = l;
      break;
    }
    t.off[l] = bytes;
    bytes += 4LL * (t.w >> l) * (t.h >> l);
  }
  return t;
}
// ImageData::hasTransparentPart, src/material.cpp:102-107: some level-0
// alpha below 255.
bool has_transparent_part(const rmn_texture& t) {
  const size_t n = (size_t)t.width * t.height * 4;
  for (size_t i = 3; i < n; i += 4)
    if (t.texels[i] < 255) return true;
  return false;
}

void release_sky(rmn_scene* s) {
  if (!s->sky_share) return;
  std::lock_guard<std::mutex> lock(g_sky_mu);
  SkyShare* e = static_cast<SkyShare*>(s->sky_share);
  s->sky_share = nullptr;
  if (--e->refs > 0) return;
  for (void* p : e->dev)
    if (p) cudaFree(p);
  g_skies.erase(std::remove(g_skies.begin(), g_skies.end(), e), g_skies.end());
  delete e;
}

}  // namespace

rmn_status build_scene(const rmn_scene_desc* d, rmn_scene* s) {
  if (!d || !d->positions || !d->indices || !d->mesh_first || !d->mesh_material || !d->materials)
    return fail(RMN_ERR_INVALID_ARGUMENT, "scene description has a NULL array");
  if (d->num_vertices <= 0 || d->num_triangles <= 0 || d->num_meshes <= 0 || d->num_materials <= 0)
    return fail(RMN_ERR_INVALID_ARGUMENT, "scene needs at least one vertex, triangle, mesh and material");
  if (d->num_triangles >= (1 << 27))
    return fail(RMN_ERR_INVALID_ARGUMENT, "at most 2^27 - 1 triangles per scene");
  if (d->mesh_first[0] != 0 || d->mesh_first[d->num_meshes] != d->num_triangles)
    return fail(RMN_ERR_INVALID_ARGUMENT, "mesh_first must start at 0 and end at num_triangles");
  for (int m = 0; m < d->num_meshes; ++m) {
    if (d->mesh_first[m + 1] < d->mesh_first[m]) return fail(RMN_ERR_INVALID_ARGUMENT, "mesh_first must not decrease");
    if (d->mesh_material[m] < 0 || d->mesh_material[m] >= d->num_materials)
      return fail(RMN_ERR_INVALID_ARGUMENT, "mesh %d has material %d out of range", m, d->mesh_material[m]);
  }
  for (int64_t i = 0; i < 3LL * d->num_triangles; ++i)
    if (d->indices[i] < 0 || d->indices[i] >= d->num_vertices)
      return fail(RMN_ERR_INVALID_ARGUMENT, "vertex index %d of triangle %lld out of range", d->indices[i],
                  (long long)(i / 3));
  bool glass = false;
  for (int m = 0; m < d->num_materials; ++m) glass = glass || !(d->materials[m].opacity > 1.0f - RMN_EPS);
  if (d->env_rgb && (d->env_width <= 0 || d->env_height <= 0))
    return fail(RMN_ERR_INVALID_ARGUMENT, "sky map needs positive width and height");
  if (d->num_textures < 0 || (d->num_textures > 0 && !d->textures))
    return fail(RMN_ERR_INVALID_ARGUMENT, "num_textures must be >= 0, with a texture array when positive");
  for (int i = 0; i < d->num_textures; ++i) {
    const rmn_texture& t = d->textures[i];
    if (t.width <= 0 || t.height <= 0 || t.width > 32768 || t.height > 32768 || !t.texels)
      return fail(RMN_ERR_INVALID_ARGUMENT, "texture %d needs 1..32768 x 1..32768 texels", i);
    if (is_device_pointer(t.texels))
      return fail(RMN_ERR_INVALID_ARGUMENT, "texture %d: texels must be in host memory", i);
    if (t.channels != 4)
      return fail(RMN_ERR_UNSUPPORTED,
                  "texture %d has %d channels: textures are RGBA8 (the reference reads 4-byte texels)", i,
                  t.channels);
  }
  bool textured = false;
  if (d->material_textures) {
    for (int k = 0; k < 4 * d->num_materials; ++k) {
      const int t = d->material_textures[k];
      if (t < -1 || t >= d->num_textures)
        return fail(RMN_ERR_INVALID_ARGUMENT, "material %d slot %d has texture %d out of range", k / 4, k % 4, t);
      textured = textured || t >= 0;
    }
  }
  auto mat_tex = [&](int m, int slot) { return d->material_textures ? d->material_textures[4 * m + slot] : -1; };

  const int nt = d->num_triangles;
  FillVec<float3> pos(d->num_vertices);
  parallel_ranges(d->num_vertices, [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; ++i) pos[i] = f3(d->positions[3 * i], d->positions[3 * i + 1], d->positions[3 * i + 2]);
  });

  // ---- BVH (BVH::build, src/bvh.cpp:48-54) ----
  Builder b;
  b.pos = pos.data();
  b.idx = d->indices;
  b.items.resize(nt);
  parallel_ranges(nt, [&](size_t lo, size_t hi) {
    for (int t = (int)lo; t < (int)hi; ++t) {
      float3 c = (b.vtx(t, 0) + b.vtx(t, 1) + b.vtx(t, 2)) / 3.0f;  // Face::center, src/component.cpp:37-39
      b.items[t] = {{c.x, c.y, c.z}, t};
    }
  });
  b.heap.assign(heap_slots(1, nt) + 1, HeapNode());
  // subtrees on separate threads down to this depth: 2^par of them
  const unsigned hw = std::thread::hardware_concurrency();
  const int par = hw >= 16 ? 4 : hw >= 8 ? 3 : 1;
  b.build(1, 0, nt, par);
  Flattener fl{b.heap, {}, 0};
  int root = fl.ref_of(1, 0);
  if (fl.max_depth + 1 > RMN_STACK)
    return fail(RMN_ERR_UNSUPPORTED, "BVH depth %d exceeds the traversal stack", fl.max_depth);

  // ---- triangles in leaf order ----
  std::vector<int> tri_mesh_mat(nt);
  for (int m = 0; m < d->num_meshes; ++m)
    for (int t = d->mesh_first[m]; t < d->mesh_first[m + 1]; ++t) tri_mesh_mat[t] = d->mesh_material[m];
  static const float zero2[2] = {0.0f, 0.0f};
  FillVec<float4> tri(3 * (size_t)nt), shade(3 * (size_t)nt);
  parallel_ranges(nt, [&](size_t lo, size_t hi) {
    for (int i = (int)lo; i < (int)hi; ++i) {
      int t = b.items[i].id;
      int i0 = d->indices[3 * t], i1 = d->indices[3 * t + 1], i2 = d->indices[3 * t + 2];
      float3 v0 = pos[i0], e1 = pos[i1] - v0, e2 = pos[i2] - v0;
      int flags = 0;
      float area = len3(cross3(e1, e2)) / 2.0f;
      if (!(area > 1e-2f)) flags |= RMN_TRI_SMOOTH;
      const float* u0 = d->uvs ? d->uvs + 2 * i0 : zero2;
      const float* u1 = d->uvs ? d->uvs + 2 * i1 : zero2;
      const float* u2 = d->uvs ? d->uvs + 2 * i2 : zero2;
      if (tangent_frame_finite(e1, e2, u0, u1, u2)) flags |= RMN_TRI_RENORM;
      tri[3 * i + 0] = make_float4(v0.x, v0.y, v0.z, bits_float(t));
      tri[3 * i + 1] = make_float4(e1.x, e1.y, e1.z, len3(e1));
      tri[3 * i + 2] = make_float4(e2.x, e2.y, e2.z, bits_float(flags));
      for (int k = 0; k < 3; ++k) {
        int v = d->indices[3 * t + k];
        float3 n = d->normals ? f3(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]) : f3(0.0f);
        shade[3 * i + k] = make_float4(n.x, n.y, n.z, k == 0 ? bits_float(tri_mesh_mat[t]) : 0.0f);
      }
    }
  });

  // ---- textures: mip chains, packed level after level ----
  std::vector<DevTex> dtex(textured ? d->num_textures : 0);
  long long texel_bytes = 0;
  for (size_t i = 0; i < dtex.size(); ++i) dtex[i] = texture_layout(d->textures[i], texel_bytes);
  std::vector<char> alpha_mat(d->num_materials, 0);
  bool has_alpha = false;
  for (int m = 0; m < d->num_materials; ++m) {
    const int t = mat_tex(m, RMN_TEX_DIFFUSE);
    alpha_mat[m] = (textured && t >= 0 && has_transparent_part(d->textures[t])) ? 1 : 0;
    has_alpha = has_alpha || alpha_mat[m];
  }
  if (has_alpha)
    for (int i = 0; i < nt; ++i) {
      int flags = float_bits(tri[3 * i + 2].w);
      if (alpha_mat[tri_mesh_mat[b.items[i].id]]) flags |= RMN_TRI_ALPHA;
      tri[3 * i + 2].w = bits_float(flags);
    }
  std::vector<float4> uvs;
  if (textured) {
    uvs.resize(2 * (size_t)nt);
    for (int i = 0; i < nt; ++i) {
      int t = b.items[i].id;
      float w[6];
      for (int k = 0; k < 3; ++k) {
        int v = d->indices[3 * t + k];
        w[2 * k] = d->uvs ? d->uvs[2 * v] : 0.0f;
        w[2 * k + 1] = d->uvs ? d->uvs[2 * v + 1] : 0.0f;
      }
      uvs[2 * i] = make_float4(w[0], w[1], w[2], w[3]);
      uvs[2 * i + 1] = make_float4(w[4], w[5], 0.0f, 0.0f);
    }
  }
  // Material::getEmissiveColor(u, v, NaN): level 0 of the emissive texture,
  // gamma 2.2, or the constant texel.
  auto emissive_at = [&](int m, float u, float v) -> float3 {
    const int t = textured ? mat_tex(m, RMN_TEX_EMISSIVE) : -1;
    if (t >= 0) {  // level 0 only (level of detail 0): read from the caller's texels
      DevTex level0 = dtex[t];
      level0.off[0] = 0;
      return tex_gamma(tex_get<4>(level0, d->textures[t].texels, u, v, 0.0f));
    }
    const rmn_material& q = d->materials[m];
    return q.has_emission != 0.0f ? f3(q.emission[0], q.emission[1], q.emission[2]) : f3(0.0f);
  };

  // ---- materials (Material::get*, src/material.cpp:349-383) ----
  std::vector<DevMat> mats(d->num_materials);
  for (int m = 0; m < d->num_materials; ++m) {
    const rmn_material& q = d->materials[m];
    float3 base = q.has_base != 0.0f ? f3(q.base_color[0], q.base_color[1], q.base_color[2]) : f3(1.0f);
    float3 emis = q.has_emission != 0.0f ? f3(q.emission[0], q.emission[1], q.emission[2]) : f3(0.0f);
    float rough = q.roughness, metal = 0.0f;
    if (q.has_specular != 0.0f) {
      metal = std::min(q.metallic, 0.99f);
      rough = std::max(q.roughness, 1e-3f);
    }
    mats[m].base = make_float4(base.x, base.y, base.z, rough);
    mats[m].emis = make_float4(emis.x, emis.y, emis.z, metal);
    mats[m].misc = make_float4(q.opacity, q.ior, q.has_emission != 0.0f ? 1.0f : 0.0f, (float)m);
    mats[m].trans = make_float4(q.transmitting_color[0], q.transmitting_color[1], q.transmitting_color[2], 0.0f);
    mats[m].tex = make_int4(-1, -1, -1, -1);
    if (textured)
      mats[m].tex = make_int4(mat_tex(m, 0), mat_tex(m, 1), mat_tex(m, 2), mat_tex(m, 3));
  }

  // ---- light objects (Model::checkLightObject, src/model.cpp:44-82) ----
  // One per mesh with an emissive texel or texture, built before the sky is
  // loaded as in the reference (so also when a sky map is present, where
  // they stay unused by light sampling). Each face's colour is its emission
  // averaged over an 8x8 grid of barycentric points
  // (getAverageEmissiveColor, src/model.cpp:23-42).
  std::vector<DevLight> lights;
  std::vector<float4> lfaces;
  std::vector<float> lprefix;
  for (int m = 0; m < d->num_meshes; ++m) {
    const int mi = d->mesh_material[m];
    const rmn_material& q = d->materials[mi];
    if (q.has_emission == 0.0f && !(textured && mat_tex(mi, RMN_TEX_EMISSIVE) >= 0)) continue;
    float3 color = f3(0.0f), center = f3(0.0f);
    float power = 0.0f;
    std::vector<float> w;
    std::vector<int> faces;
    for (int t = d->mesh_first[m]; t < d->mesh_first[m + 1]; ++t) {
      float uv[3][2] = {};
      for (int k = 0; k < 3 && d->uvs; ++k) {
        uv[k][0] = d->uvs[2 * d->indices[3 * t + k]];
        uv[k][1] = d->uvs[2 * d->indices[3 * t + k] + 1];
      }
      float3 avg = f3(0.0f);
      for (int gi = 0; gi < 8; ++gi)
        for (int gj = 0; gj < 8; ++gj) {
          float ga = static_cast<float>(gi) / 7.0f, gb = static_cast<float>(gj) / 7.0f;
          if (ga + gb > 1.0f) {
            ga = 1.0f - ga;
            gb = 1.0f - gb;
          }
          float gc = 1.0f - ga - gb;
          float u = ga * uv[0][0] + gb * uv[1][0] + gc * uv[2][0];
          float v = ga * uv[0][1] + gb * uv[1][1] + gc * uv[2][1];
          avg += emissive_at(mi, u, v);
        }
      avg = avg / static_cast<float>(64);
      float cl = dot3(avg, f3(0.3f, 0.6f, 0.1f));
      float3 v0 = pos[d->indices[3 * t]], v1 = pos[d->indices[3 * t + 1]], v2 = pos[d->indices[3 * t + 2]];
      float area = len3(cross3(v1 - v0, v2 - v0)) / 2.0f;
      if (cl < RMN_EPS || area < RMN_EPS) continue;
      color += avg * area;
      faces.push_back(t);
      w.push_back(area * cl);
    }
    if (faces.empty()) continue;
    color = color / dot3(color, f3(0.3f, 0.6f, 0.1f));
    for (size_t j = 0; j < faces.size(); ++j) {
      int t = faces[j];
      float3 v0 = pos[d->indices[3 * t]], v1 = pos[d->indices[3 * t + 1]], v2 = pos[d->indices[3 * t + 2]];
      power += w[j];
      center += (v0 + v1 + v2) / 3.0f * w[j];
    }
    center /= power;
    DevLight L{};
    L.center = make_float4(center.x, center.y, center.z, power);
    L.color = make_float4(color.x, color.y, color.z, (float)faces.size());
    L.first_face = (int)(lfaces.size() / RMN_LIGHT_FACE_F4);
    L.material = d->mesh_material[m];
    lights.push_back(L);
    float acc = 0.0f;
    for (size_t j = 0; j < faces.size(); ++j) {
      int t = faces[j];
      for (int k = 0; k < 3; ++k) {
        float3 v = pos[d->indices[3 * t + k]];
        lfaces.push_back(make_float4(v.x, v.y, v.z, 0.0f));
      }
      for (int k = 0; k < 3; ++k) {
        int v = d->indices[3 * t + k];
        float3 n = d->normals ? f3(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]) : f3(0.0f);
        lfaces.push_back(make_float4(n.x, n.y, n.z, 0.0f));
      }
      acc = j == 0 ? w[0] : acc + w[j];  // RandomDistribution::Init, src/component.cpp:12-18
      lprefix.push_back(acc);
    }
  }

  // ---- sky (SkyBox::Init, src/component.cpp:54-67) ----
  std::vector<float4> sky;
  std::vector<float> sky_prefix;
  if (d->env_rgb) {
    const int W = d->env_width, H = d->env_height;
    sky.resize((size_t)W * H);
    sky_prefix.resize((size_t)W * H);
    float acc = 0.0f;
    for (int v = 0; v < H; ++v)
      for (int u = 0; u < W; ++u) {
        size_t i = (size_t)v * W + u;
        float phi = RMN_PI * (float(v) + 0.5f) / float(H);
        float area = std::sin(phi) * 2.0f * RMN_PI / float(W * H);
        float3 c = f3(d->env_rgb[3 * i], d->env_rgb[3 * i + 1], d->env_rgb[3 * i + 2]) * area;
        sky[i] = make_float4(c.x, c.y, c.z, 0.0f);
        float l = dot3(c, f3(0.3f, 0.6f, 0.1f));
        acc = i == 0 ? l : acc + l;
        sky_prefix[i] = acc;
      }
  }

  // ---- upload ----
  s->info.num_triangles = nt;
  s->info.num_inner_nodes = (int)fl.out.size();
  s->info.bvh_depth = fl.max_depth;
  s->info.heap_slots = (int)b.heap.size();
  s->info.num_lights = (int)lights.size();
  s->info.num_materials = d->num_materials;
  DevScene& g = s->dev;
  rmn_status st;
  if ((st = upload(s, fl.out, &g.nodes)) != RMN_OK) return st;
  if ((st = upload(s, tri, &g.tri)) != RMN_OK) return st;
  if ((st = upload(s, shade, &g.shade)) != RMN_OK) return st;
  if ((st = upload(s, mats, &g.mats)) != RMN_OK) return st;
  if ((st = upload(s, lights, &g.lights)) != RMN_OK) return st;
  if ((st = upload(s, lfaces, &g.light_faces)) != RMN_OK) return st;
  if ((st = upload(s, lprefix, &g.light_prefix)) != RMN_OK) return st;
  if (!sky.empty() && (st = acquire_sky(s, d->env_width, d->env_height, sky, sky_prefix)) != RMN_OK) return st;
  if ((st = upload(s, uvs, &g.uv)) != RMN_OK) return st;
  if ((st = upload(s, dtex, &g.texs)) != RMN_OK) return st;
  s->textures = dtex;
  g.texels = nullptr;
  if (texel_bytes > 0) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (size_t)texel_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (textures)");
    s->device_allocations.push_back(p);
    uint8_t* tx = static_cast<uint8_t*>(p);
    for (size_t i = 0; i < dtex.size(); ++i) {
      const rmn_texture& t = d->textures[i];
      e = cudaMemcpy(tx + dtex[i].off[0], t.texels, (size_t)t.width * t.height * 4, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (textures)");
    }
    e = launch_build_mips(tx, dtex.data(), (int)dtex.size(), nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "mip chains");
    s->info.device_bytes += texel_bytes;
    g.texels = tx;
  }
  g.root = root;
  g.num_tris = nt;
  g.num_mats = d->num_materials;
  g.num_lights = (int)lights.size();
  g.sky_w = d->env_rgb ? d->env_width : 0;
  g.sky_h = d->env_rgb ? d->env_height : 0;
  g.depth = fl.max_depth;
  g.has_glass = glass ? 1 : 0;
  g.has_tex = textured ? 1 : 0;
  g.has_alpha = has_alpha ? 1 : 0;
  return RMN_OK;
}

void free_scene(rmn_scene* s) {
  release_sky(s);
  for (void* p : s->device_allocations) cudaFree(p);
  s->device_allocations.clear();
}

}  // namespace rmn
