// Oracle test infrastructure -- not part of the shipped library.
//
// Harness around the reference's own, unmodified sources
// (src/geometry.cpp, bvh.cpp, component.cpp, sampling.cpp, model.cpp,
// render.cpp, image.cpp of lemonchu/Raym0nade), compiled by oracle/ref/Makefile
// into oracle/_ref/libref.so with the shims in oracle/shim standing in for
// glm, assimp and libpng. It exports the ref_* functions of
// oracle/port/oracle_api.h so tests can hold the CPU restatement
// (oracle/port) against the reference itself.
//
// What the harness supplies in place of the reference's asset layer:
//  * libref.so: src/material.cpp is replaced by the definitions below
//    (ORC_REAL_MATERIAL undefined): a material holds
//    at most one constant float texel per texture slot (diffuse, specular,
//    emissive), stored as four floats in the slot's level-0 byte vector;
//    getDiffuseColor / getEmissiveColor / getSurfaceData return that texel
//    (with getSurfaceData's clamps) and getNormal returns the zero texel of a
//    missing normal map, as src/material.cpp:349-383 does without textures.
//  * libref_tex.so (ORC_REAL_MATERIAL): the reference's own src/material.cpp
//    is linked; texture slots receive the scene's 8-bit textures (what
//    Material::loadImageFromFile leaves in ImageData after a DDS load),
//    ImageData::generateMipmaps builds their mip chains and
//    hasFullyTransparentPart is set as Material::loadMaterialProperties
//    sets it. A constant texel cannot be expressed there, so a material
//    record that asks for one without a texture in that slot is refused.
//  * Model's public members are filled directly (what Model::Model does
//    through assimp, src/model.cpp:172-215), including the per-mesh
//    checkLightObject call, SkyBox::Init and BVH::build.
//  * Each triangle owns three VertexData copies, so the input triangle index
//    of a Face is (data[0] - &vertexDatas[0]) / 3 after BVH::build permutes
//    the faces.
//  * renderPixel (src/render.cpp:448) is driven per pixel with its own
//    RenderData seeded by orc_pixel_seed, instead of render_multiThread's
//    per-thread seeds.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <csetjmp>
#include <cstring>
#include <iostream>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include <Python.h>
#include <glm/glm.hpp>
#include <assimp/Importer.hpp>
#include <assimp/material.h>
#include <assimp/postprocess.h>
#include <assimp/scene.h>
#include <png.h>

// The harness needs Model::checkLightObject, SkyBox::Init and BVH's node
// array, which the reference declares private (BVH by class default).
#define private public
#define class struct
#include "bvh.h"
#include "component.h"
#include "geometry.h"
#include "image.h"
#include "material.h"
#include "model.h"
#include "render.h"
#include "sampling.h"
#undef class
#undef private

#include "../port/oracle_api.h"

#ifndef ORC_REAL_MATERIAL
// ---------------------------------------------------------------------------
// src/material.cpp replacement (constant texels).
static void put_texel(ImageData& img, float a, float b, float c, float d) {
  float v[4] = {a, b, c, d};
  img.width = img.height = 1;
  img.channels = 4;
  img.map_depth = 1;
  img.data[0].resize(sizeof v);
  std::memcpy(img.data[0].data(), v, sizeof v);
}
static vec4 get_texel(const ImageData& img) {
  float v[4];
  std::memcpy(v, img.data[0].data(), sizeof v);
  return vec4(v[0], v[1], v[2], v[3]);
}

std::string urlDecode(const std::string& src) { return src; }
PyObject* call_image_to_array(const std::string&, const std::string&) { return nullptr; }
ImageData::ImageData() : width(0), height(0), channels(0), map_depth(0) {}
bool ImageData::empty() const { return data[0].empty(); }
bool ImageData::hasTransparentPart() const { return false; }
void ImageData::generateMipmaps() {}
Material::Material()
    : hasFullyTransparentPart(false), opacity(1.0f), ior(1.0f), roughness(0.8f), transmittingColor(0.0f), id(0) {}
bool Material::loadImageFromDDS(ImageData&, const std::string&) { return false; }
bool Material::loadImageFromPNG(ImageData&, const std::string&) { return false; }
void Material::loadImageFromFile(int, const std::string&) {}
void Material::loadMaterialProperties(const aiMaterial*) {}
vec4 Material::getDiffuseColor(float, float, float) const {
  if (texture[aiTextureType_DIFFUSE].empty()) return vec4(1.0f);
  return get_texel(texture[aiTextureType_DIFFUSE]);
}
vec3 Material::getNormal(float, float, float) const { return vec3(0.0f); }
vec3 Material::getEmissiveColor(float, float, float) const {
  if (texture[aiTextureType_EMISSIVE].empty()) return vec3(0.0f);
  return get_texel(texture[aiTextureType_EMISSIVE]);
}
void Material::getSurfaceData(float, float, float& r, float& m) const {
  if (texture[aiTextureType_SPECULAR].empty()) {
    m = 0.0f;
    r = this->roughness;
    return;
  }
  vec4 t = get_texel(texture[aiTextureType_SPECULAR]);
  m = std::min(t[2], 0.99f);
  r = std::max(t[1], 1e-3f);
}
#endif

// ---------------------------------------------------------------------------
// libpng entry points. Writing records the IHDR size and the rows handed to
// png_write_row (ref_save_rows reads them back: the bytes Photo::save
// produces); nothing is compressed or read.
static jmp_buf g_png_jmp;
static unsigned g_png_w = 0, g_png_h = 0;
static std::vector<png_byte> g_png_rows;
jmp_buf* oracle_png_jmpbuf(png_structp) { return &g_png_jmp; }
png_structp png_create_write_struct(const char*, void*, void*, void*) { return nullptr; }
png_structp png_create_read_struct(const char*, void*, void*, void*) { return nullptr; }
png_infop png_create_info_struct(png_structp) { return nullptr; }
void png_destroy_write_struct(png_structp*, png_infop*) {}
void png_destroy_read_struct(png_structp*, png_infop*, png_infop*) {}
void png_init_io(png_structp, FILE*) {}
void png_set_IHDR(png_structp, png_infop, unsigned w, unsigned h, int, int, int, int, int) {
  g_png_w = w;
  g_png_h = h;
  g_png_rows.clear();
}
void png_write_info(png_structp, png_infop) {}
void png_write_row(png_structp, png_bytep row) { g_png_rows.insert(g_png_rows.end(), row, row + 3 * g_png_w); }
void png_write_end(png_structp, png_infop) {}
void png_read_info(png_structp, png_infop) {}
unsigned png_get_image_width(png_structp, png_infop) { return 0; }
unsigned png_get_image_height(png_structp, png_infop) { return 0; }
png_byte png_get_color_type(png_structp, png_infop) { return 0; }
png_byte png_get_bit_depth(png_structp, png_infop) { return 8; }
unsigned png_get_valid(png_structp, png_infop, unsigned) { return 0; }
void png_set_strip_16(png_structp) {}
void png_set_palette_to_rgb(png_structp) {}
void png_set_expand_gray_1_2_4_to_8(png_structp) {}
void png_set_tRNS_to_alpha(png_structp) {}
void png_set_filler(png_structp, unsigned, int) {}
void png_set_gray_to_rgb(png_structp) {}
void png_set_strip_alpha(png_structp) {}
void png_read_update_info(png_structp, png_infop) {}
void png_read_row(png_structp, png_bytep, png_bytep) {}

// Defined with external linkage in the reference but declared in no header.
int nodeCount(int u, int n);
void renderPixel(const Model& model, const RenderArgs& args, RenderData& renderData, Photo& image, int x, int y);

template <class F>
static void for_each_index(long n, int threads, F&& f, long chunk = 64) {
  if (threads <= 1 || n <= chunk) {
    for (long i = 0; i < n; ++i) f(i);
    return;
  }
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

static int face_id(const Model& m, const Face* f) { return (int)((f->data[0] - &m.vertexDatas[0]) / 3); }

extern "C" {

void* ref_scene_create(const orc_scene_in* in) {
  Model* m = new Model();
  m->materials.resize(in->num_materials);
  for (int i = 0; i < in->num_materials; ++i) {
    const float* p = in->materials + ORC_MAT_FLOATS * i;
    Material& q = m->materials[i];
    q.id = i;
#ifdef ORC_REAL_MATERIAL
    static const int slot[4] = {aiTextureType_DIFFUSE, aiTextureType_SPECULAR, aiTextureType_EMISSIVE,
                                aiTextureType_NORMALS};
    static const int flag[4] = {3, 10, 7, -1};
    for (int k = 0; k < 4; ++k) {
      int t = in->mat_tex ? in->mat_tex[4 * i + k] : -1;
      if (t < 0) {
        if (flag[k] >= 0 && p[flag[k]] != 0.0f) {
          std::cerr << "libref_tex: material " << i << " asks for a constant texel" << std::endl;
          delete m;
          return nullptr;
        }
        continue;
      }
      ImageData& img = q.texture[slot[k]];
      img.width = in->tex_dims[3 * t];
      img.height = in->tex_dims[3 * t + 1];
      img.channels = in->tex_dims[3 * t + 2];
      img.data[0].assign(in->tex_data[t], in->tex_data[t] + (size_t)img.width * img.height * img.channels);
      img.generateMipmaps();
    }
    if (q.texture[aiTextureType_DIFFUSE].hasTransparentPart()) q.hasFullyTransparentPart = true;
    q.roughness = p[8];
#else
    if (p[3] != 0.0f) put_texel(q.texture[aiTextureType_DIFFUSE], p[0], p[1], p[2], 1.0f);
    if (p[7] != 0.0f) put_texel(q.texture[aiTextureType_EMISSIVE], p[4], p[5], p[6], 1.0f);
    if (p[10] != 0.0f) put_texel(q.texture[aiTextureType_SPECULAR], 0.0f, p[8], p[9], 1.0f);
    else q.roughness = p[8];
#endif
    q.opacity = p[11];
    q.ior = p[12];
    q.transmittingColor = vec3(p[13], p[14], p[15]);
  }
  m->vertexDatas.reserve(3 * (size_t)in->num_triangles);
  m->faces.reserve(in->num_triangles);
  for (int mesh = 0; mesh < in->num_meshes; ++mesh) {
    int first = in->mesh_first[mesh], last = in->mesh_first[mesh + 1];
    const Material& mat = m->materials[in->mesh_material[mesh]];
    size_t off = m->faces.size();
    for (int t = first; t < last; ++t) {
      Face f;
      for (int k = 0; k < 3; ++k) {
        int v = in->indices[3 * t + k];
        vec2 uv = in->uvs ? vec2(in->uvs[2 * v], in->uvs[2 * v + 1]) : vec2(0.0f);
        vec3 n = in->normals ? vec3(in->normals[3 * v], in->normals[3 * v + 1], in->normals[3 * v + 2]) : vec3(0.0f);
        m->vertexDatas.emplace_back(uv, n);
        f.v[k] = vec3(in->positions[3 * v], in->positions[3 * v + 1], in->positions[3 * v + 2]);
        f.data[k] = &m->vertexDatas.back();
      }
      f.material = &mat;
      m->faces.push_back(f);
    }
    // src/model.cpp:121-122; the sky map is loaded after the meshes, so it
    // is still empty here.
    if (!mat.texture[aiTextureType_EMISSIVE].empty() && m->skyMap.empty()) {
      aiMesh am;
      am.mNumFaces = (unsigned)(last - first);
      m->checkLightObject(&m->faces[off], &am, mat);
    }
  }
  if (in->env_rgb && in->env_width > 0 && in->env_height > 0) {
    m->skyMap.width = in->env_width;
    m->skyMap.height = in->env_height;
    size_t n = (size_t)in->env_width * in->env_height;
    m->skyMap.data.reserve(n);
    for (size_t i = 0; i < n; ++i)
      m->skyMap.data.emplace_back(in->env_rgb[3 * i], in->env_rgb[3 * i + 1], in->env_rgb[3 * i + 2]);
    m->skyMap.Init();
  }
  m->bvh.build(m->faces);
  return m;
}

void ref_scene_destroy(void* h) { delete static_cast<Model*>(h); }

int ref_bvh_size(void* h) { return nodeCount(1, (int)static_cast<Model*>(h)->faces.size()) + 1; }

void ref_bvh_export(void* h, float* boxes, int32_t* ranges, int32_t* order) {
  const Model& m = *static_cast<Model*>(h);
  int n = ref_bvh_size(h);
  for (int u = 0; u < n; ++u) {
    const BVH_Node& nd = m.bvh.node[u];
    float b[6] = {nd.box.v0.x, nd.box.v0.y, nd.box.v0.z, nd.box.v1.x, nd.box.v1.y, nd.box.v1.z};
    std::memcpy(boxes + 6 * u, b, sizeof b);
    ranges[2 * u] = nd.faceL;
    ranges[2 * u + 1] = nd.faceR;
  }
  for (size_t i = 0; i < m.faces.size(); ++i) order[i] = face_id(m, &m.faces[i]);
}

int ref_light_count(void* h) { return (int)static_cast<Model*>(h)->lightObjects.size(); }
void ref_light_export(void* h, float* out) {
  const Model& m = *static_cast<Model*>(h);
  for (size_t i = 0; i < m.lightObjects.size(); ++i) {
    const LightObject& l = m.lightObjects[i];
    float r[8] = {l.center.x, l.center.y, l.center.z, l.color.x, l.color.y, l.color.z, l.power, (float)l.faces.size()};
    std::memcpy(out + 8 * i, r, sizeof r);
  }
}

void ref_trace_closest(void* h, const float* rays, int64_t n, int32_t* face, float* t, float* bc, int threads) {
  const Model& m = *static_cast<Model*>(h);
  for_each_index(n, threads, [&](long i) {
    const float* r = rays + 8 * i;
    Ray ray{vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6])};
    HitRecord hit;
    if (r[3] == eps_zero && std::isinf(r[7]) && r[7] > 0) {
      hit = m.rayHit(ray);
    } else {
      hit = HitRecord(r[3], r[7]);
      m.bvh.rayHit(ray, hit);
    }
    if (!hit.face) {
      face[i] = -1; t[i] = hit.t_max; bc[3 * i] = bc[3 * i + 1] = bc[3 * i + 2] = 0.0f;
      return;
    }
    face[i] = face_id(m, hit.face);
    t[i] = hit.t_max;
    vec3 b = barycentric(hit.face->v[0], hit.face->v[1], hit.face->v[2], ray.origin + ray.direction * hit.t_max);
    bc[3 * i] = b.x; bc[3 * i + 1] = b.y; bc[3 * i + 2] = b.z;
  });
}

void ref_trace_shadow(void* h, const float* rays, int64_t n, uint8_t* occ, int threads) {
  const Model& m = *static_cast<Model*>(h);
  for_each_index(n, threads, [&](long i) {
    const float* r = rays + 8 * i;
    occ[i] = m.rayHit_test(Ray{vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6])}, r[7]) ? 1 : 0;
  });
}

static RenderArgs unpack(const float* p) {
  RenderArgs a;
  a.position = vec3(p[0], p[1], p[2]);
  a.direction = vec3(p[3], p[4], p[5]);
  a.up = vec3(p[6], p[7], p[8]);
  a.right = vec3(p[9], p[10], p[11]);
  a.accuracy = p[12]; a.focus = p[13]; a.CoC = p[14]; a.exposure = p[15]; a.P_Direct = p[16];
  a.width = (int)p[17]; a.height = (int)p[18]; a.spp = (int)p[19]; a.threads = (int)p[20];
  return a;
}

static void put_pixel(const Photo& ph, int id, float* rec) {
  const RadianceData* rr[4] = {&ph.radiance_Dd[id], &ph.radiance_Ds[id], &ph.radiance_Id[id], &ph.radiance_Is[id]};
  for (int k = 0; k < 4; ++k) {
    rec[4 * k] = rr[k]->radiance.x; rec[4 * k + 1] = rr[k]->radiance.y; rec[4 * k + 2] = rr[k]->radiance.z;
    rec[4 * k + 3] = rr[k]->Var;
  }
  const HitInfo& g = ph.Gbuffer[id];
  auto put3 = [&](int o, const vec3& v) { rec[o] = v.x; rec[o + 1] = v.y; rec[o + 2] = v.z; };
  put3(16, g.baseColor); put3(19, g.emission); put3(22, g.position); put3(25, g.shapeNormal); put3(28, g.surfaceNormal);
  rec[31] = g.roughness; rec[32] = g.metallic; rec[33] = g.opacity; rec[34] = g.specular; rec[35] = g.eta;
  rec[36] = (float)g.id; rec[37] = g.entering ? 1.0f : 0.0f; rec[38] = -1.0f; rec[39] = -1.0f;
}

// mode must be 0 (the reference's own mt19937 stream); max depth is the
// reference's compile-time 16 (src/render.cpp:125) whatever args[21] says.
void ref_render(void* h, const float* args, uint64_t seed, int mode, int x0, int y0, int x1, int y1, float* out,
                int threads) {
  if (mode != 0) return;
  const Model& m = *static_cast<Model*>(h);
  RenderArgs a = unpack(args);
  Photo ph(a.width, a.height);
  ph.exposure = a.exposure;
  int rw = x1 - x0;
  long n = (long)rw * (y1 - y0);
  for_each_index(n, threads, [&](long i) {
    int x = x0 + (int)(i % rw), y = y0 + (int)(i / rw);
    int id = y * a.width + x;
    RenderData rd((int)orc_pixel_seed(seed, (uint32_t)id));
    renderPixel(m, a, rd, ph, x, y);
    put_pixel(ph, id, out + ORC_PIX_FLOATS * i);
  }, 1);
}

// renderPixel for the listed pixels (row-major indices), each with its
// per-pixel seeded Generator; out holds ORC_PIX_FLOATS per listed pixel.
void ref_render_pixels(void* h, const float* args, uint64_t seed, int mode, const int32_t* pixels, int64_t n,
                       float* out, int threads) {
  if (mode != 0) return;
  const Model& m = *static_cast<Model*>(h);
  RenderArgs a = unpack(args);
  Photo ph(a.width, a.height);
  ph.exposure = a.exposure;
  for_each_index((long)n, threads, [&](long i) {
    const int id = pixels[i];
    RenderData rd((int)orc_pixel_seed(seed, (uint32_t)id));
    renderPixel(m, a, rd, ph, id % a.width, id / a.width);
    put_pixel(ph, id, out + ORC_PIX_FLOATS * i);
  }, 1);
}

void ref_compose(const float* recs, int64_t n, float exposure, int apply_gamma, float* rgb) {
  Photo ph((int)n, 1);
  ph.exposure = exposure;
  for (int64_t i = 0; i < n; ++i) {
    const float* r = recs + ORC_PIX_FLOATS * i;
    ph.radiance_Dd[i].radiance = vec3(r[0], r[1], r[2]);
    ph.radiance_Ds[i].radiance = vec3(r[4], r[5], r[6]);
    ph.radiance_Id[i].radiance = vec3(r[8], r[9], r[10]);
    ph.radiance_Is[i].radiance = vec3(r[12], r[13], r[14]);
    ph.Gbuffer[i].baseColor = vec3(r[16], r[17], r[18]);
    ph.Gbuffer[i].emission = vec3(r[19], r[20], r[21]);
  }
  ph.shade(Photo::Full);
  if (apply_gamma) ph.gammaCorrection();
  for (int64_t i = 0; i < n; ++i) {
    rgb[3 * i] = ph.pixelarray[i].x; rgb[3 * i + 1] = ph.pixelarray[i].y; rgb[3 * i + 2] = ph.pixelarray[i].z;
  }
}

// Photo::reverseGammaCorrection (src/image.cpp:610-613) over n rgb pixels.
void ref_reverse_gamma(const float* in, int64_t n, float* out) {
  Photo ph((int)n, 1);
  for (int64_t i = 0; i < n; ++i) ph.pixelarray[i] = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  ph.reverseGammaCorrection();
  for (int64_t i = 0; i < n; ++i) {
    out[3 * i] = ph.pixelarray[i].x; out[3 * i + 1] = ph.pixelarray[i].y; out[3 * i + 2] = ph.pixelarray[i].z;
  }
}

void ref_gamma(const float* in, int64_t n, float* out) {
  Photo ph((int)n, 1);
  for (int64_t i = 0; i < n; ++i) ph.pixelarray[i] = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  ph.gammaCorrection();
  for (int64_t i = 0; i < n; ++i) {
    out[3 * i] = ph.pixelarray[i].x; out[3 * i + 1] = ph.pixelarray[i].y; out[3 * i + 2] = ph.pixelarray[i].z;
  }
}

void ref_photo(float* recs, int w, int h, int stages, int options, const float* post, float* rgb) {
  Photo ph(w, h);
  ph.exposure = post[0];
  ph.focus = post[1];
  ph.CoC = post[2];
  ph.cameraPosition = vec3(post[3], post[4], post[5]);
  const long n = (long)w * h;
  RadianceData* bufs[4] = {ph.radiance_Dd, ph.radiance_Ds, ph.radiance_Id, ph.radiance_Is};
  for (long i = 0; i < n; ++i) {
    const float* r = recs + ORC_PIX_FLOATS * i;
    for (int b = 0; b < 4; ++b) {
      bufs[b][i].radiance = vec3(r[4 * b], r[4 * b + 1], r[4 * b + 2]);
      bufs[b][i].Var = r[4 * b + 3];
    }
    HitInfo& G = ph.Gbuffer[i];
    G.baseColor = vec3(r[16], r[17], r[18]);
    G.emission = vec3(r[19], r[20], r[21]);
    G.position = vec3(r[22], r[23], r[24]);
    G.shapeNormal = vec3(r[25], r[26], r[27]);
    G.surfaceNormal = vec3(r[28], r[29], r[30]);
    G.roughness = r[31]; G.metallic = r[32]; G.opacity = r[33]; G.specular = r[34]; G.eta = r[35];
    G.id = (int)r[36]; G.entering = r[37] != 0.0f;
  }
  if (stages & 1) ph.spatialClamp();
  if (stages & 2) ph.filter();
  if (stages & 4) ph.postProcessing(options);
  if (stages & 8) {  // postProcessing without gammaCorrection and FXAA
    ph.shade(options);
    if (options & Photo::DoDepthFieldBlur) ph.depthFeildBlur();
    if (options & Photo::DoBloom) ph.bloom();
  }
  if (stages & (4 | 8))
    for (long i = 0; i < n; ++i) {
      rgb[3 * i] = ph.pixelarray[i].x; rgb[3 * i + 1] = ph.pixelarray[i].y; rgb[3 * i + 2] = ph.pixelarray[i].z;
    }
  for (long i = 0; i < n; ++i) {
    float* r = recs + ORC_PIX_FLOATS * i;
    for (int b = 0; b < 4; ++b) {
      r[4 * b] = bufs[b][i].radiance.x; r[4 * b + 1] = bufs[b][i].radiance.y; r[4 * b + 2] = bufs[b][i].radiance.z;
      r[4 * b + 3] = bufs[b][i].Var;
    }
  }
}

#ifdef ORC_REAL_MATERIAL
// ImageData::generateMipmaps (src/material.cpp:107-129) on an 8-bit image:
// the levels packed one after the other into out (capacity bytes). Returns
// the number of levels, or -1 when out is too small.
int ref_mip_chain(const uint8_t* texels, int w, int h, int channels, uint8_t* out, size_t capacity) {
  ImageData img;
  img.width = w;
  img.height = h;
  img.channels = channels;
  img.data[0].assign(texels, texels + (size_t)w * h * channels);
  img.generateMipmaps();
  size_t at = 0;
  for (int l = 0; l < img.map_depth; ++l) {
    const size_t n = img.data[l].size();
    if (at + n > capacity) return -1;
    std::memcpy(out + at, img.data[l].data(), n);
    at += n;
  }
  return img.map_depth;
}

// SkyBox::load (src/component.cpp:69-114) as the reference runs it: through
// call_image_to_array and the Python function hdr_to_array of module
// hdr_to_array on the interpreter's path (./scripts). Call with the GIL held.
// out receives the SkyBox's texels after SkyBox::Init (premultiplied by the
// texel solid angle). Returns 0, or -1 for an empty sky or a small buffer.
int ref_sky_load(const char* path, float* out, long capacity, int* w, int* h) {
  SkyBox sky;
  sky.load(path);
  if (sky.empty() || (long)sky.data.size() * 3 > capacity) return -1;
  *w = sky.width;
  *h = sky.height;
  for (size_t i = 0; i < sky.data.size(); ++i)
    for (int c = 0; c < 3; ++c) out[3 * i + c] = sky.data[i][c];
  return 0;
}

// Material::loadImageFromDDS (src/material.cpp:190-215) through the Python
// function dds_to_array, as above: level 0 of the ImageData it fills.
int ref_dds_load(const char* path, uint8_t* out, long capacity, int* dims) {
  ImageData img;
  if (!Material::loadImageFromDDS(img, path) || img.data[0].empty()) return -1;
  if ((long)img.data[0].size() > capacity) return -1;
  dims[0] = img.width;
  dims[1] = img.height;
  dims[2] = img.channels;
  std::memcpy(out, img.data[0].data(), img.data[0].size());
  return 0;
}

// Material::loadMaterialProperties (src/material.cpp:300-336) for a material
// of this name and (when has_opacity) opacity, without textures: out =
// opacity, ior, roughness, transmitting colour (3), hasFullyTransparentPart.
void ref_material_properties(const char* name, float opacity, int has_opacity, float* out) {
  aiMaterial am;
  am.has_name = true;
  am.name = name;
  am.has_opacity = has_opacity != 0;
  am.opacity = opacity;
  Material m;
  m.loadMaterialProperties(&am);
  out[0] = m.opacity;
  out[1] = m.ior;
  out[2] = m.roughness;
  out[3] = m.transmittingColor.x;
  out[4] = m.transmittingColor.y;
  out[5] = m.transmittingColor.z;
  out[6] = m.hasFullyTransparentPart ? 1.0f : 0.0f;
}

// urlDecode (src/material.cpp:9-24) into out (NUL-terminated); returns the
// decoded length or -1 when out is too small.
int ref_url_decode(const char* in, char* out, int capacity) {
  const std::string s = urlDecode(in);
  if ((int)s.size() + 1 > capacity) return -1;
  std::memcpy(out, s.data(), s.size());
  out[s.size()] = 0;
  return (int)s.size();
}
#endif

// Photo::save (src/image.cpp:481-532) of an RGB image: the 8-bit rows it
// hands to libpng, into out (w * h * 3 bytes). Returns 0, or -1 when the
// rows did not arrive (path not writable).
int ref_save_rows(const float* rgb, int w, int h, const char* path, uint8_t* out) {
  Photo ph(w, h);
  for (long i = 0; i < (long)w * h; ++i) ph.pixelarray[i] = vec3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
  g_png_rows.clear();
  ph.save(path);
  if (g_png_rows.size() != (size_t)w * h * 3) return -1;
  std::memcpy(out, g_png_rows.data(), g_png_rows.size());
  return 0;
}

void ref_fxaa(const float* in, float* out, int w, int h) {
  Photo ph(w, h);
  for (long i = 0; i < (long)w * h; ++i) ph.pixelarray[i] = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  ph.FXAA();
  for (long i = 0; i < (long)w * h; ++i) {
    out[3 * i] = ph.pixelarray[i].x; out[3 * i + 1] = ph.pixelarray[i].y; out[3 * i + 2] = ph.pixelarray[i].z;
  }
}

}  // extern "C"
