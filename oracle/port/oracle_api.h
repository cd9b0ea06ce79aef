// Oracle test infrastructure -- not part of the shipped library.
//
// One C interface, exported twice: by the CPU restatement (oracle/port,
// functions prefixed port_) and by the reference's own sources compiled with
// shims (oracle/ref, functions prefixed ref_, built into oracle/_ref/). The
// tests call both through ctypes and compare them, which pins the
// restatement; the restatement then checks the CUDA library.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Per-material record, 16 floats, shared with the library's rmn_material.
//  [0..2] base colour  [3] has base texel (0: white, Material::getDiffuseColor
//  without a texture, src/material.cpp:349-351)
//  [4..6] emission     [7] has emissive texel
//  [8] roughness [9] metallic [10] has specular texel (src/material.cpp:374-383)
//  [11] opacity  [12] ior     [13..15] transmitting colour
#define ORC_MAT_FLOATS 16

typedef struct orc_scene_in {
  int32_t num_vertices;
  const float* positions;  // 3 per vertex
  const float* normals;    // 3 per vertex
  const float* uvs;        // 2 per vertex
  int32_t num_triangles;
  const int32_t* indices;  // 3 per triangle
  int32_t num_meshes;
  const int32_t* mesh_first;  // num_meshes + 1 triangle offsets
  const int32_t* mesh_material;
  int32_t num_materials;
  const float* materials;  // ORC_MAT_FLOATS per material
  int32_t env_width, env_height;
  const float* env_rgb;  // 3 per texel, row-major from the top row; NULL if none
  // 8-bit textures, row-major as the reference's loaders deliver them:
  // tex_dims 3 per texture (width, height, channels), tex_data one pointer
  // per texture; mat_tex 4 per material (diffuse, specular, emissive, normal
  // map texture index, -1 none), or NULL for no textures at all. A texture
  // slot takes precedence over the record's constant texel.
  int32_t num_textures;
  const int32_t* tex_dims;
  const uint8_t* const* tex_data;
  const int32_t* mat_tex;
} orc_scene_in;

// RenderArgs (include/render.h:8-15) packed as 24 floats:
//  [0..2] position [3..5] direction [6..8] up [9..11] right
//  [12] accuracy [13] focus [14] CoC [15] exposure [16] P_Direct
//  [17] width [18] height [19] spp [20] threads [21] max depth (16)
#define ORC_ARGS_FLOATS 24

// Per-pixel output record of a render, ORC_PIX_FLOATS floats:
//  [0..3] Dd  [4..7] Ds  [8..11] Id  [12..15] Is   (RadianceData: rgb, Var)
//  [16..18] G-buffer base colour  [19..21] emission  [22..24] position
//  [25..27] shape normal  [28..30] surface normal
//  [31] roughness [32] metallic [33] opacity [34] specular [35] eta
//  [36] material id [37] entering [38] indirect sample count [39] spp_indirect
#define ORC_PIX_FLOATS 40

// Photo's post passes (src/image.cpp:30-356, 454-479) on a W x H render
// given as records (radiance with Var, G-buffer fields; in place):
//   stages bit 1  Photo::spatialClamp of the four radiance buffers;
//          bit 2  Photo::filter (filterVar + five a-trous passes);
//          bit 4  Photo::postProcessing(options) into rgb (3 per pixel):
//                 shade, depth-of-field blur (1024), bloom (256), gamma,
//                 FXAA (512);
//          bit 8  the same without gamma and FXAA (linear).
// post: exposure, focus, CoC, camera position (3).
void port_photo(float* recs, int w, int h, int stages, int options, const float* post, float* rgb);
void ref_photo(float* recs, int w, int h, int stages, int options, const float* post, float* rgb);

#ifdef __cplusplus
}
#endif

// Per-pixel seed of the reference's Generator in the deterministic render
// loop: the reference seeds one mt19937 per worker thread
// (src/render.cpp:658-661), which makes images depend on scheduling; this
// loop seeds one per pixel instead.
static inline uint32_t orc_pixel_seed(uint64_t seed, uint32_t pixel) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)pixel * 0xBF58476D1CE4E5B9ULL + 1u;
  z = (z ^ (z >> 31)) * 0x94D049BB133111EBULL;
  return (uint32_t)(z >> 32);
}
