/*
 * rmn.h -- C ABI of the GB300 path-tracing core (librmn.so).
 *
 * This is the drop-in boundary behind the reference renderer's render.h
 * (lemonchu/Raym0nade). The reference's only render entry point is
 *     void render_multiThread(Model &model, const RenderArgs &args);
 * (include/render.h:43, src/render.cpp:593-677), fed by a Model built from an
 * FBX file (include/model.h:25-43) and RenderArgs (include/render.h:8-15).
 * Under this ABI a caller:
 *   1. describes the scene it would have loaded into Model as flat arrays
 *      (rmn_scene_desc) and calls rmn_scene_create -- the host runs the
 *      reference's BVH construction (src/bvh.cpp:18-54), light-object
 *      construction (src/model.cpp:44-82) and sky tables
 *      (src/component.cpp:54-67), then uploads everything to HBM;
 *   2. renders with rmn_render (the renderPixel loop of render_multiThread,
 *      src/render.cpp:448-551, 593-631) into caller-owned buffers;
 *   3. post-processes with rmn_compose / rmn_fxaa (Photo::shade,
 *      gammaCorrection and FXAA, src/image.cpp:215-246, 363-468).
 * The ray queries of the reference's Model (Model::rayHit and
 * Model::rayHit_test, include/model.h:41-42) are exported as
 * rmn_trace_closest / rmn_trace_shadow.
 *
 * Conventions: every function returns an rmn_status; no C++ exception
 * crosses the ABI; rmn_last_error() describes the last failure of the calling
 * thread. Array arguments may be host memory (pageable or pinned) or device
 * memory of the current device: the library detects which and stages host
 * arrays through the device itself. `stream` is a cudaStream_t (NULL: the
 * legacy default stream); calls return after their work on that stream has
 * completed.
 */
#ifndef RMN_H
#define RMN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rmn_status {
  RMN_OK = 0,
  RMN_ERR_INVALID_ARGUMENT = 1,
  RMN_ERR_CUDA = 2,           /* a CUDA runtime call failed (see rmn_last_error) */
  RMN_ERR_OUT_OF_MEMORY = 3,
  RMN_ERR_UNSUPPORTED = 4,    /* feature outside the GPU path (e.g. glass), see rmn_last_error */
  RMN_ERR_DEVICE_LIMIT = 5,   /* a kernel hit one of its bounds (stack depth, wait limit) and stopped */
  RMN_ERR_INTERNAL = 6
} rmn_status;

/* Material record, 16 floats: per slot a constant texel, resolved exactly
 * as Material::getDiffuseColor, getEmissiveColor and getSurfaceData resolve
 * a texel (src/material.cpp:349-383), unless rmn_scene_desc gives the slot a
 * texture (rmn_texture), which then takes precedence. */
typedef struct rmn_material {
  float base_color[3];   /* diffuse texel, linear RGB */
  float has_base;        /* 0: no diffuse texture -> white */
  float emission[3];     /* emissive texel, linear RGB */
  float has_emission;    /* 0: no emissive texture -> black, and no light object */
  float roughness;       /* specular texel G, or Material::roughness without one */
  float metallic;        /* specular texel B (clamped to <= 0.99); 0 without one */
  float has_specular;    /* 1: roughness/metallic come from a specular texel */
  float opacity;         /* 1 opaque; < 1e-4 transmissive (refraction, media); between: half-opaque */
  float ior;
  float transmitting_color[3];
} rmn_material;

/* 8-bit texture as the reference's DDS loader leaves it in ImageData
 * (Material::loadImageFromDDS, src/material.cpp:190-215): width x height
 * texels of `channels` bytes, row-major, row 0 = the image's top row
 * (texture v = 1). channels must be 4 (RGBA): the reference reads every
 * diffuse, specular and emissive lookup with a 4-byte stride and normal-map
 * lookups with a 3-byte stride whatever the channel count
 * (get_bilinear, src/material.cpp:48-80). The library builds the mip chain
 * of ImageData::generateMipmaps (src/material.cpp:107-129). */
typedef struct rmn_texture {
  int32_t width, height, channels;
  const uint8_t* texels;
} rmn_texture;

/* Texture slots of material_textures (4 per material). */
#define RMN_TEX_DIFFUSE 0   /* aiTextureType_DIFFUSE: base colour (gamma 2.2) and alpha test */
#define RMN_TEX_SPECULAR 1  /* aiTextureType_SPECULAR: G roughness, B metallic, level 0 */
#define RMN_TEX_EMISSIVE 2  /* aiTextureType_EMISSIVE: emission (gamma 2.2); makes the mesh a light object */
#define RMN_TEX_NORMALS 3   /* aiTextureType_NORMALS: tangent-space normal map */

/* Scene arrays; what Model::Model builds from an assimp scene
 * (src/model.cpp:84-123,172-215). Triangles are grouped in meshes with one
 * material each; a mesh whose material has an emissive texel becomes one
 * light object (checkLightObject, src/model.cpp:44-82). */
typedef struct rmn_scene_desc {
  int32_t num_vertices;
  const float* positions;      /* 3 per vertex */
  const float* normals;        /* 3 per vertex, or NULL */
  const float* uvs;            /* 2 per vertex, or NULL */
  int32_t num_triangles;
  const int32_t* indices;      /* 3 per triangle */
  int32_t num_meshes;
  const int32_t* mesh_first;   /* num_meshes + 1 triangle offsets, mesh_first[0] = 0 */
  const int32_t* mesh_material;
  int32_t num_materials;
  const rmn_material* materials;
  int32_t env_width, env_height;  /* lat-long sky (SkyBox, include/component.h:56-67) */
  const float* env_rgb;           /* 3 per texel, row 0 = zenith; NULL: no sky */
  /* Textures (zero / NULL for an untextured scene). material_textures holds
   * 4 texture indices per material (RMN_TEX_*), -1 for none. A diffuse
   * texture with a texel of alpha < 255 makes its material alpha-tested
   * (Material::hasFullyTransparentPart; TransparentTest, src/model.cpp:
   * 217-230). Texels are copied; the caller's arrays may be freed after
   * rmn_scene_create returns. */
  int32_t num_textures;
  const rmn_texture* textures;
  const int32_t* material_textures;
} rmn_scene_desc;

typedef struct rmn_scene rmn_scene;

typedef struct rmn_scene_info {
  int32_t num_triangles;
  int32_t num_inner_nodes;     /* 64-byte two-child nodes in HBM */
  int32_t bvh_depth;           /* deepest leaf, root = 0 */
  int32_t heap_slots;          /* node-array size of the reference builder */
  int32_t num_lights;
  int32_t num_materials;
  int64_t device_bytes;
} rmn_scene_info;

/* A ray: 8 floats (origin, t_min, direction, t_max). Model::rayHit queries
 * use t_min = 1e-4, t_max = +inf (src/model.cpp:333). */
typedef struct rmn_ray {
  float origin[3];
  float t_min;
  float dir[3];
  float t_max;
} rmn_ray;

/* Closest hit: input triangle index (-1: miss), t, and the reference's
 * barycentric(v0, v1, v2, origin + t dir) (src/geometry.cpp:89-103). */
typedef struct rmn_hit {
  int32_t face;
  float t;
  float bary[2]; /* (alpha, beta); gamma = 1 - alpha - beta */
} rmn_hit;

/* RenderArgs (include/render.h:8-15) plus the GPU's own knobs. */
typedef struct rmn_render_args {
  float position[3], direction[3], up[3], right[3];
  float accuracy, focus, CoC, exposure, P_Direct;
  int32_t width, height, spp, threads; /* threads: ignored on the GPU */
  int32_t max_depth;                   /* 16 in the reference (src/render.cpp:125); 1..16 */
  uint64_t seed;                       /* counter-based random stream key */
  int32_t lanes_per_pixel;             /* work units per pixel, each of consecutive sample slots (0: from
                                          slots_per_unit); 1..64 */
  int32_t slots_per_unit;              /* sample slots per path unit; the light-sample slots go in units of
                                          max(slots_per_unit, 8). 0: library default: 2 for renders of up to
                                          2^26 sample slots, else 4, doubled while the render's own per-unit
                                          records, 112 B each, would exceed 16 GiB -- a choice of the render
                                          alone, so its image does not depend on the batch or free memory */
  int32_t reserved[2];
} rmn_render_args;

/* Caller-owned per-pixel outputs (width*height entries each, row-major).
 * radiance_*: 4 floats per pixel (RadianceData: rgb, Var) for
 * direct/indirect x diffuse/specular (Photo, include/image.h:36-39).
 * gbuffer: 21 floats per pixel, the HitInfo of the primary hit
 * (include/model.h:12-18) -- base colour[3], emission[3], position[3]
 * (NaN: the primary ray missed), shape normal[3], surface normal[3],
 * roughness, metallic, opacity, eta, material id, entering (1/0). rmn_render needs the four
 * radiance buffers; gbuffer may be NULL (then it lives in scratch memory). */
typedef struct rmn_image {
  float* radiance_Dd;
  float* radiance_Ds;
  float* radiance_Id;
  float* radiance_Is;
  float* gbuffer;
  int32_t* dropped; /* optional: per pixel, the indirect sample the firefly clamp
                       (src/render.cpp:532-547) dropped, as slot * 8 + sample, or -1 */
} rmn_image;
#define RMN_GBUFFER_FLOATS 21

/* Photo::ShadeOption bits (include/image.h:17-34) used by rmn_compose and
 * rmn_post_process. */
enum {
  RMN_SHADE_BASECOLOR = 1, RMN_SHADE_EMISSION = 2, RMN_SHADE_DIRECT = 4, RMN_SHADE_INDIRECT = 8,
  RMN_SHADE_DIFFUSE = 16, RMN_SHADE_SPECULAR = 32, RMN_SHADE_FULL = 63,
  RMN_SHADE_SHAPE_NORMAL = 64, RMN_SHADE_SURFACE_NORMAL = 128,
  RMN_SHADE_BLOOM = 256,           /* Photo::bloom (rmn_post_process only) */
  RMN_SHADE_FXAA = 512,            /* then Photo::FXAA (display-referred, as postProcessing does) */
  RMN_SHADE_DEPTH_OF_FIELD = 1024, /* Photo::depthFeildBlur (rmn_post_process only) */
  RMN_SHADE_GAMMA = 4096           /* apply Photo::gammaCorrection */
};

/* Photo's post-processing state (include/image.h:36-38). */
typedef struct rmn_post_args {
  int32_t width, height;
  float exposure;
  float focus, CoC;          /* depth of field: focus distance, circle-of-confusion scale (finite, >= 0) */
  float camera_position[3];  /* depth is measured from here */
} rmn_post_args;

const char* rmn_last_error(void);
const char* rmn_version(void);

/* Scene construction: replaces Model::Model's geometry/BVH/light/sky steps
 * (src/model.cpp:172-215) and Material's texture loading and mip chains
 * (src/material.cpp:107-129, 291-302). The arrays of rmn_scene_desc are read
 * on the host (host memory). The host part runs on up to 16 threads of the
 * calling process (disjoint BVH subtrees, per-triangle arrays); the result
 * does not depend on their number. */
rmn_status rmn_scene_create(const rmn_scene_desc* desc, rmn_scene** out);
rmn_status rmn_scene_destroy(rmn_scene* scene);
rmn_status rmn_scene_info_get(const rmn_scene* scene, rmn_scene_info* info);

/* Renders keep the device memory of their worker pools and queues for the
 * next render (up to 16 GiB per device), and the calls' short-lived
 * buffers come from a memory pool of the library's own that keeps up to
 * 1 GiB per device between calls; this frees both, and makes
 * rmn_compose_noalloc resolve its array's device address again (call it
 * after a cudaDeviceReset). No counterpart in the reference. */
rmn_status rmn_release_cached_memory(void);

/* Replaces Model::rayHit (src/model.cpp:332-341): closest hit per ray. */
rmn_status rmn_trace_closest(rmn_scene* scene, const rmn_ray* rays, int64_t n, rmn_hit* hits, void* stream);

/* Replaces Model::rayHit_test (src/model.cpp:343-354): occluded[i] = 1 iff a
 * triangle is hit at t in (1e-4, t_max) where t_max is the aim depth. */
rmn_status rmn_trace_shadow(rmn_scene* scene, const rmn_ray* rays, int64_t n, uint8_t* occluded, void* stream);

/* Replaces the per-pixel work of render_multiThread (src/render.cpp:593-631:
 * renderPixel for every pixel); the export/post steps are rmn_compose and
 * rmn_fxaa. */
rmn_status rmn_render(rmn_scene* scene, const rmn_render_args* args, const rmn_image* image, void* stream);

/* Visit counters and kernel times of one render: rmn_render run twice on
 * the same arguments -- once with counting traversal, once with CUDA events
 * around every kernel -- leaving the same images. For roofline figures
 * (bytes per ray) and ray throughput; not needed to render. */
typedef struct rmn_render_profile {
  double primary_ms;            /* set-up + G-buffer kernel */
  double path_ms;               /* wavefront iterations + finalize */
  double logic_ms, trace_ms;    /* summed over iterations: shading/sampling kernel, the two traversal kernels */
  int64_t iterations;
  uint64_t closest_rays, shadow_rays;
  uint64_t inner_visits, leaf_visits, triangle_tests;
  uint64_t sample_slots, pixels;
} rmn_render_profile;
rmn_status rmn_render_profile_get(rmn_scene* scene, const rmn_render_args* args, const rmn_image* image,
                                  rmn_render_profile* out, void* stream);

/* Batched rendering: many (scene, args, image) renders of uneven size in one
 * persistent launch -- the pixels of every item feed one G-buffer kernel and
 * the sample tasks of every item one persistent path kernel -- optionally
 * captured once into a CUDA graph and replayed by rmn_batch_render. The
 * reference has no counterpart (it renders one Model per render_multiThread
 * call, src/render.cpp:593); each item's images are identical to rmn_render's
 * for the same arguments. All image buffers of a batch must be device memory
 * (their addresses are baked into the batch). */
typedef struct rmn_batch rmn_batch;
typedef struct rmn_batch_item {
  rmn_scene* scene;
  rmn_render_args args;
  rmn_image image;
} rmn_batch_item;
/* Launch knobs of a batch; NULL options = {1, 0, 0}. */
typedef struct rmn_batch_options {
  int32_t use_graph;     /* replay the wavefront iterations from captured CUDA graphs */
  int32_t pool_workers;  /* paths in flight per lane (0: library default, 2^22, halved while the workers
                            would take over a quarter of the free device memory) */
  int32_t lanes;         /* independent wavefronts run side by side, 1..4 (0: library default, 3) */
  int32_t stack_entries; /* traversal stack, 23 or 27 entries (0: library default, the smallest that holds
                            every item's tree: 23 when all trees are at most 22 levels deep); a stack too
                            small for a tree is RMN_ERR_INVALID_ARGUMENT */
  int32_t ray_order;     /* 1: before each traversal launch, reorder its ray queue by bucket (the ray's render,
                            the octant of its direction, the cell of its origin in an 8^3 grid over the scene
                            box) so that a warp traces rays that start close and head alike; 0: as queued.
                            Images do not depend on it. */
  int32_t reserved;
} rmn_batch_options;
rmn_status rmn_batch_create(const rmn_batch_item* items, int32_t n, const rmn_batch_options* options, void* stream,
                            rmn_batch** out);
rmn_status rmn_batch_render(rmn_batch* batch, void* stream);
/* New camera poses, seeds and exposures for the items of a batch (args[i]
 * for items[i] of rmn_batch_create), e.g. per frame of an animation; the
 * next rmn_batch_render on `stream` uses them. Image size, spp, P_Direct,
 * max_depth, lanes_per_pixel and slots_per_unit must stay as the batch was
 * built (RMN_ERR_INVALID_ARGUMENT otherwise). The library uploads its job
 * table, rmn_batch_update_bytes(batch) bytes, from pinned host memory. */
rmn_status rmn_batch_update(rmn_batch* batch, const rmn_render_args* args, int32_t n, void* stream);
int64_t rmn_batch_update_bytes(const rmn_batch* batch);
rmn_status rmn_batch_profile(rmn_batch* batch, rmn_render_profile* out, void* stream);
rmn_status rmn_batch_destroy(rmn_batch* batch);
/* Device bytes rmn_batch_create would take for these items with these
 * options, the scenes and caller-owned images excluded: the per-unit records
 * (112 B per unit of every item, at its slots_per_unit or the library's
 * default split) and the worker pool (per worker its path state, shadow-ray
 * slots and queue entries, times pool_workers per lane -- at most one
 * worker per unit -- times lanes; the library's default pool counted at its
 * full 2^22 per lane). No counterpart in the reference; for callers that
 * plan device memory, and the autotuner's memory cap. */
rmn_status rmn_batch_device_bytes(const rmn_batch_item* items, int32_t n, const rmn_batch_options* options,
                                  int64_t* out);

/* Project-written autotuner for batches. Times candidate launch
 * configurations -- slots per work unit in {2, 4, 8, 16} x workers per lane
 * in {2^20, ..., 2^23} x lanes in {2, 3, 4}, leaving out those whose
 * full-size batch would take more than half of the free device memory (the
 * library's own choice is always timed) -- on a proxy of the batch whose
 * images keep every item's scene, spp, depth and field of view but only
 * `pixel_fraction` (0 < f <= 1) of its pixels, each candidate's workers
 * per lane scaled by the same fraction for its proxy run (at least 4096),
 * so that a worker has as much work as in the full batch
 * (rmn_batch_device_bytes gives a candidate's full size); then the fastest
 * of those
 * once more with the other traversal stack build where the batch's trees
 * allow both (27 entries instead of 23), then the fastest with its ray
 * queues binned (ray_order 1). Returns the fastest. Set each item's
 * slots_per_unit and the batch's pool_workers, lanes, stack_entries and
 * ray_order from the result. The images do not depend on the choice
 * beyond float summation order across units (slots_per_unit); pool size,
 * lanes and stack change nothing. RMN_ERR_OUT_OF_MEMORY when not even the
 * library's default split with the smallest pool (4096 workers, one lane)
 * fits in the free device memory. */
typedef struct rmn_tune_result {
  int32_t slots_per_unit, pool_workers;  /* 0: the library's default won */
  double best_ms, default_ms;  /* proxy render time: best and library default */
  int32_t candidates;          /* configurations timed */
  int32_t lanes;               /* 0: the library's default won */
  int32_t stack_entries;       /* 23 or 27 (the value to pass in rmn_batch_options) */
  int32_t ray_order;           /* 0 or 1 (likewise) */
} rmn_tune_result;
rmn_status rmn_batch_autotune(const rmn_batch_item* items, int32_t n, float pixel_fraction, rmn_tune_result* out,
                              void* stream);

/* Adjoint of rmn_render (path-replay backpropagation). No counterpart in the
 * reference. Given a forward rmn_render of `scene` with `args` -- its
 * G-buffer and its `dropped` record, both required in `image` -- and
 * d_image = dL/dI for the linear composed image
 *   I = base (*) (Dd + Id) + Ds + Is + emission * exposure
 * (Photo::shade(Full), src/image.cpp:215-246; rmn_compose with
 * RMN_SHADE_FULL and no gamma), 3 floats per pixel, writes
 * d_materials[m * RMN_GRAD_PER_MATERIAL + k] = dL/d(parameter k of material
 * m): k = 0..2 the base colour (rmn_material.base_color as resolved: white
 * without a diffuse texel), 3 the roughness (as resolved), 4 the emission
 * scale s (emission = s * rmn_material.emission, at s = 1). The paths are
 * recomputed from the same random streams, so the gradient is that of the
 * forward's own estimate; sampling that depends on the roughness enters by
 * its score function (the estimate is unbiased, not the derivative of one
 * realisation). Buffers may be host or device memory. */
#define RMN_GRAD_PER_MATERIAL 5
rmn_status rmn_adjoint(const rmn_scene* scene, const rmn_render_args* args, const rmn_image* image,
                       const float* d_image, float* d_materials, void* stream);

/* Photo::shade(options) [+ gammaCorrection] [+ FXAA] (src/image.cpp:215-246,
 * 454-479) over rmn_render's buffers -> rgb (3 floats per pixel). */
rmn_status rmn_compose(const rmn_image* image, int32_t width, int32_t height, float exposure, int32_t options,
                       float* rgb, void* stream);

/* rmn_compose without any device allocation. No counterpart in the
 * reference. For callers that cannot allocate device memory (an engine whose
 * arena allocator owns the device memory, or a frame loop that must not let
 * cudaMalloc/cudaFree synchronise the device): the image between compose and
 * FXAA lives in a fixed file-scope device array of RMN_NOALLOC_MAX_PIXELS
 * pixels (24 MiB, held by every GPU that loads the library); larger images
 * are rejected with RMN_ERR_INVALID_ARGUMENT. All buffers must be device
 * memory. The first call on each device resolves the array's address
 * (cudaGetSymbolAddress) and must come before any stream capture; after a
 * cudaDeviceReset, call rmn_release_cached_memory before the next call, so
 * that it resolves the address anew. Calls share the array: calls whose
 * work overlaps on the GPU race. The call returns once its work on `stream`
 * has finished (it synchronises the stream). */
#define RMN_NOALLOC_MAX_PIXELS (1 << 21)
rmn_status rmn_compose_noalloc(const rmn_image* image, int32_t width, int32_t height, float exposure,
                               int32_t options, float* rgb, void* stream);

/* Photo::FXAA (src/image.cpp:363-452) on an rgb image (3 floats per pixel). */
rmn_status rmn_fxaa(const float* rgb_in, float* rgb_out, int32_t width, int32_t height, void* stream);

/* Photo::postProcessing (src/image.cpp:470-479) over rmn_render's buffers:
 * Photo::shade(options), then the depth-of-field blur (RMN_SHADE_DEPTH_OF_FIELD,
 * src/image.cpp:282-356) and bloom (RMN_SHADE_BLOOM, :248-280) when asked,
 * gammaCorrection when RMN_SHADE_GAMMA is set (postProcessing always applies
 * it), FXAA last -> rgb (3 floats per pixel). The depth-of-field blur sorts
 * the pixels' depths on the host (std::stable_sort, as the reference) and
 * synchronises the stream once. */
rmn_status rmn_post_process(const rmn_image* image, const rmn_post_args* args, int32_t options, float* rgb,
                            void* stream);

/* Photo::spatialClamp (src/image.cpp:30-82): clamps fireflies of the four
 * radiance buffers in place. */
rmn_status rmn_spatial_clamp(const rmn_image* image, int32_t width, int32_t height, void* stream);

/* Photo::filter (src/image.cpp:84-213): the G-buffer-guided a-trous filter
 * (filterVar, then passes of step 1..16) of the four radiance buffers, in
 * place (the specular buffers weight by roughness). */
rmn_status rmn_filter(const rmn_image* image, int32_t width, int32_t height, void* stream);

/* The export set of render_multiThread (src/render.cpp:641-674): images
 * k = 0..count-1 (tags from rmn_export_tag) into rgb + 3 * width * height * k,
 * each through Photo::postProcessing (gamma applied): RMN_EXPORTS images, plus
 * RMN_EXPORTS_DOF more when args->CoC > 1e-4 (the depth-of-field exports).
 * As in the reference the radiance buffers are modified on the way:
 * spatialClamp after export 3, filter after export 11. `rgb` holds
 * (RMN_EXPORTS + RMN_EXPORTS_DOF) images; *count receives how many were
 * written. */
#define RMN_EXPORTS 20
#define RMN_EXPORTS_DOF 5
rmn_status rmn_export_set(const rmn_image* image, const rmn_post_args* args, float* rgb, int32_t* count,
                          void* stream);
/* Photo::save (src/image.cpp:481-532) without libpng: rgb (3 floats per
 * pixel, host or device memory) as an 8-bit RGB PNG at `path`, each byte
 * static_cast<uint8_t>(value * 255) as the reference writes it (values
 * outside [0, 1] clamp; the reference leaves them undefined). Rows are
 * filtered adaptively and deflated (LZ77 + dynamic Huffman; stored blocks for
 * incompressible data), as libpng writes by default. */
rmn_status rmn_save_png(const float* rgb, int32_t width, int32_t height, const char* path);

/* Photo::reverseGammaCorrection (src/image.cpp:610-613) on the host: every
 * channel of n rgb pixels to the power 2.2f with the C library's powf, as
 * the reference's glm::pow of floats computes it (the step before FXAA in
 * the reference's fxaa.cpp tool). In place when in == out. */
rmn_status rmn_reverse_gamma(const float* in, int64_t n, float* out);

/* Image decoders of the asset front-end (host memory, no GPU involved). */
#define RMN_IMAGE_PNG 0 /* Material::loadImageFromPNG (src/material.cpp:217-285): 8-bit RGB,
                           16-bit samples keep their high byte, gray and palette expand to RGB,
                           alpha is dropped (libpng's strip_16 / expand / palette_to_rgb /
                           gray_to_rgb / strip_alpha); Adam7-interlaced files are de-interlaced */
#define RMN_IMAGE_DDS 1 /* scripts/dds_to_array.py as Material::loadImageFromDDS
                           (src/material.cpp:190-215) takes it: DXT1/DXT3/DXT5 -> 8-bit RGBA,
                           uncompressed 32-bit -> RGBA, 24-bit -> RGB */
#define RMN_IMAGE_HDR 2 /* scripts/hdr_to_array.py as SkyBox::load (src/component.cpp:69-114)
                           takes it: Radiance RGBE (flat or run-length encoded, "-Y H +X W")
                           -> float32 RGB */

typedef struct rmn_image_desc {
  int32_t width, height, channels;
  int32_t bytes_per_channel;   /* 1 (uint8) or 4 (float32) */
} rmn_image_desc;

/* Decode the image file `path` of the given kind into `data` (capacity
 * bytes, host memory): width x height pixels of `channels` samples,
 * row-major, row 0 = the image's top row. With data == NULL only `info` is
 * filled (the header is read, the pixels are not decoded). Replaces the
 * libpng call of Material::loadImageFromPNG and the embedded-Python calls of
 * call_image_to_array (src/material.cpp:150-188). A malformed file, a
 * missing file or a capacity below width*height*channels*bytes_per_channel
 * gives RMN_ERR_INVALID_ARGUMENT; a valid variant outside the list above
 * (DX10/BC4-BC7 DDS, XYZE or rotated HDR, unknown critical PNG chunks)
 * gives RMN_ERR_UNSUPPORTED. */
rmn_status rmn_image_load(const char* path, int32_t kind, rmn_image_desc* info, void* data, size_t capacity);

/* Copy mip level `level` of scene texture `texture` (RGBA8, built by
 * rmn_scene_create as ImageData::generateMipmaps builds it,
 * src/material.cpp:107-129) from the device into host memory `out`
 * (capacity bytes); `info` receives its size (channels 4, 1 byte each).
 * With out == NULL only `info` is filled. A texture or level the scene does
 * not hold gives RMN_ERR_INVALID_ARGUMENT. */
rmn_status rmn_scene_texture_get(const rmn_scene* scene, int32_t texture, int32_t level, rmn_image_desc* info,
                                 uint8_t* out, size_t capacity);

/* A model read from disk as Model::Model(model_folder, model_name,
 * skyMap_name) reads it (src/model.cpp:124-215): a Wavefront OBJ file
 * (model_folder + model_name) with its MTL libraries, or a binary FBX file
 * (a name ending in .fbx, any case; versions with 32- and 64-bit records,
 * raw or zlib arrays), the textures they name decoded (PNG / DDS, RGB
 * expanded to RGBA) and the sky map (model_folder + skyMap_name, Radiance
 * HDR; "null" or NULL: none). Meshes, materials and texture slots follow
 * assimp's OBJ and FBX imports (FBX: every vertex through its model's world
 * and geometric transform, normals through the inverse transpose) and
 * Material::loadMaterialProperties: name, opacity and textures only. An
 * ASCII FBX file gives RMN_ERR_UNSUPPORTED.
 * rmn_model_desc lays it out for rmn_scene_create; the arrays stay owned by
 * the model until rmn_model_free. A file that cannot be read or parsed gives
 * RMN_ERR_INVALID_ARGUMENT (the message names file and line); a texture of
 * another type, a DDS that does not decode or a sky map that does not decode
 * is left out with a message on stderr, as the reference goes on without it.
 * The OBJ text (in pieces of at least 64 KB) and the texture files are
 * parsed on up to 16 threads of the calling process; the model does not
 * depend on their number. */
typedef struct rmn_model rmn_model;
rmn_status rmn_model_read(const char* model_folder, const char* model_name, const char* skyMap_name,
                          rmn_model** out);
rmn_status rmn_model_desc(const rmn_model* model, rmn_scene_desc* desc);
const char* rmn_model_material_name(const rmn_model* model, int32_t material);  /* NULL out of range */
rmn_status rmn_model_free(rmn_model* model);

/* The file tag of export k ("DiffuseColor", ..., "Filter_DepthFieldBlur_Bloom_FXAA") and its shade
 * options; NULL / -1 out of range. */
const char* rmn_export_tag(int32_t k);
int32_t rmn_export_options(int32_t k);

#ifdef __cplusplus
}
#endif
#endif /* RMN_H */
