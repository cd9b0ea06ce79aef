// Internal layout of a scene in HBM and the float3 arithmetic shared by the
// host builder (C++) and the kernels (CUDA).
//
// Arithmetic follows the reference's glm expressions operation by operation
// (dot = (x*x' + y*y') + z*z', cross, normalize = v * (1/sqrt(dot(v,v))),
// scalar division component-wise). Every translation unit is compiled
// without floating-point contraction (-ffp-contract=off / nvcc -fmad=false),
// so closest-hit ids and t values come out bit-identical to the reference's
// CPU traversal.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>

#if defined(__CUDACC__)
#define RMN_HD __host__ __device__ __forceinline__
#define RMN_D __device__ __forceinline__
#else
#define RMN_HD inline
#endif

#include "rmn_rng.h"

// ------------------------------------------------------------ float3 ------
RMN_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
RMN_HD float3 f3(float s) { return make_float3(s, s, s); }
RMN_HD float3 f3(const float4& v) { return make_float3(v.x, v.y, v.z); }
RMN_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
RMN_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
RMN_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
RMN_HD float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
RMN_HD float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
RMN_HD float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
RMN_HD float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
RMN_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
RMN_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
RMN_HD float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
RMN_HD float3& operator*=(float3& a, float s) { a = a * s; return a; }
RMN_HD float3& operator/=(float3& a, float s) { a = a / s; return a; }
RMN_HD float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RMN_HD float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
RMN_HD float len3(float3 v) { return sqrtf(dot3(v, v)); }
RMN_HD float3 norm3(float3 v) {
  float inv = 1.0f / sqrtf(dot3(v, v));
  return v * inv;
}
// The reference's isfinite(vec3): true if ANY component is finite (src/geometry.cpp:8-10).
#if defined(__CUDA_ARCH__)
RMN_HD bool finite1(float x) { return isfinite(x); }
#else
RMN_HD bool finite1(float x) { return std::isfinite(x); }
#endif
RMN_HD bool any_finite3(float3 v) { return finite1(v.x) || finite1(v.y) || finite1(v.z); }
RMN_HD bool all_finite3(float3 v) { return finite1(v.x) && finite1(v.y) && finite1(v.z); }
RMN_HD float3 min3(float3 a, float3 b) { return f3(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z); }
RMN_HD float3 max3(float3 a, float3 b) { return f3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z); }
RMN_HD float3 mix3(float3 x, float3 y, float a) { return x * (1.0f - a) + y * a; }

// ------------------------------------------------------------ constants ---
#define RMN_EPS 1e-4f                 // eps_zero, include/geometry.h:13
#define RMN_PI 3.14159265358979323846f
#define RMN_LEAF_MAX 10               // LeafBagSize, src/bvh.cpp:16
// traversal stack entries: trees up to depth 26 (median splits of < 2^27
// triangles stay below 26 levels); 27 x 8 B x 128 threads of shared memory
// (with the leaf keys) lets 7 persistent traversal blocks share an SM
#define RMN_STACK 27
// A shallower stack for batches whose trees are at most RMN_STACK_SMALL - 1
// deep: less shared memory, one more persistent traversal block per SM.
#define RMN_STACK_SMALL 23
// Persistent traversal kernels (trace.cuh, warp-cooperative leaves): inner-
// node steps per round, and blocks per SM for a shared stack of S entries
// (S * 1 KiB of stack plus 1 KiB of leaf keys per 128-thread block).
constexpr int kCoopSteps = 4;
constexpr int kOccSteps = 10;  // occlusion queries with pending leaves (trace.cuh, occ_nodes)
// Occlusion kernels: a stack of node references (S * 512 B) and the leaf
// exchange (about 11 KB) per 128-thread block leave room for 8 blocks per SM.
#define RMN_OCC_BLOCKS 8
#define RMN_COOP_BLOCKS(S) ((S) <= RMN_STACK_SMALL ? 8 : 7)

// ------------------------------------------------------------ layout ------
// Two-child node (64 B): the boxes of both children plus their references,
// so one node fetch serves the reference's two rayInBox tests
// (src/bvh.cpp:74-75). Child reference >= 0: inner node index; < 0: leaf,
// ~(first_triangle << 4 | count).
struct __align__(16) DevNode {
  float4 a;  // L.lo.x L.lo.y L.lo.z L.hi.x
  float4 b;  // L.hi.y L.hi.z R.lo.x R.lo.y
  float4 c;  // R.lo.z R.hi.x R.hi.y R.hi.z
  int4 d;    // L ref, R ref, -, -
};
RMN_HD int leaf_ref(int first, int count) { return ~((first << 4) | count); }

// Triangles in BVH leaf order, 3 float4 each (48 B):
//   [0] v0.xyz, w = input triangle index (int bits)
//   [1] e1 = v1 - v0, w = |e1|
//   [2] e2 = v2 - v0, w = flags (int bits): RMN_TRI_SMOOTH, RMN_TRI_RENORM
// Shading data, 3 float4 each: vertex normals n0, n1, n2; [0].w = material.
#define RMN_TRI_SMOOTH 1  // area <= 1e-2: interpolated vertex normals (src/model.cpp:250-265)
#define RMN_TRI_RENORM 2  // calcSurfaceNormal's tangent frame is finite (src/model.cpp:279-298)
#define RMN_TRI_ALPHA 4   // the material is alpha-tested (Material::hasFullyTransparentPart)
// Texture coordinates of a scene with textures, 2 float4 per triangle in
// leaf order: (u0, v0, u1, v1), (u2, v2, -, -).

// Material (80 B): constant texels resolved, plus texture indices.
struct __align__(16) DevMat {
  float4 base;   // diffuse colour (white without a texel), w = roughness
  float4 emis;   // emission (0 without a texel), w = metallic
  float4 misc;   // opacity, ior, has emission, material id
  float4 trans;  // transmitting colour
  int4 tex;      // texture index per slot (diffuse, specular, emissive, normal map), -1 none
};

// Texture (ImageData, include/material.h:12-24): RGBA8 texels of all mip
// levels in one array; level l is (w >> l) x (h >> l) texels at byte off[l].
#define RMN_MIP_LEVELS 8  // MAX_MIPMAP_LEVEL, include/material.h:10
struct __align__(16) DevTex {
  int w, h, depth, pad;
  long long off[RMN_MIP_LEVELS];
};

// Light object (LightObject, include/component.h:47-54) and its faces.
struct __align__(16) DevLight {
  float4 center;  // xyz, w = power
  float4 color;   // xyz, w = face count (float)
  int first_face; // into light_faces / light_prefix
  int material;   // material of the emissive mesh
  int pad[2];
};
// Light face: 6 float4 -- v0, v1, v2 (w unused), n0, n1, n2.
#define RMN_LIGHT_FACE_F4 6

struct DevScene {
  const DevNode* nodes;
  const float4* tri;
  const float4* shade;
  const DevMat* mats;
  const DevLight* lights;
  const float4* light_faces;
  const float* light_prefix;
  const float4* sky;          // premultiplied texels (SkyBox::Init), w unused
  const float* sky_prefix;
  // guide table of the sky prefix sums: bucket k covers draws x in
  // [sky_gt[k], sky_gt[k+1]), whose lower_bound lies in [sky_gi[k], sky_gi[k+1]]
  const float* sky_gt;
  const int* sky_gi;
  int sky_gk;                 // buckets (0: no table)
  float sky_ginv;             // sky_gk / total, to guess the bucket
  int root;                   // root reference (inner index or leaf ref)
  int num_tris;
  int num_mats;
  int num_lights;
  int sky_w, sky_h;
  int depth;
  int has_glass;              // some material is transmissive or half-opaque (opacity <= 1 - 1e-4)
  // textures (scenes without any: null / 0)
  const float4* uv;           // 2 per triangle, leaf order
  const DevTex* texs;
  const uint8_t* texels;
  int has_tex;                // some material has a texture: textured shading with ray differentials
  int has_alpha;              // some material is alpha-tested: traversal retries past cut-away texels
};
