// Texture lookups of the reference's ImageData / Material
// (src/material.cpp:26-129, 335-383), shared by the host scene builder
// (light objects average their emissive texture) and the kernels.
//
// Texels are RGBA8. A lookup returns N = 4 channels (diffuse, specular,
// emissive) or N = 3 (normal maps); as in get_bilinear the byte stride of a
// texel is N, whatever the texture's channel count, so a 3-channel lookup
// of RGBA data reads the bytes the reference reads. Every float operation
// follows the reference's order; only log2 (level of detail) and pow (gamma
// 2.2) are library calls whose last bit may differ between CPU and GPU.
#pragma once
#include "rmn_internal.h"

#if defined(__CUDA_ARCH__)
#define RMN_POWF powf
#define RMN_LOG2F log2f
#else
#define RMN_POWF std::pow
#define RMN_LOG2F std::log2
#endif

// get_basic<vec3/vec4>: N bytes from p, each / 255.
template <int N>
RMN_HD float4 tex_basic(const uint8_t* p) {
#if defined(__CUDA_ARCH__)
  if (N == 4) {
    uchar4 c = __ldg(reinterpret_cast<const uchar4*>(p));
    return make_float4((float)c.x / 255.0f, (float)c.y / 255.0f, (float)c.z / 255.0f, (float)c.w / 255.0f);
  }
  return make_float4((float)__ldg(p) / 255.0f, (float)__ldg(p + 1) / 255.0f, (float)__ldg(p + 2) / 255.0f, 0.0f);
#else
  return make_float4((float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f,
                     N == 4 ? (float)p[3] / 255.0f : 0.0f);
#endif
}

RMN_HD float4 lerp4(float4 a, float wa, float4 b, float wb) {  // a * wa + b * wb, per channel
  return make_float4(a.x * wa + b.x * wb, a.y * wa + b.y * wb, a.z * wa + b.z * wb, a.w * wa + b.w * wb);
}

RMN_HD void tex_wrap(int& x, int m) {  // get_bilinear's _mod
  if (x < 0 || x >= m) {
    x %= m;
    if (x < 0) x += m;
  }
}

// get_bilinear, src/material.cpp:48-80: bilinear filter with wrap-around on
// one level of width x height texels.
template <int N>
RMN_HD float4 tex_bilinear(const uint8_t* d, int width, int height, float u, float v) {
  float x = u * float(width), y = v * float(height);
  int x0 = int(floorf(x)), y0 = int(floorf(y));
  float dx = x - float(x0), dy = y - float(y0);
  tex_wrap(x0, width);
  tex_wrap(y0, height);
  int x1 = (x0 + 1) % width, y1 = (y0 + 1) % height;
  float4 c00 = tex_basic<N>(d + ((size_t)y0 * width + x0) * N);
  float4 c01 = tex_basic<N>(d + ((size_t)y0 * width + x1) * N);
  float4 c10 = tex_basic<N>(d + ((size_t)y1 * width + x0) * N);
  float4 c11 = tex_basic<N>(d + ((size_t)y1 * width + x1) * N);
  float4 c0 = lerp4(c00, 1.0f - dx, c01, dx);
  float4 c1 = lerp4(c10, 1.0f - dx, c11, dx);
  return lerp4(c0, 1.0f - dy, c1, dy);
}

// ImageData::get, src/material.cpp:82-94: v flipped, the level clamped to
// [0, depth - 1] and two levels blended. A blend of 0 returns the first
// level's texel exactly (texels are finite), so its second lookup is skipped.
template <int N>
RMN_HD float4 tex_get(const DevTex& t, const uint8_t* texels, float u, float v, float dep) {
  v = 1.0f - v;
  const float top = static_cast<float>(t.depth - 1);
  dep = top < dep ? top : dep;   // std::min(depth, map_depth - 1)
  dep = dep < 0.0f ? 0.0f : dep; // std::max(..., 0.0f)
  int level = static_cast<int>(dep);
  int next = level + 1 < t.depth - 1 ? level + 1 : t.depth - 1;
  float blend = dep - float(level);
  float4 a = tex_bilinear<N>(texels + t.off[level], t.w >> level, t.h >> level, u, v);
  if (blend == 0.0f) return a;
  float4 b = tex_bilinear<N>(texels + t.off[next], t.w >> next, t.h >> next, u, v);
  return lerp4(a, 1.0f - blend, b, blend);
}

// Level of detail of Material::get*Color: log2(duv * width), duv = NaN -> 0.
RMN_HD float tex_level(const DevTex& t, float duv) {
  return duv != duv ? 0.0f : RMN_LOG2F(duv * float(t.w));
}

// gammaPow, src/material.cpp:335-346.
RMN_HD float3 tex_gamma(float4 c) {
  const float g = 2.2f;
  return f3(RMN_POWF(c.x, g), RMN_POWF(c.y, g), RMN_POWF(c.z, g));
}
