// Post passes over the render buffers: Photo::shade + gammaCorrection
// (src/image.cpp:215-246, 454-468) and Photo::FXAA (src/image.cpp:358-452).
//
// FXAA reads, per output pixel, its 3x3 luminance neighbourhood and up to 12
// samples marching in +x or +y (never negative: the step is
// clamp(edge / range, -2, 2) of two non-negative numbers). The reference's
// step length is 1/width for a horizontal edge but is applied along y, and
// 1/height along x for a vertical one, so the march reaches at most
// 24 * H / W rows or 24 * W / H columns. A block computes luminance for its
// 32 x 8 tile plus that halo once into shared memory (luma is the only
// per-sample quantity the march needs) and fetches the colour of the winning
// sample once at the end. Samples outside the staged halo are read from
// global memory, so the result does not depend on the halo size.
#include <algorithm>
#include <cmath>

#include "rmn_host.h"

namespace {

constexpr int TX = 32, TY = 8, HALO_LO = 1;

__device__ __forceinline__ float luma3(const float* p) { return p[0] * 0.3f + p[1] * 0.6f + p[2] * 0.1f; }

__global__ void __launch_bounds__(TX* TY) fxaa_kernel(const float* __restrict__ in, float* __restrict__ out, int W,
                                                       int H, int SW, int SH) {
  extern __shared__ float lum_s[];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.y * TX + threadIdx.x;
  for (int k = tid; k < SW * SH; k += TX * TY) {
    int ly = k / SW, lx = k % SW;
    int gx = min(max(x0 - HALO_LO + lx, 0), W - 1), gy = min(max(y0 - HALO_LO + ly, 0), H - 1);
    lum_s[k] = luma3(in + 3 * ((size_t)gy * W + gx));
  }
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= W || y >= H) return;
  auto L = [&](int gx, int gy) -> float {
    int lx = gx - x0 + HALO_LO, ly = gy - y0 + HALO_LO;
    if (lx >= 0 && lx < SW && ly >= 0 && ly < SH) return lum_s[ly * SW + lx];
    return luma3(in + 3 * ((size_t)gy * W + gx));
  };
  const float* c = in + 3 * ((size_t)y * W + x);
  float cr = c[0], cg = c[1], cb = c[2];
  float M = L(x, y);
  float N = y > 0 ? L(x, y - 1) : M, S = y < H - 1 ? L(x, y + 1) : M;
  float E = x < W - 1 ? L(x + 1, y) : M, Wl = x > 0 ? L(x - 1, y) : M;
  float lo = fminf(fminf(N, S), fminf(E, Wl)), hi = fmaxf(fmaxf(N, S), fmaxf(E, Wl));
  float range = hi - lo;
  float* o = out + 3 * ((size_t)y * W + x);
  if (range < fmaxf(0.0312f, hi * 0.125f)) {
    o[0] = cr; o[1] = cg; o[2] = cb;
    return;
  }
  float NW = (y > 0 && x > 0) ? L(x - 1, y - 1) : M;
  float NE = (y > 0 && x < W - 1) ? L(x + 1, y - 1) : M;
  float SW_ = (y < H - 1 && x > 0) ? L(x - 1, y + 1) : M;
  float SE = (y < H - 1 && x < W - 1) ? L(x + 1, y + 1) : M;
  float eh = fabsf((NW + Wl + SW_) - (NE + E + SE)) * (1.0f / 3.0f);
  float ev = fabsf((NW + N + NE) - (SW_ + S + SE)) * (1.0f / 3.0f);
  bool horiz = eh >= ev;
  float step = horiz ? 1.0f / float(W) : 1.0f / float(H);
  float g = (horiz ? eh : ev) / range;
  g = g < -2.0f ? -2.0f : (2.0f < g ? 2.0f : g);
  float ux = float(x) / float(W), uy = float(y) / float(H);
  float best = 0.0f;
  int bx = x, by = y;
  for (int i = 0; i < 12; ++i) {
    float off = g * step * float(i + 1);
    float sx_f = ux + (horiz ? 0.0f : off), sy_f = uy + (horiz ? off : 0.0f);
    if (sx_f < 0.0f || sx_f > 1.0f || sy_f < 0.0f || sy_f > 1.0f) continue;
    int sx = min(max((int)(sx_f * float(W)), 0), W - 1);
    int sy = min(max((int)(sy_f * float(H)), 0), H - 1);
    float d = fabsf(L(sx, sy) - M);
    if (d > best) {
      best = d;
      bx = sx;
      by = sy;
    }
  }
  const float* f = in + 3 * ((size_t)by * W + bx);
  float sub = fminf((fabsf(N + S - 2.0f * M) * 2.0f + fabsf(E + Wl - 2.0f * M)) * 0.25f, 1.0f);
  float a = sub * 0.75f;
  o[0] = cr * (1.0f - a) + f[0] * a;
  o[1] = cg * (1.0f - a) + f[1] * a;
  o[2] = cb * (1.0f - a) + f[2] * a;
}

__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

__global__ void compose_kernel(const float4* __restrict__ dd, const float4* __restrict__ ds,
                               const float4* __restrict__ id, const float4* __restrict__ is,
                               const float* __restrict__ gbuf, int n, float exposure, int opt, float* __restrict__ rgb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* g = gbuf + (size_t)RMN_GBUFFER_FLOATS * i;
  float3 p;
  if (opt & 64) {
    p = (ld3(g + 9) + f3(1.0f)) / 2.0f;
  } else if (opt & 128) {
    p = (ld3(g + 12) + f3(1.0f)) / 2.0f;
  } else {
    float3 rd = f3(0.0f), rs = f3(0.0f);
    if (opt & RMN_SHADE_DIRECT) {
      if (opt & RMN_SHADE_DIFFUSE) rd += f3(dd[i]);
      if (opt & RMN_SHADE_SPECULAR) rs += f3(ds[i]);
    }
    if (opt & RMN_SHADE_INDIRECT) {
      if (opt & RMN_SHADE_DIFFUSE) rd += f3(id[i]);
      if (opt & RMN_SHADE_SPECULAR) rs += f3(is[i]);
    }
    if (!(opt & (RMN_SHADE_DIRECT | RMN_SHADE_INDIRECT))) rd = f3(1.0f);
    float3 dc = (opt & RMN_SHADE_BASECOLOR) ? ld3(g) : f3(1.0f);
    p = dc * rd + rs;
    if (opt & RMN_SHADE_EMISSION) p += ld3(g + 3) * exposure;
  }
  if (opt & RMN_SHADE_GAMMA) {
    p = max3(p, f3(0.0f));
    float c = dot3(p, f3(0.3f, 0.6f, 0.1f));
    if (c > 0.75f) p = p / c * (tanhf(3.0f * (c - 0.75f)) / 3.0f + 0.75f);
    p = min3(p, f3(1.0f));
    const float e = 1.0f / 2.2f;
    p = f3(powf(p.x, e), powf(p.y, e), powf(p.z, e));
  }
  rgb[3 * (size_t)i] = p.x;
  rgb[3 * (size_t)i + 1] = p.y;
  rgb[3 * (size_t)i + 2] = p.z;
}

}  // namespace

namespace rmn {

cudaError_t launch_fxaa(const float* in, float* out, int w, int h, cudaStream_t stream) {
  if (w <= 0 || h <= 0) return cudaSuccess;
  int hx = (int)std::ceil(24.0 * w / h) + 2, hy = (int)std::ceil(24.0 * h / w) + 2;
  hx = std::min(hx, 96);
  hy = std::min(hy, 96);
  int sw = TX + HALO_LO + hx, sh = TY + HALO_LO + hy;
  dim3 grid((w + TX - 1) / TX, (h + TY - 1) / TY), block(TX, TY);
  fxaa_kernel<<<grid, block, sizeof(float) * sw * sh, stream>>>(in, out, w, h, sw, sh);
  return cudaGetLastError();
}

cudaError_t launch_compose(const float* dd, const float* ds, const float* id, const float* is, const float* gbuf,
                           int w, int h, float exposure, int options, float* rgb, cudaStream_t stream) {
  int n = w * h;
  compose_kernel<<<(n + 255) / 256, 256, 0, stream>>>(
      reinterpret_cast<const float4*>(dd), reinterpret_cast<const float4*>(ds), reinterpret_cast<const float4*>(id),
      reinterpret_cast<const float4*>(is), gbuf, n, exposure, options, rgb);
  return cudaGetLastError();
}

}  // namespace rmn
