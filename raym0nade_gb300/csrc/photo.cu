// Photo's post passes beside compose and FXAA (src/image.cpp:30-356):
// spatialClamp, the a-trous filter, bloom and the depth-of-field blur, on
// the device, each pass restating the reference's float operations in the
// reference's order.
//
//  * spatialClamp: a row kernel (7-tap blur of luminance) and a column kernel
//    (7-tap blur, clamp in place), the four buffers in one grid (z).
//  * filter: filterVar and five a-trous passes, ping-ponging between the
//    caller's buffers and a scratch copy (the sixth write lands back in the
//    caller's); the G-buffer fields the edge-stopping weight reads are packed
//    once into 48 bytes per pixel.
//  * bloom: the bright part, then five a-trous passes, each adding its
//    result to the image (ping-pong scratch).
//  * depth of field: the reference scatters pixels in stable depth order and
//    every receiving pixel stops taking weight at 0.99, so what a pixel
//    receives depends on the order of its senders. That order is per
//    receiver: the blur is a gather in which each receiver folds its
//    senders in the reference's order. The pixels of each tile of T x T
//    pixels (T >= the largest radius) are listed in that order with a sort
//    key; a receiver merges the lists of its 3 x 3 tiles by key, so it meets
//    every sender that can reach it, in order (a block per tile first keeps
//    the senders whose square reaches the tile and merges them once, so a
//    receiver only walks its tile's candidates). Without NaN depths a stable
//    sort by depth is the order by (depth, raster index), whose key is
//    (depth bits, index): each tile ranks its own pixels on the device. A
//    NaN depth (a pixel without a hit) compares false both ways in the
//    reference's comparator, so its place depends on std::stable_sort's
//    algorithm: then the host runs that very sort and the key is the rank.
//    A plan (order, radii, weights) serves every blur of the same G-buffer.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rmn_host.h"

namespace {

constexpr float kLumR = 0.3f, kLumG = 0.6f, kLumB = 0.1f;
__device__ __forceinline__ float lum3(float3 v) { return dot3(v, f3(kLumR, kLumG, kLumB)); }
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }

// ------------------------------------------------------- spatialClamp -----
__constant__ float c_h7[7] = {0.03125f, 0.109375f, 0.21875f, 0.28125f, 0.21875f, 0.109375f, 0.03125f};

struct Bufs {
  float4* b[4];  // Dd, Ds, Id, Is (radiance, Var)
};

__global__ void clamp_rows_kernel(Bufs in, float* __restrict__ b1, int W, int H) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= W) return;
  const float4* r = in.b[z] + (size_t)y * W;
  float sum = 0.0f;
  for (int dx = -3; dx <= 3; ++dx) {
    int nx = x + dx;
    if (nx >= 0 && nx < W) sum += lum3(xyz(r[nx])) * c_h7[dx + 3];
  }
  b1[(size_t)z * W * H + (size_t)y * W + x] = sum;
}

__global__ void clamp_cols_kernel(Bufs io, const float* __restrict__ b1, int W, int H) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= W) return;
  const float* c = b1 + (size_t)z * W * H;
  float sum = 0.0f;
  for (int dy = -3; dy <= 3; ++dy) {
    int ny = y + dy;
    if (ny >= 0 && ny < H) sum += c[(size_t)ny * W + x] * c_h7[dy + 3];
  }
  float4& p = io.b[z][(size_t)y * W + x];
  const float l = lum3(xyz(p));
  const float h3 = c_h7[3];
  const float bl = sum - h3 * h3 * l;
  if (l > 36.0f * bl) {
    const float s = bl / (l + RMN_EPS) / (1.0f - h3 * h3);
    p.x *= s;
    p.y *= s;
    p.z *= s;
  }
}

// ------------------------------------------------------------- filter -----
// Guide record of a pixel for the edge-stopping weight (48 B):
// (position, metallic), (surface normal, opacity), (shape normal, roughness).
__global__ void guide_kernel(const float* __restrict__ gbuf, float4* __restrict__ guide, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* g = gbuf + (size_t)RMN_GBUFFER_FLOATS * i;
  guide[3 * (size_t)i] = make_float4(g[6], g[7], g[8], g[16]);
  guide[3 * (size_t)i + 1] = make_float4(g[12], g[13], g[14], g[17]);
  guide[3 * (size_t)i + 2] = make_float4(g[9], g[10], g[11], g[15]);
}

// filterVar, src/image.cpp:84-108.
__global__ void filter_var_kernel(Bufs in, Bufs out, int W, int H) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= W) return;
  const float h[3] = {0.25f, 0.5f, 0.25f};
  const float4* r = in.b[z];
  float3 E = f3(0.0f);
  float E2 = 0.0f, V = 0.0f;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      int nx = x + dx, ny = y + dy;
      if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
      const float4 q = r[(size_t)ny * W + nx];
      const float wt = h[dx + 1] * h[dy + 1];
      E += xyz(q) * wt;
      E2 += dot3(xyz(q), xyz(q)) * wt;
      V += q.w * wt;
    }
  const size_t i = (size_t)y * W + x;
  const float4 p = r[i];
  out.b[z][i] = make_float4(p.x, p.y, p.z, V + E2 - dot3(E, E));
}

// getWeight, src/image.cpp:110-158 (sigma_z = sigma_l = sigma_m = 1,
// sigma_n = 1024, eps 1e-2, eps_r 4e-2; every pixel's specular is the
// HitInfo default 0.04, so its difference is 0).
__device__ __forceinline__ float edge_weight(const float4* __restrict__ guide, size_t ip, size_t iq, float4 Lp,
                                             float4 Lq, bool specular) {
  const float4 q0 = guide[3 * iq], q1 = guide[3 * iq + 1];
  if (!any_finite3(xyz(q0))) return 0.0f;
  const float4 p0 = guide[3 * ip], p1 = guide[3 * ip + 1], p2 = guide[3 * ip + 2];
  const float d = dot3(xyz(p1), xyz(q1));
  float w = powf(0.0f < d ? d : 0.0f, 1024.0f);
  if (w < 1e-6f) return 0.0f;
  float k = 0.0f;
  const float3 dir = norm3(xyz(q0) - xyz(p0));
  const float st = fabsf(dot3(xyz(p2), dir));
  const float tt = st / (sqrtf(1.0f - st * st) + RMN_EPS);
  k += -tt / 1.0f;
  const float rd = len3(xyz(Lp) - xyz(Lq)) / (1.0f * sqrtf(Lp.w) + 1e-2f);
  k += -rd;
  const float md = len3(f3(p0.w - q0.w, 0.04f - 0.04f, p1.w - q1.w));
  k += -md / 1.0f;
  if (k < -7.5f) return 0.0f;
  w *= expf(k);
  if (specular) w *= p2.w < 4e-2f ? 4e-2f : p2.w;
  if (!isfinite(w)) return 0.0f;
  return w;
}

// filterRadiance(..., step), src/image.cpp:160-199.
__global__ void filter_pass_kernel(Bufs in, Bufs out, const float4* __restrict__ guide, int W, int H, int step) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= W) return;
  const float h[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  const bool specular = (z & 1) != 0;  // Ds, Is
  const float4* r = in.b[z];
  const size_t i = (size_t)y * W + x;
  float3 rb = f3(0.0f);
  float vb = 0.0f;
  if (any_finite3(xyz(guide[3 * i]))) {
    const float4 Lp = r[i];
    float ws = 0.0f;
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        int nx = x + dx * step, ny = y + dy * step;
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        float wt = h[dx + 2] * h[dy + 2];
        const size_t j = (size_t)ny * W + nx;
        const float4 Lq = r[j];
        if (dx != 0 || dy != 0) wt *= edge_weight(guide, i, j, Lp, Lq, specular);
        ws += wt;
        rb += xyz(Lq) * wt;
        vb += Lq.w * wt * wt;
      }
    rb = rb / ws;
    vb /= ws * ws;
  }
  out.b[z][i] = make_float4(rb.x, rb.y, rb.z, vb);
}

// --------------------------------------------------------------- bloom ----
__global__ void bloom_init_kernel(const float* __restrict__ rgb, float3* __restrict__ bc, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 p = f3(rgb[3 * (size_t)i], rgb[3 * (size_t)i + 1], rgb[3 * (size_t)i + 2]);
  const float c = lum3(p);
  float3 b = f3(0.0f);
  if (!(c < 1.0f)) {
    b = p / powf(c, 0.65f);
    b.x = b.x - 1.0f < 0.0f ? 0.0f : b.x - 1.0f;  // std::max(v - 1, 0)
    b.y = b.y - 1.0f < 0.0f ? 0.0f : b.y - 1.0f;
    b.z = b.z - 1.0f < 0.0f ? 0.0f : b.z - 1.0f;
  }
  bc[i] = b;
}

// One bloom pass: out = blur(in, step); rgb += out / 6.
__global__ void bloom_pass_kernel(const float3* __restrict__ in, float3* __restrict__ out, float* __restrict__ rgb,
                                  int W, int H, int step) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const float h[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  float3 col = f3(0.0f);
  for (int ky = -2; ky <= 2; ++ky)
    for (int kx = -2; kx <= 2; ++kx) {
      int nx = x + kx * step, ny = y + ky * step;
      if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
      col += in[(size_t)ny * W + nx] * h[ky + 2] * h[kx + 2];
    }
  const size_t i = (size_t)y * W + x;
  out[i] = col;
  const float3 a = col / 6.0f;
  rgb[3 * i] += a.x;
  rgb[3 * i + 1] += a.y;
  rgb[3 * i + 2] += a.z;
}

// ----------------------------------------------------- depth of field -----
// float -> int of the radii: truncation, 0 for NaN (CUDA's and aarch64's
// conversion; in C++ the conversion of NaN is undefined).
__host__ __device__ __forceinline__ int dof_int(float v) {
  if (v != v) return 0;
  if (v >= 2147483647.0f) return 2147483647;
  if (v <= -2147483648.0f) return (-2147483647 - 1);
  return (int)v;
}
__host__ __device__ __forceinline__ float dof_coc(float coc, float focus, float depth) {
  const float c = coc * fabsf(1.0f - focus / depth) + RMN_EPS;
  return 96.0f < c ? 96.0f : c;  // std::min(..., MaxCoC)
}

// depth = length(position - camera); flags[0] |= a NaN depth.
__global__ void depth_kernel(const float* __restrict__ gbuf, float3 cam, float* __restrict__ depth, int n,
                             int* __restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* g = gbuf + (size_t)RMN_GBUFFER_FLOATS * i;
  const float d = len3(f3(g[6], g[7], g[8]) - cam);
  depth[i] = d;
  if (d != d) atomicOr(&flags[0], 1);
}

// Per sending pixel: CoC0, its total weight (the reference's two loops per
// row, inwards from the disc's edge until a weight reaches 1), radius.
// flags[1] = max radius.
__global__ void dof_source_kernel(const float* __restrict__ depth, float coc, float focus, float4* __restrict__ src,
                                  int n, int* __restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float c0 = dof_coc(coc, focus, depth[i]);
  const int radius = dof_int(c0);
  atomicMax(&flags[1], radius);
  float tw = 0.0f;
  for (int dy = -radius; dy <= radius; ++dy) {
    const int xlen = dof_int(sqrtf(c0 * c0 - (float)(dy * dy)));
    int xl, xr;
    for (xl = -xlen; xl <= 0; xl++) {
      float w = c0 - sqrtf((float)(xl * xl + dy * dy));
      w = 1.0f < w ? 1.0f : w;
      if (w == 1.0f) break;
      tw += w;
    }
    for (xr = xlen; xr > 0; xr--) {
      float w = c0 - sqrtf((float)(xr * xr + dy * dy));
      w = 1.0f < w ? 1.0f : w;
      if (w == 1.0f) break;
      tw += w;
    }
    tw += (float)(xr - xl + 1);
  }
  src[i] = make_float4(c0, tw, __int_as_float(radius), 0.0f);
}

// Tile t = (tx, ty) of a T-grid covers x in [tx T, min(W, tx T + T)) and
// likewise y; its list occupies [tile_start[t], tile_start[t + 1]).
__global__ void dof_rank_kernel(const float* __restrict__ depth, const int* __restrict__ tile_start, int W, int H,
                                int T, int TW, unsigned long long* __restrict__ key, int* __restrict__ pix) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const int tx = x / T, ty = y / T;
  const int x0 = tx * T, y0 = ty * T, x1 = min(W, x0 + T), y1 = min(H, y0 + T);
  const int p = y * W + x;
  const unsigned long long kp = ((unsigned long long)__float_as_uint(depth[p]) << 32) | (unsigned)p;
  int rank = 0;
  for (int qy = y0; qy < y1; ++qy)
    for (int qx = x0; qx < x1; ++qx) {
      const int q = qy * W + qx;
      const unsigned long long kq = ((unsigned long long)__float_as_uint(depth[q]) << 32) | (unsigned)q;
      rank += kq < kp ? 1 : 0;
    }
  const int slot = tile_start[ty * TW + tx] + rank;
  key[slot] = kp;
  pix[slot] = p;
}

// Per receiving tile: the senders of its 3 x 3 tiles whose square of
// half-width radius touches the tile, in the reference's order. A block per
// tile compacts each neighbour list (order kept) into `tmp`, then places every
// survivor at its rank in the merged order: its index in its own list plus,
// for every other list, the number of survivors with a smaller key.
constexpr int kCandThreads = 256;

__device__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kCandThreads / 32 ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kCandThreads / 32) warp_sums[lane] = w;  // inclusive
  }
  __syncthreads();
  const int before = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
  total = warp_sums[kCandThreads / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kCandThreads) dof_candidates_kernel(
    const float4* __restrict__ src, const int* __restrict__ tile_start, const unsigned long long* __restrict__ key,
    const int* __restrict__ pix, const long long* __restrict__ cand_off, int W, int H, int T, int TW, int TH,
    unsigned long long* __restrict__ tmp_key, int* __restrict__ tmp_pix, int* __restrict__ cand,
    int* __restrict__ cand_count) {
  __shared__ int warp_sums[kCandThreads / 32];
  __shared__ int lst_begin[9], lst_len[9];
  const int t = blockIdx.x, tx = t % TW, ty = t / TW;
  const int x0 = tx * T, y0 = ty * T, x1 = min(W, x0 + T) - 1, y1 = min(H, y0 + T) - 1;
  const long long base = cand_off[t];
  int nl = 0, filled = 0;
  for (int j = ty - 1; j <= ty + 1; ++j)
    for (int i = tx - 1; i <= tx + 1; ++i) {
      if (i < 0 || i >= TW || j < 0 || j >= TH) continue;
      const int u = j * TW + i, b = tile_start[u], len = tile_start[u + 1] - b;
      int kept = 0;
      for (int c0 = 0; c0 < len; c0 += kCandThreads) {
        const int c = c0 + threadIdx.x;
        bool keep = false;
        int s = 0;
        if (c < len) {
          s = pix[b + c];
          const int sx = s % W, sy = s / W, r = __float_as_int(src[s].z);
          keep = sx - r <= x1 && sx + r >= x0 && sy - r <= y1 && sy + r >= y0;
        }
        int total;
        const int at = block_exclusive_scan(keep ? 1 : 0, warp_sums, total);
        if (keep) {
          tmp_key[base + filled + kept + at] = key[b + c];
          tmp_pix[base + filled + kept + at] = s;
        }
        kept += total;
      }
      if (threadIdx.x == 0) {
        lst_begin[nl] = filled;
        lst_len[nl] = kept;
      }
      filled += kept;
      ++nl;
    }
  __syncthreads();
  for (int c = threadIdx.x; c < filled; c += kCandThreads) {
    const unsigned long long k = tmp_key[base + c];
    int rank = 0;
    for (int l = 0; l < nl; ++l) {
      const int b = lst_begin[l], len = lst_len[l];
      if (c >= b && c < b + len) {
        rank += c - b;
        continue;
      }
      int lo = 0, hi = len;  // survivors of list l with a smaller key
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (tmp_key[base + b + mid] < k) lo = mid + 1;
        else hi = mid;
      }
      rank += lo;
    }
    cand[base + rank] = tmp_pix[base + c];
  }
  if (threadIdx.x == 0) cand_count[t] = filled;
}

// The receiving pixel (x, y): its tile's candidates, in order.
__global__ void dof_fold_kernel(const float* __restrict__ rgb, const float4* __restrict__ src,
                                const long long* __restrict__ cand_off, const int* __restrict__ cand,
                                const int* __restrict__ cand_count, int W, int H, int T, int TW,
                                float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const int t = (y / T) * TW + x / T;
  const int* c = cand + cand_off[t];
  const int n = cand_count[t];
  float3 blur = f3(0.0f);
  float gained = 0.0f;
  for (int k = 0; k < n; ++k) {
    const int s = c[k];
    const int sx = s % W, sy = s / W;
    const int dx = x - sx, dy = y - sy;
    const float4 sv = src[s];
    const int radius = __float_as_int(sv.z);
    if (dy < -radius || dy > radius) continue;
    const float c0 = sv.x;
    const int xlen = dof_int(sqrtf(c0 * c0 - (float)(dy * dy)));
    if (dx < -xlen || dx > xlen) continue;
    float w = c0 - sqrtf((float)(dx * dx + dy * dy));
    w = (1.0f < w ? 1.0f : w) / sv.y;
    if (w < RMN_EPS) continue;
    if (gained + w > 0.99f) w = 0.99f - gained;
    if (w < RMN_EPS) continue;
    blur += f3(rgb[3 * (size_t)s], rgb[3 * (size_t)s + 1], rgb[3 * (size_t)s + 2]) * w;
    gained += w;
  }
  const float3 o = blur / gained;
  const size_t i = (size_t)y * W + x;
  out[3 * i] = o.x;
  out[3 * i + 1] = o.y;
  out[3 * i + 2] = o.z;
}

__global__ void gamma_kernel(float* __restrict__ rgb, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 p = f3(rgb[3 * (size_t)i], rgb[3 * (size_t)i + 1], rgb[3 * (size_t)i + 2]);
  p = max3(p, f3(0.0f));
  const float c = lum3(p);
  if (c > 0.75f) p = p / c * (tanhf(3.0f * (c - 0.75f)) / 3.0f + 0.75f);
  p = min3(p, f3(1.0f));
  const float e = 1.0f / 2.2f;
  rgb[3 * (size_t)i] = powf(p.x, e);
  rgb[3 * (size_t)i + 1] = powf(p.y, e);
  rgb[3 * (size_t)i + 2] = powf(p.z, e);
}

struct DevScratch {
  std::vector<void*> ptrs;
  cudaStream_t st;
  cudaError_t err = cudaSuccess;
  template <class T>
  T* get(size_t count) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = rmn::staging_malloc(&p, count * sizeof(T) + 16, st);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~DevScratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
};

dim3 row_grid(int W, int H, int z = 1) { return dim3((W + 127) / 128, H, z); }

}  // namespace

namespace rmn {

cudaError_t launch_spatial_clamp(float* const bufs[4], int W, int H, cudaStream_t st) {
  DevScratch sc{{}, st};
  float* b1 = sc.get<float>((size_t)4 * W * H);
  if (sc.err != cudaSuccess) return sc.err;
  Bufs b;
  for (int k = 0; k < 4; ++k) b.b[k] = reinterpret_cast<float4*>(bufs[k]);
  clamp_rows_kernel<<<row_grid(W, H, 4), 128, 0, st>>>(b, b1, W, H);
  clamp_cols_kernel<<<row_grid(W, H, 4), 128, 0, st>>>(b, b1, W, H);
  return cudaGetLastError();
}

cudaError_t launch_filter(float* const bufs[4], const float* gbuf, int W, int H, cudaStream_t st) {
  const size_t n = (size_t)W * H;
  DevScratch sc{{}, st};
  float4* guide = sc.get<float4>(3 * n);
  float4* tmp = sc.get<float4>(4 * n);
  if (sc.err != cudaSuccess) return sc.err;
  Bufs A, B;
  for (int k = 0; k < 4; ++k) {
    A.b[k] = reinterpret_cast<float4*>(bufs[k]);
    B.b[k] = tmp + k * n;
  }
  guide_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(gbuf, guide, (int)n);
  filter_var_kernel<<<row_grid(W, H, 4), 128, 0, st>>>(A, B, W, H);
  // passes of step 1, 2, 4, 8, 16: B -> A -> B -> A -> B -> A
  bool toA = true;
  for (int step = 1; step <= 16; step *= 2) {
    if (toA) filter_pass_kernel<<<row_grid(W, H, 4), 128, 0, st>>>(B, A, guide, W, H, step);
    else filter_pass_kernel<<<row_grid(W, H, 4), 128, 0, st>>>(A, B, guide, W, H, step);
    toA = !toA;
  }
  return cudaGetLastError();
}

cudaError_t launch_bloom(float* rgb, int W, int H, cudaStream_t st) {
  const size_t n = (size_t)W * H;
  DevScratch sc{{}, st};
  float3* a = sc.get<float3>(n);
  float3* b = sc.get<float3>(n);
  if (sc.err != cudaSuccess) return sc.err;
  bloom_init_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rgb, a, (int)n);
  for (int step = 1; step <= 16; step *= 2) {
    bloom_pass_kernel<<<row_grid(W, H), 128, 0, st>>>(a, b, rgb, W, H, step);
    std::swap(a, b);
  }
  return cudaGetLastError();
}

struct DofPlan {
  int W = 0, H = 0, T = 0, TW = 0, TH = 0;
  float4* src = nullptr;
  int* tile_start = nullptr;
  unsigned long long* key = nullptr;
  int* pix = nullptr;
  // per receiving tile: its candidate senders in order
  long long* cand_off = nullptr;
  int* cand = nullptr;
  int* cand_count = nullptr;
  float* out = nullptr;
  std::vector<void*> allocs;
};

void dof_plan_destroy(DofPlan* p, cudaStream_t st) {
  if (!p) return;
  for (void* a : p->allocs) cudaFreeAsync(a, st);
  delete p;
}

// Order, radii and weights of the depth-of-field blur of one G-buffer and
// camera. Synchronises `st` (the tile size depends on the largest radius).
cudaError_t dof_plan_create(const float* gbuf, int W, int H, float focus, float coc, const float cam[3],
                            cudaStream_t st, DofPlan** out) {
  *out = nullptr;
  const int n = W * H;
  DofPlan* p = new DofPlan();
  p->W = W;
  p->H = H;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](size_t bytes) -> void* {
    void* q = nullptr;
    if (e == cudaSuccess) e = rmn::staging_malloc(&q, bytes + 16, st);
    if (e == cudaSuccess) p->allocs.push_back(q);
    return e == cudaSuccess ? q : nullptr;
  };
  float* depth = static_cast<float*>(alloc(sizeof(float) * n));
  int* flags = static_cast<int*>(alloc(2 * sizeof(int)));
  p->src = static_cast<float4*>(alloc(sizeof(float4) * n));
  p->key = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long) * n));
  p->pix = static_cast<int*>(alloc(sizeof(int) * n));
  p->out = static_cast<float*>(alloc(sizeof(float) * 3 * n));
  int hflags[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess) {
    depth_kernel<<<(n + 255) / 256, 256, 0, st>>>(gbuf, f3(cam[0], cam[1], cam[2]), depth, n, flags);
    dof_source_kernel<<<(n + 255) / 256, 256, 0, st>>>(depth, coc, focus, p->src, n, flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hflags, flags, sizeof hflags, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    dof_plan_destroy(p, st);
    return e;
  }
  p->T = std::max(hflags[1], 8);
  p->TW = (W + p->T - 1) / p->T;
  p->TH = (H + p->T - 1) / p->T;
  std::vector<int> tile_start((size_t)p->TW * p->TH + 1, 0);
  for (int ty = 0; ty < p->TH; ++ty)
    for (int tx = 0; tx < p->TW; ++tx) {
      const int w = std::min(W, tx * p->T + p->T) - tx * p->T, h = std::min(H, ty * p->T + p->T) - ty * p->T;
      tile_start[(size_t)ty * p->TW + tx + 1] = w * h;
    }
  for (size_t t = 0; t + 1 < tile_start.size(); ++t) tile_start[t + 1] += tile_start[t];
  p->tile_start = static_cast<int*>(alloc(sizeof(int) * tile_start.size()));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p->tile_start, tile_start.data(), sizeof(int) * tile_start.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !hflags[0]) {
    dof_rank_kernel<<<row_grid(W, H), 128, 0, st>>>(depth, p->tile_start, W, H, p->T, p->TW, p->key, p->pix);
    e = cudaGetLastError();
  } else if (e == cudaSuccess) {
    // NaN depths: the reference's own std::stable_sort decides the order
    std::vector<float> hd(n);
    e = cudaMemcpyAsync(hd.data(), depth, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
      struct PixelPos {
        int x, y;
        float depth;
      };
      std::vector<PixelPos> pixs;
      pixs.reserve(n);
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) pixs.push_back({x, y, hd[(size_t)y * W + x]});
      std::stable_sort(pixs.begin(), pixs.end(),
                       [](const PixelPos& a, const PixelPos& b) { return a.depth < b.depth; });
      std::vector<unsigned long long> hkey(n);
      std::vector<int> hpix(n);
      std::vector<int> fill(tile_start.begin(), tile_start.end() - 1);
      for (int r = 0; r < n; ++r) {  // ranks ascend within each tile
        const PixelPos& q = pixs[r];
        const int slot = fill[(size_t)(q.y / p->T) * p->TW + q.x / p->T]++;
        hkey[slot] = (unsigned long long)r;
        hpix[slot] = q.y * W + q.x;
      }
      e = cudaMemcpyAsync(p->key, hkey.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(p->pix, hpix.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host vectors go out of scope
    }
  }
  // candidate lists: capacity of tile t = the pixels of its 3 x 3 tiles
  const size_t ntiles = (size_t)p->TW * p->TH;
  std::vector<long long> cand_off(ntiles + 1, 0);
  for (int ty = 0; ty < p->TH; ++ty)
    for (int tx = 0; tx < p->TW; ++tx) {
      long long cap = 0;
      for (int j = ty - 1; j <= ty + 1; ++j)
        for (int i = tx - 1; i <= tx + 1; ++i)
          if (i >= 0 && i < p->TW && j >= 0 && j < p->TH) {
            const size_t u = (size_t)j * p->TW + i;
            cap += tile_start[u + 1] - tile_start[u];
          }
      cand_off[(size_t)ty * p->TW + tx + 1] = cap;
    }
  for (size_t t = 0; t < ntiles; ++t) cand_off[t + 1] += cand_off[t];
  const size_t total = (size_t)cand_off[ntiles];
  p->cand_off = static_cast<long long*>(alloc(sizeof(long long) * (ntiles + 1)));
  p->cand = static_cast<int*>(alloc(sizeof(int) * total));
  p->cand_count = static_cast<int*>(alloc(sizeof(int) * ntiles));
  unsigned long long* tmp_key = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long) * total));
  int* tmp_pix = static_cast<int*>(alloc(sizeof(int) * total));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p->cand_off, cand_off.data(), sizeof(long long) * (ntiles + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    dof_candidates_kernel<<<(unsigned)ntiles, kCandThreads, 0, st>>>(p->src, p->tile_start, p->key, p->pix,
                                                                     p->cand_off, W, H, p->T, p->TW, p->TH, tmp_key,
                                                                     tmp_pix, p->cand, p->cand_count);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host arrays were copied from
  if (e != cudaSuccess) {
    dof_plan_destroy(p, st);
    return e;
  }
  *out = p;
  return cudaSuccess;
}

// Photo::depthFeildBlur in place on rgb (device) with a plan of its G-buffer.
cudaError_t dof_apply(const DofPlan* p, float* rgb, cudaStream_t st) {
  dim3 grid((p->W + 15) / 16, (p->H + 15) / 16), block(16, 16);
  dof_fold_kernel<<<grid, block, 0, st>>>(rgb, p->src, p->cand_off, p->cand, p->cand_count, p->W, p->H, p->T, p->TW,
                                          p->out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rgb, p->out, sizeof(float) * 3 * (size_t)p->W * p->H, cudaMemcpyDeviceToDevice, st);
  return e;
}

cudaError_t launch_dof(float* rgb, const float* gbuf, int W, int H, float focus, float coc, const float cam[3],
                       cudaStream_t st) {
  DofPlan* p = nullptr;
  cudaError_t e = dof_plan_create(gbuf, W, H, focus, coc, cam, st, &p);
  if (e != cudaSuccess) return e;
  e = dof_apply(p, rgb, st);
  dof_plan_destroy(p, st);
  return e;
}

cudaError_t launch_gamma(float* rgb, int n, cudaStream_t st) {
  gamma_kernel<<<(n + 255) / 256, 256, 0, st>>>(rgb, n);
  return cudaGetLastError();
}

}  // namespace rmn
