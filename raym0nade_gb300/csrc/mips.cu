// ImageData::generateMipmaps (src/material.cpp:107-129) on the device.
//
// Level l of a texture halves level l-1: each texel is the 2x2 box of the
// level above, per channel (a + b + c + d) / 4 truncated. The reference wraps
// the box's coordinates modulo the level above, but a box never reaches past
// it: with cw = pw >> 1 the box's columns are 2x and 2x + 1 <= 2 cw - 1 <=
// pw - 1 (rows alike), so the wrap is the identity and every box is four
// aligned 32-bit RGBA loads. One launch per level covers every texture that
// has it (blockIdx.y = texture), so a scene's chain costs at most seven
// launches in stream order; level 0 is uploaded, the rest built in HBM.
#include <algorithm>
#include <vector>

#include "rmn_host.h"

namespace {

struct MipJob {
  long long src, dst;  // byte offsets of level l-1 and level l in the texel array
  int pw;              // texels per row of level l-1
  int cw, ch;          // size of level l
  int pad;
};

__global__ void __launch_bounds__(256) mip_level_kernel(uint8_t* __restrict__ texels, const MipJob* __restrict__ jobs) {
  const MipJob j = jobs[blockIdx.y];
  const uint32_t* __restrict__ src = reinterpret_cast<const uint32_t*>(texels + j.src);
  uint32_t* __restrict__ dst = reinterpret_cast<uint32_t*>(texels + j.dst);
  const long long n = (long long)j.cw * j.ch;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / j.cw), x = (int)(i - (long long)y * j.cw);
    const size_t r0 = (size_t)(2 * y) * j.pw + 2 * x, r1 = r0 + j.pw;
    const uint32_t a = src[r0], b = src[r0 + 1], c = src[r1], d = src[r1 + 1];
    uint32_t out = 0;
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
      const uint32_t s = ((a >> k) & 255u) + ((b >> k) & 255u) + ((c >> k) & 255u) + ((d >> k) & 255u);
      out |= (s >> 2) << k;
    }
    dst[i] = out;
  }
}

}  // namespace

namespace rmn {

cudaError_t launch_build_mips(uint8_t* texels, const DevTex* tex, int ntex, cudaStream_t stream) {
  std::vector<MipJob> jobs;
  int first[RMN_MIP_LEVELS + 1] = {0};
  long long most[RMN_MIP_LEVELS] = {0};
  for (int l = 1; l < RMN_MIP_LEVELS; ++l) {
    first[l] = (int)jobs.size();
    for (int t = 0; t < ntex; ++t) {
      if (tex[t].depth <= l) continue;
      MipJob j{tex[t].off[l - 1], tex[t].off[l], tex[t].w >> (l - 1), tex[t].w >> l, tex[t].h >> l, 0};
      most[l] = std::max(most[l], (long long)j.cw * j.ch);
      jobs.push_back(j);
    }
  }
  first[RMN_MIP_LEVELS] = (int)jobs.size();
  if (jobs.empty()) return cudaSuccess;
  MipJob* djobs = nullptr;
  cudaError_t e = cudaMalloc(&djobs, jobs.size() * sizeof(MipJob));
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(djobs, jobs.data(), jobs.size() * sizeof(MipJob), cudaMemcpyHostToDevice, stream);
  for (int l = 1; l < RMN_MIP_LEVELS && e == cudaSuccess; ++l) {
    for (int k = first[l]; k < first[l + 1] && e == cudaSuccess; k += 65535) {  // gridDim.y <= 65535
      const int count = std::min(65535, first[l + 1] - k);
      const unsigned bx = (unsigned)std::min<long long>((most[l] + 255) / 256, 4096);
      mip_level_kernel<<<dim3(bx, count), 256, 0, stream>>>(texels, djobs + k);
      e = cudaGetLastError();
    }
  }
  const cudaError_t s = cudaStreamSynchronize(stream);  // the job table is freed below
  if (e == cudaSuccess) e = s;
  cudaFree(djobs);
  return e;
}

}  // namespace rmn
