// Counter-based random stream of the GPU path tracer.
//
// The reference draws every random number of a render thread from one
// std::mt19937 mapped to U(1e-6, 1 - 1e-6) (src/component.cpp:5-10). A GPU
// thread cannot carry 2.5 KB of Mersenne-Twister state, and the adjoint pass
// must replay paths, so each (render seed, pixel, sample slot) owns a stream
// whose n-th draw is a pure function of those four integers: a SplitMix64
// finaliser (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) applied to key + n * golden-ratio increment.
// The float mapping keeps the reference's open interval: the top 24 bits give
// u in [0, 1), and u * (b - a) + a with a = 1e-6f, b = 1 - 1e-6f, both
// products rounded as float, exactly as libstdc++'s
// uniform_real_distribution<float> maps its canonical draw.
//
// Host (the oracle) and device compile the same integer code, so both sides
// see bit-identical streams; the float step has no fused multiply-add
// (__fmul_rn / __fadd_rn on the device).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RMN_HD __host__ __device__ __forceinline__
#else
#define RMN_HD inline
#endif

RMN_HD uint64_t rmn_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Stream key of one sample slot of one pixel. Slots [0, spp_direct) are the
// first-vertex light samples, slots spp_direct + k the k-th indirect path.
RMN_HD uint64_t rmn_stream_key(uint64_t seed, uint32_t pixel, uint32_t slot) {
  uint64_t k = rmn_mix64(seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(pixel + 1u));
  return rmn_mix64(k + 0xD1B54A32D192ED03ULL * (uint64_t)(slot + 1u));
}

struct RmnRng {
  uint64_t key;
  uint32_t ctr;
  RMN_HD uint32_t next_u32() {
    ++ctr;
    return (uint32_t)(rmn_mix64(key + 0x9E3779B97F4A7C15ULL * (uint64_t)ctr) >> 32);
  }
  RMN_HD float next() {
    const float lo = 1e-6f;
    const float span = 0.99999797344207763671875f;  // (1 - 1e-6f) - 1e-6f in float
    float u = (float)(next_u32() >> 8) * 5.9604644775390625e-8f;  // * 2^-24, exact
#if defined(__CUDA_ARCH__)
    return __fadd_rn(__fmul_rn(u, span), lo);
#else
    return u * span + lo;
#endif
  }
};

RMN_HD RmnRng rmn_rng(uint64_t seed, uint32_t pixel, uint32_t slot) {
  RmnRng r;
  r.key = rmn_stream_key(seed, pixel, slot);
  r.ctr = 0;
  return r;
}
