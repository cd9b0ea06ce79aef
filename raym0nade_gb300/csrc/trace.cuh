// Device-side BVH traversal shared by the ray-query kernels and the
// integrator. Included by the .cu files only.
//
// Order of visits and every float operation follow the reference's
// recursive BVH::dfs_rayHit (src/bvh.cpp:56-88) so that closest-hit ids are
// the reference's:
//  * at an inner node both child boxes are tested with rayInBox
//    (src/geometry.cpp:40-61) from [t_min, current t_max];
//  * the child with the smaller entry distance goes first (ties: the right
//    child); the other is deferred on a per-thread stack together with its
//    entry distance and is visited only if that distance is still below the
//    current t_max when it is popped -- the moment the recursion would return
//    to it;
//  * a leaf tests its triangles in order and keeps t only if
//    t_min < t < t_max (first hit wins ties).
#pragma once
#include "rmn_internal.h"
#include "texture.h"

struct TRay {
  float3 o, d, inv;
  int par;  // bit i: |d_i| < 1e-4 (origin-inside rule)
  int neg;  // bit i: 1/d_i < 0
};

RMN_D TRay make_tray(float3 o, float3 d) {
  TRay r;
  r.o = o;
  r.d = d;
  r.par = (fabsf(d.x) < RMN_EPS ? 1 : 0) | (fabsf(d.y) < RMN_EPS ? 2 : 0) | (fabsf(d.z) < RMN_EPS ? 4 : 0);
  r.inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  r.neg = (r.inv.x >= 0.0f ? 0 : 1) | (r.inv.y >= 0.0f ? 0 : 2) | (r.inv.z >= 0.0f ? 0 : 4);
  return r;
}

// One axis of rayInBox. `stop` freezes tL/tR once the reference would have
// returned (tL > tR, or origin outside a slab the ray is parallel to).
RMN_D void slab_axis(bool par, bool neg, float o, float inv, float lo, float hi, float& tL, float& tR, bool& stop) {
  if (stop) return;
  if (par) {
    if (o < lo || o > hi) {
      tR = -1.0f;
      stop = true;
    }
    return;
  }
  float a = neg ? hi : lo, b = neg ? lo : hi;
  tL = fmaxf(tL, (a - o) * inv);
  tR = fminf(tR, (b - o) * inv);
  tR += RMN_EPS;
  if (tL > tR) stop = true;
}

// rayInBox + the node test `tL < tR` of dfs_rayHit.
RMN_D bool box_hit(const TRay& r, float3 lo, float3 hi, float tmin, float tmax, float& tL) {
  float L = tmin, R = tmax;
  bool stop = false;
  slab_axis(r.par & 1, r.neg & 1, r.o.x, r.inv.x, lo.x, hi.x, L, R, stop);
  slab_axis(r.par & 2, r.neg & 2, r.o.y, r.inv.y, lo.y, hi.y, L, R, stop);
  slab_axis(r.par & 4, r.neg & 4, r.o.z, r.inv.z, lo.z, hi.z, L, R, stop);
  tL = L;
  return L < R;
}

// A box test that accepts every box box_hit accepts (and a few more), for
// queries whose answer does not depend on the order of visits or on the
// entry distances (occlusion), on rays with no axis under the
// origin-inside rule (r.par == 0). The slab distances are box_hit's own
// values (same operations); L = max(tmin, entries) is box_hit's final tL
// whenever box_hit runs to the end; box_hit's final tR is
// g(min(g(min(g(min(tmax, fx)), fy)), fz)) with g(m) = RN(m + eps),
// monotone with g(m) >= m, which is at most g(g(g(min(tmax, fx, fy, fz))))
// = R here. So box_hit's tL < tR implies L < R.
RMN_D bool box_any(const TRay& r, float3 lo, float3 hi, float tmin, float tmax, float& tL) {
  const float x0 = (lo.x - r.o.x) * r.inv.x, x1 = (hi.x - r.o.x) * r.inv.x;
  const float y0 = (lo.y - r.o.y) * r.inv.y, y1 = (hi.y - r.o.y) * r.inv.y;
  const float z0 = (lo.z - r.o.z) * r.inv.z, z1 = (hi.z - r.o.z) * r.inv.z;
  const float L = fmaxf(fmaxf(tmin, fminf(x0, x1)), fmaxf(fminf(y0, y1), fminf(z0, z1)));
  float R = fminf(fminf(tmax, fmaxf(x0, x1)), fminf(fmaxf(y0, y1), fmaxf(z0, z1)));
  R += RMN_EPS;
  R += RMN_EPS;
  R += RMN_EPS;
  tL = L;
  return L < R;
}

// RayTriangleIntersection (Moller-Trumbore), src/geometry.cpp:63-87, with
// a division-free pre-test: u = RN(RN(1/a) * x), x = dot(s, h). Where x / a
// lies below -1e-5 or above 1 + 1e-5 (compared as x * sign(a) against the
// rounded products 1e-5 * |a| and 1.00001 * |a|), the two roundings (a
// relative error below 2^-23) cannot bring u into [0, 1], so the
// reference rejects the triangle too -- by its u test, or earlier by its
// degeneracy test; both give "no hit". Such triangles, most of the tested
// ones, skip the two divisions. Non-finite a or x fail both comparisons and
// take the reference's path, as does every triangle that may be hit: the
// values computed for a hit are the reference's, operation for operation.
RMN_D float tri_t(const TRay& r, float3 v0, float3 e1, float3 e2, float len_e1) {
  float3 h = cross3(r.d, e2);
  float a = dot3(e1, h);
  float3 s = r.o - v0;
  const float x = dot3(s, h);
  const float aa = fabsf(a);
  const float xs = a < 0.0f ? -x : x;
  if (xs < -1e-5f * aa || xs > 1.00001f * aa) return INFINITY;
  if (fabsf(a) / len_e1 < RMN_EPS) return INFINITY;
  float f = 1.0f / a;
  float u = f * x;
  if (u < 0.0f || u > 1.0f) return INFINITY;
  float3 q = cross3(s, e1);
  float v = f * dot3(r.d, q);
  if (v < 0.0f || u + v > 1.0f) return INFINITY;
  return f * dot3(e2, q);
}

// Per-thread visit counters of the counting build (rmn_render_profile).
struct TraceCounters {
  uint32_t closest, shadow, inner, leaves, tris;
};

// Resumable traversal state: the deferred children (reference plus entry
// distance), the current node and the position within the current leaf, so
// a warp can hand a lane a new ray while its other lanes are still
// traversing.
// Stack storage: per-thread local memory, or a slice of shared memory (the
// persistent traversal kernels; entry e of thread i at base[e * 128 + i], so
// a warp's accesses to one level fall in distinct banks). kCap entries.
struct LocalStack {
  static constexpr int kCap = RMN_STACK;
  int2 e[RMN_STACK];  // (reference, entry distance as float bits)
  RMN_D void put(int i, int2 v) { e[i] = v; }
  RMN_D int2 get(int i) const { return e[i]; }
};
template <int N = RMN_STACK>
struct SharedStackN {
  static constexpr int kCap = N;
  int2* base;
  RMN_D void put(int i, int2 v) { base[i * 128] = v; }
  RMN_D int2 get(int i) const { return base[i * 128]; }
};
using SharedStack = SharedStackN<RMN_STACK>;
// References only (order-free occlusion): get() reports an entry distance of
// -inf, so a pop never skips an entry.
template <int N>
struct SharedStackRefN {
  static constexpr int kCap = N;
  int* base;
  RMN_D void put(int i, int2 v) { base[i * 128] = v.x; }
  RMN_D int2 get(int i) const { return make_int2(base[i * 128], __float_as_int(-INFINITY)); }
};

template <class Stack>
struct TravT {
  int cur;     // next node reference to visit
  int sp;
  int hit;     // leaf-order triangle index of the closest hit so far, -1 none
  int ti, te;  // triangles [ti, te) of the current leaf still to test
  float tmax;
  bool pop;    // cooperative traversal: the next step pops the stack
  Stack stack;
};
using Trav = TravT<LocalStack>;

template <class Stack>
RMN_D void trav_begin(int root, TravT<Stack>& t, float tmax) {
  t.cur = root;
  t.sp = 0;
  t.hit = -1;
  t.ti = t.te = 0;
  t.tmax = tmax;
  t.pop = false;
}
template <class Stack>
RMN_D void trav_begin(const DevScene& s, TravT<Stack>& t, float tmax) {
  trav_begin(s.root, t, tmax);
}

// One inner-node step of dfs_rayHit (src/bvh.cpp:70-88): both child boxes
// against [tmin, tmax]; the nearer entry goes first (ties: the right child),
// the other is deferred with its entry distance when both are hit, or taken
// directly when only it is hit and it starts before tmax. Returns 0 with
// `cur` the next node (inner or leaf), 1 when neither child is entered (the
// caller pops), -2 when the stack would overflow. WIDE (occlusion): rays
// without an axis under the origin-inside rule take box_any.
template <bool COUNT, bool WIDE = false, class Stack>
RMN_D int inner_step(const DevNode* __restrict__ nodes, const TRay& r, float tmin, float tmax, int& cur, int& sp,
                     Stack& stack, TraceCounters* cnt) {
  const DevNode* n = nodes + cur;
  float4 A = __ldg(&n->a), B = __ldg(&n->b), C = __ldg(&n->c);
  int4 D = __ldg(&n->d);
  if (COUNT) cnt->inner++;
  float tl0, tl1;
  bool h0, h1;
  if (WIDE && r.par == 0) {
    h0 = box_any(r, f3(A.x, A.y, A.z), f3(A.w, B.x, B.y), tmin, tmax, tl0);
    h1 = box_any(r, f3(B.z, B.w, C.x), f3(C.y, C.z, C.w), tmin, tmax, tl1);
  } else {
    h0 = box_hit(r, f3(A.x, A.y, A.z), f3(A.w, B.x, B.y), tmin, tmax, tl0);
    h1 = box_hit(r, f3(B.z, B.w, C.x), f3(C.y, C.z, C.w), tmin, tmax, tl1);
  }
  int nref, fref;
  bool hn, hf;
  float tlf;
  if (tl0 < tl1) {
    nref = D.x; hn = h0; fref = D.y; hf = h1; tlf = tl1;
  } else {
    nref = D.y; hn = h1; fref = D.x; hf = h0; tlf = tl0;
  }
  if (hn) {
    if (hf) {
      if (sp >= Stack::kCap) return -2;
      stack.put(sp, make_int2(fref, __float_as_int(tlf)));
      ++sp;
    }
    cur = nref;
    return 0;
  }
  if (hf && tlf < tmax) {
    cur = fref;
    return 0;
  }
  return 1;
}

// Runs up to `budget` steps; a step is one inner node (both child boxes) or
// one triangle of a leaf, so lanes of a warp at inner nodes and lanes in
// leaves advance together instead of waiting for a whole leaf. Returns 1
// when the query is answered (t.hit / t.tmax final), 0 when the budget ran
// out first, -2 if the stack would overflow (never for trees the builder
// accepts). With ANY and `early` set, answers as soon as a hit closer than
// `aim` is recorded (Model::rayHit_test's question, after the same visits
// as the closest-hit query up to that point); scenes with alpha-tested
// materials clear `early`, since their occlusion test needs the closest hit.
template <bool ANY, bool COUNT, class Stack>
RMN_D int trav_run(const DevScene& s, const TRay& r, float tmin, float aim, TravT<Stack>& t, int budget,
                   TraceCounters* cnt, bool early = true) {
  for (;;) {
    if (budget-- <= 0) return 0;
    if (t.ti < t.te) {  // next triangle of the current leaf, in leaf order
      const int i = t.ti++;
      const float4* tp = s.tri + 3 * i;
      float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
      float th = tri_t(r, f3(a), f3(b), f3(c), b.w);
      if (tmin < th && th < t.tmax) {
        t.tmax = th;
        t.hit = i;
        if (ANY && early && th < aim) return 1;
      }
      if (t.ti < t.te) continue;
    } else {
      const int cur = t.cur;
      if (cur >= 0) {
        const int k = inner_step<COUNT>(s.nodes, r, tmin, t.tmax, t.cur, t.sp, t.stack, cnt);
        if (k == -2) return -2;
        if (k == 0) continue;
      } else {
        const int x = ~cur;
        const int count = x & 15;
        if (COUNT) { cnt->leaves++; cnt->tris += count; }
        if (count > 0) {
          t.ti = x >> 4;
          t.te = t.ti + count;
          continue;
        }
      }
    }
    // pop: the deferred child is visited only if it still starts before the
    // current closest hit
    for (;;) {
      if (t.sp == 0) return 1;
      --t.sp;
      const int2 e = t.stack.get(t.sp);
      if (__int_as_float(e.y) < t.tmax) {
        t.cur = e.x;
        break;
      }
    }
  }
}


// ------------------------------------------------ warp-cooperative leaves
// The persistent traversal kernels split each round in two warp-wide
// phases. (1) Every lane takes up to `steps` inner-node steps exactly as
// trav_run does (same boxes, same near-first order, same deferred pops),
// stopping when it reaches a leaf. (2) The triangles of all the warp's
// pending leaves are spread over the 32 lanes, 32 at a time, and each ray
// keeps the smallest (t, leaf-order index) among its leaf's triangles with
// t_min < t < t_max: what testing the leaf in order with a strict t < t_max
// gives (the first of equal distances wins). The next round pops the stack
// with that t_max, as the recursion returns after the leaf. So every ray
// visits the nodes and leaves it visits in trav_run and ends with the same
// hit and distance, while a leaf's 6-10 triangles no longer occupy one lane
// for 6-10 steps with the other lanes idle or on another branch. An
// occlusion query with `early` is answered by the leaf that holds a hit
// nearer than aim (trav_run stops at that hit inside the leaf: the same
// answer).

// Order of (t, index) as an unsigned key: t's bits made monotone (zero's
// sign dropped, as float comparison ignores it), the index below.
RMN_D unsigned long long leaf_key(float t, int tri) {
  unsigned u = __float_as_uint(t + 0.0f);
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((unsigned long long)u << 32) | (unsigned)tri;
}
RMN_D float leaf_key_t(unsigned long long k) {
  unsigned u = (unsigned)(k >> 32);
  u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  return __uint_as_float(u);
}

// Phase 1, called by all 32 lanes of a warp; `go`: the lane has a query in
// flight. Returns 1 when the lane's query is answered (its stack ran out),
// -2 on stack overflow, 0 otherwise (a leaf pending: t.ti < t.te, or steps
// left over).
template <bool COUNT, class Stack>
RMN_D int coop_nodes(const DevNode* __restrict__ nodes, const TRay& r, float tmin, TravT<Stack>& t, bool go,
                     int steps, TraceCounters* cnt) {
  int res = 0;
#pragma unroll 1
  for (int step = 0; step < steps; ++step) {
    const bool g = go && res == 0 && t.ti >= t.te;
    if (!__any_sync(0xffffffffu, g)) break;
    if (!g) continue;
    if (t.pop) {
      t.pop = false;
      for (;;) {
        if (t.sp == 0) {
          res = 1;
          break;
        }
        --t.sp;
        const int2 e = t.stack.get(t.sp);
        if (__int_as_float(e.y) < t.tmax) {
          t.cur = e.x;
          break;
        }
      }
      if (res) continue;
    }
    if (t.cur >= 0) {
      const int k = inner_step<COUNT>(nodes, r, tmin, t.tmax, t.cur, t.sp, t.stack, cnt);
      if (k == -2) {
        res = -2;
        continue;
      }
      if (k == 1) {
        t.pop = true;
        continue;
      }
    }
    if (t.cur < 0) {  // a leaf: its triangles wait for phase 2, then a pop
      const int x = ~t.cur;
      const int count = x & 15;
      if (COUNT) { cnt->leaves++; cnt->tris += count; }
      if (count > 0) {
        t.ti = x >> 4;
        t.te = t.ti + count;
      }
      t.pop = true;
    }
  }
  return res;
}

// Phase 2, called by all 32 lanes of a warp. `tri`: the lane's triangle
// records (SAME_TRI: one scene for the whole warp, so its pointer is not
// exchanged); `keys`: 32 entries of shared memory for this warp. Clears the
// pending leaves; returns true for a lane whose occlusion query (ANY with
// `early`) is answered.
template <bool ANY, bool SAME_TRI, class Stack>
RMN_D bool coop_leaves(const float4* __restrict__ tri, const TRay& r, float tmin, float aim, TravT<Stack>& t,
                       bool early, unsigned long long* keys) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int cnt = t.ti < t.te ? t.te - t.ti : 0;
  if (!__any_sync(FULL, cnt > 0)) return false;
  int incl = cnt;  // inclusive prefix sum of the lanes' triangle counts
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += v;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const int excl = incl - cnt;
  keys[lane] = ~0ull;
  __syncwarp();
#pragma unroll 1
  for (int base = 0; base < total; base += 32) {
    const int k = base + lane;
    // owner: the first lane whose inclusive count exceeds k
    int lo = 0;
#pragma unroll
    for (int st = 16; st >= 1; st >>= 1) {
      const int v = __shfl_sync(FULL, incl, lo + st - 1);
      if (v <= k) lo += st;
    }
    const int ow = min(lo, 31);
    const int first = __shfl_sync(FULL, t.ti, ow) - __shfl_sync(FULL, excl, ow);
    TRay q;
    q.o.x = __shfl_sync(FULL, r.o.x, ow);
    q.o.y = __shfl_sync(FULL, r.o.y, ow);
    q.o.z = __shfl_sync(FULL, r.o.z, ow);
    q.d.x = __shfl_sync(FULL, r.d.x, ow);
    q.d.y = __shfl_sync(FULL, r.d.y, ow);
    q.d.z = __shfl_sync(FULL, r.d.z, ow);
    const float qmin = __shfl_sync(FULL, tmin, ow);
    const float qmax = __shfl_sync(FULL, t.tmax, ow);
    const float4* qtri = tri;
    if (!SAME_TRI) {
      const unsigned long long p = reinterpret_cast<unsigned long long>(tri);
      const unsigned lo32 = __shfl_sync(FULL, (unsigned)p, ow), hi32 = __shfl_sync(FULL, (unsigned)(p >> 32), ow);
      qtri = reinterpret_cast<const float4*>(((unsigned long long)hi32 << 32) | lo32);
    }
    if (k < total) {
      const int i = first + k;
      const float4* tp = qtri + 3 * i;
      float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
      const float th = tri_t(q, f3(a), f3(b), f3(c), b.w);
      if (qmin < th && th < qmax) atomicMin(&keys[ow], leaf_key(th, i));
    }
  }
  __syncwarp();
  bool answered = false;
  if (cnt > 0) {
    const unsigned long long kk = keys[lane];
    if (kk != ~0ull) {
      t.hit = (int)(unsigned)(kk & 0xffffffffu);
      float th = leaf_key_t(kk);
      if (th == 0.0f) {  // a zero distance keeps the sign its own test gives
        const float4* tp = tri + 3 * t.hit;
        float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        th = tri_t(r, f3(a), f3(b), f3(c), b.w);
      }
      t.tmax = th;
      answered = ANY && early && th < aim;
    }
    t.ti = t.te;
  }
  __syncwarp();
  return answered;
}


// ------------------------------------------ occlusion with pending leaves
// An occlusion query asks whether any triangle lies at eps < t < aim. The
// reference answers it with a closest-hit search over (eps, aim + eps) and
// compares the distance found with aim (Model::rayHit_test); any hit nearer
// than aim makes that distance nearer than aim, whatever the order of
// visits. So the occlusion kernels of scenes without alpha-tested materials
// drop the order: a lane that reaches a leaf keeps it pending and goes on
// stepping -- popping its stack -- until it holds two leaves or its steps
// for the round are used up, and the warp then tests the triangles of all
// pending leaves together, 32 at a time, one bit per ray for "a hit nearer
// than aim". The boxes are tested against the query's interval as it
// starts, (eps, aim + eps), which the reference's interval never exceeds,
// so every triangle the reference tests is tested here: the answers agree
// unless an occluder's distance lies within float rounding of a box's entry
// distance while another surface lies between aim and aim + eps (the
// reference can then skip the box). Scenes with alpha-tested materials keep
// the ordered search, which their retry past cut-away hits needs.
template <class Stack>
struct OccT {
  int cur, sp;
  int a0, c0, a1, c1;  // pending leaves: first triangle, count (c1 > 0 only with c0 > 0)
  bool pop;
  Stack stack;
};

template <class Stack>
RMN_D void occ_begin(int root, OccT<Stack>& t) {
  t.cur = root;
  t.sp = 0;
  t.c0 = t.c1 = 0;
  t.pop = false;
}

// Phase 1 (all 32 lanes): up to `steps` inner-node steps for lanes with
// `go` that hold fewer than two pending leaves. Returns 1 once the lane's
// stack is used up (its pending leaves, if any, still to test), -2 on
// stack overflow, 0 otherwise.
template <bool COUNT, class Stack>
RMN_D int occ_nodes(const DevNode* __restrict__ nodes, const TRay& r, float tmin, float tmax, OccT<Stack>& t,
                    bool go, int steps, TraceCounters* cnt) {
  int res = 0;
#pragma unroll 1
  for (int step = 0; step < steps; ++step) {
    const bool g = go && res == 0 && t.c1 == 0;
    if (!__any_sync(0xffffffffu, g)) break;
    if (!g) continue;
    if (t.pop) {
      t.pop = false;
      for (;;) {
        if (t.sp == 0) {
          res = 1;
          break;
        }
        --t.sp;
        const int2 e = t.stack.get(t.sp);
        if (__int_as_float(e.y) < tmax) {
          t.cur = e.x;
          break;
        }
      }
      if (res) continue;
    }
    if (t.cur >= 0) {
      const int k = inner_step<COUNT, true>(nodes, r, tmin, tmax, t.cur, t.sp, t.stack, cnt);
      if (k == -2) {
        res = -2;
        continue;
      }
      if (k == 1) {
        t.pop = true;
        continue;
      }
    }
    if (t.cur < 0) {  // a leaf: kept pending, and on to the next node
      const int x = ~t.cur;
      const int count = x & 15;
      if (COUNT) { cnt->leaves++; cnt->tris += count; }
      if (count > 0) {
        if (t.c0 == 0) {
          t.a0 = x >> 4;
          t.c0 = count;
        } else {
          t.a1 = x >> 4;
          t.c1 = count;
        }
      }
      t.pop = true;
    }
  }
  return res;
}

// The leaf phase's exchange in shared memory, per 128-thread block: each
// lane with pending triangles writes its ray, its leaves and (batch
// kernels) its triangle array once, and its lane index into its warp's
// owner table for each of its triangles; the lane testing triangle k of the
// warp's list reads its owner and the owner's data from there.
constexpr int kOccOwn = 32 * 30;  // per warp: 32 lanes x two leaves of at most 15 triangles
struct OccExchange {
  float4 ray[2 * 128];         // (origin, aim), (direction, t_min)
  int4 leaf[128];              // a0, c0, a1, first index of the lane's triangles in the warp's list
  const float4* tri[128];
  unsigned char own[4][kOccOwn];
};

// Phase 2 (all 32 lanes): the pending leaves' triangles, 32 at a time;
// true for a lane whose ray has a hit at tmin < t < aim. Clears the pending
// leaves. SAME_TRI: one scene for the whole warp (its triangle array is not
// exchanged).
template <bool SAME_TRI, class Stack>
RMN_D bool occ_leaves(const float4* __restrict__ tri, const TRay& r, float tmin, float aim, OccT<Stack>& t,
                      OccExchange& x) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int wb = threadIdx.x & ~31;
  unsigned char* own = x.own[threadIdx.x >> 5];
  const int cnt = t.c0 + t.c1;  // at most 30
  if (!__any_sync(FULL, cnt > 0)) return false;
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += v;
  }
  const int total = __shfl_sync(FULL, incl, 31);  // at most kOccOwn
  const int excl = incl - cnt;
  if (cnt > 0) {
    x.ray[2 * threadIdx.x] = make_float4(r.o.x, r.o.y, r.o.z, aim);
    x.ray[2 * threadIdx.x + 1] = make_float4(r.d.x, r.d.y, r.d.z, tmin);
    x.leaf[threadIdx.x] = make_int4(t.a0, t.c0, t.a1, excl);
    if (!SAME_TRI) x.tri[threadIdx.x] = tri;
    for (int k = excl; k < incl; ++k) own[k] = (unsigned char)lane;
  }
  __syncwarp();
  unsigned occluded = 0;  // bit per owner lane
#pragma unroll 1
  for (int base = 0; base < total; base += 32) {
    const int k = base + lane;
    bool h = false;
    int ow = 0;
    if (k < total) {
      ow = own[k];
      const int o = wb + ow;
      const int4 lf = x.leaf[o];
      const float4 ra = x.ray[2 * o], rb = x.ray[2 * o + 1];
      const int loc = k - lf.w;  // in [0, c0 + c1) of the owner; loc >= c0 only when c1 > 0
      const int i = loc < lf.y ? lf.x + loc : lf.z + (loc - lf.y);
      TRay q;
      q.o = f3(ra.x, ra.y, ra.z);
      q.d = f3(rb.x, rb.y, rb.z);
      const float4* tp = (SAME_TRI ? tri : x.tri[o]) + 3 * i;
      float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
      const float th = tri_t(q, f3(a), f3(b), f3(c), b.w);
      h = rb.w < th && th < ra.w;
    }
    // the owners of the lanes that found an occluder
    unsigned m = __ballot_sync(FULL, h);
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      occluded |= 1u << __shfl_sync(FULL, ow, src);
    }
  }
  __syncwarp();
  t.c0 = t.c1 = 0;
  return (occluded >> lane) & 1u;
}

// One whole query without the alpha retry (scenes without alpha-tested
// materials), its deferred-child stack in shared memory at `stk` (entry e
// at stk[e * 128], see SharedStackN). Same answer as trace().
template <bool ANY>
RMN_D int trace_shared(const DevScene& s, const TRay& r, float tmin, float& tmax, float aim, int2* stk) {
  TravT<SharedStackN<RMN_STACK>> t;
  t.stack.base = stk;
  trav_begin(s, t, tmax);
  int st = trav_run<ANY, false>(s, r, tmin, aim, t, 0x7fffffff, nullptr);
  tmax = t.tmax;
  return st == -2 ? -2 : t.hit;
}

// barycentric(v0, v1, v2, P), src/geometry.cpp:89-103, with e1 = v1 - v0 and
// e2 = v2 - v0 precomputed. Returns (gamma, alpha, beta).
RMN_D float3 bary(float3 v0, float3 e1, float3 e2, float3 p) {
  float3 n = cross3(e1, e2);
  float den = dot3(n, n);
  float3 vp = p - v0;
  float al = dot3(cross3(vp, e2), n) / den;
  float be = dot3(cross3(e1, vp), n) / den;
  return f3(1.0f - al - be, al, be);
}

// TransparentTest, src/model.cpp:217-230: a hit at distance t on triangle i
// (leaf order) of an alpha-tested material is cut away where the level-0
// diffuse alpha at the hit is below eps (getDiffuseColor(u, v, NaN); gamma
// leaves alpha alone). The scene's arrays come as plain pointers so that a
// caller's scene copy can stay in registers.
RMN_D bool alpha_cut_at(const float4* __restrict__ tri, const float4* __restrict__ uv,
                        const float4* __restrict__ shade, const DevMat* __restrict__ mats,
                        const DevTex* __restrict__ texs, const uint8_t* __restrict__ texels,
                        float3 o, float3 d, int i, float t) {
  const float4* tp = tri + 3 * i;
  const float4 C = __ldg(tp + 2);
  if (!(__float_as_int(C.w) & RMN_TRI_ALPHA)) return false;
  const float4 A = __ldg(tp), B = __ldg(tp + 1);
  const float3 b = bary(f3(A), f3(B), f3(C), o + d * t);
  const float4 u01 = __ldg(uv + 2 * i), u2 = __ldg(uv + 2 * i + 1);
  const float u = b.x * u01.x + b.y * u01.z + b.z * u2.x;
  const float v = b.x * u01.y + b.y * u01.w + b.z * u2.y;
  const int mat = __float_as_int(__ldg(&shade[3 * i].w));
  const int tx = __ldg(&mats[mat].tex.x);
  return tex_get<4>(texs[tx], texels, u, v, 0.0f).w < RMN_EPS;
}
RMN_D bool alpha_cut(const DevScene& s, const TRay& r, int i, float t) {
  return alpha_cut_at(s.tri, s.uv, s.shade, s.mats, s.texs, s.texels, r.o, r.d, i, t);
}

// The retry loop of Model::rayHit / rayHit_test (src/model.cpp:330-354)
// after an answered search: if the closest hit is cut away and fewer than 8
// searches ran, begins the next search from eps beyond it (up to
// `restart_tmax`) and returns true. `searches` counts the finished searches.
// When the eighth hit is cut away too, the reference leaves its loop with
// the record reset for a next search: Model::rayHit (`closest`) then
// answers a miss, rayHit_test answers occluded (t stays below the aim).
template <class Stack>
RMN_D bool alpha_again(const DevScene& s, const TRay& r, TravT<Stack>& t, float& tmin, float restart_tmax,
                       int& searches, bool closest) {
  if (t.hit < 0 || !alpha_cut(s, r, t.hit, t.tmax)) return false;
  if (++searches >= 8) {
    if (closest) {
      t.hit = -1;
      t.tmax = restart_tmax;
    }
    return false;
  }
  tmin = t.tmax + RMN_EPS;
  trav_begin(s, t, restart_tmax);
  return true;
}

// One whole query: closest hit in (tmin, tmax) (with ANY: whether a hit is
// nearer than aim). In a scene with alpha-tested materials the query is
// Model::rayHit's (tmin = eps, tmax = inf) or rayHit_test's (tmax = aim +
// eps), retried past cut-away hits; ALPHA = false builds the query for
// scenes known to have none. Returns the leaf-order triangle index or -1
// (tmax becomes the hit distance), -2 on stack overflow.
template <bool ANY, bool COUNT, bool ALPHA = true>
RMN_D int trace(const DevScene& s, const TRay& r, float tmin, float& tmax, float aim, TraceCounters* cnt) {
  Trav t;
  const float tmax0 = tmax;
  trav_begin(s, t, tmax);
  if (COUNT) {
    if (ANY) cnt->shadow++;
    else cnt->closest++;
  }
  if (!ALPHA) {
    int st = trav_run<ANY, COUNT>(s, r, tmin, aim, t, 0x7fffffff, cnt);
    tmax = t.tmax;
    return st == -2 ? -2 : t.hit;
  }
  int searches = 0;
  for (;;) {
    const bool alpha = ALPHA && s.has_alpha;
    int st = trav_run<ANY, COUNT>(s, r, tmin, aim, t, 0x7fffffff, cnt, !alpha);
    if (st == -2) {
      tmax = t.tmax;
      return -2;
    }
    if (alpha && !(ANY && t.tmax >= aim) && alpha_again(s, r, t, tmin, tmax0, searches, !ANY)) continue;
    tmax = t.tmax;
    return t.hit;
  }
}
