// or3_device.cuh -- device-side scene view, RNG, intersection and traversal.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "or3.h"
#include "or3_common.h"

namespace or3 {

// Device view of one uploaded scene.
struct DevScene {
  const uint4 *nodes;          // WideNode[num_nodes] as 4 x uint4
  const float4 *fnodes;        // WideNodeF[num_nodes] as 8 x float4 (optional FP32-box copy)
  const float4 *fnodes8;       // WideNode8F as 16 x float4: the 8-wide traversal variant (made on first use)
  const float4 *prims;         // 3 x float4 per record
  const PrimInfo *info;        // per record
  const TriShade *tri_shade;   // per record (triangles)
  const PlaneRec *planes;      // not-in-BVH objects
  const MaterialDev *materials;
  const LayerDev *layers;
  const float *env;            // RGB, env_w * env_h
  const TextureDev *textures;
  const float *texels;
  // next-event estimation: local lights chosen by power, and the environment
  const LightDev *lights;      // [num_lights]
  const float *light_cdf;      // [num_lights] inclusive CDF, last = 1
  const float *light_pdf;      // [num_lights] selection probability among local lights
  const float *env_marg;       // [env_h] inclusive marginal CDF over rows
  const float *env_cond;       // [env_h * env_w] inclusive conditional CDF per row
  const uint32_t *env_gmarg;   // [env_h + 1] guide table of env_marg
  const uint32_t *env_gcond;   // [env_h * (env_w + 1)] guide table of each env_cond row
  uint32_t num_nodes, num_prims, num_planes, num_lights;
  uint32_t env_w, env_h, num_textures;
  int32_t env_light;           // 0 none, 1 equirect map (CDF), 2 constant background
  float env_prob;              // probability that a light sample goes to the environment
  float bg[3];
};

// ---------------------------------------------------------------- math
struct V3 {
  float x, y, z;
};
OR3_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
OR3_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
OR3_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
OR3_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
OR3_HD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
OR3_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
OR3_HD V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ V3 normalize(V3 a) {
  const float l = sqrtf(dot(a, a));
  return v3(a.x / l, a.y / l, a.z / l);
}

// ---------------------------------------------------------------- RNG
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), counter-based so a path's random numbers depend
// only on (path, leaf, depth, call) and not on execution order.  Replaces the
// reference's per-row xorshift stream (src/tools/Random.h:7-30), which cannot
// be replayed in wavefront order.
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}
// 24-bit uniform in [0, 1)
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// counter for bounce randoms of a path leaf
__device__ __forceinline__ uint4 path_counter(uint64_t g, uint32_t leaf, uint32_t depth, uint32_t call) {
  return make_uint4((uint32_t)g, (uint32_t)(g >> 32), (depth & 0xFFFFu) | (leaf << 16) | (call << 24), 0u);
}

// ---------------------------------------------------------------- hits
constexpr uint32_t kMissRec = 0xFFFFFFFFu;
constexpr uint32_t kPlaneBit = 0x80000000u;

struct Hit {
  float t;
  uint32_t rec;  // record index, kPlaneBit|plane, or kMissRec
  float u, v;    // barycentric rates (triangles)
};

// Reference triangle test, single-sided with det > EPS
// (Polygon::CheckIntersection, src/renderer/Polygon.h:63-106), in FP32.
__device__ __forceinline__ bool isect_triangle(const float4 a, const float4 b, const float4 c, V3 o, V3 d,
                                               float tbest, float &t, float &ur, float &vr) {
  const V3 v0 = v3(a.x, a.y, a.z);
  const V3 e1 = v3(a.w, b.x, b.y);
  const V3 e2 = v3(b.z, b.w, c.x);
  const V3 P = cross(d, e2);
  const float det = dot(P, e1);
  if (!(det > kEps)) return false;
  const V3 T = o - v0;
  const float u = dot(P, T);
  if (!(u >= 0.f && u <= det)) return false;
  const V3 Q = cross(T, e1);
  const float v = dot(Q, d);
  if (!(v >= 0.f && u + v <= det)) return false;
  const float inv = 1.0f / det;  // one division for t, u and v
  const float tt = dot(Q, e2) * inv;
  if (!(tt >= kEps) || !(tt < tbest)) return false;
  t = tt;
  ur = u * inv;
  vr = v * inv;
  return true;
}

// Sphere test with the reference's root choice (Sphere::CheckIntersection,
// src/renderer/Sphere.h:21-78): nearest root > EPS.  The discriminant is
// formed from the ray-to-centre perpendicular and the near root from the
// product of roots (Haines, Guenther, Akenine-Moller, "Precision Improvements
// for Ray/Sphere Intersection", Ray Tracing Gems ch. 7), which keeps FP32
// close to the reference's FP64 values.
__device__ __forceinline__ bool isect_sphere(const float4 s, V3 o, V3 d, float tbest, float &t) {
  const V3 cx = v3(s.x - o.x, s.y - o.y, s.z - o.z);
  const float a = dot(d, d);
  const float b = dot(d, cx);  // = v.(c - x)
  const V3 l = cx - d * (b / a);
  const float r2 = s.w * s.w;
  const float D = r2 - dot(l, l);  // discriminant / a
  if (D < 0.f) return false;
  const float sq = sqrtf(a * D);
  const float q = b + copysignf(sq, b);
  const float cc = dot(cx, cx) - r2;
  float t1, t2;  // far, near (reference t1 = b + sqrtD, t2 = b - sqrtD, scaled by 1/a)
  if (q == 0.f) {
    t1 = t2 = 0.f;
  } else {
    const float ra = q / a, rb = cc / q;
    t1 = fmaxf(ra, rb);
    t2 = fminf(ra, rb);
  }
  if (t1 <= kEps && t2 <= kEps) return false;
  const float tt = t2 > kEps ? t2 : t1;
  if (!(tt < tbest)) return false;
  t = tt;
  return true;
}

// AxisAlignedPlane (src/renderer/AxisAlignedPlane.h:38-64) and InfiniteFloor
// (src/renderer/InfiniteFloor.h:19-37).
__device__ __forceinline__ bool isect_plane(const PlaneRec &p, V3 o, V3 d, float tbest, float &t) {
  float tt;
  if (p.kind == kPrimFloor) {
    if (fabsf(d.y) < kEps) return false;
    tt = (p.offset - o.y) / d.y;
  } else {
    const float dd = p.axis == 0 ? d.z : p.axis == 1 ? d.y : d.x;
    const float oo = p.axis == 0 ? o.z : p.axis == 1 ? o.y : o.x;
    if (dd == 0.f) return false;
    tt = (p.offset - oo) / dd;
  }
  if (!(tt >= kEps) || !(tt < tbest)) return false;
  t = tt;
  return true;
}

// byte i of w as an exact float (PRMT into a 2^23 mantissa + FADD)
__device__ __forceinline__ float qbyte(uint32_t w, uint32_t i) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + i)) - 8388608.0f;
}

__device__ __forceinline__ float safe_inv(float x) {
  return 1.0f / (fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x));
}

// ---------------------------------------------------------------- stepped traversal
// Traversal as a per-lane state machine, one unit of work per step: either
// one 64-byte node (4 boxes) or one leaf (<= 4 primitives).  Leaf children are
// ordered with internal children by entry distance and go through the same
// stack, so a step never runs a variable-length leaf loop inside a node test
// and lanes of a warp stay on the same branch more often.  The persistent
// kernels (or3_kernels.cu) refill a lane with a new ray the moment its ray
// finishes.
constexpr uint32_t kLeafEntry = 0x80000000u;   // entry = kLeafEntry | count << 23 | first record
constexpr uint32_t kMaxLeafFirst = 1u << 23;   // records addressable by a leaf entry
constexpr uint32_t kNoEntry = 0xFFFFFFFFu;

struct TravState {
  V3 o, d;
  V3 inv, oi;
  uint32_t signs;  // bit a: inv[a] < 0
  float tmax;      // best distance so far (or the any-hit limit)
  uint32_t rec;
  float u, v;
  uint32_t entry;
  int sp;
};

__device__ __forceinline__ void trav_init(TravState &s, V3 o, V3 d, float tmax, uint32_t num_nodes) {
  s.o = o;
  s.d = d;
  s.inv = v3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  s.oi = v3(-o.x * s.inv.x, -o.y * s.inv.y, -o.z * s.inv.z);
  s.signs = (s.inv.x < 0.f ? 1u : 0u) | (s.inv.y < 0.f ? 2u : 0u) | (s.inv.z < 0.f ? 4u : 0u);
  s.tmax = tmax;
  s.rec = kMissRec;
  s.u = s.v = 0.f;
  s.entry = num_nodes > 0 ? 0u : kNoEntry;
  s.sp = 0;
}

// Traversal stack for trav_step_inline: put(i, entry, key), pair(i) =
// (entry, key bits), over the thread's arrays (local memory).
struct LocalStack {
  uint32_t *e;
  float *t;
  __device__ __forceinline__ void put(int i, uint32_t ee, float tt) {
    e[i] = ee;
    t[i] = tt;
  }
  __device__ __forceinline__ uint2 pair(int i) const { return make_uint2(e[i], __float_as_uint(t[i])); }
};

// The same with (entry, key) side by side: one 8-byte store per push and one
// 8-byte load per pop.
struct PairStack {
  uint2 *s;
  __device__ __forceinline__ void put(int i, uint32_t ee, float tt) { s[i] = make_uint2(ee, __float_as_uint(tt)); }
  __device__ __forceinline__ uint2 pair(int i) const { return s[i]; }
};

template <class STK>
__device__ __forceinline__ bool trav_pop_stk(TravState &s, const STK &stk) {
  while (s.sp > 0) {
    s.sp--;
    const uint2 p = stk.pair(s.sp);
    if (__uint_as_float(p.y) <= s.tmax * 1.0000010f) {
      s.entry = p.x;
      return true;
    }
  }
  s.entry = kNoEntry;
  return false;
}

// Pops the nearest pending entry that can still hold a closer hit; false when none.
__device__ __forceinline__ bool trav_pop(TravState &s, const uint32_t *stk_e, const float *stk_t) {
  while (s.sp > 0) {
    s.sp--;
    if (stk_t[s.sp] <= s.tmax * 1.0000010f) {
      s.entry = stk_e[s.sp];
      return true;
    }
  }
  s.entry = kNoEntry;
  return false;
}

// One step.  Returns true when the traversal of the BVH is over (the
// not-in-BVH list is then tested by trav_finish).
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trav_step(const DevScene &S, TravState &s, uint32_t *stk_e, float *stk_t,
                                          const uint4 *snodes, uint32_t ns, uint32_t *cnt, uint32_t *err) {
  const uint32_t e = s.entry;
  if (e == kNoEntry) return true;
  if (!(e & kLeafEntry)) {
    uint4 n0, n1, n2, n3;
    if (COUNT) cnt[0]++;
    if (e < ns) {
      n0 = snodes[4 * e + 0];
      n1 = snodes[4 * e + 1];
      n2 = snodes[4 * e + 2];
      n3 = snodes[4 * e + 3];
    } else {
      const uint4 *np = S.nodes + 4 * (size_t)e;
      n0 = __ldg(np + 0);
      n1 = __ldg(np + 1);
      n2 = __ldg(np + 2);
      n3 = __ldg(np + 3);
    }
    const uint32_t ew = n0.w;
    const float ax = __uint_as_float((ew & 0xFFu) << 23) * s.inv.x;
    const float ay = __uint_as_float(((ew >> 8) & 0xFFu) << 23) * s.inv.y;
    const float az = __uint_as_float(((ew >> 16) & 0xFFu) << 23) * s.inv.z;
    const uint32_t imask = ew >> 24;
    const float bx = fmaf(__uint_as_float(n0.x), s.inv.x, s.oi.x);
    const float by = fmaf(__uint_as_float(n0.y), s.inv.y, s.oi.y);
    const float bz = fmaf(__uint_as_float(n0.z), s.inv.z, s.oi.z);
    // byte words: lo x,y,z = n1.x,n1.y,n1.z ; hi x,y,z = n1.w,n2.x,n2.y
    const uint32_t wnx = (s.signs & 1u) ? n1.w : n1.x, wfx = (s.signs & 1u) ? n1.x : n1.w;
    const uint32_t wny = (s.signs & 2u) ? n2.x : n1.y, wfy = (s.signs & 2u) ? n1.y : n2.x;
    const uint32_t wnz = (s.signs & 4u) ? n2.y : n1.z, wfz = (s.signs & 4u) ? n1.z : n2.y;
    const uint32_t counts = n3.z;
    const float tlimit = s.tmax * 1.0000010f;
    float key[4];
    uint32_t kid[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const float tnx = fmaf(qbyte(wnx, i), ax, bx), tfx = fmaf(qbyte(wfx, i), ax, bx);
      const float tny = fmaf(qbyte(wny, i), ay, by), tfy = fmaf(qbyte(wfy, i), ay, by);
      const float tnz = fmaf(qbyte(wnz, i), az, bz), tfz = fmaf(qbyte(wfz, i), az, bz);
      const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
      const float tf = fminf(fminf(tfx, tfy), tfz) * 1.0000010f;
      const bool internal = (imask >> i) & 1u;
      const uint32_t c = (counts >> (8 * i)) & 0xFFu;
      const uint32_t ch = i == 0 ? n2.z : i == 1 ? n2.w : i == 2 ? n3.x : n3.y;
      const bool valid = internal || c != 0u;
      key[i] = (valid && tn <= tf && tn <= tlimit) ? tn : kInf * 2.f;
      kid[i] = internal ? ch : (kLeafEntry | (c << 23) | ch);
    }
#define OR3_CSWAP(a, b)                                       \
  if (key[b] < key[a]) {                                      \
    const float tk = key[a]; key[a] = key[b]; key[b] = tk;     \
    const uint32_t tc = kid[a]; kid[a] = kid[b]; kid[b] = tc;  \
  }
    OR3_CSWAP(0, 1) OR3_CSWAP(2, 3) OR3_CSWAP(0, 2) OR3_CSWAP(1, 3) OR3_CSWAP(1, 2)
#undef OR3_CSWAP
    const float inf2 = kInf * 2.f;
    if (key[0] < inf2) {
#pragma unroll
      for (int j = 3; j >= 1; j--) {
        if (key[j] < inf2) {
          if (s.sp < kStackSize) {
            stk_e[s.sp] = kid[j];
            stk_t[s.sp] = key[j];
            s.sp++;
          } else {
            atomicOr(err, 1u);  // not reachable: the builder bounds the tree depth
          }
        }
      }
      s.entry = kid[0];
      return false;
    }
    return !trav_pop(s, stk_e, stk_t);
  }
  // leaf: triangles then spheres
  const uint32_t first = e & (kMaxLeafFirst - 1u);
  const uint32_t c = (e >> 23) & 0xFFu;
  const uint32_t ntri = c & 15u, nsph = c >> 4;
  if (COUNT) {
    cnt[1] += ntri;
    cnt[2] += nsph;
  }
  for (uint32_t k = 0; k < ntri; k++) {
    const float4 *pr = S.prims + 3 * (size_t)(first + k);
    const float4 a = __ldg(pr), b = __ldg(pr + 1), cc = __ldg(pr + 2);
    float t, u, v;
    if (isect_triangle(a, b, cc, s.o, s.d, s.tmax, t, u, v)) {
      s.tmax = t;
      s.rec = first + k;
      s.u = u;
      s.v = v;
    }
  }
  for (uint32_t k = ntri; k < ntri + nsph; k++) {
    const float4 a = __ldg(S.prims + 3 * (size_t)(first + k));
    float t;
    if (isect_sphere(a, s.o, s.d, s.tmax, t)) {
      s.tmax = t;
      s.rec = first + k;
      s.u = s.v = 0.f;
    }
  }
  if (ANY && s.rec != kMissRec) return true;
  return !trav_pop(s, stk_e, stk_t);
}

// What a traversal step reads of a scene (fnodes or nodes every step, prims
// per leaf): a DevScene, or a TravView for the batched kernels, whose rays
// each name their scene.  TravView holds the node array in registers, copied
// once when a lane takes a ray, so the dependent node fetch of every step
// does not wait on a reload of the scene descriptor; the record array is
// read through the descriptor (`prims` refers to its field), once per leaf.
struct TravView {
  const float4 *fnodes;
  const uint4 *nodes;
  const float4 *const &prims;
};

// Tests the primitives of one leaf slot (triangles then spheres).
template <bool COUNT, class SV>
__device__ __forceinline__ void trav_leaf(const SV &S, TravState &s, uint32_t first, uint32_t c,
                                          uint32_t *cnt) {
  const uint32_t ntri = c & 15u, nsph = c >> 4;
  if (COUNT) {
    cnt[1] += ntri;
    cnt[2] += nsph;
  }
  for (uint32_t k = 0; k < ntri; k++) {
    const float4 *pr = S.prims + 3 * (size_t)(first + k);
    const float4 a = __ldg(pr), b = __ldg(pr + 1), cc = __ldg(pr + 2);
    float t, u, v;
    if (isect_triangle(a, b, cc, s.o, s.d, s.tmax, t, u, v)) {
      s.tmax = t;
      s.rec = first + k;
      s.u = u;
      s.v = v;
    }
  }
  for (uint32_t k = ntri; k < ntri + nsph; k++) {
    const float4 a = __ldg(S.prims + 3 * (size_t)(first + k));
    float t;
    if (isect_sphere(a, s.o, s.d, s.tmax, t)) {
      s.tmax = t;
      s.rec = first + k;
      s.u = s.v = 0.f;
    }
  }
}

// One node per step; the node's hit leaf children are tested right away and
// only internal children go through the stack (stack entries are node indices).
// SORT: visit internal children nearest first (closest hit); an any-hit
// query may take them in slot order.
// FN: test the node's FP32 child boxes (S.fnodes); false: the quantised
// boxes (S.nodes, optionally staged in shared memory as snodes[0..ns)).
// The stack cannot overflow here (depth bound checked at upload, push index
// clamped), so `err` is not written on this path; the signature matches
// trav_step's.
// NEAREST (with SORT false): the nearest internal child hit is next and the
// others go on the stack in slot order (an argmin instead of the sorting
// network; popped entries are still pruned by their entry distance).
template <bool ANY, bool COUNT, bool SORT = true, class STK = LocalStack, bool FN = true, class SV = DevScene,
          bool NEAREST = false>
__device__ __forceinline__ bool trav_step_inline(const SV &S, TravState &s, STK &stk,
                                                 const uint4 *snodes, uint32_t ns, uint32_t *cnt, uint32_t *err) {
  const uint32_t e = s.entry;
  if (e == kNoEntry) return true;
  if (COUNT) cnt[0]++;
  float key[4];
  uint32_t kid[4];
  uint4 slots;  // the four child words; read by a runtime slot index below without a local-memory array
  uint32_t leafmask = 0, counts;
  if (FN) {
    // near / far planes picked by the ray's direction signs through the load offset
    const float4 *np = S.fnodes + 8 * (size_t)e;
    const uint32_t sx = s.signs & 1u, sy = (s.signs >> 1) & 1u, sz = (s.signs >> 2) & 1u;
    const float4 bnx = __ldg(np + sx), bfx = __ldg(np + (sx ^ 1u));
    const float4 bny = __ldg(np + 2 + sy), bfy = __ldg(np + 3 - sy);
    const float4 bnz = __ldg(np + 4 + sz), bfz = __ldg(np + 5 - sz);
    const uint4 ch = __ldg(reinterpret_cast<const uint4 *>(np + 6));
    slots = ch;
    const uint4 mt = __ldg(reinterpret_cast<const uint4 *>(np + 7));
    counts = mt.x;
    const uint32_t imask = mt.y;
    const float tlimit = s.tmax * 1.0000010f;
    const float nxa[4] = {bnx.x, bnx.y, bnx.z, bnx.w}, fxa[4] = {bfx.x, bfx.y, bfx.z, bfx.w};
    const float nya[4] = {bny.x, bny.y, bny.z, bny.w}, fya[4] = {bfy.x, bfy.y, bfy.z, bfy.w};
    const float nza[4] = {bnz.x, bnz.y, bnz.z, bnz.w}, fza[4] = {bfz.x, bfz.y, bfz.z, bfz.w};
    const uint32_t cha[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const float tnx = fmaf(nxa[i], s.inv.x, s.oi.x), tfx = fmaf(fxa[i], s.inv.x, s.oi.x);
      const float tny = fmaf(nya[i], s.inv.y, s.oi.y), tfy = fmaf(fya[i], s.inv.y, s.oi.y);
      const float tnz = fmaf(nza[i], s.inv.z, s.oi.z), tfz = fmaf(fza[i], s.inv.z, s.oi.z);
      const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
      // one compare against min(far, tlimit): tn <= far && tn <= tlimit
      const float tf = fminf(fminf(fminf(tfx, tfy), tfz) * 1.0000010f, tlimit);
      const bool internal = (imask >> i) & 1u;
      const bool hitbox = tn <= tf;  // never for an empty slot (+inf / -inf planes)
      key[i] = (hitbox && internal) ? tn : kInf * 2.f;
      kid[i] = cha[i];
      if (hitbox && !internal) leafmask |= 1u << i;
    }
  } else {
  uint4 n0, n1, n2, n3;
  if (e < ns) {
    n0 = snodes[4 * e + 0];
    n1 = snodes[4 * e + 1];
    n2 = snodes[4 * e + 2];
    n3 = snodes[4 * e + 3];
  } else {
    const uint4 *np = S.nodes + 4 * (size_t)e;
    n0 = __ldg(np + 0);
    n1 = __ldg(np + 1);
    n2 = __ldg(np + 2);
    n3 = __ldg(np + 3);
  }
  const uint32_t ew = n0.w;
  const float ax = __uint_as_float((ew & 0xFFu) << 23) * s.inv.x;
  const float ay = __uint_as_float(((ew >> 8) & 0xFFu) << 23) * s.inv.y;
  const float az = __uint_as_float(((ew >> 16) & 0xFFu) << 23) * s.inv.z;
  const uint32_t imask = ew >> 24;
  const float bx = fmaf(__uint_as_float(n0.x), s.inv.x, s.oi.x);
  const float by = fmaf(__uint_as_float(n0.y), s.inv.y, s.oi.y);
  const float bz = fmaf(__uint_as_float(n0.z), s.inv.z, s.oi.z);
  const uint32_t wnx = (s.signs & 1u) ? n1.w : n1.x, wfx = (s.signs & 1u) ? n1.x : n1.w;
  const uint32_t wny = (s.signs & 2u) ? n2.x : n1.y, wfy = (s.signs & 2u) ? n1.y : n2.x;
  const uint32_t wnz = (s.signs & 4u) ? n2.y : n1.z, wfz = (s.signs & 4u) ? n1.z : n2.y;
  counts = n3.z;
  slots = make_uint4(n2.z, n2.w, n3.x, n3.y);
  const float tlimit = s.tmax * 1.0000010f;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float tnx = fmaf(qbyte(wnx, i), ax, bx), tfx = fmaf(qbyte(wfx, i), ax, bx);
    const float tny = fmaf(qbyte(wny, i), ay, by), tfy = fmaf(qbyte(wfy, i), ay, by);
    const float tnz = fmaf(qbyte(wnz, i), az, bz), tfz = fmaf(qbyte(wfz, i), az, bz);
    const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
    const float tf = fminf(fminf(tfx, tfy), tfz) * 1.0000010f;
    const bool internal = (imask >> i) & 1u;
    const uint32_t c = (counts >> (8 * i)) & 0xFFu;
    const bool hitbox = tn <= tf && tn <= tlimit;
    key[i] = (hitbox && internal) ? tn : kInf * 2.f;
    kid[i] = i == 0 ? n2.z : i == 1 ? n2.w : i == 2 ? n3.x : n3.y;
    if (hitbox && !internal && c != 0u) leafmask |= 1u << i;
  }
  }
  while (leafmask) {
    const uint32_t i = __ffs(leafmask) - 1;
    leafmask &= leafmask - 1;
    const uint32_t first = i == 0 ? slots.x : i == 1 ? slots.y : i == 2 ? slots.z : slots.w;
    trav_leaf<COUNT>(S, s, first, (counts >> (8 * i)) & 0xFFu, cnt);
  }
  if (ANY && s.rec != kMissRec) return true;
  const float inf2 = kInf * 2.f;
  if (!SORT && NEAREST) {
    float kmin = key[0];
    uint32_t next = kid[0];
    int jmin = 0;
#pragma unroll
    for (int j = 1; j < 4; j++) {
      if (key[j] < kmin) {
        kmin = key[j];
        next = kid[j];
        jmin = j;
      }
    }
    if (kmin < inf2 && kmin <= s.tmax * 1.0000010f) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (j != jmin && key[j] < inf2) {
          stk.put(s.sp, kid[j], key[j]);  // index below kStackSize: see the sorted push below
          s.sp = min(s.sp + 1, kStackSize - 1);
        }
      }
      s.entry = next;
      return false;
    }
    return !trav_pop_stk(s, stk);
  }
  if (!SORT) {
    // slot order: the first internal child hit is next, the others go on the stack
    uint32_t nxt = kNoEntry;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (key[j] < inf2) {
        if (nxt == kNoEntry) {
          nxt = kid[j];
        } else {
          stk.put(s.sp, kid[j], key[j]);  // index below kStackSize: see the push below
          s.sp = min(s.sp + 1, kStackSize - 1);
        }
      }
    }
    if (nxt != kNoEntry) {
      s.entry = nxt;
      return false;
    }
    return !trav_pop_stk(s, stk);
  }
#define OR3_CSWAP(a, b)                                       \
  if (key[b] < key[a]) {                                      \
    const float tk = key[a]; key[a] = key[b]; key[b] = tk;     \
    const uint32_t tc = kid[a]; kid[a] = kid[b]; kid[b] = tc;  \
  }
  OR3_CSWAP(0, 1) OR3_CSWAP(2, 3) OR3_CSWAP(0, 2) OR3_CSWAP(1, 3) OR3_CSWAP(1, 2)
#undef OR3_CSWAP
  const float tl2 = s.tmax * 1.0000010f;
  if (key[0] < inf2 && key[0] <= tl2) {
    // siblings beyond a hit found in this node's leaves are pruned when popped
#pragma unroll
    for (int j = 3; j >= 1; j--) {
      if (key[j] < inf2) {
        // at most 3 entries per wide level and wide depth <= kMaxBinaryDepth / 2
        // (checked at upload), so sp stays below kStackSize; the clamp keeps
        // the index in bounds without a branch
        stk.put(s.sp, kid[j], key[j]);
        s.sp = min(s.sp + 1, kStackSize - 1);
      }
    }
    s.entry = kid[0];
    return false;
  }
  return !trav_pop_stk(s, stk);
}

// One step over the 8-wide FP32-box nodes (S.fnodes8): the node's hit leaf
// children are tested in place, the nearest internal child is next and the
// others go on the stack (popped entries pruned by their entry distance).
// The stack holds kStackSize8 entries (bound checked when the tree is made).
template <bool ANY, bool COUNT, class STK>
__device__ __forceinline__ bool trav_step_w8(const DevScene &S, TravState &s, STK &stk, uint32_t *cnt) {
  const uint32_t e = s.entry;
  if (e == kNoEntry) return true;
  if (COUNT) cnt[0]++;
  const float4 *np = S.fnodes8 + 16 * (size_t)e;
  const uint32_t sx = s.signs & 1u, sy = (s.signs >> 1) & 1u, sz = (s.signs >> 2) & 1u;
  const uint4 c0 = __ldg(reinterpret_cast<const uint4 *>(np + 12));
  const uint4 c1 = __ldg(reinterpret_cast<const uint4 *>(np + 13));
  const uint4 mt = __ldg(reinterpret_cast<const uint4 *>(np + 14));
  const float tlimit = s.tmax * 1.0000010f;
  const float inf2 = kInf * 2.f;
  float key[8];
  uint32_t leafmask = 0;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const float4 bnx = __ldg(np + 2 * sx + h), bfx = __ldg(np + 2 * (sx ^ 1u) + h);
    const float4 bny = __ldg(np + 4 + 2 * sy + h), bfy = __ldg(np + 4 + 2 * (sy ^ 1u) + h);
    const float4 bnz = __ldg(np + 8 + 2 * sz + h), bfz = __ldg(np + 8 + 2 * (sz ^ 1u) + h);
    const float nxa[4] = {bnx.x, bnx.y, bnx.z, bnx.w}, fxa[4] = {bfx.x, bfx.y, bfx.z, bfx.w};
    const float nya[4] = {bny.x, bny.y, bny.z, bny.w}, fya[4] = {bfy.x, bfy.y, bfy.z, bfy.w};
    const float nza[4] = {bnz.x, bnz.y, bnz.z, bnz.w}, fza[4] = {bfz.x, bfz.y, bfz.z, bfz.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int c = 4 * h + i;
      const float tnx = fmaf(nxa[i], s.inv.x, s.oi.x), tfx = fmaf(fxa[i], s.inv.x, s.oi.x);
      const float tny = fmaf(nya[i], s.inv.y, s.oi.y), tfy = fmaf(fya[i], s.inv.y, s.oi.y);
      const float tnz = fmaf(nza[i], s.inv.z, s.oi.z), tfz = fmaf(fza[i], s.inv.z, s.oi.z);
      const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
      const float tf = fminf(fminf(fminf(tfx, tfy), tfz) * 1.0000010f, tlimit);
      const bool internal = (mt.z >> c) & 1u;
      const bool hitbox = tn <= tf;  // never for an empty slot
      key[c] = (hitbox && internal) ? tn : inf2;
      if (hitbox && !internal) leafmask |= 1u << c;
    }
  }
  while (leafmask) {
    const uint32_t i = __ffs(leafmask) - 1;
    leafmask &= leafmask - 1;
    const uint4 cw = i < 4 ? c0 : c1;
    const uint32_t j = i & 3u;
    const uint32_t first = j == 0 ? cw.x : j == 1 ? cw.y : j == 2 ? cw.z : cw.w;
    trav_leaf<COUNT>(S, s, first, ((i < 4 ? mt.x : mt.y) >> (8 * j)) & 0xFFu, cnt);
  }
  if (ANY && s.rec != kMissRec) return true;
  const uint32_t kids[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  float kmin = key[0];
  uint32_t next = kids[0];
  int jmin = 0;
#pragma unroll
  for (int j = 1; j < 8; j++) {
    if (key[j] < kmin) {
      kmin = key[j];
      next = kids[j];
      jmin = j;
    }
  }
  if (kmin < inf2 && kmin <= s.tmax * 1.0000010f) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (j != jmin && key[j] < inf2) {
        stk.put(s.sp, kids[j], key[j]);
        s.sp = min(s.sp + 1, kStackSize8 - 1);
      }
    }
    s.entry = next;
    return false;
  }
  return !trav_pop_stk(s, stk);
}

// After the BVH: the not-in-BVH objects, strictly closer only (Scene.cpp:73-83).
template <bool ANY>
__device__ __forceinline__ Hit trav_finish(const DevScene &S, const TravState &s) {
  Hit h;
  h.t = s.tmax;
  h.rec = s.rec;
  h.u = s.u;
  h.v = s.v;
  if (ANY && h.rec != kMissRec) return h;
  for (uint32_t p = 0; p < S.num_planes; p++) {
    float t;
    if (isect_plane(S.planes[p], s.o, s.d, h.t, t)) {
      h.t = t;
      h.rec = kPlaneBit | p;
      h.u = h.v = 0.f;
      if (ANY) return h;
    }
  }
  return h;
}

// Closest hit (ANY = false) or first hit (ANY = true) against the wide BVH
// and the not-in-BVH list.  Replaces Scene::CheckIntersection
// (src/scenes/Scene.cpp:51-85), BVH::CheckIntersection (src/renderer/BVH.cpp:19-88)
// and QBVH::CheckIntersection (src/renderer/QBVH.cpp:30-144):
//   * boxes are tested 4 at a time from one 64-byte node;
//   * leaf children are intersected as soon as their box is hit;
//   * internal children are visited nearest first, the others pushed with
//     their entry distance and pruned on pop against the best hit;
//   * a primitive replaces the best hit only if strictly closer, BVH first,
//     then the not-in-BVH objects, as in the reference.
// `nodes_smem`/`smem_nodes`: the first smem_nodes nodes may be read from
// shared memory instead of global.
// COUNT: adds nodes fetched, triangles and spheres tested to counts_out[0..2].
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ Hit trace(const DevScene &S, V3 o, V3 d, float tmax, uint32_t *err,
                                     const uint4 *nodes_smem = nullptr, uint32_t smem_nodes = 0,
                                     uint32_t *counts_out = nullptr) {
  Hit h;
  h.t = tmax;
  h.rec = kMissRec;
  h.u = h.v = 0.f;
  if (S.num_nodes > 0) {
    const V3 inv = v3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    const V3 oi = v3(-o.x * inv.x, -o.y * inv.y, -o.z * inv.z);
    // per axis: which byte word is the near plane
    const bool nx = inv.x < 0.f, ny = inv.y < 0.f, nz = inv.z < 0.f;
    uint32_t stack_node[kStackSize];
    float stack_t[kStackSize];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
      uint4 n0, n1, n2, n3;
      if (COUNT) counts_out[0]++;
      if (node < smem_nodes) {
        n0 = nodes_smem[4 * node + 0];
        n1 = nodes_smem[4 * node + 1];
        n2 = nodes_smem[4 * node + 2];
        n3 = nodes_smem[4 * node + 3];
      } else {
        const uint4 *np = S.nodes + 4 * (size_t)node;
        n0 = __ldg(np + 0);
        n1 = __ldg(np + 1);
        n2 = __ldg(np + 2);
        n3 = __ldg(np + 3);
      }
      const uint32_t ew = n0.w;
      const float sx = __uint_as_float((ew & 0xFFu) << 23);
      const float sy = __uint_as_float(((ew >> 8) & 0xFFu) << 23);
      const float sz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
      const uint32_t imask = ew >> 24;
      const float ax = sx * inv.x, ay = sy * inv.y, az = sz * inv.z;
      const float bx = fmaf(__uint_as_float(n0.x), inv.x, oi.x);
      const float by = fmaf(__uint_as_float(n0.y), inv.y, oi.y);
      const float bz = fmaf(__uint_as_float(n0.z), inv.z, oi.z);
      // byte words: lo x,y,z = n1.x,n1.y,n1.z ; hi x,y,z = n1.w,n2.x,n2.y
      const uint32_t wnx = nx ? n1.w : n1.x, wfx = nx ? n1.x : n1.w;
      const uint32_t wny = ny ? n2.x : n1.y, wfy = ny ? n1.y : n2.x;
      const uint32_t wnz = nz ? n2.y : n1.z, wfz = nz ? n1.z : n2.y;
      const uint32_t counts = n3.z;
      const float tlimit = h.t * 1.0000010f;
      float key[4];
      uint32_t kid[4];
      uint32_t leafmask = 0;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const float tnx = fmaf(qbyte(wnx, i), ax, bx), tfx = fmaf(qbyte(wfx, i), ax, bx);
        const float tny = fmaf(qbyte(wny, i), ay, by), tfy = fmaf(qbyte(wfy, i), ay, by);
        const float tnz = fmaf(qbyte(wnz, i), az, bz), tfz = fmaf(qbyte(wfz, i), az, bz);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
        const float tf = fminf(fminf(tfx, tfy), tfz) * 1.0000010f;
        const bool internal = (imask >> i) & 1u;
        const uint32_t cnt = (counts >> (8 * i)) & 0xFFu;
        const bool hitbox = tn <= tf && tn <= tlimit;
        const uint32_t ch = i == 0 ? n2.z : i == 1 ? n2.w : i == 2 ? n3.x : n3.y;
        key[i] = (hitbox && internal) ? tn : kInf * 2.f;
        kid[i] = ch;
        if (hitbox && !internal && cnt != 0u) leafmask |= 1u << i;
      }
      // leaf children: triangles then spheres
      while (leafmask) {
        const uint32_t i = __ffs(leafmask) - 1;
        leafmask &= leafmask - 1;
        const uint32_t first = i == 0 ? n2.z : i == 1 ? n2.w : i == 2 ? n3.x : n3.y;
        const uint32_t cnt = (counts >> (8 * i)) & 0xFFu;
        const uint32_t ntri = cnt & 15u, nsph = cnt >> 4;
        if (COUNT) {
          counts_out[1] += ntri;
          counts_out[2] += nsph;
        }
        for (uint32_t k = 0; k < ntri; k++) {
          const float4 *pr = S.prims + 3 * (size_t)(first + k);
          const float4 a = __ldg(pr), b = __ldg(pr + 1), c = __ldg(pr + 2);
          float t, u, v;
          if (isect_triangle(a, b, c, o, d, h.t, t, u, v)) {
            h.t = t;
            h.rec = first + k;
            h.u = u;
            h.v = v;
          }
        }
        for (uint32_t k = ntri; k < ntri + nsph; k++) {
          const float4 a = __ldg(S.prims + 3 * (size_t)(first + k));
          float t;
          if (isect_sphere(a, o, d, h.t, t)) {
            h.t = t;
            h.rec = first + k;
            h.u = h.v = 0.f;
          }
        }
        if (ANY && h.rec != kMissRec) return h;
      }
      // nearest-first order of the internal children hit (sorting network)
#define OR3_CSWAP(a, b)                                   \
  if (key[b] < key[a]) {                                  \
    const float tk = key[a]; key[a] = key[b]; key[b] = tk; \
    const uint32_t tc = kid[a]; kid[a] = kid[b]; kid[b] = tc; \
  }
      OR3_CSWAP(0, 1) OR3_CSWAP(2, 3) OR3_CSWAP(0, 2) OR3_CSWAP(1, 3) OR3_CSWAP(1, 2)
#undef OR3_CSWAP
      const float inf2 = kInf * 2.f;
      const float tl2 = h.t * 1.0000010f;
      bool advanced = false;
      if (key[0] < inf2 && key[0] <= tl2) {
#pragma unroll
        for (int j = 3; j >= 1; j--) {
          if (key[j] < inf2 && key[j] <= tl2) {
            if (sp < kStackSize) {
              stack_node[sp] = kid[j];
              stack_t[sp] = key[j];
              sp++;
            } else {
              atomicOr(err, 1u);  // cannot happen with builder depth bound
            }
          }
        }
        node = kid[0];
        advanced = true;
      }
      if (!advanced) {
        bool found = false;
        while (sp > 0) {
          sp--;
          if (stack_t[sp] <= h.t * 1.0000010f) {
            node = stack_node[sp];
            found = true;
            break;
          }
        }
        if (!found) break;
      }
    }
  }
  for (uint32_t p = 0; p < S.num_planes; p++) {
    float t;
    if (isect_plane(S.planes[p], o, d, h.t, t)) {
      h.t = t;
      h.rec = kPlaneBit | p;
      h.u = h.v = 0.f;
      if (ANY) return h;
    }
  }
  return h;
}

// Distance to the winning primitive re-evaluated in FP64 with the reference's
// own formulas (Polygon.h:63-106, Sphere.h:21-78, AxisAlignedPlane.h:38-64,
// InfiniteFloor.h:19-37).  The FP32 tests pick the primitive; one FP64
// evaluation per ray then gives the reference's distance on the same inputs
// even where FP32 is ill-conditioned (grazing exits, very short hops).
__device__ __forceinline__ float refine_t(const DevScene &S, const Hit &h, V3 of, V3 df) {
  if (h.rec == kMissRec) return h.t;
  const double ox = of.x, oy = of.y, oz = of.z, dx = df.x, dy = df.y, dz = df.z;
  double t;
  if (h.rec & kPlaneBit) {
    const PlaneRec &p = S.planes[h.rec & ~kPlaneBit];
    if (p.kind == kPrimFloor) {
      t = ((double)p.offset - oy) / dy;
    } else {
      const double dd = p.axis == 0 ? dz : p.axis == 1 ? dy : dx;
      const double oo = p.axis == 0 ? oz : p.axis == 1 ? oy : ox;
      t = ((double)p.offset - oo) / dd;
    }
  } else if ((S.info[h.rec].kind_flags & 0xFFu) == kPrimTriangle) {
    const float4 *pr = S.prims + 3 * (size_t)h.rec;
    const float4 a = __ldg(pr), b = __ldg(pr + 1), c = __ldg(pr + 2);
    const double e1x = a.w, e1y = b.x, e1z = b.y, e2x = b.z, e2y = b.w, e2z = c.x;
    const double px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
    const double det = px * e1x + py * e1y + pz * e1z;
    const double tx = ox - a.x, ty = oy - a.y, tz = oz - a.z;
    const double qx = ty * e1z - tz * e1y, qy = tz * e1x - tx * e1z, qz = tx * e1y - ty * e1x;
    t = (qx * e2x + qy * e2y + qz * e2z) / det;
  } else {
    const float4 s = __ldg(S.prims + 3 * (size_t)h.rec);
    const double cx = s.x - ox, cy = s.y - oy, cz = s.z - oz, r = s.w;
    const double b = dx * cx + dy * cy + dz * cz;
    const double D = b * b - (dx * dx + dy * dy + dz * dz) * (cx * cx + cy * cy + cz * cz - r * r);
    const double sq = sqrt(D > 0.0 ? D : 0.0);
    const double t1 = sq + b, t2 = -sq + b;
    t = t2 > (double)kEpsD ? t2 : t1;
  }
  // keep the FP32 result if the FP64 re-evaluation falls outside the accepted range
  return (t >= (double)kEpsD && t < 1e30) ? (float)t : h.t;
}

// Surface data at a hit, as HitInformation reports it (normal not yet
// oriented toward the ray, uv when a layer is textured).
struct Surface {
  V3 p;          // hit position orig + dir * t
  V3 n;          // hit.normal
  float uvx, uvy;
  uint32_t layer_begin, layer_count, object_id, flags, kind;
};

__device__ __forceinline__ Surface surface_at(const DevScene &S, const Hit &h, V3 o, V3 d) {
  Surface s;
  s.p = o + d * h.t;
  s.uvx = s.uvy = 0.f;
  if (h.rec & kPlaneBit) {
    const PlaneRec &pl = S.planes[h.rec & ~kPlaneBit];
    s.layer_begin = pl.layer_begin;
    s.layer_count = pl.layer_count;
    s.object_id = pl.object_id;
    s.flags = pl.flags;
    s.kind = pl.kind;
    if (pl.kind == kPrimFloor) {
      s.n = v3(0.f, d.y < 0.f ? 1.f : -1.f, 0.f);
    } else {
      s.n = pl.axis == 0 ? v3(0, 0, pl.normal_sign) : pl.axis == 1 ? v3(0, pl.normal_sign, 0) : v3(pl.normal_sign, 0, 0);
    }
    return s;
  }
  const PrimInfo inf = S.info[h.rec];
  s.layer_begin = inf.layer_begin;
  s.layer_count = inf.layer_count;
  s.object_id = inf.object_id;
  s.kind = inf.kind_flags & 0xFFu;
  s.flags = inf.kind_flags >> 8;
  if (s.kind == kPrimTriangle) {
    const float4 *ts = reinterpret_cast<const float4 *>(S.tri_shade + h.rec);
    const float4 a = __ldg(ts), b = __ldg(ts + 1), c = __ldg(ts + 2), e = __ldg(ts + 3);
    // n0=(a.xyz) dn1=(a.w,b.xy) dn2=(b.zw,c.x) uv0=(c.yz) duv1=(c.w,e.x) duv2=(e.yz)
    s.n = normalize(v3(fmaf(a.w, h.u, fmaf(b.z, h.v, a.x)), fmaf(b.x, h.u, fmaf(b.w, h.v, a.y)),
                       fmaf(b.y, h.u, fmaf(c.x, h.v, a.z))));
    if (s.flags & kFlagTexturedUV) {
      s.uvx = fmaf(c.w, h.u, fmaf(e.y, h.v, c.y));
      s.uvy = fmaf(e.x, h.u, fmaf(e.z, h.v, c.z));
    }
  } else {
    const float4 sp = __ldg(S.prims + 3 * (size_t)h.rec);
    s.n = normalize(v3(s.p.x - sp.x, s.p.y - sp.y, s.p.z - sp.z));
    if (s.flags & kFlagTexturedUV) {
      // lat-long uv (src/renderer/Sphere.h:61-75)
      float v = (asinf(fminf(fmaxf(s.n.y, -1.f), 1.f)) + kPi * 0.5f) / kPi;
      while (v > 1.f) v -= 1.f;
      while (v < 0.f) v += 1.f;
      float u = (atan2f(s.n.z, s.n.x) + kPi) / (2.f * kPi);
      while (u > 1.f) u -= 1.f;
      while (u < 0.f) u += 1.f;
      s.uvx = u;
      s.uvy = 1.f - v;
    }
  }
  return s;
}

// Image::GetPixelByUV (src/tools/Image.h:21-31): clamp, *0.99999, nearest.
__device__ __forceinline__ V3 texel(const DevScene &S, int tex, float u, float v) {
  const TextureDev td = S.textures[tex];
  u = fminf(fmaxf(u, 0.f), 1.f) * 0.99999f;
  v = fminf(fmaxf(v, 0.f), 1.f) * 0.99999f;
  const uint32_t x = (uint32_t)(u * (float)td.width), y = (uint32_t)(v * (float)td.height);
  const float *p = S.texels + td.offset + 3 * ((size_t)y * td.width + x);
  return v3(p[0], p[1], p[2]);
}

// IBL::Sample(dir) (src/renderer/IBL.h:30-45): nearest texel of the equirect map.
__device__ __forceinline__ V3 env_lookup(const DevScene &S, V3 d) {
  if (S.env == nullptr) return v3(S.bg[0], S.bg[1], S.bg[2]);
  const float theta = acosf(fminf(fmaxf(d.y, -1.f), 1.f));
  const float rxz = sqrtf(d.x * d.x + d.z * d.z);
  float phi = rxz > 0.f ? acosf(fminf(fmaxf(d.x / rxz, -1.f), 1.f)) : 0.f;
  if (d.z < 0.f) phi = 2.f * kPi - phi;
  const float u = phi / (2.f * kPi), v = theta / kPi;
  const uint32_t x = (uint32_t)(u * (float)S.env_w) % S.env_w;
  const uint32_t y = (uint32_t)(v * (float)S.env_h) % S.env_h;
  const float *p = S.env + 3 * ((size_t)y * S.env_w + x);
  return v3(p[0], p[1], p[2]);
}

}  // namespace or3
