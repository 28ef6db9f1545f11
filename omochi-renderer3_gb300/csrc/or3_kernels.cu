// or3_kernels.cu -- the wavefront path-tracing kernels.
//
// One bounce of the reference's recursive estimator (PathTracer::Radiance ->
// Radiance_internal -> Radiance_Lambert/Specular/Refraction,
// src/renderer/PathTracer.cpp:180-591) becomes
//     extend (closest hit for every queued ray)  ->  shade (one vertex of every path)
// over structure-of-arrays queues in HBM; the recursion's return values become
// a per-ray throughput and per-path radiance sums:
//   Radiance(r, d) = E_d + w_d * Radiance(r', d+1)  ==>  L += beta * E_d;  beta *= w_d
// The glass split at depth <= 2 (PathTracer.cpp:581-588) emits two child rays,
// each with its own share of the throughput.
#include <cuda_runtime.h>

#include "or3_kernels.cuh"

namespace or3 {

namespace {

__device__ __forceinline__ void add_radiance(float4 *L, V3 v) {
  if (v.x != 0.f) atomicAdd(&L->x, v.x);
  if (v.y != 0.f) atomicAdd(&L->y, v.y);
  if (v.z != 0.f) atomicAdd(&L->z, v.z);
}

__device__ __forceinline__ V3 ld3(const float4 &f) { return v3(f.x, f.y, f.z); }

// The queues with ray queue `in` in slot 0 and the other queue in slot 1.
// Kernels orient their Queues parameter once and then index the ray pointer
// pairs with constants only: indexing a parameter's array with a run-time
// value makes the compiler copy the whole struct to local memory and load
// every pointer from there.  Queue lengths stay indexed by the physical
// queue (counters[in], counters[out]).
__device__ __forceinline__ Queues oriented(const Queues &p, int in) {
  Queues q = p;
  const bool sw = in != 0;
  q.orig[0] = sw ? p.orig[1] : p.orig[0];
  q.orig[1] = sw ? p.orig[0] : p.orig[1];
  q.dir[0] = sw ? p.dir[1] : p.dir[0];
  q.dir[1] = sw ? p.dir[0] : p.dir[1];
  q.beta[0] = sw ? p.beta[1] : p.beta[0];
  q.beta[1] = sw ? p.beta[0] : p.beta[1];
  return q;
}

// Camera::SampleRayForPixel (src/renderer/Camera.h:65-93) for sub-pixel
// position (x + rx, y + ry), rx = (2 sx + 1) / (2 ss)
// (PathTracer::scanPixelsOnYAndCastRays, src/renderer/PathTracer.cpp:156-161).
__device__ __forceinline__ void camera_ray(const RenderConst &rc, uint32_t x, uint32_t y, uint32_t sx,
                                           uint32_t sy, uint32_t lens_key, uint32_t pass_first, V3 &o,
                                           V3 &d) {
  const Camera32 &c = rc.cam;
  const float inv2ss = 1.0f / (2.0f * (float)rc.ss);
  const float rx = (2.0f * (float)sx + 1.0f) * inv2ss;
  const float ry = (2.0f * (float)sy + 1.0f) * inv2ss;
  const float fx = ((float)x + rx) / (float)rc.W - 0.5f;
  const float fy = ((float)y + ry) / (float)rc.H - 0.5f;
  const V3 target = v3(c.center[0] + c.xaxis[0] * fx + c.yaxis[0] * fy,
                       c.center[1] + c.xaxis[1] * fx + c.yaxis[1] * fy,
                       c.center[2] + c.xaxis[2] * fx + c.yaxis[2] * fy);
  const V3 pos = v3(c.pos[0], c.pos[1], c.pos[2]);
  d = normalize(target - pos);
  o = pos;
  if (c.aperture > 0.f) {
    // CircleAperture::SampleOnePoint (src/renderer/Aperture.h:23-35): one lens
    // sample per sub-pixel per pass, as the reference reuses its camera ray
    // for every sample of a pass (PathTracer.cpp:161-167).
    const uint4 r = philox(make_uint4(lens_key, pass_first, 0u, 1u), rc.seed_lo, rc.seed_hi);
    float sn, cs;
    sincospif(2.0f * u01(r.x), &sn, &cs);
    const float rr = c.aperture * sqrtf(u01(r.y));
    const float tf = c.focal / fabsf(d.z);
    const V3 focus = pos + d * tf;
    o = v3(pos.x + rr * cs, pos.y + rr * sn, pos.z);
    d = normalize(focus - o);
  }
}

__global__ void k_raygen(RenderConst rc, Wave w, Queues qp, int out) {
  const Queues q = oriented(qp, out);  // the queue written is slot 0
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    q.counters[out] = w.num_paths;
    q.counters[4 + out] = 0;  // extend fetch counter of this queue
  }
  if (i >= w.num_paths) return;
  const uint64_t g = w.g_first + i;
  const uint32_t sub = (uint32_t)(g % rc.ss2);
  const uint64_t pg = g / rc.ss2;
  const uint32_t pix = (uint32_t)(pg % ((uint64_t)rc.W * rc.H));
  const uint32_t x = pix % rc.W, y = pix / rc.W;
  V3 o, d;
  camera_ray(rc, x, y, sub % rc.ss, sub / rc.ss, pix * rc.ss2 + sub, w.pass_first, o, d);
  q.orig[0][i] = make_float4(o.x, o.y, o.z, __uint_as_float(i));
  q.dir[0][i] = make_float4(d.x, d.y, d.z, __uint_as_float(0u));
  q.beta[0][i] = make_float4(1.f, 1.f, 1.f, 0.f);
  q.pathL[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

constexpr int kSmemNodes = 256;  // top nodes staged in shared memory (16 KB)
// Node steps a lane takes between two warp votes of the persistent traversal
// (persistent_trace): the vote, the refill test and the loop's branches are
// paid once per pair (measured: extend -3% on the mesh, shadow -2% on the
// terrain; 3 and 4 steps spill at 64 registers and are slower).  The batched
// extend takes two where it reads each step's node array through the ray's
// scene descriptor (its default); with the array held in registers the pair
// spills (-1.5%) and it takes one.
constexpr int kStepsPerVote = 2;
// The shadow kernel (fewer live registers: no hit record to keep) takes three.
constexpr int kShadowStepsPerVote = 3;

// Persistent traversal over a ray source: every lane traces one ray at a time
// and takes the next one the moment its ray is finished (warp-aggregated
// fetch from a global counter that starts at zero), so no lane idles behind
// the slowest ray of a fixed batch and the grid has no tail of its own.
// All 32 lanes of every warp must enter (blockDim is a multiple of 32).
// STEP 1: one node or one leaf per step (leaves go through the stack), refill
//         any idle lane every step;
// STEP 2: one node per step with its hit leaves tested in place, up to
//         VOTE_STEPS steps per vote, refill only once at least half of
//         the warp is idle (amortises the atomic).
// REFILL (STEP 2): refill once at least this many lanes are idle.  SORT:
// nearest-first child order (off only for any-hit queries).  FN: STEP 2 over
// the FP32-box nodes (else the quantised ones).
template <bool ANY, bool COUNT, int STEP, class Src, class Sink, int REFILL = 16, bool SORT = true, bool FN = true,
          bool NEAREST = false, bool W8 = false, int VOTE_STEPS = kStepsPerVote>
__device__ __forceinline__ void persistent_trace(const DevScene &S, uint32_t n, uint32_t *fetch, const Src &src,
                                                 const Sink &sink, const uint4 *snodes, uint32_t ns, uint32_t *cnt,
                                                 uint32_t *err) {
  uint32_t stk_e[kStackSize];
  float stk_t[kStackSize];
  uint2 stk_p[W8 ? kStackSize8 : kStackSize];
  PairStack stk{stk_p};
  TravState st;
  uint32_t r = kNoEntry;
  bool drained = false;  // warp-uniform: the shared fetch counter has passed n
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    // one vote per step: the idle lanes
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, r == kNoEntry);
    if (!drained && idle != 0u && (STEP == 1 || __popc(idle) >= REFILL || idle == 0xFFFFFFFFu)) {
      const int leader = __ffs(idle) - 1;
      const uint32_t want = (uint32_t)__popc(idle);
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, want);
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      const uint32_t idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
      if (r == kNoEntry && idx < n) {
        V3 o, d;
        float tmax;
        src.load(idx, o, d, tmax);
        trav_init(st, o, d, tmax, S.num_nodes);
        r = idx;
      }
      drained = base + want >= n;
    } else if (drained && idle == 0xFFFFFFFFu) {
      break;
    }
    if (r != kNoEntry) {
      // STEP 2 takes up to VOTE_STEPS node steps per vote (a lane whose ray
      // ends early sits out the rest)
      constexpr int kSteps = STEP == 2 && !W8 ? VOTE_STEPS : 1;
      bool done = false;
#pragma unroll
      for (int k = 0; k < kSteps; k++) {
        if (done) break;
        done = W8          ? trav_step_w8<ANY, COUNT>(S, st, stk, cnt)
               : STEP == 1 ? trav_step<ANY, COUNT>(S, st, stk_e, stk_t, snodes, ns, cnt, err)
                           : trav_step_inline<ANY, COUNT, SORT, PairStack, FN, DevScene, NEAREST>(
                                 S, st, stk, snodes, ns, cnt, err);
      }
      if (done) {
        sink.store(S, r, trav_finish<ANY>(S, st), st.o, st.d);
        r = kNoEntry;
      }
    }
  }
}

struct QueueSrc {
  const float4 *orig, *dir;
  __device__ __forceinline__ void load(uint32_t i, V3 &o, V3 &d, float &tmax) const {
    o = ld3(orig[i]);
    d = ld3(dir[i]);
    tmax = kInf;
  }
};

// The render keeps the FP32 distance: GB300 runs FP64 at a small fraction of
// the FP32 rate, and one FP64 re-evaluation per ray cost more than the whole
// traversal (measured: 2.7x slower extend).  The ray-query API refines.
struct HitSink {
  float4 *hits;
  __device__ __forceinline__ void store(const DevScene &, uint32_t i, Hit h, V3, V3) const {
    hits[i] = make_float4(h.t, __uint_as_float(h.rec), h.u, h.v);
  }
};

__device__ __forceinline__ uint32_t stage_nodes(const DevScene &S, uint4 *snodes, int smem_nodes) {
  const uint32_t ns = min((uint32_t)smem_nodes, S.num_nodes);
  if (ns > 0) {
    for (uint32_t k = threadIdx.x; k < ns * 4; k += blockDim.x) snodes[k] = S.nodes[k];
    __syncthreads();
  }
  return ns;
}

// One thread per ray over a grid-stride loop; the whole traversal of a ray
// (trace) runs in one go.
template <bool ANY, bool COUNT, class Src, class Sink>
__device__ __forceinline__ void gridstride_trace(const DevScene &S, uint32_t n, const Src &src, const Sink &sink,
                                                 const uint4 *snodes, uint32_t ns, uint32_t *cnt, uint32_t *err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V3 o, d;
    float tmax;
    src.load(i, o, d, tmax);
    const Hit h = trace<ANY, COUNT>(S, o, d, tmax, err, snodes, ns, cnt);
    sink.store(S, i, h, o, d);
  }
}

// Closest hit for every queued ray.  COUNT adds the nodes, triangles and
// spheres each ray touched to stats[3..5] (the algorithmic byte count).
// VARIANT 0: gridstride_trace; 1: persistent_trace STEP 1; 2, 4, 5: STEP 2
// refilling at 16, 8 or 24 idle lanes; 6: STEP 2 over the quantised nodes;
// 7: STEP 2, nearest internal child next and its siblings pushed unsorted;
// 8: the 8-wide nodes (S.fnodes8), as 7.
// 0, 1 and 6 read the quantised nodes (and may stage the top ones in shared
// memory), 2, 4 and 5 the FP32-box nodes.
template <bool COUNT, int VARIANT>
__device__ __forceinline__ void extend_body(const DevScene &S, const Queues &q, int in, int smem_nodes,
                                            uint4 *snodes);

template <bool COUNT, int VARIANT>
__global__ void __launch_bounds__(256, 4) k_extend(DevScene S, Queues q, int in, int smem_nodes) {
  __shared__ uint4 snodes[kSmemNodes * 4];
  extend_body<COUNT, VARIANT>(S, oriented(q, in), in, smem_nodes, snodes);
}

template <bool COUNT, int VARIANT>
__device__ __forceinline__ void extend_body(const DevScene &S, const Queues &q, int in, int smem_nodes,
                                            uint4 *snodes) {
  const uint32_t n = min(q.counters[in], q.capacity);  // an overflowed queue (error bit set) is read to capacity only
  const uint32_t ns = stage_nodes(S, snodes, smem_nodes);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&q.stats[0], (unsigned long long)n);
    if (n) atomicAdd(&q.stats[2], 1ull);
  }
  uint32_t cnt[3] = {0u, 0u, 0u};
  if (VARIANT == 0) {
    gridstride_trace<false, COUNT>(S, n, QueueSrc{q.orig[0], q.dir[0]}, HitSink{q.hits}, snodes, ns, cnt,
                                   &q.counters[2]);
  } else {
    constexpr int kStep = VARIANT == 1 ? 1 : 2;
    constexpr int kRefill = VARIANT == 4 ? 8 : VARIANT == 5 ? 24 : 16;
    persistent_trace<false, COUNT, kStep, QueueSrc, HitSink, kRefill, VARIANT != 7, VARIANT != 6, VARIANT == 7,
                     VARIANT == 8>(
        S, n, &q.counters[4 + in], QueueSrc{q.orig[0], q.dir[0]}, HitSink{q.hits}, snodes, ns, cnt,
        &q.counters[2]);
  }
  if (COUNT) {
    unsigned long long c0 = cnt[0], c1 = cnt[1], c2 = cnt[2];
#pragma unroll
    for (int ofs = 16; ofs > 0; ofs >>= 1) {
      c0 += __shfl_xor_sync(0xFFFFFFFFu, c0, ofs);
      c1 += __shfl_xor_sync(0xFFFFFFFFu, c1, ofs);
      c2 += __shfl_xor_sync(0xFFFFFFFFu, c2, ofs);
    }
    if ((threadIdx.x & 31u) == 0) {
      atomicAdd(&q.stats[3], c0);
      atomicAdd(&q.stats[4], c1);
      atomicAdd(&q.stats[5], c2);
    }
  }
}

struct NewRay {
  V3 o, d, beta;
  uint32_t meta;
};

struct ShadowRay {
  V3 o, d, c;  // c: radiance the path gains if nothing lies on [o, o + d * tmax)
  float tmax;
};

// orthonormal basis {t1, t2, a} about unit a (Duff et al., "Building an
// Orthonormal Basis, Revisited", JCGT 2017)
__device__ __forceinline__ V3 onb_t1(V3 a) {
  const float sg = a.z >= 0.f ? 1.0f : -1.0f;
  const float aa = -1.0f / (sg + a.z);
  return v3(1.0f + sg * a.x * a.x * aa, sg * a.x * a.y * aa, -sg * a.x);
}
__device__ __forceinline__ V3 onb_t2(V3 a) {
  const float sg = a.z >= 0.f ? 1.0f : -1.0f;
  const float aa = -1.0f / (sg + a.z);
  return v3(a.x * a.y * aa, sg + a.y * a.y * aa, -a.y);
}

// first index whose inclusive CDF value exceeds u (u < 1 = cdf[n - 1])
__device__ __forceinline__ uint32_t cdf_find(const float *cdf, uint32_t n, float u) {
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid) > u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// cdf_find through a guide table (the cutpoint method of Chen and Asau,
// 1974): guide[k] is the first index whose CDF value exceeds k / n (n - 1
// if none), k = 0..n.  u in cell k = floor(u n) has its answer between
// guide[k - 1] and guide[k + 2]: the one-cell margins cover the rounding of
// u n and of k / n, so the result is cdf_find's, in a few steps instead of
// log2(n).
__device__ __forceinline__ uint32_t cdf_find_guided(const float *cdf, const uint32_t *guide, uint32_t n, float u) {
  const uint32_t k = min((uint32_t)(u * (float)n), n - 1u);
  uint32_t lo = __ldg(guide + (k ? k - 1u : 0u)), hi = __ldg(guide + min(k + 2u, n));
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid) > u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// BRDF times colour of the vertex: Lambert rho/pi, or the Phong lobe
// rho (n+2)/(2 pi) cos^n about the mirror direction.
struct Brdf {
  V3 col, mirror;
  float exponent;
  bool phong;
  __device__ __forceinline__ V3 eval(V3 d) const {
    if (!phong) return col * (1.0f / kPi);
    const float c = dot(d, mirror);
    return col * ((exponent + 2.0f) / (2.0f * kPi) * (c > 0.f ? powf(c, exponent) : 0.f));
  }
};

// One next-event light sample seen from x (oriented normal nl), with the
// draws (rl.x select, rl.y / rl.z position).  The reference's
// DirectRadiance_Lambert (src/renderer/PathTracer.cpp:239-323) picks a
// SphereLight by TotalPower and samples its visible cap
// (SphereLight::SampleOnePointWithTargetPoint, src/renderer/SphereLight.h:39-69),
// but weights the sample by the receiver's emission, which is zero there.
// This samples what it describes, with the light's own emission, and adds
// emissive triangles (uniform by area) and the environment (marginal /
// conditional CDF over the equirect map, or cosine-weighted directions about
// nl for a constant background).  c = brdf * Le * cos * G / (pdf * p_select).
__device__ __forceinline__ bool sample_light(const DevScene &S, uint4 rl, V3 x, V3 nl, const Brdf &b,
                                             ShadowRay &sr) {
  const float usel = u01(rl.x), u1 = u01(rl.y), u2 = u01(rl.z);
  sr.o = x;
  if (usel < S.env_prob) {
    V3 d, le;
    float pdf;
    if (S.env_light == 1) {
      const uint32_t W = S.env_w, H = S.env_h;
      const uint32_t i = cdf_find_guided(S.env_marg, S.env_gmarg, H, u1);
      const float prev = i ? __ldg(S.env_marg + i - 1) : 0.f, pr = __ldg(S.env_marg + i) - prev;
      const float *row = S.env_cond + (size_t)i * W;
      const uint32_t j = cdf_find_guided(row, S.env_gcond + (size_t)i * (W + 1), W, u2);
      const float prevc = j ? __ldg(row + j - 1) : 0.f, pc = __ldg(row + j) - prevc;
      const float u = ((float)j + (u2 - prevc) / pc) / (float)W;
      const float v = ((float)i + (u1 - prev) / pr) / (float)H;
      float sp, cp, st, ct;
      sincospif(2.0f * u, &sp, &cp);
      sincospif(v, &st, &ct);
      if (!(st > 0.f)) return false;
      d = v3(st * cp, ct, st * sp);
      pdf = pr * pc * (float)W * (float)H / (2.0f * kPi * kPi * st);
      const float *p = S.env + 3 * ((size_t)i * W + j);
      le = v3(p[0], p[1], p[2]);
    } else {
      // constant background: cosine-weighted about the receiver's normal
      const V3 t1 = onb_t1(nl), t2 = onb_t2(nl);
      const float ct = sqrtf(u1), st = sqrtf(1.0f - u1);
      float sp, cp;
      sincospif(2.0f * u2, &sp, &cp);
      d = t1 * (st * cp) + t2 * (st * sp) + nl * ct;
      pdf = ct * (1.0f / kPi);
      if (!(pdf > 0.f)) return false;
      le = v3(S.bg[0], S.bg[1], S.bg[2]);
    }
    const float cs = dot(d, nl);
    if (!(cs > 0.f)) return false;
    sr.d = d;
    sr.tmax = kInf;
    sr.c = b.eval(d) * le * (cs / (pdf * S.env_prob));
    return true;
  }
  if (S.num_lights == 0) return false;
  const float ul = S.env_prob > 0.f ? (usel - S.env_prob) / (1.0f - S.env_prob) : usel;
  const uint32_t k = cdf_find(S.light_cdf, S.num_lights, ul);
  const float psel = (1.0f - S.env_prob) * __ldg(S.light_pdf + k);
  if (!(psel > 0.f)) return false;
  const float4 *lp = reinterpret_cast<const float4 *>(S.lights + k);
  const float4 q0 = __ldg(lp), q1 = __ldg(lp + 1), q2 = __ldg(lp + 2), q3 = __ldg(lp + 3);
  V3 p;
  float pdf_a, cl;
  V3 d;
  float dist2;
  if (__float_as_uint(q0.w) == kLightTriangle) {
    // uniform over the triangle (sqrt warping of the barycentrics)
    const V3 v0 = v3(q0.x, q0.y, q0.z), e1 = v3(q1.x, q1.y, q1.z), e2 = v3(q2.x, q2.y, q2.z);
    const float su = sqrtf(u1);
    p = v0 + e1 * (su * (1.0f - u2)) + e2 * (su * u2);
    const V3 ng = cross(e1, e2);
    const float ln = sqrtf(dot(ng, ng));
    pdf_a = 2.0f / ln;
    const V3 L = p - x;
    dist2 = dot(L, L);
    d = L * rsqrtf(dist2);
    // the face is only ever hit from its front (Polygon::CheckIntersection's det > EPS)
    const float det = -dot(d, ng);
    if (!(det > kEps)) return false;
    cl = det / ln;
  } else {
    // uniform over the cap of the sphere visible from x
    const V3 c = v3(q0.x, q0.y, q0.z);
    const float r = q1.w;
    const V3 diff = x - c;
    const float dd = sqrtf(dot(diff, diff)), cmax = r / dd;
    if (!(cmax < 1.0f)) return false;  // x inside the light (the reference skips it too)
    const V3 ax = diff * (1.0f / dd);
    const V3 t1 = onb_t1(ax), t2 = onb_t2(ax);
    const float ct = 1.0f - (1.0f - cmax) * u1, st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    const V3 nlight = ax * ct + t1 * (st * cp) + t2 * (st * sp);
    p = c + nlight * r;
    pdf_a = 1.0f / (2.0f * kPi * r * r * (1.0f - cmax));
    const V3 L = p - x;
    dist2 = dot(L, L);
    d = L * rsqrtf(dist2);
    cl = -dot(d, nlight);
    if (!(cl > 0.f)) return false;
  }
  const float cs = dot(d, nl);
  if (!(cs > 0.f)) return false;
  sr.d = d;
  sr.tmax = sqrtf(dist2) * (1.0f - 1e-3f);
  sr.c = b.eval(d) * v3(q3.x, q3.y, q3.z) * (cs * cl / (dist2 * pdf_a * psel));
  return true;
}

// The layer a vertex uses: the roulette over the object's layer rates
// (PathTracer.cpp:370-382), val uniform in [0, 1).
__device__ __forceinline__ uint32_t pick_layer(const DevScene &S, uint32_t begin, uint32_t count, float val) {
  uint32_t sel = count - 1;
  for (uint32_t k = 0; k < count; k++) {
    const float rate = S.layers[begin + k].rate;
    if (val <= rate) {
      sel = k;
      break;
    }
    val -= rate;
  }
  return sel;
}

// One path vertex: PathTracer::Radiance_internal (src/renderer/PathTracer.cpp:349-442)
// and the three BSDFs (:445-591).  Writes 0, 1 or 2 continuation rays, and
// with next-event estimation on, at most one shadow ray (has_sr).  NEE
// compiles the light-sampling code in (a separate instance keeps the
// registers of the plain shade kernel at their NEE-free count).
template <bool NEE>
__device__ __forceinline__ int shade_one(const DevScene &S, const RenderConst &rc, const Wave &w,
                                         const Queues &q, int in, uint32_t i, NewRay &r0, NewRay &r1,
                                         ShadowRay &sr, bool &has_sr) {
  const float4 ro = q.orig[0][i], rd = q.dir[0][i], rb = q.beta[0][i], hh = q.hits[i];
  const V3 o = ld3(ro), d = ld3(rd);
  V3 beta = ld3(rb);
  const uint32_t path = __float_as_uint(ro.w);
  const uint32_t meta = __float_as_uint(rd.w);
  const uint32_t depth = meta & 0xFFFFu;
  const uint32_t leaf = (meta >> 16) & 0xFFu;
  float4 *L = q.pathL + path;
  Hit h;
  h.t = hh.x;
  h.rec = __float_as_uint(hh.y);
  h.u = hh.z;
  h.v = hh.w;
  // With next-event estimation a vertex that sampled a light (Lambert,
  // Phong) does not also count the emission its BSDF ray reaches; a camera
  // or mirror/glass ray (depth 0 or kMetaSpec) still does.  The reference
  // instead counts emission at the eye vertex only (PathTracer.cpp:433-439).
  const bool after_light_sample = rc.nee && depth > 0 && !(meta & kMetaSpec);
  if (h.rec == kMissRec) {
    // miss: IBL::Sample(ray.dir) or Scene::Background() (PathTracer.cpp:357-364)
    if (!after_light_sample) add_radiance(L, beta * env_lookup(S, d));
    return 0;
  }
  const Surface s = surface_at(S, h, o, d);
  // normal oriented toward the incoming ray (PathTracer.cpp:188-190)
  const V3 nl = dot(s.n, d) < 0.f ? s.n : s.n * -1.f;
  const uint4 rn = philox(path_counter(w.g_first + path, leaf, depth, 0u), rc.seed_lo, rc.seed_hi);

  // material layer roulette (PathTracer.cpp:370-382)
  const uint32_t sel = pick_layer(S, s.layer_begin, s.layer_count, u01(rn.x));
  const MaterialDev &m = S.materials[S.layers[s.layer_begin + sel].material];
  V3 col = v3(m.color[0], m.color[1], m.color[2]);
  if (m.texture >= 0) col = col * texel(S, m.texture, s.uvx, s.uvy);  // GetTexturedColor (:327-346)

  // emission: at every vertex without NEE (PathTracer.cpp:404-411, :433-439);
  // with NEE not where a light sample already covered it (in-BVH emitters
  // are the lights; planes are not)
  const bool is_light = !(h.rec & kPlaneBit) && (s.flags & kFlagEmissive);
  if (m.emissive && !(after_light_sample && is_light))
    add_radiance(L, beta * v3(m.emission[0], m.emission[1], m.emission[2]));

  // Russian roulette (PathTracer.cpp:398-416)
  float prr = fmaxf(col.x, fmaxf(col.y, col.z));
  if (depth > 64u) prr *= exp2f(-(float)(depth - 64u));
  if ((int)depth > rc.rr_min_depth) {
    if (u01(rn.y) >= prr) return 0;
  } else {
    prr = 1.0f;
  }
  // hard depth cut (not in the reference): rays at depth >= max_depth are not traced
  if (rc.max_depth > 0 && (int)depth + 1 >= rc.max_depth) return 0;

  const uint32_t nmeta = (depth + 1u) | (leaf << 16);
  r0.o = s.p;
  r0.meta = nmeta;
  // next-event estimation at a Lambert or Phong vertex that survived Russian
  // roulette; the sample is weighted 1/p_rr like the reference's direct term
  // (Radiance_Lambert, PathTracer.cpp:453-500)
  if (NEE && rc.nee && ((m.type == OR3_LAMBERT && !m.emissive) || m.type == OR3_PHONG)) {
    Brdf b;
    b.col = col;
    b.phong = m.type == OR3_PHONG;
    b.exponent = m.phong_exponent;
    b.mirror = normalize(d - nl * (2.0f * dot(d, nl)));
    const uint4 rl = philox(path_counter(w.g_first + path, leaf, depth, 2u), rc.seed_lo, rc.seed_hi);
    if (sample_light(S, rl, s.p, nl, b, sr)) {
      sr.c = sr.c * beta * (1.0f / prr);
      has_sr = sr.c.x > 0.f || sr.c.y > 0.f || sr.c.z > 0.f;
    }
  }
  switch (m.type) {
    case OR3_LAMBERT: {
      // Radiance_Lambert (PathTracer.cpp:445-500).  An emitter does not
      // continue.  The tangent vectors are the reference's unnormalised
      // cross products (:461-469), so the sampled density matches its
      // estimator exactly, including for normals off the coordinate axes.
      if (m.emissive) return 0;
      const V3 ww = nl;
      const V3 uu = fabsf(ww.x) > kEps ? cross(v3(0.f, 1.f, 0.f), ww) : cross(v3(1.f, 0.f, 0.f), ww);
      const V3 vv = cross(ww, uu);
      float sn, cs;
      sincospif(2.0f * u01(rn.z), &sn, &cs);
      const float u2 = u01(rn.w);
      const float r2 = sqrtf(u2), r3 = sqrtf(1.0f - u2);
      r0.d = normalize(uu * (r3 * cs) + vv * (r3 * sn) + ww * r2);
      r0.beta = beta * col * (1.0f / prr);
      return 1;
    }
    case OR3_SPECULAR: {
      // Radiance_Specular (PathTracer.cpp:503-520)
      r0.d = normalize(d - nl * (2.0f * dot(d, nl)));
      r0.beta = beta * col * (1.0f / prr);
      r0.meta = nmeta | kMetaSpec;
      return 1;
    }
    case OR3_REFRACTION: {
      // Radiance_Refraction (PathTracer.cpp:523-591)
      r0.meta = nmeta | kMetaSpec;
      const bool into = dot(s.n, nl) > 0.f;
      const V3 refl = normalize(d - nl * (2.0f * dot(d, nl)));
      const float nobj = m.ior;
      const float nratio = into ? 1.0f / nobj : nobj;
      const float dd = dot(d, nl);
      const float cos2t = 1.0f - nratio * nratio * (1.0f - dd * dd);
      if (cos2t < 0.f) {
        // total internal reflection: weight uses material.color (:543-548)
        r0.d = refl;
        r0.beta = beta * v3(m.color[0], m.color[1], m.color[2]) * (1.0f / prr);
        return 1;
      }
      const V3 refr = normalize(d * nratio - nl * (dd * nratio + sqrtf(cos2t)));
      const float F0 = (nobj - 1.0f) * (nobj - 1.0f) / ((nobj + 1.0f) * (nobj + 1.0f));
      const float c = 1.0f - (into ? -dd : -dot(refr, nl));
      const float c2 = c * c;
      const float Fr = F0 + (1.0f - F0) * c2 * c2 * c;
      const float Tr = (1.0f - Fr) * nratio * nratio;
      if (depth > 2u) {
        const uint4 rn2 = philox(path_counter(w.g_first + path, leaf, depth, 1u), rc.seed_lo, rc.seed_hi);
        const float pr = 0.1f + 0.8f * Fr;
        if (u01(rn2.x) < pr) {
          r0.d = refl;
          r0.beta = beta * col * (Fr / (prr * pr));
        } else {
          r0.d = refr;
          r0.beta = beta * col * (Tr / (prr * (1.0f - pr)));
        }
        return 1;
      }
      // depth <= 2: trace both, each child with its own leaf bit
      r0.d = refl;
      r0.beta = beta * col * (Fr / prr);
      r1.o = s.p;
      r1.d = refr;
      r1.beta = beta * col * (Tr / prr);
      r1.meta = (depth + 1u) | ((leaf | (1u << depth)) << 16) | kMetaSpec;
      return 2;
    }
    default: {
      // Phong lobe about the mirror direction (not in the reference):
      // pdf = (n+1)/(2 pi) cos^n(a), brdf = rho (n+2)/(2 pi) cos^n(a),
      // weight = rho (n+2)/(n+1) cos(theta).
      const V3 r = normalize(d - nl * (2.0f * dot(d, nl)));
      const float e = m.phong_exponent;
      const float ca = powf(u01(rn.z), 1.0f / (e + 1.0f));
      const float sa = sqrtf(fmaxf(0.f, 1.0f - ca * ca));
      float sn, cs;
      sincospif(2.0f * u01(rn.w), &sn, &cs);
      const V3 wi = normalize(onb_t1(r) * (sa * cs) + onb_t2(r) * (sa * sn) + r * ca);
      const float cosn = dot(wi, nl);
      if (cosn <= 0.f) return 0;
      r0.d = wi;
      r0.beta = beta * col * ((e + 2.0f) / (e + 1.0f) * cosn / prr);
      return 1;
    }
  }
}

__device__ __forceinline__ uint32_t find_segment(const Segment *segs, uint32_t nseg, uint32_t wave_index) {
  uint32_t lo = 0, hi = nseg;  // last segment with wave_first <= wave_index
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (segs[mid].wave_first <= wave_index) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Writes continuation ray r at position pos of the output queue (slot 1 of an
// oriented q; a position past the capacity sets the queue error bit and
// drops the ray).
__device__ __forceinline__ void append_ray(const Queues &q, uint32_t pos, const NewRay &r,
                                           uint32_t pathbits, uint32_t tag) {
  if (pos >= q.capacity) {
    atomicOr(&q.counters[2], kErrQueue);
    return;
  }
  q.orig[1][pos] = make_float4(r.o.x, r.o.y, r.o.z, __uint_as_float(pathbits));
  q.dir[1][pos] = make_float4(r.d.x, r.d.y, r.d.z, __uint_as_float(r.meta));
  q.beta[1][pos] = make_float4(r.beta.x, r.beta.y, r.beta.z, __uint_as_float(tag));
}

// Shades queue entry i when `valid` and appends its continuation and shadow
// rays (warp-aggregated: every lane of the warp calls this together).
// BATCH: the ray's segment (beta.w) selects the job's scene, constants and
// RNG numbering; continuation rays inherit it.  BLK: block-aggregated
// appends (one atomic per queue and block iteration instead of per warp; the
// queue lengths are single addresses every warp updates); every thread of
// the block calls this together.
template <bool BATCH, bool NEE, bool BLK = false>
__device__ __forceinline__ void shade_item(const DevScene &S0, const RenderConst &rc0, const Wave &w0,
                                           const Queues &q, int in, const Batch &b, bool valid, uint32_t i) {
  const int out = in ^ 1;
  const uint32_t lane = threadIdx.x & 31u;
  NewRay r0, r1;
  ShadowRay sr;
  bool has_sr = false;
  int cnt = 0;
  uint32_t tag = 0;
  if (valid) {
    if (BATCH) {
      tag = __float_as_uint(q.beta[0][i].w);
      const Segment sg = b.segs[tag];
      const JobDev &job = b.jobs[sg.job];
      Wave w = w0;
      w.g_first = sg.g_first - sg.wave_first;
      cnt = shade_one<NEE>(b.scenes[job.scene], job.rc, w, q, in, i, r0, r1, sr, has_sr);
    } else {
      cnt = shade_one<NEE>(S0, rc0, w0, q, in, i, r0, r1, sr, has_sr);
    }
  }
  const unsigned sm = NEE ? __ballot_sync(0xFFFFFFFFu, has_sr) : 0u;
  int incl = cnt;  // inclusive scan of the warp's continuation rays
#pragma unroll
  for (int ofs = 1; ofs < 32; ofs <<= 1) {
    const int v = __shfl_up_sync(0xFFFFFFFFu, incl, ofs);
    if ((int)lane >= ofs) incl += v;
  }
  const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  uint32_t sbase = 0, wbase = 0;
  if (BLK) {
    __shared__ uint32_t bc[2][8], bb[2];  // per queue: warp counts (then offsets), the block's base
    const uint32_t warp = threadIdx.x >> 5;
    if (lane == 0) {
      bc[0][warp] = (uint32_t)total;
      bc[1][warp] = (uint32_t)__popc(sm);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      const uint32_t c = threadIdx.x;
      uint32_t t = 0;
      for (uint32_t k = 0; k < (blockDim.x >> 5); k++) {
        const uint32_t v = bc[c][k];
        bc[c][k] = t;
        t += v;
      }
      bb[c] = t ? atomicAdd(&q.counters[c == 0 ? out : 3], t) : 0u;
    }
    __syncthreads();
    wbase = bb[0] + bc[0][warp];
    sbase = bb[1] + bc[1][warp];
    __syncthreads();  // bc / bb are rewritten by the next call
  } else {
    if (sm) {
      const int leader = __ffs(sm) - 1;
      if ((int)lane == leader) sbase = atomicAdd(&q.counters[3], (uint32_t)__popc(sm));
      sbase = __shfl_sync(0xFFFFFFFFu, sbase, leader);
    }
    if (lane == 31 && total > 0) wbase = atomicAdd(&q.counters[out], (uint32_t)total);
    wbase = __shfl_sync(0xFFFFFFFFu, wbase, 31);
  }
  // append to the shadow queue
  if (sm) {
    if (has_sr) {
      const uint32_t pos = sbase + (uint32_t)__popc(sm & ((1u << lane) - 1u));
      if (pos < q.capacity) {
        q.sorig[pos] = make_float4(sr.o.x, sr.o.y, sr.o.z, q.orig[0][i].w);
        q.sdir[pos] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.tmax);
        q.scontrib[pos] = make_float4(sr.c.x, sr.c.y, sr.c.z, __uint_as_float(tag));
      } else {
        atomicOr(&q.counters[2], kErrQueue);
      }
    }
  }
  // append to the output queue (each ray written by name, so neither needs an
  // addressable copy in local memory)
  const uint32_t pos = wbase + (uint32_t)(incl - cnt);
  const uint32_t pathbits = cnt ? __float_as_uint(q.orig[0][i].w) : 0u;
  if (cnt > 0) append_ray(q, pos, r0, pathbits, tag);
  if (cnt > 1) append_ray(q, pos + 1u, r1, pathbits, tag);
}

// One path vertex for every queued ray (grid-stride; the loop bound is
// uniform over the block, as BLK's barriers need).
// IN: the input queue as a template constant, so the oriented pointers come
// straight from the parameter bank (no registers held across the loop).
template <bool BATCH, bool NEE, int MINB = NEE ? 3 : 4, bool BLK = false, int IN = 0>
__global__ void __launch_bounds__(256, MINB) k_shade(DevScene S0, RenderConst rc0, Wave w0, Queues qp, Batch b) {
  constexpr int in = IN;
  const Queues q = oriented(qp, IN);
  const uint32_t n = min(q.counters[in], q.capacity);  // an overflowed queue (error bit set) is read to capacity only
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    shade_item<BATCH, NEE, BLK>(S0, rc0, w0, q, in, b, i < n, i);
  }
}

// Sorted shade, first step (after extend).  A missed ray is shaded here
// (IBL::Sample or Scene::Background, PathTracer.cpp:357-364, counted as in
// shade_one), and every surface hit is filed by the material of the layer its
// roulette picks -- the reference dispatches on that layer's reflection type
// (PathTracer.cpp:419-429): with next-event estimation, a Lambert layer that
// does not emit or a Phong layer (a light sample is taken there) goes to the
// front of q.slist, every other surface (mirror, glass, emitters, any
// surface without light sampling) to the back.  The two lists are then shaded
// by separate kernel instances, so no warp mixes misses, light-sampling
// vertices and delta vertices.  The roulette is recomputed by the shade
// kernel from the same Philox counter, so the path is unchanged.
// The class of one queued ray (-1: a miss, shaded here; 0: a light-sampling
// surface; 1: any other surface), for the ray's scene S, constants rc and
// the wave's first path number g_first.
template <bool NEE>
__device__ __forceinline__ int classify_one(const DevScene &S, const RenderConst &rc, uint64_t g_first,
                                            const Queues &q, uint32_t i, uint32_t rec, float4 rd) {
  const uint32_t meta = __float_as_uint(rd.w);
  const uint32_t depth = meta & 0xFFFFu;
  if (rec == kMissRec) {
    if (!(rc.nee && depth > 0 && !(meta & kMetaSpec))) {
      const float4 ro = q.orig[0][i], rb = q.beta[0][i];
      add_radiance(q.pathL + __float_as_uint(ro.w), ld3(rb) * env_lookup(S, ld3(rd)));
    }
    return -1;
  }
  if (!NEE) return 1;
  uint32_t lb, lc;
  if (rec & kPlaneBit) {
    const PlaneRec &pl = S.planes[rec & ~kPlaneBit];
    lb = pl.layer_begin;
    lc = pl.layer_count;
  } else {
    const PrimInfo &inf = S.info[rec];
    lb = inf.layer_begin;
    lc = inf.layer_count;
  }
  uint32_t sel = 0;  // a one-layer object needs no roulette draw
  if (lc > 1) {
    const uint32_t path = __float_as_uint(q.orig[0][i].w);
    const uint4 rn = philox(path_counter(g_first + path, (meta >> 16) & 0xFFu, depth, 0u), rc.seed_lo, rc.seed_hi);
    sel = pick_layer(S, lb, lc, u01(rn.x));
  }
  const MaterialDev &m = S.materials[S.layers[lb + sel].material];
  return ((m.type == OR3_LAMBERT && !m.emissive) || m.type == OR3_PHONG) ? 0 : 1;
}

// BATCH: each ray's segment (beta.w) names its job, scene and constants.
template <bool NEE, int IN, bool BATCH = false>
__global__ void __launch_bounds__(256) k_classify(DevScene S0, RenderConst rc0, Wave w0, Queues qp, Batch b) {
  constexpr int in = IN;
  const Queues q = oriented(qp, IN);
  __shared__ uint32_t wcount[2][8], wbase[2];  // per class: warp counts (then offsets), the block's base
  const uint32_t n = min(q.counters[in], q.capacity);
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    int cls = -1;  // -1: done here (a miss), 0: front list, 1: back list
    if (i < n) {
      const uint32_t rec = __float_as_uint(q.hits[i].y);
      const float4 rd = q.dir[0][i];
      if (BATCH) {
        const Segment sg = b.segs[__float_as_uint(q.beta[0][i].w)];
        const JobDev &job = b.jobs[sg.job];
        cls = classify_one<NEE>(b.scenes[job.scene], job.rc, sg.g_first - sg.wave_first, q, i, rec, rd);
      } else {
        cls = classify_one<NEE>(S0, rc0, w0.g_first, q, i, rec, rd);
      }
    }
    // block-aggregated appends (one atomic per class and block iteration: the
    // two list lengths are single addresses every block updates); the lists
    // hold at most n <= capacity entries together
    const unsigned m0 = __ballot_sync(0xFFFFFFFFu, cls == 0), m1 = __ballot_sync(0xFFFFFFFFu, cls == 1);
    const uint32_t warp = threadIdx.x >> 5;
    if (lane == 0) {
      wcount[0][warp] = (uint32_t)__popc(m0);
      wcount[1][warp] = (uint32_t)__popc(m1);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      const uint32_t c = threadIdx.x;
      uint32_t total = 0;
      for (uint32_t k = 0; k < (blockDim.x >> 5); k++) {
        const uint32_t v = wcount[c][k];
        wcount[c][k] = total;  // exclusive prefix over the block's warps
        total += v;
      }
      wbase[c] = total ? atomicAdd(&q.counters[10 + c], total) : 0u;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    if (cls == 0) q.slist[wbase[0] + wcount[0][warp] + (uint32_t)__popc(m0 & below)] = i;
    else if (cls == 1) q.slist[q.capacity - 1u - (wbase[1] + wcount[1][warp] + (uint32_t)__popc(m1 & below))] = i;
    __syncthreads();  // wcount / wbase are rewritten by the next iteration
  }
}

// Sorted shade, second step: the entries of one list (back = 0: the front
// list, light-sampling vertices; 1: the back list).
template <bool NEE, int IN, bool BATCH = false, int MINB = NEE ? 3 : 4>
__global__ void __launch_bounds__(256, MINB) k_shade_list(DevScene S, RenderConst rc, Wave w, Queues qp, Batch b,
                                                          int back) {
  constexpr int in = IN;
  const Queues q = oriented(qp, IN);
  const uint32_t cap = q.capacity;
  const uint32_t n = min(q.counters[back ? 11 : 10], cap);
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t k = base + threadIdx.x;
    const bool valid = k < n;
    const uint32_t i = valid ? q.slist[back ? cap - 1u - k : k] : 0u;
    shade_item<BATCH, NEE, true>(S, rc, w, q, in, b, valid, i);
  }
}

// a[i] += b[i], b[i] = 0 over n doubles of two pixel-sum pairs (the second
// wave lane's sums folded into the first lane's at the end of a pass)
__global__ void k_merge_sums(size_t n, double *a, double *aq, double *b, double *bq) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    a[i] += b[i];
    aq[i] += bq[i];
    b[i] = 0.0;
    bq[i] = 0.0;
  }
}

// Clears a consumed queue's length and its extend fetch counter, the shadow
// queue's length and fetch counter, and the sorted shade's list lengths.
__global__ void k_reset_count(uint32_t *counters, int which) {
  counters[which] = 0;
  counters[4 + which] = 0;
  counters[3] = 0;
  counters[6] = 0;
  counters[10] = 0;
  counters[11] = 0;
}

struct ShadowSrc {
  const float4 *orig, *dir;
  __device__ __forceinline__ void load(uint32_t i, V3 &o, V3 &d, float &tmax) const {
    o = ld3(orig[i]);
    const float4 dd = dir[i];
    d = v3(dd.x, dd.y, dd.z);
    tmax = dd.w;
  }
};

struct ShadowSink {
  const float4 *orig, *contrib;
  float4 *pathL;
  __device__ __forceinline__ void store(const DevScene &, uint32_t i, Hit h, V3, V3) const {
    if (h.rec != kMissRec) return;
    add_radiance(pathL + __float_as_uint(orig[i].w), ld3(contrib[i]));
  }
};

// Any-hit test of every queued shadow ray (persistent, lane-refilled).
// SORT false: children in slot order (no distance sort).
// FN: FP32-box nodes (else the quantised ones).
// REFILL: a warp fetches new rays once this many lanes are idle (24 at
// three steps per vote: terrain shadow time 267 ms at 16, 265 ms at 24,
// 295 ms at 8 per step).
template <bool SORT, bool FN, bool W8 = false, int REFILL = 24>
__global__ void __launch_bounds__(256, 4) k_shadow(DevScene S, Queues q) {
  const uint32_t n = min(q.counters[3], q.capacity);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  persistent_trace<true, false, 2, ShadowSrc, ShadowSink, REFILL, SORT, FN, false, W8, kShadowStepsPerVote>(
      S, n, &q.counters[6], ShadowSrc{q.sorig, q.sdir}, ShadowSink{q.sorig, q.scontrib, q.pathL}, nullptr, 0u,
      nullptr, &q.counters[2]);
}

// After a wave's accumulation: a queue overflow is filed in fail ([0] the
// count, then wave indices; cap entries) and its bit cleared, so the lane's
// next wave is judged on its own.
__global__ void k_wave_check(uint32_t *counters, uint32_t *fail, uint32_t cap, uint32_t wave) {
  if (!(counters[2] & kErrQueue)) return;
  const uint32_t k = atomicAdd(fail, 1u);
  if (k < cap) fail[1 + k] = wave;
  counters[2] &= ~kErrQueue;
}

// Per-pixel sums of the wave's path radiance: one warp per pixel, lanes over
// the pixel's samples (coalesced), FP32 partials added into FP64 sums.
// A wave whose ray queue overflowed (a glass split past the queue's
// capacity: the error bit kErrQueue) is not accumulated; k_wave_check files
// it for a re-render.
__global__ void k_accumulate(Queues q, Wave w, uint32_t ss2, double *sum, double *sumsq) {
  if (q.counters[2] & kErrQueue) return;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t per = w.ns * ss2;
  for (uint32_t p = warp; p < w.npix; p += nwarps) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f;
    for (uint32_t j = lane; j < per; j += 32u) {
      const uint32_t sl = j / ss2, k = j - sl * ss2;
      const float4 L = q.pathL[((size_t)sl * w.npix + p) * ss2 + k];
      s0 += L.x; s1 += L.y; s2 += L.z;
      q0 += L.x * L.x; q1 += L.y * L.y; q2 += L.z * L.z;
    }
#pragma unroll
    for (int ofs = 16; ofs > 0; ofs >>= 1) {
      s0 += __shfl_xor_sync(0xFFFFFFFFu, s0, ofs);
      s1 += __shfl_xor_sync(0xFFFFFFFFu, s1, ofs);
      s2 += __shfl_xor_sync(0xFFFFFFFFu, s2, ofs);
      q0 += __shfl_xor_sync(0xFFFFFFFFu, q0, ofs);
      q1 += __shfl_xor_sync(0xFFFFFFFFu, q1, ofs);
      q2 += __shfl_xor_sync(0xFFFFFFFFu, q2, ofs);
    }
    if (lane == 0) {
      const size_t px = (size_t)(w.pix0 + p);
      sum[3 * px] += s0; sum[3 * px + 1] += s1; sum[3 * px + 2] += s2;
      sumsq[3 * px] += q0; sumsq[3 * px + 1] += q1; sumsq[3 * px + 2] += q2;
    }
  }
}

// Frame in the reference's layout: ScreenPixels::ScreenViewport::calcIndex
// (src/renderer/ScreenPixels.cpp:50-65) flips y, the image is viewport 0 of a
// 2 x 1 grid (PathTracer.cpp:63).  The right viewport is cleared by the host.
__global__ void k_frame(const double *sum, uint32_t W, uint32_t H, int layout, double scale, double *out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= W * H) return;
  const uint32_t x = p % W, y = p / W;
  const uint32_t rowW = layout == 0 ? 2 * W : W;
  const size_t o = ((size_t)(H - 1 - y) * rowW + x) * 3;
  out[o] = sum[3 * (size_t)p] * scale;
  out[o + 1] = sum[3 * (size_t)p + 1] * scale;
  out[o + 2] = sum[3 * (size_t)p + 2] * scale;
}

__global__ void k_moments(const double *sum, const double *sumsq, uint32_t W, uint32_t H, double *so,
                          double *qo) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= W * H) return;
  const uint32_t x = p % W, y = p / W;
  const size_t o = ((size_t)(H - 1 - y) * W + x) * 3;
  for (int c = 0; c < 3; c++) {
    if (so) so[o + c] = sum[3 * (size_t)p + c];
    if (qo) qo[o + c] = sumsq[3 * (size_t)p + c];
  }
}

// Ray-set queries run the render's own traversal (persistent_trace), so their
// parity tests cover the extend kernel's code.
struct ArraySrc {
  const float *orig, *dir, *tmax;
  __device__ __forceinline__ void load(uint32_t i, V3 &o, V3 &d, float &tm) const {
    o = v3(orig[3 * (size_t)i], orig[3 * (size_t)i + 1], orig[3 * (size_t)i + 2]);
    d = v3(dir[3 * (size_t)i], dir[3 * (size_t)i + 1], dir[3 * (size_t)i + 2]);
    tm = tmax ? tmax[i] : kInf;
  }
};

struct QuerySink {
  int32_t *prim;
  float *tout, *nout;
  __device__ __forceinline__ void store(const DevScene &S, uint32_t i, Hit h, V3 o, V3 d) const {
    h.t = refine_t(S, h, o, d);
    if (h.rec == kMissRec) {
      prim[i] = -1;
      tout[i] = kInf;
      if (nout) nout[3 * (size_t)i] = nout[3 * (size_t)i + 1] = nout[3 * (size_t)i + 2] = 0.f;
    } else {
      const Surface s = surface_at(S, h, o, d);
      prim[i] = (int32_t)s.object_id;
      tout[i] = h.t;
      if (nout) {
        nout[3 * (size_t)i] = s.n.x;
        nout[3 * (size_t)i + 1] = s.n.y;
        nout[3 * (size_t)i + 2] = s.n.z;
      }
    }
  }
};

struct OccludedSink {
  uint8_t *occ;
  __device__ __forceinline__ void store(const DevScene &, uint32_t i, Hit h, V3, V3) const {
    occ[i] = h.rec != kMissRec ? 1 : 0;
  }
};

// counters[2] = error bits, counters[8] = fetch counter (zeroed by the launcher)
__global__ void __launch_bounds__(256) k_trace_closest(DevScene S, uint32_t n, const float *orig, const float *dir,
                                                       int32_t *prim, float *tout, float *nout, uint32_t *counters,
                                                       int smem_nodes) {
  __shared__ uint4 snodes[kSmemNodes * 4];
  const uint32_t ns = stage_nodes(S, snodes, smem_nodes);
  persistent_trace<false, false, 2>(S, n, &counters[8], ArraySrc{orig, dir, nullptr}, QuerySink{prim, tout, nout},
                                    snodes, ns, nullptr, &counters[2]);
}

__global__ void __launch_bounds__(256) k_trace_occluded(DevScene S, uint32_t n, const float *orig, const float *dir,
                                                        const float *tmax, uint8_t *occ, uint32_t *counters,
                                                        int smem_nodes) {
  __shared__ uint4 snodes[kSmemNodes * 4];
  const uint32_t ns = stage_nodes(S, snodes, smem_nodes);
  persistent_trace<true, false, 2>(S, n, &counters[8], ArraySrc{orig, dir, tmax}, OccludedSink{occ}, snodes, ns,
                                   nullptr, &counters[2]);
}

int g_query_grid = 1;  // set from the device's SM count and occupancy when a context is created

// IBL::Sample(dir) (src/renderer/IBL.h:30-45) for a set of directions: the
// render's own env_lookup, so its parity test covers the miss shading.
__global__ void k_env_sample(DevScene S, uint32_t n, const float *dir, float *rgb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V3 c = env_lookup(S, v3(dir[3 * (size_t)i], dir[3 * (size_t)i + 1], dir[3 * (size_t)i + 2]));
  rgb[3 * (size_t)i] = c.x;
  rgb[3 * (size_t)i + 1] = c.y;
  rgb[3 * (size_t)i + 2] = c.z;
}

// Image::GetPixelByUV (src/tools/Image.h:21-31) of texture `tex` at n (u, v)
// pairs: the render's own texel().
__global__ void k_texture_sample(DevScene S, int tex, uint32_t n, const float *uv, float *rgb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V3 c = texel(S, tex, uv[2 * (size_t)i], uv[2 * (size_t)i + 1]);
  rgb[3 * (size_t)i] = c.x;
  rgb[3 * (size_t)i + 1] = c.y;
  rgb[3 * (size_t)i + 2] = c.z;
}

// ---------------------------------------------------------------- batched form kernels

// The camera ray of wave path i into queue slot 0 of q (oriented).
__device__ __forceinline__ void raygen_batch_one(const Batch &b, const Queues &q, uint32_t i) {
  const uint32_t si = find_segment(b.segs, b.info->nseg, i);
  const Segment sg = b.segs[si];
  const RenderConst &rc = b.jobs[sg.job].rc;
  const uint64_t g = sg.g_first + (i - sg.wave_first);
  const uint32_t sub = (uint32_t)(g % rc.ss2);
  const uint64_t pg = g / rc.ss2;
  const uint32_t pix = (uint32_t)(pg % ((uint64_t)rc.W * rc.H));
  V3 o, d;
  camera_ray(rc, pix % rc.W, pix / rc.W, sub % rc.ss, sub / rc.ss, pix * rc.ss2 + sub, sg.pass_first, o, d);
  q.orig[0][i] = make_float4(o.x, o.y, o.z, __uint_as_float(i));
  q.dir[0][i] = make_float4(d.x, d.y, d.z, __uint_as_float(0u));
  q.beta[0][i] = make_float4(1.f, 1.f, 1.f, __uint_as_float(si));
  q.pathL[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_raygen_batch(Batch b, uint32_t num_paths, Queues qp, int out) {
  const Queues q = oriented(qp, out);  // the queue written is slot 0
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    q.counters[out] = num_paths;
    q.counters[4 + out] = 0;
  }
  if (i < num_paths) raygen_batch_one(b, q, i);
}

// Device loop: the camera rays of a wave taken in this iteration, into queue
// 0 (a grid-stride loop: the grid is fixed when the loop is captured).
__global__ void k_raygen_batch_loop(Batch b, Queues q, const BatchLoop *L, int lane) {
  if (!L->lane[lane].fresh) return;
  const uint32_t n = b.info->num_paths;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    q.counters[0] = n;
    q.counters[4] = 0;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    raygen_batch_one(b, q, i);
}

// Device loop head: an idle lane takes the next wave from the shared queue
// and copies its segments into the lane's table; the lane's loop ends (its
// conditional handle set to 0) when no wave is left or the batch aborts.
// One block; thread 0 alone touches the loop state and the handle.
__global__ void k_wave_take(BatchLoop *L, int lane, const WaveDesc *waves, const Segment *segs_all, Segment *segs,
                            WaveInfo *info, const uint32_t *counters, cudaGraphConditionalHandle h) {
  __shared__ int w;
  if (threadIdx.x == 0) {
    BatchLoop::Lane &me = L->lane[lane];
    w = -1;
    if (counters[2] & ~kErrQueue) atomicOr(&L->abort, 2u);  // an overflow spoils only its own wave
    if (me.active && ++me.iters > L->max_iters) atomicOr(&L->abort, 1u);
    bool stop = atomicOr(&L->abort, 0u) != 0u;
    if (!stop && !me.active) {
      const uint32_t t = atomicAdd(&L->next_wave, 1u);
      if (t < L->nwaves) {
        w = (int)t;
        me.wave = t;
        me.active = 1u;
        me.fresh = 1u;
        me.iters = 0u;
      } else {
        stop = true;
      }
    }
    if (stop) cudaGraphSetConditional(h, 0u);
  }
  __syncthreads();
  if (w < 0) return;
  const WaveDesc d = waves[w];
  for (uint32_t k = threadIdx.x; k < d.nseg; k += blockDim.x) segs[k] = segs_all[d.seg_first + k];
  if (threadIdx.x == 0) *info = WaveInfo{d.nseg, d.ngroups, d.num_paths, 0u};
}

// Device loop tail: the wave's camera rays are out; a wave whose queue ran
// empty is complete (accumulated just before) and the lane takes the next.
__global__ void k_wave_finish(BatchLoop *L, int lane, const WaveInfo *info, uint32_t *counters, uint32_t *fail) {
  BatchLoop::Lane &me = L->lane[lane];
  me.fresh = 0u;
  if (me.active && counters[0] == 0u) {
    me.active = 0u;
    if (counters[2] & kErrQueue) {  // not accumulated: filed for a re-render in smaller waves
      const uint32_t k = atomicAdd(&L->nfail, 1u);
      if (k < L->fail_cap) fail[k] = me.wave;
      counters[2] &= ~kErrQueue;
    } else {
      me.waves++;
      me.paths += info->num_paths;
    }
  }
}

// persistent_trace (STEP 2) with the scene chosen per ray by its segment
// (src.load also returns the ray's segment).  The scene's node and record
// arrays are copied into registers when a lane takes a ray (TravView), so a
// step's node fetch does not wait on a reload of the scene descriptor.
// FN: the FP32-box nodes (else the 64-byte quantised ones).  HOIST false:
// every step reads the node array through the scene descriptor instead.
template <bool ANY, bool COUNT, class Src, class Sink, bool FN = true, bool HOIST = true, int VOTE_STEPS = 1>
__device__ __forceinline__ void batch_trace(const Batch &b, uint32_t n, uint32_t *fetch, const Src &src,
                                            const Sink &sink, uint32_t *cnt, uint32_t *err) {
  uint2 stk_p[kStackSize];
  PairStack stk{stk_p};
  TravState st;
  const DevScene *sp = b.scenes;  // the ray's scene
  const float4 *fnodes = nullptr;
  const uint4 *nodes = nullptr;
  uint32_t r = kNoEntry;
  bool drained = false;  // warp-uniform: the shared fetch counter has passed n
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, r == kNoEntry);
    if (!drained && (__popc(idle) >= 16 || idle == 0xFFFFFFFFu)) {
      const int leader = __ffs(idle) - 1;
      const uint32_t want = (uint32_t)__popc(idle);
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, want);
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      const uint32_t idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
      if (r == kNoEntry && idx < n) {
        V3 o, d;
        float tmax;
        uint32_t tag;
        src.load(idx, o, d, tmax, tag);
        sp = &b.scenes[b.jobs[b.segs[tag].job].scene];
        if (HOIST) {
          fnodes = sp->fnodes;
          nodes = sp->nodes;
        }
        trav_init(st, o, d, tmax, sp->num_nodes);
        r = idx;
      }
      drained = base + want >= n;
    } else if (drained && idle == 0xFFFFFFFFu) {
      break;
    }
    if (r != kNoEntry) {
      bool done = false;
#pragma unroll
      for (int k = 0; k < VOTE_STEPS; k++) {
        if (done) break;
        if (HOIST) {
          const TravView tv{fnodes, nodes, sp->prims};
          done = trav_step_inline<ANY, COUNT, true, PairStack, FN>(tv, st, stk, nullptr, 0u, cnt, err);
        } else {
          done = trav_step_inline<ANY, COUNT, true, PairStack, FN>(*sp, st, stk, nullptr, 0u, cnt, err);
        }
      }
      if (done) {
        sink.store(*sp, r, trav_finish<ANY>(*sp, st), st.o, st.d);
        r = kNoEntry;
      }
    }
  }
}

struct BatchQueueSrc {
  const float4 *orig, *dir, *beta;
  __device__ __forceinline__ void load(uint32_t i, V3 &o, V3 &d, float &tmax, uint32_t &tag) const {
    o = ld3(orig[i]);
    d = ld3(dir[i]);
    tmax = kInf;
    tag = __float_as_uint(beta[i].w);
  }
};

struct BatchShadowSrc {
  const float4 *orig, *dir, *contrib;
  __device__ __forceinline__ void load(uint32_t i, V3 &o, V3 &d, float &tmax, uint32_t &tag) const {
    ShadowSrc{orig, dir}.load(i, o, d, tmax);
    tag = __float_as_uint(contrib[i].w);
  }
};

template <bool COUNT, bool FN = true, bool HOIST = true, int VS = 1>
__global__ void __launch_bounds__(256, 4) k_extend_batch(Batch b, Queues q, int in) {
  const Queues qo = oriented(q, in);
  const uint32_t n = min(q.counters[in], q.capacity);  // an overflowed queue (error bit set) is read to capacity only
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&q.stats[0], (unsigned long long)n);
    if (n) atomicAdd(&q.stats[2], 1ull);
  }
  uint32_t cnt[3] = {0u, 0u, 0u};
  batch_trace<false, COUNT, BatchQueueSrc, HitSink, FN, HOIST, VS>(
      b, n, &q.counters[4 + in], BatchQueueSrc{qo.orig[0], qo.dir[0], qo.beta[0]}, HitSink{q.hits}, cnt,
      &q.counters[2]);
  if (COUNT) {
    unsigned long long c0 = cnt[0], c1 = cnt[1], c2 = cnt[2];
#pragma unroll
    for (int ofs = 16; ofs > 0; ofs >>= 1) {
      c0 += __shfl_xor_sync(0xFFFFFFFFu, c0, ofs);
      c1 += __shfl_xor_sync(0xFFFFFFFFu, c1, ofs);
      c2 += __shfl_xor_sync(0xFFFFFFFFu, c2, ofs);
    }
    if ((threadIdx.x & 31u) == 0) {
      atomicAdd(&q.stats[3], c0);
      atomicAdd(&q.stats[4], c1);
      atomicAdd(&q.stats[5], c2);
    }
  }
}

template <bool FN = true, bool HOIST = true>
__global__ void __launch_bounds__(256, 4) k_shadow_batch(Batch b, Queues q) {
  const uint32_t n = min(q.counters[3], q.capacity);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  batch_trace<true, false, BatchShadowSrc, ShadowSink, FN, HOIST, kShadowStepsPerVote>(
      b, n, &q.counters[6], BatchShadowSrc{q.sorig, q.sdir, q.scontrib}, ShadowSink{q.sorig, q.scontrib, q.pathL},
      nullptr, &q.counters[2]);
}

// One thread per pixel-sample group (ss2 consecutive paths of one pixel and
// sample); FP32 partial sums added to the job's FP64 pixel sums.
__device__ __forceinline__ void accumulate_batch_one(const Batch &b, const Queues &q, uint32_t gi) {
  uint32_t lo = 0, hi = b.info->nseg;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (b.segs[mid].group_first <= gi) lo = mid;
    else hi = mid;
  }
  const Segment sg = b.segs[lo];
  const JobDev &job = b.jobs[sg.job];
  const uint32_t ss2 = job.rc.ss2;
  const uint32_t local = gi - sg.group_first;
  const uint64_t gstart = sg.g_first + (uint64_t)local * ss2;
  const uint32_t wstart = sg.wave_first + local * ss2;
  const uint64_t pix = (gstart / ss2) % ((uint64_t)job.rc.W * job.rc.H);
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f;
  for (uint32_t k = 0; k < ss2; k++) {
    const float4 L = q.pathL[wstart + k];
    s0 += L.x; s1 += L.y; s2 += L.z;
    q0 += L.x * L.x; q1 += L.y * L.y; q2 += L.z * L.z;
  }
  double *S = job.sum + 3 * pix;
  double *Q = job.sumsq + 3 * pix;
  atomicAdd(S, (double)s0); atomicAdd(S + 1, (double)s1); atomicAdd(S + 2, (double)s2);
  atomicAdd(Q, (double)q0); atomicAdd(Q + 1, (double)q1); atomicAdd(Q + 2, (double)q2);
}

__global__ void k_accumulate_batch(Batch b, Queues q) {
  const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi < b.info->ngroups) accumulate_batch_one(b, q, gi);
}

// Device loop: accumulate the lane's wave once its queue 0 is empty.
__global__ void k_accumulate_batch_loop(Batch b, Queues q, const BatchLoop *L, int lane) {
  if (!L->lane[lane].active || q.counters[0] != 0u || (q.counters[2] & kErrQueue)) return;
  const uint32_t ng = b.info->ngroups;
  for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ng; gi += gridDim.x * blockDim.x)
    accumulate_batch_one(b, q, gi);
}

}  // namespace

void launch_raygen(const RenderConst &rc, const Wave &w, const Queues &q, int out, int grid, int block,
                   cudaStream_t st) {
  (void)grid;
  const int g = (int)((w.num_paths + block - 1) / block);
  k_raygen<<<g > 0 ? g : 1, block, 0, st>>>(rc, w, q, out);
}

void launch_extend(const DevScene &S, const Queues &q, int in, int grid, int block, int smem_nodes, bool count,
                   int variant, cudaStream_t st) {
  const int sn = smem_nodes > kSmemNodes ? kSmemNodes : smem_nodes;
  if (variant == 8) {  // the 8-wide nodes
    if (count) k_extend<true, 8><<<grid, block, 0, st>>>(S, q, in, 0);
    else k_extend<false, 8><<<grid, block, 0, st>>>(S, q, in, 0);
    return;
  }
  switch ((count ? 8 : 0) | (variant & 7)) {
    case 1: k_extend<false, 1><<<grid, block, 0, st>>>(S, q, in, sn); break;
    case 2: k_extend<false, 2><<<grid, block, 0, st>>>(S, q, in, 0); break;
    case 4: k_extend<false, 4><<<grid, block, 0, st>>>(S, q, in, 0); break;
    case 5: k_extend<false, 5><<<grid, block, 0, st>>>(S, q, in, 0); break;
    case 6: k_extend<false, 6><<<grid, block, 0, st>>>(S, q, in, sn); break;
    case 7: k_extend<false, 7><<<grid, block, 0, st>>>(S, q, in, 0); break;
    case 8: k_extend<true, 0><<<grid, block, 0, st>>>(S, q, in, sn); break;
    case 9: k_extend<true, 1><<<grid, block, 0, st>>>(S, q, in, sn); break;
    case 10: case 12: case 13: case 14:  // counting runs use the default traversal
      k_extend<true, 2><<<grid, block, 0, st>>>(S, q, in, 0); break;
    case 15: k_extend<true, 7><<<grid, block, 0, st>>>(S, q, in, 0); break;
    default: k_extend<false, 0><<<grid, block, 0, st>>>(S, q, in, sn); break;
  }
}

template <int IN>
static void launch_shade_in(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q, int grid,
                            int block, cudaStream_t st, bool nee4, bool blk) {
  const bool nee = rc.nee && (S.num_lights > 0 || S.env_light != 0);
  if (nee && nee4)
    k_shade<false, true, 4, false, IN><<<grid, block, 0, st>>>(S, rc, w, q, Batch{});
  else if (nee && blk)
    k_shade<false, true, 3, true, IN><<<grid, 256, 0, st>>>(S, rc, w, q, Batch{});
  else if (nee)
    k_shade<false, true, 3, false, IN><<<grid, block, 0, st>>>(S, rc, w, q, Batch{});
  else if (blk)
    k_shade<false, false, 4, true, IN><<<grid, 256, 0, st>>>(S, rc, w, q, Batch{});
  else
    k_shade<false, false, 4, false, IN><<<grid, block, 0, st>>>(S, rc, w, q, Batch{});
}

void launch_shade(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q, int in,
                  int grid, int block, cudaStream_t st, bool nee4, bool blk) {
  if (in) launch_shade_in<1>(S, rc, w, q, grid, block, st, nee4, blk);
  else launch_shade_in<0>(S, rc, w, q, grid, block, st, nee4, blk);
}

template <int IN, bool BATCH>
static void launch_shade_sorted_in(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q,
                                   const Batch &b, bool nee, int grid_classify, int grid_nee, int grid_plain,
                                   cudaStream_t st) {
  if (nee) {
    k_classify<true, IN, BATCH><<<grid_classify, 256, 0, st>>>(S, rc, w, q, b);
    k_shade_list<true, IN, BATCH><<<grid_nee, 256, 0, st>>>(S, rc, w, q, b, 0);
  } else {
    k_classify<false, IN, BATCH><<<grid_classify, 256, 0, st>>>(S, rc, w, q, b);
  }
  k_shade_list<false, IN, BATCH><<<grid_plain, 256, 0, st>>>(S, rc, w, q, b, 1);
}

void launch_shade_sorted(const DevScene &S, const RenderConst &rc, const Wave &w, const Queues &q, int in,
                         int grid_classify, int grid_nee, int grid_plain, cudaStream_t st) {
  const bool nee = rc.nee && (S.num_lights > 0 || S.env_light != 0);
  if (in) launch_shade_sorted_in<1, false>(S, rc, w, q, Batch{}, nee, grid_classify, grid_nee, grid_plain, st);
  else launch_shade_sorted_in<0, false>(S, rc, w, q, Batch{}, nee, grid_classify, grid_nee, grid_plain, st);
}

void launch_shade_batch_sorted(const Batch &b, const Queues &q, int in, bool nee, int grid_classify, int grid_nee,
                               int grid_plain, cudaStream_t st) {
  const DevScene S{};
  const RenderConst rc{};
  const Wave w{};
  if (in) launch_shade_sorted_in<1, true>(S, rc, w, q, b, nee, grid_classify, grid_nee, grid_plain, st);
  else launch_shade_sorted_in<0, true>(S, rc, w, q, b, nee, grid_classify, grid_nee, grid_plain, st);
}

void launch_merge_sums(size_t n, double *a, double *aq, double *b, double *bq, int max_grid, cudaStream_t st) {
  const size_t g = (n + 255) / 256;
  if (n) k_merge_sums<<<(unsigned)(g < (size_t)max_grid ? g : (size_t)max_grid), 256, 0, st>>>(n, a, aq, b, bq);
}

void launch_reset_count(const Queues &q, int which, cudaStream_t st) {
  k_reset_count<<<1, 1, 0, st>>>(q.counters, which);
}

void launch_shadow(const DevScene &S, const Queues &q, int grid, bool unsorted, bool quantised, cudaStream_t st,
                   bool wide8, bool refill8) {
  if (wide8) k_shadow<false, true, true><<<grid, 256, 0, st>>>(S, q);
  else if (refill8) k_shadow<true, true, false, 8><<<grid, 256, 0, st>>>(S, q);
  else if (quantised) k_shadow<true, false><<<grid, 256, 0, st>>>(S, q);
  else if (unsorted) k_shadow<false, true><<<grid, 256, 0, st>>>(S, q);
  else k_shadow<true, true><<<grid, 256, 0, st>>>(S, q);
}

void launch_shadow_batch(const Batch &b, const Queues &q, int grid, int variant, cudaStream_t st) {
  switch (variant & 3) {
    case 1: k_shadow_batch<false, true><<<grid, 256, 0, st>>>(b, q); break;
    case 2: k_shadow_batch<true, false><<<grid, 256, 0, st>>>(b, q); break;
    case 3: k_shadow_batch<false, false><<<grid, 256, 0, st>>>(b, q); break;
    default: k_shadow_batch<true, true><<<grid, 256, 0, st>>>(b, q); break;
  }
}

void launch_accumulate(const Queues &q, const Wave &w, uint32_t ss2, double *sum, double *sumsq, int grid,
                       int block, cudaStream_t st) {
  k_accumulate<<<grid, block, 0, st>>>(q, w, ss2, sum, sumsq);
}

void launch_wave_check(const Queues &q, uint32_t *fail, uint32_t cap, uint32_t wave, cudaStream_t st) {
  k_wave_check<<<1, 1, 0, st>>>(q.counters, fail, cap, wave);
}

void launch_frame(const double *sum, uint32_t W, uint32_t H, int layout, double scale, double *out,
                  cudaStream_t st) {
  const uint32_t n = W * H;
  k_frame<<<(n + 255) / 256, 256, 0, st>>>(sum, W, H, layout, scale, out);
}

void launch_moments(const double *sum, const double *sumsq, uint32_t W, uint32_t H, double *so, double *qo,
                    cudaStream_t st) {
  const uint32_t n = W * H;
  k_moments<<<(n + 255) / 256, 256, 0, st>>>(sum, sumsq, W, H, so, qo);
}

void set_query_grid(int grid) { g_query_grid = grid > 0 ? grid : 1; }

void launch_trace_closest(const DevScene &S, size_t n, const float *orig, const float *dir, int32_t *prim,
                          float *t, float *normal, uint32_t *counters, cudaStream_t st) {
  const int sn = 0;  // no shared-memory node staging by default (measured slower)
  for (size_t b = 0; b < n; b += (size_t)1 << 30) {
    const uint32_t m = (uint32_t)((n - b) < ((size_t)1 << 30) ? (n - b) : ((size_t)1 << 30));
    cudaMemsetAsync(counters + 8, 0, sizeof(uint32_t), st);
    k_trace_closest<<<g_query_grid, 256, 0, st>>>(S, m, orig + 3 * b, dir + 3 * b, prim + b, t + b,
                                                  normal ? normal + 3 * b : nullptr, counters, sn);
  }
}

void launch_trace_occluded(const DevScene &S, size_t n, const float *orig, const float *dir,
                           const float *tmax, uint8_t *occ, uint32_t *counters, cudaStream_t st) {
  const int sn = 0;  // no shared-memory node staging by default (measured slower)
  for (size_t b = 0; b < n; b += (size_t)1 << 30) {
    const uint32_t m = (uint32_t)((n - b) < ((size_t)1 << 30) ? (n - b) : ((size_t)1 << 30));
    cudaMemsetAsync(counters + 8, 0, sizeof(uint32_t), st);
    k_trace_occluded<<<g_query_grid, 256, 0, st>>>(S, m, orig + 3 * b, dir + 3 * b, tmax + b, occ + b, counters,
                                                   sn);
  }
}

void launch_env_sample(const DevScene &S, uint32_t n, const float *dir, float *rgb, cudaStream_t st) {
  if (n) k_env_sample<<<(n + 255) / 256, 256, 0, st>>>(S, n, dir, rgb);
}

void launch_texture_sample(const DevScene &S, int tex, uint32_t n, const float *uv, float *rgb, cudaStream_t st) {
  if (n) k_texture_sample<<<(n + 255) / 256, 256, 0, st>>>(S, tex, n, uv, rgb);
}

const void *kernel_extend_ptr() { return (const void *)k_extend<false, 0>; }
const void *kernel_shade_ptr(bool batch, bool nee) {
  if (batch) return nee ? (const void *)k_shade<true, true, 3, false, 0> : (const void *)k_shade<true, false, 4, false, 0>;
  return nee ? (const void *)k_shade<false, true, 3, false, 0> : (const void *)k_shade<false, false, 4, false, 0>;
}

// ---------------------------------------------------------------- batched form

void launch_raygen_batch(const Batch &b, uint32_t num_paths, const Queues &q, int out, cudaStream_t st) {
  k_raygen_batch<<<(num_paths + 255) / 256 > 0 ? (num_paths + 255) / 256 : 1, 256, 0, st>>>(b, num_paths, q, out);
}

// variant bit 0: quantised 64-byte nodes; bit 1: node array read through the
// scene descriptor every step (the form before it was hoisted)
void launch_extend_batch(const Batch &b, const Queues &q, int in, int grid, bool count, int variant,
                         cudaStream_t st) {
  if (count) {
    k_extend_batch<true><<<grid, 256, 0, st>>>(b, q, in);
    return;
  }
  switch (variant & 3) {
    case 1: k_extend_batch<false, false, true><<<grid, 256, 0, st>>>(b, q, in); break;
    case 2: k_extend_batch<false, true, false, 2><<<grid, 256, 0, st>>>(b, q, in); break;
    case 3: k_extend_batch<false, false, false><<<grid, 256, 0, st>>>(b, q, in); break;
    default: k_extend_batch<false, true, true><<<grid, 256, 0, st>>>(b, q, in); break;
  }
}

void launch_shade_batch(const Batch &b, const Queues &q, int in, int grid, bool nee, cudaStream_t st) {
  const DevScene S{};
  const RenderConst rc{};
  const Wave w{};
  if (nee && in) k_shade<true, true, 3, false, 1><<<grid, 256, 0, st>>>(S, rc, w, q, b);
  else if (nee) k_shade<true, true, 3, false, 0><<<grid, 256, 0, st>>>(S, rc, w, q, b);
  else if (in) k_shade<true, false, 4, false, 1><<<grid, 256, 0, st>>>(S, rc, w, q, b);
  else k_shade<true, false, 4, false, 0><<<grid, 256, 0, st>>>(S, rc, w, q, b);
}

void launch_accumulate_batch(const Batch &b, uint32_t max_groups, const Queues &q, cudaStream_t st) {
  const uint32_t g = (max_groups + 255) / 256;
  k_accumulate_batch<<<g > 0 ? g : 1, 256, 0, st>>>(b, q);
}

void launch_wave_take(BatchLoop *L, int lane, const WaveDesc *waves, const Segment *segs_all, Segment *segs,
                      WaveInfo *info, const uint32_t *counters, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_wave_take<<<1, 256, 0, st>>>(L, lane, waves, segs_all, segs, info, counters, h);
}

void launch_raygen_batch_loop(const Batch &b, const Queues &q, const BatchLoop *L, int lane, int grid,
                              cudaStream_t st) {
  k_raygen_batch_loop<<<grid > 0 ? grid : 1, 256, 0, st>>>(b, q, L, lane);
}

void launch_accumulate_batch_loop(const Batch &b, const Queues &q, const BatchLoop *L, int lane, int grid,
                                  cudaStream_t st) {
  k_accumulate_batch_loop<<<grid > 0 ? grid : 1, 256, 0, st>>>(b, q, L, lane);
}

void launch_wave_finish(BatchLoop *L, int lane, const WaveInfo *info, uint32_t *counters, uint32_t *fail,
                        cudaStream_t st) {
  k_wave_finish<<<1, 1, 0, st>>>(L, lane, info, counters, fail);
}

}  // namespace or3
