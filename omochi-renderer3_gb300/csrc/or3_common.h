// or3_common.h -- data layouts shared by the host builder and the CUDA kernels.
//
// Everything the kernels read lives in flat arrays in HBM:
//   WideNode   64 B   4-wide BVH node with 8-bit quantised child boxes
//   prim rec   48 B   3 x float4 per in-BVH primitive, in leaf order
//                     triangle: (v0.xyz, e1.x) (e1.yz, e2.xy) (e2.z, -, -, -)
//                     sphere:   (c.xyz, r) (-) (-)
//   PrimInfo   16 B   object id, layer range, flags (read once per hit)
//   TriShade   64 B   normal and uv bases (read once per triangle hit)
// The layouts replace the reference's per-object heap records
// (src/renderer/Polygon.h:108-111, src/renderer/BVH.h:20-38,
// src/renderer/QBVH.h:45-52).
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define OR3_HD __host__ __device__ __forceinline__
#else
#define OR3_HD inline
#endif

namespace or3 {

// src/tools/Constant.h:4-8
constexpr float kEps = 0.0005f;              // EPS
constexpr double kEpsD = 0.0005;
constexpr float kInf = 1.7014117e38f;         // INF = (FLT_MAX-1)/2
constexpr float kPi = 3.14159265358979323846f;

constexpr int kStackSize = 64;       // traversal stack entries per ray
constexpr int kMaxBinaryDepth = 40;  // builder bound: wide depth <= 20, stack <= 61
static_assert(3 * (kMaxBinaryDepth / 2) < kStackSize, "a path of wide nodes pushes at most 3 entries per level");

// Wide node.  For child i and axis a the box is
//   origin[a] + q[a][i] * 2^(exp[a]-127),  q in [0, 255]
// Leaf children: child[i] = first prim record, count[i] = ntri | nsph << 4.
// Internal children: child[i] = node index, bit i of imask set.
// Empty slots: count 0 and imask bit clear.
struct alignas(64) WideNode {
  float origin[3];
  uint8_t exp[3];
  uint8_t imask;
  uint8_t lo[3][4];
  uint8_t hi[3][4];
  uint32_t child[4];
  uint8_t count[4];
  uint32_t pad;
};
static_assert(sizeof(WideNode) == 64, "WideNode must be 64 bytes");

// Wide node with FP32 child boxes (128 bytes): b[2a] are the lower and
// b[2a+1] the upper bounds of the 4 children on axis a (empty slots +inf /
// -inf), so a ray picks its near and far planes by which of the two it loads;
// child / count / imask as in WideNode.  Twice the bytes of WideNode, no
// dequantisation in the node test.
struct alignas(16) WideNodeF {
  float b[6][4];
  uint32_t child[4];
  uint8_t count[4];
  uint32_t imask;
  uint32_t pad[2];
};
static_assert(sizeof(WideNodeF) == 128, "WideNodeF must be 128 bytes");

// 8-wide node with FP32 child boxes (256 bytes), for the 8-wide traversal
// variant: b[2a] / b[2a+1] the lower / upper bounds of the 8 children on axis
// a (so float4 2p + h holds plane p of children 4h..4h+3), then the child
// words (node index or first record), the counts (ntri | nsph << 4) and the
// internal mask as in WideNodeF.
struct alignas(16) WideNode8F {
  float b[6][8];
  uint32_t child[8];
  uint8_t count[8];
  uint32_t imask;
  uint32_t pad[5];
};
static_assert(sizeof(WideNode8F) == 256, "WideNode8F must be 256 bytes");
constexpr int kStackSize8 = 96;  // traversal stack entries per ray over 8-wide nodes

// One child slab of a WideNodeF: the exact bound [lo, hi] widened by 2^-18
// of the parent's extent on that axis and then two ulps, so that the
// rounding of the slab distances cannot drop a ray that grazes a box face.
// Host and device builds give the same bits (round-to-nearest float ops).
OR3_HD void fnode_slab(float plo, float phi, float lo, float hi, float *olo, float *ohi) {
#ifdef __CUDA_ARCH__
  const float pad = __fmul_rn(__fsub_rn(phi, plo), 0x1p-18f);
  lo = __fsub_rn(lo, pad);
  hi = __fadd_rn(hi, pad);
#else
  const float pad = (phi - plo) * 0x1p-18f;
  lo = lo - pad;
  hi = hi + pad;
#endif
  *olo = nextafterf(nextafterf(lo, -INFINITY), -INFINITY);
  *ohi = nextafterf(nextafterf(hi, INFINITY), INFINITY);
}

enum PrimKind : uint32_t { kPrimTriangle = 0, kPrimSphere = 1, kPrimPlane = 2, kPrimFloor = 3 };

// flags
constexpr uint32_t kFlagSphereLight = 1u;   // SphereLight
constexpr uint32_t kFlagTexturedUV = 2u;    // some layer has a texture: compute uv
constexpr uint32_t kFlagEmissive = 4u;      // some layer emits (NEE light candidate)

struct PrimInfo {
  uint32_t object_id;
  uint32_t layer_begin;
  uint32_t layer_count;
  uint32_t kind_flags;  // kind | flags << 8
};

struct TriShade {
  float n0[3];
  float dn1[3];
  float dn2[3];
  float uv0[2];
  float duv1[2];
  float duv2[2];
  float pad;
};
static_assert(sizeof(TriShade) == 64, "TriShade must be 64 bytes");

// Not-in-BVH objects (AxisAlignedPlane, InfiniteFloor)
struct PlaneRec {
  uint32_t kind;   // kPrimPlane / kPrimFloor
  uint32_t axis;   // 0 XY (normal z), 1 XZ (normal y), 2 YZ (normal x)
  float offset;
  float normal_sign;  // +1 or -1 (flip)
  uint32_t object_id;
  uint32_t layer_begin;
  uint32_t layer_count;
  uint32_t flags;
};

struct MaterialDev {
  float emission[3];
  float color[3];
  float ior;
  float phong_exponent;
  int32_t type;
  int32_t texture;
  uint32_t emissive;  // emission.lengthSq() != 0
  uint32_t pad;
};

// Next-event light: an in-BVH object with an emissive layer.
//   kind kLightTriangle: p = v0, e1, e2 (the FP32 geometry the kernels test)
//   kind kLightSphere:   p = centre, r
// le = emission expected over the object's layer roulette.
constexpr uint32_t kLightTriangle = 0u;
constexpr uint32_t kLightSphere = 1u;
struct LightDev {
  float p[3];
  uint32_t kind;
  float e1[3];
  float r;
  float e2[3];
  float pad0;
  float le[3];
  float pad1;
};
static_assert(sizeof(LightDev) == 64, "LightDev must be 64 bytes");

struct LayerDev {
  uint32_t material;
  float rate;
};

struct TextureDev {
  uint64_t offset;  // float offset into texel array (RGB)
  uint32_t width, height;
};

}  // namespace or3
