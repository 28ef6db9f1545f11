// bvh_build_gpu.cu -- the binned-SAH 4-wide build of bvh_build.cpp, on the device.
//
// Replaces the host build (itself replacing the reference's full-sweep SAH,
// src/renderer/BVH.cpp:164-312, and its 4-wide collapse,
// src/renderer/QBVH.cpp:208-272) for large scenes, with the same tree rules:
// binned SAH over centroids with 16 bins (node cost trav_cost, primitive
// cost 1); leaves of at most
// leaf_max primitives when a leaf is not costlier than the best split; the
// binary depth bound kMaxBinaryDepth kept by median splits; the greedy 4-wide
// collapse by largest child area, breadth first when that tree would be too
// deep; 8-bit child boxes on a power-of-two grid, rounded outward.
//
//   phase 1  nodes of more than kSmallTask primitives, one tree level per
//            round: a bounds pass and a binning pass over every primitive of
//            the level (a block whose chunk lies in one node reduces in
//            shared memory first), one thread per node to choose the split,
//            and a stable partition of the index array through a global
//            prefix sum, so the build is deterministic;
//   phase 2  subtrees of at most kSmallTask primitives, one warp each,
//            depth first;
//   phase 3  the 4-wide collapse, one level per round, with quantisation;
//            leaves put triangles before spheres.
// A median split of a large node halves its current index range (the host
// build selects by centroid); it happens only for identical centroids or at
// the depth bound.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "bvh_build_gpu.h"
#include "or3_common.h"

namespace or3 {
namespace {

constexpr int kBins = 16;
constexpr uint32_t kSmallTask = 256;  // subtrees of at most this many primitives: one warp each
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kBinWords = 3 * kBins * 7;  // per node: [axis][bin] lo[3], hi[3] (ordered), count
constexpr int kSmallStack = 64;

// Floats as order-preserving unsigned integers (for atomicMin / atomicMax).
__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

struct DNode {
  float lo[3], hi[3];
  int left, right;
  uint32_t first, count;
};

struct Task {
  uint32_t first, count;
  int node, depth;
};

// per large node of the current level
struct Decision {
  int axis;        // -1: halve the index range
  int bin;         // primitives in bins <= bin go left
  uint32_t nleft;
  uint32_t left_task, right_task;  // next-level task ids (kNone: small subtree)
  float cblo, scale;               // binning of the chosen axis
};

struct Counters {
  uint32_t nodes;       // binary nodes allocated
  uint32_t next_tasks;  // large tasks of the next level
  uint32_t small;       // small subtrees
  uint32_t wide;        // wide nodes allocated
  uint32_t items;       // collapse items of the next level
  int bin_depth, wide_depth;
  uint32_t error;
};

__device__ __forceinline__ void cent(const BuildPrim &p, float c[3]) {
  for (int a = 0; a < 3; a++) c[a] = 0.5f * (p.lo[a] + p.hi[a]);
}

__device__ __forceinline__ double box_area(const float lo[3], const float hi[3]) {
  if (!(lo[0] <= hi[0])) return 0.0;
  const double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// The same surface measure in FP32: the device build compares SAH costs
// scaled by the parent's area (no division) in FP32, since GB300's FP64 pipe
// is a small fraction of its FP32 rate.
__device__ __forceinline__ float box_area_f(const float lo[3], const float hi[3]) {
  if (!(lo[0] <= hi[0])) return 0.f;
  const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int ceil_log2(uint64_t v) {
  int r = 0;
  while ((uint64_t(1) << r) < v) r++;
  return r;
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
  int b = (int)((c - lo) * scale);
  return min(max(b, 0), kBins - 1);
}

// ------------------------------------------------------------ phase 1

__global__ void k_init(uint32_t n, uint32_t *idx, uint32_t *ptask) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  idx[i] = i;
  ptask[i] = 0;
}

// node boxes: [lo(3) hi(3) centroid lo(3) centroid hi(3)]; bins: kBinWords per node
__global__ void k_clear_level(uint32_t ntasks, uint32_t *tbox, uint32_t *bins) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ntasks * 12) {
    const uint32_t k = i % 12;
    tbox[i] = (k < 3 || (k >= 6 && k < 9)) ? 0xFFFFFFFFu : 0u;
  }
  if (i < ntasks * kBinWords) {
    const uint32_t k = i % 7;
    bins[i] = k < 3 ? 0xFFFFFFFFu : 0u;
  }
}

constexpr int kChunk = 1024;  // positions per block in the level passes (256 threads x 4)

// Bounds of every large node of the level.  Positions of one node are
// contiguous, so a warp whose 32 positions lie in one node reduces them by
// shuffles and issues one set of atomics; a block whose 1024 positions lie in
// one node reduces across its warps in shared memory first.
__global__ void __launch_bounds__(256) k_bounds(uint32_t n, const uint32_t *idx, const uint32_t *ptask,
                                                const BuildPrim *prims, uint32_t *tbox) {
  __shared__ float red[8][12];
  const uint32_t c0 = blockIdx.x * kChunk;
  if (c0 >= n) return;
  const uint32_t c1 = min(c0 + kChunk, n);
  const uint32_t t0 = ptask[c0], t1 = ptask[c1 - 1];
  const bool uniform = t0 == t1 && t0 != kNone;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float v[12];
  for (int k = 0; k < 12; k++) v[k] = (k < 3 || (k >= 6 && k < 9)) ? FLT_MAX : -FLT_MAX;
  // warp-uniform trip count: every lane takes part in the shuffles
  for (uint32_t base = c0 + warp * 32; base < c1; base += blockDim.x) {
    const uint32_t i = base + lane;
    const uint32_t t = i < c1 ? ptask[i] : kNone;
    float u[12];
    for (int k = 0; k < 12; k++) u[k] = (k < 3 || (k >= 6 && k < 9)) ? FLT_MAX : -FLT_MAX;
    if (t != kNone) {
      const BuildPrim p = prims[idx[i]];
      float c[3];
      cent(p, c);
      for (int a = 0; a < 3; a++) {
        u[a] = p.lo[a];
        u[3 + a] = p.hi[a];
        u[6 + a] = c[a];
        u[9 + a] = c[a];
      }
    }
    if (uniform) {
      for (int k = 0; k < 12; k++) {
        const bool mn = k < 3 || (k >= 6 && k < 9);
        v[k] = mn ? fminf(v[k], u[k]) : fmaxf(v[k], u[k]);
      }
      continue;
    }
    const uint32_t tl = __shfl_sync(0xFFFFFFFFu, t, 0);
    if (__all_sync(0xFFFFFFFFu, t == tl) && tl != kNone) {
      for (int k = 0; k < 12; k++) {
        const bool mn = k < 3 || (k >= 6 && k < 9);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float w = __shfl_xor_sync(0xFFFFFFFFu, u[k], o);
          u[k] = mn ? fminf(u[k], w) : fmaxf(u[k], w);
        }
      }
      if (lane == 0) {
        uint32_t *b = tbox + 12 * (size_t)tl;
        for (int k = 0; k < 12; k++) {
          const bool mn = k < 3 || (k >= 6 && k < 9);
          if (mn) atomicMin(b + k, f2o(u[k]));
          else atomicMax(b + k, f2o(u[k]));
        }
      }
    } else if (t != kNone) {
      uint32_t *b = tbox + 12 * (size_t)t;
      for (int k = 0; k < 12; k++) {
        const bool mn = k < 3 || (k >= 6 && k < 9);
        if (mn) atomicMin(b + k, f2o(u[k]));
        else atomicMax(b + k, f2o(u[k]));
      }
    }
  }
  if (!uniform) return;
  for (int k = 0; k < 12; k++) {
    const bool mn = k < 3 || (k >= 6 && k < 9);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float w = __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
      v[k] = mn ? fminf(v[k], w) : fmaxf(v[k], w);
    }
  }
  if (lane == 0)
    for (int k = 0; k < 12; k++) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    const bool mn = k < 3 || (k >= 6 && k < 9);
    float r = red[0][k];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) r = mn ? fminf(r, red[w][k]) : fmaxf(r, red[w][k]);
    uint32_t *b = tbox + 12 * (size_t)t0;
    if (mn) atomicMin(b + k, f2o(r));
    else atomicMax(b + k, f2o(r));
  }
}

// Per-axis bins of every large node of the level.
__global__ void __launch_bounds__(256) k_bin(uint32_t n, const uint32_t *idx, const uint32_t *ptask,
                                             const BuildPrim *prims, const uint32_t *tbox, uint32_t *bins) {
  __shared__ uint32_t sb[kBinWords];
  const uint32_t c0 = blockIdx.x * kChunk;
  if (c0 >= n) return;
  const uint32_t c1 = min(c0 + kChunk, n);
  const uint32_t t0 = ptask[c0], t1 = ptask[c1 - 1];
  const bool uniform = t0 == t1 && t0 != kNone;
  if (uniform) {
    for (int k = threadIdx.x; k < kBinWords; k += blockDim.x) sb[k] = (k % 7) < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
  }
  for (uint32_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
    const uint32_t t = ptask[i];
    if (t == kNone) continue;
    const BuildPrim p = prims[idx[i]];
    float c[3];
    cent(p, c);
    const uint32_t *tb = tbox + 12 * (size_t)t;
    uint32_t *dst = uniform ? sb : bins + (size_t)kBinWords * t;
    for (int a = 0; a < 3; a++) {
      const float lo = o2f(tb[6 + a]), ext = o2f(tb[9 + a]) - lo;
      const float scale = ext > 0.f ? (float)kBins / ext : 0.f;
      uint32_t *w = dst + (a * kBins + bin_of(c[a], lo, scale)) * 7;
      for (int k = 0; k < 3; k++) {
        atomicMin(w + k, f2o(p.lo[k]));
        atomicMax(w + 3 + k, f2o(p.hi[k]));
      }
      atomicAdd(w + 6, 1u);
    }
  }
  if (!uniform) return;
  __syncthreads();
  uint32_t *g = bins + (size_t)kBinWords * t0;
  for (int k = threadIdx.x; k < kBinWords; k += blockDim.x) {
    const int f = k % 7;
    if (sb[k] == ((f < 3) ? 0xFFFFFFFFu : 0u)) continue;
    if (f < 3) atomicMin(g + k, sb[k]);
    else if (f < 6) atomicMax(g + k, sb[k]);
    else atomicAdd(g + k, sb[k]);
  }
}

// One warp per large node: node record, split choice, children.  Lane b
// evaluates the split after bin b of each axis; the box unions left and right
// of it come from shuffle scans (min/max are exact, so the costs equal a
// sequential scan's), and ties go to the lowest (axis, bin) as in one.
constexpr int kDecideWarps = 4;
__global__ void __launch_bounds__(32 * kDecideWarps) k_decide(uint32_t ntasks, const Task *tasks, const uint32_t *tbox,
                                                              const uint32_t *bins, int leaf_max, double ct,
                                                              DNode *nodes, Decision *dec, Task *next, Task *small,
                                                              Counters *ctr) {
  const uint32_t ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  if (ti >= ntasks) return;  // warp-uniform
  const Task t = tasks[ti];
  const uint32_t *tb = tbox + 12 * (size_t)ti;
  float lo[3], hi[3], cblo[3], cbhi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = o2f(tb[a]);
    hi[a] = o2f(tb[3 + a]);
    cblo[a] = o2f(tb[6 + a]);
    cbhi[a] = o2f(tb[9 + a]);
  }
  Decision d;
  d.axis = -1;
  d.bin = 0;
  d.nleft = t.count / 2;
  d.cblo = 0.f;
  d.scale = 0.f;
  const int need = ceil_log2((t.count + leaf_max - 1) / leaf_max);
  if (t.depth + need < kMaxBinaryDepth) {
    // cost x parent area: ct * A + A_left * n_left + A_right * n_right
    const float parent = fmaxf(box_area_f(lo, hi), 1e-30f), ctp = (float)ct * parent;
    float best = FLT_MAX;
    const uint32_t *B = bins + (size_t)kBinWords * ti;
    for (int a = 0; a < 3; a++) {
      const float ext = cbhi[a] - cblo[a];
      if (!(ext > 0.f)) continue;  // warp-uniform
      float blo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
      uint32_t bc = 0;
      if (lane < (uint32_t)kBins) {
        const uint32_t *w = B + (a * kBins + lane) * 7;
        bc = w[6];
        if (bc)
          for (int k = 0; k < 3; k++) {
            blo[k] = o2f(w[k]);
            bhi[k] = o2f(w[3 + k]);
          }
      }
      // inclusive prefix (bins 0..b) and suffix (bins b..kBins-1) unions
      float plo[3], phi[3], slo[3], shi[3];
      uint32_t pc = bc, sc = bc;
      for (int k = 0; k < 3; k++) {
        plo[k] = slo[k] = blo[k];
        phi[k] = shi[k] = bhi[k];
      }
#pragma unroll
      for (int o = 1; o < kBins; o <<= 1) {
        const uint32_t upc = __shfl_up_sync(0xFFFFFFFFu, pc, o), dnc = __shfl_down_sync(0xFFFFFFFFu, sc, o);
        const bool up = lane >= (uint32_t)o, dn = lane + o < (uint32_t)kBins;
        for (int k = 0; k < 3; k++) {
          const float ul = __shfl_up_sync(0xFFFFFFFFu, plo[k], o), uh = __shfl_up_sync(0xFFFFFFFFu, phi[k], o);
          const float dl = __shfl_down_sync(0xFFFFFFFFu, slo[k], o), dh = __shfl_down_sync(0xFFFFFFFFu, shi[k], o);
          if (up) {
            plo[k] = fminf(plo[k], ul);
            phi[k] = fmaxf(phi[k], uh);
          }
          if (dn) {
            slo[k] = fminf(slo[k], dl);
            shi[k] = fmaxf(shi[k], dh);
          }
        }
        if (up) pc += upc;
        if (dn) sc += dnc;
      }
      // split after bin `lane`: left = prefix[lane], right = suffix[lane + 1]
      const float rarea = __shfl_down_sync(0xFFFFFFFFu, box_area_f(slo, shi), 1);
      const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, sc, 1);
      float cost = FLT_MAX;
      if (lane < (uint32_t)(kBins - 1) && pc != 0 && rc != 0) {
        cost = ctp + box_area_f(plo, phi) * (float)pc + rarea * (float)rc;
        if (!(cost < FLT_MAX)) cost = FLT_MAX;
      }
      float mc = cost;
      uint32_t ml = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(0xFFFFFFFFu, mc, o);
        const uint32_t ol = __shfl_xor_sync(0xFFFFFFFFu, ml, o);
        if (oc < mc || (oc == mc && ol < ml)) {
          mc = oc;
          ml = ol;
        }
      }
      const uint32_t nl = __shfl_sync(0xFFFFFFFFu, pc, ml);
      if (mc < best) {
        best = mc;
        d.axis = a;
        d.bin = (int)ml;
        d.nleft = nl;
      }
    }
    if (d.axis >= 0) {
      d.cblo = cblo[d.axis];
      d.scale = (float)kBins / (cbhi[d.axis] - cblo[d.axis]);
    }
  }
  if (lane != 0) return;
  DNode &nd = nodes[t.node];
  for (int a = 0; a < 3; a++) {
    nd.lo[a] = lo[a];
    nd.hi[a] = hi[a];
  }
  nd.first = t.first;
  nd.count = t.count;
  atomicMax(&ctr->bin_depth, t.depth);
  // large nodes always split (a leaf needs at most leaf_max <= kSmallTask primitives)
  const int l = (int)atomicAdd(&ctr->nodes, 2u);
  nd.left = l;
  nd.right = l + 1;
  const Task kids[2] = {{t.first, d.nleft, l, t.depth + 1}, {t.first + d.nleft, t.count - d.nleft, l + 1, t.depth + 1}};
  uint32_t ids[2];
  for (int k = 0; k < 2; k++) {
    if (kids[k].count > kSmallTask) {
      ids[k] = atomicAdd(&ctr->next_tasks, 1u);
      next[ids[k]] = kids[k];
    } else {
      ids[k] = kNone;
      small[atomicAdd(&ctr->small, 1u)] = kids[k];
    }
  }
  d.left_task = ids[0];
  d.right_task = ids[1];
  dec[ti] = d;
}

__global__ void k_flags(uint32_t n, const uint32_t *idx, const uint32_t *ptask, const Task *tasks,
                        const Decision *dec, const BuildPrim *prims, uint32_t *flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = ptask[i];
  uint32_t f = 0;
  if (t != kNone) {
    const Decision d = dec[t];
    if (d.axis < 0) {
      f = (i - tasks[t].first) < d.nleft ? 1u : 0u;
    } else {
      float c[3];
      cent(prims[idx[i]], c);
      f = bin_of(c[d.axis], d.cblo, d.scale) <= d.bin ? 1u : 0u;
    }
  }
  flags[i] = f;
}

// exclusive prefix sum: blocks of 1024 values, then the block sums (one block), then offsets
constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(256) k_scan_blocks(uint32_t n, const uint32_t *in, uint32_t *out,
                                                     uint32_t *sums) {
  __shared__ uint32_t ws[8];
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  uint32_t v[4], s = 0;
  for (int k = 0; k < 4; k++) {
    v[k] = base + k < n ? in[base + k] : 0u;
    s += v[k];
  }
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if ((int)lane >= o) incl += y;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int w = 0; w < 8; w++) {
      const uint32_t x = ws[w];
      ws[w] = acc;
      acc += x;
    }
    sums[blockIdx.x] = acc;
  }
  __syncthreads();
  uint32_t run = ws[warp] + incl - s;
  for (int k = 0; k < 4; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

// one block of 1024 threads over up to 1024 * 64 block sums
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t nb, uint32_t *sums) {
  __shared__ uint32_t ws[32];
  const uint32_t per = (nb + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per;
  uint32_t s = 0;
  for (uint32_t k = 0; k < per; k++)
    if (b0 + k < nb) s += sums[b0 + k];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if ((int)lane >= o) incl += y;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int w = 0; w < 32; w++) {
      const uint32_t x = ws[w];
      ws[w] = acc;
      acc += x;
    }
  }
  __syncthreads();
  uint32_t run = ws[warp] + incl - s;
  for (uint32_t k = 0; k < per; k++) {
    if (b0 + k < nb) {
      const uint32_t x = sums[b0 + k];
      sums[b0 + k] = run;
      run += x;
    }
  }
}

__global__ void k_scan_add(uint32_t n, uint32_t *out, const uint32_t *sums) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / kScanBlock];
}

// Stable partition of every large node's range; leaves the rest in place.
__global__ void k_scatter(uint32_t n, const uint32_t *idx, const uint32_t *ptask, const Task *tasks,
                          const Decision *dec, const uint32_t *flags, const uint32_t *scan, uint32_t *idx2,
                          uint32_t *ptask2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = ptask[i];
  if (t == kNone) {
    idx2[i] = idx[i];
    ptask2[i] = kNone;
    return;
  }
  const Task tk = tasks[t];
  const Decision d = dec[t];
  const uint32_t lrank = scan[i] - scan[tk.first];
  uint32_t dst;
  uint32_t nt;
  if (flags[i]) {
    dst = tk.first + lrank;
    nt = d.left_task;
  } else {
    dst = tk.first + d.nleft + (i - tk.first - lrank);
    nt = d.right_task;
  }
  idx2[dst] = idx[i];
  ptask2[dst] = nt;
}

// ------------------------------------------------------------ phase 2

// (centroid on axis, primitive index) order, for median splits
__device__ __forceinline__ bool cent_less(const BuildPrim *prims, int axis, uint32_t x, uint32_t y) {
  const float cx = 0.5f * (prims[x].lo[axis] + prims[x].hi[axis]);
  const float cy = 0.5f * (prims[y].lo[axis] + prims[y].hi[axis]);
  if (cx != cy) return cx < cy;
  return x < y;
}

constexpr int kSmallWarps = 4;  // warps per block of k_small

struct SmallShared {
  uint32_t bins[kBinWords];  // [axis][bin] lo[3], hi[3] (ordered), count
  uint32_t tmp[kSmallTask];  // partition buffer
  Task stk[kSmallStack];
};

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}

// One warp builds a whole subtree of at most kSmallTask primitives, depth
// first, with the host builder's per-node rules: lanes share the bounds,
// binning (shared-memory atomics) and partition (stable, through a shared
// buffer); lane 0 evaluates the SAH and owns the stack.
__global__ void __launch_bounds__(32 * kSmallWarps) k_small(uint32_t nsmall, const Task *small,
                                                            const BuildPrim *prims, uint32_t *idx, int leaf_max,
                                                            double ct, DNode *nodes, Counters *ctr) {
  __shared__ SmallShared sh_all[kSmallWarps];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t si = blockIdx.x * kSmallWarps + (threadIdx.x >> 5);
  if (si >= nsmall) return;  // whole warps only; no block-wide barrier below
  SmallShared &sh = sh_all[threadIdx.x >> 5];
  const Task root = small[si];
  uint32_t next = 0;
  if (lane == 0 && root.count > 1) next = atomicAdd(&ctr->nodes, 2 * root.count - 2);
  next = __shfl_sync(0xFFFFFFFFu, next, 0);
  if (lane == 0) sh.stk[0] = root;
  int sp = 1;
  int maxd = root.depth;
  __syncwarp();
  while (sp > 0) {
    sp--;
    const Task t = sh.stk[sp];
    __syncwarp();
    maxd = max(maxd, t.depth);
    const uint32_t end = t.first + t.count;
    float lo[3], hi[3], clo[3], chi[3];
    for (int a = 0; a < 3; a++) {
      lo[a] = clo[a] = FLT_MAX;
      hi[a] = chi[a] = -FLT_MAX;
    }
    for (uint32_t i = t.first + lane; i < end; i += 32) {
      const BuildPrim p = prims[idx[i]];
      float c[3];
      cent(p, c);
      for (int a = 0; a < 3; a++) {
        lo[a] = fminf(lo[a], p.lo[a]);
        hi[a] = fmaxf(hi[a], p.hi[a]);
        clo[a] = fminf(clo[a], c[a]);
        chi[a] = fmaxf(chi[a], c[a]);
      }
    }
    for (int a = 0; a < 3; a++) {
      lo[a] = warp_min(lo[a]);
      hi[a] = warp_max(hi[a]);
      clo[a] = warp_min(clo[a]);
      chi[a] = warp_max(chi[a]);
    }
    if (lane == 0) {
      DNode &nd = nodes[t.node];
      for (int a = 0; a < 3; a++) {
        nd.lo[a] = lo[a];
        nd.hi[a] = hi[a];
      }
      nd.first = t.first;
      nd.count = t.count;
      nd.left = nd.right = -1;
    }
    if (t.count <= 1) continue;
    const int need = ceil_log2((t.count + leaf_max - 1) / leaf_max);
    int axis = -1, bin = 0, mode = 0;  // mode 0 SAH split, 1 median split, 2 leaf
    uint32_t nleft = 0;
    float scale = 0.f;
    if (t.depth + need >= kMaxBinaryDepth) {
      mode = t.count <= (uint32_t)leaf_max ? 2 : 1;
    } else {
      for (int k = lane; k < kBinWords; k += 32) sh.bins[k] = (k % 7) < 3 ? 0xFFFFFFFFu : 0u;
      __syncwarp();
      float sc[3];
      for (int a = 0; a < 3; a++) {
        const float ext = chi[a] - clo[a];
        sc[a] = ext > 0.f ? (float)kBins / ext : 0.f;
      }
      for (uint32_t i = t.first + lane; i < end; i += 32) {
        const BuildPrim p = prims[idx[i]];
        float c[3];
        cent(p, c);
        for (int a = 0; a < 3; a++) {
          uint32_t *w = sh.bins + (a * kBins + bin_of(c[a], clo[a], sc[a])) * 7;
          for (int k = 0; k < 3; k++) {
            atomicMin(w + k, f2o(p.lo[k]));
            atomicMax(w + 3 + k, f2o(p.hi[k]));
          }
          atomicAdd(w + 6, 1u);
        }
      }
      __syncwarp();
      // SAH over the 3 x 15 split candidates, one bin per lane: prefix and
      // suffix unions by shuffle scans (min / max are exact); costs scaled by
      // the parent's area in FP32; ties go to the lowest (axis, bin) like a
      // sequential scan with a strict <
      const float parent = fmaxf(box_area_f(lo, hi), 1e-30f), ctp = (float)ct * parent;
      float bestc = FLT_MAX;
      uint32_t bidx = 0xFFFFFFFFu, bcnt = 0;
      for (int a = 0; a < 3; a++) {
        if (!(chi[a] - clo[a] > 0.f)) continue;
        float plo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, phi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t pc = 0;
        if (lane < (uint32_t)kBins) {
          const uint32_t *w = sh.bins + (a * kBins + lane) * 7;
          pc = w[6];
          if (pc)
            for (int k = 0; k < 3; k++) {
              plo[k] = o2f(w[k]);
              phi[k] = o2f(w[3 + k]);
            }
        }
        float slo[3] = {plo[0], plo[1], plo[2]}, shi[3] = {phi[0], phi[1], phi[2]};
        uint32_t sc2 = pc;
#pragma unroll
        for (int o = 1; o < kBins; o <<= 1) {
          float ulo[3], uhi[3], dlo[3], dhi[3];
          for (int k = 0; k < 3; k++) {
            ulo[k] = __shfl_up_sync(0xFFFFFFFFu, plo[k], o);
            uhi[k] = __shfl_up_sync(0xFFFFFFFFu, phi[k], o);
            dlo[k] = __shfl_down_sync(0xFFFFFFFFu, slo[k], o);
            dhi[k] = __shfl_down_sync(0xFFFFFFFFu, shi[k], o);
          }
          const uint32_t uc = __shfl_up_sync(0xFFFFFFFFu, pc, o), dc = __shfl_down_sync(0xFFFFFFFFu, sc2, o);
          if (lane >= (uint32_t)o) {
            for (int k = 0; k < 3; k++) {
              plo[k] = fminf(plo[k], ulo[k]);
              phi[k] = fmaxf(phi[k], uhi[k]);
            }
            pc += uc;
          }
          if (lane + o < 32u) {
            for (int k = 0; k < 3; k++) {
              slo[k] = fminf(slo[k], dlo[k]);
              shi[k] = fmaxf(shi[k], dhi[k]);
            }
            sc2 += dc;
          }
        }
        // the right side of the split after bin `lane` is the suffix from lane + 1
        float rlo[3], rhi[3];
        for (int k = 0; k < 3; k++) {
          rlo[k] = __shfl_down_sync(0xFFFFFFFFu, slo[k], 1);
          rhi[k] = __shfl_down_sync(0xFFFFFFFFu, shi[k], 1);
        }
        const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, sc2, 1);
        if (lane < (uint32_t)kBins - 1 && pc != 0 && rc != 0) {
          const float cost = ctp + box_area_f(plo, phi) * (float)pc + box_area_f(rlo, rhi) * (float)rc;
          if (cost < bestc) {
            bestc = cost;
            bidx = (uint32_t)(a * kBins) + lane;
            bcnt = pc;
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float c2 = __shfl_xor_sync(0xFFFFFFFFu, bestc, o);
        const uint32_t i2 = __shfl_xor_sync(0xFFFFFFFFu, bidx, o), n2 = __shfl_xor_sync(0xFFFFFFFFu, bcnt, o);
        if (c2 < bestc || (c2 == bestc && i2 < bidx)) {
          bestc = c2;
          bidx = i2;
          bcnt = n2;
        }
      }
      if (bidx != 0xFFFFFFFFu) {
        axis = (int)(bidx / kBins);
        bin = (int)(bidx % kBins);
        nleft = bcnt;
      }
      if (t.count <= (uint32_t)leaf_max && (axis < 0 || (float)t.count * parent <= bestc)) mode = 2;
      else if (axis < 0) mode = 1;
      if (axis >= 0) scale = sc[axis];
    }
    if (mode == 2) continue;
    if (mode == 1) {
      // the count/2 smallest by (centroid on the widest centroid axis, index): rank sort
      int ma = 0;
      float wd = -1.f;
      for (int a = 0; a < 3; a++)
        if (chi[a] - clo[a] > wd) {
          wd = chi[a] - clo[a];
          ma = a;
        }
      for (uint32_t j = t.first + lane; j < end; j += 32) {
        const uint32_t v = idx[j];
        uint32_t rank = 0;
        for (uint32_t k = t.first; k < end; k++) rank += cent_less(prims, ma, idx[k], v) ? 1u : 0u;
        sh.tmp[rank] = v;
      }
      nleft = t.count / 2;
    } else {
      // stable partition by the chosen bin
      uint32_t nl = 0, nr = 0;
      for (uint32_t b = t.first; b < end; b += 32) {
        const uint32_t i = b + lane;
        bool in = i < end, left = false;
        uint32_t v = 0;
        if (in) {
          v = idx[i];
          float c[3];
          cent(prims[v], c);
          left = bin_of(c[axis], clo[axis], scale) <= bin;
        }
        const uint32_t ml = __ballot_sync(0xFFFFFFFFu, in && left), mr = __ballot_sync(0xFFFFFFFFu, in && !left);
        const uint32_t below = (1u << lane) - 1u;
        if (in) sh.tmp[left ? nl + __popc(ml & below) : nleft + nr + __popc(mr & below)] = v;
        nl += __popc(ml);
        nr += __popc(mr);
      }
    }
    __syncwarp();
    for (uint32_t j = lane; j < t.count; j += 32) idx[t.first + j] = sh.tmp[j];
    __syncwarp();
    const uint32_t split = t.first + nleft;
    if (sp + 2 > kSmallStack) {
      if (lane == 0) atomicOr(&ctr->error, 1u);
      continue;
    }
    const int l = (int)next;
    next += 2;
    if (lane == 0) {
      nodes[t.node].left = l;
      nodes[t.node].right = l + 1;
      sh.stk[sp] = {split, end - split, l + 1, t.depth + 1};
      sh.stk[sp + 1] = {t.first, split - t.first, l, t.depth + 1};
    }
    sp += 2;
    __syncwarp();
  }
  if (lane == 0) atomicMax(&ctr->bin_depth, maxd);
}

// ------------------------------------------------------------ phase 3

struct WItem {
  int root;
  uint32_t slot;
  int depth;
};

// Child boxes against the node box: step 2^e per axis, 255 steps, rounded
// outward and re-checked in float (the host build's quantise()).
__device__ void quantise(WideNode &w, const float *nlo, const float *nhi, const float (*clo)[3],
                         const float (*chi)[3], int nchild) {
  for (int a = 0; a < 3; a++) {
    const float org = nlo[a];
    w.origin[a] = org;
    const double ext = (double)nhi[a] - (double)org;
    int e = -126;
    if (ext > 0) e = max((int)ceil(log2(ext / 255.0)), -126);
    for (;;) {
      const float step = ldexpf(1.0f, e);
      bool ok = __fadd_rn(org, __fmul_rn(255.0f, step)) >= nhi[a];
      for (int c = 0; c < nchild && ok; c++) {
        double ql = floor(((double)clo[c][a] - org) / step);
        double qh = ceil(((double)chi[c][a] - org) / step);
        ql = fmax(0.0, fmin(255.0, ql));
        qh = fmax(0.0, fmin(255.0, qh));
        while (ql > 0 && __fadd_rn(org, __fmul_rn((float)ql, step)) > clo[c][a]) ql -= 1;
        while (qh < 255 && __fadd_rn(org, __fmul_rn((float)qh, step)) < chi[c][a]) qh += 1;
        if (__fadd_rn(org, __fmul_rn((float)ql, step)) > clo[c][a] ||
            __fadd_rn(org, __fmul_rn((float)qh, step)) < chi[c][a]) {
          ok = false;
          break;
        }
        w.lo[a][c] = (uint8_t)ql;
        w.hi[a][c] = (uint8_t)qh;
      }
      if (ok) break;
      e++;
    }
    w.exp[a] = (uint8_t)(e + 127);
  }
}

__device__ __forceinline__ double node_area(const DNode &n) { return box_area(n.lo, n.hi); }

// wbox: per wide node the 24 FP32 child bounds in WideNodeF::b order.
__global__ void k_collapse(uint32_t nin, const WItem *in, const DNode *bn, int breadth_first, WideNode *wn,
                           float *wbox, WItem *out, Counters *ctr) {
  const uint32_t ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= nin) return;
  const WItem it = in[ii];
  int kids[4];
  int nk = 0;
  const DNode &r = bn[it.root];
  if (r.left < 0) {
    kids[nk++] = it.root;
  } else {
    kids[nk++] = r.left;
    kids[nk++] = r.right;
    if (breadth_first) {
      int nx[4];
      int m = 0;
      for (int k = 0; k < 2; k++) {
        const DNode &c = bn[kids[k]];
        if (c.left < 0) {
          nx[m++] = kids[k];
        } else {
          nx[m++] = c.left;
          nx[m++] = c.right;
        }
      }
      for (int k = 0; k < m; k++) kids[k] = nx[k];
      nk = m;
    } else {
      while (nk < 4) {
        int best = -1;
        double ba = -1;
        for (int k = 0; k < nk; k++) {
          if (bn[kids[k]].left < 0) continue;
          const double a = node_area(bn[kids[k]]);
          if (a > ba) {
            ba = a;
            best = k;
          }
        }
        if (best < 0) break;
        const int k = kids[best];
        kids[best] = bn[k].left;
        kids[nk++] = bn[k].right;
      }
    }
  }
  WideNode w;
  memset(&w, 0, sizeof(w));
  float clo[4][3], chi[4][3];
  for (int k = 0; k < nk; k++) {
    const DNode &c = bn[kids[k]];
    for (int a = 0; a < 3; a++) {
      clo[k][a] = c.lo[a];
      chi[k][a] = c.hi[a];
    }
    if (c.left < 0) {
      w.child[k] = c.first;
      w.count[k] = (uint8_t)c.count;  // total; split by kind in k_leaf_kinds
    } else {
      const uint32_t s = atomicAdd(&ctr->wide, 1u);
      w.child[k] = s;
      w.imask |= (uint8_t)(1u << k);
      out[atomicAdd(&ctr->items, 1u)] = {kids[k], s, it.depth + 1};
    }
  }
  quantise(w, r.lo, r.hi, clo, chi, nk);
  wn[it.slot] = w;
  float *fb = wbox + 24 * (size_t)it.slot;
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 4; k++) {
      float lo = INFINITY, hi = -INFINITY;
      if (k < nk) fnode_slab(r.lo[a], r.hi[a], clo[k][a], chi[k][a], &lo, &hi);
      fb[(2 * a) * 4 + k] = lo;
      fb[(2 * a + 1) * 4 + k] = hi;
    }
  atomicMax(&ctr->wide_depth, it.depth);
}

// FP32-box nodes: the child bounds with the final child / count / imask.
__global__ void k_make_fnodes(uint32_t nw, const WideNode *wn, const float *wbox, WideNodeF *fn) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nw) return;
  const WideNode w = wn[i];
  WideNodeF f;
  for (int k = 0; k < 24; k++) f.b[k / 4][k % 4] = wbox[24 * (size_t)i + k];
  for (int c = 0; c < 4; c++) {
    f.child[c] = w.child[c];
    f.count[c] = w.count[c];
  }
  f.imask = w.imask;
  f.pad[0] = f.pad[1] = 0u;
  fn[i] = f;
}

// Leaves: triangles before spheres, count = ntri | nsph << 4.
__global__ void k_leaf_kinds(uint32_t nw, WideNode *wn, uint32_t *order, const BuildPrim *prims) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nw) return;
  WideNode &w = wn[i];
  for (int k = 0; k < 4; k++) {
    if (w.imask & (1u << k)) continue;
    const uint32_t cnt = w.count[k];
    if (cnt == 0) continue;
    uint32_t *b = order + w.child[k];
    uint32_t tri[15], sph[15], nt = 0, ns = 0;
    for (uint32_t j = 0; j < cnt; j++) {
      if (prims[b[j]].kind == kPrimTriangle) tri[nt++] = b[j];
      else sph[ns++] = b[j];
    }
    for (uint32_t j = 0; j < nt; j++) b[j] = tri[j];
    for (uint32_t j = 0; j < ns; j++) b[nt + j] = sph[j];
    w.count[k] = (uint8_t)(nt | (ns << 4));
  }
}

// Temporaries: stream-ordered from `pool` when given (no device-wide sync
// on free), else cudaMalloc / cudaFree.
struct TempAlloc {
  cudaMemPool_t pool;
  cudaStream_t st;
  template <class T>
  cudaError_t get(T **p, size_t n) const {
    *p = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (pool) return cudaMallocFromPoolAsync(reinterpret_cast<void **>(p), bytes, pool, st);
    return cudaMalloc(p, bytes);
  }
  void put(void *p) const {
    if (!p) return;
    if (pool) cudaFreeAsync(p, st);
    else cudaFree(p);
  }
};

template <class T>
cudaError_t grow(const TempAlloc &ta, T **p, size_t &cap, size_t n) {
  if (n <= cap) return cudaSuccess;
  ta.put(*p);
  *p = nullptr;
  cap = 0;
  const cudaError_t e = ta.get(p, n);
  if (e == cudaSuccess) cap = n;
  return e;
}

}  // namespace

bool build_wide_bvh_device(const BuildPrim *prims, uint32_t n, int leaf_max, cudaStream_t st, DeviceBVH &out,
                           std::string *err, double trav_cost, cudaMemPool_t pool) {
  out = DeviceBVH();
  const TempAlloc ta{pool, st};
  auto fail = [&](const char *what, cudaError_t e) {
    if (err) *err = std::string("device BVH build: ") + what + ": " + cudaGetErrorString(e);
    return false;
  };
  if (n == 0 || n > (1u << 26) || leaf_max < 1 || leaf_max > 8 || !(trav_cost > 0)) {
    if (err) *err = "device BVH build: 1 <= primitives <= 2^26, leaf_max in [1,8], traversal cost > 0";
    return false;
  }
  uint32_t *idx = nullptr, *idx2 = nullptr, *pt = nullptr, *pt2 = nullptr, *flags = nullptr, *scan = nullptr,
           *sums = nullptr, *tbox = nullptr, *bins = nullptr;
  Task *tasks = nullptr, *next = nullptr, *small = nullptr;
  Decision *dec = nullptr;
  DNode *nodes = nullptr;
  WItem *wa = nullptr, *wb = nullptr;
  WideNode *wide = nullptr;
  float *wbox = nullptr;
  Counters *ctr = nullptr;
  Counters hc{};
  const uint32_t ntmax = n / (kSmallTask + 1) + 2;  // large tasks of one level
  const uint32_t nsb = (n + kScanBlock - 1) / kScanBlock;
  bool ok = false;
  cudaError_t e = cudaSuccess;
  do {
    size_t c0 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, c5 = 0, c6 = 0, c7 = 0, c8 = 0, c9 = 0, c10 = 0, c11 = 0,
           c12 = 0, c13 = 0, c14 = 0, c15 = 0, c16 = 0;
    if ((e = grow(ta, &idx, c0, n)) || (e = grow(ta, &idx2, c1, n)) || (e = grow(ta, &pt, c2, n)) ||
        (e = grow(ta, &pt2, c3, n)) || (e = grow(ta, &flags, c4, n)) || (e = grow(ta, &scan, c5, n)) ||
        (e = grow(ta, &sums, c6, nsb)) || (e = grow(ta, &tbox, c7, 12 * (size_t)ntmax)) ||
        (e = grow(ta, &bins, c8, (size_t)kBinWords * ntmax)) || (e = grow(ta, &tasks, c9, ntmax)) ||
        (e = grow(ta, &next, c10, ntmax)) || (e = grow(ta, &small, c11, n)) || (e = grow(ta, &dec, c12, ntmax)) ||
        (e = grow(ta, &nodes, c13, 2 * (size_t)n)) || (e = grow(ta, &wa, c14, n)) || (e = grow(ta, &wb, c15, n)) ||
        (e = grow(ta, &ctr, c16, 1))) {
      fail("allocation", e);
      break;
    }
    if ((e = ta.get(&wide, (size_t)n)) || (e = ta.get(&wbox, (size_t)n * 24))) {
      fail("allocation", e);
      break;
    }
    // phase 1
    hc = Counters{};
    hc.nodes = 1;
    const Task root{0, n, 0, 1};
    uint32_t ntasks = 0;
    if (n > kSmallTask) {
      ntasks = 1;
      cudaMemcpyAsync(tasks, &root, sizeof(Task), cudaMemcpyHostToDevice, st);
    } else {
      hc.small = 1;
      cudaMemcpyAsync(small, &root, sizeof(Task), cudaMemcpyHostToDevice, st);
    }
    cudaMemcpyAsync(ctr, &hc, sizeof(Counters), cudaMemcpyHostToDevice, st);
    k_init<<<(n + 255) / 256, 256, 0, st>>>(n, idx, pt);
    const uint32_t nblk = (n + kChunk - 1) / kChunk;
    while (ntasks > 0) {
      const size_t clear = std::max<size_t>(12 * (size_t)ntasks, (size_t)kBinWords * ntasks);
      k_clear_level<<<(unsigned)((clear + 255) / 256), 256, 0, st>>>(ntasks, tbox, bins);
      k_bounds<<<nblk, 256, 0, st>>>(n, idx, pt, prims, tbox);
      k_bin<<<nblk, 256, 0, st>>>(n, idx, pt, prims, tbox, bins);
      cudaMemsetAsync(&ctr->next_tasks, 0, sizeof(uint32_t), st);
      k_decide<<<(ntasks + kDecideWarps - 1) / kDecideWarps, 32 * kDecideWarps, 0, st>>>(
          ntasks, tasks, tbox, bins, leaf_max, trav_cost, nodes, dec, next, small, ctr);
      k_flags<<<(n + 255) / 256, 256, 0, st>>>(n, idx, pt, tasks, dec, prims, flags);
      k_scan_blocks<<<nsb, 256, 0, st>>>(n, flags, scan, sums);
      k_scan_sums<<<1, 1024, 0, st>>>(nsb, sums);
      k_scan_add<<<(n + 255) / 256, 256, 0, st>>>(n, scan, sums);
      k_scatter<<<(n + 255) / 256, 256, 0, st>>>(n, idx, pt, tasks, dec, flags, scan, idx2, pt2);
      std::swap(idx, idx2);
      std::swap(pt, pt2);
      std::swap(tasks, next);
      if ((e = cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st)) ||
          (e = cudaStreamSynchronize(st))) {
        fail("large nodes", e);
        break;
      }
      ntasks = hc.next_tasks;
    }
    if (e) break;
    // phase 2
    if ((e = cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st))) {
      fail("counters", e);
      break;
    }
    if (hc.small)
      k_small<<<(hc.small + kSmallWarps - 1) / kSmallWarps, 32 * kSmallWarps, 0, st>>>(hc.small, small, prims, idx,
                                                                                       leaf_max, trav_cost, nodes, ctr);
    // phase 3: greedy collapse, breadth first if that is deeper than the stack allows
    for (int pass = 0; pass < 2; pass++) {
      const uint32_t one = 1, zero = 0;
      const int izero = 0;
      cudaMemcpyAsync(&ctr->wide, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(&ctr->wide_depth, &izero, sizeof(int), cudaMemcpyHostToDevice, st);
      const WItem r{0, 0u, 1};
      cudaMemcpyAsync(wa, &r, sizeof(WItem), cudaMemcpyHostToDevice, st);
      uint32_t nin = 1;
      WItem *a = wa, *b = wb;
      while (nin > 0) {
        cudaMemcpyAsync(&ctr->items, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice, st);
        k_collapse<<<(nin + 127) / 128, 128, 0, st>>>(nin, a, nodes, pass, wide, wbox, b, ctr);
        if ((e = cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st))) {
          fail("collapse", e);
          break;
        }
        nin = hc.items;
        std::swap(a, b);
      }
      if (e) break;
      if (hc.wide_depth <= kMaxBinaryDepth / 2) break;
    }
    if (e) break;
    if (hc.error) {
      if (err) *err = "device BVH build: subtree stack exhausted";
      break;
    }
    k_leaf_kinds<<<(hc.wide + 127) / 128, 128, 0, st>>>(hc.wide, wide, idx, prims);
    // exact-size outputs
    if ((e = cudaMalloc(&out.nodes, (size_t)hc.wide * sizeof(WideNode))) ||
        (e = cudaMemcpyAsync(out.nodes, wide, (size_t)hc.wide * sizeof(WideNode), cudaMemcpyDeviceToDevice, st)) ||
        (e = cudaMalloc(&out.fnodes, (size_t)hc.wide * sizeof(WideNodeF)))) {
      fail("output", e);
      break;
    }
    k_make_fnodes<<<(hc.wide + 127) / 128, 128, 0, st>>>(hc.wide, wide, wbox, out.fnodes);
    out.order = idx;
    idx = nullptr;  // handed to the caller
    out.num_nodes = hc.wide;
    out.binary_depth = hc.bin_depth;
    out.wide_depth = hc.wide_depth;
    out.binary_nodes = hc.nodes;
    if ((e = cudaStreamSynchronize(st))) {
      fail("finish", e);
      break;
    }
    ok = true;
  } while (false);
  cudaStreamSynchronize(st);
  for (void *p : {(void *)idx, (void *)idx2, (void *)pt, (void *)pt2, (void *)flags, (void *)scan, (void *)sums,
                  (void *)tbox, (void *)bins, (void *)tasks, (void *)next, (void *)small, (void *)dec,
                  (void *)nodes, (void *)wa, (void *)wb, (void *)wide, (void *)wbox, (void *)ctr})
    ta.put(p);
  if (!ok) {
    cudaFree(out.nodes);
    cudaFree(out.fnodes);
    ta.put(out.order);
    out = DeviceBVH();
  }
  return ok;
}

__global__ void k_gather_leaf_order(uint32_t n, const uint32_t *order, const float4 *prims_in,
                                    const PrimInfo *info_in, const TriShade *shade_in, float4 *prims_out,
                                    PrimInfo *info_out, TriShade *shade_out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint32_t s = order[r];
  for (int k = 0; k < 3; k++) prims_out[3 * (size_t)r + k] = prims_in[3 * (size_t)s + k];
  info_out[r] = info_in[s];
  shade_out[r] = shade_in[s];
}

void gather_leaf_order(uint32_t n, const uint32_t *order, const float4 *prims_in, const PrimInfo *info_in,
                       const TriShade *shade_in, float4 *prims_out, PrimInfo *info_out, TriShade *shade_out,
                       cudaStream_t st) {
  if (n) k_gather_leaf_order<<<(n + 255) / 256, 256, 0, st>>>(n, order, prims_in, info_in, shade_in, prims_out,
                                                              info_out, shade_out);
}

}  // namespace or3
