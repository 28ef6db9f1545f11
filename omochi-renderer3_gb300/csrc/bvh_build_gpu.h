// bvh_build_gpu.h -- device build of the 4-wide BVH (bvh_build_gpu.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "bvh_build.h"

namespace or3 {

// Device-resident result: nodes[num_nodes] (root at 0), the same tree with
// FP32 child boxes (fnodes) and the leaf order (record r holds input
// primitive order[r]), all cudaMalloc'd and owned by the caller.
struct DeviceBVH {
  WideNode *nodes = nullptr;
  WideNodeF *fnodes = nullptr;
  uint32_t *order = nullptr;
  uint32_t num_nodes = 0;
  int binary_depth = 0;
  int wide_depth = 0;
  size_t binary_nodes = 0;
};

// prims: device array of n primitive bounds (input order).  Blocks on `st`.
// Returns false (with *err) on invalid input or a CUDA error.  pool: where
// the temporaries (and out.order) come from, stream-ordered on `st`; null =
// cudaMalloc (then out.order is freed with cudaFree).
bool build_wide_bvh_device(const BuildPrim *prims, uint32_t n, int leaf_max, cudaStream_t st, DeviceBVH &out,
                           std::string *err, double trav_cost = 1.0, cudaMemPool_t pool = nullptr);

// Records, PrimInfo and TriShade from input order into leaf order.
void gather_leaf_order(uint32_t n, const uint32_t *order, const float4 *prims_in, const PrimInfo *info_in,
                       const TriShade *shade_in, float4 *prims_out, PrimInfo *info_out, TriShade *shade_out,
                       cudaStream_t st);

}  // namespace or3
