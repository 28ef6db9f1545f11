// bvh_build.h -- host build of the 4-wide quantised BVH.
//
// Replaces the reference's full-sweep object SAH (BVH::Construct_internal,
// src/renderer/BVH.cpp:164-312) and its 4-wide collapse
// (QBVH::Construct_internal, src/renderer/QBVH.cpp:208-272) with a binned SAH
// build (16 bins by default, leaves of at most 4 primitives) collapsed into
// 64-byte WideNode records.
#pragma once

#include <string>
#include <vector>

#include "or3_common.h"

namespace or3 {

struct BuildPrim {
  float lo[3], hi[3];
  uint32_t kind;  // kPrimTriangle or kPrimSphere
};

struct WideBVH {
  std::vector<WideNode> nodes;   // node 0 is the root
  std::vector<float> boxes;      // per node 24 floats: the children's exact boxes as WideNodeF::b
  std::vector<uint32_t> order;   // leaf order: record i holds input prim order[i]
  int binary_depth = 0;
  int wide_depth = 0;
  size_t binary_nodes = 0;
};

// Returns false (with *err) on invalid input.  An empty prim list yields an
// empty node array.
// trav_cost: SAH cost of visiting a node, relative to one primitive test.
bool build_wide_bvh(const std::vector<BuildPrim> &prims, int bins, int leaf_max, WideBVH &out,
                    std::string *err, double trav_cost = 1.0);

// FP32-box nodes (WideNodeF) from a built tree's topology and exact child boxes.
void make_float_nodes(const WideBVH &bvh, std::vector<WideNodeF> &out);
// The 8-wide tree of the 8-wide traversal variant from a 4-wide FP32-box tree
// (bvh_wide8.cpp); false if a ray could need more than kStackSize8 stack
// entries (*max_push: the bound found).
bool make_wide8_nodes(const std::vector<WideNodeF> &n4, std::vector<WideNode8F> &out, int *max_push);

// Decoded child box of a quantised node, exactly as the kernels compute it.
void decode_child_box(const WideNode &n, int child, float lo[3], float hi[3]);

}  // namespace or3
