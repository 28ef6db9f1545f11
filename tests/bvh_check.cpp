// bvh_check.cpp -- CPU property check of the host wide-BVH builder, compiled
// by tests/test_bvh_builder.py together with csrc/bvh_build.cpp.
//
//   bvh_check <n> <seed> <mode>     mode 0: random boxes, 1: all identical,
//                                   2: thin slivers along x, 3: mixed kinds
// Checks: every primitive sits in exactly one leaf slot; every primitive box
// lies inside each decoded box (as the kernels decode them) on its path from
// the root; leaf slots hold <= 4 primitives, triangles before spheres; the
// wide depth stays within the traversal stack bound.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "bvh_build.h"

using namespace or3;

static int fails = 0;
#define CHECK(c, ...)                       \
  do {                                      \
    if (!(c)) {                             \
      if (fails < 10) printf(__VA_ARGS__);  \
      fails++;                              \
    }                                       \
  } while (0)

struct Box { float lo[3], hi[3]; };

static void visit(const WideBVH &b, const std::vector<BuildPrim> &prims, uint32_t node, std::vector<Box> &anc,
                  std::vector<int> &seen, int depth) {
  CHECK(depth <= 20, "depth %d\n", depth);
  CHECK(node < b.nodes.size(), "node index %u out of range\n", node);
  if (node >= b.nodes.size() || depth > 64) return;
  const WideNode &w = b.nodes[node];
  for (int c = 0; c < 4; c++) {
    Box bx;
    decode_child_box(w, c, bx.lo, bx.hi);
    if (w.imask & (1u << c)) {
      anc.push_back(bx);
      visit(b, prims, w.child[c], anc, seen, depth + 1);
      anc.pop_back();
    } else if (w.count[c]) {
      const uint32_t nt = w.count[c] & 15u, ns = w.count[c] >> 4;
      CHECK(nt + ns >= 1 && nt + ns <= 4, "leaf size %u\n", nt + ns);
      for (uint32_t k = 0; k < nt + ns; k++) {
        const uint32_t r = w.child[c] + k;
        CHECK(r < prims.size(), "record out of range\n");
        if (r >= prims.size()) continue;
        const uint32_t src = b.order[r];
        seen[src]++;
        CHECK((k < nt) == (prims[src].kind == kPrimTriangle), "kind order in leaf\n");
        anc.push_back(bx);
        for (const Box &a : anc)
          for (int ax = 0; ax < 3; ax++)
            CHECK(a.lo[ax] <= prims[src].lo[ax] && a.hi[ax] >= prims[src].hi[ax],
                  "prim %u axis %d [%g,%g] outside [%g,%g]\n", src, ax, prims[src].lo[ax], prims[src].hi[ax],
                  a.lo[ax], a.hi[ax]);
        anc.pop_back();
      }
    }
  }
}

int main(int argc, char **argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 1000;
  const int seed = argc > 2 ? atoi(argv[2]) : 1;
  const int mode = argc > 3 ? atoi(argv[3]) : 0;
  std::mt19937 rng(seed);
  std::uniform_real_distribution<float> U(-100.f, 100.f), S(0.01f, 5.f);
  std::vector<BuildPrim> prims(n);
  for (int i = 0; i < n; i++) {
    BuildPrim &q = prims[i];
    for (int a = 0; a < 3; a++) {
      const float c = mode == 1 ? 1.f : U(rng);
      float s = mode == 1 ? 0.5f : S(rng);
      if (mode == 2 && a != 0) s = 1e-4f;
      q.lo[a] = c - s;
      q.hi[a] = c + s;
    }
    q.kind = (mode == 3 && (i % 3 == 0)) ? kPrimSphere : kPrimTriangle;
  }
  WideBVH b;
  std::string err;
  if (!build_wide_bvh(prims, 16, 4, b, &err)) {
    printf("build failed: %s\n", err.c_str());
    return 2;
  }
  std::vector<int> seen(n, 0);
  std::vector<Box> anc;
  if (n > 0) visit(b, prims, 0, anc, seen, 1);
  for (int i = 0; i < n; i++) CHECK(seen[i] == 1, "prim %d seen %d times\n", i, seen[i]);
  printf("nodes %zu wide_depth %d binary_depth %d fails %d\n", b.nodes.size(), b.wide_depth, b.binary_depth, fails);
  return fails ? 1 : 0;
}
