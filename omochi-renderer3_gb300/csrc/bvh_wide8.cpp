// bvh_wide8.cpp -- the 8-wide tree of the 8-wide traversal variant, made from
// a built 4-wide FP32-box tree (host or device build alike).
//
// Each 8-wide node starts from a 4-wide node's children and repeatedly
// replaces its internal child of largest surface area by that child's own
// children while the node keeps at most 8; the other internal children
// become 8-wide nodes in turn.  Child boxes are copied bit for bit from the
// 4-wide nodes (already widened for a conservative FP32 slab test), so every
// ray enters the same leaves and finds the same closest hit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "bvh_build.h"
#include "or3_common.h"

namespace or3 {
namespace {

struct Slot {
  float lo[3], hi[3];
  bool internal;
  uint32_t ref;   // 4-wide node index (internal) or first record (leaf)
  uint8_t count;  // leaf: ntri | nsph << 4
};

void slots_of(const std::vector<WideNodeF> &n4, uint32_t i, std::vector<Slot> &out) {
  const WideNodeF &n = n4[i];
  for (int c = 0; c < 4; c++) {
    const bool internal = (n.imask >> c) & 1u;
    if (!internal && n.count[c] == 0) continue;  // empty slot
    Slot s;
    for (int a = 0; a < 3; a++) {
      s.lo[a] = n.b[2 * a][c];
      s.hi[a] = n.b[2 * a + 1][c];
    }
    s.internal = internal;
    s.ref = n.child[c];
    s.count = n.count[c];
    out.push_back(s);
  }
}

float area(const Slot &s) {
  const float dx = s.hi[0] - s.lo[0], dy = s.hi[1] - s.lo[1], dz = s.hi[2] - s.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

struct Builder {
  const std::vector<WideNodeF> &n4;
  std::vector<WideNode8F> &out;
  int max_push = 0;

  // Emits the 8-wide node for 4-wide node i (pre-order); returns its index.
  uint32_t emit(uint32_t i, int pushes_above) {
    std::vector<Slot> slots;
    slots_of(n4, i, slots);
    for (;;) {
      int best = -1;
      float best_area = -1.f;
      for (size_t k = 0; k < slots.size(); k++) {
        if (!slots[k].internal) continue;
        std::vector<Slot> sub;
        slots_of(n4, slots[k].ref, sub);
        if (slots.size() - 1 + sub.size() > 8) continue;
        const float a = area(slots[k]);
        if (a > best_area) {
          best_area = a;
          best = (int)k;
        }
      }
      if (best < 0) break;
      std::vector<Slot> sub;
      slots_of(n4, slots[best].ref, sub);
      slots.erase(slots.begin() + best);
      slots.insert(slots.begin() + best, sub.begin(), sub.end());
    }
    const uint32_t me = (uint32_t)out.size();
    out.emplace_back();
    {
      WideNode8F &n = out[me];
      std::memset(&n, 0, sizeof(n));
      for (int p = 0; p < 6; p++)
        for (int c = 0; c < 8; c++) n.b[p][c] = (p & 1) ? -INFINITY : INFINITY;  // empty slots are never hit
    }
    // a ray can push every sibling but one on each level
    const int pushes = pushes_above + std::max<int>((int)slots.size() - 1, 0);
    max_push = std::max(max_push, pushes);
    for (size_t c = 0; c < slots.size(); c++) {
      const Slot &s = slots[c];
      uint32_t child = s.ref;
      if (s.internal) child = emit(s.ref, pushes);
      WideNode8F &n = out[me];  // out may have grown
      for (int a = 0; a < 3; a++) {
        n.b[2 * a][c] = s.lo[a];
        n.b[2 * a + 1][c] = s.hi[a];
      }
      n.child[c] = child;
      n.count[c] = s.internal ? 0 : s.count;
      if (s.internal) n.imask |= 1u << c;
    }
    return me;
  }
};

}  // namespace

bool make_wide8_nodes(const std::vector<WideNodeF> &n4, std::vector<WideNode8F> &out, int *max_push) {
  out.clear();
  if (n4.empty()) return true;
  out.reserve(n4.size());
  Builder b{n4, out};
  b.emit(0, 0);
  if (max_push) *max_push = b.max_push;
  return b.max_push < kStackSize8;
}

}  // namespace or3
