// bvh_build.cpp -- binned-SAH binary build, 4-wide collapse, 8-bit quantisation.
//
// Design (own, not the reference's):
//   * binned SAH over centroids (bins per axis configurable, 16 by default),
//     primitive cost 1 and a node cost (1 by default -- the same unit costs
//     the reference's sweep uses, T_aabb = T_tri = 1,
//     src/renderer/BVH.cpp:235-236);
//   * leaves of at most `leaf_max` primitives; a node of <= leaf_max
//     primitives becomes a leaf when that is not costlier than its best split;
//   * a hard binary depth bound (kMaxBinaryDepth) enforced by switching to
//     median splits when a subtree could not finish inside the bound, so the
//     kernels' fixed traversal stack can never overflow;
//   * collapse to 4-wide by repeatedly opening the child of largest surface
//     area, or breadth-first (grandchildren, as the reference QBVH does,
//     src/renderer/QBVH.cpp:208-272) when the greedy tree would be too deep;
//   * child boxes quantised to 8 bits per axis against the node's own box
//     with a power-of-two step, rounded outward and re-checked in float.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

namespace or3 {
namespace {

struct AABB {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const AABB &b) {
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  void grow(const float p[3]) {
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], p[a]);
      hi[a] = std::max(hi[a], p[a]);
    }
  }
  bool valid() const { return lo[0] <= hi[0]; }
  double area() const {
    if (!valid()) return 0.0;
    const double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
  }
};

struct BNode {
  AABB box;
  int left = -1, right = -1;
  uint32_t first = 0, count = 0;
  bool leaf() const { return left < 0; }
};

struct Builder {
  const std::vector<BuildPrim> &prims;
  int bins, leaf_max;
  double trav_cost = 1.0;  // SAH cost of a node relative to one primitive test
  std::vector<uint32_t> idx;
  std::vector<float> cent;  // 3 per prim
  std::vector<BNode> nodes;
  int max_depth = 0;

  Builder(const std::vector<BuildPrim> &p, int b, int l, double ct) : prims(p), bins(b), leaf_max(l), trav_cost(ct) {}

  AABB prim_box(uint32_t i) const {
    AABB b;
    for (int a = 0; a < 3; a++) {
      b.lo[a] = prims[i].lo[a];
      b.hi[a] = prims[i].hi[a];
    }
    return b;
  }

  static int ceil_log2(uint64_t v) {
    int r = 0;
    while ((uint64_t(1) << r) < v) r++;
    return r;
  }

  // Median split on the widest centroid axis; returns split position.
  uint32_t median_split(uint32_t first, uint32_t count, const AABB &cb) {
    int axis = 0;
    float best = -1.f;
    for (int a = 0; a < 3; a++)
      if (cb.hi[a] - cb.lo[a] > best) { best = cb.hi[a] - cb.lo[a]; axis = a; }
    const uint32_t mid = first + count / 2;
    std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
                     [&](uint32_t x, uint32_t y) {
                       if (cent[3 * x + axis] != cent[3 * y + axis])
                         return cent[3 * x + axis] < cent[3 * y + axis];
                       return x < y;
                     });
    return mid;
  }

  struct Task { int node; uint32_t first, count; int depth; };
  struct Scratch {
    std::vector<AABB> binBox;
    std::vector<uint32_t> binCnt;
    std::vector<double> rightArea;
    std::vector<uint32_t> rightCnt;
    explicit Scratch(int bins) : binBox(3 * bins), binCnt(3 * bins), rightArea(bins), rightCnt(bins) {}
  };

  // Builds the tree.  The top of the tree is split serially, breadth first,
  // until there are enough independent subtrees; those are then built on all
  // host threads (each into its own node array, over its own disjoint range
  // of the index array) and merged.  The tree is the same as a serial build's.
  void build() {
    const uint32_t n = (uint32_t)prims.size();
    idx.resize(n);
    cent.resize(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
      idx[i] = i;
      for (int a = 0; a < 3; a++) cent[3 * i + a] = 0.5f * (prims[i].lo[a] + prims[i].hi[a]);
    }
    nodes.reserve(2 * (size_t)n);
    nodes.push_back(BNode());
    unsigned threads = std::thread::hardware_concurrency();
    threads = std::max(1u, std::min(threads, 64u));
    host_threads = threads;  // large top nodes bin on all threads
    Scratch sc(bins);
    std::vector<Task> fifo;
    fifo.push_back({0, 0, n, 1});
    std::vector<Task> pending, kids;
    size_t head = 0;
    while (head < fifo.size() && fifo.size() - head < 4 * (size_t)threads) {
      const Task t = fifo[head++];
      if (t.count < 4096 || threads == 1) {
        pending.push_back(t);
        continue;
      }
      kids.clear();
      process(t, nodes, kids, sc, max_depth);
      for (const Task &k : kids) fifo.push_back(k);
    }
    for (; head < fifo.size(); head++) pending.push_back(fifo[head]);

    host_threads = 1;  // subtrees run one per thread
    struct Local { std::vector<BNode> nodes; int maxd = 0; };
    std::vector<Local> locals(pending.size());
    std::atomic<size_t> next(0);
    auto worker = [&]() {
      Scratch wsc(bins);
      std::vector<Task> st;
      for (size_t i; (i = next.fetch_add(1)) < pending.size();) {
        Local &L = locals[i];
        L.nodes.push_back(BNode());
        st.clear();
        st.push_back({0, pending[i].first, pending[i].count, pending[i].depth});
        while (!st.empty()) {
          const Task t = st.back();
          st.pop_back();
          process(t, L.nodes, st, wsc, L.maxd);
        }
      }
    };
    std::vector<std::thread> pool;
    const unsigned nt = (unsigned)std::min<size_t>(threads, pending.size());
    for (unsigned k = 1; k < nt; k++) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();

    for (size_t i = 0; i < pending.size(); i++) {
      Local &L = locals[i];
      const int slot = pending[i].node;
      const int base = (int)nodes.size() - 1;  // local index k >= 1 -> base + k
      auto remap = [&](int k) { return k == 0 ? slot : base + k; };
      for (size_t k = 1; k < L.nodes.size(); k++) {
        BNode b = L.nodes[k];
        if (!b.leaf()) {
          b.left = remap(b.left);
          b.right = remap(b.right);
        }
        nodes.push_back(b);
      }
      BNode r = L.nodes[0];
      if (!r.leaf()) {
        r.left = remap(r.left);
        r.right = remap(r.right);
      }
      nodes[slot] = r;
      max_depth = std::max(max_depth, L.maxd);
    }
  }

  // Node bounds and centroid bounds of idx[first, first+count); large ranges
  // are split over host threads.
  void bounds(uint32_t first, uint32_t count, AABB &box, AABB &cb, unsigned threads) const {
    const unsigned nt = count > (1u << 13) ? threads : 1u;
    if (nt == 1) {
      for (uint32_t i = first; i < first + count; i++) {
        box.grow(prim_box(idx[i]));
        cb.grow(&cent[3 * idx[i]]);
      }
      return;
    }
    std::vector<AABB> b(nt), c(nt);
    auto run = [&](unsigned k) {
      const uint32_t s = first + (uint32_t)((uint64_t)count * k / nt), e = first + (uint32_t)((uint64_t)count * (k + 1) / nt);
      for (uint32_t i = s; i < e; i++) {
        b[k].grow(prim_box(idx[i]));
        c[k].grow(&cent[3 * idx[i]]);
      }
    };
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; k++) pool.emplace_back(run, k);
    run(0);
    for (auto &th : pool) th.join();
    for (unsigned k = 0; k < nt; k++) {
      box.grow(b[k]);
      cb.grow(c[k]);
    }
  }

  // Per-axis bin boxes and counts of idx[first, first+count) (all three axes
  // in one pass; large ranges over host threads).
  void bin_all(uint32_t first, uint32_t count, const AABB &cb, AABB *binBox, uint32_t *binCnt,
               unsigned threads) const {
    const unsigned nt = count > (1u << 13) ? threads : 1u;
    float scale[3];
    for (int a = 0; a < 3; a++) {
      const float ext = cb.hi[a] - cb.lo[a];
      scale[a] = ext > 0.f ? (float)bins / ext : 0.f;
    }
    auto bin_range = [&](uint32_t s, uint32_t e, AABB *bb, uint32_t *bc) {
      for (uint32_t i = s; i < e; i++) {
        const uint32_t p = idx[i];
        const AABB pbox = prim_box(p);
        for (int a = 0; a < 3; a++) {
          int bi = (int)((cent[3 * p + a] - cb.lo[a]) * scale[a]);
          bi = std::min(std::max(bi, 0), bins - 1);
          bb[a * bins + bi].grow(pbox);
          bc[a * bins + bi]++;
        }
      }
    };
    if (nt == 1) {
      for (int j = 0; j < 3 * bins; j++) {
        binBox[j] = AABB();
        binCnt[j] = 0;
      }
      bin_range(first, first + count, binBox, binCnt);
      return;
    }
    std::vector<AABB> pb((size_t)nt * 3 * bins);
    std::vector<uint32_t> pc((size_t)nt * 3 * bins, 0);
    auto run = [&](unsigned k) {
      const uint32_t s = first + (uint32_t)((uint64_t)count * k / nt), e = first + (uint32_t)((uint64_t)count * (k + 1) / nt);
      AABB *bb = &pb[(size_t)k * 3 * bins];
      uint32_t *bc = &pc[(size_t)k * 3 * bins];
      bin_range(s, e, bb, bc);
    };
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; k++) pool.emplace_back(run, k);
    run(0);
    for (auto &th : pool) th.join();
    for (int j = 0; j < 3 * bins; j++) {
      binBox[j] = AABB();
      binCnt[j] = 0;
      for (unsigned k = 0; k < nt; k++) {
        binBox[j].grow(pb[(size_t)k * 3 * bins + j]);
        binCnt[j] += pc[(size_t)k * 3 * bins + j];
      }
    }
  }

  unsigned host_threads = 1;

  // One node: bounds, then leaf or split; children are allocated in `nodes`
  // and pushed on `stack`.
  void process(const Task &t, std::vector<BNode> &nodes, std::vector<Task> &stack, Scratch &sc, int &maxd) {
    std::vector<AABB> &binBox = sc.binBox;
    std::vector<uint32_t> &binCnt = sc.binCnt;
    std::vector<double> &rightArea = sc.rightArea;
    std::vector<uint32_t> &rightCnt = sc.rightCnt;
    {
      maxd = std::max(maxd, t.depth);
      AABB box, cb;
      bounds(t.first, t.count, box, cb, host_threads);
      BNode &nd = nodes[t.node];
      nd.box = box;
      nd.first = t.first;
      nd.count = t.count;
      if (t.count <= 1) return;

      // Depth guard: finishing with median splits needs ceil(log2(count/leaf_max)) levels.
      const int need = ceil_log2((t.count + leaf_max - 1) / leaf_max);
      uint32_t split = 0;
      bool have = false;
      if (t.depth + need >= kMaxBinaryDepth) {
        if (t.count <= (uint32_t)leaf_max) return;
        split = median_split(t.first, t.count, cb);
        have = true;
      } else {
        // binned SAH
        const double parentArea = box.area();
        double bestCost = DBL_MAX;
        int bestAxis = -1, bestBin = -1;
        bin_all(t.first, t.count, cb, binBox.data(), binCnt.data(), host_threads);
        for (int a = 0; a < 3; a++) {
          const float ext = cb.hi[a] - cb.lo[a];
          if (!(ext > 0.f)) continue;
          AABB *bb = &binBox[a * bins];
          uint32_t *bc = &binCnt[a * bins];
          AABB acc;
          uint32_t cnt = 0;
          for (int b = bins - 1; b > 0; b--) {
            acc.grow(bb[b]);
            cnt += bc[b];
            rightArea[b] = acc.area();
            rightCnt[b] = cnt;
          }
          acc = AABB();
          cnt = 0;
          for (int b = 0; b < bins - 1; b++) {
            acc.grow(bb[b]);
            cnt += bc[b];
            if (cnt == 0 || rightCnt[b + 1] == 0) continue;
            const double cost = trav_cost + (acc.area() * cnt + rightArea[b + 1] * rightCnt[b + 1]) /
                                          std::max(parentArea, 1e-30);
            if (cost < bestCost) { bestCost = cost; bestAxis = a; bestBin = b; }
          }
        }
        if (t.count <= (uint32_t)leaf_max && (bestAxis < 0 || (double)t.count <= bestCost)) return;
        if (bestAxis < 0) {
          split = median_split(t.first, t.count, cb);
        } else {
          const float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
          const float scale = (float)bins / ext;
          auto mid = std::partition(idx.begin() + t.first, idx.begin() + t.first + t.count,
                                    [&](uint32_t p) {
                                      int b = (int)((cent[3 * p + bestAxis] - cb.lo[bestAxis]) * scale);
                                      b = std::min(std::max(b, 0), bins - 1);
                                      return b <= bestBin;
                                    });
          split = (uint32_t)(mid - idx.begin());
          if (split == t.first || split == t.first + t.count) split = median_split(t.first, t.count, cb);
        }
        have = true;
      }
      if (!have) return;
      const int l = (int)nodes.size();
      nodes.push_back(BNode());
      nodes.push_back(BNode());
      nodes[t.node].left = l;
      nodes[t.node].right = l + 1;
      stack.push_back({l + 1, split, t.first + t.count - split, t.depth + 1});
      stack.push_back({l, t.first, split - t.first, t.depth + 1});
    }
  }
};

// Node quantisation: step 2^e per axis with 255 steps covering the node box.
void quantise(WideNode &w, const AABB &nodeBox, const AABB *childBox, int nchild) {
  for (int a = 0; a < 3; a++) {
    const float org = nodeBox.lo[a];
    w.origin[a] = org;
    const double ext = (double)nodeBox.hi[a] - (double)org;
    int e = -126;
    if (ext > 0) {
      e = (int)std::ceil(std::log2(ext / 255.0));
      e = std::max(e, -126);
    }
    for (;;) {
      const float step = std::ldexp(1.0f, e);
      bool ok = (org + 255.0f * step >= nodeBox.hi[a]);
      for (int c = 0; c < nchild && ok; c++) {
        double ql = std::floor(((double)childBox[c].lo[a] - org) / step);
        double qh = std::ceil(((double)childBox[c].hi[a] - org) / step);
        ql = std::max(0.0, std::min(255.0, ql));
        qh = std::max(0.0, std::min(255.0, qh));
        while (ql > 0 && org + (float)ql * step > childBox[c].lo[a]) ql -= 1;
        while (qh < 255 && org + (float)qh * step < childBox[c].hi[a]) qh += 1;
        if (org + (float)ql * step > childBox[c].lo[a] || org + (float)qh * step < childBox[c].hi[a]) {
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

// Child boxes of one wide node in WideNodeF::b order (empty slots +inf / -inf).
void set_boxes(float *dst, const AABB &parent, const AABB *boxes, int nchild) {
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 4; c++) {
      float lo = INFINITY, hi = -INFINITY;
      if (c < nchild) fnode_slab(parent.lo[a], parent.hi[a], boxes[c].lo[a], boxes[c].hi[a], &lo, &hi);
      dst[(2 * a) * 4 + c] = lo;
      dst[(2 * a + 1) * 4 + c] = hi;
    }
}

struct Collapser {
  const std::vector<BNode> &bn;
  std::vector<WideNode> &out;
  std::vector<float> &fbox;
  bool breadth_first;
  int max_depth = 0;

  Collapser(const std::vector<BNode> &b, std::vector<WideNode> &o, std::vector<float> &f, bool bf)
      : bn(b), out(o), fbox(f), breadth_first(bf) {}

  void gather(int root, std::vector<int> &kids) const {
    kids.clear();
    if (bn[root].leaf()) { kids.push_back(root); return; }
    kids.push_back(bn[root].left);
    kids.push_back(bn[root].right);
    if (breadth_first) {
      std::vector<int> next;
      for (int k : kids) {
        if (bn[k].leaf()) next.push_back(k);
        else { next.push_back(bn[k].left); next.push_back(bn[k].right); }
      }
      kids = next;
      return;
    }
    while (kids.size() < 4) {
      int best = -1;
      double bestA = -1;
      for (size_t i = 0; i < kids.size(); i++) {
        if (bn[kids[i]].leaf()) continue;
        const double a = bn[kids[i]].box.area();
        if (a > bestA) { bestA = a; best = (int)i; }
      }
      if (best < 0) break;
      const int k = kids[best];
      kids[best] = bn[k].left;
      kids.push_back(bn[k].right);
    }
  }

  // Emits the wide nodes breadth first from binary node 0 into slot 0, so the
  // top levels are contiguous (the kernels stage the first nodes in shared
  // memory).
  void emit_all() {
    // structure (serial, cheap): children and indices, breadth first
    struct Item { int root; uint32_t slot; int depth; int kids[4]; int nkids; };
    std::vector<Item> fifo;
    fifo.push_back({0, 0, 1, {0, 0, 0, 0}, 0});
    std::vector<int> kids;
    for (size_t head = 0; head < fifo.size(); head++) {
      Item &it = fifo[head];
      max_depth = std::max(max_depth, it.depth);
      gather(it.root, kids);
      it.nkids = (int)kids.size();
      const uint32_t slot = it.slot;
      const int depth = it.depth;
      WideNode w;
      std::memset(&w, 0, sizeof(w));
      for (size_t i = 0; i < kids.size(); i++) {
        fifo[head].kids[i] = kids[i];
        const BNode &k = bn[kids[i]];
        if (k.leaf()) {
          w.child[i] = k.first;
          w.count[i] = (uint8_t)k.count;  // total for now; split by kind below
        } else {
          const uint32_t c = (uint32_t)out.size();
          out.push_back(WideNode());
          w.child[i] = c;
          w.imask |= (uint8_t)(1u << i);
          fifo.push_back({kids[i], c, depth + 1, {0, 0, 0, 0}, 0});
        }
      }
      out[slot] = w;
    }
    fbox.assign(24 * out.size(), 0.f);
    // quantised boxes (independent per node): all host threads
    unsigned threads = std::thread::hardware_concurrency();
    threads = std::max(1u, std::min(threads, 64u));
    if (fifo.size() < 4096) threads = 1;
    std::atomic<size_t> next(0);
    auto worker = [&]() {
      for (size_t b; (b = next.fetch_add(1024)) < fifo.size();) {
        const size_t e = std::min(fifo.size(), b + 1024);
        for (size_t i = b; i < e; i++) {
          const Item &it = fifo[i];
          AABB boxes[4];
          for (int k = 0; k < it.nkids; k++) boxes[k] = bn[it.kids[k]].box;
          quantise(out[it.slot], bn[it.root].box, boxes, it.nkids);
          set_boxes(&fbox[24 * (size_t)it.slot], bn[it.root].box, boxes, it.nkids);
        }
      }
    };
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < threads; k++) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();
  }
};

}  // namespace

void make_float_nodes(const WideBVH &bvh, std::vector<WideNodeF> &out) {
  out.resize(bvh.nodes.size());
  for (size_t i = 0; i < bvh.nodes.size(); i++) {
    const WideNode &w = bvh.nodes[i];
    WideNodeF &f = out[i];
    std::memset(&f, 0, sizeof(f));
    std::memcpy(f.b, &bvh.boxes[24 * i], 24 * sizeof(float));
    for (int c = 0; c < 4; c++) {
      f.child[c] = w.child[c];
      f.count[c] = w.count[c];
    }
    f.imask = w.imask;
  }
}

void decode_child_box(const WideNode &n, int c, float lo[3], float hi[3]) {
  for (int a = 0; a < 3; a++) {
    const float step = std::ldexp(1.0f, (int)n.exp[a] - 127);
    lo[a] = n.origin[a] + (float)n.lo[a][c] * step;
    hi[a] = n.origin[a] + (float)n.hi[a][c] * step;
  }
}

bool build_wide_bvh(const std::vector<BuildPrim> &prims, int bins, int leaf_max, WideBVH &out,
                    std::string *err, double trav_cost) {
  out = WideBVH();
  if (bins < 2 || bins > 256 || leaf_max < 1 || leaf_max > 8 || !(trav_cost > 0)) {
    if (err) *err = "build_wide_bvh: bins must be in [2,256], leaf_max in [1,8], traversal cost > 0";
    return false;
  }
  for (const BuildPrim &p : prims)
    for (int a = 0; a < 3; a++)
      if (!(p.lo[a] <= p.hi[a]) || !std::isfinite(p.lo[a]) || !std::isfinite(p.hi[a])) {
        if (err) *err = "build_wide_bvh: primitive with invalid or non-finite bounds";
        return false;
      }
  if (prims.empty()) return true;

  Builder b(prims, bins, leaf_max, trav_cost);
  b.build();
  out.binary_depth = b.max_depth;
  out.binary_nodes = b.nodes.size();

  // A root that is itself a leaf still gets a wide node with one leaf child.
  std::vector<BNode> bn = b.nodes;
  if (bn[0].leaf()) {
    BNode top = bn[0];
    BNode leaf = bn[0];
    top.left = 1;
    top.right = -1;
    bn.clear();
    bn.push_back(top);
    bn.push_back(leaf);
  }

  for (int pass = 0; pass < 2; pass++) {
    out.nodes.clear();
    out.nodes.push_back(WideNode());
    Collapser c(bn, out.nodes, out.boxes, pass == 1);
    if (bn[0].right < 0) {
      // single leaf child under the root
      WideNode w;
      std::memset(&w, 0, sizeof(w));
      AABB box = bn[1].box;
      quantise(w, bn[0].box, &box, 1);
      w.child[0] = bn[1].first;
      w.count[0] = (uint8_t)bn[1].count;
      out.nodes[0] = w;
      out.boxes.assign(24, 0.f);
      set_boxes(out.boxes.data(), bn[0].box, &box, 1);
      c.max_depth = 1;
    } else {
      c.emit_all();
    }
    out.wide_depth = c.max_depth;
    if (out.wide_depth <= kMaxBinaryDepth / 2) break;
  }

  // Leaf order: the index array is already leaf-contiguous; put triangles
  // before spheres inside each leaf and encode the slot count as ntri | nsph << 4.
  out.order = b.idx;
  for (WideNode &w : out.nodes) {
    for (int i = 0; i < 4; i++) {
      if (w.imask & (1u << i)) continue;
      const uint32_t cnt = w.count[i];
      if (cnt == 0) continue;  // empty slot
      uint32_t *beg = out.order.data() + w.child[i];
      std::stable_partition(beg, beg + cnt, [&](uint32_t p) { return prims[p].kind == kPrimTriangle; });
      uint32_t ntri = 0;
      for (uint32_t k = 0; k < cnt; k++) ntri += prims[beg[k]].kind == kPrimTriangle;
      w.count[i] = (uint8_t)(ntri | ((cnt - ntri) << 4));
    }
  }
  return true;
}

}  // namespace or3
