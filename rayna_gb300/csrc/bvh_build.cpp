// bvh_build.cpp — binned-SAH builder producing 64-byte node pairs.
//
// The reference builds an exhaustive-SAH tree with up to four children per
// node (shared/generic_bvh.rs:97-290), which is O(n^2) per node and does not
// finish for meshes of a million triangles. The device tree is binary
// (one 64-byte node holds both child boxes, so one vectorised fetch serves a
// traversal step) and built with 16-bin SAH. Traversal results do not depend
// on the tree shape except for exact-distance ties.
#include "bvh_build.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace rg {

namespace {

struct Box {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const float* l, const float* h) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], l[a]); hi[a] = std::max(hi[a], h[a]); }
  }
  void grow(const Box& b) { grow(b.lo, b.hi); }
  double area() const {
    if (lo[0] > hi[0]) return 0.0;
    double x = (double)hi[0] - lo[0], y = (double)hi[1] - lo[1], z = (double)hi[2] - lo[2];
    return 2.0 * (x * y + y * z + z * x);
  }
};

struct ChildRef {
  Box box;
  int index = -1;
  int count = 0;  // > 0: leaf
};

class Builder {
 public:
  Builder(const float* lo, const float* hi, uint32_t n, int max_leaf, int bins, int sah_depth)
      : lo_(lo), hi_(hi), n_(n), max_leaf_(max_leaf), bins_(bins), sah_depth_(sah_depth) {
    cent_.resize(3ull * n);
    idx_.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
      idx_[i] = i;
      for (int a = 0; a < 3; ++a) cent_[3ull * i + a] = 0.5f * (lo[3ull * i + a] + hi[3ull * i + a]);
    }
  }

  BvhBuildResult run() {
    BvhBuildResult r;
    if (n_ == 0) return r;
    if ((int)n_ <= max_leaf_) {
      nodes_.push_back(BvhNode2{});
      ChildRef leaf = leaf_ref(0, n_);
      set_node(0, leaf, ChildRef{});
    } else {
      make(0, n_, 0);
    }
    r.nodes = std::move(nodes_);
    r.order = std::move(idx_);
    r.max_depth = max_depth_;
    return r;
  }

 private:
  const float *lo_, *hi_;
  uint32_t n_;
  int max_leaf_, bins_, sah_depth_;
  std::vector<float> cent_;
  std::vector<uint32_t> idx_;
  std::vector<BvhNode2> nodes_;
  int max_depth_ = 0;

  float cent(uint32_t i, int a) const { return cent_[3ull * i + a]; }

  Box bounds(uint32_t b, uint32_t e) const {
    Box bx;
    for (uint32_t i = b; i < e; ++i) bx.grow(lo_ + 3ull * idx_[i], hi_ + 3ull * idx_[i]);
    return bx;
  }

  ChildRef leaf_ref(uint32_t b, uint32_t e) const {
    ChildRef c;
    c.box = bounds(b, e);
    c.index = (int)b;
    c.count = (int)(e - b);
    return c;
  }

  static void put_child(BvhNode2& nd, int slot, const ChildRef& c) {
    float lx = c.box.lo[0], hx = c.box.hi[0], ly = c.box.lo[1], hy = c.box.hi[1], lz = c.box.lo[2], hz = c.box.hi[2];
    if (c.index < 0) {  // absent child (only beside a root leaf): skipped by its index
      lx = ly = lz = 0.0f;
      hx = hy = hz = 0.0f;
    }
    if (slot == 0) {
      nd.xs.x = lx; nd.xs.y = hx; nd.ys.x = ly; nd.ys.y = hy; nd.zs.x = lz; nd.zs.y = hz;
      nd.meta.x = c.index; nd.meta.z = c.count;
    } else {
      nd.xs.z = lx; nd.xs.w = hx; nd.ys.z = ly; nd.ys.w = hy; nd.zs.z = lz; nd.zs.w = hz;
      nd.meta.y = c.index; nd.meta.w = c.count;
    }
  }

  void set_node(int node, const ChildRef& c0, const ChildRef& c1) {
    put_child(nodes_[node], 0, c0);
    put_child(nodes_[node], 1, c1);
  }

  // Returns the split position in [b, e) after partitioning idx_.
  uint32_t split(uint32_t b, uint32_t e, int depth) {
    const uint32_t n = e - b;
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = b; i < e; ++i)
      for (int a = 0; a < 3; ++a) { cmin[a] = std::min(cmin[a], cent(idx_[i], a)); cmax[a] = std::max(cmax[a], cent(idx_[i], a)); }
    int wide = 0;
    for (int a = 1; a < 3; ++a) if (cmax[a] - cmin[a] > cmax[wide] - cmin[wide]) wide = a;
    auto median = [&](int a) {
      uint32_t mid = b + n / 2;
      std::nth_element(idx_.begin() + b, idx_.begin() + mid, idx_.begin() + e,
                       [&](uint32_t x, uint32_t y) { return cent(x, a) < cent(y, a); });
      return mid;
    };
    if (!(cmax[wide] > cmin[wide])) return b + n / 2;  // all centroids coincide
    if (depth >= sah_depth_) return median(wide);
    const int B = bins_;
    double best = INFINITY;
    int best_axis = -1, best_bin = -1;
    std::vector<Box> bin(B);
    std::vector<uint32_t> cnt(B);
    std::vector<double> la(B), ra(B);
    std::vector<uint32_t> lc(B), rc(B);
    for (int a = 0; a < 3; ++a) {
      float ext = cmax[a] - cmin[a];
      if (!(ext > 0.0f)) continue;
      float scale = (float)B / ext;
      std::fill(bin.begin(), bin.end(), Box{});
      std::fill(cnt.begin(), cnt.end(), 0u);
      for (uint32_t i = b; i < e; ++i) {
        uint32_t p = idx_[i];
        int k = std::min(B - 1, (int)((cent(p, a) - cmin[a]) * scale));
        bin[k].grow(lo_ + 3ull * p, hi_ + 3ull * p);
        ++cnt[k];
      }
      Box acc;
      uint32_t c = 0;
      for (int k = 0; k < B; ++k) { acc.grow(bin[k]); c += cnt[k]; la[k] = acc.area(); lc[k] = c; }
      acc = Box{};
      c = 0;
      for (int k = B - 1; k >= 0; --k) { acc.grow(bin[k]); c += cnt[k]; ra[k] = acc.area(); rc[k] = c; }
      for (int k = 0; k + 1 < B; ++k) {
        if (lc[k] == 0 || rc[k + 1] == 0) continue;
        double cost = (double)lc[k] * la[k] + (double)rc[k + 1] * ra[k + 1];
        if (cost < best) { best = cost; best_axis = a; best_bin = k; }
      }
    }
    if (best_axis < 0) return median(wide);
    float ext = cmax[best_axis] - cmin[best_axis];
    float scale = (float)B / ext;
    float cm = cmin[best_axis];
    auto it = std::partition(idx_.begin() + b, idx_.begin() + e, [&](uint32_t p) {
      return std::min(B - 1, (int)((cent(p, best_axis) - cm) * scale)) <= best_bin;
    });
    uint32_t mid = (uint32_t)(it - idx_.begin());
    if (mid == b || mid == e) return median(wide);
    return mid;
  }

  ChildRef make(uint32_t b, uint32_t e, int depth) {
    max_depth_ = std::max(max_depth_, depth);
    if ((int)(e - b) <= max_leaf_) return leaf_ref(b, e);
    int me = (int)nodes_.size();
    nodes_.push_back(BvhNode2{});
    uint32_t mid = split(b, e, depth);
    ChildRef l = make(b, mid, depth + 1);
    ChildRef r = make(mid, e, depth + 1);
    set_node(me, l, r);
    ChildRef self;
    self.box = l.box;
    self.box.grow(r.box);
    self.index = me;
    self.count = 0;
    return self;
  }
};

}  // namespace

BvhBuildResult build_bvh(const float* lo, const float* hi, uint32_t n, int max_leaf, int bins, int sah_depth_limit) {
  Builder b(lo, hi, n, max_leaf, bins, sah_depth_limit);
  return b.run();
}

// ---------------------------------------------------------------------------
// 8-wide collapse
// ---------------------------------------------------------------------------
namespace {

struct WRef {
  Box box;
  int index = -1;  // binary node (count == 0) or first primitive (count > 0)
  int count = 0;
};

int binary_children(const BvhNode2& n, WRef out[2]) {
  int k = 0;
  for (int c = 0; c < 2; ++c) {
    int idx = c ? n.meta.y : n.meta.x;
    if (idx < 0) continue;  // absent child beside a root leaf
    WRef r;
    r.index = idx;
    r.count = c ? n.meta.w : n.meta.z;
    r.box.lo[0] = c ? n.xs.z : n.xs.x; r.box.hi[0] = c ? n.xs.w : n.xs.y;
    r.box.lo[1] = c ? n.ys.z : n.ys.x; r.box.hi[1] = c ? n.ys.w : n.ys.y;
    r.box.lo[2] = c ? n.zs.z : n.zs.x; r.box.hi[2] = c ? n.zs.w : n.zs.y;
    out[k++] = r;
  }
  return k;
}

// Whether the real number p + q*s may lie above c (resp. below): evaluated in
// double and widened by 2^-52 relative, which covers the double rounding.
bool maybe_above(float p, int q, double s, float c) {
  double d = (double)p + q * s;
  return d + std::ldexp(std::fabs(d), -52) > (double)c;
}
bool maybe_below(float p, int q, double s, float c) {
  double d = (double)p + q * s;
  return d - std::ldexp(std::fabs(d), -52) < (double)c;
}

void set_byte(uint32_t& w, int b, uint32_t v) { w = (w & ~(0xFFu << (8 * b))) | ((v & 0xFFu) << (8 * b)); }
uint32_t* qword(uint4& q, int i) { return i == 0 ? &q.x : i == 1 ? &q.y : i == 2 ? &q.z : &q.w; }

// Quantises the children's boxes on the node's grid, axis by axis: the origin
// is the node box's lower corner and the step the smallest power of two with
// 255 steps covering the box; each child plane is rounded outward (verified in
// double), and the step doubles if a child's upper plane would pass 255.
void quantise(const Box& node, const WRef* slot_ref, const bool* used, WideNode& w, uint32_t exps[3]) {
  uint4* qs[3] = {&w.qx, &w.qy, &w.qz};
  for (int a = 0; a < 3; ++a) {
    const float p = node.lo[a];
    const double ext = (double)node.hi[a] - (double)p;
    int e = -100;
    if (ext > 0.0) {
      int ex;
      std::frexp(ext / 255.0, &ex);  // ext / 255 < 2^ex
      e = std::max(-100, std::min(127, ex));
    }
    uint8_t qlo[8], qhi[8];
    for (;; ++e) {
      const double s = std::ldexp(1.0, e);
      bool ok = true;
      for (int k = 0; k < 8 && ok; ++k) {
        if (!used[k]) { qlo[k] = 0; qhi[k] = 0; continue; }
        const float lo = slot_ref[k].box.lo[a], hi = slot_ref[k].box.hi[a];
        double fl = std::floor(((double)lo - p) / s);
        int ql = (int)std::max(0.0, std::min(255.0, fl));
        while (ql > 0 && maybe_above(p, ql, s, lo)) --ql;
        double fh = std::ceil(((double)hi - p) / s);
        int qh = (int)std::max((double)ql, std::min(256.0, fh));
        while (qh <= 255 && maybe_below(p, qh, s, hi)) ++qh;
        if (qh > 255) ok = false;
        qlo[k] = (uint8_t)ql;
        qhi[k] = (uint8_t)std::min(qh, 255);
      }
      if (ok || e >= 127) break;
    }
    exps[a] = (uint32_t)(e + 127);
    uint4& q = *qs[a];
    q = uint4{0, 0, 0, 0};
    for (int k = 0; k < 8; ++k) {
      set_byte(*qword(q, k >> 2), k & 3, qlo[k]);
      set_byte(*qword(q, 2 + (k >> 2)), k & 3, qhi[k]);
    }
  }
}

}  // namespace

WideBvhResult build_wide_bvh(std::vector<BvhNode2>& bin, uint32_t n_prims) {
  WideBvhResult res;
  if (bin.empty() || n_prims == 0) return res;
  std::vector<int> new_first(n_prims, -1);  // binary leaf first position -> new position
  struct Work { int wide; int bnode; int depth; };
  std::vector<Work> work;
  res.nodes.emplace_back();
  work.push_back({0, 0, 0});
  while (!work.empty()) {
    Work wk = work.back();
    work.pop_back();
    res.max_depth = std::max(res.max_depth, wk.depth);
    // Children: open the internal child of largest area until eight.
    std::vector<WRef> ch;
    {
      WRef two[2];
      int k = binary_children(bin[wk.bnode], two);
      for (int i = 0; i < k; ++i) ch.push_back(two[i]);
    }
    while (ch.size() < 8) {
      int best = -1;
      double best_area = -1.0;
      for (size_t i = 0; i < ch.size(); ++i)
        if (ch[i].count == 0 && ch[i].box.area() > best_area) { best_area = ch[i].box.area(); best = (int)i; }
      if (best < 0) break;
      WRef two[2];
      int k = binary_children(bin[ch[best].index], two);
      ch.erase(ch.begin() + best);
      for (int i = 0; i < k; ++i) ch.push_back(two[i]);
    }
    Box node;
    for (const WRef& c : ch) node.grow(c.box);
    // Slots: a ray of octant o visits internal hits in the order of
    // slot ^ o, so slot o should hold the child lying furthest upstream along
    // o's diagonal. Greedy assignment by ascending projection.
    float cn[3];
    for (int a = 0; a < 3; ++a) cn[a] = 0.5f * (node.lo[a] + node.hi[a]);
    struct Cand { double cost; int child, slot; };
    std::vector<Cand> cand;
    for (size_t c = 0; c < ch.size(); ++c) {
      double d[3];
      for (int a = 0; a < 3; ++a) d[a] = 0.5 * ((double)ch[c].box.lo[a] + ch[c].box.hi[a]) - cn[a];
      for (int sl = 0; sl < 8; ++sl) {
        double cost = 0.0;
        for (int a = 0; a < 3; ++a) cost += ((sl >> a) & 1) ? -d[a] : d[a];
        cand.push_back({cost, (int)c, sl});
      }
    }
    std::sort(cand.begin(), cand.end(), [](const Cand& x, const Cand& y) {
      if (x.cost != y.cost) return x.cost < y.cost;
      if (x.child != y.child) return x.child < y.child;
      return x.slot < y.slot;
    });
    int slot_child[8];
    bool child_done[8] = {}, used[8] = {};
    for (int k = 0; k < 8; ++k) slot_child[k] = -1;
    for (const Cand& c : cand) {
      if (child_done[c.child] || used[c.slot]) continue;
      child_done[c.child] = true;
      used[c.slot] = true;
      slot_child[c.slot] = c.child;
    }
    WRef slot_ref[8];
    for (int k = 0; k < 8; ++k)
      if (used[k]) slot_ref[k] = ch[slot_child[k]];
    // Internal children get consecutive node indices in slot order; leaf
    // primitives are appended contiguously, also in slot order.
    WideNode w{};
    uint32_t imask = 0, meta[8] = {};
    const uint32_t child_base = (uint32_t)res.nodes.size();
    const uint32_t prim_base = (uint32_t)res.perm.size();
    uint32_t n_inner = 0, offset = 0;
    std::vector<Work> kids;
    for (int k = 0; k < 8; ++k) {
      if (!used[k]) continue;
      const WRef& c = slot_ref[k];
      if (c.count == 0) {
        imask |= 1u << k;
        meta[k] = 0x20u | (24u + (uint32_t)k);
        kids.push_back({(int)(child_base + n_inner), c.index, wk.depth + 1});
        ++n_inner;
      } else {
        if (c.count > kWideMaxLeaf || offset + (uint32_t)c.count > 24u) {
          res.nodes.clear();
          res.perm.clear();
          res.max_depth = -1;  // caller keeps the binary tree only
          return res;
        }
        meta[k] = (((1u << c.count) - 1u) << 5) | offset;
        new_first[c.index] = (int)(prim_base + offset);
        for (int i = 0; i < c.count; ++i) res.perm.push_back((uint32_t)(c.index + i));
        offset += (uint32_t)c.count;
      }
    }
    res.nodes.resize(res.nodes.size() + n_inner);
    uint32_t exps[3];
    quantise(node, slot_ref, used, w, exps);
    w.w0 = float4{node.lo[0], node.lo[1], node.lo[2], 0.0f};
    uint32_t hdr = exps[0] | (exps[1] << 8) | (exps[2] << 16) | (imask << 24);
    std::memcpy(&w.w0.w, &hdr, 4);
    w.w1 = uint4{child_base, prim_base, meta[0] | meta[1] << 8 | meta[2] << 16 | meta[3] << 24,
                      meta[4] | meta[5] << 8 | meta[6] << 16 | meta[7] << 24};
    res.nodes[wk.wide] = w;
    for (auto it = kids.rbegin(); it != kids.rend(); ++it) work.push_back(*it);
  }
  // Binary leaves now index the shared new order.
  for (BvhNode2& n : bin) {
    if (n.meta.z > 0) n.meta.x = new_first[n.meta.x];
    if (n.meta.w > 0) n.meta.y = new_first[n.meta.y];
  }
  return res;
}

std::string check_wide_bvh(const std::vector<WideNode>& nodes, const float* lo, const float* hi, uint32_t n_prims) {
  if (nodes.empty()) return n_prims == 0 ? std::string() : std::string("no nodes");
  const size_t nn = nodes.size();
  char buf[256];
  auto byte_of = [](uint32_t w, int b) { return (w >> (8 * b)) & 0xFFu; };
  auto header = [](const WideNode& w) {
    uint32_t h;
    std::memcpy(&h, &w.w0.w, 4);
    return h;
  };
  // Pass 1: ranges, reachability (children after parents), primitive coverage.
  std::vector<uint8_t> node_seen(nn, 0), prim_seen(n_prims, 0);
  node_seen[0] = 1;
  for (size_t i = 0; i < nn; ++i) {
    if (!node_seen[i]) { snprintf(buf, sizeof buf, "node %zu unreachable", i); return buf; }
    const WideNode& w = nodes[i];
    const uint32_t imask = header(w) >> 24;
    uint32_t rank = 0, prim_total = 0;
    for (int k = 0; k < 8; ++k) {
      const uint32_t meta = byte_of(k < 4 ? w.w1.z : w.w1.w, k & 3);
      if ((imask >> k) & 1u) {
        if (meta != (0x38u | (uint32_t)k)) { snprintf(buf, sizeof buf, "node %zu slot %d: meta %u", i, k, meta); return buf; }
        const uint64_t c = (uint64_t)w.w1.x + rank++;
        if (c >= nn || c <= i) { snprintf(buf, sizeof buf, "node %zu slot %d: child %llu", i, k, (unsigned long long)c); return buf; }
        if (node_seen[c]) { snprintf(buf, sizeof buf, "node %llu reached twice", (unsigned long long)c); return buf; }
        node_seen[c] = 1;
      } else if (meta) {
        const uint32_t count = (uint32_t)__builtin_popcount(meta >> 5), first = meta & 31u;
        if ((meta >> 5) != ((1u << count) - 1u) || count > (uint32_t)kWideMaxLeaf || first + count > 24u) {
          snprintf(buf, sizeof buf, "node %zu slot %d: leaf meta %u", i, k, meta);
          return buf;
        }
        prim_total += count;
        for (uint32_t t = 0; t < count; ++t) {
          const uint64_t pi = (uint64_t)w.w1.y + first + t;
          if (pi >= n_prims) { snprintf(buf, sizeof buf, "node %zu slot %d: prim %llu", i, k, (unsigned long long)pi); return buf; }
          if (prim_seen[pi]) { snprintf(buf, sizeof buf, "prim %llu reached twice", (unsigned long long)pi); return buf; }
          prim_seen[pi] = 1;
        }
      }
    }
    if (prim_total > 24u) { snprintf(buf, sizeof buf, "node %zu: %u primitives", i, prim_total); return buf; }
  }
  for (uint32_t i = 0; i < n_prims; ++i)
    if (!prim_seen[i]) { snprintf(buf, sizeof buf, "prim %u not in any leaf", i); return buf; }
  // Pass 2, children before parents (reverse index order): subtree bounds, and
  // every child's real grid box containing its subtree's bounds.
  std::vector<Box> sub(nn);
  for (size_t ii = nn; ii-- > 0;) {
    const WideNode& w = nodes[ii];
    const uint32_t hdr = header(w), imask = hdr >> 24;
    const float p[3] = {w.w0.x, w.w0.y, w.w0.z};
    const uint4* q[3] = {&w.qx, &w.qy, &w.qz};
    uint32_t rank = 0;
    for (int k = 0; k < 8; ++k) {
      const uint32_t meta = byte_of(k < 4 ? w.w1.z : w.w1.w, k & 3);
      Box cb;
      if ((imask >> k) & 1u) {
        cb = sub[w.w1.x + rank++];
      } else if (meta) {
        for (uint32_t t = 0; t < (uint32_t)__builtin_popcount(meta >> 5); ++t) {
          const size_t pi = (size_t)w.w1.y + (meta & 31u) + t;
          cb.grow(lo + 3 * pi, hi + 3 * pi);
        }
      } else {
        continue;
      }
      for (int a = 0; a < 3; ++a) {
        const int e = (int)((hdr >> (8 * a)) & 0xFFu) - 127;
        const double st = std::ldexp(1.0, e);
        const uint32_t ql = byte_of(k < 4 ? q[a]->x : q[a]->y, k & 3), qh = byte_of(k < 4 ? q[a]->z : q[a]->w, k & 3);
        const bool lo_bad = ql > 0 ? maybe_above(p[a], (int)ql, st, cb.lo[a]) : (p[a] > cb.lo[a]);
        if (lo_bad || maybe_below(p[a], (int)qh, st, cb.hi[a])) {
          snprintf(buf, sizeof buf, "node %zu slot %d axis %d: grid box does not contain the child", ii, k, a);
          return buf;
        }
      }
      sub[ii].grow(cb);
    }
  }
  return std::string();
}

}  // namespace rg
