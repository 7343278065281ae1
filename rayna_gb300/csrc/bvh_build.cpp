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

}  // namespace rg
