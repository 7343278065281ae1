// bvh_build.h — host construction of the device BVH.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "gpu_scene.h"

namespace rg {

struct BvhBuildResult {
  std::vector<BvhNode2> nodes;   // node 0 is the root (empty when there are no primitives)
  std::vector<uint32_t> order;   // order[i] = input primitive stored at position i
  int max_depth = 0;
};

// Binned SAH (`bins` bins over centroid bounds on each axis, cost N_L*A_L +
// N_R*A_R), leaves of at most `max_leaf` primitives. Below depth
// `sah_depth_limit` the split switches to the centroid median of the widest
// axis, which bounds the depth by sah_depth_limit + log2(n).
// `lo`/`hi` are n x 3 primitive bounds.
BvhBuildResult build_bvh(const float* lo, const float* hi, uint32_t n, int max_leaf = 4, int bins = 16,
                         int sah_depth_limit = 40);

struct WideBvhResult {
  std::vector<WideNode> nodes;   // node 0 is the root (empty when there are no primitives)
  std::vector<uint32_t> perm;    // perm[j] = binary-order position of the primitive now stored at j
  int max_depth = 0;
};

// Collapses a binary tree (leaves of at most kWideMaxLeaf primitives) into the
// compressed 8-wide layout. A wide node takes its binary node's two children
// and repeatedly opens the internal child of largest surface area until it
// has eight children or only leaves. The primitives of each wide node's leaf
// children are laid out contiguously; `bin` is rewritten in place so that its
// leaves index the new primitive order, which both trees then share. Child
// boxes come from the binary nodes.
WideBvhResult build_wide_bvh(std::vector<BvhNode2>& bin, uint32_t n_prims);

// Structural check of a wide tree over primitives with bounds lo/hi (n x 3,
// in the tree's primitive order): child and primitive ranges in bounds, each
// node and each primitive reached exactly once, children stored after their
// parent (so traversal cannot cycle), and every child's grid box (the real
// numbers p + q 2^e) containing the bounds of every primitive below it.
// Returns an empty string when the tree is valid, else the first violation.
std::string check_wide_bvh(const std::vector<WideNode>& nodes, const float* lo, const float* hi, uint32_t n_prims);

}  // namespace rg
