// bvh_build.h — host construction of the device BVH.
#pragma once

#include <stdint.h>

#include <vector>

#include "gpu_scene.h"

namespace rg {

struct BvhBuildResult {
  std::vector<BvhNode2> nodes;   // node 0 is the root (empty when there are no primitives)
  std::vector<uint32_t> order;   // order[i] = input primitive stored at position i
  int max_depth = 0;
};

// Binned SAH (16 bins over centroid bounds on each axis, cost N_L*A_L +
// N_R*A_R), leaves of at most `max_leaf` primitives. Below depth
// `sah_depth_limit` the split switches to the centroid median of the widest
// axis, which bounds the depth by sah_depth_limit + log2(n).
// `lo`/`hi` are n x 3 primitive bounds.
BvhBuildResult build_bvh(const float* lo, const float* hi, uint32_t n, int max_leaf = 4, int bins = 16,
                         int sah_depth_limit = 40);

}  // namespace rg
