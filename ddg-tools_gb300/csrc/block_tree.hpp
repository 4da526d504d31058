// Block cluster tree structure (host C++): the admissible (far) and inadmissible (near) blocks
// of a BVH, grouped by row node, as BlockTree::build_impl classifies them
// (RS/src/spatial/block_tree.rs:159-247): level by level from (root, root); a pair of distinct
// nodes is far when separated (max(r_a, r_b)^2 <= chi^2 d_box^2, d_box > 0;
// RS/src/metric/hierarchical.rs:116-123), near when both are leaves or |a||b| <= leaf_pairs,
// else both non-leaf sides are split. classify_blocks_device (block_tree_gpu.cu) runs the
// classification on the device, in the same order as the crate's sequential pass.
#pragma once
#include <cstdint>
#include <vector>

#include "common.hpp"
#include "host_tree.hpp"

namespace rsg {

// The blocks stay on the device, where the products use them; the host keeps their counts
// and copies the lists only on request (download).
struct Blocks {
  DevBuf<uint32_t> far_ptr, far_col;    // CSR by row node (stable: level order)
  DevBuf<uint32_t> near_ptr, near_col;  // CSR by row node
  size_t n_far = 0, n_near = 0;
  uint64_t near_entries = 0;            // off-diagonal element pairs of the near blocks
  uint64_t far_pairs = 0;               // element pairs covered by far blocks
  size_t depth = 0;
  void download(std::vector<uint32_t> &fp, std::vector<uint32_t> &fc, std::vector<uint32_t> &np,
                std::vector<uint32_t> &nc) const;
};

// Classifies on a stream of its own and returns when the blocks are on the device.
Blocks classify_blocks_device(const Tree &T, double chi, size_t leaf_pairs);

}  // namespace rsg
