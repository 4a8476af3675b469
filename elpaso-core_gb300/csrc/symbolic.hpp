// Symbolic multifrontal analysis: ordering, assembly tree, front maps.
#pragma once
#include <cstdint>
#include <vector>

#include "model.hpp"

namespace elp {

struct FrontInfo {
  int32_t p = 0;          // pivots (fully summed DOFs)
  int32_t b = 0;          // border (contribution block) size
  int32_t parent = -1;    // parent front, -1 for a root
  int32_t level = 0;      // 0 = leaves; parents are processed after children
  int32_t child_slot = 0; // index among the parent's children
  int32_t idx_off = 0;    // offset into front_dofs (m = p + b entries)
  int32_t map_off = 0;    // offset into parent_map (b entries)
  int32_t piv_off = 0;    // offset of the first pivot in elimination order
  int32_t cb_off = 0;     // offset of the contribution vector (b entries) in solve buffers
  int64_t off = 0;        // offset (complex entries) of the m x m front in the arena
};

struct Symbolic {
  std::vector<FrontInfo> fronts;       // postorder: children before parents
  std::vector<int32_t> front_dofs;     // per front: pivots then border (global rows)
  std::vector<int32_t> parent_map;     // per front: position of each border dof in the parent's list
  std::vector<int64_t> entry_off;      // per CSR entry: arena offset inside its owner front
  std::vector<int32_t> elim_dof;       // elimination position -> dof
  std::vector<std::vector<int32_t>> level_fronts;
  std::vector<std::vector<int32_t>> level_children;  // per level: fronts whose parent is in a later level
  int n_levels = 0;
  int max_children = 0;
  int max_front = 0;
  int64_t arena = 0;                   // sum of m^2
  int64_t cb_total = 0;                // sum of b
  double flops = 0.0;                  // real flops of one complex factorisation
  double gemm_flops = 0.0;             // of which trailing (Schur) updates
  double factor_bytes = 0.0;           // factor bytes read per forward + backward sweep (FP32)
};

// Geometric nested dissection on the node graph; leaf_dofs bounds leaf size.
int symbolic_analyse(const Model& m, Symbolic& s, int leaf_dofs);

}  // namespace elp
