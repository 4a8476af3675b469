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
  int64_t off = 0;        // offset (complex entries) of the full m x m front in the front pool
  int64_t off_full = 0;   // its offset when every front is kept whole (sum of the earlier m^2)
  int64_t fac_off = 0;    // offset of its factors in the factor store: the m x p panel (L11\U11
                          // and L21, column-major, ld m), then U12 (p x b, column-major, ld p)
  int32_t start_level = 0;  // first level the full front is alive (its first child's, or its own)
};

struct Symbolic {
  std::vector<FrontInfo> fronts;       // postorder: children before parents
  std::vector<int32_t> front_dofs;     // per front: pivots then border (global rows)
  std::vector<int32_t> parent_map;     // per front: position of each border dof in the parent's list
  std::vector<int64_t> entry_local;    // per CSR entry: offset inside its owner front (column-major)
  std::vector<int32_t> entry_owner;    // per CSR entry: the front that owns it
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
  int64_t factor_stored = 0;           // sum of p^2 + 2 p b: the L and U parts of every front
  int64_t pool_peak = 0;               // most m^2 entries of full fronts alive at once when levels
                                       // run in order (a front lives from its first child's level
                                       // to its own)
  int64_t pool = 0;                    // entries of the front pool (>= pool_peak: first-fit offsets)
  std::vector<std::vector<int32_t>> level_new;  // per level: fronts whose full front starts there
  std::vector<int32_t> scatter_order;  // CSR entries grouped by the start level of their owner front
  std::vector<int64_t> level_entry_start;  // per level + 1: range of scatter_order
  std::vector<int32_t> entry_row;      // per CSR entry: its row
};

// Geometric nested dissection on the node graph; leaf_dofs bounds leaf size.
int symbolic_analyse(const Model& m, Symbolic& s, int leaf_dofs);

}  // namespace elp
