// Symbolic multifrontal analysis.
//
// The reference hands this to MUMPS (KSPPREONLY + PCLU + MUMPS,
// analysis/analysis.cpp:1071-1226): ordering, elimination tree and front
// sizes are computed inside the library. Here they are project code:
//
//  1. node graph from the CSR pattern (two nodes are adjacent when any of
//     their DOFs share an entry; this includes the FSI coupling);
//  2. geometric nested dissection: recursive median bisection along the
//     longest axis of the node coordinates; the vertex separator is the
//     boundary layer of one side (the smaller one) and becomes the parent
//     front of the two halves; subsets at or below `leaf_dofs` DOFs are
//     leaf fronts;
//  3. fronts in postorder; front s holds its pivots (the separator's DOFs)
//     followed by its border: every later-eliminated DOF adjacent to a pivot
//     or in a child's border, sorted by elimination position;
//  4. per CSR entry, the pool offset of its slot in the front that owns it
//     (the front of whichever of row/column is eliminated first);
//  5. per border DOF, its position in the parent front (extend-add map).
#include "symbolic.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>

namespace elp {

namespace {

struct NodeGraph {
  std::vector<int64_t> ptr;
  std::vector<int32_t> adj;
};

struct Builder {
  const Model& m;
  const NodeGraph& g;
  std::vector<int32_t> first_row, ndof;
  std::vector<int32_t> mark;    // per node: stamp * 4 + side
  int32_t stamp = 0;
  int leaf_dofs;
  std::vector<std::vector<int32_t>> tnodes;     // tree node -> graph nodes (pivots)
  std::vector<std::vector<int32_t>> tchildren;  // tree node -> children

  Builder(const Model& mm, const NodeGraph& gg, int leaf) : m(mm), g(gg), leaf_dofs(leaf) {}

  int64_t dofs_of(const std::vector<int32_t>& set) const {
    int64_t s = 0;
    for (int32_t v : set) s += ndof[v];
    return s;
  }

  int make_node(std::vector<int32_t>&& nodes, std::vector<int32_t>&& children) {
    tnodes.push_back(std::move(nodes));
    tchildren.push_back(std::move(children));
    return (int)tnodes.size() - 1;
  }

  // returns the roots of the subtree built over `set`
  std::vector<int32_t> nd(std::vector<int32_t>& set) {
    std::vector<int32_t> roots;
    if (set.empty()) return roots;
    if (dofs_of(set) <= leaf_dofs || set.size() <= 2) {
      roots.push_back(make_node(std::move(set), {}));
      return roots;
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int32_t v : set)
      for (int d = 0; d < 3; ++d) {
        double x = m.coords[3 * (size_t)v + d];
        lo[d] = std::min(lo[d], x);
        hi[d] = std::max(hi[d], x);
      }
    int axis = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[axis] - lo[axis]) axis = d;
    std::vector<int32_t> left, right;
    if (hi[axis] - lo[axis] > 0.0) {
      std::vector<double> vals(set.size());
      for (size_t i = 0; i < set.size(); ++i) vals[i] = m.coords[3 * (size_t)set[i] + axis];
      std::nth_element(vals.begin(), vals.begin() + vals.size() / 2, vals.end());
      double xm = vals[vals.size() / 2];
      for (int32_t v : set) (m.coords[3 * (size_t)v + axis] < xm ? left : right).push_back(v);
      if (left.empty() || right.empty()) {
        left.clear();
        right.clear();
        for (int32_t v : set) (m.coords[3 * (size_t)v + axis] <= xm ? left : right).push_back(v);
      }
    }
    if (left.empty() || right.empty()) {
      // coincident coordinates: split by index
      left.assign(set.begin(), set.begin() + set.size() / 2);
      right.assign(set.begin() + set.size() / 2, set.end());
    }
    ++stamp;
    for (int32_t v : left) mark[v] = stamp * 4 + 1;
    for (int32_t v : right) mark[v] = stamp * 4 + 2;
    auto boundary = [&](const std::vector<int32_t>& side, int other) {
      std::vector<int32_t> sep;
      for (int32_t v : side) {
        for (int64_t q = g.ptr[v]; q < g.ptr[v + 1]; ++q)
          if (mark[g.adj[q]] == stamp * 4 + other) { sep.push_back(v); break; }
      }
      return sep;
    };
    std::vector<int32_t> sepL = boundary(left, 2), sepR = boundary(right, 1);
    bool takeL = dofs_of(sepL) < dofs_of(sepR);
    std::vector<int32_t>& sep = takeL ? sepL : sepR;
    std::vector<int32_t>& side = takeL ? left : right;
    if (!sep.empty()) {
      ++stamp;
      for (int32_t v : sep) mark[v] = stamp * 4 + 3;
      std::vector<int32_t> rest;
      rest.reserve(side.size());
      for (int32_t v : side)
        if (mark[v] != stamp * 4 + 3) rest.push_back(v);
      side.swap(rest);
    }
    std::vector<int32_t> sep_nodes(sep.begin(), sep.end());
    std::vector<int32_t> r1 = nd(left);
    std::vector<int32_t> r2 = nd(right);
    std::vector<int32_t> children(r1);
    children.insert(children.end(), r2.begin(), r2.end());
    if (sep_nodes.empty()) return children;  // disconnected halves: a forest
    roots.push_back(make_node(std::move(sep_nodes), std::move(children)));
    return roots;
  }
};

}  // namespace

int symbolic_analyse(const Model& m, Symbolic& S, int leaf_dofs) {
  const int64_t N = m.n_nodes, n = m.n;
  // ---- per node dof range (a node's active dofs have consecutive rows)
  std::vector<int32_t> first_row(N, -1), ndof(N, 0);
  for (int64_t r = 0; r < n; ++r) {
    int32_t v = m.dof_node[r];
    if (first_row[v] < 0) first_row[v] = (int32_t)r;
    ndof[v]++;
  }
  // ---- node graph from the pattern
  NodeGraph g;
  g.ptr.assign(N + 1, 0);
  std::vector<std::vector<int32_t>> nb(N);
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t v = 0; v < N; ++v) {
    if (ndof[v] == 0) continue;
    std::vector<int32_t>& L = nb[v];
    for (int32_t r = first_row[v]; r < first_row[v] + ndof[v]; ++r)
      for (int32_t q = m.row_ptr[r]; q < m.row_ptr[r + 1]; ++q) {
        int32_t u = m.dof_node[m.col_idx[q]];
        if (u != v) L.push_back(u);
      }
    std::sort(L.begin(), L.end());
    L.erase(std::unique(L.begin(), L.end()), L.end());
  }
  for (int64_t v = 0; v < N; ++v) g.ptr[v + 1] = g.ptr[v] + (int64_t)nb[v].size();
  g.adj.resize(g.ptr[N]);
  for (int64_t v = 0; v < N; ++v) {
    std::copy(nb[v].begin(), nb[v].end(), g.adj.begin() + g.ptr[v]);
    std::vector<int32_t>().swap(nb[v]);
  }

  // ---- nested dissection, per connected component of the node graph (the
  // members of a group, disconnected bodies): each gets its own subtree, so
  // no separator front mixes unconnected parts however their coordinates lie
  Builder B(m, g, leaf_dofs);
  B.first_row = first_row;
  B.ndof = ndof;
  B.mark.assign(N, 0);
  {
    std::vector<int32_t> comp(N, -1), stack;
    int nc = 0;
    for (int64_t v0 = 0; v0 < N; ++v0) {
      if (ndof[v0] == 0 || comp[v0] >= 0) continue;
      comp[v0] = nc;
      stack.assign(1, (int32_t)v0);
      while (!stack.empty()) {
        const int32_t v = stack.back();
        stack.pop_back();
        for (int64_t q = g.ptr[v]; q < g.ptr[v + 1]; ++q)
          if (comp[g.adj[q]] < 0) { comp[g.adj[q]] = nc; stack.push_back(g.adj[q]); }
      }
      ++nc;
    }
    std::vector<std::vector<int32_t>> parts(nc);
    for (int64_t v = 0; v < N; ++v)
      if (ndof[v] > 0) parts[comp[v]].push_back((int32_t)v);
    for (auto& part : parts) B.nd(part);
  }
  const int T = (int)B.tnodes.size();

  // ---- elimination order
  std::vector<int32_t> snode(N, -1), node_rank(N, -1);
  S.elim_dof.clear();
  S.elim_dof.reserve(n);
  std::vector<int32_t> dof_pos(n, -1);
  int32_t rank = 0;
  for (int t = 0; t < T; ++t)
    for (int32_t v : B.tnodes[t]) {
      snode[v] = t;
      node_rank[v] = rank++;
      for (int32_t r = first_row[v]; r < first_row[v] + ndof[v]; ++r) {
        dof_pos[r] = (int32_t)S.elim_dof.size();
        S.elim_dof.push_back(r);
      }
    }
  if ((int64_t)S.elim_dof.size() != n) { set_error("ordering lost degrees of freedom"); return ELP_ERR_ARG; }

  // ---- parents, levels, borders
  std::vector<int32_t> parent(T, -1), level(T, 0), slot(T, 0);
  int maxc = 0;
  for (int t = 0; t < T; ++t) {
    int c = 0;
    for (int32_t ch : B.tchildren[t]) {
      parent[ch] = t;
      slot[ch] = c++;
      level[t] = std::max(level[t], level[ch] + 1);
    }
    maxc = std::max(maxc, c);
  }
  std::vector<std::vector<int32_t>> border(T);
  std::vector<int32_t> seen(N, -1);
  for (int t = 0; t < T; ++t) {
    std::vector<int32_t> cand;
    auto consider = [&](int32_t u) {
      if (snode[u] > t && seen[u] != t) { seen[u] = t; cand.push_back(u); }
    };
    for (int32_t v : B.tnodes[t])
      for (int64_t q = g.ptr[v]; q < g.ptr[v + 1]; ++q) consider(g.adj[q]);
    for (int32_t ch : B.tchildren[t]) {
      for (int32_t u : border[ch]) consider(u);
    }
    std::sort(cand.begin(), cand.end(), [&](int32_t a, int32_t b) { return node_rank[a] < node_rank[b]; });
    border[t].swap(cand);
  }

  // ---- fronts
  S.fronts.assign(T, FrontInfo());
  S.front_dofs.clear();
  int64_t arena = 0, cbt = 0;
  double flops = 0.0;
  int32_t piv = 0;
  int maxm = 0;
  for (int t = 0; t < T; ++t) {
    FrontInfo& F = S.fronts[t];
    F.parent = parent[t];
    F.level = level[t];
    F.child_slot = slot[t];
    F.idx_off = (int32_t)S.front_dofs.size();
    int p = 0, b = 0;
    for (int32_t v : B.tnodes[t])
      for (int32_t r = first_row[v]; r < first_row[v] + ndof[v]; ++r) { S.front_dofs.push_back(r); ++p; }
    for (int32_t v : border[t])
      for (int32_t r = first_row[v]; r < first_row[v] + ndof[v]; ++r) { S.front_dofs.push_back(r); ++b; }
    F.p = p;
    F.b = b;
    F.piv_off = piv;
    piv += p;
    F.off_full = arena;
    const int64_t mm = (int64_t)p + b;
    arena += mm * mm;
    F.cb_off = (int32_t)cbt;
    cbt += b;
    maxm = std::max<int>(maxm, (int)mm);
    for (int k = 0; k < p; ++k) {
      double r = (double)(mm - k - 1);
      flops += 8.0 * r * r + 8.0 * r;
    }
    // trailing updates of the blocked LU (panel width 32): rows/cols t0..m-1, depth w
    for (int k0 = 0; k0 < p; k0 += 32) {
      const int w = std::min(32, p - k0);
      const double t = (double)(mm - k0 - w);
      S.gemm_flops += 8.0 * t * t * w;
    }
    // factors read by one forward + backward sweep: L (m x p) and U12 (p x b), complex FP32
    S.factor_bytes += 8.0 * ((double)mm * p + (double)p * b);
    if (S.front_dofs.size() > (size_t)INT32_MAX) { set_error("front index lists too large"); return ELP_ERR_NOMEM; }
  }
  S.arena = arena;
  S.cb_total = cbt;
  S.flops = flops;
  S.max_front = maxm;
  S.max_children = maxc;

  // ---- extend-add maps
  std::vector<int32_t> loc(n, -1);
  S.parent_map.clear();
  for (int t = 0; t < T; ++t) S.fronts[t].map_off = 0;
  {
    // map offsets in front order
    int32_t mo = 0;
    for (int t = 0; t < T; ++t) { S.fronts[t].map_off = mo; mo += S.fronts[t].b; }
    S.parent_map.assign(mo, -1);
  }
  for (int t = 0; t < T; ++t) {
    const FrontInfo& P = S.fronts[t];
    const int mP = P.p + P.b;
    for (int k = 0; k < mP; ++k) loc[S.front_dofs[P.idx_off + k]] = k;
    for (int32_t ch : B.tchildren[t]) {
      const FrontInfo& C = S.fronts[ch];
      for (int k = 0; k < C.b; ++k) {
        int32_t d = S.front_dofs[C.idx_off + C.p + k];
        int32_t pos = loc[d];
        if (pos < 0) { set_error("extend-add map: border dof missing in parent"); return ELP_ERR_ARG; }
        S.parent_map[C.map_off + k] = pos;
      }
    }
    for (int k = 0; k < mP; ++k) loc[S.front_dofs[P.idx_off + k]] = -1;
  }
  for (int t = 0; t < T; ++t)
    if (S.fronts[t].parent < 0 && S.fronts[t].b != 0) { set_error("root front with a border"); return ELP_ERR_ARG; }

  // ---- per-entry arena offsets
  // Entry (r, c) belongs to the front F that eliminates min(pos r, pos c);
  // that DOF is one of F's pivots, whose positions are consecutive, so its
  // local index is its position minus F's first. The other DOF is a later
  // pivot of F or in F's border; the border runs in ascending elimination
  // position (its nodes are sorted by rank and all come after F's pivots),
  // so its local index is a binary search there. Rows are independent.
  const int64_t nnz = m.nnz;
  std::vector<int32_t> front_of_pos(n);
  for (int t = 0; t < T; ++t)
    for (int k = 0; k < S.fronts[t].p; ++k) front_of_pos[S.fronts[t].piv_off + k] = t;
  std::vector<int32_t> list_pos(S.front_dofs.size());
  for (size_t k = 0; k < S.front_dofs.size(); ++k) list_pos[k] = dof_pos[S.front_dofs[k]];
  S.entry_local.assign(nnz, -1);
  S.entry_owner.assign(nnz, -1);
  int outside = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : outside)
  for (int64_t r = 0; r < n; ++r) {
    const int32_t pr = dof_pos[r];
    for (int32_t q = m.row_ptr[r]; q < m.row_ptr[r + 1]; ++q) {
      const int32_t pc = dof_pos[m.col_idx[q]];
      const int32_t first = std::min(pr, pc), later = std::max(pr, pc);
      const FrontInfo& F = S.fronts[front_of_pos[first]];
      int32_t loc_later = later - F.piv_off;
      if (loc_later >= F.p) {
        const int32_t* lo = list_pos.data() + F.idx_off + F.p;
        const int32_t* hi = lo + F.b;
        const int32_t* it = std::lower_bound(lo, hi, later);
        if (it == hi || *it != later) { outside = 1; continue; }
        loc_later = F.p + (int32_t)(it - lo);
      }
      const int32_t loc_first = first - F.piv_off;
      const int32_t lr = pr == first ? loc_first : loc_later, lc = pr == first ? loc_later : loc_first;
      S.entry_local[q] = (int64_t)lc * (F.p + F.b) + lr;
      S.entry_owner[q] = front_of_pos[first];
    }
  }
  if (outside) { set_error("entry outside its owner front"); return ELP_ERR_ARG; }

  // ---- levels
  int L = 0;
  for (int t = 0; t < T; ++t) L = std::max(L, level[t] + 1);
  S.n_levels = L;
  S.level_fronts.assign(L, {});
  for (int t = 0; t < T; ++t) S.level_fronts[level[t]].push_back(t);
  // ---- factor-only storage. The factors of every front (its m x p panel and
  // U12) stay in the factor store for the solves; the full m x m front lives
  // in the front pool only while it is assembled and factorised: from the
  // level of its first child (or its own, for a leaf) to its own level. Pool
  // offsets are assigned first-fit, level by level, largest fronts first;
  // regions of fronts that ended at level l - 1 are free for level l.
  {
    std::vector<int> first(T);
    for (int t = 0; t < T; ++t) first[t] = level[t];
    for (int t = 0; t < T; ++t)
      if (parent[t] >= 0) first[parent[t]] = std::min(first[parent[t]], level[t]);
    std::vector<int64_t> delta(L + 1, 0);
    S.factor_stored = 0;
    S.level_new.assign(L, {});
    for (int t = 0; t < T; ++t) {
      FrontInfo& F = S.fronts[t];
      const int64_t p = F.p, b = F.b, mm = p + b;
      F.fac_off = S.factor_stored;
      S.factor_stored += p * p + 2 * p * b;
      F.start_level = first[t];
      S.level_new[first[t]].push_back(t);
      delta[first[t]] += mm * mm;
      delta[level[t] + 1] -= mm * mm;
    }
    int64_t live = 0;
    S.pool_peak = 0;
    for (int l = 0; l < L; ++l) {
      live += delta[l];
      S.pool_peak = std::max(S.pool_peak, live);
    }
    // first-fit over free intervals [off, off + len), kept sorted and merged
    std::vector<std::pair<int64_t, int64_t>> free_list;
    int64_t top = 0;
    auto release = [&](int64_t off, int64_t len) {
      auto it = std::lower_bound(free_list.begin(), free_list.end(), std::make_pair(off, (int64_t)0));
      it = free_list.insert(it, {off, len});
      size_t i = it - free_list.begin();
      if (i + 1 < free_list.size() && free_list[i].first + free_list[i].second == free_list[i + 1].first) {
        free_list[i].second += free_list[i + 1].second;
        free_list.erase(free_list.begin() + i + 1);
      }
      if (i > 0 && free_list[i - 1].first + free_list[i - 1].second == free_list[i].first) {
        free_list[i - 1].second += free_list[i].second;
        free_list.erase(free_list.begin() + i);
      }
    };
    for (int l = 0; l < L; ++l) {
      if (l > 0)
        for (int t : S.level_fronts[l - 1]) {
          const int64_t mm = (int64_t)S.fronts[t].p + S.fronts[t].b;
          release(S.fronts[t].off, mm * mm);
        }
      std::vector<int32_t> order = S.level_new[l];
      std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t c) {
        return (int64_t)S.fronts[a].p + S.fronts[a].b > (int64_t)S.fronts[c].p + S.fronts[c].b;
      });
      for (int t : order) {
        const int64_t mm = (int64_t)S.fronts[t].p + S.fronts[t].b, need = mm * mm;
        int64_t off = -1;
        for (size_t i = 0; i < free_list.size(); ++i)
          if (free_list[i].second >= need) {
            off = free_list[i].first;
            free_list[i].first += need;
            free_list[i].second -= need;
            if (free_list[i].second == 0) free_list.erase(free_list.begin() + i);
            break;
          }
        if (off < 0) {  // grow the pool (a free interval at its end is extended)
          if (!free_list.empty() && free_list.back().first + free_list.back().second == top) {
            off = free_list.back().first;
            free_list.pop_back();
          } else {
            off = top;
          }
          top = off + need;
        }
        S.fronts[t].off = off;
      }
    }
    S.pool = std::max<int64_t>(top, 1);
    // check: the fronts alive at each level occupy disjoint pool regions
    std::vector<std::pair<int64_t, int64_t>> alive;
    for (int l = 0; l < L; ++l) {
      alive.clear();
      for (int t = 0; t < T; ++t)
        if (S.fronts[t].start_level <= l && l <= level[t]) {
          const int64_t mm = (int64_t)S.fronts[t].p + S.fronts[t].b;
          alive.push_back({S.fronts[t].off, S.fronts[t].off + mm * mm});
        }
      std::sort(alive.begin(), alive.end());
      for (size_t i = 0; i < alive.size(); ++i)
        if (alive[i].first < 0 || alive[i].second > S.pool || (i > 0 && alive[i].first < alive[i - 1].second)) {
          set_error("front pool regions overlap");
          return ELP_ERR_ARG;
        }
    }
  }
  // ---- entries grouped by the start level of their owner (the scatter of a
  // level writes them before its fronts are used)
  S.entry_row.resize(nnz);
  std::vector<int64_t> cnt(L + 1, 0);
  for (int64_t r = 0; r < n; ++r)
    for (int32_t q = m.row_ptr[r]; q < m.row_ptr[r + 1]; ++q) {
      S.entry_row[q] = (int32_t)r;
      cnt[S.fronts[S.entry_owner[q]].start_level + 1]++;
    }
  for (int l = 0; l < L; ++l) cnt[l + 1] += cnt[l];
  S.level_entry_start = cnt;
  S.scatter_order.resize(nnz);
  for (int64_t q = 0; q < nnz; ++q) S.scatter_order[cnt[S.fronts[S.entry_owner[q]].start_level]++] = (int32_t)q;
  return ELP_OK;
}

}  // namespace elp
