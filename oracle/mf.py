"""Test infrastructure (CPU oracle), not product code.

A CPU multifrontal LU for the FP64 direct-solve oracle and the CPU baseline,
restating the published algorithm of the reference's solver, MUMPS
(KSPPREONLY + PCLU + MUMPS, elpasoCore/source/analysis/analysis.cpp:1159-1169,
1293-1332; PETSc 3.19.1's MUMPS, version not pinned in the reference tree):
a fill-reducing nested-dissection order, an assembly tree of dense fronts,
partial pivoting within each front's fully summed block, and Schur
complements extend-added into the parent. Dense work goes to LAPACK/BLAS
(SciPy). Like MUMPS, it uses tree parallelism: the fronts of one tree level
are independent, so the fronts of a level are spread over a pool of host
threads that share the BLAS threads: single-threaded BLAS for the many small
fronts near the leaves, multithreaded BLAS for the few large ones near the
root.

It is written independently of the product's symbolic phase. The ordering
is a geometric nested dissection on node coordinates (median cut along the
longest box axis, separator = the side boundary of the smaller cost).
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

_THREADS = os.cpu_count() or 1
_SET_NAMES = ("openblas_set_num_threads", "openblas_set_num_threads64_", "scipy_openblas_set_num_threads",
              "scipy_openblas_set_num_threads64_")
_blas_setters = None


def _blas_libs():
    """(set, get) pairs of every OpenBLAS loaded in this process (numpy and
    SciPy may each carry their own); empty where none is found."""
    global _blas_setters
    if _blas_setters is None:
        found, seen = [], set()
        try:
            paths = {ln.split()[-1] for ln in open("/proc/self/maps") if "blas" in ln.lower() and ".so" in ln}
        except OSError:
            paths = set()
        for path in sorted(paths):
            try:
                lib = ctypes.CDLL(path)
            except OSError:
                continue
            for name in _SET_NAMES:
                get = name.replace("set_num", "get_num")
                if hasattr(lib, name) and hasattr(lib, get):
                    fs, fg = getattr(lib, name), getattr(lib, get)
                    key = ctypes.cast(fs, ctypes.c_void_p).value
                    if key not in seen:
                        seen.add(key)
                        fs.argtypes, fs.restype, fg.restype = [ctypes.c_int], None, ctypes.c_int
                        found.append((fs, fg))
        _blas_setters = found
    return _blas_setters


# BLAS thread counts are process-wide: factorisations that change them run
# one at a time (values would not change, but interleaved set / restore pairs
# could leave BLAS oversubscribed or at one thread)
_FACTOR_LOCK = threading.Lock()


@contextlib.contextmanager
def _blas_threads(n):
    """Run the block with n BLAS threads, then restore the previous counts."""
    libs = _blas_libs()
    old = [g() for _, g in libs]
    for s, _ in libs:
        s(n)
    try:
        yield
    finally:
        for (s, _), k in zip(libs, old):
            s(k)


def _node_graph(indptr, indices, dof_node, n_nodes):
    rows = np.repeat(np.arange(len(indptr) - 1), np.diff(indptr))
    a = dof_node[rows]
    b = dof_node[indices]
    keep = a != b
    G = sp.coo_matrix((np.ones(int(keep.sum()), np.int8), (a[keep], b[keep])), shape=(n_nodes, n_nodes)).tocsr()
    G.sum_duplicates()
    return G.indptr, G.indices


def _dissect(nodes, coords, gptr, gidx, ndof, leaf, mark, stamp, out):
    """Appends (pivot_nodes, children) tuples in postorder; returns root ids."""
    if ndof[nodes].sum() <= leaf or len(nodes) <= 2:
        out.append((nodes, []))
        return [len(out) - 1]
    xyz = coords[nodes]
    ext = xyz.max(0) - xyz.min(0)
    ax = int(np.argmax(ext))
    if ext[ax] <= 0:
        left, right = nodes[: len(nodes) // 2], nodes[len(nodes) // 2:]
    else:
        med = np.median(xyz[:, ax])
        lm = xyz[:, ax] < med
        if lm.all() or not lm.any():
            lm = xyz[:, ax] <= med
        if lm.all() or not lm.any():
            lm = np.zeros(len(nodes), bool)
            lm[: len(nodes) // 2] = True
        left, right = nodes[lm], nodes[~lm]
    stamp[0] += 1
    s = stamp[0]
    mark[left] = 2 * s
    mark[right] = 2 * s + 1

    def boundary(side, other):
        sep = []
        for v in side:
            nb = gidx[gptr[v]:gptr[v + 1]]
            if np.any(mark[nb] == other):
                sep.append(v)
        return np.asarray(sep, np.int64)
    sl, sr = boundary(left, 2 * s + 1), boundary(right, 2 * s)
    if ndof[sl].sum() < ndof[sr].sum():
        sep, left = sl, np.setdiff1d(left, sl, assume_unique=True)
    else:
        sep, right = sr, np.setdiff1d(right, sr, assume_unique=True)
    kids = []
    if len(left):
        kids += _dissect(left, coords, gptr, gidx, ndof, leaf, mark, stamp, out)
    if len(right):
        kids += _dissect(right, coords, gptr, gidx, ndof, leaf, mark, stamp, out)
    if len(sep) == 0:
        return kids
    out.append((sep, kids))
    return [len(out) - 1]


class Multifrontal:
    """Symbolic analysis once per pattern; factor + solve per matrix."""

    def __init__(self, indptr, indices, dof_node, coords, leaf=96):
        n = len(indptr) - 1
        n_nodes = len(coords)
        dof_node = np.asarray(dof_node)
        ndof = np.bincount(dof_node, minlength=n_nodes)
        node_dofs = [[] for _ in range(n_nodes)]
        for d, v in enumerate(dof_node):
            node_dofs[v].append(d)
        gptr, gidx = _node_graph(indptr, indices, dof_node, n_nodes)
        import sys
        sys.setrecursionlimit(10000)
        out = []
        mark = np.zeros(n_nodes, np.int64)
        active = np.nonzero(ndof)[0]
        _dissect(active, np.asarray(coords, float), gptr, gidx, ndof, leaf, mark, [0], out)
        T = len(out)
        snode = np.full(n_nodes, -1, np.int64)
        for t, (nodes, _) in enumerate(out):
            snode[nodes] = t
        rank = np.empty(n_nodes, np.int64)
        r = 0
        for nodes, _ in out:
            rank[nodes] = np.arange(r, r + len(nodes))
            r += len(nodes)
        parent = np.full(T, -1, np.int64)
        level = np.zeros(T, np.int64)  # 0 at the leaves, 1 + the highest child above them
        for t, (_, kids) in enumerate(out):
            for c in kids:
                parent[c] = t
                level[t] = max(level[t], level[c] + 1)
        self.levels = [np.nonzero(level == L)[0].tolist() for L in range(int(level.max()) + 1 if T else 0)]
        borders = []
        for t, (nodes, kids) in enumerate(out):
            cand = set()
            for v in nodes:
                for u in gidx[gptr[v]:gptr[v + 1]]:
                    if snode[u] > t:
                        cand.add(int(u))
            for c in kids:
                cand.update(x for x in borders[c] if snode[x] > t)
            borders.append(sorted(cand, key=lambda u: rank[u]))
        self.fronts = []
        pos = np.empty(n, np.int64)   # elimination position of every dof
        owner_of_pos = np.empty(n, np.int64)
        e = 0
        for t, (nodes, kids) in enumerate(out):
            piv = np.asarray([d for v in nodes for d in node_dofs[v]], np.int64)
            bor = np.asarray([d for v in borders[t] for d in node_dofs[v]], np.int64)
            self.fronts.append((piv, bor, list(kids)))
            pos[piv] = np.arange(e, e + len(piv))
            owner_of_pos[e:e + len(piv)] = t
            e += len(piv)
        # every CSR entry goes to the front of whichever of row/column is eliminated first
        rows = np.repeat(np.arange(n), np.diff(indptr))
        owner = owner_of_pos[np.minimum(pos[rows], pos[indices])]
        order = np.argsort(owner, kind="stable")
        bounds = np.searchsorted(owner[order], np.arange(T + 1))
        local = np.full(n, -1, np.int64)
        self.assembly = []
        for t, (piv, bor, kids) in enumerate(self.fronts):
            idx = np.concatenate([piv, bor])
            local[idx] = np.arange(len(idx))
            q = order[bounds[t]:bounds[t + 1]]
            kid_maps = [local[np.concatenate([self.fronts[c][1]])] for c in kids]
            self.assembly.append((q, local[rows[q]], local[indices[q]], kid_maps))
            local[idx] = -1
        self.n = n
        self.indptr, self.indices = indptr, indices

    def factor(self, A):
        """A: scipy CSR (complex128) on the analysed pattern. Levels run in
        order (children before parents); the fronts of a level of k >= 2
        fronts are spread over the thread pool, each with 1/k of the BLAS
        threads (only where this process's BLAS thread count can be set;
        else all run in order). Calls from several Python threads run one
        after another (the BLAS thread count is process-wide)."""
        A = A.tocsr()
        assert np.array_equal(A.indptr, self.indptr) and np.array_equal(A.indices, self.indices)
        data = A.data
        self.F = [None] * len(self.fronts)
        self._cb = {}
        parallel = _THREADS > 1 and bool(_blas_libs())
        with _FACTOR_LOCK, ThreadPoolExecutor(max_workers=_THREADS) as pool:
            for group in self.levels:
                if parallel and len(group) >= 2:
                    with _blas_threads(max(1, _THREADS // len(group))):
                        list(pool.map(lambda t: self._factor_front(t, data), group))
                else:
                    for t in group:
                        self._factor_front(t, data)
        del self._cb

    def _factor_front(self, t, data):
        piv, bor, kids = self.fronts[t]
        p, m = len(piv), len(piv) + len(bor)
        q, lr, lc, kid_maps = self.assembly[t]
        F = np.zeros((m, m), np.complex128)
        F[lr, lc] = data[q]
        for c, loc in zip(kids, kid_maps):
            F[np.ix_(loc, loc)] += self._cb.pop(c)
        lu, perm = sla.lu_factor(F[:p, :p], check_finite=False)
        pv = list(range(p))  # LAPACK's row interchanges, in order, as one permutation
        for k, pk in enumerate(perm.tolist()):
            if pk != k:
                pv[k], pv[pk] = pv[pk], pv[k]
        pv = np.asarray(pv, np.int64)
        U12 = sla.solve_triangular(lu, F[:p, p:][pv], lower=True, unit_diagonal=True, check_finite=False)
        L21 = sla.solve_triangular(lu, F[p:, :p].T, trans="T", lower=False, check_finite=False).T
        if m > p:
            self._cb[t] = F[p:, p:] - L21 @ U12
        self.F[t] = (lu, pv, L21, U12)

    def solve_h(self, c):
        """Solves A^H y = c with the factors of A (for condition estimates).
        A^-1 = B F with the forward sweep F = G_T..G_1 (G_t: the front's row
        interchanges, then L11^-1 and the L21 update) and the backward sweep
        B = B_1..B_T (B_t: U11^-1 after the U12 update); so A^-H = F^H B^H:
        the adjoint backward steps in elimination order, then the adjoint
        forward steps in reverse order, each ending with the interchanges
        scattered back."""
        y = np.array(c, np.complex128, copy=True)
        for (piv, bor, _), (lu, perm, L21, U12) in zip(self.fronts, self.F):
            yp = sla.solve_triangular(lu, y[piv], trans="C", lower=False, check_finite=False)
            y[piv] = yp
            if len(bor):
                y[bor] -= U12.conj().T @ yp
        for (piv, bor, _), (lu, perm, L21, U12) in zip(reversed(self.fronts), reversed(self.F)):
            t = y[piv]
            if len(bor):
                t = t - L21.conj().T @ y[bor]
            t = sla.solve_triangular(lu, t, trans="C", lower=True, unit_diagonal=True, check_finite=False)
            out = np.empty_like(t)
            out[perm] = t
            y[piv] = out
        return y

    def solve(self, b):
        y = np.array(b, np.complex128, copy=True)
        for (piv, bor, _), (lu, perm, L21, U12) in zip(self.fronts, self.F):
            yp = y[piv][perm]
            yp = sla.solve_triangular(lu, yp, lower=True, unit_diagonal=True, check_finite=False)
            y[piv] = yp
            if len(bor):
                y[bor] -= L21 @ yp
        for (piv, bor, _), (lu, perm, L21, U12) in zip(reversed(self.fronts), reversed(self.F)):
            t = y[piv]
            if len(bor):
                t = t - U12 @ y[bor]
            y[piv] = sla.solve_triangular(lu, t, lower=False, check_finite=False)
        return y
