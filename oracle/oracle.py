"""Test infrastructure (CPU oracle), not product code.

Only tests/, `__graft_entry__.smoke()` and bench.py's CPU baseline use this
module, and only as the checker. It restates, independently of the product
code, the reference's host-side flow for one frequency (paths inside
elpasoCore/source/ of the reference):

  numbering      analysis/analysis.cpp:475-520 (nodes by id, DOF enum order)
  pattern        analysis/analysis.cpp:806-867 + 1238-1246, interface blocks
                 element/interface/elementinterfacestructural.cpp:152-179;
                 negative rows dropped by PETSc, explicit zeros kept,
                 diagonal inserted by preallocateMatrix (analysis.cpp:791)
  BC rows        analysis/analysis.cpp:366-454 (MatZeroRows diag = 1, F[row] = value)
  RHS            analysis/analysis.cpp:171-364 (nodal forces, fluid point
                 sources, nodal moments, ADD); normal-velocity face loads of
                 Fluid8 elements as the 1/w part (elementfluid3d.cpp:241-309);
                 constant Brick8 face tractions, C t with the face matrix C
                 (elementstructurebrick.cpp:556-662), before the nodal loads
  values         element matrices EM(w) of oracle/elp_oracle.c, inserted per
                 element, interfaces with -ori (analysisfrequencybasic.cpp:101-157)
  stresses       cell stresses after the solve (analysis.cpp:869-905)
  materials      E_vis(w), E and eta from frequency tables where given
                 (material/.../viscoelastic/materialstructurevisco.cpp:229-287)
  solve          SciPy SuperLU, complex128, on the system with the Dirichlet
                 columns lifted to the right-hand side (stand-in for MUMPS,
                 which is not available here) -- the FP64 direct-solve oracle

The element restatement itself is pinned against the reference's own
element code compiled from its sources (oracle/_ref, tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libelpref.so")

BRICK8, DSG4, FLUID8 = 1, 2, 3
ELA, VIS, FLU = 1, 2, 3
ELEM_DOFS = {BRICK8: (0, 1, 2), DSG4: (2, 3, 4), FLUID8: (16,)}
NPE = {BRICK8: 8, DSG4: 4, FLUID8: 8}

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "elp_oracle.c")):
            build_oracle()
        _lib = C.CDLL(LIB)
        for f in ("orc_brick8", "orc_dsg4", "orc_fluid8", "orc_interface_mindlin", "orc_assemble", "orc_assemble_rows"):
            getattr(_lib, f).restype = C.c_int
    return _lib


def ref_lib():
    """The reference's own element code (oracle/_ref), or None when absent."""
    if not os.path.exists(REF_LIB):
        return None
    return C.CDLL(REF_LIB)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _d(x):
    return C.c_double(float(x))


# ------------------------------------------------------------------ elements
def brick8(xyz, E, nu, rho, omega):
    K = np.zeros(2 * 576); M = np.zeros(2 * 576); EM = np.zeros(2 * 576)
    x = np.ascontiguousarray(xyz, np.float64)
    lib().orc_brick8(_p(x), _d(complex(E).real), _d(complex(E).imag), _d(nu), _d(rho), _d(omega), _p(K), _p(M), _p(EM))
    f = lambda a: a.view(np.complex128).reshape(24, 24)
    return f(K), f(M), f(EM)


def dsg4(xyz, E, nu, rho, t, omega):
    K = np.zeros(2 * 144); M = np.zeros(2 * 144); EM = np.zeros(2 * 144)
    x = np.ascontiguousarray(xyz, np.float64)
    rc = lib().orc_dsg4(_p(x), _d(complex(E).real), _d(complex(E).imag), _d(nu), _d(rho), _d(t), _d(omega),
                        _p(K), _p(M), _p(EM))
    f = lambda a: a.view(np.complex128).reshape(12, 12)
    return f(K), f(M), f(EM), rc


def fluid8(xyz, c, rho, omega):
    K = np.zeros(128); M = np.zeros(128); EM = np.zeros(128)
    x = np.ascontiguousarray(xyz, np.float64)
    lib().orc_fluid8(_p(x), _d(c), _d(rho), _d(omega), _p(K), _p(M), _p(EM))
    f = lambda a: a.view(np.complex128).reshape(8, 8)
    return f(K), f(M), f(EM)


def interface_mindlin(xyz_fluid, transform=False):
    Cm = np.zeros(96)
    x = np.ascontiguousarray(xyz_fluid, np.float64)
    lib().orc_interface_mindlin(_p(x), int(bool(transform)), _p(Cm))
    return Cm.view(np.complex128).reshape(12, 4)


def table_value(table, omega):
    """A frequency table at angular frequency omega, by the rule of
    cMaterialStructureVisco::updateMaterial (materialstructurevisco.cpp:229-281):
    rows (frequency [Hz], value) are read as (2 pi f, value)
    (readEFromFile / readEtaFromFile, :75-170); at or below the first row the
    first value, at or above the last row the last value, otherwise linear
    interpolation between the rows k-1, k with w_{k-1} <= omega < w_k."""
    t = np.asarray(table, dtype=np.float64).reshape(-1, 2)
    om, v = 2.0 * np.pi * t[:, 0], t[:, 1]
    if omega <= om[0]:
        return v[0]
    if omega >= om[-1]:
        return v[-1]
    for k in range(1, len(om)):
        if om[k - 1] <= omega < om[k]:
            return ((v[k] - v[k - 1]) * (omega - om[k - 1]) / (om[k] - om[k - 1])) + v[k - 1]
    raise ValueError("frequency table not ascending")


def e_vis(mat, omega):
    """E_vis of materialstructurevisco.cpp:284-285 (E and eta from their
    frequency tables when the material has them), real E for the elastic kind."""
    if mat["kind"] == VIS:
        E = table_value(mat["E_table"], omega) if len(mat.get("E_table", ())) else mat["E"]
        eta = table_value(mat["eta_table"], omega) if len(mat.get("eta_table", ())) else mat["eta"]
        if int(mat.get("visco_type", 1)) == 2:
            return E * (1.0 + 1j * omega * eta)
        return E * (1.0 + 1j * eta)
    return complex(mat["E"])


# faces of a hexahedron as cShapeHex8::getIndicesOfFaceNodes numbers them
# (shape/shapehex8.cpp:119-150); an input face f is surfaces[f - 1]
HEX8_FACES = ((0, 1, 5, 4), (2, 3, 7, 6), (0, 3, 2, 1), (1, 2, 6, 5), (4, 5, 6, 7), (0, 4, 7, 3))


def face_integrals(xyz):
    """int N_z dA over a 4-node face (rows: the face's nodes in order), the
    row sums of C(z, s) = int N_z N_s dA of evaluateSurfaceIntegral
    (element/fluid/elementfluid3d.cpp:169-233): bilinear N on
    [-1, 1]^2 with nodes at (-1,-1), (1,-1), (1,1), (-1,1), 2 x 2 Gauss points
    (weight 1), surface Jacobian sqrt(|a1|^2 |a2|^2 - (a1.a2)^2)."""
    xyz = np.asarray(xyz, np.float64)
    cx = np.array([-1.0, 1.0, 1.0, -1.0])
    cy = np.array([-1.0, -1.0, 1.0, 1.0])
    out = np.zeros(4)
    g = 1.0 / np.sqrt(3.0)
    for u in (-g, g):
        for v in (-g, g):
            N = 0.25 * (1 + cx * u) * (1 + cy * v)
            a1 = (0.25 * cx * (1 + cy * v)) @ xyz
            a2 = (0.25 * cy * (1 + cx * u)) @ xyz
            jac = np.sqrt(a1 @ a1 * (a2 @ a2) - (a1 @ a2) ** 2)
            out += N * jac
    return out


def face_matrix(xyz):
    """C(z, s) = int N_z N_s dA over a 4-node face, evaluateSurfaceIntegral of
    the Brick8 element (element/structure/linear/brick/elementstructurebrick.cpp:597-662;
    the same quadrature as face_integrals, whose results are the row sums)."""
    xyz = np.asarray(xyz, np.float64)
    cx = np.array([-1.0, 1.0, 1.0, -1.0])
    cy = np.array([-1.0, -1.0, 1.0, 1.0])
    C = np.zeros((4, 4))
    g = 1.0 / np.sqrt(3.0)
    for u in (-g, g):
        for v in (-g, g):
            N = 0.25 * (1 + cx * u) * (1 + cy * v)
            a1 = (0.25 * cx * (1 + cy * v)) @ xyz
            a2 = (0.25 * cy * (1 + cx * u)) @ xyz
            jac = np.sqrt(a1 @ a1 * (a2 @ a2) - (a1 @ a2) ** 2)
            C += np.outer(N, N) * jac
    return C


# ------------------------------------------------------------------ host flow
class System:
    """Numbering, pattern, BC rows and RHS of a model description."""

    def __init__(self, d):
        self.d = d
        N = len(d.node_ids)
        order = np.argsort(np.asarray(d.node_ids), kind="stable")
        active = [set() for _ in range(N)]
        for typ, _, conn in d.blocks:
            for e in np.asarray(conn):
                for v in e:
                    active[v].update(ELEM_DOFS[typ])
        rows = -np.ones((N, 21), np.int64)
        r = 0
        for v in order:
            for k in range(21):
                if k in active[v]:
                    rows[v, k] = r
                    r += 1
        self.rows = rows
        self.n = r
        pattern = [set([i]) for i in range(r)]
        for typ, _, conn in d.blocks:
            for e in np.asarray(conn):
                g = [rows[v, k] for v in e for k in ELEM_DOFS[typ]]
                g = [x for x in g if x >= 0]
                for i in g:
                    pattern[i].update(g)
        self.iface_rows = []
        if d.interfaces is not None:
            for q in range(len(d.interfaces["ori"])):
                sr = [rows[d.interfaces["snodes"][q][k], dd] for k in range(4) for dd in (0, 1, 2)]
                fr = [rows[d.interfaces["fnodes"][q][k], 16] for k in range(4)]
                self.iface_rows.append(sr + fr)
                for z in sr:
                    if z < 0:
                        continue
                    for s in fr:
                        if s >= 0:
                            pattern[z].add(s)
                            pattern[s].add(z)
        self.row_ptr = np.zeros(r + 1, np.int32)
        cols = []
        for i in range(r):
            c = sorted(pattern[i])
            cols.extend(c)
            self.row_ptr[i + 1] = self.row_ptr[i] + len(c)
        self.col_idx = np.asarray(cols, np.int32)
        # BC rows in reference order
        self.bc_rows, self.bc_vals = [], []
        if d.fixed is not None:
            by_node = {}
            for k in range(len(d.fixed["node"])):
                by_node.setdefault(int(d.fixed["node"][k]), []).append(k)
            for v in order:
                for k in by_node.get(int(v), []):
                    dof = int(d.fixed["dof"][k])
                    if rows[v, dof] >= 0:
                        self.bc_rows.append(int(rows[v, dof]))
                        self.bc_vals.append(complex(d.fixed["value"][k]) if "value" in d.fixed else 0j)
        f = np.zeros(r, np.complex128)
        # element load vectors come first (assembleGlobalTensors, then the nodal
        # loads): a constant traction t on a Brick8 face adds
        # LV[3 z + d] = sum_s C(z, s) t_d (elementstructurebrick.cpp:556-595)
        if getattr(d, "face_tractions", None) is not None:
            ft = d.face_tractions
            for k in range(len(ft["element"])):
                conn = np.asarray(d.blocks[int(ft["block"][k])][2])[int(ft["element"][k])]
                face = conn[list(HEX8_FACES[int(ft["face"][k]) - 1])]
                C = face_matrix(d.coords[face])
                t = np.asarray(ft["t"][k], np.complex128)
                lv = C @ np.tile(t, (4, 1))  # F[3 s + d] = t_d at every face node
                for z in range(4):
                    for dd in range(3):
                        if rows[face[z], dd] >= 0:
                            f[rows[face[z], dd]] += lv[z, dd]
        if d.forces is not None:
            for k in range(len(d.forces["node"])):
                v = int(d.forces["node"][k])
                for dd in range(3):
                    if rows[v, dd] >= 0:
                        f[rows[v, dd]] += d.forces["f"][k][dd]
        # fluid point sources: F += 4 pi p on the fluid row (analysis.cpp:243-265)
        if getattr(d, "fluid_sources", None) is not None:
            for k in range(len(d.fluid_sources["node"])):
                v = int(d.fluid_sources["node"][k])
                if rows[v, 16] >= 0:
                    f[rows[v, 16]] += 4.0 * np.pi * d.fluid_sources["p"][k]
        # nodal moments on the active w1 w2 w3 (analysis.cpp:281-364)
        if getattr(d, "moments", None) is not None:
            for k in range(len(d.moments["node"])):
                v = int(d.moments["node"][k])
                for dd in range(3):
                    if rows[v, 3 + dd] >= 0:
                        f[rows[v, 3 + dd]] += d.moments["m"][k][dd]
        # normal-velocity loads: the 1/w part G of F(w) = f + G / w
        g = np.zeros(r, np.complex128)
        if getattr(d, "vn_loads", None) is not None:
            for k in range(len(d.vn_loads["element"])):
                conn = np.asarray(d.blocks[int(d.vn_loads["block"][k])][2])[int(d.vn_loads["element"][k])]
                face = conn[list(HEX8_FACES[int(d.vn_loads["face"][k]) - 1])]
                for z, nz in enumerate(face_integrals(d.coords[face])):
                    if rows[face[z], 16] >= 0:
                        g[rows[face[z], 16]] += -1j * d.vn_loads["vn"][k] * nz
        for rr, val in zip(self.bc_rows, self.bc_vals):
            f[rr] = val
            g[rr] = 0.0
        self.f = f
        self.f_vn = g

    def rhs(self, omega):
        """F(w) = f + G / w (G: normal-velocity loads, zero on BC rows)."""
        return self.f + self.f_vn / omega

    def values(self, omega):
        """A(w) on the pattern after BC rows (complex128, nnz)."""
        return _assemble(self.d, self.rows, self.n, self.row_ptr, self.col_idx, self.d, self.iface_rows,
                         self.bc_rows, omega, None)

    def matrix(self, omega):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values(omega), self.col_idx, self.row_ptr), shape=(self.n, self.n))

    def lifted(self, omega, f=None):
        """A(w) x = f with the Dirichlet columns moved to the right-hand side.

        The boundary rows are identity rows (MatZeroRows with diagonal 1,
        elpasoCore/source/analysis/analysis.cpp:426-441), so they fix
        x_c = rhs_c; every other row i then gets rhs_i -= A_ic x_c and
        A_ic = 0. Same solution in exact arithmetic, same pattern (the lifted
        entries stay as explicit zeros). A direct solver on the unlifted
        matrix pivots the identity rows against column entries of ~1e11 and
        loses up to four digits on a clamped thin plate; on the lifted one
        it sees the free block, whose conditioning is the physical one."""
        A = self.matrix(omega)
        rhs = np.array(self.rhs(omega) if f is None else f, np.complex128, copy=True)
        if self.bc_rows:
            bc = np.zeros(self.n, bool)
            bc[self.bc_rows] = True
            g = np.where(bc, rhs, 0)
            rhs[~bc] -= (A @ g)[~bc]
            rows = np.repeat(np.arange(self.n), np.diff(A.indptr))
            A.data[bc[A.indices] & ~bc[rows]] = 0
        return A, rhs

    def free_block(self, omega):
        """(A_ff, free rows): A(w) restricted to the rows and columns that
        carry no Dirichlet condition."""
        free = np.ones(self.n, bool)
        free[self.bc_rows] = False
        idx = np.nonzero(free)[0]
        return self.matrix(omega)[idx][:, idx], idx

    def solve(self, omega, f=None):
        """FP64 direct solve (SuperLU) of the lifted system."""
        import scipy.sparse.linalg as sla
        A, rhs = self.lifted(omega, f)
        return sla.splu(A.tocsc()).solve(rhs)


def material_c6(E, nu):
    """The 3D constitutive matrix of cMaterialStructureVisco::setupC
    (materialstructurevisco.cpp:349-372), from the C restatement."""
    C6 = np.zeros(72); Cb = np.zeros(18); Cs = np.zeros(8)
    lib().orc_material(_d(complex(E).real), _d(complex(E).imag), _d(nu), _d(1.0), _p(C6), _p(Cb), _p(Cs))
    return C6.view(np.complex128).reshape(6, 6)


def _centre_shape_derivatives(nn):
    """dN/dxi (rows: xi, eta[, zeta]) of the hex8 / quad4 shape functions at the
    element centre, nodes ordered as cShapeHex8 / cShapeQuad4."""
    sx = np.array([-1, 1, 1, -1, -1, 1, 1, -1], float)
    sy = np.array([-1, -1, 1, 1, -1, -1, 1, 1], float)
    sz = np.array([-1, -1, -1, -1, 1, 1, 1, 1], float)
    if nn == 8:
        return np.stack([sx, sy, sz]) / 8.0
    return np.stack([sx[:4], sy[:4]]) / 4.0


def cell_stresses(system, omega, x):
    """computeStressesCells of every structure element (elements in the
    description's block order): 9 slots per element, (upper, lower).
    Brick8 (elementstructurebrick.cpp:48-159): Bm (6 x 24) at the centre,
    stress = C(w) Bm u. DSG4 (elementstructuremindlin.cpp:51-175): per node
    (w2, w1, w2), Bm rows (Nx, 0, 0), (0, Ny, 0), (0, 0, Ny), strains scaled
    to the upper (t/2, -t/2, t) and lower (-t/2, t/2, -t) surface,
    stress = Cm(w) strain into slots 0, 1, 3 (setupCm,
    materialstructurevisco.cpp:331-345)."""
    d, rows = system.d, system.rows
    x = np.asarray(x)
    val = lambda v, k: x[rows[v, k]] if rows[v, k] >= 0 else 0.0  # noqa: E731
    up, lo = [], []
    for typ, mi, conn in d.blocks:
        mat = d.materials[mi]
        for e in np.asarray(conn):
            s1 = np.zeros(9, complex); s2 = np.zeros(9, complex)
            if typ == BRICK8:
                dN = _centre_shape_derivatives(8)
                J = dN @ d.coords[e]
                G = np.linalg.inv(J) @ dN  # rows: d/dx, d/dy, d/dz per node
                Bm = np.zeros((6, 24))
                for k in range(8):
                    Nx, Ny, Nz = G[:, k]
                    Bm[0, 3 * k] = Nx; Bm[1, 3 * k + 1] = Ny; Bm[2, 3 * k + 2] = Nz
                    Bm[3, 3 * k] = Ny; Bm[3, 3 * k + 1] = Nx
                    Bm[4, 3 * k + 1] = Nz; Bm[4, 3 * k + 2] = Ny
                    Bm[5, 3 * k] = Nz; Bm[5, 3 * k + 2] = Nx
                u = np.array([val(v, k) for v in e for k in (0, 1, 2)], complex)
                s1[:6] = material_c6(e_vis(mat, omega), mat["nu"]) @ (Bm @ u)
            elif typ == DSG4:
                dN = _centre_shape_derivatives(4)
                J = dN @ d.coords[e][:, :2]
                G = np.linalg.inv(J) @ dN
                Bm = np.zeros((3, 12))
                for k in range(4):
                    Bm[0, 3 * k] = G[0, k]; Bm[1, 3 * k + 1] = G[1, k]; Bm[2, 3 * k + 2] = G[1, k]
                loc = [val(v, k) for v in e for k in (2, 3, 4)]  # x3, w1, w2
                rel = np.array([loc[3 * k + j] for k in range(4) for j in (2, 1, 2)], complex)
                eps = Bm @ rel
                t, nu = mat["t"], mat["nu"]
                f = e_vis(mat, omega) / (1.0 - nu * nu)
                Cm = f * np.array([[1.0, nu, 0.0], [nu, 1.0, 0.0], [0.0, 0.0, 0.5 * (1.0 - nu)]])
                a = Cm @ (np.array([0.5 * t, -0.5 * t, t]) * eps)
                b = Cm @ (np.array([-0.5 * t, 0.5 * t, -t]) * eps)
                s1[[0, 1, 3]] = a
                s2[[0, 1, 3]] = b
            up.append(s1)
            lo.append(s2)
    return np.array(up), np.array(lo)


def node_stresses(system, omega, x):
    """computeStressesNodes (analysis.cpp:907-935): 9 slots per node, nodes in
    ascending id (GlobalSeqId, analysis.cpp:516). Brick8: centre stress / the
    number of mesh elements at the node (countElementsPerNode, :455-469) added
    to slots 0..5 (elementstructurebrick.cpp:161-270). Fluid8: grad p at each
    corner, J^-1 dN/dxi p evaluated at that corner, added to slots 6..8
    without averaging (elementfluid3d.cpp:380-557). Plates: nothing."""
    d, rows = system.d, system.rows
    x = np.asarray(x)
    N = len(d.node_ids)
    seq = np.empty(N, np.int64)
    seq[np.argsort(np.asarray(d.node_ids), kind="stable")] = np.arange(N)
    count = np.zeros(N)
    for _, _, conn in d.blocks:
        np.add.at(count, np.asarray(conn).ravel(), 1.0)
    centre, _ = cell_stresses(system, omega, x)
    out = np.zeros((N, 9), complex)
    s = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)
    idx = 0
    for typ, _, conn in d.blocks:
        for e in np.asarray(conn):
            if typ == BRICK8:
                for v in e:
                    out[seq[v], :6] += centre[idx, :6] * (1.0 / count[v])
            elif typ == FLUID8:
                pv = np.array([x[rows[v, 16]] if rows[v, 16] >= 0 else 0.0 for v in e], complex)
                for k, v in enumerate(e):
                    g = 1.0 + s * s[k]  # (1 + s_f xi_k) per direction
                    dN = 0.125 * np.stack([s[:, 0] * g[:, 1] * g[:, 2], s[:, 1] * g[:, 0] * g[:, 2],
                                           s[:, 2] * g[:, 0] * g[:, 1]])
                    J = dN @ d.coords[e]
                    out[seq[v], 6:] += np.linalg.inv(J) @ dN @ pv
            idx += 1
    return out


def dof_nodes(system):
    """Node index of every dof (global row) of an oracle System."""
    out = np.empty(system.n, np.int64)
    r, k = np.nonzero(system.rows >= 0)
    out[system.rows[r, k]] = r
    return out


def _assemble(d, rows, n, row_ptr, col_idx, elements, iface_rows, bc_rows, omega, keep):
    """The oracle's C insertion loop (orc_assemble; orc_assemble_rows with a
    row mask `keep`) over the element blocks of `elements` (d itself or a
    ModelSubset of it) and the interface quads of d, on the pattern
    (row_ptr, col_idx)."""
    def pack(typ):
        # per element, in block order: node coordinates, material row,
        # global rows (node-major, then the family's DOFs)
        xyz, mat, rr = [np.zeros(0)], [np.zeros(0)], [np.zeros(0, np.int32)]
        ne = 0
        for btyp, mi, conn in elements.blocks:
            if btyp != typ:
                continue
            conn = np.asarray(conn)
            m = d.materials[mi]
            if typ == FLUID8:
                mm = [m["c"], m["rho"]]
            else:
                E = e_vis(m, omega)
                mm = [E.real, E.imag, m["nu"], m["rho"]] + ([m["t"]] if typ == DSG4 else [])
            xyz.append(d.coords[conn].reshape(-1))
            mat.append(np.tile(np.asarray(mm, np.float64), len(conn)))
            rr.append(rows[conn][:, :, ELEM_DOFS[typ]].reshape(-1))
            ne += len(conn)
        return (np.ascontiguousarray(np.concatenate(xyz), np.float64),
                np.ascontiguousarray(np.concatenate(mat), np.float64),
                np.ascontiguousarray(np.concatenate(rr), np.int32), ne)
    b, p, fl = pack(BRICK8), pack(DSG4), pack(FLUID8)
    nq = len(iface_rows)
    if nq:
        ixyz = np.ascontiguousarray(np.concatenate(
            [d.coords[np.asarray(d.interfaces["fnodes"][q])].reshape(-1) for q in range(nq)]))
        iori = np.ascontiguousarray(np.asarray(d.interfaces["ori"], np.float64))
        irows = np.ascontiguousarray(np.asarray(iface_rows, np.int32).reshape(-1))
        itr = np.ascontiguousarray(np.asarray(
            [1 if rows[d.interfaces["snodes"][q][0], 0] >= 0 else 0 for q in range(nq)], np.int32))
    else:
        ixyz = np.zeros(1); iori = np.zeros(1); irows = np.zeros(16, np.int32); itr = np.zeros(1, np.int32)
    bc = np.ascontiguousarray(np.asarray(bc_rows, np.int32)) if len(bc_rows) else np.zeros(1, np.int32)
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col_idx = np.ascontiguousarray(col_idx, np.int32)

    class S(C.Structure):
        _fields_ = [("n", C.c_int64), ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p),
                    ("n_brick", C.c_int64), ("n_plate", C.c_int64), ("n_fluid", C.c_int64), ("n_iface", C.c_int64),
                    ("brick_xyz", C.c_void_p), ("brick_mat", C.c_void_p), ("brick_rows", C.c_void_p),
                    ("plate_xyz", C.c_void_p), ("plate_mat", C.c_void_p), ("plate_rows", C.c_void_p),
                    ("fluid_xyz", C.c_void_p), ("fluid_mat", C.c_void_p), ("fluid_rows", C.c_void_p),
                    ("iface_xyz", C.c_void_p), ("iface_ori", C.c_void_p), ("iface_rows", C.c_void_p),
                    ("iface_transform", C.c_void_p), ("n_bc", C.c_int64), ("bc_rows", C.c_void_p)]
    s = S(n, _p(row_ptr), _p(col_idx), b[3], p[3], fl[3], nq,
          _p(b[0]), _p(b[1]), _p(b[2]), _p(p[0]), _p(p[1]), _p(p[2]), _p(fl[0]), _p(fl[1]), _p(fl[2]),
          _p(ixyz), _p(iori), _p(irows), _p(itr), len(bc_rows), _p(bc))
    out = np.zeros(2 * len(col_idx))
    if keep is None:
        rc = lib().orc_assemble(C.byref(s), _d(omega), _p(out))
    else:
        keep = np.ascontiguousarray(keep, np.uint8)
        rc = lib().orc_assemble_rows(C.byref(s), _p(keep), _d(omega), _p(out))
    if rc:
        raise RuntimeError(f"oracle assembly failed ({rc})")
    return out.view(np.complex128)


def numbering(d):
    """Global rows (N x 21, -1 inactive) and n: the numbering rule of
    activateDofsAtNodes (elpasoCore/source/analysis/analysis.cpp:475-520) --
    nodes in ascending id, per node the active DOFs in enum order -- written
    with array operations for models too large for System's loop."""
    N = len(d.node_ids)
    active = np.zeros((N, 21), bool)
    for typ, _, conn in d.blocks:
        conn = np.asarray(conn)
        if len(conn):
            active[np.ix_(np.unique(conn.reshape(-1)), ELEM_DOFS[typ])] = True
    order = np.argsort(np.asarray(d.node_ids), kind="stable")
    act = active[order].reshape(-1)
    num = np.cumsum(act) - 1
    rows = -np.ones(N * 21, np.int64)
    rows[act] = num[act]
    out = -np.ones((N, 21), np.int64)
    out[order] = rows.reshape(N, 21)
    return out, int(act.sum())


def _incident(conn, n_nodes):
    """CSR of node -> elements of one block."""
    conn = np.asarray(conn)
    ne, k = conn.shape
    nodes = conn.reshape(-1)
    elems = np.repeat(np.arange(ne), k)
    order = np.argsort(nodes, kind="stable")
    ptr = np.zeros(n_nodes + 1, np.int64)
    np.add.at(ptr, nodes + 1, 1)
    return np.cumsum(ptr), elems[order]


def sample_rows(d, sample, omega):
    """A(w) on a sample of global rows of a model too large for the full
    pattern (the 100^3 Brick8 cube: 245M nonzeros). For every sampled row i
    of node v: its pattern is the union of the element blocks of the
    elements at v (node-major DOFs of their nodes, inactive -1 dropped, the
    diagonal always in), as getLocalSparsityPattern builds it
    (analysis.cpp:806-867, insertElementMatrix :1238-1246); its values are
    the element matrices of exactly those elements added by the oracle's C
    restatement (orc_assemble_rows), then the Dirichlet rows. Returns
    (sample sorted, row_ptr over the sample, col_idx, values)."""
    if d.interfaces is not None and len(d.interfaces["ori"]):
        raise ValueError("row samples cover element blocks only (no interface quads)")
    rows, n = numbering(d)
    N = len(d.node_ids)
    sample = np.unique(np.asarray(sample, np.int64))
    node_of = np.empty(n, np.int64)
    r, _ = np.nonzero(rows >= 0)
    node_of[rows[rows >= 0]] = r
    keep = np.zeros(n, np.uint8)
    keep[sample] = 1
    snodes = np.unique(node_of[sample])
    # elements at the sampled nodes, per block
    picks = []
    cols = [[] for _ in range(len(sample))]
    pos = {int(x): k for k, x in enumerate(sample)}
    for bi, (typ, mi, conn) in enumerate(d.blocks):
        conn = np.asarray(conn)
        ptr, el = _incident(conn, N)
        es = np.unique(np.concatenate([el[ptr[v]:ptr[v + 1]] for v in snodes] or [np.zeros(0, np.int64)]))
        picks.append(es)
        for e in es:
            g = rows[conn[e]][:, ELEM_DOFS[typ]].reshape(-1)
            g = g[g >= 0]
            for i in g:
                k = pos.get(int(i))
                if k is not None:
                    cols[k].append(g)
    row_ptr = np.zeros(n + 1, np.int64)
    col_list = []
    for k, i in enumerate(sample):
        c = np.unique(np.concatenate(cols[k] + [np.array([i])]))
        col_list.append(c)
        row_ptr[i + 1] = len(c)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    col_idx = np.ascontiguousarray(np.concatenate(col_list).astype(np.int32))
    sub = ModelSubset(d, picks)
    bc_rows = []
    if d.fixed is not None:
        for v, dof in zip(np.asarray(d.fixed["node"]), np.asarray(d.fixed["dof"])):
            if rows[v, dof] >= 0 and keep[rows[v, dof]]:
                bc_rows.append(int(rows[v, dof]))
    vals = _assemble(d, rows, n, row_ptr, col_idx, sub, [], bc_rows, omega, keep)
    cp = np.concatenate([[0], np.cumsum([len(c) for c in col_list])]).astype(np.int64)
    return sample, cp, col_idx, vals[np.concatenate([np.arange(row_ptr[i], row_ptr[i + 1]) for i in sample])]


class ModelSubset:
    """The elements `picks[b]` of each block b of a model description."""

    def __init__(self, d, picks):
        self.blocks = [(typ, mi, np.asarray(conn)[picks[b]]) for b, (typ, mi, conn) in enumerate(d.blocks)]


def multifrontal(system, leaf=96):
    """CPU multifrontal LU (oracle/mf.py) analysed on the system's pattern."""
    from oracle.mf import Multifrontal
    return Multifrontal(system.row_ptr, system.col_idx, dof_nodes(system), system.d.coords, leaf=leaf)


def free_block_cond1(system, omega, mf):
    """kappa_1(A_ff) of the free block, estimated with Hager / Higham's
    1-norm estimator (scipy onenormest; a lower bound, usually exact) from
    the factors `mf` of the LIFTED matrix (mf.factor(system.lifted(w)[0])
    done by the caller). The lifted matrix is the free block A_ff plus
    identity rows and columns for the Dirichlet dofs, so A_ff^-1 v is the
    free part of A_lifted^-1 applied to v with zero Dirichlet entries."""
    import scipy.sparse.linalg as sla
    Aff, idx = system.free_block(omega)
    n = system.n

    def embed(v):
        z = np.zeros(n, np.complex128)
        z[idx] = v
        return z

    inv = sla.LinearOperator((len(idx), len(idx)), dtype=complex,
                             matvec=lambda v: mf.solve(embed(np.ravel(v)))[idx],
                             rmatvec=lambda v: mf.solve_h(embed(np.ravel(v)))[idx])
    return sla.onenormest(Aff) * sla.onenormest(inv)
