"""GB300 frequency-response path of elPaSo-Core: Python host layer.

A thin ctypes layer over libelpaso_gb300.so (C ABI in include/elpaso_gb300.h).
It mirrors the reference's model vocabulary (nodes by id, element blocks of
"Brick8" / "DSG4" / "Fluid8", materials STR_LIN_ELA_ISO_DIR /
STR_LIN_VIS_ISO_DIR / AF_LIN_UAF_ISO_DIR, InterfaceMindlin quads, nodal
constraints and forces) and the flow of elpasoC's `frequency-basic`
analysis (analysis/frequency/analysisfrequencybasic.cpp:74-279 in the
reference): create -> assemble -> analyse -> solve per frequency.

There is no CPU path: every numeric call runs on the GPU and raises
`ElpasoError` when the CUDA library or a device is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "ElpasoError", "ModelDesc", "Model", "Group", "Server", "load_library", "library_path",
    "BRICK8", "DSG4", "FLUID8", "STR_LIN_ELA_ISO_DIR", "STR_LIN_VIS_ISO_DIR",
    "AF_LIN_UAF_ISO_DIR", "FP64_PLAIN", "MIXED", "DOF",
]

BRICK8, DSG4, FLUID8 = 1, 2, 3
STR_LIN_ELA_ISO_DIR, STR_LIN_VIS_ISO_DIR, AF_LIN_UAF_ISO_DIR = 1, 2, 3
FP64_PLAIN, MIXED = 0, 1
# arithmetic of the Brick8 / Fluid8 element contractions (elp_model_set_assembly)
ASSEMBLY_FP64, ASSEMBLY_DOUBLE_FLOAT = 0, 1
NODES_PER_ELEMENT = {BRICK8: 8, DSG4: 4, FLUID8: 8}
# fedata/basics_dof.h:24-60
DOF = {"disp_x1": 0, "disp_x2": 1, "disp_x3": 2, "disp_w1": 3, "disp_w2": 4, "fluid": 16}
NUM_KNOWN_DOFS = 21

ERRORS = {
    1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "geometry",
    5: "singular", 6: "no convergence", 7: "state", 8: "timeout",
}


class ElpasoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


HERE = os.path.dirname(os.path.abspath(__file__))


def library_path() -> str:
    return os.path.join(HERE, "lib", "libelpaso_gb300.so")


# ---------------------------------------------------------------- ctypes mirror of the header
class _Material(C.Structure):
    _fields_ = [("kind", C.c_int), ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("t", C.c_double), ("eta", C.c_double), ("visco_type", C.c_int), ("c", C.c_double),
                ("n_E_table", C.c_int), ("E_table", C.POINTER(C.c_double)),
                ("n_eta_table", C.c_int), ("eta_table", C.POINTER(C.c_double))]


class _Block(C.Structure):
    _fields_ = [("type", C.c_int), ("material", C.c_int), ("n_elements", C.c_int64),
                ("connectivity", C.POINTER(C.c_int32))]


class _Interface(C.Structure):
    _fields_ = [("ori", C.c_double), ("structure_nodes", C.c_int32 * 4), ("fluid_nodes", C.c_int32 * 4),
                ("fluid_material", C.c_int)]


class _Fixed(C.Structure):
    _fields_ = [("node", C.c_int32), ("dof", C.c_int32), ("value_re", C.c_double), ("value_im", C.c_double)]


class _Force(C.Structure):
    _fields_ = [("node", C.c_int32), ("f", C.c_double * 3)]


class _Moment(C.Structure):
    _fields_ = [("node", C.c_int32), ("m", C.c_double * 3)]


class _FluidSource(C.Structure):
    _fields_ = [("node", C.c_int32), ("p", C.c_double)]


class _VnLoad(C.Structure):
    _fields_ = [("block", C.c_int32), ("face", C.c_int32), ("element", C.c_int64), ("vn", C.c_double)]


class _FaceTraction(C.Structure):
    _fields_ = [("block", C.c_int32), ("face", C.c_int32), ("element", C.c_int64), ("t", C.c_double * 6)]


class _Desc(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("node_ids", C.POINTER(C.c_int64)), ("coords", C.POINTER(C.c_double)),
                ("n_materials", C.c_int), ("materials", C.POINTER(_Material)),
                ("n_blocks", C.c_int), ("blocks", C.POINTER(_Block)),
                ("n_interfaces", C.c_int64), ("interfaces", C.POINTER(_Interface)),
                ("n_fixed", C.c_int64), ("fixed", C.POINTER(_Fixed)),
                ("n_forces", C.c_int64), ("forces", C.POINTER(_Force)),
                ("n_moments", C.c_int64), ("moments", C.POINTER(_Moment)),
                ("n_fluid_sources", C.c_int64), ("fluid_sources", C.POINTER(_FluidSource)),
                ("n_vn_loads", C.c_int64), ("vn_loads", C.POINTER(_VnLoad)),
                ("n_face_tractions", C.c_int64), ("face_tractions", C.POINTER(_FaceTraction))]


def _plain(v):
    """ctypes arrays (nested) as lists, other values unchanged."""
    return [_plain(e) for e in v] if isinstance(v, C.Array) else v


class _Info(C.Structure):
    _fields_ = [("n_dofs", C.c_int64), ("nnz", C.c_int64), ("n_elements", C.c_int64), ("n_fronts", C.c_int64),
                ("factor_entries", C.c_int64), ("factor_flops", C.c_double), ("n_levels", C.c_int),
                ("max_front", C.c_int), ("n_struct_groups", C.c_int), ("gemm_flops", C.c_double),
                ("factor_bytes", C.c_double), ("n_nonpositive_jacobians", C.c_int64), ("factor_stored", C.c_int64),
                ("front_pool_peak", C.c_int64), ("front_pool", C.c_int64), ("device_array_bytes", C.c_int64),
                ("workspace_bytes_per_frequency", (C.c_int64 * 2) * 2)]


class SolveInfo(C.Structure):
    _fields_ = [("rel_residual", C.c_double), ("growth", C.c_double), ("iterations", C.c_int),
                ("static_pivots", C.c_int), ("converged", C.c_int), ("ms_combine", C.c_double),
                ("ms_factor", C.c_double), ("ms_solve", C.c_double), ("ms_refine", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_inflight", C.c_int), ("precision", C.c_int),
                ("tol", C.c_double), ("omega_batch", C.c_int)]


class Tuning(C.Structure):
    """elp_tuning: leaf, schur_tile, pack_count, pack_min_border, lanes (0 / negative: default;
    pack_count 0: never)."""
    _fields_ = [("leaf", C.c_int), ("schur_tile", C.c_int), ("pack_count", C.c_int),
                ("pack_min_border", C.c_int), ("lanes", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

    @classmethod
    def of(cls, knobs: dict):
        """The knobs given; every other field -1 (its default)."""
        vals = {k: -1 for k, _ in cls._fields_}
        vals.update({k: int(v) for k, v in knobs.items()})
        return cls(**vals)


class RequestResult(C.Structure):
    _fields_ = [("request_id", C.c_int64), ("status", C.c_int), ("n_omega", C.c_int),
                ("latency_ms", C.c_double), ("max_rel_residual", C.c_double)]


# every symbol of include/elpaso_gb300.h
EXPORTS = [
    "elp_model_create", "elp_model_assemble", "elp_model_analyse", "elp_model_get_info",
    "elp_model_pattern", "elp_model_global_rows", "elp_model_system_values", "elp_model_rhs",
    "elp_model_rhs_omega", "elp_cell_stresses", "elp_node_stresses",
    "elp_solve", "elp_model_destroy", "elp_last_error", "elp_solve_device", "elp_model_time_assembly",
    "elp_server_create", "elp_server_add_model", "elp_server_submit", "elp_server_wait",
    "elp_server_destroy", "elp_profile", "elp_profile_read", "elp_residual_noalloc", "elp_fault_inject",
    "elp_front_update_test", "elp_group_create", "elp_group_info", "elp_group_solve", "elp_group_destroy",
    "elp_model_set_tuning", "elp_model_get_tuning", "elp_model_autotune", "elp_group_set_tuning",
    "elp_group_autotune", "elp_peak_fp64", "elp_model_set_assembly",
]
KERNEL_CLASSES = ["assemble", "dscale", "scatter", "panel", "border", "urow", "gemm", "extend_add", "forward",
                  "backward", "residual", "norms", "rhs", "update", "values", "gemm_tc", "spmv", "fwd_border",
                  "bwd_u12", "krylov", "schur_tc", "pack"]

_lib = None


def load_library(path: str | None = None):
    """Loads the CUDA library; raises when it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise ElpasoError(2, f"{p} is missing: run __graft_entry__.build() (there is no CPU fallback)")
    lib = C.CDLL(p)
    P = C.c_void_p
    lib.elp_last_error.restype = C.c_char_p
    lib.elp_model_create.argtypes = [C.POINTER(_Desc), C.POINTER(P)]
    lib.elp_model_assemble.argtypes = [P]
    lib.elp_model_analyse.argtypes = [P]
    lib.elp_model_get_info.argtypes = [P, C.POINTER(_Info)]
    lib.elp_model_pattern.argtypes = [P, P, P, C.POINTER(C.c_int64)]
    lib.elp_model_global_rows.argtypes = [P, P]
    lib.elp_model_system_values.argtypes = [P, C.c_double, P]
    lib.elp_model_rhs.argtypes = [P, P]
    lib.elp_model_rhs_omega.argtypes = [P, C.c_double, P]
    lib.elp_cell_stresses.argtypes = [P, C.c_double, P, P, P]
    lib.elp_node_stresses.argtypes = [P, C.c_double, P, P]
    lib.elp_solve.argtypes = [P, P, C.c_int, C.c_int, P, P, P, C.c_double]
    lib.elp_solve_device.argtypes = [P, P, C.c_int, C.c_int, P, P, P, C.c_double, P]
    lib.elp_model_time_assembly.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.elp_model_destroy.argtypes = [P]
    lib.elp_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(P)]
    lib.elp_server_add_model.argtypes = [P, P, C.POINTER(C.c_int)]
    lib.elp_server_submit.argtypes = [P, C.c_int, P, C.c_int, P, C.POINTER(C.c_int64)]
    lib.elp_server_wait.argtypes = [P, C.POINTER(RequestResult), C.c_double]
    lib.elp_server_destroy.argtypes = [P]
    lib.elp_residual_noalloc.argtypes = [P, P, C.c_int, P, P, P, P, P]
    lib.elp_fault_inject.argtypes = [C.c_int, C.c_int]
    lib.elp_group_create.argtypes = [P, C.c_int, C.POINTER(P)]
    lib.elp_group_info.argtypes = [P, C.POINTER(_Info)]
    lib.elp_group_solve.argtypes = [P, P, C.c_int, C.c_int, P, P, C.c_double]
    lib.elp_group_destroy.argtypes = [P]
    lib.elp_model_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.elp_model_set_assembly.argtypes = [P, C.c_int]
    lib.elp_model_get_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.elp_model_autotune.argtypes = [P, P, C.c_int, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int)]
    lib.elp_group_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.elp_peak_fp64.argtypes = [C.POINTER(C.c_double)]
    lib.elp_group_autotune.argtypes = [P, P, C.c_int, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int)]
    lib.elp_front_update_test.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int, P, P]
    lib.elp_profile.argtypes = [C.c_int]
    lib.elp_profile_read.argtypes = [P, P, P, C.POINTER(C.c_int)]
    if path is None:
        _lib = lib
    return lib


def _check(rc: int):
    if rc != 0:
        raise ElpasoError(rc, load_library().elp_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- model description
@dataclass
class ModelDesc:
    """Host description of an elpasoC frequency-basic model.

    Nodes are numbered by ascending `node_ids` (cMesh keeps nodes in a
    std::map, fedata/mesh.h:49); element connectivity, interfaces, constraints
    and loads refer to node INDICES into these arrays.
    """
    node_ids: np.ndarray
    coords: np.ndarray
    materials: list = field(default_factory=list)     # dicts: kind, E, nu, rho, t, eta, visco_type, c,
                                                      # optional E_table / eta_table: rows (Hz, value)
    blocks: list = field(default_factory=list)        # (type, material index, conn[ne, npe])
    interfaces: dict | None = None                    # ori[q], snodes[q,4], fnodes[q,4], fmat[q]
    fixed: dict | None = None                         # node[k], dof[k], value[k] complex
    forces: dict | None = None                        # node[k], f[k,3]
    moments: dict | None = None                       # node[k], m[k,3] (on w1 w2 w3)
    fluid_sources: dict | None = None                 # node[k], p[k] (F += 4 pi p on the fluid row)
    vn_loads: dict | None = None                      # block[k], element[k], face[k] (1..6), vn[k]
    face_tractions: dict | None = None                # Brick8: block[k], element[k], face[k] (1..6), t[k,3] complex
    name: str = "model"

    @property
    def n_nodes(self) -> int:
        return int(len(self.node_ids))

    def n_elements(self) -> int:
        return int(sum(len(b[2]) for b in self.blocks))


class _DescHolder:
    """Keeps the ctypes arrays alive while the C side copies them."""

    def __init__(self, d: ModelDesc):
        self.ids = np.ascontiguousarray(d.node_ids, dtype=np.int64)
        self.xyz = np.ascontiguousarray(d.coords, dtype=np.float64).reshape(-1)
        mats = (_Material * max(1, len(d.materials)))()
        self.tables = []
        for i, m in enumerate(d.materials):
            mats[i] = _Material(int(m["kind"]), float(m.get("E", 0.0)), float(m.get("nu", 0.0)),
                                float(m.get("rho", 0.0)), float(m.get("t", 0.0)), float(m.get("eta", 0.0)),
                                int(m.get("visco_type", 1)), float(m.get("c", 0.0)))
            for key in ("E_table", "eta_table"):
                tab = m.get(key)
                if tab is None or len(tab) == 0:
                    continue
                tab = np.ascontiguousarray(np.asarray(tab, dtype=np.float64).reshape(-1, 2))
                self.tables.append(tab)
                setattr(mats[i], "n_" + key, int(tab.shape[0]))
                setattr(mats[i], key, tab.ctypes.data_as(C.POINTER(C.c_double)))
        self.mats = mats
        self.conns = []
        blocks = (_Block * max(1, len(d.blocks)))()
        for i, (typ, mat, conn) in enumerate(d.blocks):
            cn = np.ascontiguousarray(conn, dtype=np.int32)
            self.conns.append(cn)
            blocks[i] = _Block(int(typ), int(mat), int(cn.shape[0]), cn.ctypes.data_as(C.POINTER(C.c_int32)))
        self.blocks = blocks
        nq = 0 if d.interfaces is None else len(d.interfaces["ori"])
        ifs = (_Interface * max(1, nq))()
        for q in range(nq):
            ifs[q].ori = float(d.interfaces["ori"][q])
            for k in range(4):
                ifs[q].structure_nodes[k] = int(d.interfaces["snodes"][q][k])
                ifs[q].fluid_nodes[k] = int(d.interfaces["fnodes"][q][k])
            ifs[q].fluid_material = int(d.interfaces["fmat"][q]) if "fmat" in d.interfaces else 0
        self.ifs = ifs
        nf = 0 if d.fixed is None else len(d.fixed["node"])
        fx = (_Fixed * max(1, nf))()
        for k in range(nf):
            v = complex(d.fixed["value"][k]) if "value" in d.fixed else 0j
            fx[k] = _Fixed(int(d.fixed["node"][k]), int(d.fixed["dof"][k]), v.real, v.imag)
        self.fx = fx
        nl = 0 if d.forces is None else len(d.forces["node"])
        fo = (_Force * max(1, nl))()
        for k in range(nl):
            fo[k].node = int(d.forces["node"][k])
            for j in range(3):
                fo[k].f[j] = float(d.forces["f"][k][j])
        self.fo = fo
        nm = 0 if d.moments is None else len(d.moments["node"])
        mo = (_Moment * max(1, nm))()
        for k in range(nm):
            mo[k].node = int(d.moments["node"][k])
            for j in range(3):
                mo[k].m[j] = float(d.moments["m"][k][j])
        self.mo = mo
        ns = 0 if d.fluid_sources is None else len(d.fluid_sources["node"])
        so = (_FluidSource * max(1, ns))()
        for k in range(ns):
            so[k] = _FluidSource(int(d.fluid_sources["node"][k]), float(d.fluid_sources["p"][k]))
        self.so = so
        nv = 0 if d.vn_loads is None else len(d.vn_loads["element"])
        vl = (_VnLoad * max(1, nv))()
        for k in range(nv):
            vl[k] = _VnLoad(int(d.vn_loads["block"][k]), int(d.vn_loads["face"][k]), int(d.vn_loads["element"][k]),
                            float(d.vn_loads["vn"][k]))
        self.vl = vl
        nt = 0 if d.face_tractions is None else len(d.face_tractions["element"])
        tr = (_FaceTraction * max(1, nt))()
        for k in range(nt):
            tr[k].block = int(d.face_tractions["block"][k])
            tr[k].face = int(d.face_tractions["face"][k])
            tr[k].element = int(d.face_tractions["element"][k])
            for j in range(3):
                t = complex(d.face_tractions["t"][k][j])
                tr[k].t[2 * j], tr[k].t[2 * j + 1] = t.real, t.imag
        self.tr = tr
        self.desc = _Desc(len(self.ids), self.ids.ctypes.data_as(C.POINTER(C.c_int64)),
                          self.xyz.ctypes.data_as(C.POINTER(C.c_double)), len(d.materials), mats,
                          len(d.blocks), blocks, nq, ifs, nf, fx, nl, fo, nm, mo, ns, so, nv, vl, nt, tr)


class Model:
    """One elpasoC model on the GPU: numbering, pattern, assembled arrays,
    symbolic factorisation (all resident while the object lives)."""

    def __init__(self, desc: ModelDesc):
        self.lib = load_library()
        self.desc = desc
        h = _DescHolder(desc)
        self.handle = C.c_void_p()
        _check(self.lib.elp_model_create(C.byref(h.desc), C.byref(self.handle)))
        self._info = None

    def close(self):
        if getattr(self, "handle", None):
            self.lib.elp_model_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble(self):
        _check(self.lib.elp_model_assemble(self.handle))
        return self

    def analyse(self):
        _check(self.lib.elp_model_analyse(self.handle))
        return self

    def info(self) -> dict:
        i = _Info()
        _check(self.lib.elp_model_get_info(self.handle, C.byref(i)))
        return {k: _plain(getattr(i, k)) for k, _ in i._fields_}

    @property
    def n(self) -> int:
        return int(self.info()["n_dofs"])

    def pattern(self):
        nnz = C.c_int64()
        _check(self.lib.elp_model_pattern(self.handle, None, None, C.byref(nnz)))
        rp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        _check(self.lib.elp_model_pattern(self.handle, _ptr(rp), _ptr(ci), C.byref(nnz)))
        return rp, ci

    def global_rows(self) -> np.ndarray:
        out = np.zeros((self.desc.n_nodes, NUM_KNOWN_DOFS), np.int32)
        _check(self.lib.elp_model_global_rows(self.handle, _ptr(out)))
        return out

    def system_values(self, omega: float) -> np.ndarray:
        nnz = self.info()["nnz"]
        out = np.zeros(2 * nnz, np.float64)
        _check(self.lib.elp_model_system_values(self.handle, float(omega), _ptr(out)))
        return out.view(np.complex128)

    def rhs(self, omega: float | None = None) -> np.ndarray:
        """F without omega (the w-independent part), F(omega) with it."""
        out = np.zeros(2 * self.n, np.float64)
        if omega is None:
            _check(self.lib.elp_model_rhs(self.handle, _ptr(out)))
        else:
            _check(self.lib.elp_model_rhs_omega(self.handle, float(omega), _ptr(out)))
        return out.view(np.complex128)

    def cell_stresses(self, omega: float, x: np.ndarray):
        """(sigma, sigma_lower): [n_elements, 9] complex per element of the
        solution x at omega (elements in descriptor order)."""
        ne = int(sum(len(b[2]) for b in self.desc.blocks))
        xs = np.ascontiguousarray(x, dtype=np.complex128)
        if xs.shape != (self.n,):
            raise ValueError("x must hold n complex values")
        up = np.zeros((ne, 9), np.complex128)
        lo = np.zeros((ne, 9), np.complex128)
        _check(self.lib.elp_cell_stresses(self.handle, float(omega), _ptr(xs), _ptr(up), _ptr(lo)))
        return up, lo

    def node_stresses(self, omega: float, x: np.ndarray) -> np.ndarray:
        """[n_nodes, 9] complex nodal stresses of the solution x at omega,
        nodes in ascending id."""
        xs = np.ascontiguousarray(x, dtype=np.complex128)
        if xs.shape != (self.n,):
            raise ValueError("x must hold n complex values")
        out = np.zeros((self.desc.n_nodes, 9), np.complex128)
        _check(self.lib.elp_node_stresses(self.handle, float(omega), _ptr(xs), _ptr(out)))
        return out

    def set_assembly(self, arithmetic: int):
        """ASSEMBLY_FP64 (default) or ASSEMBLY_DOUBLE_FLOAT for the Brick8 /
        Fluid8 contractions; an assembled model is assembled again."""
        _check(self.lib.elp_model_set_assembly(self.handle, int(arithmetic)))
        return self

    def set_tuning(self, **knobs):
        """leaf, schur_tile, pack_count, pack_min_border, lanes (unset: default)."""
        t = Tuning.of(knobs)
        _check(self.lib.elp_model_set_tuning(self.handle, C.byref(t)))
        return self

    def tuning(self) -> dict:
        t = Tuning()
        _check(self.lib.elp_model_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def autotune(self, omegas, precision: int = MIXED):
        """(chosen tuning, seconds of its timed solve, trials)."""
        om = np.ascontiguousarray(np.atleast_1d(omegas), dtype=np.float64)
        t, sec, n = Tuning(), C.c_double(), C.c_int()
        _check(self.lib.elp_model_autotune(self.handle, _ptr(om), len(om), int(precision), C.byref(t), C.byref(sec),
                                           C.byref(n)))
        return t.as_dict(), sec.value, n.value

    def time_assembly(self, repeats: int = 3):
        a, b = C.c_double(), C.c_double()
        _check(self.lib.elp_model_time_assembly(self.handle, repeats, C.byref(a), C.byref(b)))
        return a.value, b.value

    def solve(self, omegas, precision: int = FP64_PLAIN, f: np.ndarray | None = None, tol: float = 1e-10,
              raise_on_noconv: bool = True, out: np.ndarray | None = None):
        """Solves A(w) u = f for each angular frequency; returns (x[n_omega, n], infos).

        raise_on_noconv=False returns the solutions and infos when some
        frequency missed the tolerance (status 6) or hit zero pivots (5).

        f and out may be host buffers the caller owns (pinned ones copy at
        full link speed); out must be C-contiguous complex128 [n_omega, n]."""
        om = np.ascontiguousarray(np.atleast_1d(omegas), dtype=np.float64)
        n = self.n
        if out is None:
            x = np.zeros((len(om), n), np.complex128)
        else:
            if out.dtype != np.complex128 or out.shape != (len(om), n) or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous complex128 array of shape (n_omega, n)")
            x = out
        infos = (SolveInfo * max(1, len(om)))()
        fp = None
        if f is not None:
            f = np.ascontiguousarray(np.broadcast_to(np.asarray(f, np.complex128), (len(om), n)))
            fp = _ptr(f)
        rc = self.lib.elp_solve(self.handle, _ptr(om), len(om), int(precision), fp, _ptr(x),
                                C.cast(infos, C.c_void_p), float(tol))
        # 6: a frequency short of the tolerance; 5: the same with zero pivots
        # (singular); both still return every solution and info
        if rc != 0 and (rc not in (5, 6) or raise_on_noconv):
            _check(rc)
        return x, [infos[i].as_dict() for i in range(len(om))]


class Group:
    """Several models solved together as one system (elp_group_*): every tree
    level is one launch over the fronts of all members, each member with its
    own frequencies, right-hand side and numbering. The members are copied:
    the group does not refer to the Model objects afterwards."""

    def __init__(self, models):
        self.lib = load_library()
        arr = (C.c_void_p * len(models))(*[m.handle.value for m in models])
        self.ns = [m.n for m in models]
        self.handle = C.c_void_p()
        _check(self.lib.elp_group_create(C.cast(arr, C.c_void_p), len(models), C.byref(self.handle)))

    def info(self) -> dict:
        i = _Info()
        _check(self.lib.elp_group_info(self.handle, C.byref(i)))
        return {k: _plain(getattr(i, k)) for k, _ in i._fields_}

    def set_tuning(self, **knobs):
        t = Tuning.of(knobs)
        _check(self.lib.elp_group_set_tuning(self.handle, C.byref(t)))
        return self

    def autotune(self, omegas, precision: int = MIXED):
        """(chosen tuning, seconds of its timed solve, trials); omegas as for solve."""
        om = np.ascontiguousarray(np.asarray(omegas, np.float64))
        t, sec, n = Tuning(), C.c_double(), C.c_int()
        _check(self.lib.elp_group_autotune(self.handle, _ptr(om), om.shape[1], int(precision), C.byref(t),
                                           C.byref(sec), C.byref(n)))
        return t.as_dict(), sec.value, n.value

    def solve(self, omegas, precision: int = MIXED, tol: float = 1e-10, raise_on_noconv: bool = True):
        """omegas: [n_models, n_omega] angular frequencies (each member its own).
        Returns ([x_k of shape (n_omega, n_k)], [[info] per frequency] per member)."""
        om = np.ascontiguousarray(np.asarray(omegas, np.float64))
        if om.ndim != 2 or om.shape[0] != len(self.ns):
            raise ValueError("omegas must be [n_models, n_omega]")
        nw = om.shape[1]
        x = np.zeros(sum(self.ns) * nw, np.complex128)
        infos = (SolveInfo * max(1, len(self.ns) * nw))()
        rc = self.lib.elp_group_solve(self.handle, _ptr(om), nw, int(precision), _ptr(x), C.cast(infos, C.c_void_p),
                                      float(tol))
        if rc != 0 and (rc not in (5, 6) or raise_on_noconv):
            _check(rc)
        xs, off = [], 0
        for n in self.ns:
            xs.append(x[off:off + nw * n].reshape(nw, n))
            off += nw * n
        return xs, [[infos[k * nw + j].as_dict() for j in range(nw)] for k in range(len(self.ns))]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.elp_group_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def peak_fp64() -> float:
    """Measured FP64 FMA rate of the current device, TFLOP/s."""
    v = C.c_double()
    _check(load_library().elp_peak_fp64(C.byref(v)))
    return v.value


def profile(enable: bool = True):
    """Resets the launch counters; with enable, times every launch by class."""
    _check(load_library().elp_profile(int(bool(enable))))


def profile_read() -> dict:
    ms = np.zeros(len(KERNEL_CLASSES))
    launches = np.zeros(len(KERNEL_CLASSES), np.int64)
    timed = np.zeros(len(KERNEL_CLASSES), np.int64)
    nc = C.c_int()
    _check(load_library().elp_profile_read(_ptr(ms), _ptr(launches), _ptr(timed), C.byref(nc)))
    return {KERNEL_CLASSES[i]: {"ms": float(ms[i]), "launches": int(launches[i]), "timed": int(timed[i])}
            for i in range(nc.value)}


class Server:
    """Continuous-batching serving loop over resident models (C side)."""

    def __init__(self, hbm_budget_bytes: int = 64 << 30, max_inflight: int = 4, precision: int = MIXED,
                 tol: float = 1e-10, omega_batch: int = 16):
        self.lib = load_library()
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_inflight), int(precision), float(tol), int(omega_batch))
        self.handle = C.c_void_p()
        _check(self.lib.elp_server_create(C.byref(cfg), C.byref(self.handle)))
        self._keep = {}

    def add_model(self, model: Model) -> int:
        mid = C.c_int()
        _check(self.lib.elp_server_add_model(self.handle, model.handle, C.byref(mid)))
        return mid.value

    def submit(self, model_id: int, omegas, out: np.ndarray) -> int:
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        rid = C.c_int64()
        _check(self.lib.elp_server_submit(self.handle, int(model_id), _ptr(om), len(om), _ptr(out), C.byref(rid)))
        self._keep[rid.value] = (om, out)
        return rid.value

    def wait(self, timeout_ms: float = -1.0) -> dict:
        r = RequestResult()
        _check(self.lib.elp_server_wait(self.handle, C.byref(r), float(timeout_ms)))
        self._keep.pop(r.request_id, None)
        return {k: getattr(r, k) for k, _ in r._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.elp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
