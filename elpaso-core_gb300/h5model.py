"""elpasoC HDF5 model files -> ModelDesc, and reference solution files.

Mirrors the parts of the reference's HDF5 parser that feed the frequency
path (``ESC/misc/parser/femparserhdf5.cpp:202-499``; group names from
``ESC/misc/hdf5/rulesh5.h:31-157``):

* ``/Nodes/mtxFemNodes``: compound {Ids, xCoords, yCoords, zCoords};
* ``/Elements/mtxFemElemGroup*``: rows (element id, node ids...), attributes
  ``ElementType`` (DSG4 / Brick8 / Fluid8) and ``MaterialId``;
* ``/Materials/*``: attributes ``Id``, ``MaterialType`` and the parameters as
  strings (``E``, ``nu``, ``rho``, ``t``, ``eta``, ``type``, ``c``;
  ``ESC/misc/hdf5/rulesh5.h:112-141``); a visco material's ``E`` or ``eta``
  that is not a number (``isnumber``, ``ESC/basics/misc.cpp:22-45``) names a
  dataset of rows (frequency [Hz], value): the frequency table
  (``materialstructurevisco.cpp:75-170, 643-690``);
* ``/NodeConstraints/*``: structural constraints with flags ``u1..u3``,
  ``w1..w3`` and values ``valu*``/``valw*`` (reference DOF enum 0..5), and
  ``acoustic`` ones fixing the fluid dof (enum 16) at ``p``;
* ``/NodeLoads/*``: ``point_force`` loads ``Fx, Fy, Fz`` and ``fluid`` point
  sources ``P`` at ``NodeId``; ``/NodeMoments/*``: ``point_moment`` loads
  ``Mx, My, Mz``; ``/ElemLoads/*``: ``vn`` loads (``vn``, ``Face``,
  ``ElementId``) on Fluid8 faces;
* ``/Analysis`` attributes ``start``, ``steps``, ``delta``: the frequency list,
  unless a ``<input file>.frq`` list exists beside the file
  (``generateFrequencies``, ``analysisfrequencybasic.cpp:36-72``).

and the solution file elpasoC writes (``ESC/analysis/frequency/
analysisfrequencybasic.cpp:184-262``): ``/Solution/State/vecFemStep{k}``
complex vectors with ``FreqStep{k}`` attributes, ``/Solution/Maps/mtxDofMap``
(node id, dof enum) per global row.

and writes elpasoC model files (``write_model``: a ModelDesc in the layout
above, so the reference can run the package's synthetic configurations) and
both files elpasoC writes for this path: the solution file
(``write_solution``, the layout above) and the system-matrix export of
``-exportSysH5`` (``write_system_matrix``: ``/SystemMatrices/<type>`` with
integer attributes ``numrow``, ``numcol``, 1-based CSR ``vecCsrIa``,
``vecCsrJa`` and complex ``cmpCsrVal``; ``ESC/math/mathlibrary.cpp:53-86``).

``/InterfaceElements`` of type ``InterfaceMindlin`` are read
(``read_interfaces``); non-conforming interface elements raise
``NotImplementedError``.
"""
from __future__ import annotations

import importlib.util
import os

import numpy as np

try:
    from . import h5lite
except ImportError:  # loaded as a plain module
    _spec = importlib.util.spec_from_file_location("h5lite", os.path.join(os.path.dirname(__file__), "h5lite.py"))
    h5lite = importlib.util.module_from_spec(_spec)
    _spec.loader.exec_module(h5lite)

_ELEMENT_TYPES = {"Brick8": 1, "DSG4": 2, "Fluid8": 3}     # ELP_BRICK8, ELP_DSG4, ELP_FLUID8
_MATERIAL_KINDS = {"STR_LIN_ELA_ISO_DIR": 1, "STR_LIN_VIS_ISO_DIR": 2, "AF_LIN_UAF_ISO_DIR": 3}
_CONSTRAINT_DOFS = (("u1", 0), ("u2", 1), ("u3", 2), ("w1", 3), ("w2", 4), ("w3", 5))


def _num(attrs, key, default=0.0):
    v = attrs.get(key, default)
    return float(v) if not isinstance(v, str) or v.strip() else default


def _is_number(s: str) -> bool:
    """The reference's isnumber (ESC/basics/misc.cpp:22-45): digits, at most one
    '.', at most one 'e'/'E', a sign only first or right after 'e'/'E'."""
    points = exps = 0
    for i, ch in enumerate(s):
        if ch in "+-" and (i == 0 or s[i - 1] in "eE"):
            continue
        if ch == ".":
            points += 1
        elif ch in "eE":
            exps += 1
        elif not ch.isdigit():
            return False
    return points <= 1 and exps <= 1


def _num_or_table(f, attrs, key):
    """(value, table): a number, or a dataset named by the attribute holding
    rows (frequency [Hz], value) (cReaderH5::readDenseDoubleMatrix, first two
    columns)."""
    v = attrs.get(key, 0.0)
    if isinstance(v, str):
        v = v.strip()
        if v and not _is_number(v):
            t = np.asarray(f[v.lstrip("/")].read(), dtype=np.float64)
            return 0.0, t.reshape(t.shape[0], -1)[:, :2].copy()
        return (float(v) if v else 0.0), None
    return float(v), None


def frequency_list(input_path: str, start: float, delta: float, steps: int) -> np.ndarray:
    """Frequencies [Hz] of a run (generateFrequencies,
    analysisfrequencybasic.cpp:36-72): the numbers of ``<input>.frq`` (a trailing
    ``.ak3`` of the input name removed first) if that file exists, else
    start + delta * step for step < steps; sorted and unique either way (a
    std::set). A token that is not a number ends the reference's read loop
    without reaching end-of-file; here it raises ValueError."""
    name = input_path[:-4] if input_path.endswith(".ak3") else input_path
    frq = name + ".frq"
    if os.path.exists(frq):
        with open(frq) as fh:
            vals = [float(tok) for tok in fh.read().split()]
    else:
        vals = [start + delta * k for k in range(int(steps))]
    return np.unique(np.asarray(vals, dtype=np.float64))


def read_interfaces(f, index, mat_index):
    """``/InterfaceElements`` (cFemParserHDF5::getInterfaceElementsData,
    femparserhdf5.cpp:527-552; cElementInterfaceFactory::parseSingleInterfaceElement,
    elementinterfacefactory.cpp:62-97): per dataset, attribute ``type``
    (``InterfaceMindlin``), ``matF``, and integer rows (element id, ori,
    structure node ids..., fluid node ids...). Returns the ModelDesc
    ``interfaces`` dict, or None without interface elements. ``index`` maps
    node ids to indices, ``mat_index`` material ids to material indices."""
    if "InterfaceElements" not in f or not int(f["InterfaceElements"].attrs.get("N", 0)):
        return None
    ori, snodes, fnodes, fmat = [], [], [], []
    for name in sorted(f["InterfaceElements"].keys()):
        ds = f["InterfaceElements"][name]
        a = ds.attrs
        if a.get("type") != "InterfaceMindlin":
            raise NotImplementedError(f"interface type {a.get('type')}")
        nnod = int(a.get("NfluidNodes", 4))
        if nnod != 4 or int(a.get("NstructNodes", 4)) != 4:
            raise NotImplementedError("interface elements with other than 4 + 4 nodes")
        rows = np.asarray(ds.read()).astype(np.int64).reshape(-1, 2 + 2 * nnod)
        for r in rows:
            ori.append(float(r[1]))
            snodes.append([index[int(v)] for v in r[2:2 + nnod]])
            fnodes.append([index[int(v)] for v in r[2 + nnod:2 + 2 * nnod]])
            fmat.append(mat_index[int(a["matF"])])
    return dict(ori=np.array(ori), snodes=np.array(snodes, np.int64), fnodes=np.array(fnodes, np.int64),
                fmat=np.array(fmat, np.int64))


def read_model(path: str, model_desc_cls=None):
    """Reads an elpasoC model file. Returns (ModelDesc, frequencies in Hz)."""
    if model_desc_cls is None:
        from . import ModelDesc as model_desc_cls  # noqa: N813
    f = h5lite.File(path)
    nodes = f["Nodes/mtxFemNodes"].read()
    ids = nodes["Ids"].astype(np.int64)
    order = np.argsort(ids, kind="stable")
    ids = ids[order]
    coords = np.stack([nodes["xCoords"], nodes["yCoords"], nodes["zCoords"]], axis=1)[order]
    index = {int(v): i for i, v in enumerate(ids)}

    mats, mat_index = [], {}
    for name in sorted(f["Materials"].keys()):
        a = f["Materials"][name].attrs
        kind = _MATERIAL_KINDS.get(a["MaterialType"])
        if kind is None:
            raise NotImplementedError(f"material type {a['MaterialType']}")
        mat_index[int(a["Id"])] = len(mats)
        E, E_table = _num_or_table(f, a, "E") if kind == 2 else (_num(a, "E"), None)
        eta, eta_table = _num_or_table(f, a, "eta") if kind == 2 else (_num(a, "eta"), None)
        mat = dict(kind=kind, E=E, nu=_num(a, "nu"), rho=_num(a, "rho"), t=_num(a, "t"),
                   eta=eta, visco_type=int(_num(a, "type", 1.0)) or 1, c=_num(a, "c"))
        if E_table is not None:
            mat["E_table"] = E_table
        if eta_table is not None:
            mat["eta_table"] = eta_table
        mats.append(mat)

    blocks = []
    element_at = {}  # element id -> (block, index in the block)
    for name in sorted(f["Elements"].keys(), key=lambda s: int("".join(c for c in s if c.isdigit()) or 0)):
        ds = f["Elements"][name]
        typ = _ELEMENT_TYPES.get(ds.attrs["ElementType"])
        if typ is None:
            raise NotImplementedError(f"element type {ds.attrs['ElementType']}")
        rows = ds.read().astype(np.int64)
        conn = np.vectorize(index.__getitem__, otypes=[np.int64])(rows[:, 1:])
        for e, eid in enumerate(rows[:, 0]):
            element_at[int(eid)] = (len(blocks), e)
        blocks.append((typ, mat_index[int(ds.attrs["MaterialId"])], conn.astype(np.int32)))

    interfaces = read_interfaces(f, index, mat_index)
    if "NCInterfaceElements" in f and int(f["NCInterfaceElements"].attrs.get("N", 0)):
        raise NotImplementedError("NCInterfaceElements are not read")

    fnode, fdof, fval = [], [], []
    if "NodeConstraints" in f:
        for name in sorted(f["NodeConstraints"].keys()):
            a = f["NodeConstraints"][name].attrs
            kind = a.get("ConstraintType")
            if kind == "structure":
                for key, dof in _CONSTRAINT_DOFS:
                    if int(a.get(key, 0)):
                        fnode.append(index[int(a["NodeId"])])
                        fdof.append(dof)
                        fval.append(complex(float(a.get("val" + key, 0.0))))
            elif kind == "acoustic":  # fixed pressure p on the fluid dof (boundaryconditionfluid.cpp:36-57)
                fnode.append(index[int(a["NodeId"])])
                fdof.append(16)
                fval.append(complex(float(a.get("p", 0.0))))
            else:
                raise NotImplementedError(f"constraint type {kind}")
    lnode, lf, snode, sp = [], [], [], []
    if "NodeLoads" in f:  # cNodalForceFactory (nodalforcefactory.cpp:36-55)
        for name in sorted(f["NodeLoads"].keys()):
            a = f["NodeLoads"][name].attrs
            if a.get("LoadType") == "point_force":
                lnode.append(index[int(a["NodeId"])])
                lf.append([float(a["Fx"]), float(a["Fy"]), float(a["Fz"])])
            elif a.get("LoadType") == "fluid":
                snode.append(index[int(a["NodeId"])])
                sp.append(float(a["P"]))
            else:
                raise NotImplementedError(f"load type {a.get('LoadType')}")
    mnode, mm = [], []
    if "NodeMoments" in f:  # cNodalMomentFactory: point_moment (nodalmomentfactory.cpp:40)
        for name in sorted(f["NodeMoments"].keys()):
            a = f["NodeMoments"][name].attrs
            if a.get("LoadType") != "point_moment":
                raise NotImplementedError(f"moment type {a.get('LoadType')}")
            mnode.append(index[int(a["NodeId"])])
            mm.append([float(a["Mx"]), float(a["My"]), float(a["Mz"])])
    vb, ve, vf, vv = [], [], [], []
    if "ElemLoads" in f:  # cElementLoadFactory: vn (elementloadfactory.cpp:34-46)
        for name in sorted(f["ElemLoads"].keys()):
            a = f["ElemLoads"][name].attrs
            if a.get("LoadType") != "vn":
                raise NotImplementedError(f"element load type {a.get('LoadType')}")
            b, e = element_at[int(a["ElementId"])]
            vb.append(b)
            ve.append(e)
            vf.append(int(a["Face"]))
            vv.append(float(a["vn"]))

    an = f["Analysis"].attrs
    freqs = frequency_list(path, float(an["start"]), float(an["delta"]), int(an["steps"]))
    desc = model_desc_cls(
        node_ids=ids, coords=coords, materials=mats, blocks=blocks, interfaces=interfaces,
        fixed=dict(node=np.array(fnode, np.int64), dof=np.array(fdof, np.int64), value=np.array(fval, complex)),
        forces=dict(node=np.array(lnode, np.int64), f=np.array(lf).reshape(-1, 3)),
        moments=dict(node=np.array(mnode, np.int64), m=np.array(mm).reshape(-1, 3)),
        fluid_sources=dict(node=np.array(snode, np.int64), p=np.array(sp, float)),
        vn_loads=dict(block=np.array(vb, np.int64), element=np.array(ve, np.int64), face=np.array(vf, np.int64),
                      vn=np.array(vv, float)),
        name=os.path.splitext(os.path.basename(path))[0])
    return desc, freqs


def write_model(path: str, d, start: float = 1.0, delta: float = 1.0, steps: int = 1, node_order=None):
    """Writes a ModelDesc as an elpasoC model file (the layout read_model and
    the reference's cFemParserHDF5 read; group and attribute names of
    ESC/misc/hdf5/rulesh5.h:31-332), so the reference can run the same model.
    Material i gets Id i + 10, element ids run from 100 over the blocks,
    interface elements from 9000; E / eta tables go to root datasets named by
    the material's attributes. node_order permutes the rows of the node table
    (the reference sorts nodes by id). Brick8 face tractions have no entry in
    that format (its element-load factory makes vn loads only) and are refused."""
    if getattr(d, "face_tractions", None) is not None and len(d.face_tractions["element"]):
        raise ValueError("an elpasoC model file cannot hold Brick8 face tractions")
    w = h5lite.Writer(path)
    n = d.n_nodes
    ids = np.asarray(d.node_ids, np.int64)
    nodes = np.zeros(n, dtype=[("Ids", np.int64), ("xCoords", np.float64), ("yCoords", np.float64),
                                 ("zCoords", np.float64)])
    perm = np.arange(n) if node_order is None else np.asarray(node_order)
    nodes["Ids"] = ids[perm]
    for k, c in enumerate(("xCoords", "yCoords", "zCoords")):
        nodes[c] = np.asarray(d.coords)[perm, k]
    w.dataset("Nodes/mtxFemNodes", nodes)
    kinds = {v: k for k, v in _MATERIAL_KINDS.items()}
    for i, m in enumerate(d.materials):
        g = f"Materials/material{i + 1}"
        w.group(g)
        w.attr(g, "Id", i + 10)
        w.attr(g, "MaterialType", kinds[int(m["kind"])])
        for key in ("E", "nu", "rho", "t", "eta", "c"):
            tab = m.get(key + "_table")
            if tab is not None and len(tab):
                w.dataset(f"{key}_table_{i}", np.asarray(tab, float).reshape(-1, 2))
                w.attr(g, key, f"{key}_table_{i}")
            else:
                w.attr(g, key, repr(float(m.get(key, 0.0))))
        w.attr(g, "type", str(int(m.get("visco_type", 1))))
    eid = 100
    names = {v: k for k, v in _ELEMENT_TYPES.items()}
    starts = [eid]
    for b, (typ, mi, conn) in enumerate(d.blocks):
        conn = np.asarray(conn)
        rows = np.column_stack([np.arange(eid, eid + len(conn)), ids[conn]]).astype(np.int64)
        eid += len(conn)
        starts.append(eid)
        ds = f"Elements/mtxFemElemGroup{b + 1}"
        w.dataset(ds, rows)
        w.attr(ds, "ElementType", names[int(typ)])
        w.attr(ds, "MaterialId", int(mi) + 10)
    q = d.interfaces
    if q is not None and len(q["ori"]):
        fmat = np.asarray(q.get("fmat", np.zeros(len(q["ori"]), np.int64)))
        w.group("InterfaceElements")
        groups = sorted(set(int(v) for v in fmat))
        w.attr("InterfaceElements", "N", len(groups))
        for gi, fm in enumerate(groups):
            sel = np.nonzero(fmat == fm)[0]
            rows = np.column_stack([sel + 9000, np.rint(np.asarray(q["ori"])[sel]).astype(np.int64),
                                    ids[np.asarray(q["snodes"])[sel]], ids[np.asarray(q["fnodes"])[sel]]])
            ds = f"InterfaceElements/mtxFemInterfaceElements{gi + 1}"
            w.dataset(ds, rows.astype(np.int64))
            for k, v in (("type", "InterfaceMindlin"), ("matF", fm + 10), ("mats", 10), ("NfluidNodes", 4),
                         ("NstructNodes", 4)):
                w.attr(ds, k, v)
    dof_keys = ("u1", "u2", "u3", "w1", "w2", "w3")
    if d.fixed is not None:
        vals = d.fixed.get("value", np.zeros(len(d.fixed["node"]), complex))
        for k, (node, dof, val) in enumerate(zip(d.fixed["node"], d.fixed["dof"], vals)):
            g = f"NodeConstraints/nodeConstraint{k}"
            w.dataset(g, np.zeros(1))
            w.attr(g, "NodeId", int(ids[node]))
            w.attr(g, "Id", k + 1)
            if int(dof) == 16:
                w.attr(g, "ConstraintType", "acoustic")
                w.attr(g, "p", float(complex(val).real))
            else:
                w.attr(g, "ConstraintType", "structure")
                w.attr(g, dof_keys[int(dof)], 1)
                w.attr(g, "val" + dof_keys[int(dof)], float(complex(val).real))
    k = 0
    for node, f in zip(*(() if d.forces is None else (d.forces["node"], d.forces["f"]))):
        g = f"NodeLoads/load{k}"
        k += 1
        w.dataset(g, np.zeros(1))
        for key, v in (("LoadType", "point_force"), ("Id", k), ("NodeId", int(ids[node])), ("Fx", float(f[0])),
                       ("Fy", float(f[1])), ("Fz", float(f[2]))):
            w.attr(g, key, v)
    src = getattr(d, "fluid_sources", None)
    for node, p in zip(*(() if src is None else (src["node"], src["p"]))):
        g = f"NodeLoads/load{k}"
        k += 1
        w.dataset(g, np.zeros(1))
        for key, v in (("LoadType", "fluid"), ("Id", k), ("NodeId", int(ids[node])), ("P", float(p))):
            w.attr(g, key, v)
    mom = getattr(d, "moments", None)
    for j, (node, mm) in enumerate(zip(*(() if mom is None else (mom["node"], mom["m"])))):
        g = f"NodeMoments/moment{j}"
        w.dataset(g, np.zeros(1))
        for key, v in (("LoadType", "point_moment"), ("Id", j + 1), ("NodeId", int(ids[node])), ("Mx", float(mm[0])),
                       ("My", float(mm[1])), ("Mz", float(mm[2]))):
            w.attr(g, key, v)
    vl = getattr(d, "vn_loads", None)
    for j in range(0 if vl is None else len(vl["vn"])):
        g = f"ElemLoads/eload{j}"
        w.dataset(g, np.zeros(1))
        e = starts[int(vl["block"][j])] + int(vl["element"][j])
        for key, v in (("LoadType", "vn"), ("Id", j + 1), ("ElementId", e), ("Face", int(vl["face"][j])),
                       ("vn", float(vl["vn"][j]))):
            w.attr(g, key, v)
    w.group("Analysis")
    for key, v in (("start", repr(float(start))), ("delta", repr(float(delta))), ("steps", str(int(steps)))):
        w.attr("Analysis", key, v)
    w.close()


def read_solution(path: str):
    """Reads an elpasoC solution file. Returns (freqs [k], x [k, n] complex,
    dof_map [n, 2] of (node id, dof enum))."""
    f = h5lite.File(path)
    state = f["Solution/State"]
    steps = sorted((int(k[len("vecFemStep"):]) for k in state.keys() if k.startswith("vecFemStep")))
    freqs = np.array([float(state.attrs[f"FreqStep{k}"]) for k in steps])
    xs = []
    for k in steps:
        v = state[f"vecFemStep{k}"].read()
        xs.append(v["real"] + 1j * v["imag"])
    return freqs, np.array(xs), f["Solution/Maps/mtxDofMap"].read().astype(np.int64)


def dof_map(node_ids, global_rows) -> np.ndarray:
    """(node id, dof enum) of every global row, as elpasoC's mtxDofMap:
    nodes in id order, active DOFs in enum order (analysisfrequencybasic.cpp:248-256).
    `global_rows` is the [nodes, known dofs] row table of Model.global_rows()."""
    gr = np.asarray(global_rows)
    node, dof = np.nonzero(gr >= 0)
    out = np.empty((int(gr.max()) + 1, 2), np.int32)
    out[gr[node, dof], 0] = np.asarray(node_ids)[node]
    out[gr[node, dof], 1] = dof
    return out


def write_solution(path: str, freqs, xs, dofs) -> None:
    """elpasoC's solution file: /Solution/State/vecFemStep{k} (complex
    {real, imag}, k = 1..), string attributes FreqStep{k} on /Solution/State
    (the frequency as std::to_string prints it), /Solution/Maps/mtxDofMap."""
    w = h5lite.Writer(path)
    for k, (f, x) in enumerate(zip(freqs, xs)):
        w.dataset(f"/Solution/State/vecFemStep{k + 1}", np.asarray(x, np.complex128))
        w.attr("/Solution/State", f"FreqStep{k + 1}", "%f" % float(f))
    w.dataset("/Solution/Maps/mtxDofMap", np.asarray(dofs, np.int32))
    w.close()


def write_system_matrix(path: str, row_ptr, col_idx, values, ncols: int | None = None,
                        system: str = "DynamicStiffness") -> None:
    """The -exportSysH5 file of one assembled system: 0-based CSR in, 1-based
    vecCsrIa / vecCsrJa out (MathLibrary::RetrieveRowVectorsFromMat with
    offset 1), complex cmpCsrVal, numrow / numcol attributes."""
    rp = np.asarray(row_ptr, np.int64)
    n = len(rp) - 1
    w = h5lite.Writer(path)
    g = f"/SystemMatrices/{system}"
    w.group(g)
    w.attr(g, "numrow", n)
    w.attr(g, "numcol", n if ncols is None else int(ncols))
    w.dataset(g + "/vecCsrIa", (rp + 1).astype(np.int32))
    w.dataset(g + "/vecCsrJa", (np.asarray(col_idx, np.int64) + 1).astype(np.int32))
    w.dataset(g + "/cmpCsrVal", np.asarray(values, np.complex128))
    w.close()
