"""HDF5 files the reference writes for this path, written by the package.

- the elpasoC solution file (h5model.write_solution) and the -exportSysH5
  system file (h5model.write_system_matrix) round-trip through the package's
  reader (h5lite), including groups large enough for a two-level B-tree;
- the solution file's mtxDofMap built from this build's numbering
  (h5model.dof_map) equals the one elpasoC wrote for the tutorial plate.
There is no HDF5 library in this image, so the files are not cross-checked
against one.
"""
import importlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def h5model(elp):
    return importlib.import_module("elpaso_core_gb300.h5model")


def test_solution_file_round_trip(h5model, tmp_path):
    rng = np.random.default_rng(7)
    freqs = 10.0 + np.arange(300)
    xs = rng.standard_normal((300, 40)) + 1j * rng.standard_normal((300, 40))
    dofs = np.stack([np.repeat(np.arange(1, 21), 2), np.tile([2, 3], 20)], axis=1)
    path = str(tmp_path / "eGenOutput_test.hdf5")
    h5model.write_solution(path, freqs, xs, dofs)
    f2, x2, d2 = h5model.read_solution(path)
    np.testing.assert_array_equal(f2, freqs)
    np.testing.assert_array_equal(x2, xs)
    np.testing.assert_array_equal(d2, dofs)


def test_system_matrix_file_round_trip(h5model, tmp_path):
    h5 = h5model.h5lite
    rp = np.array([0, 2, 3, 5])
    ci = np.array([0, 2, 1, 0, 2])
    v = np.array([1 + 2j, 3, 4j, -1, 5.5])
    path = str(tmp_path / "eGenSystem_test.hdf5")
    h5model.write_system_matrix(path, rp, ci, v)
    g = h5.File(path)["SystemMatrices/DynamicStiffness"]
    assert int(g.attrs["numrow"]) == 3 and int(g.attrs["numcol"]) == 3
    np.testing.assert_array_equal(g["vecCsrIa"].read(), rp + 1)
    np.testing.assert_array_equal(g["vecCsrJa"].read(), ci + 1)
    val = g["cmpCsrVal"].read()
    np.testing.assert_array_equal(val["real"] + 1j * val["imag"], v)


def test_dof_map_matches_reference_tutorial(elp, h5model):
    from test_tutorial_golden import tutorial_desc
    g = np.load(os.path.join(HERE, "golden", "tutorial_plate_dsg4.npz"))
    d = tutorial_desc(elp, g)
    dm = h5model.dof_map(d.node_ids, elp.Model(d).global_rows())
    np.testing.assert_array_equal(dm, g["dof_map"])


def test_interface_elements_are_read(h5model, tmp_path):
    """/InterfaceElements rows (element id, ori, 4 structure node ids, 4 fluid
    node ids) with type InterfaceMindlin and matF (femparserhdf5.cpp:527-552,
    elementinterfacefactory.cpp:62-97) become the ModelDesc interfaces."""
    h5 = h5model.h5lite
    path = str(tmp_path / "iface.hdf5")
    rows = np.array([[7, 1, 11, 12, 13, 14, 21, 22, 23, 24],
                     [8, -1, 12, 15, 16, 13, 22, 25, 26, 23]], np.int32)
    w = h5.Writer(path)
    w.group("InterfaceElements")
    w.attr("InterfaceElements", "N", 1)
    w.dataset("InterfaceElements/mtxFemInterfaceElementGroup1", rows)
    for k, v in (("type", "InterfaceMindlin"), ("matF", 3), ("mats", 1), ("NfluidNodes", 4), ("NstructNodes", 4)):
        w.attr("InterfaceElements/mtxFemInterfaceElementGroup1", k, v)
    w.close()
    ids = [11, 12, 13, 14, 15, 16, 21, 22, 23, 24, 25, 26]
    index = {v: i for i, v in enumerate(ids)}
    q = h5model.read_interfaces(h5.File(path), index, {3: 1, 1: 0})
    np.testing.assert_array_equal(q["ori"], [1.0, -1.0])
    np.testing.assert_array_equal(q["snodes"], [[0, 1, 2, 3], [1, 4, 5, 2]])
    np.testing.assert_array_equal(q["fnodes"], [[6, 7, 8, 9], [7, 10, 11, 8]])
    np.testing.assert_array_equal(q["fmat"], [1, 1])


def test_model_file_round_trip(elp, meshes, h5model, tmp_path):
    """A coupled model with every input kind read_model handles, written in
    elpasoC's layout and read back: same numbering-relevant data, loads,
    constraints, tables, interfaces; the frequency list from <file>.frq."""
    import copy
    from test_loads import loaded_plate_cavity
    rng = np.random.default_rng(9)
    d = loaded_plate_cavity(meshes)
    d = copy.deepcopy(d)
    d.node_ids = d.node_ids * 7 + 3  # ids not equal to the indices
    d.materials[0].update(E_table=np.array([[50.0, 70e9], [400.0, 72e9]]), eta_table=np.array([[10.0, 0.02]]))
    fluid_nodes = np.unique(np.asarray([b for b in d.blocks if b[0] == 3][0][2]).ravel())
    extra = fluid_nodes[:2]
    d.fixed = dict(node=np.concatenate([d.fixed["node"], extra]), dof=np.concatenate([d.fixed["dof"], [16, 16]]),
                   value=np.concatenate([d.fixed["value"], [0.5, -0.25]]))
    path = str(tmp_path / "coupled.hdf5")
    h5model.write_model(path, d, start=10.0, delta=2.5, steps=4, node_order=rng.permutation(d.n_nodes))
    with open(path + ".frq", "w") as fh:
        fh.write("30 20 20 10\n")
    r, freqs = h5model.read_model(path)
    np.testing.assert_array_equal(freqs, [10.0, 20.0, 30.0])
    np.testing.assert_array_equal(r.node_ids, d.node_ids)  # ascending ids, as written before the shuffle
    np.testing.assert_array_equal(r.coords, d.coords)
    assert [(b[0], b[1]) for b in r.blocks] == [(b[0], b[1]) for b in d.blocks]
    for rb, db in zip(r.blocks, d.blocks):
        np.testing.assert_array_equal(rb[2], db[2])
    for rm, dm in zip(r.materials, d.materials):
        for key in ("kind", "nu", "rho", "t", "c"):
            assert rm[key] == pytest.approx(dm.get(key, 0.0)), key
    np.testing.assert_array_equal(r.materials[0]["E_table"], d.materials[0]["E_table"])
    np.testing.assert_array_equal(r.materials[0]["eta_table"], d.materials[0]["eta_table"])
    for key in ("ori", "snodes", "fnodes", "fmat"):
        np.testing.assert_array_equal(r.interfaces[key], d.interfaces[key])
    got = sorted(zip(r.fixed["node"], r.fixed["dof"], r.fixed["value"]))
    exp = sorted(zip(d.fixed["node"], d.fixed["dof"], d.fixed["value"]))
    assert got == exp
    np.testing.assert_array_equal(r.forces["node"], d.forces["node"])
    np.testing.assert_array_equal(r.forces["f"], d.forces["f"])
    np.testing.assert_array_equal(r.moments["node"], d.moments["node"])
    np.testing.assert_array_equal(r.moments["m"], d.moments["m"])
    np.testing.assert_array_equal(r.fluid_sources["node"], d.fluid_sources["node"])
    np.testing.assert_array_equal(r.fluid_sources["p"], d.fluid_sources["p"])
    for key in ("block", "element", "face", "vn"):
        np.testing.assert_array_equal(r.vn_loads[key], d.vn_loads[key])
    # the model built from the file has the same right-hand side and pattern
    m1, m2 = elp.Model(d), elp.Model(r)
    np.testing.assert_array_equal(m1.pattern()[1], m2.pattern()[1])
    np.testing.assert_allclose(m2.rhs(2 * np.pi * 20.0), m1.rhs(2 * np.pi * 20.0), rtol=0, atol=1e-15)


def test_model_file_refuses_face_tractions(meshes, h5model, tmp_path):
    """elpasoC's model file has no structure element loads: writing a model
    with Brick8 face tractions fails instead of dropping them."""
    from test_loads import traction_brick
    with pytest.raises(ValueError):
        h5model.write_model(str(tmp_path / "t.hdf5"), traction_brick(meshes))
    assert not (tmp_path / "t.hdf5").exists()


@pytest.mark.parametrize("version", [1, 3])
def test_enumeration_datatype_message(elp, version):
    """An HDF5 enumeration datatype message (class 8) as the File Format
    Specification lays it out: the 8-byte header (member count in the class
    bits, element size), the base type message, the member names (NUL
    terminated, padded to 8 bytes before version 3), then the member values.
    The {FALSE, TRUE} enum over a signed byte is how booleans are stored."""
    import importlib
    import struct
    h5lite = importlib.import_module("elpaso_core_gb300.h5lite")
    base = bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", 1) + struct.pack("<HH", 0, 8)
    pad = (lambda s: s + b"\0" * (8 - len(s) % 8)) if version < 3 else (lambda s: s + b"\0")
    names = pad(b"FALSE") + pad(b"TRUE")
    msg = bytes([(version << 4) | 8, 2, 0, 0]) + struct.pack("<I", 1) + base + names + bytes([0, 1])
    reader = h5lite.File.__new__(h5lite.File)
    dt, used = reader._datatype(msg + b"\xff" * 5, 0)
    assert used == len(msg)
    assert dt == np.dtype("i1") and dt.metadata["enum"] == {"FALSE": 0, "TRUE": 1}
