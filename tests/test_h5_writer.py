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
