"""Frequency-dependent visco materials and frequency lists (host side, CPU).

The reference reads a visco material's E and eta either as numbers or as
tables of (frequency [Hz], value) rows, interpolates them linearly in w and
holds them constant outside the table (materialstructurevisco.cpp:75-170,
229-287); a run's frequencies come from `<input>.frq` when it exists
(analysisfrequencybasic.cpp:36-72). Checked here: the oracle's restatement of
the table rule on known answers, the isnumber rule that tells a number from
a dataset name, the frequency list, the HDF5 attribute that names a table,
and the C ABI's validation and grouping of tabulated materials. The solves
with tables are checked against the oracle in test_gpu_solve.py.
"""
import copy
import importlib

import numpy as np
import pytest

E_TAB = np.array([[50.0, 200e9], [150.0, 220e9], [300.0, 180e9]])
ETA_TAB = np.array([[0.0, 0.01], [200.0, 0.05]])


@pytest.fixture(scope="module")
def h5model(elp):
    return importlib.import_module("elpaso_core_gb300.h5model")


def test_table_rule_known_answers(oracle):
    w = lambda f: 2 * np.pi * f  # noqa: E731
    assert oracle.table_value(E_TAB, w(10.0)) == 200e9          # below the table: first value
    assert oracle.table_value(E_TAB, w(50.0)) == 200e9          # at the first row
    assert oracle.table_value(E_TAB, w(150.0)) == 220e9         # at an inner row
    assert oracle.table_value(E_TAB, w(300.0)) == 180e9         # at the last row
    assert oracle.table_value(E_TAB, w(900.0)) == 180e9         # above: last value
    assert oracle.table_value(E_TAB, w(100.0)) == pytest.approx(210e9, rel=1e-15)
    assert oracle.table_value(E_TAB, w(250.0)) == pytest.approx(220e9 - 40e9 * 100.0 / 150.0, rel=1e-15)
    m = dict(kind=oracle.VIS, E=1.0, eta=0.5, visco_type=2, E_table=E_TAB, eta_table=ETA_TAB)
    om = w(100.0)
    assert oracle.e_vis(m, om) == pytest.approx(210e9 * (1 + 1j * om * 0.03), rel=1e-14)


def test_isnumber_rule(h5model):
    for s in ("210e9", "-2", "+1.5", "1e-3", "7.E+2", ".5", "3."):
        assert h5model._is_number(s), s
    for s in ("Etable", "1.2.3", "1e3e4", "1-2", "/Materials/E", "nan"):
        assert not h5model._is_number(s), s


def test_frequency_list_from_frq_file(h5model, tmp_path):
    model = str(tmp_path / "model.hdf5")
    np.testing.assert_array_equal(h5model.frequency_list(model, 10.0, 5.0, 4), [10.0, 15.0, 20.0, 25.0])
    with open(model + ".frq", "w") as fh:
        fh.write("300 12.5\n 12.5\t100\n7\n")
    np.testing.assert_array_equal(h5model.frequency_list(model, 10.0, 5.0, 4), [7.0, 12.5, 100.0, 300.0])
    ak3 = str(tmp_path / "plate.ak3")
    with open(str(tmp_path / "plate.frq"), "w") as fh:
        fh.write("1 2 3")
    np.testing.assert_array_equal(h5model.frequency_list(ak3, 0.0, 1.0, 9), [1.0, 2.0, 3.0])
    with open(model + ".frq", "w") as fh:
        fh.write("1 2 x 3")
    with pytest.raises(ValueError):
        h5model.frequency_list(model, 0.0, 1.0, 1)


def test_material_attribute_names_a_table(h5model, tmp_path):
    h5 = h5model.h5lite
    path = str(tmp_path / "mat.hdf5")
    w = h5.Writer(path)
    w.dataset("EofFreq", E_TAB)
    w.group("Materials/visco1")
    w.attr("Materials/visco1", "E", "EofFreq")
    w.attr("Materials/visco1", "eta", "0.02")
    w.close()
    f = h5.File(path)
    a = f["Materials/visco1"].attrs
    E, tab = h5model._num_or_table(f, a, "E")
    assert E == 0.0
    np.testing.assert_array_equal(tab, E_TAB)
    assert h5model._num_or_table(f, a, "eta") == (0.02, None)


def _visco_plate(meshes, **tables):
    d = copy.deepcopy(meshes.solid_plate(6, 6, 2))
    d.materials[0].update(tables)
    return d


def test_tabulated_materials_get_groups_of_their_own(elp, meshes):
    d = _visco_plate(meshes)
    d.materials.append(dict(d.materials[0]))  # same eta, no table: shares the group
    d.blocks.append((d.blocks[0][0], 1, d.blocks[0][2][:3]))
    d.blocks[0] = (d.blocks[0][0], 0, d.blocks[0][2][3:])
    assert elp.Model(d).info()["n_struct_groups"] == 1
    d.materials[1]["E_table"] = E_TAB
    assert elp.Model(d).info()["n_struct_groups"] == 2


@pytest.mark.parametrize("bad", [
    dict(E_table=E_TAB[::-1]),                                  # frequencies not increasing
    dict(eta_table=np.array([[1.0, 0.1], [1.0, 0.2]])),        # repeated frequency
    dict(E_table=np.array([[1.0, np.nan]])),                    # not finite
    dict(kind=1, E_table=E_TAB),                                # elastic material
])
def test_bad_tables_are_rejected(elp, meshes, bad):
    d = _visco_plate(meshes, **bad)
    with pytest.raises(RuntimeError):
        elp.Model(d)


def test_more_loss_factor_groups_than_supported_are_rejected(elp, meshes):
    d = copy.deepcopy(meshes.solid_plate(6, 6, 2))
    conn = d.blocks[0][2]
    base = d.materials[0]
    d.materials = [dict(base, eta=0.01 * (k + 1)) for k in range(9)]
    d.blocks = [(d.blocks[0][0], k, conn[4 * k:4 * k + 4]) for k in range(9)]
    with pytest.raises(RuntimeError):
        elp.Model(d)
    d.materials = d.materials[:8]
    d.blocks = d.blocks[:8]
    assert elp.Model(d).info()["n_struct_groups"] == 8
