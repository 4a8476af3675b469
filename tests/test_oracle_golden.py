"""The oracle's element restatement against the reference's own element code
(golden vectors produced by oracle/_ref from the reference sources) and
against the known answers of the reference's unit tests."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

TOL = 1e-13  # normwise relative: |A - B|_max / |B|_max


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_shape_tables_match_reference(oracle, golden):
    import ctypes as C
    hx = np.zeros(256)
    qd = np.zeros(48)
    oracle.lib().orc_shape_tables(hx.ctypes.data_as(C.c_void_p), qd.ctypes.data_as(C.c_void_p))
    assert np.array_equal(hx, golden["shape_hex8"])
    assert np.array_equal(qd, golden["shape_quad4"])
    ka = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))
    # the reference test reads cArray3d's storage: index = gp * 32 + deriv * 8 + node
    # (elpasoCore/source/misc/array3d.h:55-57)
    ref = np.array(ka["shape_hex8"]["values"])
    mine = hx.reshape(4, 8, 8).transpose(2, 0, 1).ravel()
    assert np.max(np.abs(mine - ref)) < ka["shape_hex8"]["tol"]


def test_visco_material_known_answers(oracle):
    import ctypes as C
    ka = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))["visco"]
    E = ka["E"] * (1 + 1j * ka["eta"])
    assert E == complex(*ka["E_vis"])
    C6 = np.zeros(72); Cb = np.zeros(18); Cs = np.zeros(8)
    oracle.lib().orc_material(C.c_double(E.real), C.c_double(E.imag), C.c_double(ka["nu"]), C.c_double(ka["t"]),
                              C6.ctypes.data_as(C.c_void_p), Cb.ctypes.data_as(C.c_void_p), Cs.ctypes.data_as(C.c_void_p))
    cs00 = complex(Cs[0], Cs[1])
    cb00 = complex(Cb[0], Cb[1])
    assert abs(cs00 - complex(*ka["Cs00"])) <= 1e-12 * abs(cs00)
    assert abs(cb00 - complex(*ka["Cb00"])) <= 1e-6


@pytest.mark.parametrize("i", range(8))
def test_brick8_matches_reference(oracle, golden, i):
    x = golden["brick_xyz"][i]
    mk, E, nu, rho, eta, vt, om = golden["brick_mat"][i]
    mat = dict(kind=2 if mk == 1 else 1, E=E, eta=eta, visco_type=int(vt))
    K, M, EM = oracle.brick8(x, oracle.e_vis(mat, om), nu, rho, om)
    assert rel(K, golden["brick_K"][i]) < TOL
    assert rel(M, golden["brick_M"][i]) < TOL
    assert rel(EM, golden["brick_EM"][i]) < TOL


@pytest.mark.parametrize("i", range(7))
def test_dsg4_matches_reference(oracle, golden, i):
    x = golden["plate_xyz"][i]
    mk, E, nu, rho, t, eta, vt, om = golden["plate_mat"][i]
    mat = dict(kind=2 if mk == 1 else 1, E=E, eta=eta, visco_type=int(vt))
    K, M, EM, rc = oracle.dsg4(x, oracle.e_vis(mat, om), nu, rho, t, om)
    assert rc == 0
    assert rel(K, golden["plate_K"][i]) < TOL
    assert rel(M, golden["plate_M"][i]) < TOL
    assert rel(EM, golden["plate_EM"][i]) < TOL


@pytest.mark.parametrize("i", range(8))
def test_fluid8_matches_reference(oracle, golden, i):
    c, rho, om = golden["fluid_mat"][i]
    K, M, EM = oracle.fluid8(golden["fluid_xyz"][i], c, rho, om)
    assert rel(K, golden["fluid_K"][i]) < TOL
    assert rel(M, golden["fluid_M"][i]) < TOL
    assert rel(EM, golden["fluid_EM"][i]) < TOL


@pytest.mark.parametrize("i", range(7))
def test_interface_matches_reference(oracle, golden, i):
    Cm = oracle.interface_mindlin(golden["iface_xyz"][i])
    assert rel(Cm, golden["iface_C"][i]) < TOL


def test_dsg4_edge_quirk_is_in_the_fixture(golden):
    # the last quad's longest edge is 3-0, which the reference does not measure
    x = golden["plate_xyz"][6]
    e = [np.linalg.norm(x[(k + 1) % 4] - x[k]) for k in range(4)]
    assert np.argmax(e) == 3
