"""Cell and nodal stresses after a solve (cAnalysis::computeStressesCells /
computeStressesNodes, analysis.cpp:869-935; Brick8
elementstructurebrick.cpp:48-270, Mindlin/DSG4 elementstructuremindlin.cpp:51-175,
Fluid8 grad p elementfluid3d.cpp:380-557), computed by the library
(`elp_cell_stresses`, `elp_node_stresses`, CUDA kernels) against the
oracle's restatement and against closed forms. The stresses are linear in
the solution, so arbitrary vectors stand in for solutions."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_brick_uniform_strain_closed_form(elp, meshes):
    d = meshes.solid_cube(3, perturb=0.0, n_materials=1)
    m = elp.Model(d)
    rows = m.global_rows()
    a = 1e-4
    x = np.zeros(m.n, complex)
    for v in range(d.n_nodes):  # u1 = a * x: eps_xx = a, all others 0
        if rows[v, 0] >= 0:
            x[rows[v, 0]] = a * d.coords[v, 0]
    up, lo = m.cell_stresses(2 * np.pi * 50.0, x)
    mat = d.materials[0]
    E, nu = mat["E"], mat["nu"]
    f = E / ((1 + nu) * (1 - 2 * nu))
    np.testing.assert_allclose(up[:, 0], f * (1 - nu) * a, rtol=1e-12)
    np.testing.assert_allclose(up[:, 1], f * nu * a, rtol=1e-12)
    np.testing.assert_allclose(up[:, 2], f * nu * a, rtol=1e-12)
    assert np.abs(up[:, 3:]).max() <= 1e-9 * f * a and not lo.any()


def test_plate_rotation_field_closed_form(elp, meshes):
    d = meshes.plate(6, 4, 0.6, 0.4, 0.003)
    m = elp.Model(d)
    rows = m.global_rows()
    b = 2e-3
    x = np.zeros(m.n, complex)
    for v in range(d.n_nodes):  # w2 = b * x: the first strain is b, the others 0
        if rows[v, 4] >= 0:
            x[rows[v, 4]] = b * d.coords[v, 0]
    om = 2 * np.pi * 80.0
    up, lo = m.cell_stresses(om, x)
    mat = d.materials[0]
    t, nu = mat["t"], mat["nu"]
    Ev = mat["E"] * (1 + 1j * mat["eta"]) if mat["kind"] == elp.STR_LIN_VIS_ISO_DIR else mat["E"]
    f = Ev / (1 - nu * nu)
    np.testing.assert_allclose(up[:, 0], f * 0.5 * t * b, rtol=1e-12)
    np.testing.assert_allclose(up[:, 1], f * nu * 0.5 * t * b, rtol=1e-12)
    np.testing.assert_allclose(lo[:, 0], -f * 0.5 * t * b, rtol=1e-12)


@pytest.mark.parametrize("model", ["cube", "plate", "plate_cavity", "visco_tables"])
def test_cell_stresses_match_oracle(elp, meshes, oracle, model):
    if model == "cube":
        d = meshes.solid_cube(4)
    elif model == "plate":
        d = meshes.plate(8, 6, 0.6, 0.4, 0.002)
    elif model == "plate_cavity":
        d = meshes.plate_cavity(6, 4, 3, 0.6, 0.4, 0.3)
    else:
        d = copy.deepcopy(meshes.solid_plate(4, 4, 2))
        d.materials[0].update(E_table=np.array([[50.0, 200e9], [300.0, 180e9]]),
                              eta_table=np.array([[10.0, 0.01], [400.0, 0.04]]))
    m = elp.Model(d)
    s = oracle.System(d)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(m.n) + 1j * rng.standard_normal(m.n)
    om = 2 * np.pi * 137.0
    up, lo = m.cell_stresses(om, x)
    ou, ol = oracle.cell_stresses(s, om, x)
    scale = max(np.abs(ou).max(), 1e-300)
    np.testing.assert_allclose(up, ou, rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose(lo, ol, rtol=0, atol=1e-13 * scale)


@pytest.mark.parametrize("model", ["cube", "plate_cavity"])
def test_node_stresses_match_oracle(elp, meshes, oracle, model):
    d = meshes.solid_cube(4) if model == "cube" else meshes.plate_cavity(6, 4, 3, 0.6, 0.4, 0.3)
    m = elp.Model(d)
    s = oracle.System(d)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(m.n) + 1j * rng.standard_normal(m.n)
    om = 2 * np.pi * 77.0
    got, ref = m.node_stresses(om, x), oracle.node_stresses(s, om, x)
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * scale)


def test_node_pressure_gradient_closed_form(elp, meshes):
    """A linear pressure field has the exact gradient g at every corner; the
    nodal slots sum it over the node's Fluid8 elements."""
    d = meshes.plate_cavity(6, 4, 3, 0.6, 0.4, 0.3)
    m = elp.Model(d)
    rows = m.global_rows()
    g = np.array([3.0, -2.0, 0.5])
    x = np.zeros(m.n, complex)
    for v in range(d.n_nodes):
        if rows[v, 16] >= 0:
            x[rows[v, 16]] = (1 + 2j) * (d.coords[v] @ g)
    out = m.node_stresses(2 * np.pi * 10.0, x)
    fluid = [b for b in d.blocks if b[0] == 3][0][2]
    nfl = np.bincount(np.asarray(fluid).ravel(), minlength=d.n_nodes)
    seq = np.empty(d.n_nodes, np.int64)
    seq[np.argsort(d.node_ids, kind="stable")] = np.arange(d.n_nodes)
    expect = np.zeros((d.n_nodes, 3), complex)
    expect[seq] = nfl[:, None] * (1 + 2j) * g[None, :]
    np.testing.assert_allclose(out[:, 6:], expect, rtol=0, atol=1e-11 * np.abs(expect).max())



def test_node_stresses_are_deterministic(elp, meshes):
    """One thread per node sums its elements in a fixed order (no atomics):
    the same input gives the same bits."""
    d = meshes.plate_cavity(6, 4, 3, 0.6, 0.4, 0.3)
    m = elp.Model(d)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(m.n) + 1j * rng.standard_normal(m.n)
    a, b = m.node_stresses(2 * np.pi * 40.0, x), m.node_stresses(2 * np.pi * 40.0, x)
    np.testing.assert_array_equal(a, b)
