"""The oracle's restatement of the stress rules (cAnalysis::computeStressesCells
/ computeStressesNodes, analysis.cpp:869-935) against closed forms, on the
CPU. The library computes the stresses on the device and is held to this
oracle by tests/test_stresses.py; these checks keep the rules themselves
covered where no GPU is present. Arbitrary vectors stand in for solutions
(the stresses are linear in them)."""
import numpy as np


def _rows_of(elp, d):
    """Global rows per node and DOF (-1 inactive), from the host model."""
    return elp.Model(d).global_rows()


def test_oracle_brick_uniform_strain(elp, meshes, oracle):
    d = meshes.solid_cube(3, perturb=0.0, n_materials=1)
    rows = _rows_of(elp, d)
    s = oracle.System(d)
    a = 1e-4
    x = np.zeros(s.n, complex)
    for v in range(d.n_nodes):  # u1 = a * x: eps_xx = a, all others 0
        if rows[v, 0] >= 0:
            x[rows[v, 0]] = a * d.coords[v, 0]
    up, lo = oracle.cell_stresses(s, 2 * np.pi * 50.0, x)
    mat = d.materials[0]
    E, nu = mat["E"], mat["nu"]
    f = E / ((1 + nu) * (1 - 2 * nu))
    np.testing.assert_allclose(up[:, 0], f * (1 - nu) * a, rtol=1e-12)
    np.testing.assert_allclose(up[:, 1], f * nu * a, rtol=1e-12)
    np.testing.assert_allclose(up[:, 2], f * nu * a, rtol=1e-12)
    assert np.abs(up[:, 3:]).max() <= 1e-9 * f * a and not lo.any()


def test_oracle_plate_rotation_field(elp, meshes, oracle):
    d = meshes.plate(6, 4, 0.6, 0.4, 0.003)
    rows = _rows_of(elp, d)
    s = oracle.System(d)
    b = 2e-3
    x = np.zeros(s.n, complex)
    for v in range(d.n_nodes):  # w2 = b * x: the first strain is b, the others 0
        if rows[v, 4] >= 0:
            x[rows[v, 4]] = b * d.coords[v, 0]
    up, lo = oracle.cell_stresses(s, 2 * np.pi * 80.0, x)
    mat = d.materials[0]
    t, nu = mat["t"], mat["nu"]
    Ev = mat["E"] * (1 + 1j * mat["eta"]) if mat["kind"] == elp.STR_LIN_VIS_ISO_DIR else mat["E"]
    f = Ev / (1 - nu * nu)
    np.testing.assert_allclose(up[:, 0], f * 0.5 * t * b, rtol=1e-12)
    np.testing.assert_allclose(up[:, 1], f * nu * 0.5 * t * b, rtol=1e-12)
    np.testing.assert_allclose(lo[:, 0], -f * 0.5 * t * b, rtol=1e-12)


def test_oracle_node_pressure_gradient(elp, meshes, oracle):
    """A linear pressure field has the exact gradient g at every corner; the
    nodal slots sum it over the node's Fluid8 elements."""
    d = meshes.plate_cavity(6, 4, 3, 0.6, 0.4, 0.3)
    rows = _rows_of(elp, d)
    s = oracle.System(d)
    g = np.array([3.0, -2.0, 0.5])
    x = np.zeros(s.n, complex)
    for v in range(d.n_nodes):
        if rows[v, 16] >= 0:
            x[rows[v, 16]] = (1 + 2j) * (d.coords[v] @ g)
    out = oracle.node_stresses(s, 2 * np.pi * 10.0, x)
    fluid = [blk for blk in d.blocks if blk[0] == 3][0][2]
    nfl = np.bincount(np.asarray(fluid).ravel(), minlength=d.n_nodes)
    seq = np.empty(d.n_nodes, np.int64)
    seq[np.argsort(d.node_ids, kind="stable")] = np.arange(d.n_nodes)
    expect = np.zeros((d.n_nodes, 3), complex)
    expect[seq] = nfl[:, None] * (1 + 2j) * g[None, :]
    np.testing.assert_allclose(out[:, 6:], expect, rtol=0, atol=1e-11 * np.abs(expect).max())
