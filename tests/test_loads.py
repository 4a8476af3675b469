"""Nodal moments, fluid point sources, normal-velocity face loads and Brick8
face tractions (CPU).

The reference adds nodal moments on the active rotations w1 w2 w3
(analysis.cpp:281-364) and fluid point sources as 4 pi p on the fluid row
(analysis.cpp:243-265); a normal-velocity load vn on a Fluid8 face adds
-(i vn / w) int N_z dA at the face's nodes (elementfluid3d.cpp:241-309, the
surface integral of :169-233), so F(w) = F + G / w. Checked here: the face
integral on known geometry, the model's F and F(w) against the oracle's
restatement on a coupled plate-cavity model, and the rejection of bad loads.
The solves with these loads are checked in test_gpu_solve.py.
"""
import copy

import numpy as np
import pytest


def test_face_integrals_known_answers(oracle):
    h = 0.3
    sq = np.array([[0, 0, 0], [h, 0, 0], [h, h, 0], [0, h, 0]], float)
    np.testing.assert_allclose(oracle.face_integrals(sq), np.full(4, h * h / 4), rtol=1e-15)
    par = np.array([[0, 0, 1], [2, 0, 1], [3, 1, 1], [1, 1, 1]], float)  # parallelogram, area 2
    assert oracle.face_integrals(par).sum() == pytest.approx(2.0, rel=1e-15)
    tilted = sq @ np.array([[1, 0, 0], [0, 0.6, 0.8], [0, -0.8, 0.6]])  # rotated: same integrals
    np.testing.assert_allclose(oracle.face_integrals(tilted), np.full(4, h * h / 4), rtol=1e-14)


def loaded_plate_cavity(meshes, seed=3):
    d = copy.deepcopy(meshes.plate_cavity(10, 8, 6, 0.6, 0.4, 0.3))
    rng = np.random.default_rng(seed)
    plate_nodes = np.unique(np.concatenate([np.asarray(b[2]).ravel() for b in d.blocks if b[0] == 2]))
    fb = [k for k, b in enumerate(d.blocks) if b[0] == 3][0]
    fconn = np.asarray(d.blocks[fb][2])
    fluid_nodes = np.unique(fconn.ravel())
    mn = rng.choice(plate_nodes, 5, replace=False)
    d.moments = dict(node=mn, m=rng.standard_normal((5, 3)))
    sn = rng.choice(fluid_nodes, 3, replace=False)
    d.fluid_sources = dict(node=sn, p=rng.standard_normal(3))
    el = rng.choice(len(fconn), 6, replace=False)
    d.vn_loads = dict(block=np.full(6, fb), element=el, face=rng.integers(1, 7, 6), vn=rng.standard_normal(6))
    return d


def test_rhs_with_loads_matches_oracle(elp, meshes, oracle):
    d = loaded_plate_cavity(meshes)
    m = elp.Model(d)
    s = oracle.System(d)
    f = m.rhs()
    assert np.abs(s.f_vn).max() > 0
    np.testing.assert_allclose(f, s.f, rtol=0, atol=1e-14 * np.abs(s.f).max())
    for hz in (3.0, 120.0, 480.0):
        om = 2 * np.pi * hz
        fo = s.rhs(om)
        np.testing.assert_allclose(m.rhs(om), fo, rtol=0, atol=1e-14 * np.abs(fo).max())
    # the moments land on rotation rows only, the sources and vn loads on fluid rows only
    rows = m.global_rows()
    for v in d.moments["node"]:
        assert all(f[rows[v, k]] != 0 for k in (3, 4) if rows[v, k] >= 0)


@pytest.mark.parametrize("bad", [
    dict(block=0),          # a DSG4 block
    dict(face=0),
    dict(face=7),
    dict(element=10 ** 6),
    dict(vn=np.nan),
])
def test_bad_normal_velocity_loads_are_rejected(elp, meshes, bad):
    d = loaded_plate_cavity(meshes)
    for k, v in bad.items():
        a = np.array(d.vn_loads[k], dtype=float if k == "vn" else np.int64)
        a[0] = v
        d.vn_loads[k] = a
    with pytest.raises(RuntimeError):
        elp.Model(d)


# ---------------------------------------------------------------- Brick8 face tractions
# A constant traction t on a Brick8 face adds sum_s C(z, s) t_d to u_d of the
# face's nodes, C(z, s) = int N_z N_s dA (elementstructurebrick.cpp:556-662);
# it does not depend on w and is added before the nodal loads.

def test_face_matrix_known_answers(oracle):
    h = 0.3
    sq = np.array([[0, 0, 0], [h, 0, 0], [h, h, 0], [0, h, 0]], float)
    lumped = np.array([[4, 2, 1, 2], [2, 4, 2, 1], [1, 2, 4, 2], [2, 1, 2, 4]], float) * h * h / 36
    np.testing.assert_allclose(oracle.face_matrix(sq), lumped, rtol=1e-14)  # exact for a bilinear square
    par = np.array([[0, 0, 1], [2, 0, 1], [3, 1, 1], [1, 1, 1]], float)
    np.testing.assert_allclose(oracle.face_matrix(par).sum(1), oracle.face_integrals(par), rtol=1e-14)


def traction_brick(meshes, nx=6, ny=5, seed=7, count=8):
    """Clamped solid plate with complex tractions on random faces of random
    Brick8 elements, besides its centre force."""
    d = copy.deepcopy(meshes.solid_plate(nx, ny, 2))
    rng = np.random.default_rng(seed)
    el = rng.choice(len(d.blocks[0][2]), count, replace=False)
    scale = 1.0 / (d.coords[1, 0] - d.coords[0, 0]) ** 2  # ~1 N on a top face
    d.face_tractions = dict(block=np.zeros(count, np.int64), element=el, face=rng.integers(1, 7, count),
                            t=scale * (rng.standard_normal((count, 3)) + 1j * rng.standard_normal((count, 3))))
    return d


def test_face_tractions_match_oracle(elp, meshes, oracle):
    d = traction_brick(meshes)
    m = elp.Model(d)
    s = oracle.System(d)
    f = m.rhs()
    free = np.ones(m.n, bool)
    free[s.bc_rows] = False
    assert np.abs(f[free]).sum() > 2 * np.abs(d.forces["f"]).sum()  # the tractions are there
    np.testing.assert_allclose(f, s.f, rtol=0, atol=1e-14 * np.abs(s.f).max())
    np.testing.assert_array_equal(m.rhs(2 * np.pi * 50.0), f)  # no 1/w part


def test_uniform_traction_total_force(elp, meshes):
    """A uniform traction on the whole top surface of an unconstrained plate:
    each component's rows sum to t_d x area, and a top node inside the
    surface gets t_d h_x h_y (four faces, h_x h_y / 4 each)."""
    nx, ny, nz, lx, ly = 6, 5, 2, 0.6, 0.5
    d = copy.deepcopy(meshes.solid_plate(nx, ny, nz, lx, ly, 0.02))
    d.fixed, d.forces = None, None
    top = np.arange(nx * ny * (nz - 1), nx * ny * nz)  # the last layer of elements
    t = np.array([1 + 2j, -3.0, 0.5j])
    d.face_tractions = dict(block=np.zeros(len(top), np.int64), element=top, face=np.full(len(top), 5),
                            t=np.tile(t, (len(top), 1)))
    m = elp.Model(d)
    f = m.rhs()
    rows = m.global_rows()
    for k in range(3):
        assert f[rows[:, k]].sum() == pytest.approx(t[k] * lx * ly, rel=1e-13)
    v = int(np.argmin(np.sum((d.coords - np.array([0.3, 0.2, 0.02])) ** 2, axis=1)))
    np.testing.assert_allclose(f[rows[v, :3]], t * (lx / nx) * (ly / ny), rtol=1e-13)
    bottom = np.abs(d.coords[:, 2]) < 1e-12
    assert not f[rows[bottom, :3].ravel()].any()


@pytest.mark.parametrize("bad", [
    dict(block=1),          # no such block
    dict(face=0),
    dict(face=7),
    dict(element=10 ** 6),
    dict(t=np.nan),
])
def test_bad_face_tractions_are_rejected(elp, meshes, bad):
    d = traction_brick(meshes)
    for k, v in bad.items():
        a = np.array(d.face_tractions[k], dtype=complex if k == "t" else np.int64)
        a[0] = v
        d.face_tractions[k] = a
    with pytest.raises(RuntimeError):
        elp.Model(d)


@pytest.mark.parametrize("kind", [2, 3])  # DSG4, Fluid8
def test_face_traction_needs_a_brick8_block(elp, meshes, kind):
    d = copy.deepcopy(meshes.plate_cavity(4, 3, 2, 0.6, 0.4, 0.3))
    b = [k for k, blk in enumerate(d.blocks) if blk[0] == kind][0]
    d.face_tractions = dict(block=np.array([b]), element=np.array([0]), face=np.array([5]),
                            t=np.array([[1.0, 0.0, 0.0]]))
    with pytest.raises(RuntimeError):
        elp.Model(d)
