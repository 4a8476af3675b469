"""Nodal moments, fluid point sources and normal-velocity face loads (CPU).

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
