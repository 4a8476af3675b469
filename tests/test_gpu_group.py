"""Groups of models solved together (elp_group_*), against the oracle.

A group is its members' disjoint union: one launch per tree level over the
fronts of all members, each member at its own frequencies. Bars, per member
and frequency, as for single models: ||f - A x||_2 / ||f||_2 <= 1e-10 with
the oracle's matrix of that member, plus the FP64 floor 4 eps || |A| |x| || /
||f|| of measuring it with a matrix summed in another order (1.4e6 eps on the
clamped solid plate at 451 Hz, whose oracle solution itself has residual
1.4e-10), the error against the oracle's FP64 solve within
3 kappa_1(A_ff) (res_1 + res_ref_1), and the reported residual within the
same bar of the one measured here. A group of one model takes the single-model
path and equals the model solved alone up to assembly rounding.
"""
import numpy as np
import pytest

from test_gpu_solve import cond1, residual_floor

pytestmark = pytest.mark.gpu


def _members(meshes):
    return [meshes.plate(12, 9, 0.3, 0.2, 0.002), meshes.plate(30, 22, 0.6, 0.4, 0.003, seed=7),
            meshes.cube(5), meshes.plate_cavity(8, 6, 4, 0.6, 0.4, 0.3), meshes.solid_plate(8, 6, 2)]


@pytest.mark.parametrize("prec", [0, 1])
def test_group_members_match_the_oracle(elp, meshes, oracle, prec):
    ds = _members(meshes)
    g = elp.Group([elp.Model(d) for d in ds])
    rng = np.random.default_rng(31 + prec)
    oms = 2 * np.pi * rng.uniform(5.0, 480.0, size=(len(ds), 4))
    # solved to 5e-11: near a clamped plate's FP64 floor (|| |A| |x| || / ||f|| ~ 1e6) the
    # oracle's own FP64 product measures the residual only to ~1e-10
    xs, infos = g.solve(oms, precision=prec, tol=5e-11)
    for k, d in enumerate(ds):
        s = oracle.System(d)
        for j, om in enumerate(oms[k]):
            A, f = s.matrix(om), s.rhs(om)
            x = xs[k][j]
            res = np.linalg.norm(f - A @ x) / np.linalg.norm(f)
            bar = 1e-10 + residual_floor(A, x, f)
            assert res <= bar, (k, j, res, bar)
            # the library's residual is double-double with its own matrix; this one is plain FP64
            # with the oracle's
            assert abs(infos[k][j]["rel_residual"] - res) <= bar, (k, j, infos[k][j], res)
            assert infos[k][j]["converged"] == 1
            xr = s.solve(om)
            n1 = np.linalg.norm(f, 1)
            res1 = np.linalg.norm(f - A @ x, 1) / n1
            res_ref1 = np.linalg.norm(f - A @ xr, 1) / n1
            err = np.linalg.norm(x - xr, 1) / np.linalg.norm(xr, 1)
            assert err <= max(1e-13, 3.0 * cond1(s.free_block(om)[0]) * (res1 + res_ref1)), (k, j, err)


def test_group_of_one_equals_the_model_alone(elp, meshes):
    """One member takes the single-model path: the same solution as the
    model alone, up to the ~1e-16 differences of two assemblies (FP64 atomic
    additions in another order) carried through one FP64 refinement."""
    d = meshes.plate(16, 12, 0.6, 0.4, 0.002)
    oms = 2 * np.pi * np.array([13.0, 170.0, 333.0])
    xa, _ = elp.Model(d).assemble().analyse().solve(oms, precision=0)
    xg, _ = elp.Group([elp.Model(d)]).solve(oms[None, :], precision=0)
    assert np.max(np.abs(xa - xg[0])) <= 1e-9 * np.max(np.abs(xa))


def test_group_of_many_plates(elp, meshes, oracle):
    """Forty plates of 363-3,468 DOFs, 8 frequencies each: the grouped launch
    covers fronts of many sizes; a sample of members is checked against the
    oracle."""
    ds = meshes.batched_plates(40, lo=10, hi=33)
    g = elp.Group([elp.Model(d) for d in ds])
    rng = np.random.default_rng(4)
    oms = 2 * np.pi * rng.uniform(10.0, 400.0, size=(len(ds), 8))
    xs, infos = g.solve(oms, precision=1, raise_on_noconv=False)
    assert all(i["converged"] == 1 for row in infos for i in row)
    for k in (0, 7, 23, 39):
        s = oracle.System(ds[k])
        for j in (0, 5):
            A, f = s.matrix(oms[k][j]), s.rhs(oms[k][j])
            assert np.linalg.norm(f - A @ xs[k][j]) / np.linalg.norm(f) <= 1e-10


def test_autotune_leaves_a_working_tuning(elp, meshes, oracle):
    """The autotuner times real solves while it varies leaf size, Schur tile,
    packed levels and lanes, keeps the fastest, and leaves the model tuned
    so: the tuning reported is the one in effect, and the next solve meets
    the residual bar against the oracle."""
    d = meshes.plate_cavity(12, 8, 6, 0.6, 0.4, 0.3)
    m = elp.Model(d).assemble().analyse()
    oms = 2 * np.pi * np.array([20.0, 140.0, 333.0, 470.0])
    chosen, sec, trials = m.autotune(oms)
    assert trials >= 5 and sec > 0
    assert chosen["leaf"] in (64, 128, 256) and chosen["schur_tile"] in (32, 64)
    assert m.tuning() == chosen
    x, info = m.solve(oms, precision=1)
    s = oracle.System(d)
    for j, om in enumerate(oms):
        A, f = s.matrix(om), s.rhs(om)
        assert np.linalg.norm(f - A @ x[j]) / np.linalg.norm(f) <= 1e-10


def test_group_autotune(elp, meshes):
    ds = meshes.batched_plates(12, lo=10, hi=30)
    g = elp.Group([elp.Model(d) for d in ds])
    rng = np.random.default_rng(9)
    oms = 2 * np.pi * rng.uniform(10.0, 400.0, size=(len(ds), 16))
    chosen, sec, trials = g.autotune(oms)
    assert trials >= 7 and sec > 0 and chosen["lanes"] in (1, 2, 4)
    xs, infos = g.solve(oms, precision=1)
    assert all(i["rel_residual"] <= 1e-10 for row in infos for i in row)
