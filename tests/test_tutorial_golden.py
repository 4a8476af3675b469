"""End-to-end golden of the DSG4 path: the reference's own tutorial run.

The fixture (tests/golden/tutorial_plate_dsg4.npz, made by
make_tutorial_golden.py from the tutorial's elpasoC input file and the
solution file elpasoC wrote for it with PETSc + MUMPS in FP64) holds a
70-node, 54-element DSG4 aluminium plate, the reference's global-row map and
its solutions at 121 frequencies of the 10..250 Hz sweep. The material has no
damping, so several frequencies sit near resonances (condition numbers up to
6e9).

Checks:
* the global-row numbering equals the reference's mtxDofMap bit for bit;
* the reference's solutions satisfy this build's A(w) u = f to a relative
  residual <= 1e-11 (matrix, BCs and load are the reference's);
* the oracle's FP64 solve and, on the GPU, both precisions (converged to
  1e-12, read back from the solution file written in elpasoC's layout by
  h5model.write_solution) differ from the reference's solution by at most
  the perturbation bound kappa_2(A_ff) (res_ours + res_ref) (+ 1e-13), A_ff
  the free block: every solution, the reference's included, holds the
  prescribed values exactly at the fixed dofs, so only the free part can err.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def tut():
    return np.load(os.path.join(HERE, "golden", "tutorial_plate_dsg4.npz"))


def tutorial_desc(elp, g):
    kind, E, nu, rho, t = g["material"]
    return elp.ModelDesc(
        node_ids=g["node_ids"], coords=g["coords"],
        materials=[dict(kind=int(kind), E=E, nu=nu, rho=rho, t=t)],
        blocks=[(int(g["elem_type"]), 0, g["elem_conn"])],
        fixed=dict(node=g["fixed_node"], dof=g["fixed_dof"], value=g["fixed_value"]),
        forces=dict(node=g["force_node"], f=g["force_f"]), name="tutorial_plate_dsg4")


def _within_bound(system, omega, x, xr):
    """(error, bound) of x against the reference's xr: both hold the
    prescribed values exactly, the free part obeys the perturbation bound."""
    bc = np.asarray(system.bc_rows)
    assert np.array_equal(x[bc], xr[bc]) and np.array_equal(xr[bc], system.f[bc])
    A = system.matrix(omega)
    nf = np.linalg.norm(system.f)
    res = np.linalg.norm(system.f - A @ x) / nf
    res_ref = np.linalg.norm(system.f - A @ xr) / nf
    kappa = np.linalg.cond(system.free_block(omega)[0].toarray())
    err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
    return err, 1.01 * kappa * (res + res_ref) + 1e-13


def _reference_residuals(system, g):
    out = []
    for f, xr in zip(g["freqs"], g["solutions"]):
        A = system.matrix(2 * np.pi * f)
        r = np.linalg.norm(system.f - A @ xr) / np.linalg.norm(system.f)
        out.append((A, r))
    return out


def test_numbering_matches_reference_dof_map(elp, tut):
    d = tutorial_desc(elp, tut)
    assert d.materials[0]["kind"] == elp.STR_LIN_ELA_ISO_DIR and int(tut["elem_type"]) == elp.DSG4
    rows = elp.Model(d).global_rows()
    index = {int(v): i for i, v in enumerate(tut["node_ids"])}
    ours = np.array([rows[index[int(nid)], int(dof)] for nid, dof in tut["dof_map"]])
    np.testing.assert_array_equal(ours, np.arange(len(tut["dof_map"])))


def test_reference_solutions_satisfy_oracle_system(elp, oracle, tut):
    s = oracle.System(tutorial_desc(elp, tut))
    assert s.n == 210
    for f, (A, r) in zip(tut["freqs"], _reference_residuals(s, tut)):
        assert r <= 1e-11, (f, r)


def test_oracle_solve_matches_reference(elp, oracle, tut):
    s = oracle.System(tutorial_desc(elp, tut))
    for f, xr in zip(tut["freqs"], tut["solutions"]):
        err, bound = _within_bound(s, 2 * np.pi * f, s.solve(2 * np.pi * f), xr)
        assert err <= bound, (f, err, bound)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["FP64_PLAIN", "MIXED"])
def test_gpu_solve_matches_reference(elp, oracle, tut, precision, tmp_path):
    import importlib
    h5model = importlib.import_module("elpaso_core_gb300.h5model")
    d = tutorial_desc(elp, tut)
    s = oracle.System(d)
    m = elp.Model(d).assemble().analyse()
    om = 2 * np.pi * tut["freqs"]
    x, info = m.solve(om, precision=getattr(elp, precision), tol=1e-12)
    # through the solution file elpasoC writes (eGenOutput layout) and back
    out = str(tmp_path / "eGenOutput_tutorial.hdf5")
    h5model.write_solution(out, tut["freqs"], x, h5model.dof_map(d.node_ids, m.global_rows()))
    f2, x, dm = h5model.read_solution(out)
    np.testing.assert_array_equal(dm, tut["dof_map"])
    np.testing.assert_allclose(f2, tut["freqs"], rtol=0, atol=1e-6)
    for k, (A, r_ref) in enumerate(_reference_residuals(s, tut)):
        xr = tut["solutions"][k]
        res = np.linalg.norm(s.f - A @ x[k]) / np.linalg.norm(s.f)
        assert info[k]["rel_residual"] <= 1e-12 and res <= 1e-11, (tut["freqs"][k], info[k], res)
        err, bound = _within_bound(s, om[k], x[k], xr)
        assert err <= bound, (tut["freqs"][k], err, bound, res, r_ref)
