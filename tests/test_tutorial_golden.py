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
* the oracle's FP64 solve differs from the reference's by <= 1e-15 kappa_2;
* on the GPU, both precisions converge to 1e-12 and differ from the
  reference's solution by at most the perturbation bound
  kappa_2 (res_ours + res_ref) (+ 1e-13), read back from the solution file
  written in elpasoC's layout (h5model.write_solution).
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
        A = s.matrix(2 * np.pi * f).toarray()
        x = s.solve(2 * np.pi * f)
        err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
        assert err <= 1e-15 * np.linalg.cond(A), (f, err)


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
        err = np.linalg.norm(x[k] - xr) / np.linalg.norm(xr)
        kappa = np.linalg.cond(A.toarray())
        assert err <= 1.01 * kappa * (res + r_ref) + 1e-13, (tut["freqs"][k], err, kappa, res, r_ref)
