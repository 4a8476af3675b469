"""Parity at the benchmark's own workload: the coupled plate-cavity model at
full size (60 x 40 DSG4 aluminium plate on a 60 x 40 x 30 Fluid8 air cavity,
n = 85,034), against the oracle's FP64 direct solve.

Frequencies: 1 Hz (the cavity's stiff low end), 44 Hz (next to the plate's
first simply supported mode, f_11 ~ 44 Hz for a 0.6 x 0.4 x 0.002 m plate),
250 Hz and 500 Hz, in both precisions. The oracle factors the lifted system
with its CPU multifrontal LU (oracle/mf.py, tree-parallel; SuperLU at this
size takes minutes per frequency) and estimates kappa_1 of the free block
with Hager / Higham's estimator from the same factors (solve and adjoint
solve). Bars, as for the smaller solve tests:
  ||f - A x||_2 / ||f||_2 <= 1e-10 with the oracle's matrix, and
  ||x - x_ref||_1 / ||x_ref||_1 <= 3 kappa_1(A_ff) (res_1 + res_ref_1).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FREQS_HZ = [1.0, 44.0, 250.0, 500.0]


def test_headline_plate_cavity_against_fp64_oracle(elp, meshes, oracle):
    d = meshes.plate_cavity()
    m = elp.Model(d).assemble().analyse()
    assert m.n == 85_034
    s = oracle.System(d)
    oms = 2 * np.pi * np.asarray(FREQS_HZ)
    xs = {}
    for prec in (elp.FP64_PLAIN, elp.MIXED):
        x, infos = m.solve(oms, precision=prec)
        assert all(i["converged"] == 1 for i in infos)
        xs[prec] = x
    mf = oracle.multifrontal(s)
    report = []
    for k, om in enumerate(oms):
        A = s.matrix(om)
        f = s.rhs(om)
        Al, rl = s.lifted(om)
        mf.factor(Al)
        xr = mf.solve(rl)
        n1 = np.linalg.norm(f, 1)
        res_ref1 = np.linalg.norm(f - A @ xr, 1) / n1
        kappa = oracle.free_block_cond1(s, om, mf)
        for prec, x in xs.items():
            res = np.linalg.norm(f - A @ x[k]) / np.linalg.norm(f)
            res1 = np.linalg.norm(f - A @ x[k], 1) / n1
            err = np.linalg.norm(x[k] - xr, 1) / np.linalg.norm(xr, 1)
            bound = 3.0 * kappa * (res1 + res_ref1)
            report.append((FREQS_HZ[k], prec, res, err, bound))
            assert res <= 1e-10, report[-1]
            assert err <= max(1e-13, bound), report[-1]
    for r in report:
        print("plate_cavity %5.0f Hz precision %d: residual %.2e, error vs FP64 oracle %.2e (bound %.1e)" % r)
