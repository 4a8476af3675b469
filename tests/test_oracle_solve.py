"""The oracle's FP64 direct solve (the reference for every GPU solve test).

The reference's boundary rows are identity rows (MatZeroRows with diagonal 1,
elpasoCore/source/analysis/analysis.cpp:426) while the columns of the fixed
dofs keep their stiffness (~1e11 on a clamped steel plate). The oracle lifts
those columns to the right-hand side before it factors; these checks pin the
lifted solve against a dense solve of the free block, on the clamped thin
plate where SuperLU on the unlifted matrix was off by 3e-4."""
import numpy as np
import pytest


def _free_block_solution(s, omega, f):
    """Dense LAPACK solve of the free block with x_c = f_c."""
    A = s.matrix(omega).toarray()
    bc = np.zeros(s.n, bool)
    bc[s.bc_rows] = True
    x = np.zeros(s.n, np.complex128)
    x[bc] = f[bc]
    fr = ~bc
    x[fr] = np.linalg.solve(A[np.ix_(fr, fr)], f[fr] - A[np.ix_(fr, bc)] @ x[bc])
    return x


@pytest.mark.parametrize("hz", [10.0, 100.0, 850.0])
def test_lifted_solve_matches_free_block(elp, meshes, oracle, hz):
    s = oracle.System(meshes.solid_plate(8, 8, 2))
    om = 2 * np.pi * hz
    x = s.solve(om)
    z = _free_block_solution(s, om, s.f)
    bc = np.asarray(s.bc_rows)
    assert np.array_equal(x[bc], s.f[bc])
    kappa = np.linalg.cond(s.free_block(om)[0].toarray())
    assert kappa < 1e8
    assert np.linalg.norm(x - z) / np.linalg.norm(z) <= 1e-15 * kappa
    A = s.matrix(om)
    assert np.linalg.norm(s.f - A @ x) / np.linalg.norm(s.f) <= 1e-10


def test_lifted_system_keeps_pattern_and_solution(elp, meshes, oracle):
    s = oracle.System(meshes.solid_cube(5))
    om = 2 * np.pi * 321.0
    rng = np.random.default_rng(3)
    f = rng.standard_normal(s.n) + 1j * rng.standard_normal(s.n)
    f[np.asarray(s.bc_rows)] = 1e-3 * (rng.standard_normal(len(s.bc_rows)))  # nonzero prescribed values
    A = s.matrix(om)
    L, rhs = s.lifted(om, f)
    assert np.array_equal(L.indptr, A.indptr) and np.array_equal(L.indices, A.indices)
    bc = np.zeros(s.n, bool)
    bc[s.bc_rows] = True
    rows = np.repeat(np.arange(s.n), np.diff(A.indptr))
    lifted = bc[A.indices] & ~bc[rows]
    assert lifted.any() and np.all(L.data[lifted] == 0) and np.array_equal(L.data[~lifted], A.data[~lifted])
    np.testing.assert_array_equal(rhs[bc], f[bc])
    x = s.solve(om, f)
    z = _free_block_solution(s, om, f)
    assert np.linalg.norm(x - z) / np.linalg.norm(z) <= 1e-12


def test_multifrontal_adjoint_solve_and_condition_estimate(elp, meshes, oracle):
    """solve_h (A^H y = c from the factors of A) against dense LAPACK, and the
    free-block kappa_1 estimate against the dense kappa_1, on a coupled
    plate-cavity system (fluid, coupling and Dirichlet rows all present)."""
    s = oracle.System(meshes.plate_cavity(6, 4, 3, 0.3, 0.2, 0.15))
    om = 2 * np.pi * 120.0
    A, rhs = s.lifted(om)
    mf = oracle.multifrontal(s, leaf=24)
    mf.factor(A)
    rng = np.random.default_rng(5)
    c = rng.standard_normal(s.n) + 1j * rng.standard_normal(s.n)
    Ad = A.toarray()
    nA = np.linalg.norm(Ad, 2)

    def backward_error(M, z):  # normwise: a wrong solve gives O(1), a stable one O(eps)
        return np.linalg.norm(M @ z - c) / (nA * np.linalg.norm(z) + np.linalg.norm(c))

    y = mf.solve_h(c)
    assert backward_error(Ad.conj().T, y) <= 1e-14
    x = mf.solve(c)
    assert backward_error(Ad, x) <= 1e-14
    y_dense = np.linalg.solve(Ad.conj().T, c)
    assert np.linalg.norm(y - y_dense) / np.linalg.norm(y_dense) <= 1e-15 * np.linalg.cond(Ad)
    Aff = s.free_block(om)[0].toarray()
    exact = np.linalg.norm(Aff, 1) * np.linalg.norm(np.linalg.inv(Aff), 1)
    est = oracle.free_block_cond1(s, om, mf)
    assert 0.3 * exact <= est <= exact * (1 + 1e-8), (est, exact)
