"""Per-frequency solve on the GPU (plain FP64 and mixed FP32 fronts + FP64
refinement) against the FP64 direct-solve oracle (SciPy SuperLU on the
oracle's own CSR, Dirichlet columns lifted).

Bars: relative residual ||f - A x||_2 / ||f||_2 <= 1e-10, measured with the
ORACLE's matrix; relative error vs the oracle's solution within what both
residuals allow, in 1-norms ||x - x_ref|| / ||x_ref|| <= kappa_1(A_ff)
(res_1 + res_ref_1) (the perturbation bound on the free block A_ff, the only
part either solution can err in: the boundary rows fix x_c exactly; kappa_1
estimated with onenormest, a lower bound, x 3; thin-hex and near-resonance
systems reach 1e7)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RES_TOL = 1e-10


def cond1(A):
    import scipy.sparse.linalg as sla
    lu = sla.splu(A.tocsc())
    n = A.shape[0]
    inv = sla.LinearOperator((n, n), matvec=lu.solve, rmatvec=lambda b: lu.solve(b, trans="H"), dtype=complex)
    return sla.onenormest(A) * sla.onenormest(inv)


def residual_floor(A, x, f, unit=2.0 ** -53):
    """4 u || |A| |x| || / ||f||: how far ||f - A x|| / ||f|| can move when A's
    entries move by a few units of roundoff u (another summation order of the
    assembly, or the FP64 product that measures it)."""
    return 4.0 * unit * np.linalg.norm(abs(A) @ np.abs(x)) / np.linalg.norm(f)


def check(elp, oracle, d, f_list, prec):
    m = elp.Model(d).assemble().analyse()
    s = oracle.System(d)
    oms = 2 * np.pi * np.asarray(f_list, float)
    x, infos = m.solve(oms, precision=prec)
    for k, om in enumerate(oms):
        A = s.matrix(om)
        f = s.rhs(om)  # F(w): the normal-velocity loads are its 1/w part
        res = np.linalg.norm(f - A @ x[k]) / np.linalg.norm(f)
        xr = s.solve(om)
        n1 = np.linalg.norm(f, 1)
        res1 = np.linalg.norm(f - A @ x[k], 1) / n1
        res_ref1 = np.linalg.norm(f - A @ xr, 1) / n1
        err = np.linalg.norm(x[k] - xr, 1) / np.linalg.norm(xr, 1)
        assert res <= RES_TOL, (k, res)
        bound = 3.0 * cond1(s.free_block(om)[0]) * (res1 + res_ref1)
        assert err <= max(1e-13, bound), (k, err, bound)
        if prec == 1:  # FP32 fronts are a good preconditioner: few GMRES steps
            assert infos[k]["iterations"] <= 24, (k, infos[k]["iterations"])
        assert infos[k]["converged"] == 1
        assert abs(infos[k]["rel_residual"] - res) <= 1e-10
    return m, infos


@pytest.mark.parametrize("prec", [0, 1])
def test_clamped_solid_plate_100hz(elp, meshes, oracle, prec):
    check(elp, oracle, meshes.solid_plate(), [100.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_plate_sweep(elp, meshes, oracle, prec):
    check(elp, oracle, meshes.plate(24, 16, 0.6, 0.4, 0.002), [5.0, 61.0, 233.0, 499.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_plate_cavity_sweep(elp, meshes, oracle, prec):
    check(elp, oracle, meshes.plate_cavity(12, 8, 6, 0.6, 0.4, 0.3), [1.0, 50.0, 173.0, 500.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_cube_user_rhs(elp, meshes, oracle, prec):
    d = meshes.cube(6)
    m = elp.Model(d).assemble().analyse()
    s = oracle.System(d)
    rng = np.random.default_rng(1)
    f = rng.standard_normal(m.n) + 1j * rng.standard_normal(m.n)
    # prescribed values stay zero, as in the model: with nonzero values the BC
    # columns (|a| ~ 1e10) put ||f - A x|| / ||f|| at an FP64 rounding floor
    # near 1e-6 for any solver
    f[np.asarray(s.bc_rows)] = 0.0
    om = 2 * np.pi * 321.0
    x, infos = m.solve([om], precision=prec, f=f)
    A = s.matrix(om)
    assert np.linalg.norm(f - A @ x[0]) / np.linalg.norm(f) <= 1e-10


def test_batch_result_equals_single(elp, meshes):
    d = meshes.plate(20, 14, 0.6, 0.4, 0.002)
    m = elp.Model(d).assemble().analyse()
    oms = 2 * np.pi * np.array([11.0, 97.0, 203.0, 351.0])
    xb, _ = m.solve(oms, precision=1)
    for k, om in enumerate(oms):
        xs, _ = m.solve([om], precision=1)
        assert np.array_equal(xs[0], xb[k])


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("visco_type", [1, 2])
def test_visco_frequency_tables(elp, meshes, oracle, prec, visco_type):
    """E(f) and eta(f) tables (materialstructurevisco.cpp:229-287): the device
    scales the assembled stiffness by E(w)/E_ref (1 + i eta(w)) per w; the
    oracle's matrix takes E_vis(w) per element. Frequencies below, inside and
    above the tables, where the FP64 floor eps || |A| |x| || / ||f|| of this
    plate is at most 4e-11 (at 310-450 Hz it is 1e-10 to 5e-10: no FP64
    solution, the oracle's included, reaches 1e-10 there)."""
    import copy
    d = copy.deepcopy(meshes.solid_plate(10, 10, 2))
    d.materials[0].update(visco_type=visco_type,
                          E_table=np.array([[50.0, 200e9], [150.0, 230e9], [300.0, 180e9]]),
                          eta_table=np.array([[20.0, 0.01], [200.0, 0.05]]) / ([1.0, 1.0] if visco_type == 1 else
                                                                              [1.0, 2 * np.pi * 100.0]))
    check(elp, oracle, d, [10.0, 90.0, 175.0, 700.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_moments_sources_and_normal_velocity_loads(elp, meshes, oracle, prec):
    """Coupled plate-cavity model with nodal moments on the plate, fluid point
    sources and normal-velocity loads on Fluid8 faces (F(w) = F + G / w,
    added per slot on the device), against the oracle's F(w). A source in
    the closed air cavity drives a near-uniform pressure (the null mode of
    K_f), whose FP64 floor eps || |A| |x| || / ||f|| is 1e-9 to 6e-8 at unit
    strength; scaled by 3e-4 (sources) and 3e-3 (vn) the floor is <= 1.1e-11
    while the G / w part is still >= 9e-10 of ||F||, so a wrong or missing
    load fails the 1e-10 residual."""
    from test_loads import loaded_plate_cavity
    d = loaded_plate_cavity(meshes)
    d.fluid_sources["p"] = d.fluid_sources["p"] * 3e-4
    d.vn_loads["vn"] = d.vn_loads["vn"] * 3e-3
    check(elp, oracle, d, [2.0, 61.0, 233.0, 499.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_brick_face_tractions(elp, meshes, oracle, prec):
    """Clamped 20 x 20 x 2 Brick8 plate (the system of the 100 Hz test above)
    with complex constant tractions on 40 random faces besides the centre
    force: the right-hand side built at model creation reaches the solve."""
    from test_loads import traction_brick
    check(elp, oracle, traction_brick(meshes, nx=20, ny=20, count=40), [100.0], prec)


@pytest.mark.parametrize("prec", [0, 1])
def test_double_float_assembled_models_solve(elp, meshes, oracle, prec):
    """Models assembled with the double-float element contractions solve to
    the residual bar against the oracle's FP64 matrix, plus the floor that
    ~2^-46 entry differences allow (4 2^-46 || |A| |x| || / ||f||, below
    1e-11 on these two models)."""
    for d in (meshes.cube(5), meshes.plate_cavity(8, 6, 4, 0.6, 0.4, 0.3)):
        m = elp.Model(d).set_assembly(elp.ASSEMBLY_DOUBLE_FLOAT).assemble().analyse()
        s = oracle.System(d)
        oms = 2 * np.pi * np.array([7.0, 180.0, 455.0])
        x, infos = m.solve(oms, precision=prec)
        for k, om in enumerate(oms):
            A, f = s.matrix(om), s.rhs(om)
            res = np.linalg.norm(f - A @ x[k]) / np.linalg.norm(f)
            assert infos[k]["converged"] == 1
            assert res <= RES_TOL + residual_floor(A, x[k], f, unit=2.0 ** -46), (d.name, k, res)
