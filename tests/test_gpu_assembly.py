"""K1 assembly on the GPU against the oracle (whose element code is pinned to
the reference's): A(w) after BC rows on the shared pattern.

Tolerance: per row, max_j |A_ij - B_ij| <= 1e-12 * max_j |B_ij| (normwise
relative per row; entries that cancel to ~0 are measured against their row)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def row_rel(rp, a, b):
    worst = 0.0
    for i in range(len(rp) - 1):
        sa, sb = a[rp[i]:rp[i + 1]], b[rp[i]:rp[i + 1]]
        den = np.max(np.abs(sb))
        if den == 0:
            assert np.max(np.abs(sa)) == 0
            continue
        worst = max(worst, np.max(np.abs(sa - sb)) / den)
    return worst


def models(meshes):
    return {
        "solid_plate": meshes.solid_plate(6, 5, 2),
        "plate": meshes.plate(7, 5, 0.3, 0.2, 0.002),
        "plate_cavity": meshes.plate_cavity(6, 4, 3, 0.3, 0.2, 0.15),
        "solid_cube_3mat": meshes.solid_cube(4, n_materials=3),
    }


@pytest.mark.parametrize("name", ["solid_plate", "plate", "plate_cavity", "solid_cube_3mat"])
@pytest.mark.parametrize("f_hz", [1.0, 100.0, 437.0])
def test_system_values_match_oracle(elp, meshes, oracle, name, f_hz):
    d = models(meshes)[name]
    m = elp.Model(d).assemble()
    om = 2 * np.pi * f_hz
    a = m.system_values(om)
    s = oracle.System(d)
    b = s.values(om)
    assert row_rel(s.row_ptr, a, b) <= TOL


def test_visco_type2_and_mixed_groups(elp, meshes, oracle):
    d = meshes.solid_plate(4, 3, 2)
    d.materials = [dict(kind=2, E=200e9, nu=0.3, rho=7800.0, eta=0.003, visco_type=2),
                   dict(kind=2, E=70e9, nu=0.33, rho=2700.0, eta=0.02, visco_type=1),
                   dict(kind=1, E=110e9, nu=0.34, rho=8900.0)]
    conn = d.blocks[0][2]
    d.blocks = [(1, i % 3, conn[i::3]) for i in range(3)]
    m = elp.Model(d).assemble()
    assert m.info()["n_struct_groups"] == 3
    s = oracle.System(d)
    for f_hz in (3.0, 250.0):
        om = 2 * np.pi * f_hz
        assert row_rel(s.row_ptr, m.system_values(om), s.values(om)) <= TOL


def test_assembly_is_deterministic_in_pattern_and_close_in_values(elp, meshes):
    d = meshes.solid_cube(6)
    m = elp.Model(d).assemble()
    a = m.system_values(2 * np.pi * 10)
    m.assemble()
    b = m.system_values(2 * np.pi * 10)
    rp, _ = m.pattern()
    assert row_rel(rp, a, b) <= 1e-14


def test_full_size_clamped_plate_matches_oracle(elp, meshes, oracle):
    d = meshes.solid_plate()   # 20 x 20 x 2 Brick8, n = 3,969
    m = elp.Model(d).assemble()
    s = oracle.System(d)
    assert m.info()["n_dofs"] == 3969 and m.info()["nnz"] == 234423
    om = 2 * np.pi * 100.0
    assert row_rel(s.row_ptr, m.system_values(om), s.values(om)) <= TOL


@pytest.mark.parametrize("name", ["solid_plate", "plate_cavity", "solid_cube_3mat"])
def test_double_float_assembly_matches_oracle(elp, meshes, oracle, name):
    """ELP_ASSEMBLY_DOUBLE_FLOAT: Brick8 / Fluid8 contractions in FP32 pairs.
    The same 1e-12 per-row bar against the oracle; the values are not the
    FP64 assembly's bits (the other arithmetic ran) but within 1e-13 per row
    of them."""
    d = models(meshes)[name]
    m64 = elp.Model(d).assemble()
    mdf = elp.Model(d).set_assembly(elp.ASSEMBLY_DOUBLE_FLOAT).assemble()
    s = oracle.System(d)
    for f_hz in (1.0, 437.0):
        om = 2 * np.pi * f_hz
        a = mdf.system_values(om)
        assert row_rel(s.row_ptr, a, s.values(om)) <= TOL
        b = m64.system_values(om)
        assert row_rel(s.row_ptr, a, b) <= 1e-13
        assert np.any(a != b)


def test_set_assembly_on_an_assembled_model_assembles_again(elp, meshes):
    d = meshes.solid_cube(3, n_materials=2)
    m = elp.Model(d).assemble()
    a64 = m.system_values(2 * np.pi * 50.0)
    m.set_assembly(elp.ASSEMBLY_DOUBLE_FLOAT)
    adf = m.system_values(2 * np.pi * 50.0)
    m.set_assembly(elp.ASSEMBLY_FP64)
    assert np.any(adf != a64)
    assert row_rel(m.pattern()[0], m.system_values(2 * np.pi * 50.0), a64) <= 1e-15
    with pytest.raises(elp.ElpasoError):
        m.set_assembly(7)
