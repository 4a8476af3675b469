"""Host-side logic on CPU: the C-ABI library loads and exports every symbol
of include/*.h; DOF numbering, CSR pattern (bit-exact), Dirichlet rows and
the right-hand side agree with the oracle's restatement of the reference.
elp_model_create runs on the host only, so none of this needs a GPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "elpaso_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(elp_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(elp):
    lib = elp.load_library()
    syms = header_symbols()
    assert len(syms) >= 17
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(elp.EXPORTS) == syms


def test_no_gpu_fails_loudly_not_falls_back(elp, meshes):
    import ctypes
    try:
        n = ctypes.c_int()
        have_gpu = ctypes.CDLL("libcudart.so").cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        have_gpu = False
    if have_gpu:
        pytest.skip("a GPU is present")
    m = elp.Model(meshes.solid_plate(4, 4, 1))
    with pytest.raises(elp.ElpasoError):
        m.assemble()


def small_models(meshes):
    return [
        meshes.solid_plate(6, 5, 2),
        meshes.plate(7, 5, 0.3, 0.2, 0.002),
        meshes.plate_cavity(6, 4, 3, 0.3, 0.2, 0.15),
        meshes.solid_cube(4, n_materials=3),
    ]


@pytest.mark.parametrize("k", range(4))
def test_numbering_pattern_bc_rhs_match_oracle(elp, meshes, oracle, k):
    d = small_models(meshes)[k]
    m = elp.Model(d)
    s = oracle.System(d)
    rows = m.global_rows()
    assert np.array_equal(rows, s.rows)
    rp, ci = m.pattern()
    assert np.array_equal(rp, s.row_ptr)
    assert np.array_equal(ci, s.col_idx)
    assert np.array_equal(m.rhs(), s.f)


def test_numbering_follows_node_ids_not_array_order(elp, meshes, oracle):
    d = meshes.plate(5, 4, 0.3, 0.2, 0.002)
    rng = np.random.default_rng(3)
    d.node_ids = rng.permutation(np.arange(100, 100 + d.n_nodes)).astype(np.int64)
    m = elp.Model(d)
    s = oracle.System(d)
    assert np.array_equal(m.global_rows(), s.rows)
    rp, ci = m.pattern()
    assert np.array_equal(ci, s.col_idx)


def test_full_size_plate_cavity_pattern_counts(elp, meshes):
    # the coupled model's size: 7,503 plate + 77,531 fluid dofs
    m = elp.Model(meshes.plate_cavity())
    info = m.info()
    assert info["n_dofs"] == 85034
    rp, ci = m.pattern()
    assert rp[-1] == info["nnz"]
    assert np.all(np.diff(rp) > 0)


def test_malformed_models_are_rejected(elp, meshes):
    d = meshes.plate(3, 3, 0.1, 0.1, 0.002)
    d.blocks = [(d.blocks[0][0], 0, d.blocks[0][2] + 1000)]
    with pytest.raises(elp.ElpasoError) as e:
        elp.Model(d)
    assert e.value.code == 1
    d = meshes.plate(3, 3, 0.1, 0.1, 0.002)
    d.node_ids[1] = d.node_ids[0]
    with pytest.raises(elp.ElpasoError):
        elp.Model(d)
    d = meshes.plate(3, 3, 0.1, 0.1, 0.002)
    d.materials[0]["kind"] = 3  # fluid material on a plate block
    with pytest.raises(elp.ElpasoError):
        elp.Model(d)


def test_pattern_of_nodes_shared_by_element_families_matches_oracle(elp, meshes, oracle):
    """A Brick8 cube whose top face also carries DSG4 plate elements on the
    same nodes: those nodes hold x1 x2 (Brick8 only), x3 (both families) and
    w1 w2 (DSG4 only), so their rows see different element sets (the
    reference's getDofs()-driven pattern, analysis.cpp:815-823). Every row
    must still equal the oracle's."""
    d = meshes.cube(4)
    conn = d.blocks[0][2]
    top = conn[:, 4:8]
    zmax = d.coords[:, 2].max()
    on_top = np.all(np.abs(d.coords[top][:, :, 2] - zmax) < 1e-9, axis=1)
    d.materials.append(dict(kind=meshes.STR_LIN_VIS_ISO_DIR, E=70e9, nu=0.33, rho=2700.0, t=0.002, eta=0.05,
                            visco_type=1))
    d.blocks.append((meshes.DSG4, 1, np.ascontiguousarray(top[on_top])))
    m = elp.Model(d)
    s = oracle.System(d)
    assert np.array_equal(m.global_rows(), s.rows)
    rp, ci = m.pattern()
    assert np.array_equal(rp, s.row_ptr)
    assert np.array_equal(ci, s.col_idx)
    rows = m.global_rows()
    shared = np.unique(top[on_top])
    lens = np.diff(rp)
    x1, x3, w1 = rows[shared, 0], rows[shared, 2], rows[shared, 3]
    assert np.all(w1 >= 0)
    # x1 sees only the bricks, w1 only the plates, x3 both
    assert np.all(lens[x3] > lens[x1]) and np.all(lens[x3] > lens[w1])
