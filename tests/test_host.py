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
