"""Parity at the assembly workload's full size: the 100^3 Brick8 cube
(1,030,301 nodes, n = 3,090,903, nnz = 245,438,109; interior nodes perturbed
by up to 10% of the spacing, 4 random materials, seeded).

The oracle's full pattern builder (one Python set per row) cannot hold 245M
nonzeros, so the oracle restates the rule per row for a seeded sample of
rows (oracle.sample_rows: the union of the DOF blocks of the elements at the
row's node, the diagonal always in) and assembles exactly those rows with its
C element loop (orc_assemble_rows). The restatement is first checked against
the full System on small models. Bars: pattern rows bit-exact, numbering
bit-exact for every node, nnz equal to the count 9 * 301^3 derived from the
pattern rule; A(w) within 1e-12 per row (max-norm relative to the row) on
>= 10k sampled rows.
"""
import numpy as np
import pytest

SAMPLE_ROWS = 12_000


def _row_rel(a, b, ptr):
    worst = 0.0
    for k in range(len(ptr) - 1):
        sa, sb = a[ptr[k]:ptr[k + 1]], b[ptr[k]:ptr[k + 1]]
        den = np.max(np.abs(sb))
        worst = max(worst, np.max(np.abs(sa - sb)) / den if den else np.max(np.abs(sa)))
    return worst


@pytest.mark.parametrize("name", ["solid_cube", "plate", "solid_plate"])
def test_row_sample_restatement_matches_full_system(elp, meshes, oracle, name):
    d = {"solid_cube": meshes.solid_cube(5, n_materials=3), "plate": meshes.plate(7, 5, 0.3, 0.2, 0.002),
         "solid_plate": meshes.solid_plate(6, 5, 2)}[name]
    s = oracle.System(d)
    rows, n = oracle.numbering(d)
    assert n == s.n and np.array_equal(rows, s.rows)
    rng = np.random.default_rng(3)
    sample = np.sort(rng.choice(s.n, size=min(40, s.n), replace=False))
    om = 2 * np.pi * 130.0
    smp, ptr, cols, vals = oracle.sample_rows(d, sample, om)
    full = s.values(om)
    for k, i in enumerate(smp):
        assert np.array_equal(cols[ptr[k]:ptr[k + 1]], s.col_idx[s.row_ptr[i]:s.row_ptr[i + 1]])
        assert np.array_equal(vals[ptr[k]:ptr[k + 1]], full[s.row_ptr[i]:s.row_ptr[i + 1]])


@pytest.fixture(scope="module")
def cube100(elp, meshes, oracle):
    d = meshes.solid_cube(100)
    m = elp.Model(d)
    rng = np.random.default_rng(20260101 + 100)
    info = m.info()
    sample = np.sort(rng.choice(info["n_dofs"], size=SAMPLE_ROWS, replace=False))
    return d, m, sample


def test_cube100_numbering_and_pattern_rows(elp, oracle, cube100):
    d, m, sample = cube100
    info = m.info()
    assert info["n_dofs"] == 3_090_903 and info["nnz"] == 9 * 301 ** 3 == 245_438_109
    rows, n = oracle.numbering(d)
    assert n == info["n_dofs"]
    assert np.array_equal(m.global_rows(), rows.astype(np.int32))
    rp, ci = m.pattern()
    assert rp[0] == 0 and rp[-1] == info["nnz"] and np.all(np.diff(rp) > 0)
    smp, ptr, cols, _ = oracle.sample_rows(d, sample, 2 * np.pi * 10.0)
    for k, i in enumerate(smp):
        assert np.array_equal(ci[rp[i]:rp[i + 1]], cols[ptr[k]:ptr[k + 1]]), i


@pytest.mark.gpu
@pytest.mark.parametrize("f_hz", [1.0, 437.0])
def test_cube100_values_on_sampled_rows(elp, oracle, cube100, f_hz):
    d, m, sample = cube100
    m.assemble()
    om = 2 * np.pi * f_hz
    a = m.system_values(om)
    rp, _ = m.pattern()
    smp, ptr, cols, vals = oracle.sample_rows(d, sample, om)
    got = np.concatenate([a[rp[i]:rp[i + 1]] for i in smp])
    assert len(got) == len(vals)
    assert _row_rel(got, vals, ptr) <= 1e-12
