"""Host symbolic phase (nested dissection + multifrontal fronts, the part of
`elp_model_analyse` that replaces MUMPS's analysis behind
initializeSolverObjects, analysis.cpp:1071-1226) on edge-case models. It runs
on the host before the device step, so these run without a GPU: analyse
either succeeds (GPU present) or fails with the no-device status, and the
front statistics are there in both cases.

Invariants: one element is one dense front (m^2 entries, sum over the
pivots of 8 r (r + 1) = 8 (m - 1) m (m + 1) / 3 real flops of a complex LU);
two identical disconnected bodies give exactly twice the fronts, entries and
flops; nodes without elements add no DOFs; the analysis is deterministic."""
import copy

import numpy as np
import pytest


def analysed(elp, d):
    m = elp.Model(d)
    try:
        m.analyse()
    except elp.ElpasoError as e:
        assert e.code == 2, e  # no device: the host phase ran
    return m, m.info()


def lu_flops(m):
    return 8.0 * (m - 1) * m * (m + 1) / 3.0


def test_one_element_is_one_dense_front(elp, meshes):
    for d, nd in ((meshes.solid_cube(1, perturb=0.0, n_materials=1), 24), (meshes.plate(2, 2, 0.1, 0.1, 0.002), 27)):
        m, i = analysed(elp, d)
        assert m.n == nd
        assert (i["n_fronts"], i["n_levels"], i["max_front"]) == (1, 1, nd)
        assert i["factor_entries"] == nd * nd
        assert i["factor_flops"] == lu_flops(nd)
        assert i["gemm_flops"] == 0.0  # a single panel sweep has no trailing rows


def two_bodies(a, shift=3.0):
    d = copy.deepcopy(a)
    n0 = len(a.node_ids)
    d.node_ids = np.concatenate([a.node_ids, a.node_ids + 10 ** 6])
    d.coords = np.vstack([a.coords, a.coords + [shift, 0.0, 0.0]])
    d.blocks = [(t, mat, np.vstack([c, c + n0])) for t, mat, c in a.blocks]
    d.fixed = {k: np.concatenate([a.fixed[k], a.fixed[k] + (n0 if k == "node" else 0)]) for k in ("node", "dof")}
    d.fixed["value"] = np.concatenate([a.fixed["value"], a.fixed["value"]])
    return d


@pytest.mark.parametrize("n", [2, 5])
def test_disconnected_bodies_double_everything(elp, meshes, n):
    a = meshes.solid_cube(n, perturb=0.0, n_materials=1)
    _, i1 = analysed(elp, a)
    m2, i2 = analysed(elp, two_bodies(a))
    assert m2.n == 2 * i1["n_dofs"]
    assert i2["n_fronts"] == 2 * i1["n_fronts"]
    assert i2["factor_entries"] == 2 * i1["factor_entries"]
    assert i2["factor_flops"] == pytest.approx(2 * i1["factor_flops"], rel=1e-15)
    assert i2["max_front"] == i1["max_front"]


def test_nodes_without_elements_add_nothing(elp, meshes):
    a = meshes.solid_cube(3, perturb=0.0, n_materials=1)
    d = copy.deepcopy(a)
    d.node_ids = np.concatenate([a.node_ids, [10 ** 7, 10 ** 7 + 1]])
    d.coords = np.vstack([a.coords, [[5.0, 5.0, 5.0], [6.0, 6.0, 6.0]]])
    _, i1 = analysed(elp, a)
    m, i2 = analysed(elp, d)
    assert not (m.global_rows()[-2:] >= 0).any()
    for k in ("n_dofs", "nnz", "n_fronts", "factor_entries", "factor_flops", "max_front"):
        assert i1[k] == i2[k], k


def test_every_dof_fixed_and_no_elements(elp, meshes):
    d = copy.deepcopy(meshes.solid_cube(2, perturb=0.0, n_materials=1))
    N = len(d.node_ids)
    d.fixed = dict(node=np.repeat(np.arange(N), 3), dof=np.tile([0, 1, 2], N), value=np.ones(3 * N, complex))
    d.forces = None
    m, i = analysed(elp, d)  # identity rows everywhere: still one valid front tree
    assert i["n_fronts"] >= 1 and i["factor_entries"] >= i["nnz"]
    np.testing.assert_array_equal(m.rhs(), np.ones(m.n))
    d.blocks, d.fixed = [], None
    with pytest.raises(elp.ElpasoError) as e:
        elp.Model(d)
    assert e.value.code == 1


@pytest.mark.parametrize("make", ["plate_cavity", "thin_strip", "fluid_only"])
def test_front_statistics_are_consistent_and_deterministic(elp, meshes, make):
    if make == "plate_cavity":
        d = meshes.plate_cavity(10, 8, 6, 0.6, 0.4, 0.3)
    elif make == "thin_strip":
        d = meshes.solid_plate(40, 1, 1, 4.0, 0.1, 0.1)
    else:
        d = copy.deepcopy(meshes.plate_cavity(6, 4, 4, 0.3, 0.2, 0.2))
        d.blocks = [b for b in d.blocks if b[0] == 3]
        d.interfaces, d.fixed, d.forces = None, None, None
    _, i = analysed(elp, d)
    n = i["n_dofs"]
    assert 1 <= i["max_front"] <= n
    assert i["factor_entries"] >= i["nnz"]  # every stored entry lives in some front
    assert 0 < i["factor_flops"] <= lu_flops(n)  # never worse than dense
    assert i["n_levels"] >= (2 if i["n_fronts"] > 1 else 1)
    _, again = analysed(elp, d)
    assert again == i


@pytest.mark.parametrize("name", ["plate_cavity", "cube", "solid_cube", "plate", "two_plates"])
def test_factor_store_and_front_pool_sizes(elp, meshes, name):
    """Factor-only storage: the factors kept are sum p^2 + 2 p b, and the
    pool of full fronts (first-fit regions, checked disjoint per level by
    the symbolic phase itself) holds at least the most fronts alive at once
    and at most every front at once."""
    d = {"plate_cavity": meshes.plate_cavity(16, 12, 8, 0.6, 0.4, 0.3), "cube": meshes.cube(12),
         "solid_cube": meshes.solid_cube(9), "plate": meshes.plate(40, 30, 0.6, 0.4, 0.002),
         "two_plates": two_bodies(meshes.plate(12, 9, 0.3, 0.2, 0.002))}[name]
    m, i = analysed(elp, d)
    assert 0 < i["factor_stored"] < i["factor_entries"]
    assert i["front_pool_peak"] <= i["front_pool"] <= i["factor_entries"]
    assert i["front_pool"] <= 1.25 * i["front_pool_peak"]  # first-fit wastes little on these trees


def test_group_keeps_each_members_tree(elp, meshes):
    """A group is the disjoint union of its members: the symbolic phase splits
    it into connected components first, so its fronts, factor entries and
    flops are exactly the sums of the members' own, whatever the members'
    coordinates (here all overlap at the origin)."""
    ds = [meshes.plate(12, 9, 0.3, 0.2, 0.002), meshes.plate(20, 15, 0.6, 0.4, 0.003), meshes.cube(4),
          meshes.plate_cavity(6, 4, 3, 0.3, 0.2, 0.15)]
    infos = [analysed(elp, d)[1] for d in ds]
    ms = [elp.Model(d) for d in ds]
    g = elp.Group(ms)
    gi = g.info()
    for key in ("n_dofs", "nnz", "n_elements", "n_fronts", "factor_entries", "factor_stored"):
        assert gi[key] == sum(i[key] for i in infos), key
    assert gi["factor_flops"] == pytest.approx(sum(i["factor_flops"] for i in infos), rel=1e-12)
    assert gi["n_levels"] == max(i["n_levels"] for i in infos)


def test_tuning_is_per_model(elp, meshes):
    """The leaf size of one model's tuning changes its tree (and nothing of
    another model's); get_tuning reports the values in effect, defaults
    resolved; bad values are refused."""
    d = meshes.plate(40, 30, 0.6, 0.4, 0.002)
    a = elp.Model(d).set_tuning(leaf=64)
    b = elp.Model(d)
    ia, ib = analysed(elp, d)[1], None
    for m in (a, b):
        try:
            m.analyse()
        except elp.ElpasoError as e:
            assert e.code == 2
    ia, ib = a.info(), b.info()
    assert ia["n_fronts"] > ib["n_fronts"]
    ta, tb = a.tuning(), b.tuning()
    assert ta["leaf"] == 64 and tb["leaf"] == 128
    assert tb["schur_tile"] == 64 and tb["lanes"] == 4 and tb["pack_count"] == 300
    a.set_tuning(leaf=128)  # the symbolic phase is redone with the new leaf size
    try:
        a.analyse()
    except elp.ElpasoError:
        pass
    assert a.info()["n_fronts"] == ib["n_fronts"]
    with pytest.raises(elp.ElpasoError):
        b.set_tuning(schur_tile=48)
    # unspecified knobs keep their defaults; 0 takes the default too, except pack_count (0: never)
    assert a.set_tuning(leaf=64).tuning()["pack_count"] == 300
    t = elp.Model(d).set_tuning(leaf=0, pack_min_border=0, lanes=0).tuning()
    assert (t["leaf"], t["pack_min_border"], t["lanes"]) == (128, 300, 4)
    assert elp.Model(d).set_tuning(pack_count=0).tuning()["pack_count"] == 0


def test_device_footprint_in_model_info(elp, meshes):
    """elp_model_info reports the resident arrays and one frequency's
    workspace per precision and front store: FP64 fronts take more than FP32
    ones, the whole fronts at least 8 B per front entry, and the compact store
    no more than the whole fronts plus its factor copy."""
    d = meshes.plate_cavity(16, 12, 8, 0.6, 0.4, 0.3)
    m, i = analysed(elp, d)
    assert i["device_array_bytes"] >= i["nnz"] * 21
    w = i["workspace_bytes_per_frequency"]
    assert w[1][0] >= 8 * i["factor_entries"] and w[0][0] >= 16 * i["factor_entries"]
    assert w[0][0] > w[1][0] and w[0][1] > w[1][1]
    assert w[1][1] <= w[1][0] + 8 * i["factor_stored"]
    fresh = elp.Model(d).info()  # no symbolic phase yet
    assert fresh["device_array_bytes"] > 0 and fresh["workspace_bytes_per_frequency"] == [[0, 0], [0, 0]]
