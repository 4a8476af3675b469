"""Serving loop on the GPU: continuous batching over resident models.

- a request's result is the same alone and in a mix of concurrent requests
  on several models (tolerance: relative difference <= 1e-12; the kernels
  compute each frequency slot independently, so equality is expected);
- every result meets the 1e-10 relative residual (checked by the oracle);
- a model that does not fit the HBM budget fails its requests with
  ELP_ERR_NOMEM (status 3) while the others complete.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SAME_TOL = 1e-12


def _models(elp, meshes):
    ds = [meshes.plate(16, 12, 0.6, 0.4, 0.002), meshes.plate_cavity(8, 6, 4, 0.6, 0.4, 0.3), meshes.cube(5)]
    return ds, [elp.Model(d) for d in ds]


def _run(srv, reqs, n_of):
    outs = {}
    ids = {}
    for key, (mid, oms) in reqs.items():
        x = np.zeros((len(oms), n_of[mid]), np.complex128)
        rid = srv.submit(mid, oms, x)
        ids[rid] = key
        outs[key] = x
    res = {}
    for _ in range(len(reqs)):
        r = srv.wait(60000.0)
        res[ids[r["request_id"]]] = r
    return outs, res


@pytest.mark.parametrize("prec", [0, 1])
def test_alone_equals_in_mix(elp, meshes, oracle, prec):
    ds, ms = _models(elp, meshes)
    srv = elp.Server(hbm_budget_bytes=8 << 30, max_inflight=3, precision=prec, tol=1e-10, omega_batch=4)
    mids = [srv.add_model(m) for m in ms]
    n_of = {mid: ms[i].n for i, mid in enumerate(mids)}
    probe = (mids[1], 2 * np.pi * np.array([17.0, 140.0, 333.0]))
    alone, res = _run(srv, {"probe": probe}, n_of)
    assert res["probe"]["status"] == 0
    rng = np.random.default_rng(7)
    mix = {"probe": probe}
    for k in range(9):
        mid = mids[k % 3]
        mix[f"r{k}"] = (mid, 2 * np.pi * rng.uniform(1.0, 500.0, size=int(rng.integers(1, 7))))
    outs, res = _run(srv, mix, n_of)
    for key, r in res.items():
        assert r["status"] == 0, (key, r)
        assert r["max_rel_residual"] <= 1e-10
        assert r["latency_ms"] > 0
    diff = np.max(np.abs(outs["probe"] - alone["probe"])) / np.max(np.abs(alone["probe"]))
    assert diff <= SAME_TOL
    # the oracle confirms the residual of a mixed-in result
    s = oracle.System(ds[1])
    A = s.matrix(probe[1][1])
    assert np.linalg.norm(s.f - A @ outs["probe"][1]) / np.linalg.norm(s.f) <= 1e-10
    srv.close()


def test_budget_admission(elp, meshes):
    small = elp.Model(meshes.plate(8, 8, 0.3, 0.3, 0.002))
    big = elp.Model(meshes.cube(10))
    srv = elp.Server(hbm_budget_bytes=24 << 20, max_inflight=2, precision=1, tol=1e-10, omega_batch=4)
    a = srv.add_model(small)
    b = srv.add_model(big)
    xa = np.zeros((2, small.n), np.complex128)
    xb = np.zeros((2, big.n), np.complex128)
    ra = srv.submit(a, 2 * np.pi * np.array([10.0, 20.0]), xa)
    rb = srv.submit(b, 2 * np.pi * np.array([10.0, 20.0]), xb)
    got = {}
    for _ in range(2):
        r = srv.wait(60000.0)
        got[r["request_id"]] = r
    assert got[ra]["status"] == 0
    assert got[rb]["status"] == 3
    srv.close()


def test_wait_times_out_without_work(elp):
    srv = elp.Server(hbm_budget_bytes=1 << 30, max_inflight=1, precision=1)
    with pytest.raises(elp.ElpasoError) as e:
        srv.wait(50.0)
    assert e.value.code == 8
    srv.close()


def test_models_added_while_batches_run(elp, meshes, oracle):
    """Model slots keep their addresses: models registered while other
    models' batches run (the slot table grows under the running workers)
    are served, and every result meets the residual target."""
    first = elp.Model(meshes.plate_cavity(12, 8, 6, 0.6, 0.4, 0.3))
    srv = elp.Server(hbm_budget_bytes=16 << 30, max_inflight=2, precision=1, tol=1e-10, omega_batch=8)
    a = srv.add_model(first)
    xa = np.zeros((8, first.n), np.complex128)
    ra = srv.submit(a, 2 * np.pi * np.linspace(20.0, 480.0, 8), xa)
    later, outs = [], {}
    for k in range(12):  # registered while model a's batch is in flight
        d = meshes.plate(6 + k, 5 + k, 0.3, 0.2, 0.002)
        m = elp.Model(d)
        mid = srv.add_model(m)
        later.append((mid, m, d))
        x = np.zeros((2, m.n), np.complex128)
        outs[srv.submit(mid, 2 * np.pi * np.array([33.0, 210.0]), x)] = (x, d)
    got = {}
    for _ in range(1 + len(later)):
        r = srv.wait(120000.0)
        got[r["request_id"]] = r
    assert all(r["status"] == 0 and r["max_rel_residual"] <= 1e-10 for r in got.values()), got
    for rid, (x, d) in list(outs.items())[:3]:
        s = oracle.System(d)
        A = s.matrix(2 * np.pi * 210.0)
        assert np.linalg.norm(s.f - A @ x[1]) / np.linalg.norm(s.f) <= 1e-10
    srv.close()


def test_admission_refuses_before_allocating(elp, meshes):
    """A model whose resident arrays alone exceed the budget is refused
    before anything is allocated for it: it is never assembled (its system
    values report ELP_ERR_STATE), and the device's free memory is unchanged."""
    torch = pytest.importorskip("torch")
    big = elp.Model(meshes.cube(14))
    srv = elp.Server(hbm_budget_bytes=4 << 20, max_inflight=1, precision=1, tol=1e-10, omega_batch=4)
    b = srv.add_model(big)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    x = np.zeros((1, big.n), np.complex128)
    rid = srv.submit(b, 2 * np.pi * np.array([10.0]), x)
    r = srv.wait(60000.0)
    assert r["request_id"] == rid and r["status"] == 3
    assert torch.cuda.mem_get_info()[0] >= free0 - (2 << 20)  # at most the worker stream's own bookkeeping
    with pytest.raises(elp.ElpasoError) as e:
        big.system_values(2 * np.pi * 10.0)
    assert e.value.code == 7
    srv.close()


def test_a_model_waits_for_room_instead_of_failing(elp, meshes):
    """The budget holds both models' resident arrays but only one of them
    with an 8-frequency workspace. While model A's 64 frequencies run, B's
    arrays do not fit: B waits for A's workspace to be released (or takes it
    once nothing runs) instead of failing its requests with ELP_ERR_NOMEM."""
    import time
    ma = elp.Model(meshes.plate_cavity(12, 8, 6, 0.6, 0.4, 0.3)).assemble().analyse()
    mb = elp.Model(meshes.plate(30, 22, 0.6, 0.4, 0.003, seed=7)).assemble().analyse()
    ia, ib = ma.info(), mb.info()
    A, B = ia["device_array_bytes"], ib["device_array_bytes"]
    W = ia["workspace_bytes_per_frequency"][1][0]
    Wb = ib["workspace_bytes_per_frequency"][1][0]
    budget = A + 8 * W + B // 2
    assert B + Wb <= budget  # B alone fits: a NOMEM would be the bug
    srv = elp.Server(hbm_budget_bytes=budget, max_inflight=2, precision=1, tol=1e-10, omega_batch=8)
    a, b = srv.add_model(ma), srv.add_model(mb)
    xa = np.zeros((64, ma.n), np.complex128)
    ra = srv.submit(a, 2 * np.pi * np.linspace(10.0, 490.0, 64), xa)
    time.sleep(0.2)  # A's first batch holds its workspace
    xb = [np.zeros((4, mb.n), np.complex128) for _ in range(3)]
    rb = [srv.submit(b, 2 * np.pi * np.array([21.0, 140.0, 260.0, 377.0]) + k, x) for k, x in enumerate(xb)]
    got = {}
    for _ in range(4):
        r = srv.wait(300000.0)
        got[r["request_id"]] = r
    assert all(got[r]["status"] == 0 and got[r]["max_rel_residual"] <= 1e-10 for r in [ra] + rb), got
    srv.close()
