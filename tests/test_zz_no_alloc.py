"""Allocation-free residual check, elp_residual_noalloc.

Callers that cannot allocate device memory while they run (device memory
owned by another framework's pool or a fixed budget, an embedding that
forbids allocation after start-up) check their solutions with this entry
point. Here it must agree with the residual
that the solve path itself reports (elp_solve_device, info.rel_residual) for
the same solutions, on two calls in a row, its residual vector must match
its own norm, and it must reject more frequencies than its fixed scratch
array holds. The file sorts last so that a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES_TOL = 1e-10  # the relative-residual bar of the solve tests


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_noalloc_residual_matches_solve_path(elp, meshes):
    torch = pytest.importorskip("torch")
    d = meshes.plate_cavity(12, 8, 6, 0.6, 0.4, 0.3)
    m = elp.Model(d).assemble().analyse()
    n = m.n
    oms = np.ascontiguousarray(2 * np.pi * np.array([3.0, 140.0, 421.0]))
    S = len(oms)
    lib = elp.load_library()
    fh = np.ascontiguousarray(np.broadcast_to(m.rhs(), (S, n)))
    f = torch.from_numpy(fh.view(np.float64).copy()).cuda()
    x = torch.zeros_like(f)
    r = torch.zeros_like(f)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    infos = (elp.SolveInfo * S)()
    rc = lib.elp_solve_device(m.handle, _p(oms), S, elp.MIXED, C.c_void_p(f.data_ptr()), C.c_void_p(x.data_ptr()),
                              C.cast(infos, C.c_void_p), RES_TOL, stream)
    assert rc == 0, lib.elp_last_error()
    ref = np.array([infos[i].rel_residual for i in range(S)])
    assert np.all(ref <= RES_TOL)
    for call in range(2):
        rel = np.zeros(S)
        r.zero_()
        rc = lib.elp_residual_noalloc(m.handle, _p(oms), S, C.c_void_p(f.data_ptr()), C.c_void_p(x.data_ptr()),
                                      C.c_void_p(r.data_ptr()), _p(rel), stream)
        assert rc == 0, lib.elp_last_error()
        assert np.all(np.abs(rel - ref) <= RES_TOL), (call, rel, ref)
        assert np.all(np.abs(rel - ref) <= 1e-6 * ref), (call, rel, ref)
        rv = r.view(S, n, 2).cpu().numpy()
        own = np.sqrt((rv ** 2).sum(axis=(1, 2))) / np.linalg.norm(fh, axis=1)
        assert np.all(np.abs(own - rel) <= 1e-6 * rel), (call, own, rel)


def test_noalloc_rejects_more_frequencies_than_its_scratch_holds(elp, meshes):
    torch = pytest.importorskip("torch")
    m = elp.Model(meshes.plate(6, 5, 0.3, 0.2, 0.002)).assemble()
    n = m.n
    S = 65
    oms = np.ascontiguousarray(np.full(S, 2 * np.pi * 50.0))
    buf = torch.zeros((S, 2 * n), dtype=torch.float64, device="cuda")
    rel = np.zeros(S)
    lib = elp.load_library()
    rc = lib.elp_residual_noalloc(m.handle, _p(oms), S, C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                                  C.c_void_p(buf.data_ptr()), _p(rel), None)
    assert rc == 1
    assert b"ELP_NOALLOC_MAX_OMEGA" in lib.elp_last_error()


def test_noalloc_full_scratch_on_an_unanalysed_model(elp, meshes):
    """ELP_NOALLOC_MAX_OMEGA frequencies at once (every row of the scratch
    array in use) on a model that is assembled but not analysed (the
    residual needs only the value arrays): each relative residual of random
    solutions equals the host's ||f - A x|| / ||f|| with A from
    elp_model_system_values, on two calls in a row."""
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    m = elp.Model(meshes.plate(10, 8, 0.3, 0.2, 0.002)).assemble()
    n = m.n
    lib = elp.load_library()
    S = 64  # ELP_NOALLOC_MAX_OMEGA
    oms = np.ascontiguousarray(2 * np.pi * np.linspace(5.0, 495.0, S))
    rng = np.random.default_rng(11)
    xh = rng.standard_normal((S, n)) + 1j * rng.standard_normal((S, n))
    fh = np.stack([m.rhs(om) for om in oms]) + 1e-3 * (rng.standard_normal((S, n)) + 1j * rng.standard_normal((S, n)))
    rp, ci = m.pattern()
    want = np.empty(S)
    for k, om in enumerate(oms):
        A = sp.csr_matrix((m.system_values(om), ci, rp), shape=(n, n))
        want[k] = np.linalg.norm(fh[k] - A @ xh[k]) / np.linalg.norm(fh[k])
    f = torch.from_numpy(np.ascontiguousarray(fh).view(np.float64).copy()).cuda()
    x = torch.from_numpy(np.ascontiguousarray(xh).view(np.float64).copy()).cuda()
    r = torch.zeros_like(f)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        rel = np.zeros(S)
        rc = lib.elp_residual_noalloc(m.handle, _p(oms), S, C.c_void_p(f.data_ptr()), C.c_void_p(x.data_ptr()),
                                      C.c_void_p(r.data_ptr()), _p(rel), stream)
        assert rc == 0, lib.elp_last_error()
        assert np.all(np.abs(rel - want) <= 1e-12 * want), (call, np.max(np.abs(rel - want) / want))
