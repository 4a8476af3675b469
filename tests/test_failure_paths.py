"""Failure paths of the C ABI, all made on the host (no test faults the GPU).

- bad element geometry: a DSG4 element with det J <= 0 fails the assembly
  with ELP_ERR_GEOMETRY, as the reference throws in setupJacobian2D
  (element/elementfem.cpp:97-100); a Brick8 element with det J <= 0 is
  counted and the assembly goes on, as the reference only prints a message
  in setupJacobian3D (:183-188, its throw commented out);
- a singular system (a structure of zero stiffness and mass): the
  static-pivot floor stands in for the zero pivots, the refinement cannot
  converge, and the solve reports ELP_ERR_SINGULAR with the pivot count;
- injected allocation failures (elp_fault_inject): a host allocation in
  model creation or the host symbolic phase, and every device allocation of
  a solve in turn, return ELP_ERR_NOMEM and leave the library usable;
- a device-side bounded wait made to run out: the packed tensor-core Schur
  kernel is launched with its producer told to issue nothing and its waits
  bounded at 2^14 polls; no copy or MMA is in flight when they run out, the
  kernel sets its error flag and returns, the solve returns ELP_ERR_CUDA, and
  the next solve on the same model succeeds.
"""
import copy
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NOMEM, GEOMETRY, SINGULAR, CUDA = 3, 4, 5, 2
FAULT_NONE, FAULT_DEVICE_ALLOC, FAULT_HOST_ALLOC, FAULT_TC_WAIT = 0, 1, 2, 3


def _inject(elp, kind, countdown):
    assert elp.load_library().elp_fault_inject(kind, countdown) == 0


def test_host_allocation_failure_in_model_creation(elp, meshes):
    d = meshes.plate(6, 5, 0.3, 0.2, 0.002)
    _inject(elp, FAULT_HOST_ALLOC, 1)
    with pytest.raises(elp.ElpasoError) as e:
        elp.Model(d)
    assert e.value.code == NOMEM
    m = elp.Model(d)  # the fault fired once: creation works again
    assert m.n == elp.Model(d).n
    _inject(elp, FAULT_NONE, 0)


def test_host_allocation_failure_in_symbolic_phase(elp, meshes):
    """The host symbolic phase runs before the library looks for a device, so
    this runs without a GPU too: the injected failure gives ELP_ERR_NOMEM, and
    the next call gets past the symbolic phase (on a machine without a GPU it
    then stops at the device check with ELP_ERR_CUDA)."""
    m = elp.Model(meshes.plate(6, 5, 0.3, 0.2, 0.002))
    _inject(elp, FAULT_HOST_ALLOC, 1)
    with pytest.raises(elp.ElpasoError) as e:
        m.analyse()
    assert e.value.code == NOMEM
    try:
        m.analyse()
    except elp.ElpasoError as e2:
        assert e2.code == CUDA
    assert m.info()["n_fronts"] > 0


def test_fault_inject_rejects_unknown_kinds(elp):
    lib = elp.load_library()
    assert lib.elp_fault_inject(99, 1) == 1
    assert lib.elp_fault_inject(FAULT_DEVICE_ALLOC, -1) == 1
    assert lib.elp_fault_inject(FAULT_NONE, 0) == 0


def _twisted_plate(meshes):
    d = copy.deepcopy(meshes.plate(6, 5, 0.3, 0.2, 0.002))
    typ, mat, conn = d.blocks[0]
    conn = np.array(conn)
    conn[7] = conn[7][[0, 3, 2, 1]]  # clockwise node order: det J < 0 at every Gauss point
    d.blocks[0] = (typ, mat, conn)
    return d


def _inverted_brick(meshes):
    d = copy.deepcopy(meshes.solid_plate(6, 5, 2))
    typ, mat, conn = d.blocks[0]
    conn = np.array(conn)
    conn[3] = conn[3][[4, 5, 6, 7, 0, 1, 2, 3]]  # top and bottom faces swapped: det J < 0
    d.blocks[0] = (typ, mat, conn)
    return d


@pytest.mark.gpu
def test_twisted_dsg4_element_fails_assembly(elp, meshes):
    m = elp.Model(_twisted_plate(meshes))
    with pytest.raises(elp.ElpasoError) as e:
        m.assemble()
    assert e.value.code == GEOMETRY
    assert b"detJac" in elp.load_library().elp_last_error()


@pytest.mark.gpu
def test_inverted_brick8_element_is_counted(elp, meshes, oracle):
    """Assembly goes on and A(w) still equals the oracle's (the reference
    integrates the element with its negative det J)."""
    d = _inverted_brick(meshes)
    m = elp.Model(d).assemble()
    assert m.info()["n_nonpositive_jacobians"] == 8  # every Gauss point of the element
    ok = elp.Model(meshes.solid_plate(6, 5, 2)).assemble()
    assert ok.info()["n_nonpositive_jacobians"] == 0
    s = oracle.System(d)
    om = 2 * np.pi * 50.0
    a, b = m.system_values(om), s.values(om)
    scale = np.max(np.abs(b))
    assert np.max(np.abs(a - b)) <= 1e-12 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_singular_system_reports_static_pivots(elp, meshes, prec):
    d = copy.deepcopy(meshes.solid_plate(4, 4, 2))
    d.materials = [dict(kind=1, E=0.0, nu=0.3, rho=0.0)]
    m = elp.Model(d).assemble().analyse()
    with pytest.raises(elp.ElpasoError) as e:
        m.solve([2 * np.pi * 100.0], precision=prec)
    assert e.value.code == SINGULAR
    x, info = m.solve([2 * np.pi * 100.0], precision=prec, raise_on_noconv=False)
    assert info[0]["static_pivots"] > 0 and info[0]["converged"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_every_device_allocation_failure_of_a_solve(elp, meshes, oracle, prec):
    """The k-th device allocation after the fault is armed fails, for every k
    a first solve makes (the C API's input/output buffers, the front
    workspace, the Krylov buffers); each time the solve returns ELP_ERR_NOMEM,
    then the same call without a fault succeeds with the oracle's residual."""
    d = meshes.plate(8, 6, 0.3, 0.2, 0.002)
    s = oracle.System(d)
    om = 2 * np.pi * 77.0
    A = s.matrix(om)
    hits = 0
    for k in range(1, 40):
        m = elp.Model(d).assemble().analyse()
        _inject(elp, FAULT_DEVICE_ALLOC, k)
        try:
            m.solve([om], precision=prec)
        except elp.ElpasoError as e:
            assert e.code == NOMEM, (k, e)
            hits += 1
        _inject(elp, FAULT_NONE, 0)
        x, info = m.solve([om], precision=prec)
        assert np.linalg.norm(s.f - A @ x[0]) / np.linalg.norm(s.f) <= 1e-10, k
        m.close()
    # allocations of a first solve: the C API's buffer, ~17 of the workspace, and
    # the mixed path's 10 Krylov buffers
    assert hits >= (15 if prec == 0 else 25), hits


PROBE = r"""
import importlib, json, sys
import numpy as np
sys.path.insert(0, ROOT)
from tests.conftest import load_package
elp = load_package()
meshes = importlib.import_module("elpaso_core_gb300.meshes")
lib = elp.load_library()
m = elp.Model(meshes.plate_cavity(10, 8, 6, 0.6, 0.4, 0.3)).assemble().analyse()
oms = 2 * np.pi * np.array([40.0, 260.0])
out = {}
x0, i0 = m.solve(oms, precision=1)
out["before"] = [i["rel_residual"] for i in i0]
assert lib.elp_fault_inject(3, 1) == 0
try:
    m.solve(oms, precision=1)
    out["faulted"] = 0
except elp.ElpasoError as e:
    out["faulted"] = e.code
    out["text"] = str(e)
x1, i1 = m.solve(oms, precision=1)
out["after"] = [i["rel_residual"] for i in i1]
out["same"] = bool(np.array_equal(x0, x1))
print(json.dumps(out))
""".replace("ROOT", repr(ROOT))


@pytest.mark.gpu
def test_tensor_core_wait_runs_out_and_the_next_solve_succeeds():
    """ELP_TC_PACK=all puts every level of this small model through the
    packed Schur kernel; the fault makes one of its launches give up."""
    env = dict(os.environ, ELP_TC="1", ELP_TC_PACK="all")
    p = subprocess.run([sys.executable, "-c", PROBE], env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    out = json.loads(p.stdout.strip().splitlines()[-1])
    assert out["faulted"] == CUDA, out
    assert "gave up waiting" in out["text"]
    assert max(out["before"]) <= 1e-10 and max(out["after"]) <= 1e-10
    assert out["same"]  # the solve after the fault equals the one before it, bit for bit
