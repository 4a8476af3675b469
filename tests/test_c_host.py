"""The C ABI driven from C: tests/c_host/elp_c_host.c includes only
include/elpaso_gb300.h, is compiled with gcc as strict C11 and linked against
the built library, fills an elp_model_desc from plain arrays (as elpasoC's
FullRun would through a shim) and prints what the host-side calls return.
Its output must equal the Python binding's bit for bit on the same model
(the ctypes mirror and the header agree) and the oracle's restatement
(numbering, pattern bit-exact; F and stresses to 1e-14 / 1e-13). The header
also compiles as C++ (the reference is C++). It runs with or without a GPU:
elp_model_analyse runs the symbolic phase and then reports a missing device;
the stresses are computed on the device and compared when one is present."""
import copy
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_host", "elp_c_host.c")
INCLUDE = os.path.join(ROOT, "include")

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")


def c_host_desc(elp):
    """The model elp_c_host.c builds, as a ModelDesc."""
    nx, ny, nz = 3, 2, 2

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    n_nodes = (nx + 1) * (ny + 1) * (nz + 1)
    coords = np.zeros((n_nodes, 3))
    for k in range(nz + 1):
        for j in range(ny + 1):
            for i in range(nx + 1):
                coords[nid(i, j, k)] = (0.1 * i, 0.1 * j, 0.01 * k)
    hexes = [[nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
              nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)]
             for k in range(nz) for j in range(ny) for i in range(nx)]
    quads = [[nid(i, j, nz), nid(i + 1, j, nz), nid(i + 1, j + 1, nz), nid(i, j + 1, nz)]
             for j in range(ny) for i in range(nx)]
    mats = [dict(kind=elp.STR_LIN_VIS_ISO_DIR, E=0.0, nu=0.3, rho=7850.0, visco_type=1,
                 E_table=np.array([[50.0, 2.0e11], [300.0, 1.8e11]]), eta_table=np.array([[10.0, 0.01], [400.0, 0.04]])),
            dict(kind=elp.STR_LIN_ELA_ISO_DIR, E=70e9, nu=0.33, rho=2700.0, t=0.002)]
    fnode, fdof, fval = [], [], []
    for k in range(nz + 1):
        for j in range(ny + 1):
            for d in range(3):
                fnode.append(nid(0, j, k))
                fdof.append(d)
                fval.append(0j)
    fnode.append(nid(nx, ny, nz))
    fdof.append(3)  # w1
    fval.append(1e-6 + 2e-6j)
    return elp.ModelDesc(
        node_ids=5000 - 7 * np.arange(n_nodes, dtype=np.int64), coords=coords, materials=mats,
        blocks=[(elp.BRICK8, 0, np.array(hexes, np.int32)), (elp.DSG4, 1, np.array(quads, np.int32))],
        fixed=dict(node=np.array(fnode), dof=np.array(fdof), value=np.array(fval)),
        forces=dict(node=np.array([nid(2, 1, nz)]), f=np.array([[0.25, 0.0, 1.0]])),
        moments=dict(node=np.array([nid(1, 1, nz)]), m=np.array([[0.3, -0.5, 0.7]])),
        face_tractions=dict(block=np.zeros(3, np.int64), face=np.array([3, 4, 2]), element=np.array([0, 7, 11]),
                            t=np.array([[120 + 40j, -30, 15j], [5, 6 - 2j, -7], [-100, 0, 30 + 10j]])),
        name="c_host_box")


@pytest.fixture(scope="module")
def c_host_output(elp, tmp_path_factory):
    libdir = os.path.dirname(elp.library_path())
    exe = str(tmp_path_factory.mktemp("c_host") / "elp_c_host")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{INCLUDE}", SRC, "-o", exe,
                    f"-L{libdir}", "-lelpaso_gb300", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    out = {}
    for line in run.stdout.splitlines():
        tag, *vals = line.split()
        out[tag] = np.array([float(v) for v in vals])
    return out


def _cplx(a):
    return a[0::2] + 1j * a[1::2]


def test_header_compiles_as_cxx():
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    subprocess.run(["g++", "-std=c++17", "-x", "c++", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    f"-I{INCLUDE}", "-"], input='#include "elpaso_gb300.h"\nint main() { return ELP_OK; }\n',
                   text=True, check=True)


def test_c_host_matches_python_binding(elp, c_host_output):
    o = c_host_output
    m = elp.Model(c_host_desc(elp))
    n, nnz, n_nodes, n_el = (int(v) for v in o["sizes"])
    assert (n, nnz, n_el) == (m.n, m.info()["nnz"], 18)
    rp, ci = m.pattern()
    np.testing.assert_array_equal(o["row_ptr"], rp)
    np.testing.assert_array_equal(o["col_idx"], ci)
    np.testing.assert_array_equal(o["rows"].reshape(n_nodes, -1), m.global_rows())
    np.testing.assert_array_equal(_cplx(o["f"]), m.rhs())
    om = 2 * np.pi * 120.0
    np.testing.assert_array_equal(_cplx(o["f_omega"]), m.rhs(om))
    x = _cplx(o["x"])
    if "sigma" in o:  # the stresses run on the device (printed only when one answered)
        up, lo = m.cell_stresses(om, x)
        np.testing.assert_array_equal(_cplx(o["sigma"]).reshape(up.shape), up)
        np.testing.assert_array_equal(_cplx(o["sigma_lower"]).reshape(lo.shape), lo)
        np.testing.assert_array_equal(_cplx(o["sigma_nodes"]).reshape(n_nodes, 9), m.node_stresses(om, x))
    rc, fronts, levels, max_front = (int(v) for v in o["analyse"])
    assert rc in (0, 2) and fronts >= 1 and levels >= 1 and 0 < max_front <= n


def test_c_host_matches_oracle(elp, oracle, c_host_output):
    o = c_host_output
    d = c_host_desc(elp)
    s = oracle.System(d)
    np.testing.assert_array_equal(o["row_ptr"], s.row_ptr)
    np.testing.assert_array_equal(o["col_idx"], s.col_idx)
    f = _cplx(o["f"])
    np.testing.assert_allclose(f, s.f, rtol=0, atol=1e-14 * np.abs(s.f).max())
    d0 = copy.deepcopy(d)
    d0.face_tractions = None
    assert np.abs(f - oracle.System(d0).f).max() > 0.1  # the tractions are in
    om = 2 * np.pi * 120.0
    x = _cplx(o["x"])
    if "sigma" not in o:  # no device: the stresses were not computed
        return
    ou, ol = oracle.cell_stresses(s, om, x)
    scale = np.abs(ou).max()
    np.testing.assert_allclose(_cplx(o["sigma"]).reshape(ou.shape), ou, rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose(_cplx(o["sigma_lower"]).reshape(ol.shape), ol, rtol=0, atol=1e-13 * scale)
    on = oracle.node_stresses(s, om, x)
    np.testing.assert_allclose(_cplx(o["sigma_nodes"]).reshape(on.shape), on, rtol=0, atol=1e-13 * np.abs(on).max())


def test_python_binding_is_the_same_descriptor(elp):
    """The model description survives a deep copy (the binding copies nothing
    the C side keeps): two models from equal descriptions are equal."""
    d = c_host_desc(elp)
    m1, m2 = elp.Model(d), elp.Model(copy.deepcopy(d))
    np.testing.assert_array_equal(m1.rhs(), m2.rhs())


@pytest.mark.gpu
def test_c_host_stresses_on_the_device(elp, oracle, c_host_output):
    """With a device the C host computes the stresses too: the same bits as
    the Python binding (both run the same kernels, which sum in a fixed
    order), and the oracle's values to 1e-13."""
    o = c_host_output
    assert "sigma" in o and "sigma_nodes" in o
    m = elp.Model(c_host_desc(elp))
    n_nodes = int(o["sizes"][2])
    om = 2 * np.pi * 120.0
    x = _cplx(o["x"])
    up, lo = m.cell_stresses(om, x)
    np.testing.assert_array_equal(_cplx(o["sigma"]).reshape(up.shape), up)
    np.testing.assert_array_equal(_cplx(o["sigma_lower"]).reshape(lo.shape), lo)
    np.testing.assert_array_equal(_cplx(o["sigma_nodes"]).reshape(n_nodes, 9), m.node_stresses(om, x))
    s = oracle.System(c_host_desc(elp))
    ou, _ = oracle.cell_stresses(s, om, x)
    np.testing.assert_allclose(up, ou, rtol=0, atol=1e-13 * np.abs(ou).max())
