"""Generates the golden fixtures in this folder (run where the reference tree
is present; the output is committed and the tests never read the reference):

  elements.npz        element matrices computed by the reference's OWN element
                      code (oracle/_ref/libelpref.so, built by `make -C oracle ref`
                      from the reference sources) on seeded geometries:
                      Brick8 K/M/EM, DSG4 K/M/EM, Fluid8 K/M/EM, InterfaceMindlin C,
                      and the reference's hex8 / quad4 shape tables;
  known_answers.json  known-answer values read from the reference's unit tests
                      (hex8 shape table, elpasoCore/test/shape/testshapehex8.h:69-101;
                      visco material E_vis, Cs, Cb, elpasoCore/test/material/structure/
                      isotrop/linear/viscoelastic/testmaterialstructurevisco.h:92-330).

    python tests/golden/make_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SEED = 20260101


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _d(x):
    return C.c_double(float(x))


def hex_unit(scale=(1.0, 1.0, 1.0)):
    x = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], np.float64)
    return 0.5 * (x + 1.0) * np.asarray(scale)


def quad_unit(scale=(1.0, 1.0)):
    x = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float64)
    x[:, 0] *= scale[0]
    x[:, 1] *= scale[1]
    return x


def cases(rng):
    hexes = [hex_unit((0.05, 0.05, 0.005)), hex_unit((0.1, 0.2, 0.3)), hex_unit((0.01, 0.01, 0.01))]
    for _ in range(5):
        h = hex_unit((0.1, 0.1, 0.1)) + rng.uniform(-0.015, 0.015, size=(8, 3))
        hexes.append(h)
    quads = [quad_unit((0.01, 0.01)), quad_unit((0.02, 0.05))]
    for _ in range(4):
        q = quad_unit((0.01, 0.01)) + np.c_[rng.uniform(-0.002, 0.002, size=(4, 2)), np.zeros(4)]
        quads.append(q)
    # edge 3-0 the longest: the hk quirk of DSG4 (elementstructuremindlindsg4.cpp:60-62)
    quads.append(np.array([[0, 0, 0], [0.01, 0.002, 0], [0.011, 0.01, 0], [-0.002, 0.02, 0]], np.float64))
    return hexes, quads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ELPASO_REFERENCE", "/root/reference"))
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.ref}"], check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libelpref.so"))
    rng = np.random.default_rng(SEED)
    hexes, quads = cases(rng)
    out = {}
    # Brick8: (mat_kind, E, nu, rho, eta, visco_type, omega)
    bmats = [(1, 210e9, 0.3, 7850.0, 0.01, 1, 2 * np.pi * 100), (0, 70e9, 0.33, 2700.0, 0.0, 1, 2 * np.pi * 37),
             (1, 120e9, 0.28, 4000.0, 0.05, 2, 2 * np.pi * 250)]
    bx, bm, bK, bM, bEM = [], [], [], [], []
    for i, x in enumerate(hexes):
        mk = bmats[i % len(bmats)]
        K = np.zeros(1152); M = np.zeros(1152); EM = np.zeros(1152)
        xx = np.ascontiguousarray(x)
        rc = lib.ref_brick8(_p(xx), mk[0], _d(mk[1]), _d(mk[2]), _d(mk[3]), _d(mk[4]), mk[5], _d(mk[6]), _p(K), _p(M), _p(EM))
        assert rc == 0
        bx.append(x); bm.append(mk); bK.append(K.view(complex).reshape(24, 24)); bM.append(M.view(complex).reshape(24, 24))
        bEM.append(EM.view(complex).reshape(24, 24))
    out.update(brick_xyz=np.array(bx), brick_mat=np.array(bm), brick_K=np.array(bK), brick_M=np.array(bM),
               brick_EM=np.array(bEM))
    # DSG4: (mat_kind, E, nu, rho, t, eta, visco_type, omega)
    pmats = [(1, 70e9, 0.33, 2700.0, 0.002, 0.02, 1, 2 * np.pi * 100), (0, 210e9, 0.3, 7850.0, 0.005, 0.0, 1, 2 * np.pi * 20),
             (1, 70e9, 0.3, 2700.0, 0.003, 0.001, 2, 2 * np.pi * 400)]
    px, pm, pK, pM, pEM = [], [], [], [], []
    for i, x in enumerate(quads):
        mk = pmats[i % len(pmats)]
        K = np.zeros(288); M = np.zeros(288); EM = np.zeros(288)
        xx = np.ascontiguousarray(x)
        rc = lib.ref_dsg4(_p(xx), mk[0], _d(mk[1]), _d(mk[2]), _d(mk[3]), _d(mk[4]), _d(mk[5]), mk[6], _d(mk[7]),
                          _p(K), _p(M), _p(EM))
        assert rc == 0
        px.append(x); pm.append(mk); pK.append(K.view(complex).reshape(12, 12)); pM.append(M.view(complex).reshape(12, 12))
        pEM.append(EM.view(complex).reshape(12, 12))
    out.update(plate_xyz=np.array(px), plate_mat=np.array(pm), plate_K=np.array(pK), plate_M=np.array(pM),
               plate_EM=np.array(pEM))
    # Fluid8: (c, rho, omega)
    fmats = [(343.0, 1.21, 2 * np.pi * 100), (1480.0, 1000.0, 2 * np.pi * 50)]
    fx, fm, fK, fM, fEM = [], [], [], [], []
    for i, x in enumerate(hexes):
        mk = fmats[i % len(fmats)]
        K = np.zeros(128); M = np.zeros(128); EM = np.zeros(128)
        xx = np.ascontiguousarray(x)
        rc = lib.ref_fluid8(_p(xx), _d(mk[0]), _d(mk[1]), _d(mk[2]), _p(K), _p(M), _p(EM))
        assert rc == 0
        fx.append(x); fm.append(mk); fK.append(K.view(complex).reshape(8, 8)); fM.append(M.view(complex).reshape(8, 8))
        fEM.append(EM.view(complex).reshape(8, 8))
    out.update(fluid_xyz=np.array(fx), fluid_mat=np.array(fm), fluid_K=np.array(fK), fluid_M=np.array(fM),
               fluid_EM=np.array(fEM))
    # InterfaceMindlin
    ix, iC = [], []
    for x in quads:
        Cm = np.zeros(96)
        xx = np.ascontiguousarray(x)
        rc = lib.ref_interface_mindlin(_p(xx), _p(xx), _d(343.0), _d(1.21), _p(Cm))
        assert rc == 0
        ix.append(x); iC.append(Cm.view(complex).reshape(12, 4))
    out.update(iface_xyz=np.array(ix), iface_C=np.array(iC))
    hx = np.zeros(256); qd = np.zeros(48)
    lib.ref_shape_hex8(_p(hx)); lib.ref_shape_quad4(_p(qd))
    out.update(shape_hex8=hx, shape_quad4=qd)
    np.savez_compressed(os.path.join(HERE, "elements.npz"), **out)

    # ---- known answers from the reference's unit tests (read as text)
    test_root = os.path.join(args.ref, "elpasoCore", "test")
    src = open(os.path.join(test_root, "shape", "testshapehex8.h")).read()
    body = src[src.index("refData[256]"):]
    body = body[body.index("{") + 1:body.index("}")]
    hex_ref = [float(v) for v in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", body)]
    assert len(hex_ref) == 256, len(hex_ref)
    visco = open(os.path.join(test_root, "material", "structure", "isotrop", "linear", "viscoelastic",
                              "testmaterialstructurevisco.h")).read()
    cs = re.search(r"refVal =\s*([0-9.e+-]+) \+ ([0-9.e+-]+) \* PETSC_i", visco)
    cb = re.search(r"refVal1 =\s*([0-9.e+-]+) \+ ([0-9.e+-]+) \* PETSC_i", visco)
    ev = re.search(r"eVis = ([0-9.e+-]+) \+ ([0-9.e+-]+) \* PETSC_i", visco)
    ka = {
        "shape_hex8": {"values": hex_ref, "tol": 1e-6, "source": "elpasoCore/test/shape/testshapehex8.h:69-101"},
        "visco": {
            "E_vis": [float(ev.group(1)), float(ev.group(2))],
            "Cs00": [float(cs.group(1)), float(cs.group(2))],
            "Cb00": [float(cb.group(1)), float(cb.group(2))],
            # material of the fixture plate_dsg4_2elem_STR_LIN_VIS_ISO_DIR.hdf5, recovered
            # from the values above: E = 7e10, eta = 1e-3, nu = 0.3, t = 3 mm
            "E": 7e10, "eta": 1e-3, "nu": 0.3, "t": 0.003,
            "source": "elpasoCore/test/material/structure/isotrop/linear/viscoelastic/testmaterialstructurevisco.h:92-330",
        },
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(ka, f, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    sys.exit(main())
