"""Solve sweeps on global front vectors. Levels whose front vector (m + p
complex entries) does not fit the 227 KB of shared memory a CTA can take --
the top separators of models past ~200k DOFs -- keep it in a global slice per
(front, frequency). ELP_SOLVE_GLOBAL=1 puts every level there; in a child
process with it set, solves of the plate-cavity and cube models in both
precisions meet the residual bar against the oracle, and equal the shared-
memory sweeps' solutions of the parent to the rounding of two assemblies."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from conftest import load_package
import importlib
elp = load_package(); meshes = importlib.import_module("elpaso_core_gb300.meshes")
from oracle import oracle
out = {{}}
for d in (meshes.plate_cavity(8, 6, 4, 0.6, 0.4, 0.3), meshes.cube(5)):
    m = elp.Model(d).assemble().analyse()
    s = oracle.System(d)
    oms = 2 * np.pi * np.array([11.0, 230.0, 470.0])
    for prec in (0, 1):
        x, infos = m.solve(oms, precision=prec)
        res = [float(np.linalg.norm(s.rhs(om) - s.matrix(om) @ x[k]) / np.linalg.norm(s.rhs(om)))
               for k, om in enumerate(oms)]
        out[f"{{d.name}}/{{prec}}"] = dict(res=res, x=[[v.real, v.imag] for v in x.ravel()])
print(json.dumps(out))
"""


def test_global_front_vectors_solve_like_shared_memory(elp, meshes):
    env = dict(os.environ, ELP_SOLVE_GLOBAL="1")
    code = CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    oms = 2 * np.pi * np.array([11.0, 230.0, 470.0])
    for d in (meshes.plate_cavity(8, 6, 4, 0.6, 0.4, 0.3), meshes.cube(5)):
        m = elp.Model(d).assemble().analyse()
        for prec in (0, 1):
            g = got[f"{d.name}/{prec}"]
            assert max(g["res"]) <= 1e-10, (d.name, prec, g["res"])
            xg = np.array(g["x"]).view(np.complex128).reshape(len(oms), -1)
            x, _ = m.solve(oms, precision=prec)
            assert np.max(np.abs(xg - x)) <= 1e-8 * np.max(np.abs(x)), (d.name, prec)
