"""Tensor-core (tcgen05, 3xTF32) Schur updates against the SIMT FP32 ones.

The mixed path runs its FP32 front updates on the tensor cores; ELP_TC=0
selects the SIMT kernels instead. Both factorisations are preconditioners
for the same FP64 GMRES, so with the 3xTF32 split the two must both converge
to the 1e-10 relative residual, the tensor-core factors needing at most
2 + half again the SIMT steps at every frequency (3xTF32 drops the lo*lo
term and rounds the lo parts to TF32, so its products are a few times less
accurate than FP32; that shows only at the most ill-conditioned, lowest
frequencies). Each variant runs in its own process because the switch is
read once per process. The packed-operand Schur kernel is checked the same
way with ELP_TC_PACK=all (every level through it).
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import importlib, json, sys
import numpy as np
sys.path.insert(0, ROOT)
from tests.conftest import load_package
elp = load_package()
meshes = importlib.import_module("elpaso_core_gb300.meshes")
out = {}
for name, d in (("pc", meshes.plate_cavity(16, 12, 8, 0.6, 0.4, 0.3)), ("cube", meshes.cube(7))):
    m = elp.Model(d).assemble().analyse()
    x, info = m.solve(2 * np.pi * np.array([2.0, 37.0, 111.0, 260.0, 499.0]), precision=1)
    out[name] = [(i["iterations"], i["rel_residual"]) for i in info]
print(json.dumps(out))
""".replace("ROOT", repr(ROOT))


def _run(tc):
    env = dict(os.environ, ELP_TC=tc)
    p = subprocess.run([sys.executable, "-c", PROBE], env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


def _run_env(**env):
    p = subprocess.run([sys.executable, "-c", PROBE], env=dict(os.environ, **env), capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


def _close(tc, simt):
    for name in tc:
        for (it_a, res_a), (it_b, res_b) in zip(tc[name], simt[name]):
            assert res_a <= 1e-10 and res_b <= 1e-10
            assert it_a <= it_b + 2 + it_b // 2, (name, tc[name], simt[name])
            assert it_b <= it_a + 2 + it_a // 2, (name, tc[name], simt[name])


def test_tensor_core_updates_match_simt_convergence():
    _close(_run("1"), _run("0"))


def test_packed_schur_updates_match_simt_convergence():
    """The packed-operand Schur kernel (k_schur_tc) runs only on the top
    levels of large models; ELP_TC_PACK=all puts every level of these small
    models through it."""
    _close(_run_env(ELP_TC="1", ELP_TC_PACK="all"), _run("0"))
