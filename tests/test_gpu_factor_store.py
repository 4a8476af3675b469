"""The two front stores of a factorisation give the same solutions: whole fronts (STORE_FULL, the solves read the factors in place) and the
compact store (STORE_COMPACT: full fronts only while a level is factorised,
in reused pool regions; each level's m x p panel and U12 copied into a
factor store the solves read, U12 with leading dimension p). The arithmetic
and its order are the same, only the factors' addresses differ. The store
is chosen by memory unless ELP_FACTOR_STORE forces one; it is read once per
process, so each store runs in its own process -- and two processes assemble
A(w) with FP64 atomic additions in different orders, which moves its values
by ~1e-16 relative; two solutions refined to 1e-10 from slightly different
FP32 factors then differ within what their residuals allow. Bars: both
stores' solutions at ||f - A x|| / ||f|| <= 1e-10 with the oracle's matrix,
and ||x_full - x_compact||_1 / ||x_full||_1 <= 3 kappa_1(A_ff) (res_1 +
res_1'), the free-block perturbation bound of the other solve tests. Models: the coupled
plate-cavity (fluid, coupling, Dirichlet rows; the packed tensor-core Schur
levels forced on every level with ELP_TC_PACK=all) and a Brick8 cube, both
precisions."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from test_gpu_solve import cond1

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import importlib, json, sys
import numpy as np
sys.path.insert(0, ROOT)
from tests.conftest import load_package
from oracle import oracle as orc
elp = load_package()
meshes = importlib.import_module("elpaso_core_gb300.meshes")
out = {}
for name, d in (("pc", meshes.plate_cavity(14, 10, 8, 0.6, 0.4, 0.3)), ("cube", meshes.cube(8))):
    m = elp.Model(d).assemble().analyse()
    s = orc.System(d)
    for prec in (0, 1):
        oms = 2 * np.pi * np.array([3.0, 88.0, 271.0, 499.0])
        x, info = m.solve(oms, precision=prec)
        res = [float(np.linalg.norm(s.rhs(om) - s.matrix(om) @ x[j]) / np.linalg.norm(s.rhs(om)))
               for j, om in enumerate(oms)]
        out[f"{name}_{prec}"] = [x.view(np.float64).tolist(), res]
print(json.dumps(out))
""".replace("ROOT", repr(ROOT))


def _run(**env):
    p = subprocess.run([sys.executable, "-c", PROBE], env=dict(os.environ, **env), capture_output=True, text=True,
                       timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("pack", ["", "all"])
def test_compact_factor_store_equals_whole_fronts(meshes, oracle, pack):
    full = _run(ELP_FACTOR_STORE="full", ELP_TC_PACK=pack)
    compact = _run(ELP_FACTOR_STORE="compact", ELP_TC_PACK=pack)
    descs = {"pc": meshes.plate_cavity(14, 10, 8, 0.6, 0.4, 0.3), "cube": meshes.cube(8)}
    oms = 2 * np.pi * np.array([3.0, 88.0, 271.0, 499.0])
    for key in full:
        xf, resf = full[key]
        xc, resc = compact[key]
        assert max(resf) <= 1e-10 and max(resc) <= 1e-10, key
        xf = np.asarray(xf).view(np.complex128)
        xc = np.asarray(xc).view(np.complex128)
        s = oracle.System(descs[key.split("_")[0]])
        for j, om in enumerate(oms):
            A, f = s.matrix(om), s.rhs(om)
            n1 = np.linalg.norm(f, 1)
            r1 = (np.linalg.norm(f - A @ xf[j], 1) + np.linalg.norm(f - A @ xc[j], 1)) / n1
            bound = 3.0 * cond1(s.free_block(om)[0]) * r1
            assert np.linalg.norm(xf[j] - xc[j], 1) / np.linalg.norm(xf[j], 1) <= max(1e-13, bound), (key, j)
