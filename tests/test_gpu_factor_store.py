"""The two front stores of a factorisation give the same solutions: whole fronts (STORE_FULL, the solves read the factors in place) and the
compact store (STORE_COMPACT: full fronts only while a level is factorised,
in reused pool regions; each level's m x p panel and U12 copied into a
factor store the solves read, U12 with leading dimension p). The arithmetic
and its order are the same, only the factors' addresses differ. The store
is chosen by memory unless ELP_FACTOR_STORE forces one; it is read once per
process, so each store runs in its own process -- and two processes assemble
A(w) with FP64 atomic additions in different orders, which moves its values
by ~1e-16 relative and the solutions by ~1e-13. The bar is therefore
rounding level: max |x_full - x_compact| <= 1e-11 max |x_full| per solution. Models: the coupled
plate-cavity (fluid, coupling, Dirichlet rows; the packed tensor-core Schur
levels forced on every level with ELP_TC_PACK=all) and a Brick8 cube, both
precisions."""
import json
import os
import subprocess
import sys

import numpy as np
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
for name, d in (("pc", meshes.plate_cavity(14, 10, 8, 0.6, 0.4, 0.3)), ("cube", meshes.cube(8))):
    m = elp.Model(d).assemble().analyse()
    i = m.info()
    out[name + "_sizes"] = [i["factor_entries"], i["factor_stored"], i["front_pool"]]
    for prec in (0, 1):
        x, info = m.solve(2 * np.pi * np.array([3.0, 88.0, 271.0, 499.0]), precision=prec)
        out[f"{name}_{prec}"] = [x.view(np.float64).tolist(), [j["rel_residual"] for j in info]]
print(json.dumps(out))
""".replace("ROOT", repr(ROOT))


def _run(**env):
    p = subprocess.run([sys.executable, "-c", PROBE], env=dict(os.environ, **env), capture_output=True, text=True,
                       timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("pack", ["", "all"])
def test_compact_factor_store_equals_whole_fronts(pack):
    full = _run(ELP_FACTOR_STORE="full", ELP_TC_PACK=pack)
    compact = _run(ELP_FACTOR_STORE="compact", ELP_TC_PACK=pack)
    for key in full:
        if key.endswith("_sizes"):  # small trees: the pool holds most fronts, so no saving is claimed here
            continue
        xf, resf = full[key]
        xc, resc = compact[key]
        assert max(resf) <= 1e-10 and max(resc) <= 1e-10, key
        xf, xc = np.asarray(xf), np.asarray(xc)
        assert np.max(np.abs(xf - xc)) <= 1e-11 * np.max(np.abs(xf)), key
