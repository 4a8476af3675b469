"""Generates tutorial_plate_dsg4.npz: the end-to-end golden of the DSG4 path.

Source: the reference's tutorial "Analysis of a rectangular plate (DSG4)"
(doc/tutorials/FEM_tutorials/Simulations/Ex_1_Analysis_of_a_rectangular_plate_DSG4/):

  Analysis_of_a_rectangular_plate.hdf5              the elpasoC input model:
      70 nodes, 54 DSG4 elements, aluminium STR_LIN_ELA_ISO_DIR (E 70 GPa,
      nu 0.34, rho 2700, t 3 mm), w fixed on 30 nodes, unit Fz at node 70,
      frequency sweep 10..250 Hz step 1;
  eGenOutput_Analysis_of_a_rectangular_plate.hdf5   the solution elpasoC
      wrote for it (PETSc + MUMPS FP64 LU; the run's log is beside it):
      /Solution/State/vecFemStep{1..241} complex vectors over the 210 global
      rows, /Solution/Maps/mtxDofMap (node id, dof enum) per row.

Both files are read with the package's own reader (h5model over h5lite). The
fixture keeps the model arrays (node indices, not ids), the reference DOF map
and every second frequency's reference solution (real: the material has no
damping).

    python tests/golden/make_tutorial_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
TUTORIAL = "doc/tutorials/FEM_tutorials/Simulations/Ex_1_Analysis_of_a_rectangular_plate_DSG4"

def _load(name):
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "elpaso-core_gb300", name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Desc:
    """Stand-in for the package's ModelDesc (no library load needed here)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ELPASO_REFERENCE", "/root/reference"))
    ap.add_argument("--out", default=os.path.join(HERE, "tutorial_plate_dsg4.npz"))
    args = ap.parse_args()
    h5model = _load("h5model")
    folder = os.path.join(args.ref, TUTORIAL)
    d, freqs_all = h5model.read_model(os.path.join(folder, "Analysis_of_a_rectangular_plate.hdf5"), _Desc)
    freqs_out, xs, dof_map = h5model.read_solution(
        os.path.join(folder, "eGenOutput_Analysis_of_a_rectangular_plate.hdf5"))
    assert np.allclose(freqs_out, freqs_all, rtol=0, atol=1e-9), "solution steps differ from the analysis"
    assert np.all(xs.imag == 0.0)
    assert len(d.blocks) == 1 and len(d.materials) == 1
    typ, _, conn = d.blocks[0]
    mat = d.materials[0]
    keep = np.arange(0, len(freqs_all), 2)
    np.savez_compressed(
        args.out,
        node_ids=d.node_ids, coords=d.coords, elem_type=np.array(typ), elem_conn=conn.astype(np.int64),
        material=np.array([mat["kind"], mat["E"], mat["nu"], mat["rho"], mat["t"]]),
        fixed_node=d.fixed["node"], fixed_dof=d.fixed["dof"], fixed_value=d.fixed["value"],
        force_node=d.forces["node"], force_f=d.forces["f"],
        dof_map=dof_map, freqs=freqs_out[keep], solutions=xs.real[keep])
    print(f"wrote {args.out}: {len(d.node_ids)} nodes, {len(conn)} elements, {len(d.fixed['node'])} fixed dofs, "
          f"{len(keep)} of {len(freqs_all)} frequencies")


if __name__ == "__main__":
    main()
