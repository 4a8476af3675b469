"""Seeded synthetic models with the shapes, sizes and value distributions of
the five benchmark configurations (no public dataset exists for this path).

  solid_plate   20x20x2 Brick8 steel plate, clamped edges, f = 100 Hz
  solid_cube    structured Brick8 cube, perturbed interior, 4 random materials
  plate_cavity  DSG4 plate on z = 0 coupled by InterfaceMindlin quads to a
                Fluid8 air cavity (the cavity occupies 0 <= z <= depth)
  plate         simply supported DSG4 plate (batched / serving models)

Element node order follows the reference's local numbering (Brick8 and
Fluid8: element/structure/linear/brick/elementstructurebrick8.cpp:31-57;
quads counter-clockwise, shape/shapefunctions.cpp LagrangeQuad4).
"""
from __future__ import annotations

import numpy as np

from . import (AF_LIN_UAF_ISO_DIR, BRICK8, DOF, DSG4, FLUID8, STR_LIN_ELA_ISO_DIR, STR_LIN_VIS_ISO_DIR,
               ModelDesc)

SEED = 20260101


def _grid3(nx, ny, nz, lx, ly, lz, x0=(0.0, 0.0, 0.0)):
    xs = np.linspace(0.0, lx, nx + 1) + x0[0]
    ys = np.linspace(0.0, ly, ny + 1) + x0[1]
    zs = np.linspace(0.0, lz, nz + 1) + x0[2]
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    return coords


def _hex_conn(nx, ny, nz):
    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")
    conn = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)],
                    axis=1)
    return conn.astype(np.int32)


def _quad_conn(nx, ny):
    def nid(i, j):
        return i + (nx + 1) * j
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    i, j = i.ravel(order="F"), j.ravel(order="F")
    return np.stack([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)], axis=1).astype(np.int32)


def solid_plate(nx=20, ny=20, nz=2, lx=1.0, ly=1.0, lz=0.01, E=210e9, nu=0.3, rho=7850.0, eta=0.01):
    """Clamped steel block plate: all nodes on x = 0 and x = lx fixed (x1 x2 x3),
    unit z force at the centre node of the top face."""
    coords = _grid3(nx, ny, nz, lx, ly, lz)
    n = len(coords)
    conn = _hex_conn(nx, ny, nz)
    mats = [dict(kind=STR_LIN_VIS_ISO_DIR, E=E, nu=nu, rho=rho, eta=eta, visco_type=1)]
    edge = np.where((np.abs(coords[:, 0]) < 1e-12) | (np.abs(coords[:, 0] - lx) < 1e-12))[0]
    fnode, fdof = [], []
    for v in edge:
        for d in (DOF["disp_x1"], DOF["disp_x2"], DOF["disp_x3"]):
            fnode.append(v)
            fdof.append(d)
    centre = int(np.argmin(np.sum((coords - np.array([lx / 2, ly / 2, lz])) ** 2, axis=1)))
    return ModelDesc(
        node_ids=np.arange(1, n + 1, dtype=np.int64), coords=coords, materials=mats,
        blocks=[(BRICK8, 0, conn)],
        fixed=dict(node=np.array(fnode), dof=np.array(fdof), value=np.zeros(len(fnode), complex)),
        forces=dict(node=np.array([centre]), f=np.array([[0.0, 0.0, 1.0]])), name=f"solid_plate_{nx}x{ny}x{nz}")


def solid_cube(n=100, seed=SEED, n_materials=4, perturb=0.1, fix_bottom=True):
    """n^3 Brick8 unit cube; interior nodes perturbed by U(-perturb h, +perturb h)
    per coordinate; materials E ~ U(50, 250) GPa, nu ~ U(0.25, 0.35),
    rho ~ U(2000, 8000), assigned uniformly at random per element (one
    element block per material, as the reference parser groups them)."""
    rng = np.random.default_rng(seed)
    coords = _grid3(n, n, n, 1.0, 1.0, 1.0)
    h = 1.0 / n
    interior = np.all((coords > 1e-12) & (coords < 1.0 - 1e-12), axis=1)
    coords[interior] += rng.uniform(-perturb * h, perturb * h, size=(int(interior.sum()), 3))
    conn = _hex_conn(n, n, n)
    mats = []
    for _ in range(n_materials):
        mats.append(dict(kind=STR_LIN_ELA_ISO_DIR, E=rng.uniform(50e9, 250e9), nu=rng.uniform(0.25, 0.35),
                         rho=rng.uniform(2000.0, 8000.0)))
    which = rng.integers(0, n_materials, size=len(conn))
    blocks = [(BRICK8, k, conn[which == k]) for k in range(n_materials)]
    fixed = None
    forces = None
    if fix_bottom:
        bot = np.where(np.abs(coords[:, 2]) < 1e-12)[0]
        fnode = np.repeat(bot, 3)
        fdof = np.tile(np.array([0, 1, 2]), len(bot))
        fixed = dict(node=fnode, dof=fdof, value=np.zeros(len(fnode), complex))
        top = int(np.argmin(np.sum((coords - np.array([0.5, 0.5, 1.0])) ** 2, axis=1)))
        forces = dict(node=np.array([top]), f=np.array([[0.0, 0.0, 1.0]]))
    return ModelDesc(node_ids=np.arange(1, len(coords) + 1, dtype=np.int64), coords=coords, materials=mats,
                     blocks=blocks, fixed=fixed, forces=forces, name=f"solid_cube_{n}")


def plate(mx, my, lx, ly, t, E=70e9, nu=0.33, rho=2700.0, eta=0.02, seed=SEED, force_node=None, id0=1):
    """Simply supported DSG4 plate in the z = 0 plane: w (x3) fixed on every
    boundary node, unit z force at a seeded random interior node."""
    coords = _grid3(mx, my, 0, lx, ly, 0.0)
    n = len(coords)
    conn = _quad_conn(mx, my)
    mats = [dict(kind=STR_LIN_VIS_ISO_DIR, E=E, nu=nu, rho=rho, t=t, eta=eta, visco_type=1)]
    bnd = np.where((np.abs(coords[:, 0]) < 1e-12) | (np.abs(coords[:, 0] - lx) < 1e-12) |
                   (np.abs(coords[:, 1]) < 1e-12) | (np.abs(coords[:, 1] - ly) < 1e-12))[0]
    if force_node is None:
        rng = np.random.default_rng(seed)
        ii = rng.integers(1, mx)
        jj = rng.integers(1, my)
        force_node = int(ii + (mx + 1) * jj)
    return ModelDesc(
        node_ids=np.arange(id0, id0 + n, dtype=np.int64), coords=coords, materials=mats,
        blocks=[(DSG4, 0, conn)],
        fixed=dict(node=bnd, dof=np.full(len(bnd), DOF["disp_x3"]), value=np.zeros(len(bnd), complex)),
        forces=dict(node=np.array([force_node]), f=np.array([[0.0, 0.0, 1.0]])), name=f"plate_{mx}x{my}")


def plate_cavity(mx=60, my=40, mz=30, lx=0.6, ly=0.4, depth=0.3, t=0.002, seed=SEED, ori=1.0):
    """Aluminium DSG4 plate (E 70 GPa, nu 0.33, rho 2700, eta 0.02, t 2 mm),
    simply supported, on z = 0; Fluid8 air cavity (c 343, rho 1.21) on
    0 <= z <= depth with its own nodes; one InterfaceMindlin quad per plate
    element couples plate node k to the coincident fluid node k (ori = +1)."""
    p = plate(mx, my, lx, ly, t, seed=seed)
    npl = p.n_nodes
    fcoords = _grid3(mx, my, mz, lx, ly, depth)
    nfl = len(fcoords)
    fconn = _hex_conn(mx, my, mz) + npl
    coords = np.concatenate([p.coords, fcoords], axis=0)
    ids = np.concatenate([p.node_ids, np.arange(1, nfl + 1, dtype=np.int64) + 10 ** 7])
    mats = p.materials + [dict(kind=AF_LIN_UAF_ISO_DIR, c=343.0, rho=1.21)]
    pconn = p.blocks[0][2]
    # fluid nodes of the z = 0 layer have the same (i, j) index as the plate nodes
    fq = _quad_conn(mx, my) + npl
    interfaces = dict(ori=np.full(len(pconn), ori), snodes=pconn, fnodes=fq, fmat=np.full(len(pconn), 1))
    return ModelDesc(node_ids=ids, coords=coords, materials=mats,
                     blocks=[(DSG4, 0, pconn), (FLUID8, 1, fconn)], interfaces=interfaces,
                     fixed=p.fixed, forces=p.forces, name=f"plate_cavity_{mx}x{my}x{mz}")


def batched_plates(count=256, lo=10, hi=80, seed=SEED, size=0.5):
    """`count` simply supported aluminium DSG4 plates (eta 0.02), meshes m x m
    with m ~ U{lo..hi}, t ~ U(1, 5) mm, on a size x size square."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        m = int(rng.integers(lo, hi + 1))
        t = float(rng.uniform(1e-3, 5e-3))
        out.append(plate(m, m, size, size, t, seed=seed + 1 + k))
    return out


def cube(k, seed=SEED):
    """k^3 Brick8 aluminium cube (visco eta 0.02), bottom face clamped, unit
    force on the top centre node: a serving model of 3 (k+1)^3 DOFs."""
    d = solid_cube(k, seed=seed, n_materials=1, perturb=0.1)
    d.materials = [dict(kind=STR_LIN_VIS_ISO_DIR, E=70e9, nu=0.33, rho=2700.0, eta=0.02, visco_type=1)]
    d.blocks = [(BRICK8, 0, np.concatenate([b[2] for b in d.blocks]))]
    d.name = f"cube_{k}"
    return d


def serving_models(count=8, lo=5_000, hi=500_000, seed=SEED):
    """Models of the serving stream: DOF targets log-uniform in [lo, hi]
    (seeded, stratified: one draw in each of `count` equal intervals of
    log DOFs, so the sizes cover the range), alternately a simply supported
    DSG4 shell plate (3 DOFs per node, square, 0.5 m) and a Brick8 steel slab
    clamped on two edges (1 m x 1 m x 10 cm, three element layers), each sized
    to the target. The slab is 10 cm thick rather than the 1 cm of the
    single-frequency solid plate: on the thin plate || |A| |x| || / ||f|| reaches
    1e6 at some frequencies, so no FP64 solution there has a residual below
    1e-10 (its FP64 floor); the slab's is ~1e3. Returns the descriptions
    sorted by DOF count."""
    rng = np.random.default_rng(seed + 91)
    u = (np.arange(count) + rng.uniform(0.0, 1.0, count)) / count
    targets = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))
    out = []
    for k, t in enumerate(targets):
        if k % 2 == 0:
            m = max(4, int(round(np.sqrt(t / 3.0))) - 1)
            d = plate(m, m, 0.5, 0.5, 0.003, seed=seed + 300 + k)
        else:
            m = max(4, int(round(np.sqrt(t / 12.0))) - 1)
            d = solid_plate(m, m, 3, lz=0.1)
            d.name = f"solid_slab_{m}x{m}x3"
        out.append(d)
    return sorted(out, key=lambda d: len(d.node_ids) * (3 if d.blocks[0][0] == BRICK8 else 1))
