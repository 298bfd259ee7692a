"""Synthetic workloads of the stage operator: meshes, boundary tables, static
data and initial states for the periodic vortex, the IMEX channel with a bump
and Manning friction, the lake at rest and the random hp mesh.

Each builder returns a configured :class:`OceanoOperator` and the initial
state as NumPy arrays (DoFHandler order).  The same inputs drive the FP64
oracle in the tests.
"""
from __future__ import annotations

import numpy as np

from .icbc import channel_problem_data, nodal_points, vortex as vortex_np, vortex_params
from .mesh import (channel_mesh, concatenate_meshes, disk_refined_mesh, random_hp_mesh,
                   vortex_mesh)
from .operator import OceanoOperator

CHANNEL_Q_IN = 4.42      # inflow discharge per unit width (m^2/s)
CHANNEL_MANNING = 0.03   # Manning coefficient
CHANNEL_BCS = {0: ("wall",), 1: ("discharge_inflow", (0.0, CHANNEL_Q_IN, 0.0)),
               2: ("height_inflow", (0.0, 0.0, 0.0))}
LAKE_BCS = {0: ("wall",), 1: ("wall",), 2: ("wall",)}


def uniform_state(mesh, zeta=0.0, q=(0.0, 0.0)):
    """Constant free surface and discharge in the FE_DGQ / FESystem layout
    (zeta cell-major; q component-blocked per cell)."""
    off = mesh.offsets()
    n = int(off[-1])
    z = np.full(n, float(zeta))
    qq = np.zeros(2 * n)
    nd = np.diff(off)
    for c in range(mesh.n_cells):
        qq[2 * off[c]:2 * off[c] + nd[c]] = q[0]
        qq[2 * off[c] + nd[c]:2 * off[c] + 2 * nd[c]] = q[1]
    return z, qq


def apply_bcs(op, bcs):
    for bid, spec in bcs.items():
        kind = spec[0]
        if kind == "wall":
            op.set_wall_boundary(bid)
        elif len(spec) > 1 and spec[1] == "vortex":
            op.set_boundary(bid, kind, "vortex")
        else:
            op.set_boundary(bid, kind, "constant", spec[1] if len(spec) > 1 else (0, 0, 0))


def vortex_operator(mesh, precision, vx=None, cell_quadrature="default"):
    """Operator of the vortex runs: walls (id 0), the vortex data; the mixed form
    measures zeta and q from the undisturbed background (depth h0, discharge
    h0 u_inf)."""
    vx = vx or vortex_params()
    op = OceanoOperator(mesh, precision=precision,
                        zeta_reference=vx[0] if precision == "mixed" else 0.0,
                        cell_quadrature=cell_quadrature)
    if precision == "mixed":
        op.set_reference_state(vx[0], (vx[0] * vx[1], 0.0))
    op.set_wall_boundary(0)
    op.set_vortex(*vx)
    return op


def vortex(refine=4, degree=3, precision="fp64"):
    """Travelling vortex on [0,2]x[0,1], periodic in x, walls in y."""
    mesh = vortex_mesh(refine, degree)
    vx = vortex_params()
    op = vortex_operator(mesh, precision, vx)
    op.set_vortex(*vx)
    n = op.n_dofs
    z, q = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, z, q)
    return op, z, q


def hp_vortex(precision="mixed", target=60000, seed=20261203):
    """The vortex on the seeded random hp mesh (degrees 1-4, hanging faces)."""
    mesh = random_hp_mesh(seed=seed, target=target)
    vx = vortex_params()
    op = vortex_operator(mesh, precision, vx)
    n = op.n_dofs
    z, q = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, z, q)
    return op, z, q


def channel(precision="fp64", nx=250, ny=10, degree=2, lake=False):
    """[0,25]x[0,1] channel over the bump zb = 2 - b(x), Manning n = 0.03 treated
    implicitly (ARK).  Flow: discharge 4.42 in at x = 0, zeta = 0 out at x = 25,
    walls in y, started from zeta = 0 and the inflow discharge.  Lake at rest
    (`lake=True`): walls everywhere, zeta = 0, q = 0."""
    mesh = channel_mesh(degree, nx, ny)
    op = OceanoOperator(mesh, friction="manning", precision=precision)
    if precision == "mixed":  # background: 2 m depth at rest level, the inflow discharge
        op.set_reference_state(2.0, (0.0 if lake else CHANNEL_Q_IN, 0.0))
    apply_bcs(op, LAKE_BCS if lake else CHANNEL_BCS)
    op.initialize_data_at_quadrature(channel_problem_data(CHANNEL_MANNING))
    z, q = uniform_state(mesh, 0.0, (0.0, 0.0) if lake else (CHANNEL_Q_IN, 0.0))
    return op, z, q


# ---- ensemble of independent vortices ---------------------------------------------
# Refined-disk meshes: with radii (2, 1.4, 1) x scale refined at levels 2, 3, 4 of
# the 20x10 grid, a scale s adds about 419,800 s^2 cells to the 3,200 of level 2.
_DISK_CELLS_PER_SCALE2 = 419800.0


def ensemble_members(n=64, seed0=1000):
    """Member i draws, from MT19937(seed0 + i): centre U([0.3,1.7]x[0.3,0.7]),
    radius U[0.1,0.25], peak speed U[0.05,0.2] and a mesh size U[5k,40k] cells."""
    out = []
    for i in range(n):
        rng = np.random.Generator(np.random.MT19937(seed0 + i))
        cx, cy = rng.uniform(0.3, 1.7), rng.uniform(0.3, 0.7)
        r0, peak = rng.uniform(0.1, 0.25), rng.uniform(0.05, 0.2)
        target = rng.uniform(5000.0, 40000.0)
        out.append(dict(center=(cx, cy), r0=r0, peak=peak, target=target,
                        vortex=vortex_params(1.0, 1.0, r0, peak, cx, cy)))
    return out


def member_mesh(m):
    scale = np.sqrt(max(m["target"] - 3200.0, 0.0) / _DISK_CELLS_PER_SCALE2)
    return disk_refined_mesh(m["center"], scale, degree_radius=1.5 * m["r0"])


def vortex_nodal_state(mesh, vx, t=0.0):
    """Nodal interpolation of the vortex (zb = 0: zeta = depth) in the operator layout."""
    pts = nodal_points(mesh)
    h, u, v = vortex_np(pts[:, 0], pts[:, 1], t, *vx)
    off = mesh.offsets()
    nd = np.diff(off)
    cell = np.repeat(np.arange(mesh.n_cells), nd)      # cell of every DoF
    iu = off[cell] + np.arange(len(h))                   # hu of DoF g: 2 off + (g - off)
    q = np.zeros(2 * len(h))
    q[iu] = h * u
    q[iu + nd[cell]] = h * v
    return h.copy(), q


def member_time_steps(op, zeta, q, member_of_cell, cfl):
    """Own step size of every member of a union mesh: dt_m = cfl / (maximum of the
    member's per-cell transport speeds).  Returns (dt_ref = min dt_m, per-cell
    scale dt_m / dt_ref) for OceanoOperator.set_cell_time_scale."""
    sp = op.cell_transport_speed(zeta, q)
    sp = sp.cpu().numpy() if hasattr(sp, "cpu") else np.asarray(sp)
    member_of_cell = np.asarray(member_of_cell)
    vmax = np.zeros(member_of_cell.max() + 1)
    np.maximum.at(vmax, member_of_cell, sp)
    dt_m = cfl / vmax
    dt_ref = float(dt_m.min())
    return dt_ref, (dt_m / dt_ref)[member_of_cell]


def ensemble(n=64, precision="mixed", seed0=1000, members=None):
    """All members as one operator over the disjoint union of their meshes
    (periodic in x, walls in y), advanced by one launch per stage.  Each member
    keeps its own step size through member_time_steps + set_cell_time_scale.
    Returns (op, zeta, q, members, meshes)."""
    members = members or ensemble_members(n, seed0)
    meshes = [member_mesh(m) for m in members]
    mesh = concatenate_meshes(meshes)
    op = vortex_operator(mesh, precision, members[0]["vortex"])
    zs, qs = zip(*[vortex_nodal_state(m, mm["vortex"]) for m, mm in zip(meshes, members)])
    return op, np.concatenate(zs), np.concatenate(qs), members, meshes
