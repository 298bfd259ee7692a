"""Shared parity cases: meshes, boundary tables, static data and stage inputs.

Every case builds the same inputs for the GPU operator and the FP64 oracle.
"""
from __future__ import annotations

import numpy as np

from oceano_gb300 import QuadForest, uniform_mesh, vortex_mesh
from oceano_gb300.icbc import channel_problem_data, vortex_params

VORTEX = vortex_params()


def hanging_mesh(degree=2, seed=3, periodic=True):
    """Small forest with hanging faces (random refinement, 2:1 balanced)."""
    rng = np.random.default_rng(seed)
    f = QuadForest(4, 2, (0.0, 2.0, 0.0, 1.0), periodic_x=periodic)
    f.refine_global(1)
    for _ in range(2):
        for leaf in sorted(f.leaves):
            if rng.random() < 0.3:
                f.refine(leaf)
    f.balance()
    return f.build(degree)


def mixed_degree(mesh, seed=5, degrees=(1, 2, 3, 4)):
    rng = np.random.default_rng(seed)
    return mesh.with_degree(rng.choice(np.asarray(degrees, np.int32), mesh.n_cells))


def perturbed_state(orc, seed=0, amp=1e-3):
    """Vortex projection plus a smooth random perturbation (non-trivial faces)."""
    z, q = orc.project_vortex(0.0)
    rng = np.random.default_rng(seed)
    z = z + amp * rng.standard_normal(z.shape)
    q = q + amp * rng.standard_normal(q.shape)
    return z, q


def static_arrays(orc, problem_data):
    """Static-data arrays in the oracle's point order (cell0..bnd)."""
    out = []
    for which in range(5):
        xy = orc.points(which)
        d = np.asarray(problem_data(xy[:, 0], xy[:, 1])).reshape(5, -1)
        if which == 0:
            out.append(np.ascontiguousarray(d.T).ravel())
        elif which == 2:
            out.append(np.ascontiguousarray(d[:2].T).ravel())
        else:
            out.append(np.ascontiguousarray(d[0]))
    return out


def bump_problem_data(x, y):
    zb = 1.0 - 0.3 * np.exp(-10 * ((x - 1.0) ** 2 + (y - 0.5) ** 2))
    return np.stack([zb, 0.02 + 0 * x, 1e-3 + 0 * x, -2e-3 + 0 * x, 0.5 + 0 * x])


CASES = {
    # name: (mesh factory, bcs, problem data or None, friction)
    "vortex_p1": (lambda: vortex_mesh(0, 1), {0: ("wall",)}, None, 0),
    "vortex_p2": (lambda: vortex_mesh(0, 2), {0: ("wall",)}, None, 0),
    "vortex_p3": (lambda: vortex_mesh(0, 3), {0: ("wall",)}, None, 0),
    "vortex_p4": (lambda: vortex_mesh(0, 4), {0: ("wall",)}, None, 0),
    "hanging_p2": (lambda: hanging_mesh(2), {0: ("wall",)}, None, 0),
    "hanging_p3_bathy": (lambda: hanging_mesh(3, seed=7), {0: ("wall",)}, bump_problem_data, 2),
    "mixed_degree": (lambda: mixed_degree(hanging_mesh(2, seed=11)), {0: ("wall",)}, None, 0),
    "open_bcs_p2": (lambda: uniform_mesh(8, 4, (0.0, 2.0, 0.0, 1.0), False, 2),
                    {0: ("wall",), 1: ("supercritical_inflow", "vortex"),
                     2: ("supercritical_outflow",)}, None, 0),
    "absorbing_p3": (lambda: uniform_mesh(6, 3, (0.0, 2.0, 0.0, 1.0), False, 3),
                     {0: ("wall",), 1: ("height_inflow", (1.0005, 0, 0)),
                      2: ("absorbing_outflow", (1.0, 0.9, 0.0))}, None, 0),
    "discharge_in_p2": (lambda: uniform_mesh(6, 3, (0.0, 2.0, 0.0, 1.0), False, 2),
                        {0: ("wall",), 1: ("discharge_inflow", (0.0, 0.95, 0.0)),
                         2: ("height_inflow", (0.0, 0, 0))}, bump_problem_data, 2),
}
