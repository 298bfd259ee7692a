"""compute_errors_hydro and prepare_for_conservative_coarsening on the GPU
against the FP64 oracle (1e-12 relative)."""
import numpy as np
import pytest

from cases import CASES, VORTEX, bump_problem_data, hanging_mesh, mixed_degree, perturbed_state, static_arrays
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make(mesh, pdata=None):
    from oceano_gb300.operator import OceanoOperator
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    op = OceanoOperator(mesh)
    op.set_wall_boundary(0)
    op.set_vortex(*VORTEX)
    if pdata is not None:
        arrs = static_arrays(orc, pdata)
        orc.set_static(*arrs)
        op.set_static_data(*arrs)
    return orc, op


@pytest.mark.parametrize("bathy", [False, True])
def test_errors_match_oracle(gpu_lib, bathy):
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    orc, op = make(mesh, bump_problem_data if bathy else None)
    z, q = perturbed_state(orc, 5, amp=1e-3)
    for t in (0.0, 0.01):
        e = op.compute_errors_hydro(t, z, q)
        eo = orc.errors_vortex(z, q, t)
        assert np.all(np.abs(e - eo) <= 1e-12 * eo), (e, eo)


def test_errors_converge_for_the_projection(gpu_lib):
    """Errors of the projected vortex shrink under refinement (sanity of the norm)."""
    from oceano_gb300 import vortex_mesh
    errs = []
    for r in (0, 1):
        _, op = make(vortex_mesh(r, 2))
        n = op.n_dofs
        z, q = np.zeros(n), np.zeros(2 * n)
        op.project_vortex(0.0, z, q)
        errs.append(op.compute_errors_hydro(0.0, z, q))
    assert errs[1][0] < errs[0][0] / 4 and errs[1][1] < errs[0][1] / 4


@pytest.mark.parametrize("bathy", [False, True])
def test_conservative_coarsening_matches_oracle(gpu_lib, bathy):
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    orc, op = make(mesh, bump_problem_data if bathy else None)
    z, q = perturbed_state(orc, 6, amp=1e-2)
    if bathy:  # zeta between -1.2 and -0.6 against zb in [0.7, 1]: partly dry cells
        from oceano_gb300.icbc import nodal_points
        x = nodal_points(mesh)[:, 0]
        z = -0.9 + 0.3 * np.cos(np.pi * x) + 1e-3 * z
    rng = np.random.default_rng(7)
    mark = (rng.random(mesh.n_cells) < 0.5).astype(np.uint8)
    zg = z.copy()
    op.prepare_for_conservative_coarsening(mark, zg)
    zo = orc.conservative_coarsening(mark, z)
    assert np.abs(zg - zo).max() <= 1e-12 * np.abs(zo).max()
    off = mesh.offsets()
    untouched = np.concatenate([np.arange(off[c], off[c + 1]) for c in np.nonzero(mark == 0)[0]])
    assert np.array_equal(zg[untouched], z[untouched])
