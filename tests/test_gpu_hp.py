"""hp meshes (degrees 1-4 and hanging faces in one mesh): the one-launch stage
kernel, the per-group launches and the launch autotuner give the oracle's
results.  FP64: 1e-12 relative L2 after several time steps; mixed: 1e-6."""
import numpy as np
import pytest

from cases import VORTEX, bump_problem_data, hanging_mesh, mixed_degree, static_arrays
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SSP = O.TABLEAUX["ssp33"]
GIR, TRB = O.TABLEAUX["giraldo32"], O.TABLEAUX["trbdf2"]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def make(mesh, precision, mode, friction=0, pdata=None):
    from oceano_gb300.operator import OceanoOperator
    orc = O.Oracle(mesh, friction=friction, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    op = OceanoOperator(mesh, friction=["none", "linear", "manning"][friction],
                        precision=precision, zeta_reference=1.0 if precision == "mixed" else 0.0)
    op.set_wall_boundary(0)
    op.set_vortex(*VORTEX)
    op.set_launch_mode(mode)
    if pdata is not None:
        arrs = static_arrays(orc, pdata)
        orc.set_static(*arrs)
        op.set_static_data(*arrs)
    return orc, op


def run(orc, op, steps, ark=False):
    z, q = orc.project_vortex(0.0)
    dt = 0.075 / orc.transport_speed(z, q)
    zo, qo, zg, qg = z.copy(), q.copy(), z.copy(), q.copy()
    for it in range(steps):
        if ark:
            O.ark_step(orc, GIR["a"], GIR["b"], GIR["c"], TRB["a"], TRB["d"], it * dt, dt, zo, qo)
            op.perform_time_step("ark_stage3_order2", it * dt, dt, zg, qg)
        else:
            O.erk_step(orc, SSP["a"], SSP["b"], SSP["c"], it * dt, dt, zo, qo)
            op.perform_time_step("ssp33", it * dt, dt, zg, qg)
    return zg, qg, zo, qo


@pytest.mark.parametrize("mode", ["per_group", "one", "auto"])
def test_fp64_launch_modes(gpu_lib, mode):
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    orc, op = make(mesh, "fp64", mode)
    zg, qg, zo, qo = run(orc, op, 5)
    assert rel(zg, zo) < 1e-12 and rel(qg, qo) < 1e-12
    cfg = op.launch_config
    assert cfg["tuned"] and cfg["one_launch"] == (mode == "one" or (mode == "auto" and cfg["one_launch"]))
    assert cfg["one_launch_warps"] in (2, 4) and set(cfg["group_warps"].values()) <= {1, 2, 4}


@pytest.mark.parametrize("mode", ["per_group", "one"])
def test_fp64_ark_bathymetry_launch_modes(gpu_lib, mode):
    """IMEX (Manning implicit) on an hp mesh with bathymetry and hanging faces."""
    mesh = mixed_degree(hanging_mesh(3, seed=7))
    orc, op = make(mesh, "fp64", mode, friction=2, pdata=bump_problem_data)
    zg, qg, zo, qo = run(orc, op, 4, ark=True)
    assert rel(zg, zo) < 1e-12 and rel(qg, qo) < 1e-12


def test_mixed_launch_modes_agree(gpu_lib):
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    res = {}
    for mode in ("per_group", "one"):
        orc, op = make(mesh, "mixed", mode)
        res[mode] = run(orc, op, 5)
    zo, qo = res["one"][2], res["one"][3]
    for mode, (zg, qg, _, _) in res.items():
        assert rel(zg, zo) < 1e-6 and rel(qg, qo) < 5e-6, mode
    assert rel(res["one"][0], res["per_group"][0]) < 1e-6


def test_random_hp_mesh_small(gpu_lib):
    """A small instance of the seeded random hp mesh (degrees 1-4, hanging faces)."""
    from oceano_gb300 import random_hp_mesh
    mesh = random_hp_mesh(target=3000, global_refine=1, max_extra=2)
    orc, op = make(mesh, "fp64", "one")
    zg, qg, zo, qo = run(orc, op, 3)
    assert rel(zg, zo) < 1e-12 and rel(qg, qo) < 1e-12
    orc, op = make(mesh, "mixed", "auto")
    zg, qg, zo, qo = run(orc, op, 3)
    assert rel(zg, zo) < 1e-6 and rel(qg, qo) < 5e-6
