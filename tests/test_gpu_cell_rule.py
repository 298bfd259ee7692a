"""The secondary cell quadrature: n_points_1d = p + 1 (4x4 Gauss points at p = 3).

The reference's only free quadrature parameter is n_points_1d (main.cc:216,
OceanDG.h:448): the Gauss rule of the cell integrals, of the boundary faces,
of the cell and boundary static data and of compute_errors_hydro; the mass
rules (Gauss-Lobatto p+2 for zeta, Gauss p+1 for the discharge) and the inner
faces (Gauss-Lobatto) are fixed.  The operator built with
cell_quadrature="p+1" is compared with the oracle built with the same rule:
FP64 stages within 1e-12 on every parity case (hanging faces, mixed degrees,
every boundary kind, bathymetry and friction, ARK), mixed stages within 1e-6,
and the 320x160 degree-3 vortex (the benchmark workload under this rule) after
three SSP-RK3 steps, FP64 and mixed.
"""
import numpy as np
import pytest

from cases import CASES, VORTEX
from oracle import oracle as O
from test_gpu_parity import TOL_FP64, rel, run_erk_stage, setup

pytestmark = pytest.mark.gpu

RULE = "p+1"


@pytest.mark.parametrize("name", sorted(CASES))
def test_erk_stage_fp64_rule_p1(gpu_lib, name):
    _, orc, op = setup(name, cell_quadrature=RULE)
    r = run_erk_stage(orc, op, 1, np.array([0.001, 0.001]), seed=5)
    o, g = r["oracle"], r["gpu"]
    for k in ("kz", "kq", "nz", "nq"):
        assert rel(g[k], o[k]) < TOL_FP64, k


@pytest.mark.parametrize("name", ["hanging_p3_bathy", "discharge_in_p2"])
def test_ark_step_fp64_rule_p1(gpu_lib, name):
    """Whole ARK steps (implicit friction, static data at the p + 1 points)."""
    _, orc, op = setup(name, cell_quadrature=RULE)
    from cases import perturbed_state
    z, q = perturbed_state(orc, 2)
    zg, qg = z.copy(), q.copy()
    tb, ti = O.TABLEAUX["giraldo32"], O.TABLEAUX["trbdf2"]
    dt = 0.003
    for it in range(2):
        O.ark_step(orc, tb["a"], tb["b"], tb["c"], ti["a"], ti["d"], it * dt, dt, z, q)
        op.perform_time_step("ark_stage3_order2", it * dt, dt, zg, qg)
    assert rel(zg, z) < TOL_FP64 and rel(qg, q) < TOL_FP64


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree", "absorbing_p3"])
def test_mixed_stage_rule_p1(gpu_lib, name):
    _, orc, op = setup(name, precision="mixed", zeta_reference=1.0,
                       reference_state=(1.0, (1.0, 0.0)), cell_quadrature=RULE)
    r = run_erk_stage(orc, op, 1, np.array([0.001, 0.001]), seed=9, k_amp=1e-4)
    o, g = r["oracle"], r["gpu"]
    assert rel(g["nz"], o["nz"]) < 1e-6 and rel(g["nq"], o["nq"]) < 1e-6


def test_rule_p1_points_sizes_and_errors(gpu_lib):
    """Static-data sizes and points at the p + 1 rule, and compute_errors_hydro."""
    from cases import perturbed_state
    _, orc, op = setup("hanging_p3_bathy", cell_quadrature=RULE)
    assert [op.static_data_size(k) for k in range(5)] == list(orc.static_sizes())
    for which in (0, 4):
        assert np.allclose(op.quadrature_points(which), orc.points(which), rtol=0, atol=1e-14)
    z, q = perturbed_state(orc, 1)
    assert np.allclose(op.compute_errors_hydro(0.01, z, q), orc.errors_vortex(z, q, 0.01),
                       rtol=1e-11)


def test_rule_p1_differs_from_default_at_p3(gpu_lib):
    """At p = 3 the two rules integrate the nonlinear flux differently (4 against
    5 points), at p = 1 they coincide (floor(1.5) + 1 = 2 = p + 1)."""
    for name, same in (("vortex_p1", True), ("vortex_p3", False)):
        _, orc0, op0 = setup(name)
        _, orc1, op1 = setup(name, cell_quadrature=RULE)
        r0 = run_erk_stage(orc0, op0, 1, np.array([0.001, 0.001]), seed=3)
        r1 = run_erk_stage(orc1, op1, 1, np.array([0.001, 0.001]), seed=3)
        d = rel(r1["gpu"]["kq"], r0["gpu"]["kq"])
        assert (d < 1e-15) if same else (d > 1e-8), (name, d)


def test_vortex_p3_320x160_rule_p1(gpu_lib):
    """The benchmark vortex (320x160, degree 3) under the 4x4 cell rule: three
    SSP-RK3 steps at CFL 0.05, FP64 within 1e-12 and mixed within 1e-6 of the
    oracle with the same rule."""
    import torch
    from oceano_gb300 import vortex_mesh
    from oceano_gb300.workloads import vortex_operator
    mesh = vortex_mesh(4, 3)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0], cell_rule=1)
    op = vortex_operator(mesh, "fp64", VORTEX, cell_quadrature=RULE)
    opm = vortex_operator(mesh, "mixed", VORTEX, cell_quadrature=RULE)
    z, q = orc.project_vortex(0.0)
    dt = 0.05 / orc.transport_speed(z, q)
    zd, qd = torch.from_numpy(z.copy()).cuda(), torch.from_numpy(q.copy()).cuda()
    zm, qm = torch.from_numpy(z.copy()).cuda(), torch.from_numpy(q.copy()).cuda()
    tb = O.TABLEAUX["ssp33"]
    for it in range(3):
        t = it * dt
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], t, dt, z, q)
        op.perform_time_step("ssp33", t, dt, zd, qd)
        opm.perform_time_step("ssp33", t, dt, zm, qm)
        op.synchronize()
        opm.synchronize()
        assert rel(zd.cpu().numpy(), z) < TOL_FP64 and rel(qd.cpu().numpy(), q) < TOL_FP64
        em = rel(zm.cpu().numpy(), z), rel(qm.cpu().numpy(), q)
        assert em[0] < 1e-6 and em[1] < 1e-6, em


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_time_steps_rule_p1_mixed_degrees(gpu_lib, precision):
    """Whole SSP-RK3 steps on a mixed-degree hanging mesh under the p + 1 rule
    (per-group launches: the one-launch hp kernel is built for the default rule):
    FP64 within 1e-12, mixed within 1e-6 of the oracle."""
    _, orc, op = setup("mixed_degree", precision=precision, cell_quadrature=RULE,
                       **({"zeta_reference": 1.0, "reference_state": (1.0, (1.0, 0.0))}
                          if precision == "mixed" else {}))
    z, q = orc.project_vortex(0.0)
    zg, qg = z.copy(), q.copy()
    dt = 0.075 / orc.transport_speed(z, q)
    tb = O.TABLEAUX["ssp33"]
    for it in range(2):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
        op.perform_time_step("ssp33", it * dt, dt, zg, qg)
    assert op.launch_config["one_launch"] is False
    tol = TOL_FP64 if precision == "fp64" else 1e-6
    assert rel(zg, z) < tol and rel(qg, q) < tol
