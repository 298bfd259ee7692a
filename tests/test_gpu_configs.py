"""The benchmark configurations and every integrator against the FP64 oracle.

* The plain FP64 travelling vortex at degree 1 on 80x40 cells (SSP-RK3,
  CFL 0.2, 200 steps, the step size policy of main.cc:1504-1555), compared
  with the oracle after every step.
* The degree-3 vortex at full size (320x160 cells, 2,457,600 DoFs): three
  SSP-RK3 steps of the FP64 and of the mixed form against the oracle.
* Forward Euler, SSP22, RK4 and the explicit 3-stage order-2 scheme
  (time_stepping.h:136-255), FP64 and mixed, whole time steps.
* apply() = M^-1 L_h (OceanDG.h:1658-1691) against the oracle's apply.
* Device-side errors of calls on device vectors surface at oc_synchronize.
* Ensemble members in one operator keep their own step size.
All GPU calls go through the C ABI (ctypes binding of liboceano_gpu.so).
"""
import numpy as np
import pytest

from cases import CASES, VORTEX, perturbed_state
from oracle import oracle as O
from test_gpu_parity import TOL_FP64, rel, setup

pytestmark = pytest.mark.gpu


def vortex_pair(refine, degree, precision="fp64"):
    from oceano_gb300 import vortex_mesh
    from oceano_gb300.workloads import vortex_operator
    mesh = vortex_mesh(refine, degree)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    op = vortex_operator(mesh, precision, VORTEX)
    return mesh, orc, op


def test_vortex_p1_80x40_200_steps_cfl02(gpu_lib):
    """Plain FP64 vortex, degree 1, 80x40 cells, SSP-RK3 at CFL 0.2 for 200
    steps.  Both sides use the same step sizes (the GPU's transport speed,
    which must equal the oracle's to 1e-12, truncated to 3 digits every 5
    steps).  Bound: 1e-12 relative L2 after every step -- both sides are FP64
    and differ only by rounding order, about 1e-16 per operation; over 600
    stages of a stable scheme that stays below 1e-12 (measured: printed)."""
    from oceano_gb300.driver import TimeLoop, truncate_to_n_digits
    mesh, orc, op = vortex_pair(2, 1)
    assert mesh.n_cells == 3200 and orc.n == 12800
    z, q = orc.project_vortex(0.0)
    zg, qg = z.copy(), q.copy()
    tl = TimeLoop(op, "ssp33", 0.2)
    dt0 = tl.start(zg, qg)
    assert abs(dt0 - 0.2 / orc.transport_speed(z, q)) <= 1e-12 * dt0
    tb = O.TABLEAUX["ssp33"]
    worst = 0.0
    for it in range(200):
        dt = tl.next_time_step(zg, qg)
        if (it + 1) % 5 == 0:  # the oracle's speed gives the same truncated step
            assert dt == 0.2 / truncate_to_n_digits(orc.transport_speed(z, q), 3)
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], tl.time, dt, z, q)
        tl.advance(zg, qg, dt=dt)
        ez, eq = rel(zg, z), rel(qg, q)
        worst = max(worst, ez, eq)
        assert ez < TOL_FP64 and eq < TOL_FP64, (it, ez, eq)
    assert tl.step_number == 200
    err = op.compute_errors_hydro(tl.time, zg, qg)
    erro = orc.errors_vortex(z, q, tl.time)
    assert np.allclose(err, erro, rtol=1e-10)
    print(f"C1: worst step error {worst:.2e}, final time {tl.time:.6f}, L2 errors {err}")


def test_vortex_p3_320x160_fp64_and_mixed(gpu_lib):
    """The degree-3 vortex at full size: 3 SSP-RK3 steps at CFL 0.05.  FP64
    form within 1e-12 of the oracle after every step; mixed form (FP32 bulk,
    FP64 accumulation, reference state = the background flow) within 1e-6."""
    import torch
    mesh, orc, op = vortex_pair(4, 3)
    _, _, opm = vortex_pair(4, 3, "mixed")
    assert mesh.n_cells == 51200 and 3 * orc.n == 2457600
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
        print(f"C2 step {it + 1}: mixed vs oracle zeta {em[0]:.2e} discharge {em[1]:.2e}")


SCHEMES = {"forward_euler": "fe", "ssp22": "ssp22", "rk4": "rk4", "stage3_order2": "giraldo32"}


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_explicit_schemes(gpu_lib, scheme, precision):
    """Two whole time steps of each explicit scheme (handle-owned registers, CUDA
    graph) against the oracle's Butcher-form integrator: FP64 1e-12, mixed 1e-6."""
    kw = dict(precision="mixed", zeta_reference=1.0, reference_state=(1.0, (1.0, 0.0))) \
        if precision == "mixed" else {}
    mesh, orc, op = setup("mixed_degree", **kw)
    z, q = perturbed_state(orc, 6)
    dt = (0.02 if scheme == "forward_euler" else 0.075) / orc.transport_speed(z, q)
    tb = O.TABLEAUX[SCHEMES[scheme]]
    zo, qo = z.copy(), q.copy()
    zg, qg = z.copy(), q.copy()
    for it in range(2):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, zo, qo)
        op.perform_time_step(scheme, it * dt, dt, zg, qg)
    tol = TOL_FP64 if precision == "fp64" else 1e-6
    assert rel(zg, zo) < tol and rel(qg, qo) < tol, (rel(zg, zo), rel(qg, qo))


@pytest.mark.parametrize("name", ["vortex_p1", "hanging_p2", "mixed_degree", "hanging_p3_bathy",
                                  "open_bcs_p2", "absorbing_p3"])
def test_apply(gpu_lib, name):
    """oc_apply = M^-1 L_h(t, src) against the oracle's apply (FP64: 1e-12),
    on host and on device vectors."""
    import torch
    mesh, orc, op = setup(name)
    z, q = perturbed_state(orc, 7)
    oz, oq = orc.apply(0.013, z, q)
    dz, dq = np.zeros_like(z), np.zeros_like(q)
    op.apply(0.013, z, q, dz, dq)
    assert rel(dz, oz) < TOL_FP64 and rel(dq, oq) < TOL_FP64
    zt, qt = torch.from_numpy(z).cuda(), torch.from_numpy(q).cuda()
    dzt, dqt = torch.zeros_like(zt), torch.zeros_like(qt)
    op.apply(0.013, zt, qt, dzt, dqt)
    op.synchronize()
    assert np.array_equal(dzt.cpu().numpy(), dz) and np.array_equal(dqt.cpu().numpy(), dq)


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree"])
def test_apply_mixed(gpu_lib, name):
    """apply() of a mixed-precision handle (FP32 bulk, FP64 in and out): the
    residual of a perturbed vortex within 1e-4 relative L2 of the oracle (FP32
    rounding of a difference of O(1) fluxes, as for the stage registers)."""
    mesh, orc, op = setup(name, precision="mixed", zeta_reference=1.0,
                          reference_state=(1.0, (1.0, 0.0)))
    z, q = perturbed_state(orc, 8)
    oz, oq = orc.apply(0.0, z, q)
    dz, dq = np.zeros_like(z), np.zeros_like(q)
    op.apply(0.0, z, q, dz, dq)
    assert rel(dz, oz) < 1e-4 and rel(dq, oq) < 1e-4, (rel(dz, oz), rel(dq, oq))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_step_reports_nonfinite(gpu_lib, precision):
    """A time step on device vectors returns once enqueued; a NaN planted in the
    state shows up as OC_ERR_NONFINITE at oc_synchronize, which clears the flag."""
    import torch
    from oceano_gb300._lib import OC_ERR_NONFINITE, OceanoError
    kw = dict(precision="mixed", zeta_reference=1.0) if precision == "mixed" else {}
    mesh, orc, op = setup("vortex_p2", **kw)
    z, q = perturbed_state(orc, 2)
    dt = 0.05 / orc.transport_speed(z, q)
    zt, qt = torch.from_numpy(z.copy()).cuda(), torch.from_numpy(q.copy()).cuda()
    op.perform_time_step("ssp33", 0.0, dt, zt, qt)
    op.synchronize()  # finite: no error
    zt[17] = float("nan")
    torch.cuda.synchronize()
    op.perform_time_step("ssp33", dt, dt, zt, qt)
    with pytest.raises(OceanoError) as e:
        op.synchronize()
    assert e.value.status == OC_ERR_NONFINITE
    op.synchronize()  # cleared


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_members_keep_their_own_dt(gpu_lib, precision):
    """Independent members in one operator (one launch per stage), each with its
    own step size through per-cell time scales, against every member advanced
    alone by its own operator with its own dt: FP64 1e-13, mixed 1e-6."""
    from oceano_gb300 import workloads as W
    from oceano_gb300.indicator import member_of_cells
    mem = W.ensemble_members(3, 1000)
    for m in mem:
        m["target"] = 5000.0
    op, z, q, mem, meshes = W.ensemble(members=mem, precision=precision)
    moc = member_of_cells(meshes)
    dt_ref, scale = W.member_time_steps(op, z, q, moc, 0.075)
    assert scale.min() == 1.0 and scale.max() > 1.0  # the members' dt differ
    op.set_cell_time_scale(scale)
    zz, qq = z.copy(), q.copy()
    for it in range(3):
        op.perform_time_step("ssp33", it * dt_ref, dt_ref, zz, qq)
    off = op.mesh.offsets()
    c0 = 0
    tol = 1e-13 if precision == "fp64" else 1e-6
    for k, (m, mesh) in enumerate(zip(mem, meshes)):
        c1 = c0 + mesh.n_cells
        opk = W.vortex_operator(mesh, precision, m["vortex"])
        zk, qk = W.vortex_nodal_state(mesh, m["vortex"])
        dtk = 0.075 / opk.compute_cell_transport_speed(zk, qk)
        assert abs(dtk - dt_ref * scale[c0]) <= 1e-13 * dtk
        for it in range(3):
            opk.perform_time_step("ssp33", it * dtk, dtk, zk, qk)
        a, b = off[c0], off[c1]
        assert rel(zz[a:b], zk) < tol and rel(qq[2 * a:2 * b], qk) < tol
        opk.close()
        c0 = c1
    op.set_cell_time_scale(None)


def test_timers_by_reference_scope_names(gpu_lib):
    """oc_set_timing / oc_timer_summary: GPU time of each call under the
    reference's TimerOutput scope names, one call counted per call made."""
    mesh, orc, op = setup("vortex_p2")
    z, q = perturbed_state(orc, 1)
    dt = 0.05 / orc.transport_speed(z, q)
    op.set_timing(True)
    for it in range(4):
        op.perform_time_step("ssp33", it * dt, dt, z, q)
    op.compute_cell_transport_speed(z, q)
    n = orc.n
    kz = [np.zeros(n) for _ in range(4)]
    kq = [np.zeros(2 * n) for _ in range(4)]
    op.perform_stage_hydro(0, 3, 0.0, np.array([dt]), [z, q], kz, kq, z.copy(), q.copy(),
                           np.zeros(n), np.zeros(2 * n))
    t = op.timer_summary()
    assert t["rk time stepping total"][0] == 4 and t["rk time stepping total"][1] > 0
    assert t["compute transport speed"][0] == 1
    assert t["rk_stage hydro - integrals L_h + inv mass + vec upd"][0] == 1
