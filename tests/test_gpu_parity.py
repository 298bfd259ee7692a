"""Parity of the GPU stage with the FP64 oracle, through the C ABI.

Plain FP64 form: 1e-12 relative L2 per stage output (the bar the reference
sets for its FP64 path).  Mixed form: errors against the same oracle are
reported and bounded (tolerances written in each test).
"""
import numpy as np
import pytest

from cases import CASES, VORTEX, perturbed_state, static_arrays
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def setup(name, precision="fp64", batch=1, zeta_reference=0.0, reference_state=None,
          cell_quadrature="default"):
    from oceano_gb300 import _lib
    from oceano_gb300.operator import OceanoOperator
    mesh_f, bcs, pdata, friction = CASES[name]
    mesh = mesh_f()
    orc = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0], batch=batch,
                   cell_rule=_lib.CELL_RULE[cell_quadrature])
    op = OceanoOperator(mesh, friction=["none", "linear", "manning"][friction],
                        precision=precision, batch_width=batch, zeta_reference=zeta_reference,
                        cell_quadrature=cell_quadrature)
    for b, spec in bcs.items():
        if len(spec) > 1 and spec[1] == "vortex":
            op.set_boundary(b, spec[0], "vortex")
        elif len(spec) > 1:
            op.set_boundary(b, spec[0], "constant", spec[1])
        else:
            op.set_boundary(b, spec[0])
    op.set_vortex(*VORTEX)
    if reference_state is not None:
        op.set_reference_state(*reference_state)
    if pdata is not None:
        arrs = static_arrays(orc, pdata)
        orc.set_static(*arrs)
        op.set_static_data(*arrs)
    return mesh, orc, op


def erk_inputs(orc, stage, seed, k_amp=1e-2):
    """Random stage registers: large ones (1e-2) also drive cells dry, which
    exercises the wet/dry branches of the zeta inverse."""
    n = orc.n
    z, q = perturbed_state(orc, seed)
    rng = np.random.default_rng(100 + seed)
    rz = z + 1e-4 * rng.standard_normal(n)
    rq = q + 1e-4 * rng.standard_normal(2 * n)
    kz = [np.zeros(n)] + [k_amp * rng.standard_normal(n) for _ in range(3)]
    kq = [np.zeros(2 * n)] + [k_amp * rng.standard_normal(2 * n) for _ in range(3)]
    return z, q, rz, rq, kz, kq


def run_erk_stage(orc, op, stage, f, seed=0, t=0.01, k_amp=1e-2):
    z, q, rz, rq, kz, kq = erk_inputs(orc, stage, seed, k_amp)
    n = orc.n
    res = {}
    for who in ("oracle", "gpu"):
        sz, sq = z.copy(), q.copy()
        kzc = [k.copy() for k in kz]
        kqc = [k.copy() for k in kq]
        nz, nq = np.zeros(n), np.zeros(2 * n)
        if who == "oracle":
            orc.stage_erk(stage, 3, t, f, rz, rq, kzc, kqc, sz, sq, nz, nq)
        else:
            op.perform_stage_hydro(stage, 3, t, f, [rz, rq], kzc, kqc, sz, sq, nz, nq)
        res[who] = dict(kz=kzc[stage + 1], kq=kqc[stage + 1], sz=sz, sq=sq, nz=nz, nq=nq)
    return res


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("stage", [0, 1, 2])
def test_erk_stage_fp64(gpu_lib, name, stage):
    mesh, orc, op = setup(name)
    f = [[0.004], [0.001, 0.001], [0.004 / 6, 0.004 / 6, 0.008 / 3]][stage]
    r = run_erk_stage(orc, op, stage, np.array(f), seed=stage)
    o, g = r["oracle"], r["gpu"]
    assert rel(g["kz"], o["kz"]) < TOL_FP64
    assert rel(g["kq"], o["kq"]) < TOL_FP64
    if stage == 2:
        assert rel(g["sz"], o["sz"]) < TOL_FP64
        assert rel(g["sq"], o["sq"]) < TOL_FP64
    else:
        assert rel(g["nz"], o["nz"]) < TOL_FP64
        assert rel(g["nq"], o["nq"]) < TOL_FP64


@pytest.mark.parametrize("batch", [1, 2])
def test_erk_batch_stop_rule(gpu_lib, batch):
    mesh, orc, op = setup("vortex_p2", batch=batch)
    r = run_erk_stage(orc, op, 1, np.array([0.001, 0.001]), seed=4)
    assert rel(r["gpu"]["nz"], r["oracle"]["nz"]) < TOL_FP64


def ark_inputs(orc, seed):
    n = orc.n
    z, q = perturbed_state(orc, seed)
    rng = np.random.default_rng(200 + seed)
    rz = z + 1e-4 * rng.standard_normal(n)
    rq = q + 1e-4 * rng.standard_normal(2 * n)
    kz = [np.zeros(n)] + [1e-2 * rng.standard_normal(n) for _ in range(3)]
    kq = [np.zeros(2 * n)] + [1e-2 * rng.standard_normal(2 * n) for _ in range(5)]
    return z, q, rz, rq, kz, kq


@pytest.mark.parametrize("name", ["hanging_p3_bathy", "discharge_in_p2", "vortex_p2"])
@pytest.mark.parametrize("stage", [0, 1, 2])
def test_ark_stage_fp64(gpu_lib, name, stage):
    mesh, orc, op = setup(name)
    n = orc.n
    tb = O.TABLEAUX
    dt = 0.003
    er, im = tb["giraldo32"], tb["trbdf2"]
    last = stage == 2
    f = np.array(er["b"] if last else er["a"][stage]) * dt
    ft = np.array(er["b"] if last else im["a"][stage]) * dt
    fm = im["d"][stage] * dt if stage < 2 else 0.0
    z, q, rz, rq, kz, kq = ark_inputs(orc, stage)
    res = {}
    for who in ("oracle", "gpu"):
        sz, sq = z.copy(), q.copy()
        kzc = [k.copy() for k in kz]
        kqc = [k.copy() for k in kq]
        nz, nq = np.zeros(n), np.zeros(2 * n)
        if who == "oracle":
            orc.stage_ark(stage, 3, 0.02, f, ft, fm, rz, rq, kzc, kqc, sz, sq, nz, nq)
        else:
            op.perform_stage_hydro(stage, 3, 0.02, f, [rz, rq], kzc, kqc, sz, sq, nz, nq,
                                   factor_tilde_residual=ft, factor_matrix=fm)
        res[who] = dict(kz=kzc, kq=kqc, sz=sz, sq=sq, nz=nz, nq=nq)
    o, g = res["oracle"], res["gpu"]
    assert rel(g["kz"][stage + 1], o["kz"][stage + 1]) < TOL_FP64
    assert rel(g["kq"][2 * stage + 1], o["kq"][2 * stage + 1]) < TOL_FP64
    if not last:
        assert rel(g["kq"][2 * stage + 2], o["kq"][2 * stage + 2]) < TOL_FP64
        assert rel(g["nz"], o["nz"]) < TOL_FP64
        assert rel(g["nq"], o["nq"]) < TOL_FP64
    else:
        assert rel(g["sz"], o["sz"]) < TOL_FP64
        assert rel(g["sq"], o["sq"]) < TOL_FP64
        assert rel(g["nq"], o["nq"]) < TOL_FP64


# reference states of the mixed form: none (q_r = 0) and a background flow that
# is not aligned with the mesh (exercises every deviation term)
REF_STATES = {"no_ref": None, "ref": (1.0, (0.8, 0.3))}


@pytest.mark.parametrize("ref", sorted(REF_STATES))
@pytest.mark.parametrize("name", ["vortex_p1", "vortex_p3", "vortex_p4", "hanging_p2",
                                  "mixed_degree", "hanging_p3_bathy", "open_bcs_p2",
                                  "absorbing_p3", "discharge_in_p2"])
def test_mixed_stage_error(gpu_lib, name, ref):
    """Mixed form vs the FP64 oracle on wet states: stage output within 1e-6
    relative L2 (FP32 bulk), residual registers within 1e-4 (FP32 rounding of
    a residual that is itself a difference of O(1) fluxes)."""
    mesh, orc, op = setup(name, precision="mixed", zeta_reference=1.0,
                          reference_state=REF_STATES[ref])
    r = run_erk_stage(orc, op, 1, np.array([0.001, 0.001]), seed=9, k_amp=1e-4)
    o, g = r["oracle"], r["gpu"]
    assert rel(g["nz"], o["nz"]) < 1e-6
    assert rel(g["nq"], o["nq"]) < 1e-6
    assert rel(g["kz"], o["kz"]) < 1e-4
    assert rel(g["kq"], o["kq"]) < 1e-4


def test_mixed_dry_cells_fall_back(gpu_lib):
    """Registers that dry cells out: the mixed form switches those cells to the
    FP64 literal iteration; wet/dry masks of FP32-perturbed inputs may differ,
    so only a loose bound holds (documented behaviour)."""
    mesh, orc, op = setup("vortex_p4", precision="mixed", zeta_reference=1.0)
    r = run_erk_stage(orc, op, 1, np.array([0.001, 0.001]), seed=9, k_amp=1e-2)
    assert rel(r["gpu"]["nz"], r["oracle"]["nz"]) < 1e-3


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree"])
def test_mixed_trajectory(gpu_lib, name):
    """10 SSP-RK3 steps of the mixed form vs the FP64 form on the GPU and the
    oracle: relative L2 state error <= 1e-6."""
    mesh, orc, op = setup(name, precision="mixed", zeta_reference=1.0)
    _, _, op64 = setup(name)
    _, _, opr = setup(name, precision="mixed", zeta_reference=1.0,
                      reference_state=(1.0, (1.0, 0.0)))  # the vortex background
    z0, q0 = orc.project_vortex(0.0)
    dt = 0.075 / orc.transport_speed(z0, q0)  # stable SSP-RK3 Courant number up to p = 4
    zo, qo = z0.copy(), q0.copy()
    zm, qm = z0.copy(), q0.copy()
    zd, qd = z0.copy(), q0.copy()
    zr, qr = z0.copy(), q0.copy()
    for it in range(10):
        O.erk_step(orc, TAB["a"], TAB["b"], TAB["c"], it * dt, dt, zo, qo)
        op.perform_time_step("ssp33", it * dt, dt, zm, qm)
        op64.perform_time_step("ssp33", it * dt, dt, zd, qd)
        opr.perform_time_step("ssp33", it * dt, dt, zr, qr)
    assert rel(zd, zo) < 1e-12 and rel(qd, qo) < 1e-12
    assert rel(zm, zo) < 1e-6 and rel(qm, qo) < 5e-6
    # deviations from the background: the FP32 error of the discharge drops (its
    # rounding no longer scales with |q| ~ 1 but with |q - q_r| ~ 0.1)
    assert rel(zr, zo) < 1e-6 and rel(qr, qo) < 1e-6
    assert rel(qr, qo) < 0.5 * rel(qm, qo)


@pytest.mark.parametrize("name", ["vortex_p1", "hanging_p2", "mixed_degree", "hanging_p3_bathy"])
def test_transport_speed(gpu_lib, name):
    mesh, orc, op = setup(name)
    z, q = perturbed_state(orc, 1)
    assert abs(op.compute_cell_transport_speed(z, q) - orc.transport_speed(z, q)) <= \
        1e-12 * orc.transport_speed(z, q)


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree"])
def test_projection_velocity_vorticity(gpu_lib, name):
    mesh, orc, op = setup(name)
    n = orc.n
    z, q = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, z, q)
    zo, qo = orc.project_vortex(0.0)
    assert rel(z, zo) < 1e-13 and rel(q, qo) < 1e-13
    u = np.zeros(2 * n)
    op.evaluate_velocity_field(z, q, u)
    uo = orc.velocity_field(zo, qo)
    assert rel(u, uo) < 1e-13
    ind = np.zeros(mesh.n_cells, np.float32)
    op.vorticity_indicator(u, int(mesh.degree.max()), ind)
    io = orc.vorticity(uo, int(mesh.degree.max()))
    assert np.allclose(ind, io, rtol=1e-5, atol=1e-6)


def test_time_step_matches_stages(gpu_lib):
    """oc_perform_time_step (graph, handle-owned registers) == the stage sequence."""
    mesh, orc, op = setup("hanging_p2")
    z, q = perturbed_state(orc, 2)
    dt = 0.075 / orc.transport_speed(z, q)
    zs, qs = z.copy(), q.copy()
    O.erk_step(orc, TAB["a"], TAB["b"], TAB["c"], 0.0, dt, zs, qs)
    zg, qg = z.copy(), q.copy()
    op.perform_time_step("ssp33", 0.0, dt, zg, qg)
    assert rel(zg, zs) < TOL_FP64 and rel(qg, qs) < TOL_FP64


TAB = O.TABLEAUX["ssp33"]


@pytest.mark.parametrize("case", ["mixed_degree", "vortex_p3"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_time_step_host_buffers(gpu_lib, precision, case):
    """oc_perform_time_step on host vectors: page-locked buffers (the last stage
    writes u^{n+1} into them directly) and pageable ones (copied back) give the
    bits of the device-vector run, over several steps and a change of buffers.
    These meshes are below the size of the chunked copy in: the same launches."""
    import ctypes as C
    import torch
    from oceano_gb300 import _lib
    kw = dict(precision="mixed", zeta_reference=1.0) if precision == "mixed" else {}
    mesh, orc, op = setup(case, **kw)
    z, q = perturbed_state(orc, 3)
    dt = 0.05 / orc.transport_speed(z, q)
    zd, qd = torch.from_numpy(z.copy()).cuda(), torch.from_numpy(q.copy()).cuda()
    pinned = [(torch.from_numpy(z.copy()).pin_memory(), torch.from_numpy(q.copy()).pin_memory())
              for _ in range(2)]
    zp, qp = z.copy(), q.copy()

    def host_step(t, zh, qh):
        _lib.check(_lib.lib().oc_perform_time_step(op.h, _lib.SCHEME["ssp33"], t, dt,
                                                   C.c_void_p(zh.data_ptr()),
                                                   C.c_void_p(qh.data_ptr()), _lib.OC_MEM_HOST),
                   op.h)

    for it in range(4):
        t = it * dt
        n0 = _lib.lib().oc_launch_count(op.h)
        op.perform_time_step("ssp33", t, dt, zd, qd)
        n1 = _lib.lib().oc_launch_count(op.h)
        a, b = pinned[it % 2]
        host_step(t, a, b)
        if it > 0:  # (the first device step tunes the launches)
            assert _lib.lib().oc_launch_count(op.h) - n1 == n1 - n0
        if it % 2 == 0:  # the other pair follows with a copy of the state
            pinned[1][0].copy_(a)
            pinned[1][1].copy_(b)
        else:
            pinned[0][0].copy_(a)
            pinned[0][1].copy_(b)
        op.perform_time_step("ssp33", t, dt, zp, qp)
    torch.cuda.synchronize()
    zr, qr = zd.cpu().numpy(), qd.cpu().numpy()
    a, b = pinned[1]
    assert np.array_equal(a.numpy(), zr) and np.array_equal(b.numpy(), qr)
    assert np.array_equal(zp, zr) and np.array_equal(qp, qr)


def test_time_step_host_buffers_chunked(gpu_lib):
    """The 320x160 degree-3 vortex in the mixed form on page-locked host vectors:
    u^n (19.7 MB) is copied in by three pieces and stage 0 runs by three chunks of
    cells, each launched once its cells' and their neighbours' DoFs are in; the
    states are the bits of the device-vector run, step after step."""
    import ctypes as C
    import torch
    from oceano_gb300 import _lib, vortex_mesh
    from oceano_gb300.icbc import vortex_params
    from oceano_gb300.workloads import vortex_operator
    op = vortex_operator(vortex_mesh(4, 3), "mixed", vortex_params())
    n = op.n_dofs
    z0, q0 = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, z0, q0)
    dt = 0.05 / op.compute_cell_transport_speed(z0, q0)
    zd, qd = torch.from_numpy(z0.copy()).cuda(), torch.from_numpy(q0.copy()).cuda()
    zh, qh = torch.from_numpy(z0.copy()).pin_memory(), torch.from_numpy(q0.copy()).pin_memory()
    for it in range(4):
        t = it * dt
        n0 = _lib.lib().oc_launch_count(op.h)
        op.perform_time_step("ssp33", t, dt, zd, qd)
        n1 = _lib.lib().oc_launch_count(op.h)
        _lib.check(_lib.lib().oc_perform_time_step(op.h, _lib.SCHEME["ssp33"], t, dt,
                                                   C.c_void_p(zh.data_ptr()),
                                                   C.c_void_p(qh.data_ptr()), _lib.OC_MEM_HOST),
                   op.h)
        if it > 0:  # stage 0 as 3 launches instead of 1
            assert _lib.lib().oc_launch_count(op.h) - n1 == n1 - n0 + 2
        torch.cuda.synchronize()
        assert np.array_equal(zh.numpy(), zd.cpu().numpy())
        assert np.array_equal(qh.numpy(), qd.cpu().numpy())


def test_unknown_boundary_id(gpu_lib):
    from oceano_gb300._lib import OceanoError
    from oceano_gb300.operator import OceanoOperator
    from oceano_gb300 import uniform_mesh
    mesh = uniform_mesh(4, 2, (0, 2, 0, 1), False, 1)
    op = OceanoOperator(mesh)
    op.set_wall_boundary(0)  # ids 1 and 2 left unset
    n = op.n_dofs
    z, q = np.ones(n), np.zeros(2 * n)
    with pytest.raises(OceanoError) as e:
        op.compute_cell_transport_speed(z, q)  # no boundary needed: fine
        op.perform_time_step("ssp33", 0.0, 1e-3, z, q)
    assert e.value.status == 2


@pytest.mark.parametrize("name", ["mixed_degree", "hanging_p3_bathy", "open_bcs_p2"])
def test_static_data_point_order(gpu_lib, name):
    """The library lays static data out at the same points as the oracle."""
    mesh, orc, op = setup(name)
    for which in range(5):
        a = op.quadrature_points(which)
        b = orc.points(which)
        assert a.shape == b.shape
        assert np.abs(a - b).max() < 1e-13
