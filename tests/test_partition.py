"""Single-mesh partition with a one-layer ghost halo (CPU oracle as the stage,
and the GPU operator per part), against the unpartitioned run."""
import numpy as np
import pytest

from cases import CASES, VORTEX, static_arrays
from oracle import oracle as O


def setup(case, n_parts):
    from oceano_gb300.partition import partition
    mesh_f, bcs, pdata, friction = CASES[case]
    mesh = mesh_f()
    full = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    if pdata is not None:
        full.set_static(*static_arrays(full, pdata))
    z, q = full.project_vortex(0.0)
    dt = 0.05 / full.transport_speed(z, q)
    parts = partition(mesh, n_parts)
    return mesh, full, z, q, dt, parts


def test_partition_covers_every_cell_once():
    from oceano_gb300.partition import partition
    from cases import hanging_mesh
    m = hanging_mesh(2)
    parts = partition(m, 4)
    owned = np.concatenate([p.global_cell[:p.n_owned] for p in parts])
    assert np.array_equal(np.sort(owned), np.arange(m.n_cells))
    for p in parts:  # every owned cell keeps all its faces
        cnt = np.zeros((p.mesh.n_cells, 4), int)
        for f in range(p.mesh.n_inner):
            cnt[p.mesh.cell_m[f], p.mesh.face_m[f]] += 1
            cnt[p.mesh.cell_p[f], p.mesh.face_p[f]] += 1
        for b in range(p.mesh.n_bnd):
            f = p.mesh.n_inner + b
            cnt[p.mesh.cell_m[f], p.mesh.face_m[f]] += 1
        assert (cnt[:p.n_owned] >= 1).all()


@pytest.mark.parametrize("case", ["hanging_p2", "mixed_degree"])
def test_local_lockstep_matches_single_mesh(case):
    import torch
    from oceano_gb300.partition import local_erk_step, with_ghost_boundary
    mesh, full, z0, q0, dt, parts = setup(case, 3)
    mesh_f, bcs, pdata, friction = CASES[case]
    stages, zs, qs = [], [], []
    for p in parts:
        orc = O.Oracle(p.mesh, friction=friction, bcs=with_ghost_boundary(bcs),
                       vortex=VORTEX + [0, 0])

        def stage(st, s, t, f, rz, rq, kz, kq, sz, sq, nz, nq, orc=orc):
            orc.stage_erk(st, s, t, f, rz.numpy(), rq.numpy(), [k.numpy() for k in kz],
                          [k.numpy() for k in kq], sz.numpy(), sq.numpy(), nz.numpy(), nq.numpy())
        stages.append(stage)
        zs.append(torch.from_numpy(z0[p.dof_index(mesh, "zeta")].copy()))
        qs.append(torch.from_numpy(q0[p.dof_index(mesh, "q")].copy()))
    tb = O.TABLEAUX["ssp33"]
    z, q = z0.copy(), q0.copy()
    for it in range(2):
        local_erk_step(stages, parts, tb, it * dt, dt, zs, qs)
        O.erk_step(full, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
    for p, zp, qp in zip(parts, zs, qs):
        no = int(p.mesh.offsets()[p.n_owned])
        assert np.abs(zp.numpy()[:no] - z[p.dof_index(mesh, "zeta")[:no]]).max() < 1e-13
        assert np.abs(qp.numpy()[:2 * no] - q[p.dof_index(mesh, "q")[:2 * no]]).max() < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["hanging_p2", "mixed_degree", "hanging_p3_bathy"])
def test_gpu_partitioned_matches_single_mesh(gpu_lib, case):
    """Three parts of one mesh, each on its own GPU operator (one GPU, in-process
    halo copies between stages), against the unpartitioned GPU run (FP64, 1e-12)."""
    import torch
    from oceano_gb300.operator import OceanoOperator
    from oceano_gb300.partition import local_erk_step, with_ghost_boundary
    from oceano_gb300.workloads import apply_bcs
    mesh, full, z0, q0, dt, parts = setup(case, 3)
    mesh_f, bcs, pdata, friction = CASES[case]

    def make(m):
        op = OceanoOperator(m, friction=["none", "linear", "manning"][friction])
        apply_bcs(op, with_ghost_boundary(bcs))
        op.set_vortex(*VORTEX)
        if pdata is not None:
            op.initialize_data_at_quadrature(pdata)
        return op

    ops = [make(p.mesh) for p in parts]

    def stage_of(op):
        def stage(st, s, t, f, rz, rq, kz, kq, sz, sq, nz, nq):
            torch.cuda.synchronize()  # halo copies ran on torch's stream
            op.perform_stage_hydro(st, s, t, f, [rz, rq], kz, kq, sz, sq, nz, nq)
            op.synchronize()
        return stage

    stages = [stage_of(op) for op in ops]
    zs = [torch.from_numpy(z0[p.dof_index(mesh, "zeta")].copy()).cuda() for p in parts]
    qs = [torch.from_numpy(q0[p.dof_index(mesh, "q")].copy()).cuda() for p in parts]
    one = make(mesh)
    z, q = z0.copy(), q0.copy()
    tb = O.TABLEAUX["ssp33"]
    for it in range(3):
        local_erk_step(stages, parts, tb, it * dt, dt, zs, qs)
        torch.cuda.synchronize()
        one.perform_time_step("ssp33", it * dt, dt, z, q)
    for p, zp, qp in zip(parts, zs, qs):
        no = int(p.mesh.offsets()[p.n_owned])
        zr, qr = z[p.dof_index(mesh, "zeta")[:no]], q[p.dof_index(mesh, "q")[:2 * no]]
        assert np.linalg.norm(zp.cpu().numpy()[:no] - zr) <= 1e-12 * np.linalg.norm(zr)
        assert np.linalg.norm(qp.cpu().numpy()[:2 * no] - qr) <= 1e-12 * np.linalg.norm(qr)


def test_halo_carries_face_traces_only():
    """The halo moves the (p+1) nodal values of zeta, hu, hv of every ghost face an
    owned cell reads: about a (p+1)-fold smaller exchange than whole ghost cells
    (a ghost bordering two owned cells sends two traces)."""
    from oceano_gb300 import vortex_mesh
    from oceano_gb300.partition import ghost_faces, halo_bytes, partition
    mesh = vortex_mesh(2, 3)  # 80x40 cells, p = 3
    parts = partition(mesh, 4)
    traces = halo_bytes(parts)
    ghosts = sum(8 * 3 * 16 * (p.mesh.n_cells - p.n_owned) for p in parts)
    n_faces = sum(len(ghost_faces(p)) for p in parts)
    assert traces == n_faces * 3 * 4 * 8
    assert traces < ghosts / 3.5  # (p+1) = 4 of the 16 nodes of a cell per face


def test_time_step_size_over_owned_cells():
    """dt of a partitioned run: the maximum over the owned cells of every rank
    (ghost speeds ignored), reduced over the ranks."""
    from oceano_gb300.partition import partitioned_time_step_size
    mesh, full, z0, q0, dt, parts = setup("hanging_p2", 3)

    class Speeds:  # per-cell speeds of a local mesh: the ghosts' are garbage
        def __init__(self, part):
            self.v = np.concatenate([np.linspace(1.0, 2.0 + part.rank, part.n_owned),
                                     np.full(part.mesh.n_cells - part.n_owned, 1e9)])

        def cell_transport_speed(self, z, q):
            return self.v

    local = [Speeds(p) for p in parts]
    vmax = max(float(s.v[:p.n_owned].max()) for s, p in zip(local, parts))
    for s, p in zip(local, parts):
        dt = partitioned_time_step_size(s, p, None, None, 0.2, reduce_max=lambda v: vmax)
        assert dt == 0.2 / vmax
        assert partitioned_time_step_size(s, p, None, None, 0.2) == 0.2 / s.v[:p.n_owned].max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["hanging_p2", "mixed_degree", "hanging_p3_bathy"])
def test_gpu_partitioned_mixed_matches_single_mesh(gpu_lib, case):
    """The mixed form (FP32 bulk) on three parts, face traces exchanged in-process
    between stages, against the same stage sequence on the unpartitioned mesh:
    the owned cells see identical inputs, so their results agree to rounding."""
    import torch
    from oceano_gb300.operator import OceanoOperator
    from oceano_gb300.partition import local_erk_step, partition, with_ghost_boundary
    from oceano_gb300.workloads import apply_bcs
    mesh, full, z0, q0, dt, parts = setup(case, 3)
    mesh_f, bcs, pdata, friction = CASES[case]

    def make(m):
        op = OceanoOperator(m, friction=["none", "linear", "manning"][friction],
                            precision="mixed", zeta_reference=1.0)
        apply_bcs(op, with_ghost_boundary(bcs))
        op.set_vortex(*VORTEX)
        if pdata is not None:
            op.initialize_data_at_quadrature(pdata)
        return op

    def stage_of(op):
        def stage(st, s, t, f, rz, rq, kz, kq, sz, sq, nz, nq):
            torch.cuda.synchronize()
            op.perform_stage_hydro(st, s, t, f, [rz, rq], kz, kq, sz, sq, nz, nq)
            op.synchronize()
        return stage

    def run(ps):
        ops = [make(p.mesh) for p in ps]
        zs = [torch.from_numpy(z0[p.dof_index(mesh, "zeta")].copy()).cuda() for p in ps]
        qs = [torch.from_numpy(q0[p.dof_index(mesh, "q")].copy()).cuda() for p in ps]
        tb = O.TABLEAUX["ssp33"]
        for it in range(3):
            local_erk_step([stage_of(op) for op in ops], ps, tb, it * dt, dt, zs, qs)
        torch.cuda.synchronize()
        return zs, qs

    zs, qs = run(parts)
    one = partition(mesh, 1)
    zf, qf = run(one)
    z, q = zf[0].cpu().numpy(), qf[0].cpu().numpy()
    for p, zp, qp in zip(parts, zs, qs):
        no = int(p.mesh.offsets()[p.n_owned])
        zr, qr = z[p.dof_index(mesh, "zeta")[:no]], q[p.dof_index(mesh, "q")[:2 * no]]
        assert np.linalg.norm(zp.cpu().numpy()[:no] - zr) <= 1e-14 * np.linalg.norm(zr)
        assert np.linalg.norm(qp.cpu().numpy()[:2 * no] - qr) <= 1e-14 * np.linalg.norm(qr)
