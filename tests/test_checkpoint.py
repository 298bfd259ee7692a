"""Checkpoint format: round trip on the CPU; resumed runs on the GPU continue
bit for bit."""
import numpy as np
import pytest

from cases import hanging_mesh, mixed_degree


def test_round_trip(tmp_path):
    from oceano_gb300 import checkpoint as ck
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    rng = np.random.default_rng(0)
    n = mesh.n_dofs()
    z, q = rng.standard_normal(n), rng.standard_normal(2 * n)
    p = tmp_path / "run.npz"
    ck.save(p, mesh, z, q, 0.125, 17, dt=np.array([1e-3]))
    c = ck.load(p)
    assert c.time == 0.125 and c.step == 17 and np.array_equal(c.extra["dt"], [1e-3])
    assert np.array_equal(c.height, z) and np.array_equal(c.discharge, q)
    for k in ("degree", "vertices", "cell_m", "cell_p", "face_m", "face_p", "subface", "orient",
              "bid", "level"):
        assert np.array_equal(getattr(c.mesh, k), getattr(mesh, k)), k
    assert c.mesh.n_inner == mesh.n_inner and c.mesh.domain == mesh.domain


def test_rejects_foreign_and_mismatched(tmp_path):
    from oceano_gb300 import checkpoint as ck
    mesh = hanging_mesh(2)
    bad = tmp_path / "bad.npz"
    np.savez(bad, height=np.zeros(3))
    with pytest.raises(ValueError):
        ck.load(bad)
    with pytest.raises(ValueError):
        ck.save(tmp_path / "x.npz", mesh, np.zeros(3), np.zeros(6), 0.0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_resume_is_bitwise(gpu_lib, tmp_path, precision):
    from cases import VORTEX
    from oceano_gb300 import checkpoint as ck
    from oceano_gb300.operator import OceanoOperator

    def make(mesh):
        op = OceanoOperator(mesh, precision=precision,
                            zeta_reference=1.0 if precision == "mixed" else 0.0)
        op.set_wall_boundary(0)
        op.set_vortex(*VORTEX)
        op.set_launch_mode("per_group")  # the same kernels on both handles
        return op

    mesh = mixed_degree(hanging_mesh(2, seed=11))
    op = make(mesh)
    n = op.n_dofs
    z, q = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, z, q)
    dt = 0.075 / op.compute_cell_transport_speed(z, q)
    za, qa = z.copy(), q.copy()
    for it in range(6):
        op.perform_time_step("ssp33", it * dt, dt, za, qa)
    zb, qb = z.copy(), q.copy()
    for it in range(3):
        op.perform_time_step("ssp33", it * dt, dt, zb, qb)
    ck.save(tmp_path / "c.npz", mesh, zb, qb, 3 * dt, 3, dt=np.array([dt]))
    c = ck.load(tmp_path / "c.npz")
    op2 = make(c.mesh)
    dt2 = float(c.extra["dt"][0])
    zc, qc = c.height, c.discharge
    for it in range(c.step, 6):
        op2.perform_time_step("ssp33", it * dt2, dt2, zc, qc)
    assert np.array_equal(zc, za) and np.array_equal(qc, qa)
