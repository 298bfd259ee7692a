"""Golden stage vectors (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle still reproduces them (libm may differ in the last bit between
x86 and Arm hosts, hence 1e-13 rather than bitwise).  GPU: the FP64 operator
reproduces them through the C ABI within 1e-12 from the stored stage inputs
(no oracle call on that side).
"""
import os

import numpy as np
import pytest

from cases import CASES, VORTEX, static_arrays

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
NAMES = ("vortex_p1", "hanging_p2", "mixed_degree", "hanging_p3_bathy")


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    ref = load(name)
    out = make_golden.compute(name)
    for k, v in ref.items():
        assert rel(np.asarray(out[k], np.float64), v) < 1e-13, k


def gpu_op(name):
    from oceano_gb300.operator import OceanoOperator
    from oceano_gb300.workloads import apply_bcs
    mesh_f, bcs, pdata, friction = CASES[name]
    mesh = mesh_f()
    op = OceanoOperator(mesh, friction=["none", "linear", "manning"][friction])
    apply_bcs(op, bcs)
    op.set_vortex(*VORTEX)
    if pdata is not None:
        op.initialize_data_at_quadrature(pdata)
    return op


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(gpu_lib, name):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as M
    ref = load(name)
    op = gpu_op(name)
    n = int(ref["n"])
    assert op.n_dofs == n
    z, q = ref["in_z"], ref["in_q"]
    kz, kq = M.stage_inputs(n, 1)
    kz, kq = [k.copy() for k in kz], [k.copy() for k in kq[:4]]
    nz, nq = np.zeros(n), np.zeros(2 * n)
    op.perform_stage_hydro(1, 3, 0.01, M.ERK_F, [z.copy(), q.copy()], kz, kq, z.copy(), q.copy(),
                           nz, nq)
    for k, v in (("erk_kz", kz[2]), ("erk_kq", kq[2]), ("erk_nz", nz), ("erk_nq", nq)):
        assert rel(v, ref[k]) < 1e-12, k
    kz, kq = M.stage_inputs(n, 2)
    nz, nq = np.zeros(n), np.zeros(2 * n)
    op.perform_stage_hydro(1, 3, 0.01, M.ARK_F, [z.copy(), q.copy()], kz, kq, z.copy(), q.copy(),
                           nz, nq, factor_tilde_residual=M.ARK_FT, factor_matrix=M.ARK_FM)
    for k, v in (("ark_kz", kz[2]), ("ark_kq_ex", kq[3]), ("ark_kq_im", kq[4]), ("ark_nz", nz),
                 ("ark_nq", nq)):
        assert rel(v, ref[k]) < 1e-12, k
    zs, qs = np.zeros(n), np.zeros(2 * n)
    op.project_vortex(0.0, zs, qs)
    dt = float(ref["step_dt"])
    for it in range(3):
        op.perform_time_step("ssp33", it * dt, dt, zs, qs)
    assert rel(zs, ref["step_z"]) < 1e-12 and rel(qs, ref["step_q"]) < 1e-12
    assert abs(op.compute_cell_transport_speed(z, q) - float(ref["speed"])) < 1e-12 * float(ref["speed"])
