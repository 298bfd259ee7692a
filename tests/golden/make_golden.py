"""Generate the golden stage vectors of tests/golden/*.npz from the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py
Each file holds, for one case of tests/cases.py, the inputs' seeds and the
outputs of one ERK stage (SSP-RK3 stage 1), one ARK stage (stage 1 of
Giraldo/TR-BDF2), three SSP-RK3 time steps from the vortex projection, and
the transport speed of the perturbed state.  The tests check that the oracle
still reproduces them and compare the GPU operator against them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cases import CASES, VORTEX, perturbed_state, static_arrays  # noqa: E402
from oracle import oracle as O  # noqa: E402

GOLDEN_CASES = ("vortex_p1", "hanging_p2", "mixed_degree", "hanging_p3_bathy")
ERK_F = np.array([0.002, 0.002])
ARK_F, ARK_FT, ARK_FM = np.array([0.0015, 0.0015]), np.array([0.001, 0.001]), 0.0008


def oracle_for(name):
    mesh_f, bcs, pdata, friction = CASES[name]
    mesh = mesh_f()
    orc = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    if pdata is not None:
        orc.set_static(*static_arrays(orc, pdata))
    return mesh, orc


def stage_inputs(n, seed):
    rng = np.random.default_rng(500 + seed)
    kz = [np.zeros(n)] + [1e-3 * rng.standard_normal(n) for _ in range(3)]
    kq = [np.zeros(2 * n)] + [1e-3 * rng.standard_normal(2 * n) for _ in range(5)]
    return kz, kq


def compute(name):
    mesh, orc = oracle_for(name)
    n = orc.n
    z, q = perturbed_state(orc, 4, amp=1e-4)
    out = {"n": n, "in_z": z.copy(), "in_q": q.copy()}
    # ERK stage 1 of 3
    kz, kq = stage_inputs(n, 1)
    kz, kq = [k.copy() for k in kz], [k.copy() for k in kq[:4]]
    nz, nq = np.zeros(n), np.zeros(2 * n)
    orc.stage_erk(1, 3, 0.01, ERK_F, z.copy(), q.copy(), kz, kq, z, q, nz, nq)
    out.update(erk_kz=kz[2], erk_kq=kq[2], erk_nz=nz, erk_nq=nq)
    # ARK stage 1 of 3
    kz, kq = stage_inputs(n, 2)
    nz, nq = np.zeros(n), np.zeros(2 * n)
    orc.stage_ark(1, 3, 0.01, ARK_F, ARK_FT, ARK_FM, z.copy(), q.copy(), kz, kq, z, q, nz, nq)
    # ARK registers of stage s: k_zeta[s+1], k_q explicit [2s+1], implicit [2s+2]
    out.update(ark_kz=kz[2], ark_kq_ex=kq[3], ark_kq_im=kq[4], ark_nz=nz, ark_nq=nq)
    # three SSP-RK3 steps from the vortex projection
    zs, qs = orc.project_vortex(0.0)
    dt = 0.075 / orc.transport_speed(zs, qs)
    tb = O.TABLEAUX["ssp33"]
    for it in range(3):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, zs, qs)
    out.update(step_dt=np.array(dt), step_z=zs, step_q=qs)
    out["speed"] = np.array(orc.transport_speed(z, q))
    return out


if __name__ == "__main__":
    for name in GOLDEN_CASES:
        out = compute(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path))
