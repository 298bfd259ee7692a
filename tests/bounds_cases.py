"""Workload of the bounds-checked build test: every parity case, FP64 and
mixed, one SSP-RK3 time step plus the transport speed and the velocity field
(stage, face-pass and auxiliary kernels), and one ARK step on the friction
case.  Run by the test in its own process with the regular library, and as a
child process with OCEANO_BOUNDS_CHECK=1 (the bounds-checked library):

    OCEANO_BOUNDS_CHECK=1 python tests/bounds_cases.py out.npz
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def run_all() -> dict:
    from cases import CASES, perturbed_state
    from test_gpu_parity import setup
    out = {}
    for name in sorted(CASES):
        for precision in ("fp64", "mixed"):
            _, orc, op = setup(name, precision)
            z, q = perturbed_state(orc, 3)
            speed = op.compute_cell_transport_speed(z, q)
            dt = 0.05 / speed
            schemes = ["ssp33"] + (["ark_stage3_order2"] if CASES[name][3] else [])
            for scheme in schemes:
                zs, qs = z.copy(), q.copy()
                op.perform_time_step(scheme, 0.0, dt, zs, qs)
                out[f"{name}/{precision}/{scheme}/z"] = zs
                out[f"{name}/{precision}/{scheme}/q"] = qs
            vel = np.zeros(2 * op.n_dofs)
            op.evaluate_velocity_field(z, q, vel)
            out[f"{name}/{precision}/speed"] = np.array([speed])
            out[f"{name}/{precision}/velocity"] = vel
            op.synchronize()
            op.close()
    return out


def selftest() -> tuple[int, str]:
    """Status and message of oc_bounds_selftest on a small operator."""
    from cases import CASES
    from test_gpu_parity import setup
    from oceano_gb300 import _lib
    _, _, op = setup(sorted(CASES)[0])
    st = _lib.lib().oc_bounds_selftest(op.h)
    msg = _lib.lib().oc_last_error(op.h).decode()
    op.close()
    return st, msg


if __name__ == "__main__":
    from oceano_gb300 import _lib
    res = run_all()
    st, msg = selftest()
    res["_checked"] = np.array([_lib.lib().oc_bounds_checked()])
    res["_selftest_status"] = np.array([st])
    np.savez(sys.argv[1], _selftest_message=np.array(msg), **res)
