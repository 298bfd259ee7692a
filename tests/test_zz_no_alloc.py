"""The allocation-free transport-speed entry point against the regular one.

oc_transport_speed_noalloc exists for callers that cannot allocate device
memory when they need dt (inside CUDA-graph stream capture, under a pooled
allocator, in allocation-free loops).  It must return the same maximum as
oc_transport_speed; two calls in a row check that the shared scratch array is
reused correctly.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _speed_noalloc(op, z, q, out):
    from oceano_gb300 import _lib
    st = _lib.lib().oc_transport_speed_noalloc(op.h, C.c_void_p(z.data_ptr()),
                                               C.c_void_p(q.data_ptr()),
                                               C.c_void_p(out.data_ptr()))
    _lib.check(st, op.h)
    op.synchronize()
    return float(out.item())


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree", "hanging_p3_bathy"])
def test_noalloc_speed_matches(gpu_lib, name):
    import torch
    from cases import VORTEX, CASES, static_arrays, perturbed_state
    from oracle import oracle as O
    from oceano_gb300.operator import OceanoOperator
    mesh_f, bcs, pdata, friction = CASES[name]
    mesh = mesh_f()
    orc = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    op = OceanoOperator(mesh, friction=["none", "linear", "manning"][friction])
    if pdata is not None:
        op.set_static_data(*static_arrays(orc, pdata))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for seed in (1, 2):  # two calls in a row on the shared scratch
        z, q = perturbed_state(orc, seed)
        ref = op.compute_cell_transport_speed(z, q)
        zt = torch.from_numpy(z).cuda()
        qt = torch.from_numpy(q).cuda()
        torch.cuda.synchronize()
        got = _speed_noalloc(op, zt, qt, out)
        assert abs(got - ref) <= 1e-12 * ref
    op.close()
