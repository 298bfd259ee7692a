"""The allocation-free transport-speed entry point against the regular one.

oc_transport_speed_noalloc exists for callers that may not allocate device
memory when they need dt: hosts whose device memory belongs to a pool or arena,
real-time loops that forbid allocation after start-up, and embedding
frameworks that account for every device byte.  It must return the same
maximum as oc_transport_speed; two calls in a row check that the shared
scratch array is reused correctly.  It also rejects meshes larger than its
fixed scratch before launching anything, and turns a non-finite state into a
NaN speed where oc_transport_speed reports OC_ERR_NONFINITE.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_CELLS = 4096 * 128  # the scratch holds one partial maximum per 128-cell block


def _call(op, z, q, out):
    from oceano_gb300 import _lib
    return _lib.lib().oc_transport_speed_noalloc(op.h, C.c_void_p(z.data_ptr()),
                                                 C.c_void_p(q.data_ptr()),
                                                 C.c_void_p(out.data_ptr()))


def _speed_noalloc(op, z, q, out):
    from oceano_gb300 import _lib
    _lib.check(_call(op, z, q, out), op.h)
    op.synchronize()
    return float(out.item())


def _operator(name):
    from cases import VORTEX, CASES, static_arrays
    from oracle import oracle as O
    from oceano_gb300.operator import OceanoOperator
    mesh_f, bcs, pdata, friction = CASES[name]
    mesh = mesh_f()
    orc = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    op = OceanoOperator(mesh, friction=["none", "linear", "manning"][friction])
    if pdata is not None:
        op.set_static_data(*static_arrays(orc, pdata))
    return orc, op


@pytest.mark.parametrize("name", ["vortex_p3", "mixed_degree", "hanging_p3_bathy"])
def test_noalloc_speed_matches(gpu_lib, name):
    import torch
    from cases import perturbed_state
    orc, op = _operator(name)
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


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_noalloc_nonfinite_state_gives_nan(gpu_lib, bad):
    """A NaN or infinite value planted in the host state gives a NaN speed; the
    regular entry point reports the same state as OC_ERR_NONFINITE.  A finite
    call afterwards recovers the regular value (no stale NaN in the scratch)."""
    import torch
    from cases import perturbed_state
    from oceano_gb300._lib import OC_ERR_NONFINITE, OceanoError
    orc, op = _operator("mixed_degree")
    z, q = perturbed_state(orc, 4)
    zb = z.copy()
    zb[len(zb) // 3] = bad
    with pytest.raises(OceanoError) as e:
        op.compute_cell_transport_speed(zb, q)
    assert e.value.status == OC_ERR_NONFINITE
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = _speed_noalloc(op, torch.from_numpy(zb).cuda(), torch.from_numpy(q).cuda(), out)
    assert np.isnan(got)
    ref = op.compute_cell_transport_speed(z, q)
    got = _speed_noalloc(op, torch.from_numpy(z).cuda(), torch.from_numpy(q).cuda(), out)
    assert abs(got - ref) <= 1e-12 * ref
    op.close()


def test_noalloc_rejects_meshes_beyond_the_scratch(gpu_lib):
    """525,312 cells (> 524,288): OC_ERR_UNSUPPORTED with a message, the output
    left untouched (nothing is launched)."""
    import torch
    from oceano_gb300 import _lib, uniform_mesh
    from oceano_gb300.operator import OceanoOperator
    mesh = uniform_mesh(1026, 512, (0.0, 2.0, 0.0, 1.0), True, 1)
    assert mesh.n_cells > MAX_CELLS
    op = OceanoOperator(mesh)
    op.set_wall_boundary(0)
    n = op.n_dofs
    z = torch.ones(n, dtype=torch.float64, device="cuda")
    q = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    out = torch.full((1,), -7.0, dtype=torch.float64, device="cuda")
    st = _call(op, z, q, out)
    assert st == _lib.OC_ERR_UNSUPPORTED
    msg = _lib.lib().oc_last_error(op.h).decode()
    assert "524288" in msg and str(mesh.n_cells) in msg
    torch.cuda.synchronize()
    assert float(out.item()) == -7.0
    op.close()
