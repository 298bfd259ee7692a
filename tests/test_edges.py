"""Edge cases of the operator: invalid meshes rejected before any device work
(CPU), and tiny or ragged meshes on the GPU (one cell, a cell that is its own
periodic neighbour, cell counts that leave a warp partly empty)."""
import numpy as np
import pytest

from oceano_gb300 import uniform_mesh
from oceano_gb300._lib import OC_ERR_INVALID_ARG, OC_ERR_UNSUPPORTED, OceanoError


def create(mesh, **kw):
    from oceano_gb300.operator import OceanoOperator
    return OceanoOperator(mesh, **kw)


def test_degree_out_of_range_rejected():
    for p in (0, 5):
        m = uniform_mesh(2, 1, (0, 1, 0, 1), False, 1).with_degree(np.array([1, p], np.int32))
        with pytest.raises(OceanoError) as e:
            create(m)
        assert e.value.status == OC_ERR_UNSUPPORTED and "degree" in str(e.value)


def test_non_affine_cell_rejected():
    m = uniform_mesh(2, 1, (0, 1, 0, 1), False, 1)
    m.vertices = m.vertices.copy()
    m.vertices[1, 7] += 0.01  # move the fourth vertex of cell 1 off the parallelogram
    with pytest.raises(OceanoError) as e:
        create(m)
    assert e.value.status == OC_ERR_UNSUPPORTED and "not affine" in str(e.value)


def test_inverted_cell_rejected():
    m = uniform_mesh(1, 1, (0, 1, 0, 1), False, 1)
    v = m.vertices.copy()
    v[0, [0, 2, 4, 6]] = v[0, [2, 0, 6, 4]]  # mirror in x: negative Jacobian
    m.vertices = v
    with pytest.raises(OceanoError) as e:
        create(m)
    assert e.value.status == OC_ERR_INVALID_ARG and "det" in str(e.value)


def test_bad_face_tables_rejected():
    m = uniform_mesh(3, 1, (0, 1, 0, 1), False, 1)
    m.cell_p = m.cell_p.copy()
    m.cell_p[0] = m.n_cells  # out of range
    with pytest.raises(OceanoError) as e:
        create(m)
    assert e.value.status == OC_ERR_INVALID_ARG
    m = uniform_mesh(3, 1, (0, 1, 0, 1), False, 1)
    m.cell_m = m.cell_m.copy()
    m.face_m = m.face_m.copy()
    m.cell_m[1], m.face_m[1] = m.cell_m[0], m.face_m[0]  # one cell face listed twice
    with pytest.raises(OceanoError) as e:
        create(m)
    assert e.value.status == OC_ERR_INVALID_ARG and "twice" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,periodic,degree", [(1, 1, False, 3), (1, 1, True, 2),
                                                   (7, 1, True, 3), (5, 1, False, 4),
                                                   (11, 1, True, 1)])
def test_tiny_and_ragged_meshes(gpu_lib, nx, ny, periodic, degree):
    """FP64 time steps on meshes with a single cell, a cell that is its own
    periodic neighbour, and cell counts that leave the last warp partly empty,
    against the oracle (1e-12)."""
    from cases import VORTEX
    from oracle import oracle as O
    mesh = uniform_mesh(nx, ny, (0.0, 2.0, 0.0, 1.0), periodic, degree)
    bcs = {0: ("wall",), 1: ("wall",), 2: ("wall",)}
    orc = O.Oracle(mesh, bcs=bcs, vortex=VORTEX + [0, 0])
    op = create(mesh)
    for b in bcs:
        op.set_wall_boundary(b)
    op.set_vortex(*VORTEX)
    z, q = orc.project_vortex(0.0)
    dt = 0.05 / orc.transport_speed(z, q)
    tb = O.TABLEAUX["ssp33"]
    zo, qo, zg, qg = z.copy(), q.copy(), z.copy(), q.copy()
    for it in range(3):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, zo, qo)
        op.perform_time_step("ssp33", it * dt, dt, zg, qg)
    assert np.linalg.norm(zg - zo) <= 1e-12 * np.linalg.norm(zo)
    assert np.linalg.norm(qg - qo) <= 1e-12 * max(np.linalg.norm(qo), 1e-300)
