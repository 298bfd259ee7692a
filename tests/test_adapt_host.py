"""Host logic of the remesh runs on CPU: face-neighbour table, flag dilation,
remesh counting and the state transfer between degree maps."""
import numpy as np
import pytest

from oceano_gb300 import uniform_mesh
from oceano_gb300.adapt import transfer_state
from oceano_gb300.basis import lobatto
from oceano_gb300.indicator import cell_info, dilate, remesh_count


def grid(nx=9, ny=7):
    mesh = uniform_mesh(nx, ny, (0.0, float(nx), 0.0, float(ny)), False, 1)
    v = mesh.vertices
    ij = np.stack([np.floor(v[:, 0::2].mean(1)), np.floor(v[:, 1::2].mean(1))], 1).astype(int)
    at = {tuple(k): c for c, k in enumerate(ij)}
    return mesh, ij, at


def test_cell_info_neighbours():
    """Columns 0..3 hold the neighbours across faces x-, x+, y-, y+ (-1 at the
    boundary), column 5 the member."""
    mesh, ij, at = grid()
    info = cell_info(mesh, np.arange(mesh.n_cells) % 3)
    for c, (i, j) in enumerate(ij):
        for f, (di, dj) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1))):
            assert info[c, f] == at.get((i + di, j + dj), -1)
    assert np.array_equal(info[:, 5], np.arange(mesh.n_cells) % 3)


@pytest.mark.parametrize("layers,count", [(0, 1), (1, 5), (2, 13), (3, 25)])
def test_dilate_grows_a_diamond(layers, count):
    """One flagged cell in the middle of the grid grows by face neighbours: the
    l1 ball of radius `layers` (1, 5, 13, 25 cells)."""
    mesh, ij, at = grid()
    flags = np.zeros(mesh.n_cells, bool)
    flags[at[(4, 3)]] = True
    out = dilate(flags, cell_info(mesh), layers)
    assert out.sum() == count
    d = np.abs(ij[:, 0] - 4) + np.abs(ij[:, 1] - 3)
    assert np.array_equal(out, d <= layers)


def test_dilate_stops_at_the_boundary():
    mesh, ij, at = grid()
    flags = np.zeros(mesh.n_cells, bool)
    flags[at[(0, 0)]] = True
    out = dilate(flags, cell_info(mesh), 1)
    assert set(map(tuple, ij[out])) == {(0, 0), (1, 0), (0, 1)}


def test_remesh_count_per_member():
    """Two members: only the one whose flags leave its refined set remeshes."""
    members = np.array([0, 0, 1, 1])
    seq = [np.array([1, 0, 1, 0], bool), np.array([1, 0, 1, 0], bool),
           np.array([0, 1, 1, 0], bool), np.array([0, 1, 1, 0], bool)]
    assert remesh_count(seq, members=members, n_members=2) == 1
    seq.append(np.array([1, 1, 0, 1], bool))
    assert remesh_count(seq, members=members, n_members=2) == 3


def _cell_means(deg, z):
    out, o = [], 0
    for p in deg:
        n = p + 1
        w = lobatto(n)[1]
        out.append(0.25 * np.kron(w, w) @ z[o:o + n * n])  # reference cell [-1, 1]^2
        o += n * n
    return np.array(out)


def test_transfer_up_is_exact_and_down_keeps_the_mean():
    """Raising the degree interpolates exactly, so lowering it back returns the
    state; lowering is the L2 projection, which keeps every cell's mean (mass)."""
    rng = np.random.default_rng(5)
    deg_old = np.array([1, 2, 3, 1, 2])
    deg_new = np.array([3, 2, 4, 2, 4])
    n = int(((deg_old + 1) ** 2).sum())
    z, q = rng.standard_normal(n), rng.standard_normal(2 * n)
    zu, qu = transfer_state(deg_old, deg_new, z, q)
    zb, qb = transfer_state(deg_new, deg_old, zu, qu)
    np.testing.assert_allclose(zb, z, atol=1e-12)
    np.testing.assert_allclose(qb, q, atol=1e-12)
    zr = rng.standard_normal(zu.size)
    zd, _ = transfer_state(deg_new, deg_old, zr, np.zeros(2 * zu.size))
    np.testing.assert_allclose(_cell_means(deg_old, zd), _cell_means(deg_new, zr), atol=1e-13)
