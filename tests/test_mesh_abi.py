"""Host-side logic without a GPU: mesh builder invariants, the reference's
vortex mesh, the closed form of the zeta sweeps, and the C ABI exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cases import hanging_mesh
from oceano_gb300 import QuadForest, random_hp_mesh, uniform_mesh, vortex_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def face_slots(mesh):
    """Number of face references per (cell, face number)."""
    cnt = np.zeros((mesh.n_cells, 4), int)
    for f in range(mesh.n_inner):
        cnt[mesh.cell_m[f], mesh.face_m[f]] += 1
        cnt[mesh.cell_p[f], mesh.face_p[f]] += 1
    for b in range(mesh.n_bnd):
        f = mesh.n_inner + b
        cnt[mesh.cell_m[f], mesh.face_m[f]] += 1
    return cnt


@pytest.mark.parametrize("mesh_f", [lambda: vortex_mesh(2, 1), lambda: hanging_mesh(2),
                                    lambda: uniform_mesh(5, 3, (0, 1, 0, 1), False, 2)])
def test_every_cell_face_covered(mesh_f):
    mesh = mesh_f()
    cnt = face_slots(mesh)
    assert cnt.min() >= 1 and cnt.max() <= 2
    # a face with two references is the coarse side of two hanging faces
    assert (cnt == 2).sum() * 2 == mesh.n_hanging


def test_vortex_mesh_sizes():
    m = vortex_mesh(2, 1)
    assert m.n_cells == 3200 and m.n_bnd == 160 and m.n_inner == 80 * 40 + 80 * 39
    m4 = vortex_mesh(4, 3)
    assert m4.n_cells == 51200 and m4.n_dofs() == 51200 * 16


def test_balance_and_hanging_consistency():
    f = QuadForest(4, 2, (0, 2, 0, 1), periodic_x=True)
    rng = np.random.default_rng(0)
    for _ in range(3):
        for leaf in sorted(f.leaves):
            if rng.random() < 0.3:
                f.refine(leaf)
    f.balance()
    m = f.build(2)
    lv = m.level
    for k in range(m.n_inner):
        dl = lv[m.cell_m[k]] - lv[m.cell_p[k]]
        assert dl in (0, 1)
        assert (dl == 1) == (m.subface[k] >= 0)
    area = sum((v[2] - v[0]) * (v[5] - v[1]) for v in m.vertices)
    assert abs(area - 2.0) < 1e-12


def test_random_hp_mesh_is_seeded():
    a = random_hp_mesh(target=3000, global_refine=1, max_extra=2)
    b = random_hp_mesh(target=3000, global_refine=1, max_extra=2)
    assert a.n_cells == b.n_cells and np.array_equal(a.degree, b.degree)
    assert abs(a.n_cells - 3000) < 0.15 * 3000
    assert set(np.unique(a.degree)) <= {1, 2, 3, 4} and a.n_hanging > 0


def test_matches_reference_vortex_mesh():
    """The 20x10 coarse grid equals the reference's Gmsh vortex mesh
    (tests/shallowWaterVortex/shallowWaterVortex_20x10cells.msh, stored as the
    fixture tests/golden/vortex_coarse_mesh.npz by make_mesh_fixture.py): the
    same cells, and boundary faces with the same ids (walls 0, inflow 1 at
    x = 0, outflow 2 at x = 2)."""
    d = np.load(os.path.join(ROOT, "tests", "golden", "vortex_coarse_mesh.npz"))
    quads = d["quads"]
    assert quads.shape == (200, 4, 2)
    ref = sorted((round(q[:, 0].min(), 9), round(q[:, 1].min(), 9)) for q in quads)
    m = uniform_mesh(20, 10, (0.0, 2.0, 0.0, 1.0), False, 1)
    ours = sorted((round(v[0], 9), round(v[1], 9)) for v in m.vertices)
    assert ref == ours

    def key(a, b):
        return tuple(sorted([(round(a[0], 9), round(a[1], 9)), (round(b[0], 9), round(b[1], 9))]))

    ref_faces = {key(*ln): int(t) for ln, t in zip(d["lines"], d["line_physical"])}
    corner = {0: (0, 2), 1: (1, 3), 2: (0, 1), 3: (2, 3)}  # face -> local vertices
    our_faces = {}
    for b in range(m.n_bnd):
        f = m.n_inner + b
        v = m.vertices[m.cell_m[f]].reshape(4, 2)
        i0, i1 = corner[int(m.face_m[f])]
        our_faces[key(v[i0], v[i1])] = int(m.bid[b])
    assert our_faces == ref_faces


def test_closed_form_sweeps_match_literal_iteration():
    """The FP32 path's closed form of K lumped-mass sweeps on wet cells."""
    from oceano_gb300.basis import lagrange_matrix, lobatto
    for p in (1, 2, 3, 4):
        N, G = p + 1, p + 2
        xN, _ = lobatto(N)
        xG, wG = lobatto(G)
        B = lagrange_matrix(xN, xG)
        M1 = B.T @ np.diag(wG) @ B
        L1 = B.T @ wG
        M, Ml = np.kron(M1, M1), np.kron(L1, L1)
        b = np.random.default_rng(p).standard_normal(N * N)
        d = np.zeros(N * N)
        for _ in range(15):
            d = d + (b - M @ d) / Ml
        Ms = M1 / np.sqrt(np.outer(L1, L1))
        lam, Qv = np.linalg.eigh(Ms)
        W1 = Qv.T / np.sqrt(L1)[None, :]
        W2 = Qv / np.sqrt(L1)[:, None]
        mu = np.outer(lam, lam).ravel()
        g = (1 - (1 - mu) ** 15) / mu
        cf = np.kron(W2, W2) @ (g * (np.kron(W1, W1) @ b))
        assert np.abs(cf - d).max() < 1e-12 * np.abs(d).max()


def header_functions():
    src = open(os.path.join(ROOT, "include", "oceano_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(oc_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    """Build the library (nvcc cross-compiles without a GPU) and check its exports."""
    from oceano_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    names = header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    from oceano_gb300 import _lib
    assert set(_lib.EXPORTS) == set(names)
