"""Quad-forest meshes in the face-list format the operator consumes.

The reference gets its mesh from deal.II / p4est (``GridIn::read_msh`` plus
``refine_global`` in oceano/source/main.cc:616-663) and its cell and face
numbering from ``MatrixFree``.  That machinery is not part of the hot path;
this module builds the same kind of mesh (a forest of quadtrees over a
rectangular coarse grid, optional periodicity in x, random refinement with
2:1 face balance, hanging faces) and emits it in the boundary format of
``include/oceano_gpu.h``:

* cells: degree, 4 vertices each (deal.II vertex order v0=(0,0), v1=(1,0),
  v2=(0,1), v3=(1,1) in reference coordinates), Morton order inside each tree;
* inner faces (MatrixFree "interior then exterior" convention): minus cell,
  plus cell, face numbers (0 x-, 1 x+, 2 y-, 3 y+), subface (-1 conforming,
  else the half of the plus cell's face covered by the finer minus cell),
  orientation (always 0 here);
* boundary faces: cell, face number, boundary id.

Boundary ids follow the reference vortex mesh tags
(tests/shallowWaterVortex/shallowWaterVortex_20x10cells.msh): left 1,
right 2, bottom and top 0.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Mesh:
    degree: np.ndarray          # int32 [n_cells]
    vertices: np.ndarray        # float64 [n_cells, 8]
    cell_m: np.ndarray          # int32 [n_inner + n_bnd]
    cell_p: np.ndarray          # int32 [n_inner]
    face_m: np.ndarray          # int8  [n_inner + n_bnd]
    face_p: np.ndarray          # int8  [n_inner]
    subface: np.ndarray         # int8  [n_inner]
    orient: np.ndarray          # int8  [n_inner]
    bid: np.ndarray             # int32 [n_bnd]
    level: np.ndarray = field(default=None)  # int32 [n_cells], refinement level
    domain: tuple = (0.0, 1.0, 0.0, 1.0)

    @property
    def n_cells(self) -> int:
        return int(self.degree.shape[0])

    @property
    def n_inner(self) -> int:
        return int(self.cell_p.shape[0])

    @property
    def n_bnd(self) -> int:
        return int(self.bid.shape[0])

    @property
    def n_hanging(self) -> int:
        return int((self.subface >= 0).sum())

    def dofs_per_cell(self) -> np.ndarray:
        return (self.degree.astype(np.int64) + 1) ** 2

    def n_dofs(self) -> int:
        """Scalar DoFs of one variable (zeta); discharge has twice as many."""
        return int(self.dofs_per_cell().sum())

    def offsets(self) -> np.ndarray:
        o = np.zeros(self.n_cells + 1, np.int64)
        np.cumsum(self.dofs_per_cell(), out=o[1:])
        return o

    def with_degree(self, degree) -> "Mesh":
        d = np.broadcast_to(np.asarray(degree, np.int32), (self.n_cells,)).copy()
        return Mesh(d, self.vertices, self.cell_m, self.cell_p, self.face_m, self.face_p,
                    self.subface, self.orient, self.bid, self.level, self.domain)


def _morton(i: np.ndarray, j: np.ndarray, bits: int) -> np.ndarray:
    key = np.zeros_like(i, dtype=np.int64)
    for b in range(bits):
        key |= ((i >> b) & 1).astype(np.int64) << (2 * b)
        key |= ((j >> b) & 1).astype(np.int64) << (2 * b + 1)
    return key


class QuadForest:
    """Leaves of a forest of quadtrees on an nx-by-ny coarse grid.

    A leaf is (level, i, j): cell index (i, j) on the uniform grid of level
    ``level`` (nx*2^level by ny*2^level cells).
    """

    def __init__(self, nx: int, ny: int, domain=(0.0, 1.0, 0.0, 1.0), periodic_x=False):
        self.nx, self.ny, self.domain, self.periodic_x = nx, ny, domain, periodic_x
        self.leaves = {(0, i, j) for i in range(nx) for j in range(ny)}

    def refine(self, leaf):
        l, i, j = leaf
        self.leaves.discard(leaf)
        for di in (0, 1):
            for dj in (0, 1):
                self.leaves.add((l + 1, 2 * i + di, 2 * j + dj))

    def refine_global(self, n: int):
        for _ in range(n):
            for leaf in list(self.leaves):
                self.refine(leaf)

    def _wrap(self, l, i, j):
        nxl, nyl = self.nx << l, self.ny << l
        if self.periodic_x:
            i %= nxl
        if i < 0 or i >= nxl or j < 0 or j >= nyl:
            return None
        return (l, i, j)

    def find_leaf(self, l, i, j):
        """Leaf containing the level-l cell (i, j), if it is at level <= l."""
        key = self._wrap(l, i, j)
        if key is None:
            return None
        l, i, j = key
        while l >= 0:
            if (l, i, j) in self.leaves:
                return (l, i, j)
            l, i, j = l - 1, i >> 1, j >> 1
        return None

    def balance(self):
        """Enforce 2:1 balance across faces (p4est face balance)."""
        changed = True
        while changed:
            changed = False
            for leaf in sorted(self.leaves, key=lambda t: -t[0]):
                if leaf not in self.leaves:
                    continue
                l, i, j = leaf
                for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                    nb = self.find_leaf(l, i + di, j + dj)
                    if nb is not None and nb[0] < l - 1:
                        self.refine(nb)
                        changed = True

    def build(self, degree=1) -> Mesh:
        x0, x1, y0, y1 = self.domain
        leaves = sorted(self.leaves)
        lmax = max(l for l, _, _ in leaves)
        arr = np.array(leaves, dtype=np.int64)
        lv, ii, jj = arr[:, 0], arr[:, 1], arr[:, 2]
        sh = lmax - lv
        fi, fj = ii << sh, jj << sh            # finest-level corner
        tree = (fj >> lmax) * self.nx + (fi >> lmax)
        key = tree * (1 << (2 * lmax + 2)) + _morton(fi & ((1 << lmax) - 1),
                                                     fj & ((1 << lmax) - 1), lmax + 1)
        order = np.argsort(key, kind="stable")
        leaves = [leaves[k] for k in order]
        index = {leaf: c for c, leaf in enumerate(leaves)}
        n = len(leaves)
        verts = np.zeros((n, 8))
        level = np.zeros(n, np.int32)
        for c, (l, i, j) in enumerate(leaves):
            hx = (x1 - x0) / (self.nx << l)
            hy = (y1 - y0) / (self.ny << l)
            xa, ya = x0 + i * hx, y0 + j * hy
            xb, yb = x0 + (i + 1) * hx, y0 + (j + 1) * hy
            verts[c] = (xa, ya, xb, ya, xa, yb, xb, yb)
            level[c] = l
        cm, cp, fm, fp, sub = [], [], [], [], []
        bcell, bface, bid = [], [], []
        for c, (l, i, j) in enumerate(leaves):
            for f, (di, dj) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1))):
                key_nb = self._wrap(l, i + di, j + dj)
                if key_nb is None:
                    bcell.append(c)
                    bface.append(f)
                    bid.append(1 if f == 0 else 2 if f == 1 else 0)
                    continue
                nb = self.find_leaf(l, i + di, j + dj)
                fo = f ^ 1
                if nb is None:
                    continue  # neighbour refined: its fine cells own the hanging faces
                if nb[0] == l:
                    if f in (1, 3):  # conforming: minus = left/bottom cell
                        cm.append(c); cp.append(index[nb]); fm.append(f); fp.append(fo)
                        sub.append(-1)
                else:  # nb coarser: this (fine) cell is the minus side
                    ln, inb, jnb = nb
                    # position of this cell's face along the coarse face
                    along = j if f < 2 else i
                    s = along & 1
                    cm.append(c); cp.append(index[nb]); fm.append(f); fp.append(fo)
                    sub.append(s)
        n_inner = len(cm)
        mesh = Mesh(
            degree=np.full(n, degree, np.int32) if np.isscalar(degree) else
            np.asarray(degree, np.int32),
            vertices=verts,
            cell_m=np.array(cm + bcell, np.int32),
            cell_p=np.array(cp, np.int32),
            face_m=np.array(fm + bface, np.int8),
            face_p=np.array(fp, np.int8),
            subface=np.array(sub, np.int8),
            orient=np.zeros(n_inner, np.int8),
            bid=np.array(bid, np.int32),
            level=level,
            domain=self.domain,
        )
        return mesh


def uniform_mesh(nx, ny, domain=(0.0, 1.0, 0.0, 1.0), periodic_x=False, degree=1,
                 refine=0) -> Mesh:
    """nx-by-ny coarse grid refined ``refine`` times globally (main.cc:616-663)."""
    f = QuadForest(nx, ny, domain, periodic_x)
    f.refine_global(refine)
    return f.build(degree)


def random_hp_mesh(seed=20261203, target=60000, coarse=(20, 10), domain=(0.0, 2.0, 0.0, 1.0),
                   global_refine=2, max_extra=4, periodic_x=True, degrees=(1, 2, 3, 4)):
    """Seeded random refinement with 2:1 balance and random per-cell degree.

    The 20x10 coarse mesh is refined ``global_refine`` times, then every cell is
    refined 0..``max_extra`` further levels: at each level a leaf is split with a
    probability tuned (bisection on the probability) so that the balanced
    forest has about ``target`` active cells.  Degrees are drawn uniformly from
    ``degrees`` with the same seeded generator.
    """
    def make(prob):
        rng = np.random.Generator(np.random.MT19937(seed))
        f = QuadForest(coarse[0], coarse[1], domain, periodic_x)
        f.refine_global(global_refine)
        for _ in range(max_extra):
            cand = sorted(f.leaves)
            draw = rng.random(len(cand))
            for leaf, r in zip(cand, draw):
                if r < prob:
                    f.refine(leaf)
        f.balance()
        return f

    lo, hi = 0.0, 1.0
    best = None
    for _ in range(14):
        mid = 0.5 * (lo + hi)
        f = make(mid)
        n = len(f.leaves)
        if best is None or abs(n - target) < abs(best[1] - target):
            best = (f, n)
        if abs(n - target) <= 0.02 * target:
            break
        if n < target:
            lo = mid
        else:
            hi = mid
    f = best[0]
    mesh = f.build(1)
    rng = np.random.Generator(np.random.MT19937(seed + 1))
    deg = rng.choice(np.asarray(degrees, np.int32), size=mesh.n_cells).astype(np.int32)
    return mesh.with_degree(deg)


def vortex_mesh(refine: int, degree: int) -> Mesh:
    """[0,2]x[0,1] as a 20x10 coarse grid, periodic in x, walls in y."""
    return uniform_mesh(20, 10, (0.0, 2.0, 0.0, 1.0), periodic_x=True, degree=degree,
                        refine=refine)


def channel_mesh(degree: int = 2, nx: int = 250, ny: int = 10, length=25.0) -> Mesh:
    """[0,length]x[0,1] channel: inflow id 1 (left), outflow id 2 (right), walls 0."""
    return uniform_mesh(nx, ny, (0.0, length, 0.0, 1.0), periodic_x=False, degree=degree)


def concatenate_meshes(meshes) -> Mesh:
    """Disjoint union of meshes (an ensemble run as one operator): cells in
    order, then every mesh's inner faces, then every mesh's boundary faces
    (the operator's inner-first face convention)."""
    off = np.cumsum([0] + [m.n_cells for m in meshes])
    inner_m, inner_p, fm, fp, sub, ori = [], [], [], [], [], []
    bnd_m, bnd_f, bid = [], [], []
    for k, m in enumerate(meshes):
        ni = m.n_inner
        inner_m.append(m.cell_m[:ni] + off[k]); inner_p.append(m.cell_p + off[k])
        fm.append(m.face_m[:ni]); fp.append(m.face_p); sub.append(m.subface); ori.append(m.orient)
        bnd_m.append(m.cell_m[ni:] + off[k]); bnd_f.append(m.face_m[ni:]); bid.append(m.bid)
    return Mesh(
        degree=np.concatenate([m.degree for m in meshes]).astype(np.int32),
        vertices=np.concatenate([m.vertices for m in meshes]),
        cell_m=np.concatenate(inner_m + bnd_m).astype(np.int32),
        cell_p=np.concatenate(inner_p).astype(np.int32),
        face_m=np.concatenate(fm + bnd_f).astype(np.int8),
        face_p=np.concatenate(fp).astype(np.int8),
        subface=np.concatenate(sub).astype(np.int8),
        orient=np.concatenate(ori).astype(np.int8),
        bid=np.concatenate(bid).astype(np.int32),
        level=np.concatenate([m.level for m in meshes]).astype(np.int32),
        domain=meshes[0].domain,
    )


def disk_refined_mesh(center, scale, coarse=(20, 10), domain=(0.0, 2.0, 0.0, 1.0),
                      global_refine=2, extra=3, periodic_x=True, radii=(2.0, 1.4, 1.0),
                      degree_radius=None):
    """Nested disks of refinement around `center` (AMR-like meshes of an
    ensemble member): after `global_refine` levels, level k of `extra` splits
    the leaves whose centre lies within radii[k] * scale of `center` (periodic
    distance in x), then 2:1 balance.  Degree 2 inside `degree_radius`, 1
    elsewhere (degree 1 everywhere when None)."""
    x0, x1, y0, y1 = domain
    f = QuadForest(coarse[0], coarse[1], domain, periodic_x)
    f.refine_global(global_refine)
    lx = x1 - x0
    for k in range(extra):
        l = global_refine + k
        r = radii[k] * scale
        hx, hy = lx / (coarse[0] << l), (y1 - y0) / (coarse[1] << l)
        for leaf in [lf for lf in f.leaves if lf[0] == l]:
            _, i, j = leaf
            dx = x0 + (i + 0.5) * hx - center[0]
            if periodic_x:
                dx -= lx * np.round(dx / lx)
            dy = y0 + (j + 0.5) * hy - center[1]
            if dx * dx + dy * dy < r * r:
                f.refine(leaf)
    f.balance()
    mesh = f.build(1)
    if degree_radius is not None:
        v = mesh.vertices
        cx = 0.5 * (v[:, 0] + v[:, 6]) - center[0]
        if periodic_x:
            cx -= lx * np.round(cx / lx)
        cy = 0.5 * (v[:, 1] + v[:, 7]) - center[1]
        deg = np.where(cx * cx + cy * cy < degree_radius ** 2, 2, 1).astype(np.int32)
        mesh = mesh.with_degree(deg)
    return mesh
