"""Cell partition of one mesh over several ranks with a one-layer ghost halo.

The reference distributes its p4est forest over MPI ranks and refreshes the
ghost face values once per stage through MatrixFree (`DataAccessOnFaces::values`,
OceanDG.h:1812-1813).  Here a mesh in Morton order is cut into contiguous cell
ranges of balanced DoF counts.  Each rank gets a local mesh made of its owned
cells followed by the ghost cells that share a face with them; faces between a
ghost and a cell outside the rank are dropped, so the operator computes the
owned cells exactly (all their faces are local) and garbage it never uses on
the ghosts.  Before every stage the ghosts' face traces are refreshed from the
owners (`HaloExchange.exchange`: the (p+1) nodal values of zeta, hu, hv per cut
face side), the only data exchange of the path; dt comes from the owned cells'
transport speeds through one allreduce MAX (OceanDG.h:2577).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import Mesh


@dataclass
class Part:
    rank: int
    mesh: Mesh                 # owned cells first, then ghosts
    n_owned: int
    global_cell: np.ndarray    # [n_local] global cell id of every local cell
    owner: np.ndarray          # [n_local] owning rank of every local cell

    def dof_index(self, global_mesh: Mesh, var: str = "zeta") -> np.ndarray:
        """Global DoF index of every local DoF (zeta: n layout; q: 2n layout)."""
        goff, loff = global_mesh.offsets(), self.mesh.offsets()
        nd = np.diff(loff)
        cells = np.repeat(np.arange(self.mesh.n_cells), nd)
        local = np.arange(int(loff[-1])) - loff[cells]
        if var == "zeta":
            return goff[self.global_cell[cells]] + local
        cells2 = np.repeat(np.arange(self.mesh.n_cells), 2 * nd)
        local2 = np.arange(2 * int(loff[-1])) - 2 * loff[cells2]
        return 2 * goff[self.global_cell[cells2]] + local2


def owner_ranges(mesh: Mesh, n_parts: int) -> np.ndarray:
    """Owning rank of every cell: contiguous ranges with balanced DoF counts."""
    nd = mesh.dofs_per_cell().astype(np.float64)
    cum = np.cumsum(nd) - 0.5 * nd
    return np.minimum((cum / nd.sum() * n_parts).astype(np.int64), n_parts - 1)


GHOST_BID = 15  # boundary id of the cut faces of ghost cells (any condition: ghosts are discarded)


def with_ghost_boundary(bcs: dict) -> dict:
    """Boundary conditions of a local mesh: those of the global mesh plus a wall on
    the cut faces of the ghost cells (their residual is never used)."""
    out = dict(bcs)
    out[GHOST_BID] = ("wall",)
    return out


def partition(mesh: Mesh, n_parts: int) -> list:
    """Local meshes of the ranks.  Ghosts = the cells sharing a face with an owned
    cell; when a ghost is the coarse side of a hanging face whose second half is
    local, its first half's fine cell joins as a ghost too (the operator wants
    subface 0 of a split face).  Ghost faces with no local cell on the other side
    become boundary faces with id GHOST_BID."""
    owner = owner_ranges(mesh, n_parts)
    ni = mesh.n_inner
    cm, cp, sub = mesh.cell_m[:ni], mesh.cell_p, mesh.subface
    bm = mesh.cell_m[ni:]
    parts = []
    for r in range(n_parts):
        owned = np.nonzero(owner == r)[0]
        is_local = owner == r
        nb = np.concatenate([cp[is_local[cm]], cm[is_local[cp]]])
        is_local = is_local.copy()
        is_local[nb] = True
        while True:  # subface closure of coarse ghost faces
            half = (sub == 1) & is_local[cm] & is_local[cp]  # second half local
            need = np.zeros(mesh.n_cells, bool)
            for f in np.nonzero(half)[0]:
                # first half of the same coarse face: same plus cell and face number
                g = np.nonzero((cp == cp[f]) & (mesh.face_p == mesh.face_p[f]) & (sub == 0))[0]
                need[cm[g][~is_local[cm[g]]]] = True
            if not need.any():
                break
            is_local |= need
        ghosts = np.nonzero(is_local & (owner != r))[0]
        cells = np.concatenate([owned, ghosts])
        local = np.full(mesh.n_cells, -1, np.int64)
        local[cells] = np.arange(len(cells))
        keep = (local[cm] >= 0) & (local[cp] >= 0)  # inner faces between two local cells
        keep_b = local[bm] >= 0
        # cut faces: a local (ghost) cell whose neighbour across a face is not local
        cut_m = (local[cm] >= 0) & (local[cp] < 0)
        cut_p = (local[cp] >= 0) & (local[cm] < 0) & (sub < 0)  # full plus-side faces only
        cut_cells = np.concatenate([local[cm[cut_m]], local[cp[cut_p]]])
        cut_faces = np.concatenate([mesh.face_m[:ni][cut_m], mesh.face_p[cut_p]])
        # a coarse ghost face cut on both halves: one boundary face
        both = (local[cp] >= 0) & (local[cm] < 0) & (sub == 0)
        for f in np.nonzero(both)[0]:
            g = np.nonzero((cp == cp[f]) & (mesh.face_p == mesh.face_p[f]) & (sub == 1))[0]
            if len(g) and local[cm[g[0]]] < 0:
                cut_cells = np.append(cut_cells, local[cp[f]])
                cut_faces = np.append(cut_faces, mesh.face_p[f])
        lm = Mesh(
            degree=mesh.degree[cells].astype(np.int32),
            vertices=mesh.vertices[cells],
            cell_m=np.concatenate([local[cm[keep]], local[bm[keep_b]], cut_cells]).astype(np.int32),
            cell_p=local[cp[keep]].astype(np.int32),
            face_m=np.concatenate([mesh.face_m[:ni][keep], mesh.face_m[ni:][keep_b],
                                   cut_faces]).astype(np.int8),
            face_p=mesh.face_p[keep].astype(np.int8),
            subface=mesh.subface[keep].astype(np.int8),
            orient=mesh.orient[keep].astype(np.int8),
            bid=np.concatenate([mesh.bid[keep_b], np.full(len(cut_cells), GHOST_BID)]).astype(np.int32),
            level=None if mesh.level is None else mesh.level[cells].astype(np.int32),
            domain=mesh.domain,
        )
        assert not (local[cells[:len(owned)]] < 0).any()
        parts.append(Part(r, lm, len(owned), cells, owner[cells]))
    return parts


def _face_dof(N: int, f: int, i: int) -> int:
    """Lexicographic node index of node i on face f of a cell with N x N nodes."""
    return i * N if f == 0 else i * N + N - 1 if f == 1 else i if f == 2 else (N - 1) * N + i


def ghost_faces(part: Part) -> list:
    """(local ghost cell, face number) pairs whose trace an owned cell of the part
    reads: the ghost side of every local inner face between an owned cell and a
    ghost (a coarse ghost split into two halves counts once), ordered by the
    ghost's global cell id and face number."""
    m, no = part.mesh, part.n_owned
    ni = m.n_inner
    cm, cp = m.cell_m[:ni], m.cell_p
    pairs = set()
    for i in np.nonzero((cm < no) & (cp >= no))[0]:
        pairs.add((int(cp[i]), int(m.face_p[i])))
    for i in np.nonzero((cp < no) & (cm >= no))[0]:
        pairs.add((int(cm[i]), int(m.face_m[i])))
    return sorted(pairs, key=lambda x: (int(part.global_cell[x[0]]), x[1]))


def _trace_idx(mesh: Mesh, pairs):
    """Local DoF indices (zeta layout, q layout) of the face traces (p+1 nodes per
    face and variable) of the given (local cell, face) pairs, in order."""
    off = mesh.offsets()
    z, q = [], []
    for c, f in pairs:
        N = int(mesh.degree[c]) + 1
        d = np.array([_face_dof(N, f, i) for i in range(N)], np.int64)
        z.append(off[c] + d)
        q.append(2 * off[c] + d)
        q.append(2 * off[c] + N * N + d)
    if not z:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    return np.concatenate(z), np.concatenate(q)


def halo_plan(parts: list, rank: int):
    """(send, recv) of one rank: {other rank: (zeta idx, q idx)} into its local vectors.
    Only face traces travel: the (p+1) nodal values of zeta, hu and hv on every face
    of a ghost that an owned cell reads (the operator reads nothing else of a ghost
    for the owned cells' results; the ghosts' own residuals are discarded).  Every
    rank derives the same plan from the same partition: the traces of rank g's
    ghosts owned by rank o travel o -> g in g's ghost_faces order."""
    me = parts[rank]
    send, recv = {}, {}
    mine = ghost_faces(me)
    for other in parts:
        if other.rank == rank:
            continue
        r = [(c, f) for c, f in mine if me.owner[c] == other.rank]
        if r:
            recv[other.rank] = _trace_idx(me.mesh, r)
        theirs = [(int(other.global_cell[c]), f) for c, f in ghost_faces(other)
                  if other.owner[c] == rank]
        if theirs:
            pos = {int(c): i for i, c in enumerate(me.global_cell[:me.n_owned])}
            send[other.rank] = _trace_idx(me.mesh, [(pos[c], f) for c, f in theirs])
    return send, recv


def halo_bytes(parts: list, itemsize: int = 8) -> int:
    """Bytes all ranks receive per exchange (one refresh of every ghost trace)."""
    return sum(itemsize * (len(z) + len(q)) for r in range(len(parts))
               for z, q in halo_plan(parts, r)[1].values())


def partitioned_time_step_size(op, part: Part, zeta, q, courant: float, reduce_max=None):
    """dt = courant / transport speed over the owned cells of all ranks
    (compute_cell_transport_speed, OceanDG.h:2505-2580, with the MPI max of
    :2577): per-cell speeds of the local mesh, the maximum over the owned cells,
    then `reduce_max` (e.g. an allreduce MAX over the ranks) on that number."""
    sp = op.cell_transport_speed(zeta, q)
    sp = sp.cpu().numpy() if hasattr(sp, "cpu") else np.asarray(sp)
    v = float(sp[:part.n_owned].max()) if part.n_owned else 0.0
    if reduce_max is not None:
        v = reduce_max(v)
    return courant / v


def torch_max(v: float) -> float:
    """Allreduce MAX of one number over the torch.distributed process group."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class HaloExchange:
    """Refresh the ghost DoFs of one rank's (zeta, q) from their owners: pack the
    owned DoFs other ranks hold as ghosts, move them, unpack into the ghosts.
    `transport(send, recv)` moves the buffers ({rank: tensor}); torch_transport
    uses torch.distributed point-to-point calls (gloo on CPU, NCCL on GPUs)."""

    def __init__(self, parts: list, rank: int, transport=None, device=None):
        import torch
        self.rank = rank
        send, recv = halo_plan(parts, rank)
        dev = device or "cpu"
        t = lambda a: torch.as_tensor(a, dtype=torch.int64, device=dev)  # noqa: E731
        self.send = {r: (t(z), t(q)) for r, (z, q) in send.items()}
        self.recv = {r: (t(z), t(q)) for r, (z, q) in recv.items()}
        self.transport = transport or torch_transport

    def exchange(self, zeta, q):
        import torch
        sbuf = {r: torch.cat([zeta[iz], q[iq]]) for r, (iz, iq) in self.send.items()}
        rbuf = {r: torch.empty(len(iz) + len(iq), dtype=zeta.dtype, device=zeta.device)
                for r, (iz, iq) in self.recv.items()}
        self.transport(sbuf, rbuf)
        for r, (iz, iq) in self.recv.items():
            zeta[iz] = rbuf[r][:len(iz)]
            q[iq] = rbuf[r][len(iz):]


def torch_transport(send: dict, recv: dict):
    import torch.distributed as dist
    reqs = [dist.irecv(buf, src=r) for r, buf in recv.items()]
    reqs += [dist.isend(buf, dst=r) for r, buf in send.items()]
    for q in reqs:
        q.wait()


def partitioned_erk_step(stage, halo, tableau, t, dt, zeta, q):
    """One explicit RK step of one rank in Butcher form (ExplicitRungeKuttaIntegrator.h:
    179-298) with a halo refresh before every stage.  `stage` has the signature of
    perform_stage_hydro on local vectors: stage(s, n_stages, time, f, rz, rq, kz, kq,
    solution_z, solution_q, next_z, next_q).  On return the owned DoFs of (zeta, q)
    hold u^{n+1}; ghosts hold values that the next refresh replaces."""
    import torch
    a, b, c = tableau["a"], tableau["b"], tableau["c"]
    s = len(b)
    n = zeta.numel()
    kz = [torch.zeros_like(zeta) for _ in range(s + 1)]
    kq = [torch.zeros_like(q) for _ in range(s + 1)]
    nz, nq = torch.zeros_like(zeta), torch.zeros_like(q)
    halo.exchange(zeta, q)
    for st in range(s):
        f = np.asarray(b if st == s - 1 else a[st], np.float64) * dt
        if st > 0:
            halo.exchange(nz, nq)
        rz, rq = (zeta.clone(), q.clone()) if st == 0 else (nz.clone(), nq.clone())
        stage(st, s, t + c[st] * dt, f, rz, rq, kz, kq, zeta, q, nz, nq)
    assert zeta.numel() == n


def local_exchange(parts: list, zetas, qs, plans=None):
    """Refresh the ghosts of all parts held by one process (an in-process
    transport): the same copies HaloExchange makes over the network."""
    import torch
    plans = plans or [halo_plan(parts, r) for r in range(len(parts))]
    for g in range(len(parts)):
        for o, (rz, rq) in plans[g][1].items():
            sz, sq = plans[o][0][g]
            dev = zetas[g].device
            zetas[g][torch.as_tensor(rz, device=dev)] = zetas[o][torch.as_tensor(sz, device=dev)]
            qs[g][torch.as_tensor(rq, device=dev)] = qs[o][torch.as_tensor(sq, device=dev)]


def local_erk_step(stages, parts, tableau, t, dt, zetas, qs, plans=None):
    """partitioned_erk_step for all parts of one process in lockstep (stage by
    stage, ghosts refreshed between stages by local_exchange)."""
    import torch
    a, b, c = tableau["a"], tableau["b"], tableau["c"]
    s = len(b)
    P = len(parts)
    plans = plans or [halo_plan(parts, r) for r in range(P)]
    kz = [[torch.zeros_like(zetas[r]) for _ in range(s + 1)] for r in range(P)]
    kq = [[torch.zeros_like(qs[r]) for _ in range(s + 1)] for r in range(P)]
    nz = [torch.zeros_like(zetas[r]) for r in range(P)]
    nq = [torch.zeros_like(qs[r]) for r in range(P)]
    local_exchange(parts, zetas, qs, plans)
    for st in range(s):
        f = np.asarray(b if st == s - 1 else a[st], np.float64) * dt
        if st > 0:
            local_exchange(parts, nz, nq, plans)
        for r in range(P):
            rz, rq = (zetas[r].clone(), qs[r].clone()) if st == 0 else (nz[r].clone(), nq[r].clone())
            stages[r](st, s, t + c[st] * dt, f, rz, rq, kz[r], kq[r], zetas[r], qs[r], nz[r], nq[r])
