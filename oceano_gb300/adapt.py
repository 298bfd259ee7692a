"""p-adaptive remeshing of one member mesh, driven by a refinement indicator.

The reference refines where the vorticity indicator exceeds a fraction of its
maximum (oceano/source/main.cc:717-847, thresholds :749-765, indicator
hpTuner.h:247-305) and transfers the solution with deal.II's SolutionTransfer
after a conservative preparation of coarsened cells (OceanDG.h:2732-2781).  Its
p4est h-refinement is not part of the GPU path; here a "remesh" changes the
degree map of a fixed cell mesh instead: cells in the refined set carry degree
`p_fine`, the others `p_coarse`, and every change of the set rebuilds the
member's operator and transfers its state:

* degree up: interpolation at the new Gauss-Lobatto nodes (exact);
* degree down: cellwise L2 projection (Gauss quadrature exact for the product),
  which keeps the cell integrals of zeta and q -- the conservation property the
  reference's preparation step provides for its coarsening.

Policies of the refined set: the flags alone (``"vorticity"``), the flags grown
by k face layers (``"dilated"``), or the flags together with the flags a learned
indicator predicts some steps ahead (``"learned"``).  A member remeshes when a
flagged cell lies outside its refined set.
"""
from __future__ import annotations

import numpy as np

from .basis import gauss, lagrange_matrix, lobatto


def _transfer_1d(p_old: int, p_new: int) -> np.ndarray:
    """[p_new+1, p_old+1]: nodal values of degree p_new from degree p_old."""
    xo, xn = lobatto(p_old + 1)[0], lobatto(p_new + 1)[0]
    if p_new >= p_old:
        return lagrange_matrix(xo, xn)
    xq, wq = gauss(p_old + 1)  # exact for the degree p_old + p_new integrand
    Bn, Bo = lagrange_matrix(xn, xq), lagrange_matrix(xo, xq)
    Mn = Bn.T @ np.diag(wq) @ Bn
    return np.linalg.solve(Mn, Bn.T @ np.diag(wq) @ Bo)


def transfer_state(deg_old, deg_new, z, q):
    """State (zeta, q in the operator's layout) from degree map deg_old to
    deg_new on the same affine cells (the L2 projection only needs the
    reference-cell mass matrix: the Jacobian cancels)."""
    deg_old = np.asarray(deg_old, np.int64)
    deg_new = np.asarray(deg_new, np.int64)
    n_old = (deg_old + 1) ** 2
    n_new = (deg_new + 1) ** 2
    off_old = np.concatenate([[0], np.cumsum(n_old)])
    off_new = np.concatenate([[0], np.cumsum(n_new)])
    zn = np.zeros(int(off_new[-1]))
    qn = np.zeros(2 * int(off_new[-1]))
    for po in np.unique(deg_old):
        for pn in np.unique(deg_new):
            cells = np.nonzero((deg_old == po) & (deg_new == pn))[0]
            if cells.size == 0:
                continue
            T1 = _transfer_1d(int(po), int(pn))
            T = np.kron(T1, T1)  # lexicographic, x fastest
            a, b = (po + 1) ** 2, (pn + 1) ** 2
            io = off_old[cells][:, None] + np.arange(a)[None, :]
            inn = off_new[cells][:, None] + np.arange(b)[None, :]
            zn[inn] = z[io] @ T.T
            for comp in range(2):
                qn[2 * off_new[cells][:, None] + comp * b + np.arange(b)[None, :]] = \
                    q[2 * off_old[cells][:, None] + comp * a + np.arange(a)[None, :]] @ T.T
    return zn, qn


class AdaptiveMember:
    """One vortex member on a fixed cell mesh with a p-adaptive degree map,
    advanced by its own operator and its own time step (independent instance)."""

    def __init__(self, mesh, vortex, refined, cfl=0.075, p_coarse=1, p_fine=2,
                 precision="mixed", dt=None):
        from .workloads import vortex_operator
        self.base = mesh
        self.vortex = list(vortex)
        self.p = (p_coarse, p_fine)
        self.precision = precision
        self.refined = np.asarray(refined, bool).copy()
        self.mesh = mesh.with_degree(self._degrees(self.refined))
        self.op = vortex_operator(self.mesh, precision, self.vortex)
        n = self.op.n_dofs
        self.z, self.q = np.zeros(n), np.zeros(2 * n)
        self.op.project_vortex(0.0, self.z, self.q)
        self.time = 0.0
        self.remeshes = 0
        if dt is None:
            fine = mesh.with_degree(np.full(mesh.n_cells, p_fine, np.int32))
            op_f = vortex_operator(fine, "fp64", self.vortex)
            zf, qf = np.zeros(op_f.n_dofs), np.zeros(2 * op_f.n_dofs)
            op_f.project_vortex(0.0, zf, qf)
            dt = cfl / op_f.compute_cell_transport_speed(zf, qf)  # stable at p_fine everywhere
            op_f.close()
        self.dt = dt

    def _degrees(self, refined):
        return np.where(refined, self.p[1], self.p[0]).astype(np.int32)

    def step(self):
        self.op.perform_time_step("ssp33", self.time, self.dt, self.z, self.q)
        self.time += self.dt

    def remesh(self, refined):
        """New refined set: rebuild the operator, transfer the state."""
        from .workloads import vortex_operator
        refined = np.asarray(refined, bool)
        old = self._degrees(self.refined)
        new = self._degrees(refined)
        self.z, self.q = transfer_state(old, new, self.z, self.q)
        self.refined = refined.copy()
        self.op.close()
        self.mesh = self.base.with_degree(new)
        self.op = vortex_operator(self.mesh, self.precision, self.vortex)
        self.remeshes += 1

    def free_surface_error(self):
        """L2 error of the depth (zeta, zb = 0) against the travelling vortex
        (compute_errors_hydro, OceanDG.h:2380-2459) at the member's time."""
        return float(self.op.compute_errors_hydro(self.time, self.z, self.q)[0])


def _flags_and_features(member, threshold):
    import torch
    from .indicator import cell_info, features
    info = torch.from_numpy(cell_info(member.mesh)).cuda()
    z = torch.from_numpy(member.z).cuda()
    q = torch.from_numpy(member.q).cuda()
    f, fl, _ = features(member.op, z, q, info, 1, threshold)
    return f, fl.cpu().numpy() > 0.5


def refined_set(policy, flags, info, feat=None, model=None, layers=1, prob=0.5):
    """Refined set of a policy from the current flags (and features)."""
    from .indicator import dilate
    if policy == "vorticity":
        return flags.copy()
    if policy == "dilated":
        return dilate(flags, info, layers)
    if policy == "learned":
        return flags | model.predict(feat, prob).cpu().numpy()
    raise ValueError(policy)


def remesh_experiment(members, policy, steps, model=None, layers=1, threshold=None, cfl=0.075,
                      precision="mixed"):
    """Run every member (its own mesh, operator and time step) for `steps` steps
    under one refinement policy; a member remeshes (degree map change with
    state transfer) whenever a flagged cell lies outside its refined set.
    Returns remeshes, refined cells over flagged cells (time average), the
    free-surface L2 error over all members at their final times and the
    number of member-steps."""
    from .indicator import REFINE_THRESHOLD, cell_info
    from .workloads import member_mesh
    thr = REFINE_THRESHOLD if threshold is None else threshold
    remeshes, ratio, err2, total = 0, [], 0.0, 0
    for m in members:
        mesh0 = member_mesh(m)
        mesh = mesh0.with_degree(np.ones(mesh0.n_cells, np.int32))
        info = cell_info(mesh)
        probe = AdaptiveMember(mesh, m["vortex"], np.zeros(mesh.n_cells, bool), cfl=cfl,
                               precision=precision)
        feat, flags = _flags_and_features(probe, thr)
        member = AdaptiveMember(mesh, m["vortex"],
                                refined_set(policy, flags, info, feat, model, layers),
                                precision=precision, dt=probe.dt)
        probe.op.close()
        for _ in range(steps):
            member.step()
            feat, flags = _flags_and_features(member, thr)
            total += 1
            if (flags & ~member.refined).any():
                member.remesh(refined_set(policy, flags, info, feat, model, layers))
                remeshes += 1
            ratio.append(member.refined.sum() / max(flags.sum(), 1))
        err2 += member.free_surface_error() ** 2
        member.op.close()
    return {"remeshes": remeshes, "refined_over_flagged": float(np.mean(ratio)),
            "free_surface_l2_error": float(np.sqrt(err2)), "member_steps": total}
