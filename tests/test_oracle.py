"""Known-answer tests of the FP64 oracle (CPU only).

The reference ships no test suite and cannot be built here, so the oracle is
pinned by properties the reference's scheme must have: free-stream
preservation (also across hanging faces and degree jumps, and through every
kind of open boundary whose data matches the flow), the lake at rest to
machine precision (well-balancing of OceanDG.h's hydrostatic reconstruction),
global mass conservation of a stage, conservation of the x discharge between
walls in y, consistency of the explicit and additive
stage drivers, invariance of the stage under periodic translations and
mirroring, and convergence to the analytic travelling vortex.  The
properties that hold for any cell quadrature are checked for both rules of
n_points_1d (floor(1.5 p) + 1 and p + 1).
"""
import numpy as np
import pytest

from cases import VORTEX, hanging_mesh, mixed_degree
from oceano_gb300 import QuadForest, uniform_mesh, vortex_mesh
from oceano_gb300.icbc import vortex as vortex_np
from oracle import oracle as O


def uniform_state(mesh, z=1.0, q=(1.0, 0.0)):
    off = mesh.offsets()
    n = int(off[-1])
    zz = np.full(n, z)
    qq = np.zeros(2 * n)
    for c in range(mesh.n_cells):
        nd = off[c + 1] - off[c]
        qq[2 * off[c]:2 * off[c] + nd] = q[0]
        qq[2 * off[c] + nd:2 * off[c] + 2 * nd] = q[1]
    return zz, qq


def residuals(orc, z, q, t=0.0):
    n = orc.n
    kz = [np.zeros(n) for _ in range(4)]
    kq = [np.zeros(2 * n) for _ in range(4)]
    nz, nq = np.zeros(n), np.zeros(2 * n)
    orc.stage_erk(0, 3, t, np.array([1e-3]), z, q, kz, kq, z.copy(), q.copy(), nz, nq)
    return kz[1], kq[0], nz, nq


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("mesh_f", [lambda: vortex_mesh(0, 1), lambda: vortex_mesh(0, 4),
                                    lambda: hanging_mesh(3), lambda: mixed_degree(hanging_mesh(2))])
def test_free_stream_preserved(mesh_f, rule):
    mesh = mesh_f()
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, cell_rule=rule)
    z, q = uniform_state(mesh)
    rz, rq, nz, nq = residuals(orc, z, q)
    assert np.abs(rz).max() < 1e-13 and np.abs(rq).max() < 1e-12
    assert np.abs(nz - z).max() < 1e-13 and np.abs(nq - q).max() < 1e-12


def bump(x, y):
    zb = 1.0 - 0.4 * np.exp(-8 * ((x - 1.0) ** 2 + (y - 0.5) ** 2))
    return np.stack([zb, 0.03 + 0 * x, 0 * x, 0 * x, 0 * x])


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("degree", [1, 3])
def test_lake_at_rest(degree, rule):
    from cases import static_arrays
    mesh = uniform_mesh(8, 4, (0.0, 2.0, 0.0, 1.0), False, degree)
    orc = O.Oracle(mesh, friction=2, bcs={b: ("wall",) for b in (0, 1, 2)}, cell_rule=rule)
    orc.set_static(*static_arrays(orc, bump))
    z, q = uniform_state(mesh, z=0.25, q=(0.0, 0.0))
    rz, rq, nz, nq = residuals(orc, z, q)
    assert np.abs(rz).max() < 1e-15 and np.abs(rq).max() < 1e-14
    assert np.abs(nz - z).max() < 1e-15 and np.abs(nq).max() < 1e-14


def cell_integrals(mesh, z):
    """int zeta over the domain (nodal GL quadrature is exact for degree 2p-1 >= p)."""
    from oceano_gb300.basis import lobatto
    off = mesh.offsets()
    tot = 0.0
    for c in range(mesh.n_cells):
        p = int(mesh.degree[c])
        _, w = lobatto(p + 1)
        v = mesh.vertices[c]
        det = (v[2] - v[0]) * (v[5] - v[1]) - (v[4] - v[0]) * (v[3] - v[1])
        tot += det * np.kron(w, w) @ z[off[c]:off[c + 1]]
    return tot


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("mesh_f", [lambda: vortex_mesh(0, 2), lambda: hanging_mesh(2)])
def test_mass_conserved(mesh_f, rule):
    mesh = mesh_f()
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0], cell_rule=rule)
    z, q = orc.project_vortex(0.0)
    m0 = cell_integrals(mesh, z)
    tb = O.TABLEAUX["ssp33"]
    dt = 0.075 / orc.transport_speed(z, q)
    for it in range(3):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
    assert abs(cell_integrals(mesh, z) - m0) < 1e-13 * abs(m0)


def test_cell_rules_coincide_at_degree_1_and_differ_at_3():
    """floor(1.5 p) + 1 = p + 1 at p = 1: the two rules give the same stage; at
    p = 3 (5 against 4 points) the nonlinear flux integrals differ, the static
    data sizes follow the rule (5 values per cell point, one per boundary point)."""
    for degree, same in ((1, True), (3, False)):
        mesh = vortex_mesh(0, degree)
        out = []
        for rule in (0, 1):
            orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0], cell_rule=rule)
            z, q = orc.project_vortex(0.0)
            out.append((residuals(orc, z, q), orc.static_sizes()))
        (r0, s0), (r1, s1) = out
        nq0, nq1 = 3 * degree // 2 + 1, degree + 1
        assert s0[0] == 5 * nq0 * nq0 * mesh.n_cells and s1[0] == 5 * nq1 * nq1 * mesh.n_cells
        assert s0[4] == nq0 * mesh.n_bnd and s1[4] == nq1 * mesh.n_bnd
        d = max(np.abs(r1[0] - r0[0]).max(), np.abs(r1[3] - r0[3]).max())  # L_h zeta, q^{n+1}
        assert (d == 0.0) if same else (d > 1e-10), (degree, d)


def test_erk_ark_same_height_residual():
    mesh = vortex_mesh(0, 2)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    z, q = orc.project_vortex(0.0)
    n = orc.n
    a = [np.zeros(n) for _ in range(4)]
    b = [np.zeros(2 * n) for _ in range(4)]
    orc.stage_erk(0, 3, 0.0, np.array([1e-3]), z, q, a, b, z.copy(), q.copy(), np.zeros(n),
                  np.zeros(2 * n))
    c = [np.zeros(n) for _ in range(4)]
    d = [np.zeros(2 * n) for _ in range(6)]
    orc.stage_ark(0, 3, 0.0, np.array([1e-3]), np.array([1e-3]), 1e-3, z, q, c, d, z.copy(),
                  q.copy(), np.zeros(n), np.zeros(2 * n))
    assert np.array_equal(a[1], c[1])


def test_tableaux_order_conditions():
    for name, order in (("ssp33", 3), ("ssp22", 2), ("rk4", 4), ("giraldo32", 2)):
        t = O.TABLEAUX[name]
        b, c = np.array(t["b"]), np.array(t["c"])
        assert abs(b.sum() - 1) < 1e-15
        assert abs(b @ c - 0.5) < 1e-15
        if order >= 3:
            assert abs(b @ c ** 2 - 1 / 3) < 1e-15
        for i, row in enumerate(t["a"]):  # row i gives the input of stage i+1
            assert abs(sum(row) - c[i + 1]) < 1e-15


def vortex_error(refine, degree, steps=20):
    """L2 error of zeta at nodes after `steps` SSP-RK3 steps of the periodic vortex."""
    from oceano_gb300.icbc import nodal_points, vortex_params
    mesh = vortex_mesh(refine, degree)
    vx = vortex_params(uoo=1.0, peak=0.1, r0=0.2)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=vx + [0, 0])
    z, q = orc.project_vortex(0.0)
    dt = 0.05 * 0.1 / 4.2 * (0.5 ** refine)  # Courant 0.05 of the coarse mesh, halved per level
    tb = O.TABLEAUX["ssp33"]
    for it in range(steps):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
    t = steps * dt
    pts = nodal_points(mesh)
    h, _, _ = vortex_np(pts[:, 0], pts[:, 1], t, *[vx[0], vx[1], vx[2], vx[3], vx[4], vx[5]])
    return np.sqrt(np.mean((z - h) ** 2)), t


def test_vortex_converges():
    """Error at a fixed final time drops at least like h^2 under refinement (p=2)."""
    e0, t0 = vortex_error(0, 2, steps=10)
    e1, t1 = vortex_error(1, 2, steps=20)
    assert abs(t0 - t1) < 1e-14
    assert e1 < e0 / 4


def test_projection_matches_nodal_interpolation():
    from oceano_gb300.icbc import nodal_points, vortex_params
    mesh = vortex_mesh(1, 3)
    vx = vortex_params()
    orc = O.Oracle(mesh, vortex=vx + [0, 0])
    z, q = orc.project_vortex(0.0)
    pts = nodal_points(mesh)
    h, u, v = vortex_np(pts[:, 0], pts[:, 1], 0.0, *vx)
    assert np.abs(z - h).max() < 1e-4


def test_unknown_boundary_id_raises():
    mesh = uniform_mesh(4, 2, (0, 2, 0, 1), False, 1)
    orc = O.Oracle(mesh, bcs={0: ("wall",)})
    z, q = uniform_state(mesh)
    with pytest.raises(RuntimeError):
        residuals(orc, z, q)


def test_transport_speed_uniform():
    mesh = uniform_mesh(20, 10, (0, 2, 0, 1), True, 1)
    orc = O.Oracle(mesh, bcs={0: ("wall",)})
    z, q = uniform_state(mesh)
    h = 0.1
    expect = np.sqrt(9.81) / h + 1.0 / h  # sigma_max(J^-1) c + |J^-1 u|
    assert abs(orc.transport_speed(z, q) - expect) < 1e-12 * expect


@pytest.mark.parametrize("mesh_f", [lambda: vortex_mesh(0, 2), lambda: mixed_degree(hanging_mesh(2))])
def test_apply_is_inverse_mass_of_the_residual(mesh_f):
    """apply(): M dst = L_h(src) with the exact cell mass matrix (Gauss p+1 on
    affine cells): zeta against the ERK stage's L_h zeta register, discharge
    against its M^-1 L_h q register (the same inverse)."""
    from cases import perturbed_state
    from oceano_gb300.basis import gauss, lagrange_matrix, lobatto
    mesh = mesh_f()
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    z, q = perturbed_state(orc, 3)
    n = orc.n
    kz = [np.zeros(n) for _ in range(4)]
    kq = [np.zeros(2 * n) for _ in range(4)]
    orc.stage_erk(0, 3, 0.01, np.array([1e-3]), z, q, kz, kq, z.copy(), q.copy(), np.zeros(n),
                  np.zeros(2 * n))
    dz, dq = orc.apply(0.01, z, q)
    assert np.array_equal(dq, kq[1])
    off = mesh.offsets()
    for c in range(mesh.n_cells):
        N = int(mesh.degree[c]) + 1
        xg, wg = gauss(N)
        B = lagrange_matrix(lobatto(N)[0], xg)
        M1 = B.T @ np.diag(wg) @ B
        v = mesh.vertices[c].reshape(4, 2)
        det = abs((v[1, 0] - v[0, 0]) * (v[2, 1] - v[0, 1]) - (v[2, 0] - v[0, 0]) * (v[1, 1] - v[0, 1]))
        Mc = det * np.kron(M1, M1)
        r = Mc @ dz[off[c]:off[c + 1]] - kz[1][off[c]:off[c + 1]]
        assert np.abs(r).max() <= 1e-12 * max(1.0, np.abs(kz[1][off[c]:off[c + 1]]).max())


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("degree", [1, 3])
def test_residual_commutes_with_periodic_translation(degree, rule):
    """On the x-periodic 20x10 mesh (walls in y), translating an arbitrary wet state
    by k cells in x translates its stage residual and update: every cell, face and
    boundary face is evaluated by the same operations, so the two agree to
    rounding.  A wrong neighbour, face orientation or periodic link shows here."""
    mesh = vortex_mesh(0, degree)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, cell_rule=rule)
    off = mesh.offsets()
    nd = (degree + 1) ** 2
    v = mesh.vertices
    cx, cy = v[:, 0::2].mean(1), v[:, 1::2].mean(1)
    rng = np.random.default_rng(7 + degree)
    z = 1.0 + 0.1 * rng.random(orc.n)
    q = 0.1 * rng.standard_normal(2 * orc.n)
    rz, rq, nz, nq = residuals(orc, z, q)
    for k in (1, 3):
        tx = (cx + 0.1 * k) % 2.0  # cell c moves to the cell centred at (tx, cy)
        key = {(round(x, 6), round(y, 6)): c for c, (x, y) in enumerate(zip(cx, cy))}
        dst = np.array([key[(round(x, 6), round(y, 6))] for x, y in zip(tx, cy)])
        zs, qs = np.empty_like(z), np.empty_like(q)
        for c in range(mesh.n_cells):
            d = dst[c]
            zs[off[d]:off[d] + nd] = z[off[c]:off[c] + nd]
            qs[2 * off[d]:2 * off[d] + 2 * nd] = q[2 * off[c]:2 * off[c] + 2 * nd]
        sz, sq, snz, snq = residuals(orc, zs, qs)
        for c in range(mesh.n_cells):
            d = dst[c]
            for a, b, s in ((rz, sz, 1), (nz, snz, 1), (rq, sq, 2), (nq, snq, 2)):
                np.testing.assert_allclose(b[s * off[d]:s * off[d] + s * nd],
                                           a[s * off[c]:s * off[c] + s * nd],
                                           rtol=0, atol=1e-12 * (1 + np.abs(a).max()))


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("degree", [1, 2, 3])
@pytest.mark.parametrize("axis", [0, 1])
def test_residual_commutes_with_mirroring(axis, degree, rule):
    """Mirroring the x-periodic, y-walled domain about x = 1 (axis 0) or y = 1/2
    (axis 1) maps an arbitrary wet state to its mirror image (the normal discharge
    component changes sign, the nodes of each cell are reversed along the axis);
    the stage residual and update must be mirrored the same way.  This checks the
    orientation of normals, face numbers and the wall flux on both sides."""
    mesh = vortex_mesh(0, degree)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, cell_rule=rule)
    off = mesh.offsets()
    N = degree + 1
    nd = N * N
    v = mesh.vertices
    cx, cy = v[:, 0::2].mean(1), v[:, 1::2].mean(1)
    key = {(round(x, 6), round(y, 6)): c for c, (x, y) in enumerate(zip(cx, cy))}
    mx, my = (2.0 - cx, cy) if axis == 0 else (cx, 1.0 - cy)
    dst = np.array([key[(round(x, 6), round(y, 6))] for x, y in zip(mx, my)])
    i, j = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")  # node i + N j
    local = (i[:, ::-1] if axis == 0 else i[::-1, :]) + N * (j[:, ::-1] if axis == 0 else j[::-1, :])
    perm = local.ravel()  # mirrored node of node k
    sign = np.array([-1.0, 1.0]) if axis == 0 else np.array([1.0, -1.0])

    def mirror(z, q):
        zs, qs = np.empty_like(z), np.empty_like(q)
        for c in range(mesh.n_cells):
            d = dst[c]
            zs[off[d] + perm] = z[off[c]:off[c] + nd]
            for comp in range(2):
                qs[2 * off[d] + comp * nd + perm] = sign[comp] * q[2 * off[c] + comp * nd:
                                                                  2 * off[c] + (comp + 1) * nd]
        return zs, qs

    rng = np.random.default_rng(11 + degree)
    z = 1.0 + 0.1 * rng.random(orc.n)
    q = 0.1 * rng.standard_normal(2 * orc.n)
    rz, rq, nz, nq = residuals(orc, z, q)
    sz, sq, snz, snq = residuals(orc, *mirror(z, q))
    mz, mq = mirror(rz, rq)
    mnz, mnq = mirror(nz, nq)
    for got, want in ((sz, mz), (sq, mq), (snz, mnz), (snq, mnq)):
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * (1 + np.abs(want).max()))


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("degree", [1, 3])
def test_x_discharge_conserved(degree, rule):
    """On the x-periodic domain with walls at y = 0 and 1, no force acts in x (the
    wall's pressure and Lax-Friedrichs terms act along its normal, y): whole SSP-RK3
    steps keep the domain integral of hu of an arbitrary wet state to rounding."""
    mesh = vortex_mesh(0, degree)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, cell_rule=rule)
    off = mesh.offsets()
    nd = (degree + 1) ** 2
    rng = np.random.default_rng(3 + degree)
    z = 1.0 + 0.1 * rng.random(orc.n)
    q = 0.1 * rng.standard_normal(2 * orc.n)

    def hu(q):
        return np.concatenate([q[2 * off[c]:2 * off[c] + nd] for c in range(mesh.n_cells)])

    m0 = cell_integrals(mesh, hu(q))
    tb = O.TABLEAUX["ssp33"]
    dt = 0.05 / orc.transport_speed(z, q)
    for it in range(3):
        O.erk_step(orc, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
    scale = cell_integrals(mesh, np.abs(hu(q)))
    assert abs(cell_integrals(mesh, hu(q)) - m0) < 1e-13 * scale


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("left,right", [
    (("supercritical_inflow", (1.0, 0.9, 0.0)), ("supercritical_outflow",)),
    (("height_inflow", (1.0, 0.0, 0.0)), ("absorbing_outflow", (1.0, 0.9, 0.0))),
    (("discharge_inflow", (0.0, 0.9, 0.0)), ("height_inflow", (1.0, 0.0, 0.0))),
])
def test_open_boundaries_keep_a_matching_uniform_flow(left, right, rule):
    """A uniform flow (zeta 1 over a flat bottom, u = 0.9 along the walls) whose
    values the inflow and outflow conditions reproduce is a steady state of every
    boundary kind (OceanDG.h:1105-1339 with the ghost states of IcbcBase.h):
    supercritical in/out, height inflow, absorbing outflow at the same far field,
    discharge inflow of the same normal discharge."""
    mesh = uniform_mesh(8, 4, (0.0, 2.0, 0.0, 1.0), False, 2)
    orc = O.Oracle(mesh, bcs={0: ("wall",), 1: left, 2: right}, cell_rule=rule)
    z, q = uniform_state(mesh, z=1.0, q=(0.9, 0.0))
    rz, rq, nz, nq = residuals(orc, z, q)
    assert np.abs(rz).max() < 1e-13 and np.abs(rq).max() < 1e-12
    assert np.abs(nz - z).max() < 1e-14 and np.abs(nq - q).max() < 1e-14
