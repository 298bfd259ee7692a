"""CPU checks of the learned-indicator oracle and host logic (no GPU)."""
import numpy as np

from oracle import indicator_oracle as IO


def test_bf16_rounding_known_answers():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -7 + 2 ** -8, -2.5, 0.0],
                 np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3*2^-9 rounds up;
    # 1 + 2^-7 + 2^-8 is a tie: to even (1 + 2^-6)
    expect = np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0], np.float32)
    assert np.array_equal(IO.bf16(x), expect)


def random_net(seed):
    rng = np.random.default_rng(seed)
    p = (0.3 * rng.standard_normal(IO.NP)).astype(np.float32)
    norm = np.concatenate([rng.standard_normal(12), 1.0 + rng.random(12)]).astype(np.float32)
    X = rng.standard_normal((64, 12)).astype(np.float32)
    y = (rng.random(64) < 0.3).astype(np.float32)
    return p, norm, X, y


def test_analytic_gradient_matches_finite_differences():
    """The oracle's backward formulas, on the FP64 network without roundings."""
    p, norm, X, y = random_net(1)
    p = p.astype(np.float64)
    _, g = IO.loss_and_grad(p, norm, X, y, 3.0, exact=True)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.choice(np.arange(IO.OB1), 8), rng.choice(np.arange(IO.OW2, IO.OB2), 8),
                          [IO.OB1 + 3, IO.OB2 + 5, IO.OW3 + 7, IO.OB3]])
    h = 1e-6
    for e in idx:
        pp, pm = p.copy(), p.copy()
        pp[e] += h
        pm[e] -= h
        fd = (IO.loss_and_grad(pp, norm, X, y, 3.0, exact=True)[0] -
              IO.loss_and_grad(pm, norm, X, y, 3.0, exact=True)[0]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-6 * max(1e-3, abs(g[e])), e


def test_rounded_forward_close_to_exact():
    p, norm, X, _ = random_net(3)
    z, _ = IO.forward(p, norm, X)
    ze, _ = IO.forward(p, norm, X, exact=True)
    assert np.abs(z - ze).max() < 0.05 * (1 + np.abs(ze).max())


def test_remesh_count():
    from oceano_gb300.indicator import remesh_count
    seq = [np.eye(1, 12, k, dtype=bool)[0] for k in range(8)]  # one flag moving right
    assert remesh_count(seq) == 7
    ahead = [seq[min(k + 1, 7)] | seq[min(k + 2, 7)] | seq[min(k + 3, 7)] for k in range(8)]
    assert remesh_count(seq, ahead) == 1  # at t = 4: {4..7} covers the rest
    members = np.array([0] * 6 + [1] * 6)
    assert remesh_count(seq, None, members, 2) == 7


def test_cell_info_neighbours_symmetric():
    from cases import hanging_mesh
    from oceano_gb300.indicator import cell_info
    m = hanging_mesh(2)
    info = cell_info(m)
    for c in range(m.n_cells):
        for f in range(4):
            nb = info[c, f]
            if nb >= 0:
                assert c in info[nb, :4] or m.level[nb] != m.level[c]
    assert (info[:, 4] == m.level).all()


def test_tensor_core_emulation_against_fp32_order():
    """forward_tensor_core (exact layer sums) against forward (FP32 fused
    multiply-adds in sequence, another valid summation order): samples not
    marked flip-prone agree to 1e-5; fewer than 1% of all samples differ by
    more (a hidden activation rounded to the neighbouring BF16 value), and none
    by more than 1e-3 of the logit scale."""
    rng = np.random.default_rng(4)
    p = (0.3 * rng.standard_normal(IO.NP)).astype(np.float32)
    norm = np.concatenate([rng.standard_normal(12), 0.5 + rng.random(12)]).astype(np.float32)
    X = (2 * rng.standard_normal((20000, 12))).astype(np.float32)
    z32, _ = IO.forward(p, norm, X)
    ztc, prone = IO.forward_tensor_core(p, norm, X)
    scale = 1 + np.abs(ztc).max()
    d = np.abs(z32.astype(np.float64) - ztc)
    assert d[~prone].max() <= 1e-5 * scale
    assert (d > 1e-5 * scale).mean() < 0.01 and d.max() <= 1e-3 * scale


def test_dilate_grows_by_face_layers():
    """dilate(): one layer adds the face neighbours (not the diagonal ones), two
    layers the cells within two face steps; boundary cells have fewer."""
    from oceano_gb300 import uniform_mesh
    from oceano_gb300.indicator import cell_info, dilate
    mesh = uniform_mesh(7, 7, (0.0, 1.0, 0.0, 1.0), False, 1)
    info = cell_info(mesh)
    centre = np.argmin(np.abs(mesh.vertices[:, 0] - 3 / 7) + np.abs(mesh.vertices[:, 1] - 3 / 7))
    f = np.zeros(mesh.n_cells, bool)
    f[centre] = True
    assert dilate(f, info, 1).sum() == 5
    assert dilate(f, info, 2).sum() == 13
    corner = np.argmin(mesh.vertices[:, 0] + mesh.vertices[:, 1])
    g = np.zeros(mesh.n_cells, bool)
    g[corner] = True
    assert dilate(g, info, 1).sum() == 3


def test_degree_transfer_round_trip_and_conservation():
    """p-adaptation transfer: degree 1 -> 2 -> 1 returns the degree-1 state;
    2 -> 1 keeps the cell integrals of zeta and q (Gauss-Lobatto quadrature of
    the nodal values is exact for these polynomial degrees)."""
    from oceano_gb300.adapt import transfer_state
    from oceano_gb300.basis import lobatto
    rng = np.random.default_rng(5)
    nc = 40
    d1 = np.ones(nc, np.int32)
    d2 = np.where(rng.random(nc) < 0.5, 2, 1).astype(np.int32)
    n1 = int(((d1 + 1) ** 2).sum())
    z1, q1 = rng.standard_normal(n1), rng.standard_normal(2 * n1)
    z2, q2 = transfer_state(d1, d2, z1, q1)
    zb, qb = transfer_state(d2, d1, z2, q2)
    assert np.allclose(zb, z1, atol=1e-13) and np.allclose(qb, q1, atol=1e-13)
    # conservation of 2 -> 1 on an arbitrary degree-2 state
    dd = np.full(nc, 2, np.int32)
    n2 = 9 * nc
    z2, q2 = rng.standard_normal(n2), rng.standard_normal(2 * n2)
    zc, qc = transfer_state(dd, d1, z2, q2)
    w2 = np.outer(lobatto(3)[1], lobatto(3)[1]).ravel()
    w1 = np.outer(lobatto(2)[1], lobatto(2)[1]).ravel()
    assert np.allclose(z2.reshape(nc, 9) @ w2, zc.reshape(nc, 4) @ w1, atol=1e-13)
    qa, qb2 = q2.reshape(nc, 2, 9), qc.reshape(nc, 2, 4)
    assert np.allclose(qa @ w2, qb2 @ w1, atol=1e-13)


def test_tensor_core_gradient_close_to_the_fp32_order_one():
    """The gradient over the tensor-core forward's activations (what the GPU's
    tensor-core gradient is checked against) and over the FP32-order forward
    agree up to the activations' BF16 rounding differences."""
    p, norm, X, y = random_net(4)
    l0, g0 = IO.loss_and_grad(p, norm, X, y, 3.0)
    l1, g1 = IO.loss_and_grad(p, norm, X, y, 3.0, tensor_core=True)
    assert abs(l1 - l0) <= 1e-3 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0)
