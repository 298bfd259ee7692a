"""Learned refinement indicator on the GPU against its CPU oracle.

* features: the 12 per-cell features vs oracle/indicator_oracle.features;
* BF16 MLP forward: logits vs the oracle's emulation of the same roundings;
* gradient: loss and gradient vs the oracle's analytic gradient (whose own
  formulas are checked against finite differences on the CPU);
* Adam and the normalisation fit vs NumPy;
* a small train / evaluate cycle on a vortex ensemble.
"""
import numpy as np
import pytest

from oracle import indicator_oracle as IO
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def random_net(seed, n):
    rng = np.random.default_rng(seed)
    p = (0.3 * rng.standard_normal(IO.NP)).astype(np.float32)
    norm = np.concatenate([rng.standard_normal(12), 0.5 + rng.random(12)]).astype(np.float32)
    X = (2 * rng.standard_normal((n, 12))).astype(np.float32)
    y = (rng.random(n) < 0.3).astype(np.float32)
    return p, norm, X, y


def model_with(p, norm):
    from oceano_gb300.indicator import LearnedIndicator
    m = LearnedIndicator(seed=7)
    m.params = p
    m.normalization = norm
    return m


def test_features_match_oracle(gpu_lib):
    import torch
    from cases import VORTEX, hanging_mesh, mixed_degree
    from oceano_gb300.indicator import cell_info, features
    from oceano_gb300.operator import OceanoOperator
    mesh = mixed_degree(hanging_mesh(2, seed=11))
    member = (np.arange(mesh.n_cells) >= mesh.n_cells // 2).astype(np.int32)
    info = cell_info(mesh, member)
    orc = O.Oracle(mesh, bcs={0: ("wall",)}, vortex=VORTEX + [0, 0])
    z, q = orc.project_vortex(0.0)
    op = OceanoOperator(mesh)
    op.set_wall_boundary(0)
    f, fl, w = features(op, torch.from_numpy(z).cuda(), torch.from_numpy(q).cuda(),
                        torch.from_numpy(info).cuda(), 2, 1e-5, want_vorticity=True)
    f, fl, w = f.cpu().numpy(), fl.cpu().numpy(), w.cpu().numpy()
    fo, flo, wo = IO.features(orc, mesh, z, q, info, 2, 1e-5)
    assert np.allclose(f[:, :3], fo[:, :3], rtol=1e-6, atol=1e-7)
    assert np.allclose(w, wo, rtol=1e-5, atol=1e-6)
    # relative vorticity magnitudes on a log10 scale: compare the magnitudes
    # (FP32 vorticity of the two sides agrees to 1e-5 relative, 1e-6 absolute)
    mag = lambda v: 10.0 ** v.astype(np.float64) - 1e-12
    assert np.allclose(mag(f[:, 3]), mag(fo[:, 3]), rtol=1e-5, atol=1e-6)
    assert np.allclose(mag(f[:, 6:10]), mag(fo[:, 6:10]), rtol=1e-5, atol=1e-6)
    # log differences across the cell: a magnitude m known to 1e-5 relative and
    # 1e-6 absolute has log10 known to (1e-5 + 1e-6 / m) / ln 10 (plus FP32 rounding)
    m = mag(fo[:, 6:10])
    tol = (1e-5 + 1e-6 / np.maximum(m, 1e-12)) / np.log(10.0) + 1e-5
    assert (np.abs(f[:, 4] - fo[:, 4]) <= 0.5 * (tol[:, 0] + tol[:, 1])).all()
    assert (np.abs(f[:, 5] - fo[:, 5]) <= 0.5 * (tol[:, 2] + tol[:, 3])).all()
    assert ((m[:, 0] > 1e-3) & (m[:, 1] > 1e-3)).sum() >= 4  # some resolved differences
    assert np.array_equal(f[:, 10:], fo[:, 10:])
    sure = np.abs(wo - 1e-5) > 1e-6  # flags away from the threshold
    assert np.array_equal(fl[sure], flo[sure])


@pytest.mark.parametrize("n", [3000, 70001])
def test_mlp_forward_matches_oracle(gpu_lib, n):
    """Tensor-core forward (BF16 MMA, FP32 accumulation) against the oracle's
    emulation: 1e-5 wherever no hidden activation lies within the hardware's
    summation-order uncertainty of a BF16 rounding boundary.  Where one does,
    the activation may round to the neighbouring BF16 value (one BF16 step,
    2^-8 relative) and move the logit through the next layer: fewer than 1%
    of the samples differ by more than 1e-5, none by more than 1e-2 of the
    logit scale."""
    import torch
    p, norm, X, _ = random_net(1, n)
    m = model_with(p, norm)
    z = m.forward(torch.from_numpy(X).cuda()).cpu().numpy().astype(np.float64)
    zo, prone = IO.forward_tensor_core(p, norm, X)
    scale = 1 + np.abs(zo).max()
    d = np.abs(z - zo)
    assert d[~prone].max() <= 1e-5 * scale
    assert (d > 1e-5 * scale).mean() < 0.01 and d.max() <= 1e-2 * scale


@pytest.mark.parametrize("n", [100, 1000, 70000])
def test_mlp_gradient_matches_oracle(gpu_lib, n):
    """The tensor-core gradient (forward, back-propagation and parameter sums on
    BF16 MMAs, back-propagated signals as two BF16 terms) against the oracle's
    gradient over the tensor-core forward's activations, on the samples that are
    not flip-prone (a different summation order may round a hidden activation
    of those to the neighbouring BF16 value): loss 1e-5, gradient 1e-4 of its
    norm (the two-term signals keep about 16 bits)."""
    import torch
    p, norm, X, y = random_net(2, n)
    _, prone = IO.forward_tensor_core(p, norm, X)
    X, y = np.ascontiguousarray(X[~prone]), np.ascontiguousarray(y[~prone])
    m = model_with(p, norm)
    loss, g = m.gradient(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), 3.0)
    lo, go = IO.loss_and_grad(p, norm, X, y, 3.0, tensor_core=True)
    assert abs(loss - lo) <= 1e-5 * abs(lo)
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)


def test_adam_step_and_normalisation(gpu_lib):
    import torch
    p, norm, X, y = random_net(3, 500)
    m = model_with(p, norm)
    _, g = m.gradient(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), 1.0)
    m.adam_step(1e-3)
    # first Adam step: m = 0.1 g, v = 0.001 g^2, bias corrections 0.1 and 0.001
    g64 = g.astype(np.float64)
    expect = p - 1e-3 * g64 / (np.abs(g64) + 1e-8)
    assert np.allclose(m.params, expect, rtol=1e-5, atol=1e-7)
    m.fit_normalization(torch.from_numpy(X).cuda())
    nrm = m.normalization
    assert np.allclose(nrm[:12], X.mean(0), rtol=1e-4, atol=1e-5)
    assert np.allclose(nrm[12:], 1 / X.std(0), rtol=1e-4)


def test_train_and_evaluate_small_ensemble(gpu_lib):
    """Train on 4 members (seeds 100..103), evaluate on 4 others (seeds 0..3):
    the loss falls and the learned refinement set needs no more remeshes than
    the vorticity indicator's."""
    import torch
    from oceano_gb300 import workloads as W
    from oceano_gb300.indicator import (LearnedIndicator, cell_info, evaluate, member_of_cells,
                                        run_and_record, training_pairs)

    def small(seed0):
        mem = W.ensemble_members(4, seed0)
        for m in mem:
            m["target"] = 5000.0
        op, z, q, mem, meshes = W.ensemble(members=mem, precision="mixed")
        info = torch.from_numpy(cell_info(op.mesh, member_of_cells(meshes))).cuda()
        zt, qt = torch.from_numpy(z).cuda(), torch.from_numpy(q).cuda()
        dt = 0.075 / op.compute_cell_transport_speed(zt, qt)
        return op, zt, qt, info, dt, member_of_cells(meshes)

    op, z, q, info, dt, _ = small(100)
    recs = run_and_record(op, z, q, info, 4, dt, 60, every=1)
    X, Y = training_pairs(recs, 10)
    model = LearnedIndicator(seed=1)
    model.fit_normalization(X)
    pos = float((Y.numel() - Y.sum()) / max(float(Y.sum()), 1.0))
    losses = model.train(X, Y, epochs=150, lr=3e-3, pos_weight=pos)
    assert losses[-1] < 0.7 * losses[0]
    op2, z2, q2, info2, dt2, members = small(0)
    recs2 = run_and_record(op2, z2, q2, info2, 4, dt2, 40, every=1)
    res = evaluate(model, recs2, 10, members, 4)
    assert res["recall"] > 0.8
    assert res["remesh_learned"] <= res["remesh_vorticity"]


def test_remesh_runs_conserve_and_count(gpu_lib):
    """p-adaptive remeshing of independent members: a remesh (degree map change
    with state transfer) keeps the member's mass; the network-free buffer
    (flags grown by one cell layer) remeshes no more often than the bare
    flags, at a free-surface error within 10% of theirs."""
    from oceano_gb300 import workloads as W
    from oceano_gb300.adapt import AdaptiveMember, remesh_experiment
    from oceano_gb300.basis import lobatto
    members = W.ensemble_members(3, 1000)
    for m in members:
        m["target"] = 5000.0
    mesh = W.member_mesh(members[0])
    mesh = mesh.with_degree(np.ones(mesh.n_cells, np.int32))
    am = AdaptiveMember(mesh, members[0]["vortex"], np.zeros(mesh.n_cells, bool))

    def mass(member):
        v = member.mesh.vertices
        det = np.abs((v[:, 2] - v[:, 0]) * (v[:, 5] - v[:, 1]) - (v[:, 4] - v[:, 0]) * (v[:, 3] - v[:, 1]))
        off = member.mesh.offsets()
        tot = 0.0
        for c in range(member.mesh.n_cells):
            N = int(member.mesh.degree[c]) + 1
            w = np.outer(lobatto(N)[1], lobatto(N)[1]).ravel()
            tot += det[c] * (w @ member.z[off[c]:off[c + 1]])
        return tot

    am.step()
    m0 = mass(am)
    rng = np.random.default_rng(0)
    am.remesh(rng.random(mesh.n_cells) < 0.3)
    assert abs(mass(am) - m0) <= 1e-13 * abs(m0)
    am.remesh(rng.random(mesh.n_cells) < 0.3)
    assert abs(mass(am) - m0) <= 1e-13 * abs(m0)
    am.step()
    am.op.close()
    bare = remesh_experiment(members, "vorticity", 15)
    grown = remesh_experiment(members, "dilated", 15, layers=1)
    assert grown["remeshes"] <= bare["remeshes"]
    assert grown["refined_over_flagged"] >= 1.0
    e0, e1 = bare["free_surface_l2_error"], grown["free_surface_l2_error"]
    assert np.isfinite(e0) and np.isfinite(e1) and abs(e1 - e0) <= 0.1 * e0
