"""CPU restatement of the learned refinement indicator (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module: it is the checker of the GPU features
kernel and of the BF16 MLP kernels of oceano_gb300/csrc/oc_mlp.cu, never a
product path.

* features(): the 12 per-cell features of oc_indicator_features, from the FP64
  oracle's velocity field and vorticity indicator (hpTuner.h:247-305, QGauss of
  the largest degree) and cell means by Gauss-Lobatto quadrature.
* forward(): the MLP forward pass with the GPU's roundings emulated: BF16
  round-to-nearest-even of weights, inputs and hidden activations, FP32 fused
  multiply-adds in the GPU's order (an FP32 product is exact in FP64, so
  fp32(fp64(a*b) + c) is the fused result except for double-rounding ties).
  exact=True: the same network in FP64 without roundings (for finite differences).
* forward_tensor_core(): the roundings of the tensor-core forward kernel, with
  the samples whose result depends on the hardware's summation order marked.
* loss_and_grad(): weighted BCE-with-logits loss and its analytic gradient,
  treating the roundings as identities, accumulated in FP64.
"""
from __future__ import annotations

import numpy as np

NF, NH = 12, 64
OW1, OB1 = 0, NH * NF
OW2, OB2 = OB1 + NH, OB1 + NH + NH * NH
OW3, OB3 = OB2 + NH, OB2 + 2 * NH
NP = OB3 + 1
f32, f64 = np.float32, np.float64


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=f32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(f32)


def fma32(a, b, c):
    return (np.asarray(a, f32).astype(f64) * np.asarray(b, f32).astype(f64)
            + np.asarray(c, f32).astype(f64)).astype(f32)


def unpack(p):
    p = np.asarray(p)
    return (p[OW1:OB1].reshape(NH, NF), p[OB1:OW2], p[OW2:OB2].reshape(NH, NH), p[OB2:OW3],
            p[OW3:OB3], p[OB3])


def forward(params, norm, X, exact=False):
    """Logits and activations (xh, h1, h2) of feature rows X [n, 12]."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    mean, istd = np.asarray(norm[:NF]), np.asarray(norm[NF:])
    if exact:
        xh = (X.astype(f64) - mean) * istd
        h1 = np.maximum(xh @ W1.T.astype(f64) + b1, 0.0)
        h2 = np.maximum(h1 @ W2.T.astype(f64) + b2, 0.0)
        return h2 @ w3.astype(f64) + b3, (xh, h1, h2)
    W1b, W2b, w3b = bf16(W1), bf16(W2), bf16(w3)
    X = np.asarray(X, f32)
    xh = bf16((X - mean.astype(f32)).astype(f32) * istd.astype(f32))
    n = X.shape[0]
    h1 = np.empty((n, NH), f32)
    for k in range(NH):
        a = np.full(n, b1[k], f32)
        for i in range(NF):
            a = fma32(W1b[k, i], xh[:, i], a)
        h1[:, k] = bf16(np.maximum(a, f32(0)))
    h2 = np.empty((n, NH), f32)
    z = np.full(n, b3, f32)
    for j in range(NH):
        a = np.full(n, b2[j], f32)
        for k in range(NH):
            a = fma32(W2b[j, k], h1[:, k], a)
        h2[:, j] = bf16(np.maximum(a, f32(0)))
        z = fma32(w3b[j], h2[:, j], z)
    return z, (xh, h1, h2)


def _bf16_boundary_distance(v):
    """Distance of FP64 values to the nearest BF16 rounding boundary (the
    midpoint between two adjacent BF16 numbers), for v > 0."""
    v = np.asarray(v, f64)
    b = bf16(v.astype(f32)).astype(f64)
    e = np.floor(np.log2(np.maximum(np.abs(v), 1e-300)))
    ulp = np.exp2(e - 7)
    return 0.5 * ulp - np.abs(v - b)


def forward_tensor_core(params, norm, X, margin=1e-6, activations=False):
    """The forward pass of the tensor-core kernel: BF16 weights, inputs and
    activations as forward(), each layer's sum of exact BF16 products formed
    at FP32 precision or better (here exactly, in FP64) before the BF16
    rounding.  Returns (logits, flip_prone): flip_prone marks the samples with
    a hidden activation whose exact value lies within `margin` x (sum of
    |terms|) of a BF16 rounding boundary, where a different summation order of
    the hardware may round the activation to the neighbouring BF16 value.
    activations=True also returns (xh, h1, h2)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    mean, istd = np.asarray(norm[:NF]), np.asarray(norm[NF:])
    W1b, W2b, w3b = (bf16(a).astype(f64) for a in (W1, W2, w3))
    X = np.asarray(X, f32)
    xh = bf16((X - mean.astype(f32)).astype(f32) * istd.astype(f32)).astype(f64)
    prone = np.zeros(X.shape[0], bool)

    def layer(a_in, W, b):
        a = a_in @ W.T + np.asarray(b, f64)
        mag = np.abs(a_in) @ np.abs(W).T + np.abs(np.asarray(b, f64))
        pos = a > 0
        near = pos & (_bf16_boundary_distance(np.where(pos, a, 1.0)) < margin * mag)
        near |= np.abs(a) < margin * mag  # sign of a cancellation
        return bf16(np.maximum(a, 0.0).astype(f32)).astype(f64), near.any(axis=1)

    h1, p1 = layer(xh, W1b, b1)
    h2, p2 = layer(h1, W2b, b2)
    z = h2 @ w3b + f64(b3)
    if activations:
        return z, p1 | p2, (xh, h1, h2)
    return z, p1 | p2


def loss_and_grad(params, norm, X, y, pos_weight, exact=False, tensor_core=False):
    """Mean weighted BCE-with-logits and its gradient (FP64 accumulation).
    tensor_core=True takes the activations of forward_tensor_core (the GPU's
    tensor-core forward pass; compare on samples that are not flip-prone)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    if tensor_core:
        z, _, (xh, h1, h2) = forward_tensor_core(params, norm, X, activations=True)
    else:
        z, (xh, h1, h2) = forward(params, norm, X, exact)
    z, xh, h1, h2 = (np.asarray(a, f64) for a in (z, xh, h1, h2))
    if not exact:  # the GPU multiplies by the BF16 weights in the backward pass as well
        W2, w3 = bf16(W2).astype(f64), bf16(w3).astype(f64)
    y = np.asarray(y, f64)
    n = len(y)
    wt = np.where(y > 0.5, pos_weight, 1.0)
    loss = np.sum(wt * (np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z))) - y * z)) / n
    dz = wt * (1.0 / (1.0 + np.exp(-z)) - y) / n
    d2 = np.where(h2 > 0, dz[:, None] * w3[None, :], 0.0)
    d1 = np.where(h1 > 0, d2 @ W2, 0.0)
    g = np.zeros(NP)
    g[OW1:OB1] = (d1.T @ xh).ravel()
    g[OB1:OW2] = d1.sum(0)
    g[OW2:OB2] = (d2.T @ h1).ravel()
    g[OB2:OW3] = d2.sum(0)
    g[OW3:OB3] = dz @ h2
    g[OB3] = dz.sum()
    return loss, g


def lobatto_weights(n):
    """Gauss-Lobatto weights on [0, 1] with n points (ordered nodes)."""
    from numpy.polynomial import legendre as L
    c = np.zeros(n)
    c[-1] = 1.0
    inner = np.sort(L.legroots(L.legder(c)).real) if n > 2 else np.zeros(0)
    x = np.concatenate([[-1.0], inner, [1.0]])
    w = 2.0 / (n * (n - 1) * L.legval(x, c) ** 2)
    return 0.5 * w


def _log_mag(x):
    """log10(|x| + 1e-12) of FP32 relative vorticities, in FP32."""
    return np.log10(np.abs(np.asarray(x, f32)) + f32(1e-12)).astype(f32)


def features(orc, mesh, z, q, info, n_members, threshold):
    """The 12 features, flags and normalised vorticity of every cell."""
    u = orc.velocity_field(z, q)
    w = np.asarray(orc.vorticity(u, int(mesh.degree.max())), f64).astype(f32).astype(f64)
    off = mesh.offsets()
    nc = mesh.n_cells
    member = info[:, 5]
    wmax = np.zeros(n_members)
    np.maximum.at(wmax, member, w)
    inv = np.where(wmax[member] > 0, 1.0 / np.maximum(wmax[member], 1e-300), 0.0)
    w0 = (w * inv).astype(f32)
    feat = np.zeros((nc, 12), f32)
    for c in range(nc):
        p = int(mesh.degree[c])
        N = p + 1
        mw = lobatto_weights(N)
        W = np.outer(mw, mw).ravel()
        a = off[c]
        n = N * N
        feat[c, 0] = W @ z[a:a + n]
        feat[c, 1] = W @ q[2 * a:2 * a + n]
        feat[c, 2] = W @ q[2 * a + n:2 * a + 2 * n]
        nb = [w[info[c, f]] * inv[c] if info[c, f] >= 0 else w0[c] for f in range(4)]
        nb = _log_mag(np.asarray(nb, f32))
        feat[c, 3] = _log_mag(w0[c])
        feat[c, 4] = 0.5 * (nb[1] - nb[0])
        feat[c, 5] = 0.5 * (nb[3] - nb[2])
        feat[c, 6:10] = nb
        feat[c, 10] = info[c, 4]
        feat[c, 11] = p
    flags = (w0 > threshold).astype(f32)
    return feat, flags, w0
