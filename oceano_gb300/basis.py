"""1D rules of the FE_DGQ basis (NumPy): Gauss-Lobatto nodes and Gauss points on [0,1]."""
from __future__ import annotations

import numpy as np


def gauss(n: int):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1), 0.5 * w


def lobatto(n: int):
    """Gauss-Lobatto points and weights on [0,1] (n >= 2)."""
    if n == 2:
        return np.array([0.0, 1.0]), np.array([0.5, 0.5])
    m = n - 1
    P = np.polynomial.legendre.Legendre.basis(m)
    inner = np.sort(P.deriv().roots().real)
    x = np.concatenate([[-1.0], inner, [1.0]])
    w = 2.0 / (m * n * P(x) ** 2)
    return 0.5 * (x + 1), 0.5 * w


def lagrange_matrix(nodes, points, derivative=False):
    """M[q, i] = l_i(points[q]) (or its derivative) for the Lagrange basis on nodes."""
    nodes = np.asarray(nodes)
    points = np.asarray(points)
    n = len(nodes)
    M = np.zeros((len(points), n))
    for i in range(n):
        others = np.delete(nodes, i)
        denom = np.prod(nodes[i] - others)
        if not derivative:
            M[:, i] = np.prod(points[:, None] - others[None, :], axis=1) / denom
        else:
            s = np.zeros(len(points))
            for k in range(n - 1):
                rest = np.delete(others, k)
                s += np.prod(points[:, None] - rest[None, :], axis=1) if len(rest) else 1.0
            M[:, i] = s / denom
    return M
