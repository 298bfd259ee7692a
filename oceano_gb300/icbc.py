"""Synthetic initial and boundary data for the workloads (NumPy, host side).

* The travelling vortex of lib/include/icbc/Icbc_ShallowWaterVortex.h:139-226
  (regularity p=2), parameterised by depth h0, background speed u_inf, radius
  r0, strength Gamma and centre.  ``gamma_for_peak`` picks Gamma so that the
  largest tangential speed equals a given peak (the configured vortices are
  specified by their peak speed).  ``gamma_for_hmin`` is the reference's own
  choice (Gamma from the depth at the centre).
* The channel bump and lake at rest of the IMEX workload (bathymetry in the
  reference convention depth = zeta + zb, ShallowWater.h:312-320).
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh


def _H(x):
    cosx, cos2x, sin2x, sinx = np.cos(x), np.cos(2 * x), np.sin(2 * x), np.sin(x)
    cosx2, cos2x2, x2 = cosx * cosx, cos2x * cos2x, x * x
    return (0.091145833 * cos2x + 0.182291667 * x * sin2x
            + cosx ** 6 * (0.015625 * cosx2 + 0.024305556) + 0.011393229 * cos2x2
            + 0.13671875 * x2 + 0.045572917 * x * cos2x * sin2x
            + 0.125 * x * cosx ** 5 * sinx * (cosx2 + 1.166666667))


def gamma_for_hmin(h0=1.0, hmin=0.9, r0=0.25, g=9.81):
    """Icbc_ShallowWaterVortex.h:160-164 (p = 2)."""
    return np.pi / (4 * r0) * np.sqrt(0.25 * g * (h0 - hmin) /
                                      (0.034179687 * np.pi ** 2 - 0.222222222))


def gamma_for_peak(peak, r0):
    """Gamma such that max_R R*4*Gamma*cos^4(pi R / (2 r0)) = peak."""
    th = np.linspace(0, np.pi / 2, 200001)
    f = (2 * r0 * th / np.pi) * np.cos(th) ** 4
    return peak / (4 * f.max())


def vortex(x, y, t, h0=1.0, uoo=1.0, r0=0.2, gamma=None, x0=0.5, y0=0.5, g=9.81):
    """(depth, u, v) of the travelling vortex at time t."""
    if gamma is None:
        gamma = gamma_for_peak(0.1, r0)
    xc, yc = x0 + uoo * t, y0
    rad = np.sqrt((x - xc) ** 2 + (y - yc) ** 2)
    rho_half = 0.5 * np.pi * rad / r0
    c2 = np.cos(rho_half) ** 2
    omega = 4 * gamma * c2 * c2
    num = 4 * gamma * r0
    inside = rad < r0
    h = np.where(inside, h0 - 1 / (g * np.pi ** 2) * num * num * 4 * (_H(0.5 * np.pi) - _H(rho_half)), h0)
    u = np.where(inside, uoo - (y - yc) * omega, uoo)
    v = np.where(inside, (x - xc) * omega, 0.0)
    return h, u, v


def vortex_params(h0=1.0, uoo=1.0, r0=0.2, peak=0.1, x0=0.5, y0=0.5):
    """The 6 numbers of OceanoOperator.set_vortex / the oracle's vortex block."""
    return [h0, uoo, r0, gamma_for_peak(peak, r0), x0, y0]


def channel_bathymetry(x):
    """zb = 2 - b(x), b = 0.2 - 0.05 (x-10)^2 on 8 < x < 12: 2 m depth at rest."""
    b = np.where((x > 8) & (x < 12), 0.2 - 0.05 * (x - 10.0) ** 2, 0.0)
    return 2.0 - b


def channel_problem_data(manning=0.03):
    def pd(x, y):
        zb = channel_bathymetry(np.asarray(x))
        return np.stack([zb, np.full_like(zb, manning), 0 * zb, 0 * zb, 0 * zb])
    return pd


def nodal_points(mesh: Mesh):
    """Physical coordinates of every DoF (Gauss-Lobatto nodes, lexicographic)."""
    from .basis import lobatto
    off = mesh.offsets()
    out = np.zeros((int(off[-1]), 2))
    for p in np.unique(mesh.degree):
        cells = np.nonzero(mesh.degree == p)[0]
        xn, _ = lobatto(int(p) + 1)
        ex, ey = np.meshgrid(xn, xn)  # ey varies along rows (iy), ex along columns (ix)
        ex, ey = ex.ravel()[None, :], ey.ravel()[None, :]
        v = mesh.vertices[cells]
        X = v[:, 0:1] + (v[:, 2:3] - v[:, 0:1]) * ex + (v[:, 4:5] - v[:, 0:1]) * ey
        Y = v[:, 1:2] + (v[:, 3:4] - v[:, 1:2]) * ex + (v[:, 5:6] - v[:, 1:2]) * ey
        idx = off[cells][:, None] + np.arange(ex.shape[1])[None, :]
        out[idx, 0] = X
        out[idx, 1] = Y
    return out
