"""ctypes front-end of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module; the product never does.  Parity unpinned: see the header
of oceano_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboceano_oracle.so")
SRC = os.path.join(HERE, "oceano_oracle.c")

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")

BC = {"none": 0, "wall": 1, "supercritical_inflow": 2, "supercritical_outflow": 3,
      "height_inflow": 4, "discharge_inflow": 5, "absorbing_outflow": 6}


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, OpenMP, no FMA contraction: same results on x86 and Arm)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               SRC, "-o", LIB, "-lm"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.oc_oracle_create.restype = C.c_void_p
        L.oc_oracle_create.argtypes = [C.c_int, _ip, _dp, C.c_int, C.c_int, _ip, _ip, _bp, _bp,
                                       _bp, _bp, _ip, _dp, _ip, _ip, _ip, _dp, _dp]
        L.oc_oracle_destroy.argtypes = [C.c_void_p]
        L.oc_oracle_n_dofs.restype = C.c_int64
        L.oc_oracle_n_dofs.argtypes = [C.c_void_p]
        L.oc_oracle_static_sizes.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.int64)]
        L.oc_oracle_points.argtypes = [C.c_void_p, C.c_int, _dp]
        L.oc_oracle_set_static.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        pp = C.POINTER(C.c_void_p)
        L.oc_oracle_stage_erk.restype = C.c_int
        L.oc_oracle_stage_erk.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, _dp,
                                          C.c_void_p, C.c_void_p, C.c_void_p, pp, pp,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oc_oracle_stage_ark.restype = C.c_int
        L.oc_oracle_stage_ark.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, _dp, _dp,
                                          C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, pp,
                                          pp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oc_oracle_apply.restype = C.c_int
        L.oc_oracle_apply.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]
        L.oc_oracle_transport_speed.restype = C.c_double
        L.oc_oracle_transport_speed.argtypes = [C.c_void_p, _dp, _dp]
        L.oc_oracle_project_vortex.argtypes = [C.c_void_p, C.c_double, _dp, _dp]
        L.oc_oracle_velocity_field.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.oc_oracle_vorticity.argtypes = [C.c_void_p, _dp, C.c_int, _fp]
        L.oc_oracle_errors_vortex.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp]
        L.oc_oracle_conservative_coarsening.argtypes = [C.c_void_p,
                                                        np.ctypeslib.ndpointer(np.uint8), _dp]
        L.oc_oracle_num_threads.restype = C.c_int
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """FP64 oracle bound to one mesh, parameter set and boundary-condition table."""

    def __init__(self, mesh, g=9.81, cu=0.1, nu=0.0, friction=0, max_iter=15, batch=1,
                 bcs=None, vortex=None, cell_rule=0):
        """cell_rule: Gauss points per direction of the cell integrals and boundary
        faces (the reference's n_points_1d, main.cc:216): 0 floor(1.5 p) + 1, 1 p + 1."""
        L = lib()
        self.mesh = mesh
        bc_kind = np.zeros(16, np.int32)
        bc_fn = np.zeros(16, np.int32)
        bc_c = np.zeros(48)
        for b, spec in (bcs or {}).items():
            bc_kind[b] = BC[spec[0]]
            if len(spec) > 1 and spec[1] == "vortex":
                bc_fn[b] = 1
            elif len(spec) > 1:
                bc_c[3 * b:3 * b + len(spec[1])] = spec[1]
        vx = np.zeros(8) if vortex is None else np.asarray(vortex, np.float64)
        self.h = L.oc_oracle_create(
            mesh.n_cells, mesh.degree, mesh.vertices.ravel(), mesh.n_inner, mesh.n_bnd,
            mesh.cell_m, mesh.cell_p if mesh.n_inner else np.zeros(1, np.int32),
            mesh.face_m, mesh.face_p if mesh.n_inner else np.zeros(1, np.int8),
            mesh.subface if mesh.n_inner else np.zeros(1, np.int8),
            mesh.orient if mesh.n_inner else np.zeros(1, np.int8),
            mesh.bid if mesh.n_bnd else np.zeros(1, np.int32),
            np.array([g, cu, nu], np.float64),
            np.array([friction, max_iter, batch, cell_rule], np.int32),
            bc_kind, bc_fn, bc_c, vx)
        self.n = int(L.oc_oracle_n_dofs(self.h))
        self._static = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().oc_oracle_destroy(self.h)
            self.h = None

    def static_sizes(self):
        out = np.zeros(5, np.int64)
        lib().oc_oracle_static_sizes(self.h, out)
        return out

    def points(self, which):
        n = int(self.static_sizes()[which])
        per = {0: 5, 1: 1, 2: 2, 3: 2, 4: 1}[which]
        npts = n // per if which != 3 else n
        xy = np.zeros((npts, 2))
        lib().oc_oracle_points(self.h, which, xy)
        return xy

    def set_static(self, cell0=None, cell1=None, cell2=None, face=None, bnd=None):
        self._static = [None if a is None else np.ascontiguousarray(a, np.float64)
                        for a in (cell0, cell1, cell2, face, bnd)]
        lib().oc_oracle_set_static(self.h, *[_ptr(a) for a in self._static])

    def stage_erk(self, stage, n_stages, t, f, rz, rq, kz, kq, sol_z, sol_q, next_z, next_q,
                  rvel=None):
        pp = C.c_void_p * len(kz)
        kzp = pp(*[k.ctypes.data for k in kz])
        kqp = pp(*[k.ctypes.data for k in kq])
        r = lib().oc_oracle_stage_erk(self.h, stage, n_stages, t, np.asarray(f, np.float64),
                                      _ptr(rz), _ptr(rq), _ptr(rvel), kzp, kqp, _ptr(sol_z),
                                      _ptr(sol_q), _ptr(next_z), _ptr(next_q))
        if r:
            raise RuntimeError("oracle: unknown boundary id")

    def stage_ark(self, stage, n_stages, t, f, ft, fm, rz, rq, kz, kq, sol_z, sol_q, next_z,
                  next_q, rvel=None):
        kzp = (C.c_void_p * len(kz))(*[k.ctypes.data for k in kz])
        kqp = (C.c_void_p * len(kq))(*[k.ctypes.data for k in kq])
        r = lib().oc_oracle_stage_ark(self.h, stage, n_stages, t, np.asarray(f, np.float64),
                                      np.asarray(ft, np.float64), fm, _ptr(rz), _ptr(rq),
                                      _ptr(rvel), kzp, kqp, _ptr(sol_z), _ptr(sol_q),
                                      _ptr(next_z), _ptr(next_q))
        if r:
            raise RuntimeError("oracle: unknown boundary id")

    def apply(self, t, z, q):
        """dst = M^-1 L_h(t, src), exact Gauss p+1 cell inverse for all variables."""
        dz, dq = np.zeros(self.n), np.zeros(2 * self.n)
        if lib().oc_oracle_apply(self.h, t, np.ascontiguousarray(z, np.float64),
                                 np.ascontiguousarray(q, np.float64), dz, dq):
            raise RuntimeError("oracle: unknown boundary id")
        return dz, dq

    def transport_speed(self, z, q):
        return float(lib().oc_oracle_transport_speed(self.h, z, q))

    def project_vortex(self, t=0.0):
        z = np.zeros(self.n)
        q = np.zeros(2 * self.n)
        lib().oc_oracle_project_vortex(self.h, t, z, q)
        return z, q

    def velocity_field(self, z, q):
        u = np.zeros(2 * self.n)
        lib().oc_oracle_velocity_field(self.h, z, q, u)
        return u

    def errors_vortex(self, z, q, t):
        out = np.zeros(2)
        lib().oc_oracle_errors_vortex(self.h, t, z, q, out)
        return out

    def conservative_coarsening(self, mark, z):
        z = np.ascontiguousarray(z, np.float64).copy()
        lib().oc_oracle_conservative_coarsening(self.h, np.ascontiguousarray(mark, np.uint8), z)
        return z

    def vorticity(self, u, n_q_1d):
        out = np.zeros(self.mesh.n_cells, np.float32)
        lib().oc_oracle_vorticity(self.h, u, n_q_1d, out)
        return out


def num_threads() -> int:
    return int(lib().oc_oracle_num_threads())


# ---------------------------------------------------------------------------
# Reference integrators restated (ExplicitRungeKuttaIntegrator.h:179-298,
# AdditiveRungeKuttaIntegrator.h:206-339) driving the oracle stages.
# ---------------------------------------------------------------------------

def erk_step(orc, a, b, c, t, dt, z, q):
    """One explicit RK step in Butcher form, in place on (z, q)."""
    s = len(b)
    n = orc.n
    kz = [np.zeros(n) for _ in range(s + 1)]
    kq = [np.zeros(2 * n) for _ in range(s + 1)]
    nz, nq = np.zeros(n), np.zeros(2 * n)
    for st in range(s):
        f = np.array(b if st == s - 1 else a[st], np.float64) * dt
        rz, rq = (z.copy(), q.copy()) if st == 0 else (nz.copy(), nq.copy())
        orc.stage_erk(st, s, t + c[st] * dt, f, rz, rq, kz, kq, z, q, nz, nq)


def ark_step(orc, a, b, c, at, dt_, t, dt, z, q):
    """One additive RK step (explicit Giraldo + TR-BDF2 implicit friction)."""
    s = len(b)
    n = orc.n
    kz = [np.zeros(n) for _ in range(s + 1)]
    kq = [np.zeros(2 * n) for _ in range(2 * s)]
    nz, nq = np.zeros(n), np.zeros(2 * n)
    for st in range(s):
        last = st == s - 1
        f = np.array(b if last else a[st], np.float64) * dt
        ft = np.array(b if last else at[st], np.float64) * dt
        fm = dt_[st] * dt if st < len(dt_) else 0.0
        rz, rq = (z.copy(), q.copy()) if st == 0 else (nz.copy(), nq.copy())
        orc.stage_ark(st, s, t + c[st] * dt, f, ft, fm, rz, rq, kz, kq, z, q, nz, nq)


# Butcher tableaux restated from time_stepping.h:136-379 (checker copy).
_chi = 2.0 - np.sqrt(2.0)
TABLEAUX = {
    "ssp33": dict(a=[[1.0], [0.25, 0.25]], b=[1 / 6, 1 / 6, 2 / 3], c=[0.0, 1.0, 0.5]),
    "ssp22": dict(a=[[1.0]], b=[0.5, 0.5], c=[0.0, 1.0]),
    "fe": dict(a=[], b=[1.0], c=[0.0]),
    "rk4": dict(a=[[0.5], [0.0, 0.5], [0.0, 0.0, 1.0]], b=[1 / 6, 1 / 3, 1 / 3, 1 / 6],
                c=[0.0, 0.5, 0.5, 1.0]),
    "giraldo32": dict(a=[[_chi], [0.5, 0.5]], b=[0.5 - _chi / 4, 0.5 - _chi / 4, _chi / 2],
                      c=[0.0, _chi, 1.0]),
    "trbdf2": dict(a=[[_chi / 2], [1 / (2 * np.sqrt(2)), 1 / (2 * np.sqrt(2))]],
                   b=[0.5 - _chi / 4, 0.5 - _chi / 4, _chi / 2], c=[0.0, _chi, 1.0],
                   d=[_chi / 2, 1 - 1 / np.sqrt(2)]),
}
