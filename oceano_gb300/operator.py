"""Host-side mirror of oceano's SpaceDiscretization::OceanoOperator.

Same method names and argument meaning as the reference class
(lib/include/space_discretization/OceanDG.h:157-380); every call goes through
the C ABI of liboceano_gpu.so.  Vectors are NumPy arrays (host memory, copied
in and out by the library) or CUDA tensors (device memory, used in place on
the operator's stream).  Errors raise :class:`oceano_gb300._lib.OceanoError`
(the reference throws deal.II exceptions, e.g. the unknown-boundary-id
AssertThrow at OceanDG.h:1199-1203).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import OC_MEM_DEVICE, OC_MEM_HOST, check, lib

FRICTION = {"none": 0, "linear": 1, "manning": 2}
PRECISION = {"fp64": 0, "mixed": 1}


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and a.is_cuda


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous")
    return a.ctypes.data_as(C.c_void_p)


def _memory(*arrays) -> int:
    dev = [_is_device(a) for a in arrays if a is not None]
    if all(dev):
        return OC_MEM_DEVICE
    if not any(dev):
        for a in arrays:
            if a is not None and a.dtype != np.float64:
                raise TypeError("host vectors must be float64")
        return OC_MEM_HOST
    raise ValueError("mixing host and device vectors in one call")


class OceanoOperator:
    """GPU operator bound to one mesh (reinit + initialize_data_at_quadrature)."""

    def __init__(self, mesh, g=9.81, threshold_wetdry=0.1, horizontal_viscosity=0.0,
                 friction="none", max_iteration_height=15, batch_width=1, precision="fp64",
                 zeta_reference=0.0, cell_quadrature="default"):
        """cell_quadrature: Gauss points per direction of the cell integrals, boundary
        faces, cell/boundary static data and errors (the reference's n_points_1d,
        main.cc:216): "default" = floor(1.5 p) + 1, "p+1" = p + 1 (4x4 at p = 3)."""
        self.mesh = mesh
        self.precision = precision
        self._keep = [np.ascontiguousarray(a) for a in (
            mesh.degree.astype(np.int32), mesh.vertices.astype(np.float64).ravel(),
            mesh.cell_m.astype(np.int32), mesh.cell_p.astype(np.int32),
            mesh.face_m.astype(np.int8), mesh.face_p.astype(np.int8),
            mesh.subface.astype(np.int8), mesh.orient.astype(np.int8),
            mesh.bid.astype(np.int32))]
        k = self._keep
        desc = _lib.MeshDesc(mesh.n_cells, _ptr(k[0]), _ptr(k[1]), mesh.n_inner, mesh.n_bnd,
                             _ptr(k[2]), _ptr(k[3]), _ptr(k[4]), _ptr(k[5]), _ptr(k[6]),
                             _ptr(k[7]), _ptr(k[8]))
        prm = _lib.Params(g, threshold_wetdry, horizontal_viscosity, FRICTION[friction],
                          max_iteration_height, batch_width, PRECISION[precision],
                          zeta_reference, _lib.CELL_RULE[cell_quadrature])
        self.cell_quadrature = cell_quadrature
        h = C.c_void_p()
        st = lib().oc_create(C.byref(desc), C.byref(prm), C.byref(h))
        self.h = h
        if st != _lib.OC_OK:
            msg = lib().oc_last_error(h).decode() if h else ""
            if h:
                lib().oc_destroy(h)
                self.h = None
            raise _lib.OceanoError(st, msg)
        self.n_dofs = int(lib().oc_n_dofs(self.h))
        self.g = g

    def close(self):
        if getattr(self, "h", None):
            lib().oc_destroy(self.h)
            self.h = None

    __del__ = close

    # ---- ICBC::BcBase setters (IcbcBase.h:141-286) --------------------------------
    def set_boundary(self, bid, kind, function="constant", values=(0.0, 0.0, 0.0)):
        v = np.zeros(3)
        v[:len(values)] = values
        fn = 1 if function == "vortex" else 0
        check(lib().oc_set_boundary(self.h, bid, _lib.BC_KIND[kind], fn, _ptr(v)), self.h)

    def set_wall_boundary(self, bid):
        self.set_boundary(bid, "wall")

    def set_supercritical_inflow_boundary(self, bid, function="constant", values=(0, 0, 0)):
        self.set_boundary(bid, "supercritical_inflow", function, values)

    def set_supercritical_outflow_boundary(self, bid):
        self.set_boundary(bid, "supercritical_outflow")

    def set_height_inflow_boundary(self, bid, zeta):
        self.set_boundary(bid, "height_inflow", values=(zeta,))

    def set_discharge_inflow_boundary(self, bid, discharge):
        self.set_boundary(bid, "discharge_inflow", values=(0.0, discharge))

    def set_absorbing_outflow_boundary(self, bid, function="constant", values=(0, 0, 0)):
        self.set_boundary(bid, "absorbing_outflow", function, values)

    def set_vortex(self, h0, uoo, r0, gamma, x0, y0):
        v = np.array([h0, uoo, r0, gamma, x0, y0], np.float64)
        check(lib().oc_set_vortex(self.h, _ptr(v)), self.h)

    # ---- static data (OceanDG.h:497-569) -----------------------------------------
    def static_data_size(self, which):
        return int(lib().oc_static_data_size(self.h, which))

    def quadrature_points(self, which):
        n = self.static_data_size(which)
        per = {0: 5, 1: 1, 2: 2, 3: 1, 4: 1}[which]
        xy = np.zeros((n // per, 2))
        check(lib().oc_quadrature_points(self.h, which, _ptr(xy)), self.h)
        return xy

    def initialize_data_at_quadrature(self, problem_data):
        """problem_data(x, y) -> array (5, npts): zb, friction coefficient, wind x, wind y, f."""
        arrays = []
        for which in range(5):
            xy = self.quadrature_points(which)
            d = np.asarray(problem_data(xy[:, 0], xy[:, 1]), np.float64).reshape(5, -1)
            if which == 0:
                arrays.append(np.ascontiguousarray(d.T).ravel())
            elif which == 2:
                arrays.append(np.ascontiguousarray(d[:2].T).ravel())
            else:
                arrays.append(np.ascontiguousarray(d[0]))
        self.set_static_data(*arrays)
        return arrays

    def set_static_data(self, cell0=None, cell1=None, cell2=None, face=None, bnd=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (cell0, cell1, cell2, face, bnd)]
        for k, a in enumerate(arrs):
            if a is not None and a.size != self.static_data_size(k):
                raise ValueError(f"static array {k}: {a.size} != {self.static_data_size(k)}")
        check(lib().oc_set_static_data(self.h, *[_ptr(a) for a in arrs]), self.h)

    # ---- the hot path ---------------------------------------------------------------
    def perform_stage_hydro(self, cur_stage, n_stages, cur_time, factor_residual, current_ri,
                            vec_ki_height, vec_ki_discharge, solution_height,
                            solution_discharge, next_ri_height, next_ri_discharge,
                            factor_tilde_residual=None, factor_matrix=0.0):
        """OceanDG.h:183-208.  current_ri = [height, discharge, (velocity)]."""
        ri_vel = current_ri[2] if len(current_ri) > 2 else None
        vecs = [current_ri[0], current_ri[1], solution_height, solution_discharge,
                next_ri_height, next_ri_discharge, *vec_ki_height, *vec_ki_discharge]
        mem = _memory(*vecs)
        fr = np.ascontiguousarray(factor_residual, np.float64)
        ft = None if factor_tilde_residual is None else np.ascontiguousarray(
            factor_tilde_residual, np.float64)
        kz = (C.c_void_p * len(vec_ki_height))(*[_ptr(k) for k in vec_ki_height])
        kq = (C.c_void_p * len(vec_ki_discharge))(*[_ptr(k) for k in vec_ki_discharge])
        sv = _lib.StageVectors(_ptr(current_ri[0]), _ptr(current_ri[1]), _ptr(ri_vel),
                               C.cast(kz, C.POINTER(C.c_void_p)), len(vec_ki_height),
                               C.cast(kq, C.POINTER(C.c_void_p)), len(vec_ki_discharge),
                               _ptr(solution_height), _ptr(solution_discharge),
                               _ptr(next_ri_height), _ptr(next_ri_discharge))
        check(lib().oc_perform_stage_hydro(self.h, cur_stage, n_stages, cur_time, _ptr(fr),
                                           _ptr(ft), factor_matrix, C.byref(sv), mem), self.h)

    def perform_time_step(self, scheme, time, dt, height, discharge):
        mem = _memory(height, discharge)
        check(lib().oc_perform_time_step(self.h, _lib.SCHEME[scheme], time, dt, _ptr(height),
                                         _ptr(discharge), mem), self.h)

    def compute_cell_transport_speed(self, height, discharge):
        out = C.c_double()
        check(lib().oc_transport_speed(self.h, _ptr(height), _ptr(discharge),
                                       _memory(height, discharge), C.byref(out)), self.h)
        return out.value

    def cell_transport_speed(self, height, discharge):
        """Per-cell maxima of compute_cell_transport_speed (NumPy in, NumPy out,
        or CUDA tensors in and a CUDA tensor out)."""
        mem = _memory(height, discharge)
        if mem == OC_MEM_DEVICE:
            import torch
            out = torch.empty(self.mesh.n_cells, dtype=torch.float64, device=height.device)
        else:
            out = np.zeros(self.mesh.n_cells)
        check(lib().oc_cell_transport_speed(self.h, _ptr(height), _ptr(discharge), mem,
                                            _ptr(out)), self.h)
        return out

    def set_cell_time_scale(self, scale=None):
        """Per-cell step-size scale of perform_time_step (None restores 1)."""
        s = None if scale is None else np.ascontiguousarray(scale, np.float64)
        if s is not None and s.size != self.mesh.n_cells:
            raise ValueError("one scale per cell")
        check(lib().oc_set_cell_time_scale(self.h, _ptr(s)), self.h)

    def apply(self, time, src_height, src_discharge, dst_height, dst_discharge):
        mem = _memory(src_height, src_discharge, dst_height, dst_discharge)
        check(lib().oc_apply(self.h, time, _ptr(src_height), _ptr(src_discharge),
                             _ptr(dst_height), _ptr(dst_discharge), mem), self.h)

    def evaluate_velocity_field(self, height, discharge, velocity):
        mem = _memory(height, discharge, velocity)
        check(lib().oc_velocity_field(self.h, _ptr(height), _ptr(discharge), _ptr(velocity),
                                      mem), self.h)

    def vorticity_indicator(self, velocity, n_q_1d, out):
        mem = OC_MEM_DEVICE if _is_device(velocity) else OC_MEM_HOST
        check(lib().oc_vorticity_indicator(self.h, _ptr(velocity), n_q_1d, _ptr(out), mem),
              self.h)

    def project_vortex(self, time, height, discharge):
        mem = _memory(height, discharge)
        check(lib().oc_project_vortex(self.h, time, _ptr(height), _ptr(discharge), mem), self.h)

    # ---- mixed form: reference state (no reference counterpart) ----------------------
    def set_reference_state(self, depth=1.0, discharge=(0.0, 0.0)):
        """Background (depth, discharge) the FP32 deviations are taken from."""
        check(lib().oc_set_reference_state(self.h, depth, discharge[0], discharge[1]), self.h)

    # ---- launch configuration (GB300-specific; no reference counterpart) -------------
    def set_launch_mode(self, mode: str):
        """"auto" (tuned at the first time step), "per_group" or "one" (hp meshes)."""
        check(lib().oc_set_launch_mode(self.h, _lib.LAUNCH_MODE[mode]), self.h)

    @property
    def launch_config(self) -> dict:
        out = np.zeros(7, np.int32)
        check(lib().oc_launch_config(self.h, _ptr(out)), self.h)
        return {"one_launch": bool(out[0]), "one_launch_warps": int(out[1]),
                "group_warps": {p: int(out[1 + p]) for p in range(1, 5)}, "tuned": bool(out[6])}

    def compute_errors_hydro(self, time, height, discharge):
        """OceanDG.h:2380-2459 against the vortex set by set_vortex: (depth, discharge)."""
        out = np.zeros(2)
        check(lib().oc_errors_vortex(self.h, time, _ptr(height), _ptr(discharge),
                                     _memory(height, discharge), _ptr(out)), self.h)
        return out

    def prepare_for_conservative_coarsening(self, mark, height):
        """OceanDG.h:2732-2778 on the cells with mark != 0 (height updated in place)."""
        mem = OC_MEM_DEVICE if _is_device(height) else OC_MEM_HOST
        if mem == OC_MEM_HOST:
            mark = np.ascontiguousarray(mark, np.uint8)
        check(lib().oc_conservative_coarsening(self.h, _ptr(mark), _ptr(height), mem), self.h)

    def set_timing(self, on=True):
        check(lib().oc_set_timing(self.h, 1 if on else 0), self.h)

    def timer_summary(self) -> dict:
        """{scope name: (calls, total seconds)} of the GPU work timed so far,
        named like the reference's TimerOutput scopes."""
        buf = C.create_string_buffer(4096)
        check(lib().oc_timer_summary(self.h, buf, len(buf)), self.h)
        out = {}
        for line in buf.value.decode().strip().split("\n"):
            name, calls, total, _ = line.split("\t")
            out[name] = (int(calls), float(total))
        return out

    def synchronize(self):
        check(lib().oc_synchronize(self.h), self.h)

    @property
    def stream(self) -> int:
        return int(lib().oc_stream(self.h) or 0)

    @property
    def launch_count(self) -> int:
        return int(lib().oc_launch_count(self.h))
