"""Checkpoint and resume of a run of the stage operator.

One ``.npz`` file holds the mesh in the operator's boundary format (degrees,
vertices, face lists, levels), the state vectors (height, discharge) in the
DoFHandler layout, the time and the step number, and any extra arrays the
caller adds (for example the dt schedule or an ensemble's member table).  A
run resumed from a checkpoint on a new handle continues bit for bit: the
operator keeps no state between time steps besides the solution.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import Mesh

FORMAT = "oceano_gb300/checkpoint/1"
_MESH_FIELDS = ("degree", "vertices", "cell_m", "cell_p", "face_m", "face_p", "subface",
                "orient", "bid", "level")


@dataclass
class Checkpoint:
    mesh: Mesh
    height: np.ndarray
    discharge: np.ndarray
    time: float
    step: int
    extra: dict = field(default_factory=dict)


def _host(a):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(a)


def save(path, mesh: Mesh, height, discharge, time: float, step: int, **extra) -> None:
    h, q = _host(height).astype(np.float64), _host(discharge).astype(np.float64)
    if h.size != mesh.n_dofs() or q.size != 2 * mesh.n_dofs():
        raise ValueError("state size does not match the mesh")
    arrays = {f"mesh_{k}": getattr(mesh, k) for k in _MESH_FIELDS if getattr(mesh, k) is not None}
    arrays["mesh_domain"] = np.asarray(mesh.domain, np.float64)
    for k, v in extra.items():
        arrays[f"extra_{k}"] = _host(v)
    np.savez(path, format=np.array(FORMAT), height=h, discharge=q, time=np.float64(time),
             step=np.int64(step), **arrays)


def load(path) -> Checkpoint:
    with np.load(path, allow_pickle=False) as d:
        if "format" not in d.files or str(d["format"]) != FORMAT:
            raise ValueError(f"{path}: not a {FORMAT} file")
        kw = {k: d[f"mesh_{k}"] for k in _MESH_FIELDS if f"mesh_{k}" in d.files}
        mesh = Mesh(domain=tuple(d["mesh_domain"]), **kw)
        extra = {k[6:]: d[k] for k in d.files if k.startswith("extra_")}
        ck = Checkpoint(mesh, d["height"].copy(), d["discharge"].copy(), float(d["time"]),
                        int(d["step"]), extra)
    if ck.height.size != mesh.n_dofs() or ck.discharge.size != 2 * mesh.n_dofs():
        raise ValueError(f"{path}: state size does not match the mesh")
    return ck
