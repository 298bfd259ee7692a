"""Learned refinement indicator: host side of the GPU features and BF16 MLP.

The reference refines a cell when its vorticity indicator (hpTuner.h:247-305)
exceeds a fraction of the maximum (main.cc:749-765; the vortex case uses
Threshold_for_mesh_refinement = 1e-5).  Here a 12-64-64-1 BF16 MLP, trained on
the GPU, predicts those flags `horizon` steps ahead from per-cell features of
the current state, so that a refinement set built from the prediction stays
valid for longer (fewer remeshes).  Everything runs through the C ABI of
liboceano_gpu.so on CUDA tensors; PyTorch only holds the device buffers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib

N_FEATURES = 12
N_PARAMS = 64 * 12 + 64 + 64 * 64 + 64 + 64 + 1
REFINE_THRESHOLD = 1e-5  # tests/shallowWaterVortex/shallowWaterVortex.prm


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def cell_info(mesh, member=None) -> np.ndarray:
    """int32 [n_cells, 6]: face neighbours 0..3 (-1 on the boundary), level, member."""
    nc = mesh.n_cells
    info = np.full((nc, 6), -1, np.int32)
    ni = mesh.n_inner
    cm, cp = mesh.cell_m[:ni].astype(np.int64), mesh.cell_p.astype(np.int64)
    fm, fp = mesh.face_m[:ni].astype(np.int64), mesh.face_p.astype(np.int64)
    info[cm, fm] = cp
    info[cp, fp] = cm
    info[:, 4] = mesh.level if mesh.level is not None else 0
    info[:, 5] = 0 if member is None else member
    return info


def member_of_cells(meshes) -> np.ndarray:
    return np.concatenate([np.full(m.n_cells, k, np.int32) for k, m in enumerate(meshes)])


def features(op, zeta, q, info, n_members, threshold=REFINE_THRESHOLD, want_flags=True,
             want_vorticity=False):
    """(features [n,12], flags [n] or None, w/max [n] or None) as CUDA tensors."""
    import torch
    nc = op.mesh.n_cells
    dev = zeta.device
    feat = torch.empty((nc, N_FEATURES), dtype=torch.float32, device=dev)
    flags = torch.empty(nc, dtype=torch.float32, device=dev) if want_flags else None
    vort = torch.empty(nc, dtype=torch.float32, device=dev) if want_vorticity else None
    check(lib().oc_indicator_features(op.h, _p(zeta), _p(q), _p(info), n_members, threshold,
                                      _p(feat), _p(flags), _p(vort), _lib.OC_MEM_DEVICE), op.h)
    return feat, flags, vort


class LearnedIndicator:
    """The BF16 MLP of oc_mlp_* (one handle, its own CUDA stream)."""

    def __init__(self, seed=0):
        h = C.c_void_p()
        st = lib().oc_mlp_create(C.c_uint64(seed), C.byref(h))
        self.h = h
        if st != _lib.OC_OK:
            raise _lib.OceanoError(st, lib().oc_mlp_last_error(h).decode() if h else "")

    def close(self):
        if getattr(self, "h", None):
            lib().oc_mlp_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, st):
        if st != _lib.OC_OK:
            raise _lib.OceanoError(st, lib().oc_mlp_last_error(self.h).decode())

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(N_PARAMS, np.float32)
        self._check(lib().oc_mlp_get_params(self.h, out.ctypes.data_as(C.c_void_p)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(lib().oc_mlp_set_params(self.h, p.ctypes.data_as(C.c_void_p)))

    @property
    def normalization(self) -> np.ndarray:
        out = np.zeros(2 * N_FEATURES, np.float32)
        self._check(lib().oc_mlp_get_normalization(self.h, out.ctypes.data_as(C.c_void_p)))
        return out

    @normalization.setter
    def normalization(self, v):
        v = np.ascontiguousarray(v, np.float32)
        self._check(lib().oc_mlp_set_normalization(self.h, v.ctypes.data_as(C.c_void_p)))

    def fit_normalization(self, feat):
        self._sync_with(feat)
        self._check(lib().oc_mlp_fit_normalization(self.h, _p(feat), feat.shape[0]))

    def _sync_with(self, *tensors):
        import torch
        torch.cuda.synchronize()  # inputs were produced on other streams

    def forward(self, feat):
        import torch
        self._sync_with(feat)
        out = torch.empty(feat.shape[0], dtype=torch.float32, device=feat.device)
        self._check(lib().oc_mlp_forward(self.h, _p(feat), feat.shape[0], _p(out)))
        self._check(lib().oc_mlp_synchronize(self.h))
        return out

    def gradient(self, feat, labels, pos_weight=1.0, want_grad=True):
        self._sync_with(feat, labels)
        g = np.zeros(N_PARAMS, np.float32) if want_grad else None
        loss = C.c_double()
        self._check(lib().oc_mlp_gradient(self.h, _p(feat), _p(labels), feat.shape[0],
                                          C.c_float(pos_weight),
                                          g.ctypes.data_as(C.c_void_p) if want_grad else None,
                                          C.byref(loss)))
        return loss.value, g

    def adam_step(self, lr):
        self._check(lib().oc_mlp_adam_step(self.h, C.c_float(lr)))

    def train(self, feat, labels, epochs=200, lr=3e-3, pos_weight=1.0):
        """Full-batch Adam on (feat, labels); returns the loss per epoch."""
        losses = []
        for _ in range(epochs):
            loss, _ = self.gradient(feat, labels, pos_weight, want_grad=False)
            self.adam_step(lr)
            losses.append(loss)
        self._check(lib().oc_mlp_synchronize(self.h))
        return losses

    def predict(self, feat, threshold=0.5):
        import torch
        return torch.sigmoid(self.forward(feat)) > threshold


def dilate(flags, info, layers=1) -> np.ndarray:
    """The flagged cells grown by `layers` layers of face neighbours (cell_info
    columns 0..3; on a coarse face with two fine neighbours the one recorded):
    the refinement buffer of a run without a network (hpTuner.h:247-305 flags,
    grown so that the refined set stays valid for longer)."""
    out = np.asarray(flags, bool).copy()
    nb = np.asarray(info)[:, :4]
    for _ in range(layers):
        grown = out.copy()
        for f in range(4):
            has = nb[:, f] >= 0
            grown[nb[has, f]] |= out[has]
            grown[has] |= out[nb[has, f]]
        out = grown
    return out


def remesh_count(flag_seq, predicted=None, members=None, n_members=1) -> int:
    """Remeshes of a run that refines where flagged.  The refined set starts as
    the flags at t = 0; afterwards a member remeshes when one of its currently
    flagged cells lies outside its refined set, and its new set is the current
    flags (vorticity indicator) or the current flags together with the predicted
    flags (learned indicator).  flag_seq[t], predicted[t]: per-cell booleans."""
    f0 = np.asarray(flag_seq[0], bool)
    members = np.zeros(f0.size, np.int64) if members is None else np.asarray(members)
    refined = None
    count = 0
    for t, f in enumerate(flag_seq):
        f = np.asarray(f, bool)
        new = f if predicted is None else (f | np.asarray(predicted[t], bool))
        if refined is None:
            refined = new.copy()
            continue
        need = np.zeros(n_members, bool)
        np.logical_or.at(need, members[f & ~refined], True)
        if need.any():
            count += int(need.sum())
            sel = need[members]
            refined[sel] = new[sel]
    return count


def run_and_record(op, zeta, q, info, n_members, dt, steps, every=1, scheme="ssp33",
                   threshold=REFINE_THRESHOLD):
    """Advance (zeta, q) (CUDA tensors, in place) by `steps` time steps and
    record (features, flags) every `every` steps, starting at step 0."""
    import torch
    stream = torch.cuda.ExternalStream(op.stream)
    out = []
    with torch.cuda.stream(stream):
        for it in range(steps + 1):
            if it % every == 0:
                f, fl, _ = features(op, zeta, q, info, n_members, threshold)
                out.append((f, fl))
            if it < steps:
                op.perform_time_step(scheme, it * dt, dt, zeta, q)
    torch.cuda.synchronize()
    return out


def training_pairs(records, horizon):
    """(features at t, flags at t + horizon) over the records (horizon counts records)."""
    import torch
    X = torch.cat([records[k][0] for k in range(len(records) - horizon)])
    Y = torch.cat([records[k + horizon][1] for k in range(len(records) - horizon)])
    return X, Y


def evaluate(model, records, horizon, members, n_members, threshold=0.5, info=None,
             dilate_layers=(1, 2)):
    """Precision / recall of the predicted flags `horizon` records ahead, the
    remesh counts of the vorticity indicator and of the learned indicator, and
    the mean size of the learned refinement set (flags or predicted) over the
    flagged set; with `info` (cell_info) also the remesh counts and set sizes of
    the network-free buffer (flags dilated by k cell layers)."""
    import torch
    tp = fp = fn = 0
    preds, flags, ratio = [], [], []
    for k, (f, fl) in enumerate(records):
        p = model.predict(f, threshold)
        preds.append(p.cpu().numpy())
        flags.append(fl.cpu().numpy() > 0.5)
        ratio.append((preds[-1] | flags[-1]).sum() / max(flags[-1].sum(), 1))
        if k + horizon < len(records):
            y = records[k + horizon][1] > 0.5
            tp += int((p & y).sum())
            fp += int((p & ~y).sum())
            fn += int((~p & y).sum())
    base = remesh_count(flags, None, members, n_members)
    learned = remesh_count(flags, preds, members, n_members)
    out = {"precision": tp / max(tp + fp, 1), "recall": tp / max(tp + fn, 1),
           "remesh_vorticity": base, "remesh_learned": learned,
           "refined_over_flagged": float(np.mean(ratio))}
    if info is not None:  # the network-free buffer: flags grown by k cell layers
        for k in dilate_layers:
            grown = [dilate(f, info, k) for f in flags]
            out[f"remesh_dilated_{k}"] = remesh_count(flags, grown, members, n_members)
            out[f"dilated_{k}_over_flagged"] = float(np.mean(
                [g.sum() / max(f.sum(), 1) for g, f in zip(grown, flags)]))
    return out
