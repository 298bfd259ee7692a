"""Benchmark: DoF-stage updates/s of the per-stage DG operator on GB300.

Workload (one "step" = one SSP-RK3 time step = 3 stages of the operator):
the degree-3 travelling vortex on [0,2]x[0,1], a 20x10 coarse grid refined
4 times (320x160 = 51,200 cells, 2,457,600 scalar DoFs), periodic in x, walls
in y, flat bathymetry (zb = 0, zeta = depth), no friction, g = 9.81, CFL 0.05.
Synthetic, seeded-free deterministic input (the vortex projected on the mesh).

value    : mixed form (FP32 bulk, FP64 accumulation), inputs resident in HBM,
           timed with CUDA events on the operator's stream, L2 flushed between
           steps (the state vectors fit the 129 MB L2).
fp64     : the plain FP64 form on the same GPU.
e2e      : mixed form through the public C ABI with pinned host buffers, copies
           in and out inside the timed region.
e2e_stage_abi: the literal drop-in call, three oc_perform_stage_hydro calls
           per step on host vectors with host-side registers (every stage
           copies its inputs in and its outputs out), mixed form.
roofline : dominant kernel = the fused stage kernel; algorithmic bytes per step
           = per scalar DoF and stage the stage input, u^n and the stage output
           at their stored precision, plus 5 doubles of geometry per cell;
           peak from MEASURED_PEAKS.json.  `traffic` (DRAM bytes per launch)
           comes from an ncu capture of the same kernel (`traffic_source`
           names it); a bench run does not run under ncu.
cpu_baseline / --impl reference: the FP64 C oracle (CPU restatement; the
           reference itself needs deal.II + MPI) with OpenMP on all host cores.
secondary_quadrature: the same vortex under the config's secondary cell rule
           (4x4 Gauss points per cell at p = 3), mixed and FP64 timed, error.

Secondary workloads (--workload; same JSON keys, not the headline line):
  hp        the vortex on the seeded random hp mesh (about 60k cells, degrees
            1-4, hanging faces), SSP-RK3, launch shape autotuned;
  channel   250x10 cells, p = 2, bump bathymetry, implicit Manning friction
            (ARK Giraldo / TR-BDF2);
  ensemble  64 vortices with seeded centres, radii and strengths on refined-disk
            meshes of 5k-40k cells each (p = 1, 2), one operator over their union;
  indicator the learned refinement indicator trained and evaluated on ensembles
            (--steps = training epochs).
--partition: the degree-3 vortex mesh cut over the N GPUs (owned cells plus a
            ghost halo whose face traces travel over NCCL before every stage),
            strong scaling, beside the default replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Courant numbers: the reference's degree-3 case runs CFL 0.075 (channelFlow.prm), but
# the degree-3 vortex diverges after about 450 SSP-RK3 steps there (in the oracle as well);
# 0.05 runs the 1000 steps of the vortex workload.  The channel (p = 2) and the
# ensemble (p <= 2) keep 0.075; the hp mesh (degrees up to 4) uses 0.05.
DEGREE, REFINE = 3, 4
CFL_VORTEX, CFL, CFL_HP = 0.05, 0.075, 0.05
METRIC = "DG DoF-stage updates/s, mixed vs FP64 on same GPU at stated L2 error; % HBM roofline"


def workload():
    from oceano_gb300 import vortex_mesh
    from oceano_gb300.icbc import vortex_params
    mesh = vortex_mesh(REFINE, DEGREE)
    return mesh, vortex_params()


class Workload:
    """Operators (mixed, FP64), initial state, dt and scheme of one workload,
    and a factory of the matching FP64 oracle for the CPU baseline."""

    def __init__(self, name, gpu=True):
        """gpu=False builds the mesh, initial state and dt on the host only (the
        reference arm: no GPU operator, the state projected by the oracle)."""
        from oceano_gb300 import workloads as W
        self.name = name
        self.scheme = "ssp33"
        self.op_m = self.op_d = None
        z0 = q0 = None
        if name == "vortex":
            mesh, vx = workload()
            if gpu:
                self.op_m, self.op_d = make_op(mesh, vx, "mixed"), make_op(mesh, vx, "fp64")
                n = self.op_d.n_dofs
                z0, q0 = np.zeros(n), np.zeros(2 * n)
                self.op_d.project_vortex(0.0, z0, q0)
            self.desc = "vortex p=3, 320x160 cells (51200), 2457600 DoFs, SSP-RK3 step"
            self.oracle_kw = dict(bcs={0: ("wall",)}, vortex=list(vx) + [0, 0])
        elif name == "hp":
            if gpu:
                self.op_m, z0, q0 = W.hp_vortex("mixed")
                self.op_d, _, _ = W.hp_vortex("fp64")
                mesh = self.op_d.mesh
            else:
                from oceano_gb300 import random_hp_mesh
                mesh = random_hp_mesh(seed=20261203, target=60000)
            self.desc = (f"vortex on the seeded random hp mesh ({mesh.n_cells} cells, "
                         f"p=1..4, hanging faces), SSP-RK3 step")
            self.oracle_kw = dict(bcs={0: ("wall",)}, vortex=list(W.vortex_params()) + [0, 0])
        elif name == "channel":
            if gpu:
                self.op_m, z0, q0 = W.channel("mixed")
                self.op_d, _, _ = W.channel("fp64")
                mesh = self.op_d.mesh
            else:
                from oceano_gb300.mesh import channel_mesh
                mesh = channel_mesh(2, 250, 10)
                z0, q0 = W.uniform_state(mesh, 0.0, (W.CHANNEL_Q_IN, 0.0))
            self.scheme = "ark_stage3_order2"
            self.desc = ("channel 250x10 cells p=2, bump, implicit Manning n=0.03, "
                         "ARK stage_3_order_2 step")
            self.oracle_kw = dict(friction=2, bcs=W.CHANNEL_BCS)
        elif name == "ensemble":
            if gpu:
                self.op_m, z0, q0, members, meshes = W.ensemble(64, "mixed")
                self.op_d = W.vortex_operator(self.op_m.mesh, "fp64", members[0]["vortex"])
                mesh = self.op_d.mesh
            else:
                from oceano_gb300.mesh import concatenate_meshes
                members = W.ensemble_members(64, 1000)
                meshes = [W.member_mesh(m) for m in members]
                mesh = concatenate_meshes(meshes)
                zs, qs = zip(*[W.vortex_nodal_state(m, mm["vortex"]) for m, mm in zip(meshes, members)])
                z0, q0 = np.concatenate(zs), np.concatenate(qs)
            self.desc = (f"64-member vortex ensemble, {mesh.n_cells} cells "
                         f"(5k-40k per member, p=1,2), one operator, own dt per member, "
                         f"SSP-RK3 step")
            self.oracle_kw = dict(bcs={0: ("wall",)})
        else:
            raise ValueError(name)
        self.mesh = mesh
        self.member_dt = None
        if name == "ensemble" and gpu:  # every member keeps its own dt (per-cell scales)
            from oceano_gb300.indicator import member_of_cells
            dt_ref, scale = W.member_time_steps(self.op_d, z0, q0, member_of_cells(meshes), CFL)
            for op in (self.op_m, self.op_d):
                op.set_cell_time_scale(scale)
            self.member_dt = (dt_ref, float(scale.min()), float(scale.max()))
        # degree-4 cells at the finest level of the hp mesh need a smaller Courant
        # number (CFL 0.075 diverges there within 20 steps, in the oracle as well)
        self.cfl = {"vortex": CFL_VORTEX, "hp": CFL_HP}.get(name, CFL)
        if gpu:
            self.n = self.op_d.n_dofs
            self.z0, self.q0 = z0, q0
            self.dt = self.cfl / self.op_d.compute_cell_transport_speed(self.z0, self.q0)
            if self.member_dt is not None:
                self.dt = self.member_dt[0]
        else:
            orc = self.oracle()
            if z0 is None:
                z0, q0 = orc.project_vortex(0.0)
            self.n = orc.n
            self.z0, self.q0 = z0, q0
            self.dt = self.cfl / orc.transport_speed(self.z0, self.q0)

    def oracle(self):
        from oracle import oracle as O
        orc = O.Oracle(self.mesh, **self.oracle_kw)
        if self.name == "channel":
            from oceano_gb300.icbc import channel_problem_data
            from oceano_gb300 import workloads as W
            arrs = []
            for which in range(5):
                xy = orc.points(which)
                d = np.asarray(channel_problem_data(W.CHANNEL_MANNING)(xy[:, 0], xy[:, 1]))
                arrs.append(np.ascontiguousarray(d.T).ravel() if which == 0 else
                            np.ascontiguousarray(d[:2].T).ravel() if which == 2 else
                            np.ascontiguousarray(d[0]))
            orc.set_static(*arrs)
        return orc

    def oracle_step(self, orc, t, z, q):
        from oracle import oracle as O
        if self.scheme == "ssp33":
            tb = O.TABLEAUX["ssp33"]
            O.erk_step(orc, tb["a"], tb["b"], tb["c"], t, self.dt, z, q)
        else:
            g, tr = O.TABLEAUX["giraldo32"], O.TABLEAUX["trbdf2"]
            O.ark_step(orc, g["a"], g["b"], g["c"], tr["a"], tr["d"], t, self.dt, z, q)


def make_op(mesh, vx, precision):
    from oceano_gb300.workloads import vortex_operator
    return vortex_operator(mesh, precision, vx)


def algorithmic_bytes(n_dofs_var, n_cells, mixed, static_bytes=0):
    """Bytes one 3-stage step must move: per stage the stage input r_i, u^n and
    the stage output at their stored precision (stage 0: r_0 = u^n, counted
    once), the affine geometry (J^-1 and det, 5 doubles per cell) and the static
    data a stage reads (bathymetry, friction coefficient; FP32 in the mixed form)."""
    n = 3 * n_dofs_var  # scalar DoFs of zeta, hu, hv
    if mixed:
        per_dof = (8 + 4) + (4 + 8 + 4) + (4 + 8 + 8)
    else:
        per_dof = (8 + 8) + (8 + 8 + 8) + (8 + 8 + 8)
    return n * per_dof + 3 * n_cells * 5 * 8 + 3 * static_bytes


TRAFFIC_PROFILE = os.path.join("profiles", "stage_kernel_p3_mixed_vortex320x160_traffic.md")


def profiled_traffic():
    """DRAM bytes per stage launch and warp instructions per launch from the ncu
    summary of the stage kernel (profiles/), or None: these counters exist only
    under ncu, which never runs inside a timed bench."""
    p = os.path.join(ROOT, TRAFFIC_PROFILE)
    out = {}
    if os.path.exists(p):
        for line in open(p):
            for key in ("traffic_bytes_per_launch", "warp_instructions_per_launch"):
                if line.startswith(key + ":"):
                    out[key] = float(line.split(":")[1])
    return out


def bf16_peak():
    """Dense BF16 TFLOP/s (burst) of MEASURED_PEAKS.json, else the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"])
    return 1900.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100", "-i",
                 os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def time_device(op, mesh, z0, q0, steps, warmup, dt, flush, scheme="ssp33"):
    """Per-step CUDA-event times (ms) of oc_perform_time_step on device vectors."""
    import torch
    stream = torch.cuda.ExternalStream(op.stream)
    z = torch.from_numpy(z0).cuda()
    q = torch.from_numpy(q0).cuda()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(warmup):
            op.perform_time_step(scheme, i * dt, dt, z, q)
        op.synchronize()
        times = []
        launches0 = op.launch_count
        for i in range(steps):
            flush.zero_()  # evict the state from L2 (outside the timed events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            op.perform_time_step(scheme, (warmup + i) * dt, dt, z, q)
            e1.record(stream)
            times.append((e0, e1))
        op.synchronize()
        launches = op.launch_count - launches0
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in times]
    return ms, z.cpu().numpy(), q.cpu().numpy(), launches


def secondary_quadrature(args, flush):
    """The same vortex under the config's secondary cell rule: 4x4 Gauss points
    per cell at p = 3 (n_points_1d = p + 1; the mass rules are fixed in the
    reference).  Mixed and FP64 steps timed like the main legs (fewer steps), the
    mixed state's error against the FP64 one under the same rule."""
    mesh, vx = workload()
    from oceano_gb300.workloads import vortex_operator
    op_m = vortex_operator(mesh, "mixed", vx, cell_quadrature="p+1")
    op_d = vortex_operator(mesh, "fp64", vx, cell_quadrature="p+1")
    n = op_d.n_dofs
    z0, q0 = np.zeros(n), np.zeros(2 * n)
    op_d.project_vortex(0.0, z0, q0)
    dt = CFL_VORTEX / op_d.compute_cell_transport_speed(z0, q0)
    steps = max(5, args.steps // 4)
    ms_m, zm, qm, _ = time_device(op_m, mesh, z0, q0, steps, args.warmup, dt, flush)
    ms_d, zd, qd, _ = time_device(op_d, mesh, z0, q0, steps, args.warmup, dt, flush)
    units = 3 * n * 3 * steps
    out = {"rule": "cell and boundary faces: Gauss p+1 = 4 points per direction at p = 3 "
                   "(n_points_1d); mass: Gauss-Lobatto 5 (zeta), Gauss 4 (discharge)",
           "steps": steps,
           "mixed": {"value": units / (sum(ms_m) / 1e3), "ms_per_step": sum(ms_m) / steps},
           "fp64": {"value": units / (sum(ms_d) / 1e3), "ms_per_step": sum(ms_d) / steps},
           "l2_error_vs_fp64": {"zeta": rel(zm, zd), "hu_hv": rel(qm, qd),
                                "after_steps": args.warmup + steps}}
    out["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    op_m.close()
    op_d.close()
    return out


def time_e2e(op, z0, q0, steps, warmup, dt, scheme="ssp33"):
    """Same steps through the C ABI with pinned host buffers (copies timed)."""
    import torch
    zh = torch.from_numpy(z0.copy()).pin_memory()
    qh = torch.from_numpy(q0.copy()).pin_memory()
    stream = torch.cuda.ExternalStream(op.stream)
    for i in range(warmup):
        _host_step(op, i * dt, dt, zh, qh, scheme)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        _host_step(op, (warmup + i) * dt, dt, zh, qh, scheme)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps, (zh.numel() + qh.numel()) * 8


def _host_step(op, t, dt, zh, qh, scheme="ssp33"):
    """oc_perform_time_step with OC_MEM_HOST on pinned tensors (host pointers)."""
    import ctypes as C
    from oceano_gb300 import _lib
    _lib.check(_lib.lib().oc_perform_time_step(op.h, _lib.SCHEME[scheme], t, dt,
                                               C.c_void_p(zh.data_ptr()),
                                               C.c_void_p(qh.data_ptr()), _lib.OC_MEM_HOST),
               op.h)


def time_e2e_stage_abi(op, z0, q0, steps, warmup, dt):
    """The drop-in call of the reference's integrator loop: per step three
    oc_perform_stage_hydro calls (SSP-RK3, ExplicitRungeKuttaIntegrator.h:179-298)
    on pinned host vectors with host-side registers, so that every stage copies
    its inputs in and its outputs out.  Returns ms per step and the bytes moved
    each way per step."""
    import torch
    a = [[1.0], [0.25, 0.25]]  # SSP-RK3 Butcher rows (time_stepping.h:170-192)
    b = [1 / 6, 1 / 6, 2 / 3]
    c = [0.0, 1.0, 0.5]
    n = z0.size

    def pinned(x):  # NumPy view of page-locked host memory
        return torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()

    z, q = pinned(z0.copy()), pinned(q0.copy())
    kz = [pinned(np.zeros(n)) for _ in range(4)]
    kq = [pinned(np.zeros(2 * n)) for _ in range(4)]
    nz, nq = pinned(np.zeros(n)), pinned(np.zeros(2 * n))
    rz, rq = pinned(np.zeros(n)), pinned(np.zeros(2 * n))

    def step(t):
        for st in range(3):
            f = np.array(b if st == 2 else a[st], np.float64) * dt
            if st == 0:
                rz[:] = z; rq[:] = q
            else:
                rz[:] = nz; rq[:] = nq
            op.perform_stage_hydro(st, 3, t + c[st] * dt, f, [rz, rq], kz, kq, z, q, nz, nq)

    for i in range(warmup):
        step(i * dt)
    t0 = time.perf_counter()
    for i in range(steps):
        step((warmup + i) * dt)
    el = time.perf_counter() - t0
    nb = 8 * n
    # per stage s: in r, u^n (3 vectors' worth each) and k_1..k_s; out k_{s+1} and next/solution
    h2d = sum(3 * nb * (2 + s) for s in range(3))
    d2h = 3 * 3 * nb * 2
    return 1e3 * el / steps, h2d, d2h


def cpu_baseline(wl, steps):
    """FP64 C oracle (OpenMP, all host cores) on `steps` full RK steps."""
    from oracle import oracle as O
    orc = wl.oracle()
    z, q = wl.z0.copy(), wl.q0.copy()
    t0 = time.perf_counter()
    for i in range(steps):
        wl.oracle_step(orc, i * wl.dt, z, q)
    el = time.perf_counter() - t0
    ndof = 3 * orc.n
    return ndof * 3 * steps / el, O.num_threads(), el


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dist_setup(n_gpus):
    import torch
    if n_gpus > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        local = int(os.environ.get("LOCAL_RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", 1))
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return rank, world
    return 0, 1


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, rank, world):
    """CPU restatement timed on the host cores (rank 0 only)."""
    if rank != 0:
        return
    wl = Workload(args.workload, gpu=False)
    orc = wl.oracle()
    z, q = wl.z0.copy(), wl.q0.copy()
    for i in range(args.warmup):
        wl.oracle_step(orc, i * wl.dt, z, q)
    t0 = time.perf_counter()
    for i in range(args.steps):
        wl.oracle_step(orc, (args.warmup + i) * wl.dt, z, q)
    el = time.perf_counter() - t0
    from oracle import oracle as O
    ndof = 3 * orc.n
    v = ndof * 3 * args.steps / el
    cores = O.num_threads()
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "DoF-stage/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.desc, "cells": wl.mesh.n_cells, "dofs": ndof},
        "cpu_baseline": {"value": v, "unit": "DoF-stage/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full time steps of the workload"},
        "e2e": {"value": v, "unit": "DoF-stage/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "FP64 C restatement of the reference operator (OpenMP); the reference "
                "build needs deal.II 9.5 + p4est + MPI, absent on this image"}))


def run_partition(args, rank, world):
    """One mesh (the degree-3 vortex) cut into `world` parts, one part per GPU:
    owned cells plus a one-layer ghost halo, face traces exchanged over NCCL
    before every stage, dt from the owned cells' speeds and one allreduce MAX,
    the mixed form through oc_perform_stage_hydro on device vectors.  Strong
    scaling: value = DoF-stage updates of the whole mesh per second."""
    import torch
    import __graft_entry__ as ge
    ge.build()
    from oceano_gb300.partition import (HaloExchange, halo_bytes, partition,
                                        partitioned_erk_step, partitioned_time_step_size,
                                        torch_max, with_ghost_boundary)
    from oceano_gb300.workloads import apply_bcs, vortex_operator
    from oceano_gb300.operator import OceanoOperator
    mesh, vx = workload()
    parts = partition(mesh, world)
    part = parts[rank]
    op = OceanoOperator(part.mesh, precision="mixed", zeta_reference=vx[0])
    op.set_reference_state(vx[0], (vx[0] * vx[1], 0.0))
    apply_bcs(op, with_ghost_boundary({0: ("wall",)}))
    op.set_vortex(*vx)
    full = vortex_operator(mesh, "fp64", vx) if rank == 0 else None
    n = int(mesh.offsets()[-1])
    z0, q0 = np.zeros(n), np.zeros(2 * n)
    if full is not None:
        full.project_vortex(0.0, z0, q0)
        full.close()
    zt, qt = torch.from_numpy(z0).cuda(), torch.from_numpy(q0).cuda()
    if world > 1:
        import torch.distributed as dist
        dist.broadcast(zt, 0)
        dist.broadcast(qt, 0)
    z = zt[torch.from_numpy(part.dof_index(mesh, "zeta")).cuda()].contiguous()
    q = qt[torch.from_numpy(part.dof_index(mesh, "q")).cuda()].contiguous()
    halo = HaloExchange(parts, rank, device="cuda")
    reduce = torch_max if world > 1 else None
    dt = partitioned_time_step_size(op, part, z, q, CFL_VORTEX, reduce)
    tb = {"a": [[1.0], [0.25, 0.25]], "b": [1 / 6, 1 / 6, 2 / 3], "c": [0.0, 1.0, 0.5]}

    def stage(st, s, t, f, rz, rq, kz, kq, sz, sq, nz, nq):
        torch.cuda.synchronize()  # the halo buffers were written on torch's stream
        op.perform_stage_hydro(st, s, t, f, [rz, rq], kz, kq, sz, sq, nz, nq)
        op.synchronize()

    for i in range(args.warmup):
        partitioned_erk_step(stage, halo, tb, i * dt, dt, z, q)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        partitioned_erk_step(stage, halo, tb, (args.warmup + i) * dt, dt, z, q)
    torch.cuda.synchronize()
    el = max_over_ranks(time.perf_counter() - t0, world)
    ndof = 3 * n
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": ndof * 3 * args.steps / el, "unit": "DoF-stage/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "vortex p=3, 320x160 cells (51200), one mesh cut into "
                                   f"{world} parts, face-trace halo, SSP-RK3 step",
                       "cells": mesh.n_cells, "dofs": ndof, "parts": world,
                       "halo_bytes_per_exchange": halo_bytes(parts),
                       "path": "oc_perform_stage_hydro on device vectors, mixed form"}}))


INDICATOR_EPOCHS = 300  # full-batch Adam epochs of the indicator training (fixed: not --steps)


def run_indicator(args):
    """Learned refinement indicator on the vortex ensemble: train the BF16 MLP on
    20 members (seeds 100..119) to predict the vorticity flags 10 steps ahead,
    evaluate it on the 64 members (seeds 1000..1063), time its kernels."""
    import torch
    import __graft_entry__ as ge
    ge.build()
    from oceano_gb300 import workloads as W
    from oceano_gb300.indicator import (LearnedIndicator, cell_info, evaluate, member_of_cells,
                                        run_and_record, training_pairs)

    def setup(n, seed0):
        op, z, q, mem, meshes = W.ensemble(n, "mixed", seed0)
        info = torch.from_numpy(cell_info(op.mesh, member_of_cells(meshes))).cuda()
        zt, qt = torch.from_numpy(z).cuda(), torch.from_numpy(q).cuda()
        dt = CFL / op.compute_cell_transport_speed(zt, qt)
        return op, zt, qt, info, dt, member_of_cells(meshes)

    horizon, every = 10, 2
    op, z, q, info, dt, _ = setup(20, 100)
    recs = run_and_record(op, z, q, info, 20, dt, 100, every=every)
    X, Y = training_pairs(recs, horizon // every)
    del recs
    model = LearnedIndicator(seed=1)
    model.fit_normalization(X)
    pos = float((Y.numel() - Y.sum()) / max(float(Y.sum()), 1.0))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = model.train(X, Y, epochs=INDICATOR_EPOCHS, lr=3e-3, pos_weight=pos)
    t_train = time.perf_counter() - t0
    ev_op, z2, q2, info2, dt2, members = setup(64, 1000)
    recs2 = run_and_record(ev_op, z2, q2, info2, 64, dt2, 60, every=1)
    res = evaluate(model, recs2, horizon, members, 64, info=info2.cpu().numpy())
    f = recs2[0][0]
    for _ in range(3):
        model.forward(f)
    torch.cuda.synchronize()
    # forward kernel alone: CUDA events on the model's stream around `reps` launches
    import ctypes as C
    from oceano_gb300._lib import lib as oclib
    stream = torch.cuda.ExternalStream(int(oclib().oc_mlp_stream(model.h) or 0))
    out = torch.empty(f.shape[0], dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    e0.record(stream)
    for _ in range(reps):
        oclib().oc_mlp_forward(model.h, C.c_void_p(f.data_ptr()), f.shape[0],
                               C.c_void_p(out.data_ptr()))
    e1.record(stream)
    e1.synchronize()
    t_fwd = e0.elapsed_time(e1) / 1e3 / reps
    flops_fwd = 2 * (12 * 64 + 64 * 64 + 64)
    # gradient kernels alone (forward, back-propagation W2^T d2 and the parameter
    # sums d2^T h1, d1^T xh on the tensor cores, then the fixed-order block
    # reduction) on the first 2^20 training samples; no host copy in the loop
    ng = min(int(X.shape[0]), 1 << 20)
    Xg, Yg = X[:ng].contiguous(), Y[:ng].contiguous()
    for _ in range(3):
        oclib().oc_mlp_gradient(model.h, C.c_void_p(Xg.data_ptr()), C.c_void_p(Yg.data_ptr()),
                                ng, C.c_float(pos), None, None)
    e0.record(stream)
    for _ in range(reps):
        oclib().oc_mlp_gradient(model.h, C.c_void_p(Xg.data_ptr()), C.c_void_p(Yg.data_ptr()),
                                ng, C.c_float(pos), None, None)
    e1.record(stream)
    e1.synchronize()
    t_grad = e0.elapsed_time(e1) / 1e3 / reps
    flops_grad = flops_fwd + 2 * (64 * 64 + 64 * 64 + 64 * 12)  # + W2^T d2, d2^T h1, d1^T xh
    # remeshing runs: 16 independent members (own mesh, operator and time step),
    # p-adaptive degree map (1 outside / 2 inside the refined set) with state
    # transfer, 40 steps, under the three policies
    from oceano_gb300.adapt import remesh_experiment
    rm_members = W.ensemble_members(16, 1000)
    remesh = {"members": 16, "steps": 40, "degrees": "1 outside, 2 inside the refined set"}
    for name, kw in (("vorticity", {}), ("dilated_1", {"layers": 1}),
                     ("learned", {"model": model})):
        policy = name.split("_")[0]
        remesh[name] = remesh_experiment(rm_members, policy, 40, **kw)
    out = {
        "metric": "learned refinement indicator: BF16 MLP forward cells/s",
        "value": f.shape[0] / t_fwd, "unit": "cells/s", "n_gpus": 1, "steps": args.steps,
        "warmup": 3, "higher_is_better": True, "dtype": "bf16 (fp32 accumulate)",
        "data": "synthetic",
        "config": {"workload": "vortex ensemble: train 20 members (seeds 100..119), evaluate "
                               "64 members (seeds 1000..1063); flags 10 steps ahead",
                   "train_samples": int(X.shape[0]), "eval_cells": int(f.shape[0]),
                   "epochs": INDICATOR_EPOCHS},
        "forward_tflops": f.shape[0] * flops_fwd / t_fwd / 1e12,
        "forward_roofline": {"bound": "tensor", "achieved": f.shape[0] * flops_fwd / t_fwd / 1e12,
                             "peak": bf16_peak(), "unit": "TFLOP/s",
                             "frac": f.shape[0] * flops_fwd / t_fwd / 1e12 / bf16_peak(),
                             "kernel": "mlp_forward_mma_kernel (mma.sync m16n8k16 bf16)",
                             "flop_per_cell": flops_fwd},
        "train_samples_per_s": X.shape[0] * INDICATOR_EPOCHS / t_train,
        "gradient_kernel": {"samples_per_s": ng / t_grad, "tflops": ng * flops_grad / t_grad / 1e12,
                            "frac_of_bf16_peak": ng * flops_grad / t_grad / 1e12 / bf16_peak(),
                            "flop_per_sample": flops_grad, "samples": ng,
                            "kernel": "mlp_grad_mma_kernel (mma.sync m16n8k16 bf16; "
                                      "back-propagated signals as two BF16 terms)"},
        "loss_first_last": [losses[0], losses[-1]],
        "eval": res,
        "remesh_runs": remesh,
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="vortex",
                    choices=["vortex", "hp", "channel", "ensemble", "indicator"])
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--partition", action="store_true",
                    help="one mesh cut over the GPUs (strong scaling) instead of replicas")
    ap.add_argument("--legs", default="mixed,fp64,e2e",
                    help="timed legs (a subset of mixed,fp64,e2e; profiling runs use 'mixed')")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "indicator":
        run_indicator(args)
        return
    if args.partition:
        run_partition(args, rank, world)
        return
    import torch
    import __graft_entry__ as ge
    ge.build()
    wl = Workload(args.workload)
    mesh, n, dt, z0, q0 = wl.mesh, wl.n, wl.dt, wl.z0, wl.q0
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    barrier(world)
    legs = set(args.legs.split(","))
    with Clocks() as clk:  # samples over both timed loops (the mixed one alone is ~30 ms)
        if "mixed" in legs:
            ms_m, zm, qm, launches = time_device(wl.op_m, mesh, z0, q0, args.steps, args.warmup,
                                                 dt, flush, wl.scheme)
        if "fp64" in legs:
            ms_d, zd, qd, launches_d = time_device(wl.op_d, mesh, z0, q0, args.steps,
                                                   args.warmup, dt, flush, wl.scheme)
        else:
            ms_d, zd, qd = [float("nan")], zm, qm
        if "mixed" not in legs:  # FP64-only run (profiling of the FP64 kernel)
            ms_m, zm, qm, launches = ms_d, zd, qd, launches_d
    t_m = max_over_ranks(sum(ms_m) / 1e3, world)
    t_d = max_over_ranks(sum(ms_d) / 1e3, world)
    ndof = 3 * n
    stages = 3
    units = ndof * stages * args.steps * world  # every rank advances its own replica
    value = units / t_m
    value_d = units / t_d
    e2e_ms, io_bytes = time_e2e(wl.op_m, z0, q0, max(2, args.steps // 4), 2, dt, wl.scheme) \
        if "e2e" in legs else (float("nan"), 0)
    e2e_ms = max_over_ranks(e2e_ms, world)
    e2e_value = ndof * stages * world / (e2e_ms / 1e3)
    stage_abi = None
    if "e2e" in legs and wl.scheme == "ssp33":
        sa_ms, sa_in, sa_out = time_e2e_stage_abi(wl.op_m, z0, q0, max(2, args.steps // 10), 1, dt)
        sa_ms = max_over_ranks(sa_ms, world)
        stage_abi = {"value": ndof * stages * world / (sa_ms / 1e3), "unit": "DoF-stage/s",
                     "ms_per_step": sa_ms, "h2d_bytes_per_step": sa_in,
                     "d2h_bytes_per_step": sa_out,
                     "call": "3 x oc_perform_stage_hydro(OC_MEM_HOST) per step, host registers"}
    peak, peak_kind = peaks()
    static_bytes = 4 * sum(wl.op_m.static_data_size(k) for k in range(5)) \
        if wl.name == "channel" else 0
    bytes_step = algorithmic_bytes(n, mesh.n_cells, True, static_bytes)
    step_s = statistics.mean(ms_m) / 1e3
    per_step_launches = launches / args.steps
    achieved = bytes_step / per_step_launches / (step_s / per_step_launches) / 1e9
    clocks = clk.summary()
    err_z, err_q = rel(zm, zd), rel(qm, qd)
    vortex = args.workload == "vortex"
    prof = profiled_traffic() if vortex else {}
    issue = None
    if prof.get("warp_instructions_per_launch") and clocks.get("sm_mhz"):
        # issue-rate roofline: 4 warp schedulers per SM, one instruction per clock each
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        launch_s = step_s / per_step_launches
        peak_issue = 4 * sms * clocks["sm_mhz"] * 1e6
        ach = prof["warp_instructions_per_launch"] / launch_s
        issue = {"achieved": ach / 1e9, "peak": peak_issue / 1e9, "unit": "G warp-inst/s",
                 "frac": ach / peak_issue, "source": "instructions: ncu capture, " + TRAFFIC_PROFILE}
    out = {
        "metric": METRIC, "value": value, "unit": "DoF-stage/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_m / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": wl.desc, "cells": mesh.n_cells, "dofs": ndof,
                   "degrees": sorted(int(p) for p in np.unique(mesh.degree)),
                   "l2": "flushed between steps (512 MB write)",
                   "replicas": world, "launch": wl.op_m.launch_config},
        "fp64": {"value": value_d, "ms_per_step": 1e3 * t_d / args.steps,
                 "launch": wl.op_d.launch_config},
        "speedup_vs_fp64": value / value_d,
        "l2_error_vs_fp64": {"zeta": err_z, "hu_hv": err_q, "after_steps": args.warmup + args.steps},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": prof.get("traffic_bytes_per_launch") if vortex else None,
                     "traffic_source": ("ncu capture, " + TRAFFIC_PROFILE) if vortex else None,
                     "peak_source": peak_kind,
                     "kernel": "oc::stage_kernel (mixed, FP32 stage input)",
                     "algorithmic_bytes_per_step": bytes_step},
        "e2e": {"value": e2e_value, "unit": "DoF-stage/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes},
        "e2e_stage_abi": stage_abi,
        "issue_roofline": issue,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if vortex and {"mixed", "fp64"} <= legs:
        out["secondary_quadrature"] = secondary_quadrature(args, flush)
    if rank == 0 and not args.no_cpu:
        v, cores, el = cpu_baseline(wl, args.cpu_steps)
        out["cpu_baseline"] = {"value": v, "unit": "DoF-stage/s", "cores": cores, "kind": "port",
                               "sample": f"{args.cpu_steps} full time step(s) of the workload "
                                         f"({el:.1f} s)"}
    if rank == 0:
        print(json.dumps(out))
    barrier(world)


if __name__ == "__main__":
    main()
