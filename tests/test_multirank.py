"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

On GB300 machines the operator runs one replica per GPU (independent ensemble
members, no data-path collective); the timing is the maximum over ranks and
the throughput the sum of the DoF-stage updates of all ranks.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    t = bench.max_over_ranks(1.0 + rank, world)  # rank 1 is the slowest
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    assert out[0] == 2.0 and out[1] == 2.0


def _halo_worker(rank, world, port, out, case):
    """One rank of a partitioned SSP-RK3 run: the FP64 oracle as the stage of
    its local mesh (owned cells + ghosts), ghosts refreshed over gloo before
    every stage; returns the owned DoFs after two steps."""
    import sys
    import numpy as np
    import torch
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from cases import CASES, VORTEX, static_arrays
    from oceano_gb300.partition import (HaloExchange, partition, partitioned_erk_step,
                                        with_ghost_boundary)
    from oracle import oracle as O
    mesh_f, bcs, pdata, friction = CASES[case]
    mesh = mesh_f()
    full = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    if pdata is not None:
        full.set_static(*static_arrays(full, pdata))
    z0, q0 = full.project_vortex(0.0)
    dt = 0.05 / full.transport_speed(z0, q0)
    parts = partition(mesh, world)
    part = parts[rank]
    orc = O.Oracle(part.mesh, friction=friction, bcs=with_ghost_boundary(bcs),
                     vortex=VORTEX + [0, 0])
    if pdata is not None:
        orc.set_static(*static_arrays(orc, pdata))
    iz, iq = part.dof_index(mesh, "zeta"), part.dof_index(mesh, "q")
    z = torch.from_numpy(z0[iz].copy())
    q = torch.from_numpy(q0[iq].copy())
    z[part.mesh.offsets()[part.n_owned]:] = 0.0  # ghosts start unknown: the halo fills them
    halo = HaloExchange(parts, rank)

    def stage(st, s, t, f, rz, rq, kz, kq, sz, sq, nz, nq):
        kzn = [k.numpy() for k in kz]
        kqn = [k.numpy() for k in kq]
        orc.stage_erk(st, s, t, f, rz.numpy(), rq.numpy(), kzn, kqn, sz.numpy(), sq.numpy(),
                      nz.numpy(), nq.numpy())

    tb = O.TABLEAUX["ssp33"]
    for it in range(2):
        partitioned_erk_step(stage, halo, tb, it * dt, dt, z, q)
    no = int(part.mesh.offsets()[part.n_owned])
    out[rank] = (iz[:no], z.numpy()[:no].copy(), iq[:2 * no], q.numpy()[:2 * no].copy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("case", ["hanging_p2", "mixed_degree", "hanging_p3_bathy"])
def test_partitioned_run_matches_single_mesh(case):
    """Three gloo ranks, one-layer halo refreshed before every stage: the owned DoFs
    equal the single-mesh oracle run (1e-13 relative)."""
    import sys
    import numpy as np
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    from cases import CASES, VORTEX, static_arrays
    from oracle import oracle as O
    world = 3
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_halo_worker, args=(world, port, out, case), nprocs=world, join=True,
                       start_method="spawn")
    mesh_f, bcs, pdata, friction = CASES[case]
    mesh = mesh_f()
    full = O.Oracle(mesh, friction=friction, bcs=bcs, vortex=VORTEX + [0, 0])
    if pdata is not None:
        full.set_static(*static_arrays(full, pdata))
    z, q = full.project_vortex(0.0)
    dt = 0.05 / full.transport_speed(z, q)
    tb = O.TABLEAUX["ssp33"]
    for it in range(2):
        O.erk_step(full, tb["a"], tb["b"], tb["c"], it * dt, dt, z, q)
    zg, qg = np.full_like(z, np.nan), np.full_like(q, np.nan)
    for r in range(world):
        iz, vz, iq, vq = out[r]
        zg[iz] = vz
        qg[iq] = vq
    assert np.isfinite(zg).all() and np.isfinite(qg).all()
    assert np.linalg.norm(zg - z) <= 1e-13 * np.linalg.norm(z)
    assert np.linalg.norm(qg - q) <= 1e-13 * np.linalg.norm(q)
