"""Multi-rank path on CPU (gloo, world size 2): target-row sharding of one
problem and longest-first sharding of an ensemble give, after an all-gather,
exactly the single-rank result (per-target summation order is unchanged)."""
import math
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import torch
    import torch.distributed as dist

    import lpm_oracle
    import lpm_oracle as O
    from lpm_gb300.partition import problem_assignment, target_slice

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lpm_oracle.set_threads(1)
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    w = 2 * math.pi / 12.5
    fz = O.ic_eval(O.IC_RH54, (w, -w), fx)
    sl = target_slice(vx.shape[0], world, rank)
    idx = np.arange(vx.shape[0])[sl]
    _, u = lpm_oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False, tgt_idx=idx)
    # all-gather slices of uneven length: pad to the longest
    n_max = max(target_slice(vx.shape[0], world, r).stop - target_slice(vx.shape[0], world, r).start
                for r in range(world))
    mine = torch.zeros(n_max, 3, dtype=torch.float64)
    mine[: u.shape[0]] = torch.from_numpy(u)
    parts = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine)
    full = torch.cat([parts[r][: target_slice(vx.shape[0], world, r).stop
                               - target_slice(vx.shape[0], world, r).start] for r in range(world)])
    # ensemble: problems sharded longest-first, no exchange needed
    levels = [0, 1, 2, 1, 0]
    costs = [O.mesh_sizes(O.MESH_ICOS_TRI, l)[1] ** 2 for l in levels]
    mine_p = problem_assignment(costs, world)[rank]
    sums = []
    for p in mine_p:
        pvx, pfx, pfa, pfm = O.mesh(O.MESH_ICOS_TRI, levels[p], 1.0)
        pz = O.ic_eval(O.IC_RH54, (w, -w), pfx)
        _, pu = lpm_oracle.bve_vertex_solve(pvx, pfx, pz, pfa, pfm, want_psi=False)
        sums.append((p, float(np.abs(pu).sum())))
    gathered = [None] * world
    dist.all_gather_object(gathered, sums)
    if rank == 0:
        np.save(os.path.join(out_dir, "sharded.npy"), full.numpy())
        np.save(os.path.join(out_dir, "ensemble.npy"),
                np.array(sorted(x for g in gathered for x in g)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_sharding_matches_single_rank(tmp_path, oracle):
    import torch.multiprocessing as mp

    import lpm_oracle as O
    from lpm_gb300.partition import problem_assignment, target_slice

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    w = 2 * math.pi / 12.5
    fz = O.ic_eval(O.IC_RH54, (w, -w), fx)
    _, u = oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False)
    sharded = np.load(tmp_path / "sharded.npy")
    assert np.array_equal(sharded, u)
    ens = np.load(tmp_path / "ensemble.npy")
    assert [int(p) for p in ens[:, 0]] == [0, 1, 2, 3, 4]
    # every problem evaluated exactly once
    assert sorted(sum(problem_assignment([1, 5, 3, 2, 2], 2), [])) == [0, 1, 2, 3, 4]
    # balanced slices cover all targets
    assert sum(target_slice(10, 3, r).stop - target_slice(10, 3, r).start for r in range(3)) == 10


def _swe_worker(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import torch
    import torch.distributed as dist

    import lpm_oracle
    import lpm_oracle as O
    from lpm_gb300.partition import target_slice

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lpm_oracle.set_threads(1)
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    zeta = np.sin(2 * fx[:, 0]) + fx[:, 2]
    sigma = np.cos(3 * fx[:, 1])
    sl = target_slice(vx.shape[0], world, rank)
    out = lpm_oracle.swe_sphere_sums(vx[sl], fx, zeta, sigma, fa, fm, 0.02)
    n = [target_slice(vx.shape[0], world, r).stop - target_slice(vx.shape[0], world, r).start
         for r in range(world)]
    mine = torch.zeros(max(n), 12, dtype=torch.float64)
    mine[: out.shape[0]] = torch.from_numpy(out)
    parts = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine)
    if rank == 0:
        full = torch.cat([parts[r][: n[r]] for r in range(world)])
        np.save(os.path.join(out_dir, "swe_sharded.npy"), full.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_swe_sharding_matches_single_rank(tmp_path, oracle):
    """The spherical SWE sums shard by targets the same way: no exchange but
    the final gather, identical bits."""
    import torch.multiprocessing as mp

    import lpm_oracle as O

    port = _free_port()
    mp.start_processes(_swe_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    zeta = np.sin(2 * fx[:, 0]) + fx[:, 2]
    sigma = np.cos(3 * fx[:, 1])
    ref = oracle.swe_sphere_sums(vx, fx, zeta, sigma, fa, fm, 0.02)
    assert np.array_equal(np.load(tmp_path / "swe_sharded.npy"), ref)
