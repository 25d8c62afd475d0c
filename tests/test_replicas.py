"""Replica sharding on CPU ranks (gloo, world size 2).

Each rank traces its own photon range (scene.replica_ray_offset, the function bench.py uses for its
replicas) through the CPU oracle, the ranks sum their integer tallies with an all-reduce, and the sum
must equal one single-process run over the union of the ranges: per-ray random streams keyed by the
global photon id make the tallies independent of the partition.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INT_KEYS = ("hw_native", "hw_mirror", "hw_native_direct", "hw_mirror_direct", "status_counts",
            "failure_code_counts", "event_counts", "entered_sums", "ray_flags", "ic_hist")
N_TOTAL = 40_000


def _scene():
    from tardiis_and_claritas_gb300 import scene as S
    cfg = S.small_cell_config()
    cfg.validate()
    return cfg, S.quartz_particles(2000.0)


def _trace(rank_offset: int, n: int) -> dict:
    import oracle_harness as H
    from tardiis_and_claritas_gb300 import scene as S
    cfg, parts = _scene()
    orc = H.OracleRun("port", cfg, parts)
    t, _ = orc.trace(S.run_params(n, seed=4, ray_offset=rank_offset), threads=1)
    orc.close()
    return {k: np.asarray(t[k], dtype=np.int64) for k in INT_KEYS}


def _rank_main(rank: int, world: int, port: int, out_path: str):
    for p in (ROOT, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    from tardiis_and_claritas_gb300 import scene as S
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = N_TOTAL // world
    mine = _trace(S.replica_ray_offset(rank, 0, 1, n), n)
    summed = {}
    for k in INT_KEYS:
        t = torch.from_numpy(mine[k].copy())
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        summed[k] = t.numpy()
    if rank == 0:
        np.savez(out_path, **summed)
    dist.barrier()
    dist.destroy_process_group()


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_tallies_sum_to_single_run(tmp_path):
    pytest.importorskip("torch")
    from tardiis_and_claritas_gb300 import scene as S
    out = str(tmp_path / "summed.npz")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    summed = np.load(out)
    whole = _trace(0, N_TOTAL)
    for k in INT_KEYS:
        np.testing.assert_array_equal(summed[k], whole[k], err_msg=k)
    assert int(summed["status_counts"].sum()) == N_TOTAL
    # the shards really are disjoint and contiguous
    assert S.replica_ray_offset(1, 0, 1, N_TOTAL // 2) == N_TOTAL // 2
