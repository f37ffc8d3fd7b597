"""The multi-rank path of bench.py on CPU: two `gloo` ranks (world_size 2).

On N GPUs every rank runs its own independent system (its own seed; no
collective in the data path) and the timed region is the slowest rank's
(barrier + max over ranks), so the whole-job value is units x N / max time.
These tests run that host logic with real process groups and real
per-rank synthetic systems, without a GPU."""
from __future__ import annotations

import multiprocessing as mp
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    try:
        sys.path.insert(0, str(ROOT))
        import torch.distributed as dist

        import bench
        import parent_gb300 as pg

        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        # each rank: its own replica of the workload generator, seeded by rank
        seed = bench.replica_seed(20260, rank)
        t = pg.synth_host(12, 3000, double_prec=0, seed=seed, frac_bimodal_dih=0.2)
        checksum = float(np.float64(t.bonds.sum()) + t.angles.sum() + t.dihedrals.sum())
        # the timed region: barrier, local time, max over ranks
        dist.barrier()
        local_ms = 100.0 + 25.0 * rank
        slowest = bench.max_over_ranks(local_ms, dist, "cpu")
        systems = bench.batch_systems(seed=bench.replica_seed(64, rank))
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, seed, checksum, slowest, systems[:3], None))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, None, None, None, None, repr(e)))


def _run(world: int):
    ctx = mp.get_context("spawn")  # no fork after any CUDA or thread state
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in range(world):
            r = q.get(timeout=180)
            out[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    return out


def test_two_gloo_ranks_run_independent_replicas():
    pytest.importorskip("torch.distributed")
    out = _run(2)
    assert sorted(out) == [0, 1]
    for r in (0, 1):
        assert out[r][5] is None, out[r][5]
    # max over ranks: both ranks see the slowest rank's time
    assert out[0][3] == out[1][3] == 125.0
    # replicas: different seeds, different data, different batch systems
    assert out[0][1] != out[1][1]
    assert out[0][2] != out[1][2]
    assert out[0][4] != out[1][4]
    # rank 0's seeds are the single-GPU workload's (the N=1 line is unchanged)
    assert out[0][1] == 20260


def test_whole_job_value_is_units_times_ranks_over_slowest():
    import bench
    units, world, slowest_s = 1.4e13, 2, 3.5
    value = units * world / slowest_s
    assert value == pytest.approx(8.0e12)
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
