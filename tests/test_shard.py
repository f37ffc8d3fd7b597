"""Splitting one trajectory's pair work over ranks (pg_entropy_shard).

CPU: the shards' body masks partition the .par body, and two gloo ranks that
each hold their shard of a body (the oracle's values on the rank's own
entries, zeros elsewhere) reproduce the whole body exactly with the SUM
reduction the driver uses. GPU: shard bodies from the CUDA path sum to the
pg_entropy body bit for bit, and each shard writes only its own entries."""
from __future__ import annotations

import multiprocessing as mp
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
import parent_gb300 as pg
import parent_gb300.shard as sh

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("n_dih,bins,n_shards", [(20, (50,) * 6, 3), (20, (30,) * 6, 2), (3, (50,) * 6, 7),
                                                  (0, (50,) * 6, 2), (60, (10, 20, 30, 100, 40, 20), 4),
                                                  (40, (50,) * 6, 1)])
def test_shard_masks_partition_the_body(n_dih, bins, n_shards):
    masks = [sh.shard_mask(n_dih, bins, s, n_shards) for s in range(n_shards)]
    owners = np.sum([m.astype(int) for m in masks], axis=0)
    assert owners.size == sum(pg.block_sizes(n_dih).values())
    assert owners.min() == 1 and owners.max() == 1
    D = 3 * n_dih + 3
    assert masks[0][:D].all()  # shard 0 owns the 1D entropies
    if n_shards > 1 and n_dih >= 20:  # shards are cut by pair work, not tile count
        sizes = [int(m[D:].sum()) for m in masks]
        assert max(sizes) <= 1.1 * (sum(sizes) / n_shards), sizes


def test_shard_mask_rejects_bad_arguments():
    with pytest.raises(pg.PGError):
        sh.shard_mask(5, (50,) * 6, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, n_dih, bins, full, q):
    try:
        sys.path.insert(0, str(ROOT))
        import torch.distributed as dist

        import parent_gb300.shard as shm
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        local = np.where(shm.shard_mask(n_dih, bins, rank, world), full, 0.0)
        merged = shm.merge_bodies(n_dih, local, dist, "cpu")
        dist.destroy_process_group()
        q.put((rank, None if merged is None else merged.flat(), None))
    except Exception as e:
        q.put((rank, None, repr(e)))


def test_two_gloo_ranks_merge_shards_exactly():
    pytest.importorskip("torch.distributed")
    n_dih, bins = 15, (50,) * 6
    t = pg.synth_host(n_dih + 3, 4000, double_prec=1, seed=3, frac_bimodal_dih=0.2)
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    full = np.concatenate([ref[k] for k in pg.block_sizes(n_dih)])
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, n_dih, bins, full, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in range(2):
            r = q.get(timeout=180)
            res[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert res[0][2] is None and res[1][2] is None, (res[0][2], res[1][2])
    assert res[1][1] is None
    assert np.array_equal(res[0][1].view(np.uint64), full.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("n_atoms,F,bins,n_shards", [(60, 20000, (50,) * 6, 3), (40, 9000, (30,) * 6, 2),
                                                       (25, 5000, (50, 50, 50, 100, 100, 100), 4)])
@pytest.mark.parametrize("stream", ["0", "1"])
def test_gpu_shards_sum_to_the_whole(monkeypatch, n_atoms, F, bins, n_shards, stream):
    # the streamed 32-slot layout where it applies (2D bins <= 50), else the
    # ring-fed or 16-slot one
    monkeypatch.setenv("PG_HIST_STREAM", stream)
    t = pg.synth_host(n_atoms, F, double_prec=0, seed=n_atoms, frac_bimodal_dih=0.2)
    n = n_atoms - 3
    with pg.Engine(0) as eng:
        whole = eng.entropy(t, bins, "hist").flat()
        acc = np.zeros_like(whole)
        for s in range(n_shards):
            part = eng.entropy_shard(t, bins, s, n_shards).flat()
            mask = sh.shard_mask(n, bins, s, n_shards)
            assert not np.any(part[~mask]), s
            acc += part
        assert np.array_equal(acc.view(np.uint64), whole.view(np.uint64))
        merged = sh.entropy_sharded(eng, t, bins)  # one rank: the whole body
        assert np.array_equal(merged.flat().view(np.uint64), whole.view(np.uint64))
        e1, t1 = eng.mist(n, merged)
        eng.entropy(t, bins, "hist")
        e2, t2 = eng.mist(n)
        assert np.array_equal(e1, e2) and np.array_equal(t1, t2)


@pytest.mark.gpu
def test_gpu_shards_into_device_memory():
    """Shard bodies written straight into CUDA tensors (DeviceParBody), summed
    on the device, equal the pg_entropy body bit for bit; entropy_sharded with
    a CUDA device keeps the merged body there, and MIST read from it gives the
    tree of the host body."""
    torch = pytest.importorskip("torch")
    t = pg.synth_host(50, 12000, double_prec=0, seed=8, frac_bimodal_dih=0.2)
    n, bins, k = 47, (50,) * 6, 3
    with pg.Engine(0) as eng:
        whole = eng.entropy(t, bins, "hist")
        total = whole.flat().size
        acc = torch.zeros(total, dtype=torch.float64, device="cuda:0")
        for s in range(k):
            part = torch.full((total,), float("nan"), dtype=torch.float64, device="cuda:0")
            torch.cuda.synchronize()
            eng.entropy_shard(t, bins, s, k, out=pg.DeviceParBody(n, part.data_ptr()))
            mask = torch.from_numpy(sh.shard_mask(n, bins, s, k)).to("cuda:0")
            assert not torch.any(part[~mask] != 0)  # every entry written, zeros outside the shard
            acc += part
        assert np.array_equal(acc.cpu().numpy().view(np.uint64), whole.flat().view(np.uint64))
        dev = sh.entropy_sharded(eng, t, bins, device="cuda:0", on_device=True)
        assert isinstance(dev, pg.DeviceParBody)
        assert np.array_equal(dev.tensor.cpu().numpy().view(np.uint64), whole.flat().view(np.uint64))
        e1, t1 = eng.mist(n, dev)
        e2, t2 = eng.mist(n, whole)
        assert np.array_equal(e1, e2) and np.array_equal(t1, t2)
        host = sh.entropy_sharded(eng, t, bins, device="cuda:0")
        assert np.array_equal(host.flat().view(np.uint64), whole.flat().view(np.uint64))


@pytest.mark.gpu
def test_gpu_shard_rejects_onehot_and_bad_index():
    t = pg.synth_host(10, 2000, double_prec=0, seed=1)
    with pg.Engine(0) as eng:
        with pytest.raises(pg.PGError) as ex:
            eng.entropy_shard(t, (50,) * 6, 0, 2, form="onehot")
        assert ex.value.code == pg.PG_ERR_UNSUPPORTED
        with pytest.raises(pg.PGError) as ex:
            eng.entropy_shard(t, (50,) * 6, 2, 2)
        assert ex.value.code == pg.PG_ERR_ARG


@pytest.mark.gpu
def test_bench_shard_mode_one_rank():
    """bench.py --shard (one system split over the ranks, strong scaling) on
    one GPU: the contract's keys, and the merged device body equals the
    one-GPU pg_entropy body bit for bit."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    p = subprocess.run([sys.executable, str(root / "bench.py"), "--shard", "--workload", "plain_294dof_20k",
                        "--steps", "2", "--warmup", "1", "--e2e-steps", "1"], cwd=root, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    d = json.loads([ln for ln in p.stdout.splitlines() if ln.strip()][-1])
    assert d["scaling"] == "strong" and d["n_gpus"] == 1 and d["value"] > 0
    assert d["check"]["merged_equals_one_gpu_body"] is True
    assert d["e2e"]["value"] > 0 and d["gpu_launches"] > 0
