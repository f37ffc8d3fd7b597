"""One trajectory over several ranks (one GPU each): the reference's MPI
split of the pair work (PARENT.cpp:333-414, 775-1119), GB300 style.

Every rank preprocesses all DOFs and computes the 2D entropies of its own
contiguous range of the pair-tile list (pg_entropy_shard); the exchange step
is one element-wise SUM reduction of the .par bodies to rank 0, exact in FP64
because every entry is non-zero on at most one rank. MIST then runs on rank 0
from the merged body.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import DeviceParBody, ParBody, _check, block_sizes, lib


def shard_mask(n_dih: int, bins, shard: int, n_shards: int) -> np.ndarray:
    """Body entries (.par body order) that shard `shard` writes."""
    total = sum(block_sizes(n_dih).values())
    m = np.zeros(total, dtype=np.uint8)
    _check(lib().pg_shard_mask(n_dih, (C.c_int * 6)(*bins), shard, n_shards,
                               m.ctypes.data_as(C.POINTER(C.c_uint8))))
    return m.astype(bool)


def body_from_flat(n_dih: int, flat: np.ndarray) -> ParBody:
    blocks, o = {}, 0
    for k, n in block_sizes(n_dih).items():
        blocks[k] = np.ascontiguousarray(flat[o:o + n])
        o += n
    return ParBody(n_dih, blocks)


def merge_bodies(n_dih: int, local: np.ndarray, dist=None, device: str = "cpu") -> ParBody | None:
    """Sums the ranks' shard bodies onto rank 0 (returns None on the others)."""
    if dist is None:
        return body_from_flat(n_dih, local)
    import torch
    t = torch.from_numpy(np.ascontiguousarray(local, dtype=np.float64)).to(device)
    dist.reduce(t, dst=0, op=dist.ReduceOp.SUM)
    if dist.get_rank() != 0:
        return None
    return body_from_flat(n_dih, t.cpu().numpy())


def entropy_sharded(eng, traj, bins, dist=None, device: str = "cpu", form: str = "auto",
                    on_device: bool = False):
    """PARENT.x over all ranks of `dist` (or alone): rank 0 returns the body.

    With a CUDA `device` (the engine's GPU) each rank's shard is written
    straight into a device tensor, the SUM reduction runs on it (NCCL), and
    rank 0 gets the host body, or with on_device=True a DeviceParBody (its
    tensor attached as `.tensor`) that Engine.mist reads without a host copy.
    Otherwise the shards are host arrays reduced on `device` (gloo on CPU)."""
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist is not None else (0, 1)
    n_dih = traj.n_dihedrals if hasattr(traj, "n_dihedrals") else traj.n_dih
    if str(device).startswith("cuda"):
        import torch
        total = sum(block_sizes(n_dih).values())
        t = torch.zeros(total, dtype=torch.float64, device=device)
        torch.cuda.synchronize(t.device)  # the zeros are written before the engine's stream writes
        eng.entropy_shard(traj, bins, rank, world, form, out=DeviceParBody(n_dih, t.data_ptr()))
        if dist is not None:
            dist.reduce(t, dst=0, op=dist.ReduceOp.SUM)
        if rank != 0:
            return None
        if on_device:
            torch.cuda.synchronize(t.device)
            body = DeviceParBody(n_dih, t.data_ptr())
            body.tensor = t
            return body
        return body_from_flat(n_dih, t.cpu().numpy())
    part = eng.entropy_shard(traj, bins, rank, world, form)
    return merge_bodies(n_dih, part.flat(), dist, device)
