"""ORACLE — test infrastructure only: full-size parity of one run.

Checks the GPU's results for a whole system against the FP64 oracle without
running the oracle on every pair: a seeded random sample of pairs (2D
entropies and MI terms), bit-exact counts on a smaller sample, every DOF's 1D
entropy, and the oracle's MIST (the reference's scan order) run on the GPU's
own .par body, which must give the GPU's edge list. Used by tests/ and by
bench.py after its timed region, as the checker only; the product never
imports it.
"""
from __future__ import annotations

import time

import numpy as np

from . import BLOCKS, mist, sample

# MI tolerance of the reference comparison (nats), per term
MI_TOL = 1e-5


def random_pairs(D: int, n: int, seed: int):
    """n pairs (g1 < g2), uniform over the D(D-1)/2 unordered pairs."""
    rng = np.random.default_rng(seed)
    a = rng.integers(0, D, size=2 * n + 64)
    b = rng.integers(0, D, size=2 * n + 64)
    keep = a != b
    a, b = a[keep][:n], b[keep][:n]
    return np.minimum(a, b).astype(np.int32), np.maximum(a, b).astype(np.int32)


def _types(g, nb, na):
    return np.where(g < nb, 0, np.where(g < nb + na, 1, 2))


def body_s2(n_dih: int, blocks: dict, g1, g2) -> np.ndarray:
    """S2D of pairs g1 < g2 read from a .par body (reverse triangles for
    bb/aa/dd: PARENT.cpp:1107-1112, util.cpp:55)."""
    nb, na, nd = n_dih + 2, n_dih + 1, n_dih
    lo = np.array([0, nb, nb + na])
    cnt = np.array([nb, na, nd])
    t1, t2 = _types(g1, nb, na), _types(g2, nb, na)
    i, j = g1 - lo[t1], g2 - lo[t2]
    out = np.empty(len(g1))
    keys = {(0, 0): "bb", (0, 1): "ba", (0, 2): "bd", (1, 1): "aa", (1, 2): "ad", (2, 2): "dd"}
    for (a, b), k in keys.items():
        m = (t1 == a) & (t2 == b)
        if not m.any():
            continue
        ii, jj = i[m].astype(np.int64), j[m].astype(np.int64)
        if a == b:
            n = int(cnt[a])
            idx = (n - ii) * (n - ii - 1) // 2 + ii - jj
        else:
            idx = ii * int(cnt[b]) + jj
        out[m] = blocks[k][idx]
    return out


def check_run(bonds, angles, dihedrals, bins, blocks: dict, edges, gpu_counts=None, n_pairs: int = 10000,
              n_count_pairs: int = 100, seed: int = 8191, with_mist: bool = True) -> dict:
    """Compares one GPU run with the oracle.

    bonds/angles/dihedrals: the run's input columns (host arrays, FP32 or FP64).
    blocks: the GPU's .par body blocks; edges: the GPU's MIST edges (structured
    array with t1, t2, i1, i2, mi, left). gpu_counts(pairs) returns the GPU
    pair kernel's counts for a list of (g1, g2) pairs (or None to skip counts).
    """
    nd = dihedrals.shape[0]
    nb, na = nd + 2, nd + 1
    D = nb + na + nd
    P = D * (D - 1) // 2
    n_pairs = min(n_pairs, P)
    g1, g2 = random_pairs(D, n_pairs, seed)
    nc = min(n_count_pairs, n_pairs) if gpu_counts is not None else 0
    t0 = time.perf_counter()
    ref = sample(bonds, angles, dihedrals, bins, g1, g2, n_counts=nc)
    t_sample = time.perf_counter() - t0
    s1_gpu = np.concatenate([blocks["s1_b"], blocks["s1_a"], blocks["s1_d"]])
    s2_gpu = body_s2(nd, blocks, g1, g2)
    mi_gpu = s1_gpu[g1] + s1_gpu[g2] - s2_gpu
    mi_ref = ref["s1"][g1] + ref["s1"][g2] - ref["s2"]
    res = {
        "pairs_sampled": int(n_pairs),
        "pairs_total": int(P),
        "max_abs_dS1_nats": float(np.max(np.abs(s1_gpu - ref["s1"]), initial=0.0)),
        "max_abs_dS2D_nats": float(np.max(np.abs(s2_gpu - ref["s2"]), initial=0.0)),
        "max_abs_dMI_nats": float(np.max(np.abs(mi_gpu - mi_ref), initial=0.0)),
        "mi_tolerance_nats": MI_TOL,
        "oracle_sample_s": round(t_sample, 2),
    }
    if nc:
        pairs = list(zip(g1[:nc].tolist(), g2[:nc].tolist()))
        got = gpu_counts(pairs)
        res["counts_pairs"] = nc
        res["counts_bit_exact"] = bool(all(np.array_equal(a, b) for a, b in zip(got, ref["counts"])))
    if with_mist:
        t0 = time.perf_counter()
        oe, _, gap = mist(nd, {k: np.ascontiguousarray(blocks[k]) for k in BLOCKS}, gaps=True)
        res["oracle_mist_s"] = round(time.perf_counter() - t0, 2)
        same = all(np.array_equal(oe[f], edges[f]) for f in ("t1", "t2", "i1", "i2", "left"))
        res["mist_edges"] = int(len(oe))
        res["mist_identical"] = bool(same)
        res["mist_max_abs_dMI_nats"] = float(np.max(np.abs(oe["mi"] - edges["mi"]), initial=0.0))
        finite = gap[np.isfinite(gap)]
        res["mist_min_gap_nats"] = float(finite.min()) if finite.size else None
        res["mist_tied_steps"] = int(np.sum(gap == 0.0))
    res["ok"] = bool(res["max_abs_dMI_nats"] <= MI_TOL and res.get("counts_bit_exact", True)
                     and res.get("mist_identical", True))
    return res
