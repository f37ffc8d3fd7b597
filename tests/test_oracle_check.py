"""CPU tests of the full-size parity checker (oracle/check.py, oracle.sample,
the oracle's parallel MIST scan): the sampled oracle equals the whole-system
oracle bit for bit, the checker reports zero differences for the oracle's own
results and catches a planted difference, and the gap output agrees with a
brute-force scan."""
from __future__ import annotations

import numpy as np

import oracle
import parent_gb300 as pg
from oracle import check


def _system(prec=0, n_atoms=30, frames=2500, seed=3):
    return pg.synth_host(n_atoms, frames, double_prec=prec, seed=seed, frac_bimodal_dih=0.3,
                         frac_bimodal_bond=0.1)


def test_sample_equals_whole_system_oracle():
    for prec in (0, 1):
        t = _system(prec)
        bins = (50, 40, 30, 20, 25, 50)
        ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
        D = 3 * t.n_dih + 3
        g1, g2 = check.random_pairs(D, 400, seed=5)
        r = oracle.sample(t.bonds, t.angles, t.dihedrals, bins, g1, g2, n_counts=4)
        s1 = np.concatenate([ref["s1_b"], ref["s1_a"], ref["s1_d"]])
        assert np.array_equal(r["s1"], s1)
        assert np.array_equal(r["s2"], check.body_s2(t.n_dih, ref, g1, g2))
        cnt = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, list(zip(g1[:4], g2[:4])))
        assert all(np.array_equal(a, b) for a, b in zip(cnt, r["counts"]))
        assert np.array_equal(r["min"][:t.n_dih + 2], oracle.extrema(t.bonds, t.angles, t.dihedrals)[0][:t.n_dih + 2])


def test_checker_reports_zero_for_the_oracle_and_catches_a_change():
    t = _system()
    bins = (50,) * 6
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    edges, _ = oracle.mist(t.n_dih, ref)
    exact = lambda pairs: oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, pairs)
    res = check.check_run(t.bonds, t.angles, t.dihedrals, bins, ref, edges, gpu_counts=exact,
                          n_pairs=500, n_count_pairs=5)
    assert res["ok"] and res["max_abs_dMI_nats"] == 0.0 and res["mist_identical"] and res["counts_bit_exact"]
    # a planted mistake: one count off, one S2D moved by 1e-4 nats
    bad_counts = lambda pairs: [c + (k == 0) * np.eye(*c.shape, dtype=np.int64) for k, c in enumerate(exact(pairs))]
    moved = {k: v.copy() for k, v in ref.items()}
    moved["dd"] += 1e-4
    res = check.check_run(t.bonds, t.angles, t.dihedrals, bins, moved, edges, gpu_counts=bad_counts,
                          n_pairs=500, n_count_pairs=5)
    assert not res["ok"] and not res["counts_bit_exact"] and res["max_abs_dMI_nats"] > 1e-5


def test_parallel_mist_scan_matches_a_brute_force_scan():
    n = 9
    rng = np.random.default_rng(4)
    # values on a coarse grid: many exact ties, decided by the scan order
    body = {k: np.round(rng.normal(1.0, 0.3, sz), 1) for k, sz in oracle.sizes(n).items()}
    edges, tot, gap = oracle.mist(n, body, gaps=True)
    nb, na, nd = n + 2, n + 1, n
    D = nb + na + nd
    lo = [0, nb, nb + na]
    ty = lambda g: 0 if g < nb else (1 if g < nb + na else 2)
    q = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4, (2, 2): 5}
    ptrs = [oracle._p(np.ascontiguousarray(body[k])) for k in oracle.BLOCKS]
    M = np.zeros((D, D))
    for i in range(D):
        for j in range(i + 1, D):
            M[i, j] = M[j, i] = oracle.lib().or_mutual(q[(ty(i), ty(j))], i - lo[ty(i)], j - lo[ty(j)], n, *ptrs)
    In, Out = [0], list(range(1, D))
    for s in range(D - 1):
        vals = sorted((M[u, v] for u in In for v in Out), reverse=True)
        best, w, u_best = -1e200, None, None
        for ti in range(3):
            for to in range(3):
                for u in (x for x in In if ty(x) == ti):
                    for v in (x for x in Out if ty(x) == to):
                        if M[u, v] > best:
                            best, w, u_best = M[u, v], v, u
        assert edges["t1"][s] == ty(u_best) and edges["t2"][s] == ty(w)
        assert edges["i1"][s] == u_best - lo[ty(u_best)] + 1 and edges["i2"][s] == w - lo[ty(w)] + 1
        assert edges["mi"][s] == best
        assert gap[s] == (vals[0] - vals[1] if len(vals) > 1 else np.inf)
        In.append(w)
        Out.remove(w)
    assert np.sum(gap == 0.0) > 0  # the grid made ties
